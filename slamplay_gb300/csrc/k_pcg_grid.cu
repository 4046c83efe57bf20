// k_pcg_grid.cu — the whole PCG of one problem in one launch spread over the
// whole GPU (FP64 form, explicit Schur complement).
//
// In the FP64 form a PCG iteration is about 0.6 M FP64 FMAs (the product
// with the 9x9 blocks of S) separated by two problem-wide reductions.  GB300
// issues FP64 at about two FMAs per clock per SM, so the product alone takes
// some 10 us on the 16 SMs of a thread-block cluster and ~1 us on all SMs;
// as two kernels per iteration (k_schur.cu's product, k_pcg.cu's camera
// kernel) the iteration costs two kernel boundaries (~27 us).  Here one CTA
// per SM runs every iteration of the problem's PCG, with a grid-wide
// barrier after each reduction:
//   A. q = S p_k for the cameras the CTA owns (runs of about equal numbers
//      of blocks of S): p_k = z_k + beta_k p_{k-1} of the owned blocks'
//      columns staged in shared memory, then per camera three row triplets
//      of eight lanes each over the blocks (spmv_triplet_fp64); each owned
//      camera's p.q.                                             barrier
//   B. p.q over the cameras (one warp), alpha; for the camera blocks (8
//      cameras) the CTA owns: p_k, x, r, z = M r, each block's r.z, r.r,
//      x.(v + r).                                                barrier
//   C. in every CTA: the stopping test and beta_{k+1} from the blocks'
//      values (one warp), while the other warps load what the next
//      iteration's staged direction needs.
// The owned rows of S stay in shared memory for the launch (S is fixed
// during the PCG) when they fit; a CTA with more blocks than the layout
// holds reads them from L2.  GB300's FP64 pipe retires about two lanes per
// clock per SM, so the kernel keeps FP64 instructions off idle lanes: the
// reductions over cameras run in one warp, the direction is formed once
// per (block, column) and not once per row.
// Every CTA takes the same decisions from the same values, so all reach the
// same barriers.  The arithmetic is the two-kernel FP64 PCG's, operation
// for operation (the same product, the same reduction trees), so both forms
// give the same bits, and no result depends on how many CTAs took part.
//
// Participation.  The CTAs that start register on a counter; the first one
// closes the registration once every CTA of the launch has registered, or
// after kRegisterNs (another stream's kernels may hold SMs), and the work is
// split over the P CTAs that registered; a CTA that arrives after the
// closing leaves at once.  So every CTA that waits at a barrier waits only
// for CTAs that are running, whatever else the GPU is doing.  Every wait is
// bounded (kWaitNs, about a second): a CTA whose wait runs out raises the
// abort word, which ends every other CTA's waits; the problem's solve then
// ends with GBA_ERR_TIMEOUT in the status word and the LM loop stops.  The
// control words are zeroed by the camera Schur kernel K3b before each
// launch.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"
#include "kernels.h"

namespace gba {

namespace {

constexpr int kGThreads = kPcgGridThreads;
constexpr int kGWarps = kGThreads / 32;
constexpr int kGCamThreads = 3 * kSpmvSub;                // threads per camera in the product
constexpr int kGCamsPerRound = kGThreads / kGCamThreads;  // cameras per round of the product
constexpr int kGMaxOwn = 64;                               // cameras a CTA's shared-memory layout indexes
constexpr int kGBlkSlot = 96;                              // threads per camera block in the update (3 warps)
constexpr int kGBlksPerRound = kGThreads / kGBlkSlot;
static_assert(kGCamsPerRound >= 1 && kGBlksPerRound >= 1 && kGThreads % 32 == 0, "whole warps, at least one slot");
static_assert(kGBlkSlot % 32 == 0 && kGCamThreads % kSpmvSub == 0, "block slots of whole warps, camera groups of whole lane groups");
static_assert(9 * kPcgBlockCams <= kGBlkSlot, "a camera block's coordinates fit its slot");

constexpr unsigned long long kClosed = 1ull << 63;
constexpr unsigned long long kCountMask = 0xffffffffull;
constexpr unsigned long long kRegisterNs = 30000ull;    // stragglers of the launch, at most
constexpr unsigned long long kWaitNs = 1000000000ull;   // any other wait, at most

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add_u32(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Raises the abort word (first one wins) and records the timeout.
__device__ void grid_abort(const DeviceBatch &B) {
  if (atomicExch(B.grid_ctl + kGridAbort, 1u) == 0u)
    atomicExch(reinterpret_cast<unsigned *>(B.status), (unsigned)GBA_ERR_TIMEOUT);
}

// Grid-wide barrier of the P registered CTAs (generation `gen`, from 1):
// every thread's earlier writes are ordered before thread 0's release
// increment; after thread 0's acquire wait and the CTA barrier every thread
// reads the other CTAs' writes (with __ldcg: L2, not a stale L1 line).
// Returns false (in every thread) when the wait ran out or was aborted.
__device__ __forceinline__ bool grid_barrier(const DeviceBatch &B, unsigned gen, unsigned P, int *s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned *bar = B.grid_ctl + kGridBar;
    __threadfence();
    red_release_add_u32(bar, 1u);
    const unsigned target = gen * P;
    if (ld_acquire_u32(bar) < target) {
      const unsigned long long t0 = global_ns();
      unsigned n = 0;
      while (ld_acquire_u32(bar) < target) {
        if ((++n & 63u) == 0u) {
          if (ld_acquire_u32(B.grid_ctl + kGridAbort) != 0u) {
            ok = 0;
            break;
          }
          if (global_ns() - t0 > kWaitNs) {
            grid_abort(B);
            ok = 0;
            break;
          }
        }
      }
    }
    __threadfence();
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

// Dynamic shared memory: the rows of the block-Jacobi inverse of the
// update's coordinates (one row per thread), per owned camera its first
// block (boff, the diagonal block last in each camera's run), per owned
// block its column camera, its 81 values (when cached) and the direction
// at its nine columns.
struct GridSmem {
  size_t mrow, boff, scol, sval, pst, total;
};
__host__ __device__ inline size_t grid_align(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline GridSmem grid_smem(int cap_blocks, bool cache_s) {
  GridSmem l;
  size_t o = 0;
  l.mrow = o, o = grid_align(o + 8 * 9 * (size_t)kGThreads);
  l.boff = o, o = grid_align(o + 4 * (size_t)(kGMaxOwn + 1));
  l.scol = o, o = grid_align(o + 4 * (size_t)cap_blocks);
  l.sval = o, o = grid_align(o + (cache_s ? 8 * 81 * (size_t)cap_blocks : 0));
  l.pst = o, o = grid_align(o + 8 * 9 * (size_t)cap_blocks);
  l.total = o;
  return l;
}

}  // namespace

__global__ void __launch_bounds__(kGThreads, 1) k_pcg_grid(DeviceBatch B, int cap_blocks, int cache_s) {
  extern __shared__ __align__(16) unsigned char g_smem[];
  __shared__ int s_ticket, s_P, s_ok, s_own0, s_own1, s_stop;
  __shared__ double pqs[kGCamsPerRound][9];
  __shared__ double sc[4];
  __shared__ double rv[kGThreads];  // r_{k+1} of the update's coordinates, for M r
  __shared__ double red3[kGWarps][3];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  LMState *L = B.lm;  // one problem
  // the same state in every CTA (written by the kernels before this one)
  if (!(L->active && L->pcg_active)) return;
  const ProblemInfo pi = B.prob[0];

  // ---- registration --------------------------------------------------------
  if (t == 0) {
    unsigned long long *reg = reinterpret_cast<unsigned long long *>(B.grid_ctl + kGridReg);
    const unsigned long long old = atomicAdd(reg, 1ull);
    int ticket = -1, P = 0;
    if (!(old & kClosed)) {
      ticket = (int)(old & kCountMask);
      if (ticket == 0) {
        const unsigned long long t0 = global_ns();
        while ((ld_acquire_u64(reg) & kCountMask) < gridDim.x && global_ns() - t0 < kRegisterNs) {
        }
        P = (int)(atomicOr(reg, kClosed) & kCountMask);
        st_release_u32(B.grid_ctl + kGridCount, (unsigned)P + 1u);
      } else {
        const unsigned long long t0 = global_ns();
        unsigned v;
        while ((v = ld_acquire_u32(B.grid_ctl + kGridCount)) == 0u) {
          if (global_ns() - t0 > kWaitNs) {
            grid_abort(B);
            break;
          }
        }
        if (v == 0u)
          ticket = -1;
        else
          P = (int)v - 1;
      }
    }
    s_ticket = ticket;
    s_P = P;
  }
  __syncthreads();
  const int w = s_ticket, P = s_P;
  if (w < 0) return;  // arrived after the closing (or the closing never came)

  // ---- ownership -------------------------------------------------------------
  // product: cameras in P runs of about equal blocks (off-diagonal + diagonal)
  const int n = pi.cam_count, c0 = pi.cam_begin;
  {
    const int r0 = B.sblk_row[c0];
    const long long wtot = (long long)(B.sblk_row[c0 + n] - r0) + n;
    const long long ta = ((long long)w * wtot + P - 1) / P, tb = ((long long)(w + 1) * wtot + P - 1) / P;
    int a = 0, b = 0;
    for (int cb = 0; cb < n; cb += kGThreads) {
      const int c = cb + t;
      const long long before = c < n ? (long long)(B.sblk_row[c0 + c] - r0) + c : wtot;
      a += __syncthreads_count(before < ta);
      b += __syncthreads_count(before < tb);
    }
    if (t == 0) s_own0 = a, s_own1 = b;
  }
  // update: camera blocks in P equal runs
  const int nblk = pi.cam_block_count;
  const int kb0 = pi.cam_block_begin + (int)((long long)w * nblk / P);
  const int kb1 = pi.cam_block_begin + (int)((long long)(w + 1) * nblk / P);
  __syncthreads();
  const int own0 = c0 + s_own0, own1 = c0 + s_own1, own_n = own1 - own0;
  const double *vals = reinterpret_cast<const double *>(B.sblk_val);
  const double *Sii = reinterpret_cast<const double *>(B.cam_Sii);
  // the owned blocks in shared memory: staged directions (and cached values)
  // when they fit the layout, else everything from L2
  const GridSmem lay = grid_smem(cap_blocks, cache_s != 0);
  int *boff = reinterpret_cast<int *>(g_smem + lay.boff);
  int *scol = reinterpret_cast<int *>(g_smem + lay.scol);
  double *sval = reinterpret_cast<double *>(g_smem + lay.sval);
  double *pst = reinterpret_cast<double *>(g_smem + lay.pst);
  const int nbo = own_n > 0 ? (B.sblk_row[own1] - B.sblk_row[own0]) + own_n : 0;
  const bool staged = own_n <= kGMaxOwn && nbo <= cap_blocks;
  const bool cached = staged && cache_s != 0;
  if (staged) {
    if (t <= own_n) boff[t] = B.sblk_row[own0 + t] - B.sblk_row[own0] + t;
    __syncthreads();
    for (int lc = 0; lc < own_n; ++lc) {
      const int c = own0 + lc;
      const int r0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - r0, b0 = boff[lc];
      for (int v = t; v <= nb; v += kGThreads) scol[b0 + v] = v < nb ? B.sblk_col[r0 + v] : c;
      if (cached)
        for (int e = t; e < 81 * (nb + 1); e += kGThreads) {
          const int v = e / 81, el = e - 81 * v;
          sval[81 * (size_t)(b0 + v) + el] = v < nb ? vals[81 * (size_t)(r0 + v) + el] : Sii[81 * (size_t)c + el];
        }
    }
    __syncthreads();
  }

  const DeviceOptions &o = B.opt;
  // the direction of iteration k lives in pbuf(k): pcg_p for even k, pcg_p2 for odd k
  auto pbuf = [&](int kk) -> double * { return (kk & 1) ? B.pcg_p2 : B.pcg_p; };
  double rz_k = L->rz, beta = L->beta, q0 = L->q0;
  double last_rr = L->rr, last_pq = L->pq;
  const double lim = o.pcg_tolerance * L->r0_norm;
  int k = 0;
  bool linear_ok = true, aborted = false;
  unsigned gen = 0;

  // the update's coordinate of this thread (the camera kernel's lead
  // threads: coordinate m of a camera block in the lanes of 3 warps); with
  // at most kGBlksPerRound owned blocks its state stays in registers
  const bool one_round = kb1 - kb0 <= kGBlksPerRound;
  const int u_slot = t / kGBlkSlot, u_m = t - kGBlkSlot * u_slot;
  const int u_lc = u_m / 9, u_q = u_m - 9 * u_lc;
  double ux = 0.0, ur = 0.0, uz = 0.0, uv = 0.0, up = 0.0;
  double *umrow = reinterpret_cast<double *>(g_smem + lay.mrow) + 9 * t;
  bool u_in = false, u_lead = false;
  size_t u_i = 0;
  if (one_round) {
    const int blk = kb0 + u_slot;
    u_in = u_slot < kGBlksPerRound && blk < kb1;
    int4 cbk = make_int4(0, 0, 0, 0);
    if (u_in) cbk = B.camblk[blk];
    u_lead = u_in && u_m < 9 * kPcgBlockCams && u_lc < cbk.z;
    u_i = 9 * (size_t)(cbk.y + (u_lead ? u_lc : 0)) + u_q;
    if (u_lead) {
      const double *M = B.cam_Minv + 9 * u_i;  // row u_q of the camera's block: 81 c + 9 q = 9 i
#pragma unroll
      for (int kk = 0; kk < 9; ++kk) umrow[kk] = M[kk];
      ux = B.pcg_x[u_i];
      ur = B.pcg_r[u_i];
      uz = B.pcg_z[u_i];
      uv = B.pcg_v[u_i];
    }
  }
  // the staged direction of the owned blocks' columns: p_0 = z_0
  if (staged) {
    for (int e = t; e < 9 * nbo; e += kGThreads) {
      const int bl = e / 9, cc = e - 9 * bl;
      pst[e] = __ldcg(B.pcg_z + 9 * (size_t)scol[bl] + cc);
    }
  }
  __syncthreads();
  for (;;) {
    // ---- A. q = S p_k, each owned camera's p.q -------------------------------
    const double *pprev = pbuf(k + 1);  // p_{k-1}
    auto pdir = [&](size_t idx) -> double {
      const double z = __ldcg(B.pcg_z + idx);
      if (k == 0) return z;
      return fma(beta, __ldcg(pprev + idx), z);
    };
    for (int cb = 0; cb < own_n; cb += kGCamsPerRound) {
      const int slot = t / kGCamThreads, m = t - kGCamThreads * slot;
      const int g = m / kSpmvSub, j = m - kSpmvSub * g;
      const int lc = cb + slot, c = own0 + lc;
      if (slot < kGCamsPerRound && lc < own_n) {
        const unsigned gmask = 0xffu << (lane & ~(kSpmvSub - 1));
        double q[3];
        if (staged) {
          const int b0 = boff[lc], nb = boff[lc + 1] - b0 - 1;
          if (cached)
            spmv_triplet_fp64(
                nb, j, gmask, [&](int v, int rr) { return sval + 81 * (size_t)(b0 + v) + 9 * (g + 3 * rr); },
                [&](int v, int cc) { return pst[9 * (b0 + v) + cc]; }, q);
          else {
            const int r0 = B.sblk_row[c];
            spmv_triplet_fp64(
                nb, j, gmask,
                [&](int v, int rr) {
                  return (v < nb ? vals + 81 * (size_t)(r0 + v) : Sii + 81 * (size_t)c) + 9 * (g + 3 * rr);
                },
                [&](int v, int cc) { return pst[9 * (b0 + v) + cc]; }, q);
          }
        } else {
          const int r0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - r0;
          spmv_triplet_fp64(
              nb, j, gmask,
              [&](int v, int rr) {
                return (v < nb ? vals + 81 * (size_t)(r0 + v) : Sii + 81 * (size_t)c) + 9 * (g + 3 * rr);
              },
              [&](int v, int cc) { return pdir(9 * (size_t)(v < nb ? B.sblk_col[r0 + v] : c) + cc); }, q);
        }
        if (j == 0) {
#pragma unroll
          for (int rr = 0; rr < 3; ++rr) {
            const int row = g + 3 * rr;
            const size_t i = 9 * (size_t)c + row;
            B.pcg_q[i] = q[rr];
            // p_k at the camera's own coordinate: its diagonal block's column
            const double pk = staged ? pst[9 * (boff[lc + 1] - 1) + row] : pdir(i);
            pqs[slot][row] = pk * q[rr];
          }
        }
      }
      __syncthreads();
      if (t < kGCamsPerRound && cb + t < own_n) {
        double s2 = 0.0;
#pragma unroll
        for (int r = 0; r < 9; ++r) s2 += pqs[t][r];
        B.spmv_red[own0 + cb + t] = s2;
      }
      __syncthreads();
    }
    if (!grid_barrier(B, ++gen, (unsigned)P, &s_ok)) {
      aborted = true;
      break;
    }
    // ---- B. p.q over the cameras (warp 0), alpha; the update ------------------
    double qv_pre = 0.0;
    if (t < 32) {
      const double s2 = warp_strided_sum(B.spmv_red + c0, n);
      if (t == 0) {
        sc[0] = s2;
        sc[1] = rz_k * recip_nr(s2);
      }
    } else if (one_round && u_lead) {
      qv_pre = __ldcg(B.pcg_q + u_i);  // in flight while warp 0 sums
    }
    __syncthreads();
    const double pq = sc[0], alpha = sc[1];
    const bool good = pq > 0.0 && isfinite(pq);  // else S is not positive definite along p_k
    if (!good) {                                  // the PCG ends with x_k
      if (k == 0) linear_ok = false;
      break;
    }
    if (one_round) {
      if (u_lead) {
        if (t < 32) qv_pre = __ldcg(B.pcg_q + u_i);
        up = k == 0 ? uz : fma(beta, up, uz);  // p_k from p_{k-1}
        ux = fma(alpha, up, ux);
        ur = fma(-alpha, qv_pre, ur);
        rv[t] = ur;
      }
      __syncthreads();
      if (u_in) {
        double rz = 0.0, rr = 0.0, qx = 0.0;
        if (u_lead) {
          double zz = 0;
#pragma unroll
          for (int kk = 0; kk < 9; ++kk) zz += umrow[kk] * rv[t - u_q + kk];
          uz = zz;
          pbuf(k)[u_i] = up;
          B.pcg_z[u_i] = uz;
          rz = ur * uz, rr = ur * ur, qx = ux * (uv + ur);
        }
        // the block's r.z, r.r, x.(v + r): butterflies in its three warps,
        // then the warps in order
        rz = warp_sum(rz), rr = warp_sum(rr), qx = warp_sum(qx);
        if (lane == 0) red3[warp][0] = rz, red3[warp][1] = rr, red3[warp][2] = qx;
      }
      __syncthreads();
      if (u_m < 3 && u_in) {
        double b = 0.0;
        for (int ww = 0; ww < 3; ++ww) b += red3[3 * u_slot + ww][u_m];
        B.blk_red[3 * (size_t)(kb0 + u_slot) + u_m] = b;
      }
    } else {
      // more owned blocks than one round: the state from L2, round by round
      for (int kb = kb0; kb < kb1; kb += kGBlksPerRound) {
        const int slot = u_slot, m = u_m;
        const int blk = kb + slot;
        const bool in = slot < kGBlksPerRound && blk < kb1;  // uniform over the slot's three warps
        int4 cbk = make_int4(0, 0, 0, 0);
        if (in) cbk = B.camblk[blk];
        const int lc = u_lc, q = u_q;
        const bool lead = in && m < 9 * kPcgBlockCams && lc < cbk.z;
        const int c = cbk.y + (lead ? lc : 0);
        const size_t i = 9 * (size_t)c + q;
        double x = 0.0, r = 0.0, z = 0.0, v = 0.0, pp = 0.0;
        if (lead) {
          const double *M = B.cam_Minv + 81 * (size_t)c + 9 * q;
#pragma unroll
          for (int kk = 0; kk < 9; ++kk) umrow[kk] = M[kk];
          x = B.pcg_x[i];
          r = B.pcg_r[i];
          z = B.pcg_z[i];
          v = B.pcg_v[i];
          pp = k == 0 ? z : fma(beta, __ldcg(pprev + i), z);
          const double qv = __ldcg(B.pcg_q + i);
          x = fma(alpha, pp, x);
          r = fma(-alpha, qv, r);
          rv[t] = r;
        }
        __syncthreads();
        if (in) {
          double rz = 0.0, rr = 0.0, qx = 0.0;
          if (lead) {
            double zz = 0;
#pragma unroll
            for (int kk = 0; kk < 9; ++kk) zz += umrow[kk] * rv[t - q + kk];
            z = zz;
            pbuf(k)[i] = pp;
            B.pcg_x[i] = x;
            B.pcg_r[i] = r;
            B.pcg_z[i] = z;
            rz = r * z, rr = r * r, qx = x * (v + r);
          }
          rz = warp_sum(rz), rr = warp_sum(rr), qx = warp_sum(qx);
          if (lane == 0) red3[warp][0] = rz, red3[warp][1] = rr, red3[warp][2] = qx;
        }
        __syncthreads();
        if (m < 3 && in) {
          double b = 0.0;
          for (int ww = 0; ww < 3; ++ww) b += red3[3 * slot + ww][m];
          B.blk_red[3 * (size_t)blk + m] = b;
        }
        __syncthreads();
      }
    }
    if (!grid_barrier(B, ++gen, (unsigned)P, &s_ok)) {
      aborted = true;
      break;
    }
    // ---- C. the stopping test on (x_{k+1}, r_{k+1}) and beta_{k+1} (warp 0),
    // while the other warps load z_{k+1} and p_k of the staged columns --------
    constexpr int kPre = 2;
    double zpre[kPre], ppre[kPre];
    if (t < 32) {
      double a3[3] = {0.0, 0.0, 0.0};
      for (int bb = t; bb < nblk; bb += 32) {
        const double *bv = B.blk_red + 3 * (size_t)(pi.cam_block_begin + bb);
        a3[0] += __ldcg(bv), a3[1] += __ldcg(bv + 1), a3[2] += __ldcg(bv + 2);
      }
      a3[0] = warp_sum(a3[0]), a3[1] = warp_sum(a3[1]), a3[2] = warp_sum(a3[2]);
      if (t == 0) {
        const double rz1 = a3[0], rr1 = a3[1], qk = -a3[2];  // Q(x) = x'Sx - 2 v'x = -x.(v + r)
        const int k1 = k + 1;
        bool stop = false;
        if (o.pcg_criterion == GBA_PCG_QUADRATIC_MODEL) {
          const double lhs = k1 * (qk - q0), rhs = o.eta * qk;
          const bool below = qk > 0.0 ? lhs < rhs : (qk < 0.0 ? lhs > rhs : q0 > 0.0);
          if (below && k1 >= o.min_pcg_iterations) stop = true;
        } else {
          if (rr1 <= lim * lim && k1 >= o.min_pcg_iterations) stop = true;
        }
        if (k1 >= o.max_pcg_iterations) stop = true;
        if (!(rz1 != 0.0 && isfinite(rz1))) stop = true;
        sc[0] = rz1 * recip_nr(rz_k);  // beta_{k+1}
        sc[1] = rz1;
        sc[2] = rr1;
        sc[3] = qk;
        s_stop = stop ? 1 : 0;
      }
    } else if (staged) {
      const double *pk = pbuf(k);
#pragma unroll
      for (int u = 0; u < kPre; ++u) {
        const int e = (t - 32) + u * (kGThreads - 32);
        zpre[u] = ppre[u] = 0.0;
        if (e < 9 * nbo) {
          const size_t gi = 9 * (size_t)scol[e / 9] + e % 9;
          zpre[u] = __ldcg(B.pcg_z + gi);
          ppre[u] = __ldcg(pk + gi);
        }
      }
    }
    __syncthreads();
    beta = sc[0];
    rz_k = sc[1];
    last_rr = sc[2];
    q0 = sc[3];
    last_pq = pq;
    ++k;
    const bool stop = s_stop != 0;
    if (stop) break;
    // p_k = z_k + beta_k p_{k-1} at the staged columns
    if (staged) {
      if (t >= 32) {
#pragma unroll
        for (int u = 0; u < kPre; ++u) {
          const int e = (t - 32) + u * (kGThreads - 32);
          if (e < 9 * nbo) pst[e] = fma(beta, ppre[u], zpre[u]);
        }
      }
      for (int e = kPre * (kGThreads - 32) + t; e < 9 * nbo; e += kGThreads) {  // beyond the prefetched ones
        const size_t gi = 9 * (size_t)scol[e / 9] + e % 9;
        pst[e] = fma(beta, __ldcg(pbuf(k + 1) + gi), __ldcg(B.pcg_z + gi));
      }
    }
    __syncthreads();  // the staged direction; sc and s_stop are written again in the next iteration
  }
  // the owned coordinates' x and r, and the last direction in pcg_p, as the
  // two-kernel form leaves them
  if (!aborted) {
    if (one_round) {
      if (u_lead) {
        B.pcg_x[u_i] = ux;
        B.pcg_r[u_i] = ur;
        if (k > 0) B.pcg_p[u_i] = up;
      }
    } else if (k > 0 && ((k - 1) & 1) == 1) {
      for (int kb = kb0; kb < kb1; ++kb) {
        const int4 cbk = B.camblk[kb];
        for (int e = t; e < 9 * cbk.z; e += kGThreads) {
          const size_t i = 9 * (size_t)cbk.y + e;
          B.pcg_p[i] = B.pcg_p2[i];
        }
      }
    }
  }
  if (w == 0 && t == 0) {
    L->pcg_iterations = k;
    if (!linear_ok) L->linear_ok = 0;
    if (k > 0) {
      L->beta = beta;
      L->rz = rz_k;
      L->rr = last_rr;
      L->q0 = q0;
      L->pq = last_pq;
    }
    L->pcg_active = 0;
    if (aborted) {
      // a wait ran out: the solve stops here with GBA_ERR_TIMEOUT
      L->linear_ok = 0;
      L->active = 0;
    }
  }
}

bool pcg_grid_plan(int num_problems, bool mixed, bool explicit_schur, int nc, const int32_t *sblk_row,
                   GridPlan *plan) {
  *plan = GridPlan();
  if (num_problems != 1 || mixed || !explicit_schur || nc <= 0 || !sblk_row) return false;
  int dev = 0, sms = 0, optin = 0;
  cudaFuncAttributes fa;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, k_pcg_grid) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  // one CTA per SM, and no more CTAs than cameras
  const int grid = std::max(1, std::min(sms, nc));
  // the kernel's split (all CTAs registered): the most blocks a CTA owns
  const long long wtot = (long long)(sblk_row[nc] - sblk_row[0]) + nc;
  int most = 0, a = 0;
  for (int r = 0; r < grid; ++r) {
    const long long tb = ((long long)(r + 1) * wtot + grid - 1) / grid;
    int b = a;
    while (b < nc && (long long)(sblk_row[b] - sblk_row[0]) + b < tb) ++b;
    most = std::max(most, (int)(sblk_row[b] - sblk_row[a]) + (b - a));
    a = b;
  }
  const size_t static_bytes = fa.sharedSizeBytes + 1024;  // the kernel's static shared memory, with margin
  int cap = most + most / 4 + 8;  // room for a few CTAs fewer than launched
  const bool cache = grid_smem(cap, true).total + static_bytes <= (size_t)optin;
  while (!cache && cap > most && grid_smem(cap, false).total + static_bytes > (size_t)optin) cap = cap * 3 / 4;
  if (!cache && grid_smem(cap, false).total + static_bytes > (size_t)optin) cap = 0;
  const size_t smem = grid_smem(cap, cache).total;
  if (cudaFuncSetAttribute(k_pcg_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_grid, kGThreads, smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return false;
  }
  plan->grid = grid;
  plan->cap_blocks = cap;
  plan->cache_s = cache ? 1 : 0;
  plan->smem = smem;
  return true;
}

cudaError_t launch_pcg_grid(const DeviceBatch &b, const GridPlan &plan, cudaStream_t s) {
  if (plan.grid <= 0) return cudaSuccess;
  k_pcg_grid<<<plan.grid, kGThreads, plan.smem, s>>>(b, plan.cap_blocks, plan.cache_s);
  return cudaGetLastError();
}

}  // namespace gba
