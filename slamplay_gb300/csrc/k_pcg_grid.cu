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
//   A. q = S p_k for the rows the CTA owns (runs of about equal numbers of
//      row blocks of S): p_k = z_k + beta_k p_{k-1} at the columns of the
//      touched cameras' blocks staged in shared memory; a thread per (row,
//      block) pair of the owned rows (a nine-column FMA chain), each row's
//      block dots summed by the pairwise tree (the additions of each tree
//      level listed once per launch and spread over all threads); each
//      row's p_i q_i.                                           barrier
//   B. every CTA: each camera's p.q (sum9_tree of its rows), their sum
//      (chunks of 32 and a tree), alpha; for the camera blocks (8 cameras)
//      the CTA owns: p_k, x, r, z = M r, each block's r.z, r.r, x.(v + r).
//                                                                barrier
//   C. in every CTA: the stopping test and beta_{k+1} from the blocks'
//      values (three warps, one sum each), while the other warps load what
//      the next iteration's staged direction needs.
// The touched cameras' blocks of S stay in shared memory for the launch (S
// is fixed during the PCG) when they fit; a CTA with more than the layout
// holds reads them from L2.  GB300's FP64 pipe retires about one warp
// instruction per 64 clocks per SM sub-partition, so the work is split by
// rows (not cameras) for an even load over the CTAs and spread over all 16
// warps of a CTA, and the direction is formed once per (block, column), not
// once per row.
// Every CTA takes the same decisions from the same values, so all reach the
// same barriers.  The arithmetic is the two-kernel FP64 PCG's, operation
// for operation (the fixed trees of kernels.cuh, k_schur.cu's product and
// the camera kernel's reductions), so both forms give the same bits, and no
// result depends on how many CTAs took part.
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
constexpr int kGMaxOwn = 64;    // touched cameras a CTA's shared-memory layout indexes
constexpr int kGRows = 64;      // rows of one pass of the product (tables in shared memory)
constexpr int kGLevels = 24;    // levels of the pairwise tree (rows of up to 2^24 blocks)
constexpr int kGBlkSlot = 96;   // threads per camera block in the update (3 warps)
constexpr int kGBlksPerRound = kGThreads / kGBlkSlot;
constexpr int kGPreThreads = kGThreads - 96;  // threads that prefetch while warps 0-2 decide
static_assert(kGBlksPerRound >= 1 && kGThreads % 32 == 0 && kGWarps >= 4, "whole warps, at least one slot");
static_assert(kGBlkSlot % 32 == 0, "block slots of whole warps");
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
// increment by the CTA barrier (causality order is transitive: CTA barrier,
// then the gpu-scope release, the other CTA's gpu-scope acquire, its CTA
// barrier), so no separate fence is needed on either side; after thread 0's
// acquire wait and the CTA barrier every thread reads the other CTAs'
// writes (with __ldcg: L2, not a stale L1 line).
// Returns false (in every thread) when the wait ran out or was aborted.
__device__ __forceinline__ bool grid_barrier(const DeviceBatch &B, unsigned gen, unsigned P, int *s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned *bar = B.grid_ctl + kGridBar;
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
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

// Dynamic shared memory: the rows of the block-Jacobi inverse of the
// update's coordinates (one row per thread), the cameras' p.q chunk sums,
// per touched camera its first block (boff, the diagonal block last in each
// camera's run), per touched block its column camera, its 81 values (when
// cached) and the direction at its nine columns; for the product's pass
// (at most kGRows rows, cap_pairs (row, block) pairs): each pair's dot and
// (row, block), each row's first pair, the tree's additions by level.
struct GridSmem {
  size_t mrow, chs, boff, scol, sval, pst, pd, pinfo, ldst, roff, lbeg, total;
};
__host__ __device__ inline size_t grid_align(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline GridSmem grid_smem(int n, int cap_blocks, bool cache_s, int cap_pairs) {
  GridSmem l;
  size_t o = 0;
  l.mrow = o, o = grid_align(o + 8 * 9 * (size_t)kGThreads);
  l.chs = o, o = grid_align(o + 8 * (size_t)((n + 31) / 32 + 1));
  l.boff = o, o = grid_align(o + 4 * (size_t)(kGMaxOwn + 1));
  l.scol = o, o = grid_align(o + 4 * (size_t)cap_blocks);
  l.sval = o, o = grid_align(o + (cache_s ? 8 * 81 * (size_t)cap_blocks : 0));
  l.pst = o, o = grid_align(o + 8 * 9 * (size_t)cap_blocks);
  l.pd = o, o = grid_align(o + 8 * (size_t)cap_pairs);
  l.pinfo = o, o = grid_align(o + 4 * (size_t)cap_pairs);
  l.ldst = o, o = grid_align(o + 4 * (size_t)cap_pairs);
  l.roff = o, o = grid_align(o + 4 * (size_t)(kGRows + 1));
  l.lbeg = o, o = grid_align(o + 4 * (size_t)(kGLevels + 1));
  l.total = o;
  return l;
}

// The rows of a CTA: row rho (camera rho / 9, row rho % 9 of the problem)
// costs the camera's blocks m_c (off-diagonal + diagonal); the 9 n rows are
// cut into P runs of about equal cost.  Rows of camera c before the cost
// bound t: min(9, ceil((t - 9 before_c) / m_c)), 0 when t <= 9 before_c.
__host__ __device__ inline int rows_below(long long t, long long before9, long long m) {
  if (t <= before9) return 0;
  const long long r = (t - before9 + m - 1) / m;
  return r > 9 ? 9 : (int)r;
}

}  // namespace

__global__ void __launch_bounds__(kGThreads, 1) k_pcg_grid(DeviceBatch B, int cap_blocks, int cache_s,
                                                         int cap_pairs) {
  extern __shared__ __align__(16) unsigned char g_smem[];
  __shared__ int s_ticket, s_P, s_ok, s_ra, s_rb, s_stop, s_pass_end, s_npairs, s_nlev, s_good;
  __shared__ double sc[4], s_inv_rz;
  __shared__ double tot3[3];
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
    s_ra = 0;
    s_rb = 0;
  }
  __syncthreads();
  const int w = s_ticket, P = s_P;
  if (w < 0) return;  // arrived after the closing (or the closing never came)

  // ---- ownership -------------------------------------------------------------
  // product: the problem's rows in P runs of about equal cost (rows_below)
  const int n = pi.cam_count, c0 = pi.cam_begin;
  const int r0 = B.sblk_row[c0];
  {
    const long long wtot = (long long)(B.sblk_row[c0 + n] - r0) + n;
    const long long ta = ((long long)w * 9 * wtot + P - 1) / P, tb = ((long long)(w + 1) * 9 * wtot + P - 1) / P;
    int a = 0, b = 0;
    for (int c = t; c < n; c += kGThreads) {
      const long long before = (long long)(B.sblk_row[c0 + c] - r0) + c;
      const long long m = (long long)(B.sblk_row[c0 + c + 1] - B.sblk_row[c0 + c]) + 1;
      a += rows_below(ta, 9 * before, m);
      b += rows_below(tb, 9 * before, m);
    }
    if (a) atomicAdd(&s_ra, a);
    if (b) atomicAdd(&s_rb, b);
  }
  // update: camera blocks in P equal runs
  const int nblk = pi.cam_block_count;
  const int kb0 = pi.cam_block_begin + (int)((long long)w * nblk / P);
  const int kb1 = pi.cam_block_begin + (int)((long long)(w + 1) * nblk / P);
  __syncthreads();
  const int ra = s_ra, rb = s_rb, own_rows = rb - ra;  // rows of the problem (local)
  const int cA = ra / 9, cB = own_rows > 0 ? (rb - 1) / 9 : cA - 1;  // touched cameras (local)
  const int ntc = cB - cA + 1;
  const double *vals = reinterpret_cast<const double *>(B.sblk_val);
  const double *Sii = reinterpret_cast<const double *>(B.cam_Sii);
  // the touched blocks in shared memory: staged directions (and cached
  // values) when they fit the layout, else everything from L2
  const GridSmem lay = grid_smem(n, cap_blocks, cache_s != 0, cap_pairs);
  double *chs = reinterpret_cast<double *>(g_smem + lay.chs);
  int *boff = reinterpret_cast<int *>(g_smem + lay.boff);
  int *scol = reinterpret_cast<int *>(g_smem + lay.scol);
  double *sval = reinterpret_cast<double *>(g_smem + lay.sval);
  double *pst = reinterpret_cast<double *>(g_smem + lay.pst);
  double *pd = reinterpret_cast<double *>(g_smem + lay.pd);
  int *pinfo = reinterpret_cast<int *>(g_smem + lay.pinfo);
  int *ldst = reinterpret_cast<int *>(g_smem + lay.ldst);
  int *roff = reinterpret_cast<int *>(g_smem + lay.roff);
  int *lbeg = reinterpret_cast<int *>(g_smem + lay.lbeg);
  const int nbo = ntc > 0 ? (B.sblk_row[c0 + cB + 1] - B.sblk_row[c0 + cA]) + ntc : 0;
  const bool staged = ntc <= kGMaxOwn && nbo <= cap_blocks;
  const bool cached = staged && cache_s != 0;
  if (staged) {
    if (t <= ntc) boff[t] = B.sblk_row[c0 + cA + t] - B.sblk_row[c0 + cA] + t;
    __syncthreads();
    for (int lc = 0; lc < ntc; ++lc) {
      const int c = c0 + cA + lc;
      const int rr0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - rr0, b0 = boff[lc];
      for (int v = t; v <= nb; v += kGThreads) scol[b0 + v] = v < nb ? B.sblk_col[rr0 + v] : c;
      if (cached)
        for (int e = t; e < 81 * (nb + 1); e += kGThreads) {
          const int v = e / 81, el = e - 81 * v;
          sval[81 * (size_t)(b0 + v) + el] = v < nb ? vals[81 * (size_t)(rr0 + v) + el] : Sii[81 * (size_t)c + el];
        }
    }
    __syncthreads();
  }
  // The product's pass over local rows [rl0, s_pass_end): at most kGRows rows
  // and cap_pairs (row, block) pairs; its tables: each row's first pair
  // (roff), each pair's (row, block) (pinfo), the tree's additions of each
  // level (their destinations, ldst[lbeg[L] ..]).
  auto row_m = [&](int rl) -> int {
    const int c = c0 + (ra + rl) / 9;
    return B.sblk_row[c + 1] - B.sblk_row[c] + 1;
  };
  auto build_pass = [&](int rl0) {
    if (t == 0) {
      int rl = rl0, np = 0, mx = 1;
      roff[0] = 0;
      while (rl < own_rows && rl - rl0 < kGRows) {
        const int m = row_m(rl);
        if (rl > rl0 && np + m > cap_pairs) break;
        np += m;
        mx = max(mx, m);
        roff[rl - rl0 + 1] = np;
        ++rl;
      }
      int nl = 0;
      while ((1 << nl) < mx) ++nl;
      int o = 0;
      for (int L2 = 0; L2 < nl; ++L2) {
        lbeg[L2] = o;
        for (int j = 0; j < rl - rl0; ++j) o += tree_adds(roff[j + 1] - roff[j], 1 << L2);
      }
      lbeg[nl] = o;
      s_pass_end = rl, s_npairs = np, s_nlev = nl;
    }
    __syncthreads();
    const int nr = s_pass_end - rl0, nl = s_nlev;
    for (int j = 0; j < nr; ++j)
      for (int v = t; v < roff[j + 1] - roff[j]; v += kGThreads) pinfo[roff[j] + v] = (j << 20) | v;
    for (int L2 = 0; L2 < nl; ++L2) {
      const int sp = 1 << L2, base = lbeg[L2], cnt = lbeg[L2 + 1] - base;
      for (int kk = t; kk < cnt; kk += kGThreads) {
        int j = 0, acc = 0;
        for (;;) {
          const int a = tree_adds(roff[j + 1] - roff[j], sp);
          if (kk < acc + a) break;
          acc += a;
          ++j;
        }
        ldst[base + kk] = roff[j] + 2 * sp * (kk - acc);
      }
    }
    __syncthreads();
  };
  bool one_pass = true;
  if (own_rows > 0) {
    build_pass(0);
    one_pass = s_pass_end == own_rows;
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
  // CTAs a barrier waits for (one more under the wait-runs-out test)
  const unsigned bar_n = (unsigned)P + (B.opt.grid_wait_test ? 1u : 0u);

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
  // the staged direction of the touched blocks' columns: p_0 = z_0
  if (staged) {
    for (int e = t; e < 9 * nbo; e += kGThreads) {
      const int bl = e / 9, cc = e - 9 * bl;
      pst[e] = __ldcg(B.pcg_z + 9 * (size_t)scol[bl] + cc);
    }
  }
  __syncthreads();
  for (;;) {
    // ---- A. q = S p_k for the owned rows, each row's p_i q_i ---------------
    const double *pprev = pbuf(k + 1);  // p_{k-1}
    auto pdir = [&](size_t idx) -> double {
      const double z = __ldcg(B.pcg_z + idx);
      if (k == 0) return z;
      return fma(beta, __ldcg(pprev + idx), z);
    };
    for (int rl0 = 0; rl0 < own_rows;) {
      if (!one_pass) build_pass(rl0);
      const int pend = one_pass ? own_rows : s_pass_end, np = s_npairs, nl = s_nlev;
      // the pairs' block dots (nine-column FMA chains)
      for (int e = t; e < np; e += kGThreads) {
        const int j = pinfo[e] >> 20, v = pinfo[e] & 0xfffff;
        const int rho = ra + rl0 + j, cl = rho / 9, q = rho - 9 * cl, c = c0 + cl;
        double d = 0.0;
        if (staged) {
          const int b0 = boff[cl - cA], nb = boff[cl - cA + 1] - b0 - 1;
          const double *row = cached ? sval + 81 * (size_t)(b0 + v) + 9 * q
                                     : (v < nb ? vals + 81 * (size_t)(B.sblk_row[c] + v) : Sii + 81 * (size_t)c) + 9 * q;
          const double *pp = pst + 9 * (b0 + v);
#pragma unroll
          for (int cc = 0; cc < 9; ++cc) d = fma(row[cc], pp[cc], d);
        } else {
          const int rr0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - rr0;
          const double *row = (v < nb ? vals + 81 * (size_t)(rr0 + v) : Sii + 81 * (size_t)c) + 9 * q;
          const int col = v < nb ? B.sblk_col[rr0 + v] : c;
#pragma unroll
          for (int cc = 0; cc < 9; ++cc) d = fma(row[cc], pdir(9 * (size_t)col + cc), d);
        }
        pd[e] = d;
      }
      __syncthreads();
      // each row's pairwise tree, level by level
      for (int L2 = 0; L2 < nl; ++L2) {
        const int sp = 1 << L2;
        for (int kk = lbeg[L2] + t; kk < lbeg[L2 + 1]; kk += kGThreads) {
          const int dst = ldst[kk];
          pd[dst] += pd[dst + sp];
        }
        __syncthreads();
      }
      if (t < pend - rl0) {
        const int rho = ra + rl0 + t, cl = rho / 9, q = rho - 9 * cl, c = c0 + cl;
        const size_t i = 9 * (size_t)c + q;
        const double qv = pd[roff[t]];
        // p_k at the row's own coordinate: the diagonal block's column
        const double pk = staged ? pst[9 * (boff[cl - cA + 1] - 1) + q] : pdir(i);
        B.pcg_q[i] = qv;
        B.pq_row[(size_t)q * n + cl] = pk * qv;  // row-major by row index: a camera's rows n apart
      }
      __syncthreads();  // pd and the pass tables are used again
      rl0 = pend;
    }
    if (!grid_barrier(B, ++gen, bar_n, &s_ok)) {
      aborted = true;
      break;
    }
    // ---- B. each camera's p.q (sum9_tree), their sum (chunks of 32 and the
    // pairwise tree: cta_chunked_sum's order), alpha; the update ---------------
    double qv_pre = 0.0, up_k = 0.0;
    if (one_round && u_lead) {
      qv_pre = __ldcg(B.pcg_q + u_i);         // in flight while the cameras are summed
      up_k = k == 0 ? uz : fma(beta, up, uz);  // p_k from p_{k-1} (alpha not needed)
    }
    {
      const int nch = (n + 31) / 32;
      for (int j = warp; j < nch; j += kGWarps) {
        const int c = 32 * j + lane;
        double x = 0.0;
        if (c < n) {
          double x9[9];  // coalesced over the lanes' cameras
#pragma unroll
          for (int r = 0; r < 9; ++r) x9[r] = __ldcg(B.pq_row + (size_t)r * n + c);
          x = sum9_tree(x9);
        }
        x = warp_sum(x);
        if (lane == 0) chs[j] = x;
      }
      if (nch == 0 && t == 0) chs[0] = 0.0;
      __syncthreads();
      if (nch <= 32) {  // the tree by one warp's shuffles (no barrier per level)
        if (warp == 0) {
          const double s2 = warp_pairwise_tree(lane < nch ? chs[lane] : 0.0, nch);
          if (lane == 0) sc[0] = s2, sc[1] = rz_k * recip_nr(s2), s_good = s2 > 0.0 && isfinite(s2);
        }
      } else {
        cta_pairwise_tree(chs, nch);
        if (t == 0) {
          const double s2 = chs[0];
          sc[0] = s2;
          sc[1] = rz_k * recip_nr(s2);
          s_good = s2 > 0.0 && isfinite(s2);
        }
      }
      __syncthreads();
    }
    const double pq = sc[0], alpha = sc[1];
    // pq > 0 and finite, tested once (else S is not positive definite along
    // p_k): an FP64 comparison in every warp would queue on the FP64 pipes
    const bool good = s_good != 0;
    if (!good) {                                  // the PCG ends with x_k
      if (k == 0) linear_ok = false;
      break;
    }
    if (one_round) {
      if (u_lead) {
        up = up_k;
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
        warp_sum3(rz, rr, qx);
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
          warp_sum3(rz, rr, qx);
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
    if (!grid_barrier(B, ++gen, bar_n, &s_ok)) {
      aborted = true;
      break;
    }
    // ---- C. the stopping test on (x_{k+1}, r_{k+1}) and beta_{k+1}: warp j < 3
    // sums quantity j over the blocks (the camera kernel's order), while the
    // other warps load z_{k+1} and p_k of the staged columns ------------------
    constexpr int kPre = 2;
    double zpre[kPre], ppre[kPre];
    if (warp < 3) {
      double a = 0.0;
      for (int bb = lane; bb < nblk; bb += 32) a += __ldcg(B.blk_red + 3 * (size_t)(pi.cam_block_begin + bb) + warp);
      a = warp_sum(a);
      if (lane == 0) tot3[warp] = a;
    } else {
      if (staged) {
        const double *pkb = pbuf(k);
#pragma unroll
        for (int u = 0; u < kPre; ++u) {
          const int e = (t - 96) + u * kGPreThreads;
          zpre[u] = ppre[u] = 0.0;
          if (e < 9 * nbo) {
            const size_t gi = 9 * (size_t)scol[e / 9] + e % 9;
            zpre[u] = __ldcg(B.pcg_z + gi);
            ppre[u] = __ldcg(pkb + gi);
          }
        }
      }
      // 1 / r_k.z_k for beta, off the deciding warps' dependent chain
      if (t == 96) s_inv_rz = recip_nr(rz_k);
    }
    __syncthreads();
    if (t == 0) {
      const double rz1 = tot3[0], rr1 = tot3[1], qk = -tot3[2];  // Q(x) = x'Sx - 2 v'x = -x.(v + r)
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
      sc[0] = rz1 * s_inv_rz;  // beta_{k+1} (the reciprocal as recip_nr(rz_k))
      sc[1] = rz1;
      sc[2] = rr1;
      sc[3] = qk;
      s_stop = stop ? 1 : 0;
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
      if (t >= 96) {
#pragma unroll
        for (int u = 0; u < kPre; ++u) {
          const int e = (t - 96) + u * kGPreThreads;
          if (e < 9 * nbo) pst[e] = fma(beta, ppre[u], zpre[u]);
        }
      }
      for (int e = kPre * kGPreThreads + t; e < 9 * nbo; e += kGThreads) {  // beyond the prefetched ones
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

bool pcg_grid_plan(int num_problems, bool mixed, bool explicit_schur, int nc, const int32_t *sblk_row, int ctas,
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
  // one CTA per SM at most, and no more CTAs than rows
  const int grid = std::max(1, std::min(ctas > 0 ? std::min(ctas, sms) : sms, 9 * nc));
  // the kernel's split of the rows (all CTAs registered): the most blocks of
  // touched cameras a CTA stages, the most touched cameras, the most (row,
  // block) pairs, the longest row
  const long long wtot = (long long)(sblk_row[nc] - sblk_row[0]) + nc;
  auto m_of = [&](int c) { return (long long)(sblk_row[c + 1] - sblk_row[c]) + 1; };
  auto rows_before = [&](long long tb) {
    long long r = 0;
    for (int c = 0; c < nc; ++c) r += rows_below(tb, 9 * ((long long)(sblk_row[c] - sblk_row[0]) + c), m_of(c));
    return r;
  };
  long long most = 0, most_pairs = 0, m_max = 0;
  int most_cams = 0;
  for (int c = 0; c < nc; ++c) m_max = std::max(m_max, m_of(c));
  long long ra = 0;
  for (int r = 0; r < grid; ++r) {
    const long long rb = rows_before(((long long)(r + 1) * 9 * wtot + grid - 1) / grid);
    if (rb > ra) {
      const int cA = (int)(ra / 9), cB = (int)((rb - 1) / 9);
      most = std::max(most, (long long)(sblk_row[cB + 1] - sblk_row[cA]) + (cB - cA + 1));
      most_cams = std::max(most_cams, cB - cA + 1);
      long long pairs = 0;
      for (long long rho = ra; rho < rb; ++rho) pairs += m_of((int)(rho / 9));
      most_pairs = std::max(most_pairs, pairs);
    }
    ra = rb;
  }
  const size_t static_bytes = fa.sharedSizeBytes + 1024;  // the kernel's static shared memory, with margin
  auto fits = [&](int cap, bool cache, int pairs) { return grid_smem(nc, cap, cache, pairs).total + static_bytes <= (size_t)optin; };
  // room for a few CTAs fewer than launched; a pass holds one whole row at least
  int cap_pairs = (int)std::max<long long>(m_max, most_pairs + most_pairs / 4 + 64);
  while (cap_pairs > m_max && !fits(0, false, cap_pairs)) cap_pairs = std::max<int>((int)m_max, cap_pairs * 3 / 4);
  if (!fits(0, false, cap_pairs)) return false;
  int cap = most_cams <= kGMaxOwn ? (int)(most + most / 4 + 16) : 0;
  const bool cache = cap > 0 && fits(cap, true, cap_pairs);
  // the form pays off while every CTA keeps its blocks of S in shared memory
  // for the launch; a complement too large for that is streamed from memory
  // on every PCG iteration, which the two-kernel product (a CTA per camera
  // row, the blocks loaded ahead of the wait) does better (1,800 cameras,
  // 5.8M observations: 85 us per PCG iteration against 378 us here)
  if (!cache) return false;
  const size_t smem = grid_smem(nc, cap, cache, cap_pairs).total;
  if (raise_smem_limit((const void *)k_pcg_grid, smem) != cudaSuccess) {
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
  plan->cap_pairs = cap_pairs;
  plan->smem = smem;
  return true;
}

cudaError_t launch_pcg_grid(const DeviceBatch &b, const GridPlan &plan, cudaStream_t s) {
  if (plan.grid <= 0) return cudaSuccess;
  k_pcg_grid<<<plan.grid, kGThreads, plan.smem, s>>>(b, plan.cap_blocks, plan.cache_s, plan.cap_pairs);
  return cudaGetLastError();
}

}  // namespace gba
