// k_pcg.cu — implicit-Schur preconditioned conjugate gradients on the
// reduced camera system  S x = v,  S = B + Dc^2 - W C^-1 W^T,  with the
// block-Jacobi preconditioner M = blockdiag(S_ii)^-1 (built by K3b).
//
// The PCG is the Chronopoulos-Gear single-reduction form of preconditioned
// CG: the same iterates as the textbook recurrence in exact arithmetic, but
// the mat-vec is applied to the preconditioned residual u = M r and both dot
// products of an iteration come from one reduction, so the camera side needs
// one cluster barrier per iteration instead of two:
//   w_k = S u_k;  gamma_k = r_k.u_k;  delta_k = u_k.w_k;
//   beta_k = gamma_k / gamma_{k-1};  alpha_k = gamma_k / (delta_k - beta_k gamma_k / alpha_{k-1})
//   (k = 0: beta = 0, alpha = gamma / delta);
//   p_k = u_k + beta_k p_{k-1};  s_k = w_k + beta_k s_{k-1}  (s = S p);
//   x_{k+1} = x_k + alpha_k p_k;  r_{k+1} = r_k - alpha_k s_k;  u_{k+1} = M r_{k+1}.
// The stopping test of call k looks at r_k and x_k (residual ratio, or Ceres'
// quadratic-model test on Q(x_k) = -x_k.(v + r_k)), i.e. one mat-vec after
// the textbook loop would have tested them; x is only updated when the loop
// goes on, so the returned x_k is the same iterate.
//
// One PCG iteration is two kernels:
//   K4a k_schur_matvec  mat-vec over point-segment chunks (one CTA per chunk,
//       one thread per observation): y = J_p^T J_c u, t_j = C_j^-1 sum_j y,
//       J_c^T J_p t_j written at the observation's slot in the chunk's
//       camera-sorted order, summed per camera run into one partial per
//       (chunk, camera), stored at the camera's contiguous (camera-major)
//       position.  No global atomics; every sum has a fixed order.
//   K4b k_pcg_camera    everything on the camera side, one thread-block
//       cluster per problem (up to 16 CTAs, one thread per camera
//       coordinate): w = (B + Dc^2) u - sum of the camera's partials; the
//       four dot products r.u, u.w, r.r, x.(v + r) in one cluster
//       reduction; stopping test; alpha, beta; p, s, x, r, u = M r.
// GB300 runs FP64 at 1/55 of FP32 throughput and with 64-cycle dependent
// latency, so in the mixed form the matrix-like inner work (partial sums,
// (B + Dc^2) u, M r) runs in FP32 with compensated sums while the vectors
// x, r, u, p, s and every dot product stay FP64.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace gba {

namespace {

template <bool MIXED>
struct MatvecSmem {
  typedef typename Prec<MIXED>::real real;
  real pseg[kChunkCap][9];
  real U[kChunkCap][9];  // first holds w (3 per obs), then u (9 per slot)
  real tpt[kChunkCap][3];
};

__device__ __forceinline__ bool pcg_live(const LMState *L) { return L->active != 0 && L->pcg_active != 0; }

// Programmatic dependent launch: the two PCG kernels alternate, each launched
// as a dependent of the other, so that one starts (and issues every load that
// does not depend on the other's results) while the other is still running.
// wait: returns once the preceding kernel of the stream has completed and
// its writes are visible (immediately when there is no such dependency).
// A kernel lets its dependent launch only after its own wait has returned:
// the dependent's early loads may then read anything the kernel before the
// preceding one wrote.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

}  // namespace

// ---------------------------------------------------------------------------
// K4a
template <bool MIXED>
__global__ void __launch_bounds__(kChunkCap) k_schur_matvec(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  typedef typename Acc<MIXED>::type Acc;
  __shared__ MatvecSmem<MIXED> sm;
  const int t = threadIdx.x;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x) {
    const ChunkInfo ci = B.chunk[ch];
    const bool valid = t < ci.obs_count;
    // every load that depends only on the chunk is issued before the first
    // barrier, so one memory round trip covers them all
    real2 Jc[9], Jp[3];
    int lp = 0, slot = 0, s = 0;
    if (valid) {
      const int64_t o = ci.obs_begin + t;
#pragma unroll
      for (int q = 0; q < 9; ++q) Jc[q] = jload<real2>(B.jac, B.no, q, o);
#pragma unroll
      for (int q = 0; q < 3; ++q) Jp[q] = jload<real2>(B.jac, B.no, 9 + q, o);
      s = B.obs_seg[o];
      slot = B.obs_slot[o];
      lp = B.obs_pt[o] - ci.pt_begin;
    }
    int pb0 = 0, pb1 = 0;
    real ci6[6] = {0, 0, 0, 0, 0, 0};
    if (t < ci.pt_count) {
      const int jj = ci.pt_begin + t;
      pb0 = B.pt_obs_begin[jj] - ci.obs_begin;
      pb1 = B.pt_obs_begin[jj + 1] - ci.obs_begin;
      const real *Ci = reinterpret_cast<const real *>(B.pt_Cinv) + 6 * (size_t)jj;
#pragma unroll
      for (int q = 0; q < 6; ++q) ci6[q] = Ci[q];
    }
    // the first (segment, coordinate) this thread reduces at the end
    int f_b0 = 0, f_b1 = 0, f_slot = 0;
    if (t < ci.seg_count * 9) {
      const int sg = t / 9;
      f_b0 = B.seg_pos[ci.seg_begin + sg];
      f_b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
      f_slot = B.seg_slot[ci.seg_begin + sg];
    }
    // everything above is fixed during the PCG; from here on the kernel reads
    // what the previous camera-side kernel wrote (and overwrites the partials
    // it read)
    pdl_wait();
    pdl_launch_dependents();
    if (!pcg_live(B.lm + ci.problem)) continue;  // uniform over the CTA
    // stage the vector u of the chunk's cameras
    const real *pdir = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_pf : (const void *)B.pcg_z);
    for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
      const int sg = i / 9, q = i - 9 * sg;
      sm.pseg[sg][q] = pdir[9 * (size_t)B.seg_cam[ci.seg_begin + sg] + q];
    }
    __syncthreads();
    if (valid) {
      real zu = 0, zv = 0;
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const real x = sm.pseg[s][q];
        zu += Jc[q].x * x;
        zv += Jc[q].y * x;
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) sm.U[t][q] = Jp[q].x * zu + Jp[q].y * zv;
    }
    __syncthreads();
    if (t < ci.pt_count) {
      Acc y0, y1, y2;
      y0.init(), y1.init(), y2.init();
      for (int k = pb0; k < pb1; ++k) {
        y0.add(sm.U[k][0]);
        y1.add(sm.U[k][1]);
        y2.add(sm.U[k][2]);
      }
      const real w0 = (real)y0.value(), w1 = (real)y1.value(), w2 = (real)y2.value();
      sm.tpt[t][0] = ci6[0] * w0 + ci6[1] * w1 + ci6[2] * w2;
      sm.tpt[t][1] = ci6[1] * w0 + ci6[3] * w1 + ci6[4] * w2;
      sm.tpt[t][2] = ci6[2] * w0 + ci6[4] * w1 + ci6[5] * w2;
    }
    __syncthreads();
    if (valid) {
      const real t0 = sm.tpt[lp][0], t1 = sm.tpt[lp][1], t2 = sm.tpt[lp][2];
      const real eu = Jp[0].x * t0 + Jp[1].x * t1 + Jp[2].x * t2;
      const real ev = Jp[0].y * t0 + Jp[1].y * t1 + Jp[2].y * t2;
#pragma unroll
      for (int q = 0; q < 9; ++q) sm.U[slot][q] = Jc[q].x * eu + Jc[q].y * ev;
    }
    __syncthreads();
    real *part = reinterpret_cast<real *>(B.seg_partial);
    for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
      const int sg = i / 9, q = i - 9 * sg;
      int b0 = f_b0, b1 = f_b1, slot9 = f_slot;
      if (i != t) {
        b0 = B.seg_pos[ci.seg_begin + sg];
        b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
        slot9 = B.seg_slot[ci.seg_begin + sg];
      }
      Acc a;
      a.init();
      for (int k = b0; k < b1; ++k) a.add(sm.U[k][q]);
      part[9 * (size_t)slot9 + q] = (real)a.value();
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// K4b: one cluster per problem.  A CTA works on camera blocks of
// kPcgBlockCams cameras with one thread per camera coordinate (9 per
// camera); a problem with more blocks than the cluster has CTAs takes
// several passes.
//
// The four problem-wide dot products are summed in a fixed order that
// depends only on the problem's camera count: the per-thread values of a
// block are staged in shared memory and warp 0 adds them (in thread order
// per lane, then a xor butterfly) -- one warp of FP64 additions instead of
// one per warp, since GB300 issues FP64 at a small fraction of its FP32
// rate; the block values are pushed into the shared memory of every CTA of
// the cluster (remote stores, one lane per destination) at the block's
// slot; after the cluster barrier every CTA adds the slots of all blocks in
// block order, strided over the lanes of one warp, and combines them with a
// butterfly.  All CTAs therefore hold the same alpha, beta and stopping
// decision, and the result depends neither on the cluster size nor on the
// other problems of a batch.  After the barrier no CTA touches another
// CTA's shared memory.
//
// The state of the first kPcgRegPasses passes stays in registers across the
// barrier; every load of a pass is issued before it.
constexpr int kPcgThreads = 9 * kPcgBlockCams;
constexpr int kPcgNv = 4;  // r.u, u.w, r.r, x.(v + r)

namespace {

__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// Fixed-order sum of NV values per block slot, slots 0..n-1 of the local
// array blk (slot e at blk[NV * e]).  Called by one whole warp; the sums are
// returned in every lane.
template <int NV>
__device__ __forceinline__ void slots_sum(const double *blk, int n, double *out) {
  const int lane = threadIdx.x & 31;
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = 0.0;
  for (int e = lane; e < n; e += 32) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += blk[NV * e + k];
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = warp_sum(v[k]);
}

// Block value of NV per-thread values v (all threads call it together):
// staged in red[NV][kPcgThreads], summed by warp 0 and pushed to slot b of
// every CTA of the cluster.
template <int NV>
__device__ __forceinline__ void block_push(cg::cluster_group &cl, double (*red)[kPcgThreads], const double *v,
                                           double *slots, int b, int cs) {
  const int tid = threadIdx.x, lane = tid & 31;
#pragma unroll
  for (int k = 0; k < NV; ++k) red[k][tid] = v[k];
  __syncthreads();
  if (tid < 32) {
    constexpr int kWarps = (kPcgThreads + 31) / 32;
    double s[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      s[k] = 0.0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w)
        if (lane + 32 * w < kPcgThreads) s[k] += red[k][lane + 32 * w];
      s[k] = warp_sum(s[k]);
    }
    if (lane < cs) {
      double *dst = cl.map_shared_rank(slots + NV * b, lane);
#pragma unroll
      for (int k = 0; k < NV; ++k) dst[k] = s[k];
    }
  }
  __syncthreads();  // red may be reused
}

// One camera coordinate of a pass.
template <typename real>
struct CamCoord {
  bool valid;
  int c;
  double x, r, u, p, s, v, w;
  real m[9];  // row of the block-Jacobi preconditioner
};

// Phase 1 of one coordinate: loads the pass state, waits for the mat-vec,
// computes w = (B + Dc^2) u - sum of partials and the four dot-product terms.
template <bool MIXED>
__device__ __forceinline__ void pcg_phase1(const DeviceBatch &B, const ProblemInfo &pi, int k, int q, bool first,
                                           CamCoord<typename Prec<MIXED>::real> &st, double *d) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Acc<MIXED>::type Acc;
  d[0] = d[1] = d[2] = d[3] = 0.0;
  st.valid = k < pi.cam_count;
  st.c = pi.cam_begin + (st.valid ? k : 0);
  if (!st.valid) return;
  const int c = st.c;
  const size_t i = 9 * (size_t)c + q;
  const real *Bc = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_Bf : (const void *)B.cam_B) + 45 * (size_t)c;
  const real *uv = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_pf : (const void *)B.pcg_z) + 9 * (size_t)c;
  const real *M = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_Minvf : (const void *)B.cam_Minv) +
                  81 * (size_t)c + 9 * q;
  const real *part = reinterpret_cast<const real *>(B.seg_partial) + q;
  const int s0 = B.cam_seg_begin[c], s1 = B.cam_seg_begin[c + 1];
  st.u = B.pcg_z[i];
  st.x = B.pcg_x[i];
  st.r = B.pcg_r[i];
  st.v = B.pcg_v[i];
  st.p = first ? 0.0 : B.pcg_p[i];
  st.s = first ? 0.0 : B.pcg_q[i];
  const real d2 = (real)B.cam_D2[i];
  real brow[9], urow[9];
#pragma unroll
  for (int kk = 0; kk < 9; ++kk) {
    brow[kk] = Bc[sym9(q, kk)];
    urow[kk] = uv[kk];
    st.m[kk] = M[kk];
  }
  pdl_wait();  // the partials come from the mat-vec kernel
  // the camera's partials: the first kBatch in one round trip, then batches.
  // FP64: four interleaved accumulators (partial s to accumulator
  // (s - s0) % 4) shorten the chain of 64-cycle additions fourfold; mixed:
  // one compensated FP32 sum (its chain is short and each extra accumulator
  // would cost FP64 conversions)
  constexpr int kBatch = MIXED ? 64 : 32;
  constexpr int kAcc = MIXED ? 1 : 4;
  Acc a[kAcc];
#pragma unroll
  for (int uu = 0; uu < kAcc; ++uu) a[uu].init();
  for (int s = s0; s < s1; s += kBatch) {
    real pv2[kBatch];
#pragma unroll
    for (int uu = 0; uu < kBatch; ++uu) pv2[uu] = (s + uu < s1) ? part[9 * (size_t)(s + uu)] : (real)0;
#pragma unroll
    for (int uu = 0; uu < kBatch; ++uu)
      if (s + uu < s1) a[uu % kAcc].add(pv2[uu]);
  }
  double asum = a[0].value();
  if (kAcc == 4) asum = (a[0].value() + a[1 % kAcc].value()) + (a[2 % kAcc].value() + a[3 % kAcc].value());
  real bu = 0;
#pragma unroll
  for (int kk = 0; kk < 9; ++kk) bu += brow[kk] * urow[kk];
  st.w = (double)(bu + d2 * (real)st.u - (real)asum);
  d[0] = st.r * st.u;
  d[1] = st.u * st.w;
  d[2] = st.r * st.r;
  d[3] = st.x * (st.v + st.r);
}

// Phase 2 of one coordinate (all threads of the CTA call it together):
// p, s, x, r and u = M r.
template <bool MIXED>
__device__ __forceinline__ void pcg_phase2(const DeviceBatch &B, int q, int lc, double alpha, double beta,
                                           CamCoord<typename Prec<MIXED>::real> &st,
                                           typename Prec<MIXED>::real *sv, bool sync_before) {
  typedef typename Prec<MIXED>::real real;
  double r = 0.0;
  if (st.valid) {
    st.p = st.u + beta * st.p;
    st.s = st.w + beta * st.s;
    st.x = st.x + alpha * st.p;
    r = st.r - alpha * st.s;
  }
  if (sync_before) __syncthreads();  // the previous pass has finished reading sv
  sv[threadIdx.x] = (real)r;
  __syncthreads();
  if (st.valid) {
    const real *rv = sv + 9 * lc;
    real u = 0;
#pragma unroll
    for (int kk = 0; kk < 9; ++kk) u += st.m[kk] * rv[kk];
    const size_t i = 9 * (size_t)st.c + q;
    B.pcg_p[i] = st.p;
    B.pcg_q[i] = st.s;
    B.pcg_x[i] = st.x;
    B.pcg_r[i] = r;
    B.pcg_z[i] = (double)u;
    if (MIXED) B.pcg_pf[i] = (float)u;
  }
}

}  // namespace

template <bool MIXED>
__global__ void __launch_bounds__(kPcgThreads) k_pcg_camera(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  constexpr int kRegPasses = MIXED ? 2 : 1;
  // slots: [nblk_max][kPcgNv]
  extern __shared__ double blk[];
  __shared__ real sv[kPcgThreads];  // the block's r, staged for u = M r
  __shared__ double red[kPcgNv][kPcgThreads];
  __shared__ double tot[kPcgNv];
  __shared__ int flag;
  cg::cluster_group cl = cg::this_cluster();
  const int cs = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int prob = blockIdx.x / cs;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int lc = tid / 9, q = tid - 9 * lc;  // camera in the block, coordinate
  LMState *L = B.lm + prob;
  if (prob < B.num_problems && pcg_live(L)) {  // uniform over the cluster
    const ProblemInfo pi = B.prob[prob];
    const int nblk = (pi.cam_count + kPcgBlockCams - 1) / kPcgBlockCams;
    // every LMState field this kernel reads is read before the cluster
    // barrier: rank 0 overwrites them after it
    const double gamma_old = L->rz, alpha_old = L->alpha, q_old = L->q0, r0_norm = L->r0_norm;
    const int k = L->pcg_iterations;  // completed iterations = this call's index
    CamCoord<real> st[kRegPasses];
    // ---- w = S u and the four dot products ---------------------------------
#pragma unroll
    for (int j = 0; j < kRegPasses; ++j) {
      const int b = rank + j * cs;
      if (b < nblk) {
        double d[kPcgNv];
        pcg_phase1<MIXED>(B, pi, b * kPcgBlockCams + lc, q, k == 0, st[j], d);
        block_push<kPcgNv>(cl, red, d, blk, b, cs);
      }
    }
    for (int b = rank + kRegPasses * cs; b < nblk; b += cs) {
      CamCoord<real> t;
      double d[kPcgNv];
      pcg_phase1<MIXED>(B, pi, b * kPcgBlockCams + lc, q, k == 0, t, d);
      block_push<kPcgNv>(cl, red, d, blk, b, cs);
      if (t.valid) B.pcg_w[9 * (size_t)t.c + q] = t.w;  // w of passes not held in registers
    }
    pdl_wait();  // every thread, whether or not it had a camera coordinate
    pdl_launch_dependents();
    cluster_arrive();
    cluster_wait();  // after this barrier no CTA touches another's shared memory
    if (warp == 0) {
      double t[kPcgNv];
      slots_sum<kPcgNv>(blk, nblk, t);
      if (lane == 0) {
#pragma unroll
        for (int v = 0; v < kPcgNv; ++v) tot[v] = t[v];
      }
    }
    __syncthreads();
    const double gamma = tot[0], delta = tot[1], rr = tot[2], qx = tot[3];
    // ---- stopping test on (x_k, r_k), then alpha_k, beta_k -----------------
    const DeviceOptions &o = B.opt;
    const double qk = -qx;  // Q(x_k) = x'Sx - 2 v'x = -x.(v + r)
    bool stop = false;
    if (k >= 1) {
      if (o.pcg_criterion == GBA_PCG_QUADRATIC_MODEL) {
        const double zeta = k * (qk - q_old) / qk;
        if (zeta < o.eta && k >= o.min_pcg_iterations) stop = true;
      } else {
        if (sqrt(rr) <= o.pcg_tolerance * r0_norm && k >= o.min_pcg_iterations) stop = true;
      }
    }
    if (k >= o.max_pcg_iterations) stop = true;
    const double beta = k == 0 ? 0.0 : gamma / gamma_old;
    const double denom = k == 0 ? delta : delta - beta * gamma / alpha_old;
    const bool good = denom > 0.0 && isfinite(denom) && isfinite(gamma) && gamma != 0.0;
    if (!good) stop = true;
    const double alpha = good ? gamma / denom : 0.0;
    if (!stop) {
#pragma unroll
      for (int j = 0; j < kRegPasses; ++j) {
        const int b = rank + j * cs;
        if (b < nblk) pcg_phase2<MIXED>(B, q, lc, alpha, beta, st[j], sv, j > 0);
      }
      for (int b = rank + kRegPasses * cs; b < nblk; b += cs) {
        CamCoord<real> t;
        const int kk = b * kPcgBlockCams + lc;
        t.valid = kk < pi.cam_count;
        t.c = pi.cam_begin + (t.valid ? kk : 0);
        if (t.valid) {
          const size_t i = 9 * (size_t)t.c + q;
          const real *M = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_Minvf
                                                               : (const void *)B.cam_Minv) +
                          81 * (size_t)t.c + 9 * q;
          t.u = B.pcg_z[i];
          t.x = B.pcg_x[i];
          t.r = B.pcg_r[i];
          t.w = B.pcg_w[i];  // stored in phase 1
          t.p = k == 0 ? 0.0 : B.pcg_p[i];
          t.s = k == 0 ? 0.0 : B.pcg_q[i];
#pragma unroll
          for (int m = 0; m < 9; ++m) t.m[m] = M[m];
        }
        pcg_phase2<MIXED>(B, q, lc, alpha, beta, t, sv, true);
      }
    }
    if (rank == 0 && tid == 0) {
      if (!stop) {
        L->pcg_iterations = k + 1;
        L->rz = gamma;
        L->alpha = alpha;
        L->beta = beta;
        L->q0 = qk;
      } else if (k == 0 && !good) {
        L->linear_ok = 0;  // S not positive definite along the first direction
      }
      L->pq = delta;
      L->rr = rr;
      if (stop) L->pcg_active = 0;
      if (B.num_problems == 1) {
        // the only problem decides the loop: no cross-cluster count needed
        B.status[2] = stop ? 0 : 1;
        if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, stop ? 0u : 1u);
      }
    }
  } else if (B.num_problems == 1 && blockIdx.x == 0 && tid == 0) {
    pdl_wait();
    pdl_launch_dependents();
    B.status[2] = 0;
    if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, 0u);
  }
  if (B.num_problems == 1) return;
  pdl_wait();
  pdl_launch_dependents();
  // several problems: the last cluster to finish sets the PCG loop condition
  if (cs > 1 && rank != 0) return;
  if (last_block_done(B.global_counter + kGC_UPDATE, (uint32_t)(gridDim.x / cs), &flag)) {
    if (tid == 0) {
      int any = 0;
      for (int p2 = 0; p2 < B.num_problems; ++p2) any |= __ldcg(&B.lm[p2].active) && __ldcg(&B.lm[p2].pcg_active);
      B.status[2] = any;
      if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, any ? 1u : 0u);
    }
  }
}

// ---------------------------------------------------------------------------
// pdl: launch as a programmatic dependent of the preceding kernel of the
// stream (which must be the other PCG kernel).
cudaError_t launch_schur_matvec(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)b.nchunks);
  cfg.blockDim = dim3(kChunkCap);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  if (mixed) return cudaLaunchKernelEx(&cfg, k_schur_matvec<true>, b);
  return cudaLaunchKernelEx(&cfg, k_schur_matvec<false>, b);
}

cudaError_t launch_pcg_camera(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(b.num_problems * b.pcg_cluster));
  cfg.blockDim = dim3(kPcgThreads);
  cfg.dynamicSmemBytes = pcg_camera_smem(b.pcg_passes, b.pcg_cluster);
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)b.pcg_cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 2 : 1;
  if (mixed) return cudaLaunchKernelEx(&cfg, k_pcg_camera<true>, b);
  return cudaLaunchKernelEx(&cfg, k_pcg_camera<false>, b);
}

void launch_pcg_iteration(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  launch_schur_matvec(b, mixed, s, false);
  launch_pcg_camera(b, mixed, s, false);
}

// Slots of every camera block of the largest problem (passes x cluster size),
// kPcgNv doubles per block.
size_t pcg_camera_smem(int passes, int cluster) {
  return sizeof(double) * kPcgNv * (size_t)(passes > 0 ? passes : 1) * (size_t)(cluster > 0 ? cluster : 1);
}

// Largest cluster the camera kernel may use on this device (16 when the
// non-portable size is allowed, else 8).
int pcg_max_cluster() {
  cudaFuncSetAttribute(k_pcg_camera<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPcgSmemMax);
  cudaFuncSetAttribute(k_pcg_camera<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPcgSmemMax);
  const cudaError_t e1 = cudaFuncSetAttribute(k_pcg_camera<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  const cudaError_t e2 = cudaFuncSetAttribute(k_pcg_camera<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaGetLastError();
    return 8;
  }
  return 16;
}

}  // namespace gba
