// k_pcg.cu — implicit-Schur preconditioned conjugate gradients on the
// reduced camera system  S x = v,  S = B + Dc^2 - W C^-1 W^T,  with the
// block-Jacobi preconditioner M = blockdiag(S_ii)^-1 (built by K3b).
//
// One PCG iteration is three phases:
//   A  mat-vec over point-segment chunks (one CTA per chunk, one thread per
//      observation):  p_c = z_c + beta p_c (staged per distinct camera of
//      the chunk), w = J_p^T J_c p, t_j = C_j^-1 sum_j w, u = J_c^T J_p t_j
//      written at the observation's slot in the chunk's camera-sorted order,
//      then summed per camera run -> one partial per (chunk, camera).
//      No global atomics; every sum has a fixed order.
//   B  camera reduce, one warp per camera: p = z + beta p, q = (B + Dc^2) p
//      - sum of the camera's partials, p.q per camera; the problem's last
//      warp forms alpha = r.z / p.q (or stops the PCG if p.q <= 0).
//   C  update, one warp per camera: x += alpha p, r -= alpha q, z = M r,
//      r.z, r.r, x.(v + r) per camera; the problem's last warp applies the
//      stopping test (residual ratio or Ceres' quadratic-model test) and beta.
// Warps own cameras, so the FP64 work of B and C (GB300's FP64 pipe is
// narrow) spreads over every SM, and lanes own matrix rows / vector
// components so no lane carries more than a handful of FP64 chains.
// Two drivers run the same phase code, so they give bitwise-equal results:
//   - three kernels per iteration inside a CUDA-graph WHILE node;
//   - one persistent cooperative kernel per LM step looping over all PCG
//     iterations with grid barriers between the phases (every wait bounded;
//     a timeout sets GBA_ERR_TIMEOUT and the kernel returns).
// Data written inside a persistent launch is read back with ld.global.cg
// (L2) so no SM sees a stale L1 line.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "kernels.h"

namespace gba {

namespace {

template <bool MIXED>
struct MatvecSmem {
  typedef typename Prec<MIXED>::real real;
  real pseg[kChunkCap][9];
  real U[kChunkCap][9];  // first holds w (3 per obs), then u (9 per slot)
  real tpt[kChunkCap][3];
};

__device__ __forceinline__ bool pcg_live(const LMState *L) {
  return __ldcg(&L->active) != 0 && __ldcg(&L->pcg_active) != 0;
}

// Fixed-order sum of a[i * stride], i in [begin, end), by one warp.
__device__ __forceinline__ double warp_range_sum_cg(const double *a, int begin, int end, int stride) {
  double s = 0.0;
  for (int i = begin + (threadIdx.x & 31); i < end; i += 32) s += __ldcg(a + (size_t)i * stride);
  return warp_sum(s);
}

// "Last warp done" over a problem's cameras: true in every lane of the warp
// that brings the counter to `total` (which also resets it).
__device__ __forceinline__ bool last_warp_done(uint32_t *counter, uint32_t total) {
  __threadfence();
  __syncwarp();
  unsigned last = 0;
  if ((threadIdx.x & 31) == 0) {
    const uint32_t prev = atomicAdd(counter, 1u);
    last = prev == total - 1u;
    if (last) *counter = 0u;
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (last) __threadfence();
  return last != 0;
}

// ---- phase A -------------------------------------------------------------
template <bool MIXED>
__device__ void phase_matvec_chunk(const DeviceBatch &B, int ch, MatvecSmem<MIXED> &sm) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  typedef typename Acc<MIXED>::type Acc;
  const int t = threadIdx.x;
  const ChunkInfo ci = B.chunk[ch];
  const bool valid = t < ci.obs_count;
  // issue the Jacobian loads first: they do not depend on the staged direction
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
  const double beta = __ldcg(&B.lm[ci.problem].beta);
  for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
    const int sg = i / 9, q = i - 9 * sg;
    const size_t k = 9 * (size_t)B.seg_cam[ci.seg_begin + sg] + q;
    sm.pseg[sg][q] = (real)(__ldcg(B.pcg_z + k) + beta * __ldcg(B.pcg_p + k));
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
    const int jj = ci.pt_begin + t;
    const int b0 = B.pt_obs_begin[jj] - ci.obs_begin, b1 = B.pt_obs_begin[jj + 1] - ci.obs_begin;
    Acc y0, y1, y2;
    y0.init(), y1.init(), y2.init();
    for (int k = b0; k < b1; ++k) {
      y0.add(sm.U[k][0]);
      y1.add(sm.U[k][1]);
      y2.add(sm.U[k][2]);
    }
    const real *Ci = reinterpret_cast<const real *>(B.pt_Cinv) + 6 * (size_t)jj;
    const real w0 = (real)y0.value(), w1 = (real)y1.value(), w2 = (real)y2.value();
    sm.tpt[t][0] = Ci[0] * w0 + Ci[1] * w1 + Ci[2] * w2;
    sm.tpt[t][1] = Ci[1] * w0 + Ci[3] * w1 + Ci[4] * w2;
    sm.tpt[t][2] = Ci[2] * w0 + Ci[4] * w1 + Ci[5] * w2;
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
  for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
    const int sg = i / 9, q = i - 9 * sg;
    const int b0 = B.seg_pos[ci.seg_begin + sg];
    const int b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
    Acc a;
    a.init();
    for (int k = b0; k < b1; ++k) a.add(sm.U[k][q]);
    __stcg(B.seg_partial + 9 * ((size_t)ci.seg_begin + sg) + q, a.value());
  }
  __syncthreads();
}

// ---- phase B: one warp per camera -------------------------------------------
// Lanes 0..26 sum the camera's partials component-wise (lane = 9 g + q sums
// component q of segments g, g + 3, ...); lanes 0..8 then own row q of p, q.
__device__ void phase_reduce_camera(const DeviceBatch &B, int c) {
  const int p = B.cam_problem[c];
  LMState *L = B.lm + p;
  const int lane = threadIdx.x & 31;
  const int g = lane / 9, q = lane - 9 * g;
  const double beta = __ldcg(&L->beta);
  double acc = 0.0;
  if (g < 3) {
    const int e = B.cam_seg_begin[c + 1];
    for (int k = B.cam_seg_begin[c] + g; k < e; k += 3)
      acc += __ldcg(B.seg_partial + 9 * (size_t)B.cam_seg_list[k] + q);
  }
  const int qq = lane < 9 ? lane : 0;
  const double a0 = __shfl_sync(0xffffffffu, acc, qq);
  const double a1 = __shfl_sync(0xffffffffu, acc, 9 + qq);
  const double a2 = __shfl_sync(0xffffffffu, acc, 18 + qq);
  const size_t i = 9 * (size_t)c + qq;
  double pc = 0.0;
  if (lane < 9) pc = __ldcg(B.pcg_z + i) + beta * __ldcg(B.pcg_p + i);
  double bp = 0.0;
  const double *Bc = B.cam_B + 45 * (size_t)c;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const double pk = __shfl_sync(0xffffffffu, pc, k);
    if (lane < 9) bp += Bc[sym9(lane, k)] * pk;
  }
  double pq = 0.0;
  if (lane < 9) {
    const double qv = bp + B.cam_D2[i] * pc - ((a0 + a1) + a2);
    __stcg(B.pcg_p + i, pc);
    __stcg(B.pcg_q + i, qv);
    pq = pc * qv;
  }
  pq = warp_sum(pq);
  if (lane == 0) __stcg(B.cam_pcg + (size_t)kPcgScal * c + kPS_PQ, pq);
  const ProblemInfo pi = B.prob[p];
  if (last_warp_done(B.prob_counter + 4 * p + kPC_REDUCE, (uint32_t)pi.cam_count)) {
    const double pqs = warp_range_sum_cg(B.cam_pcg + kPS_PQ, pi.cam_begin, pi.cam_begin + pi.cam_count, kPcgScal);
    if (lane == 0) {
      L->pq = pqs;
      if (!(pqs > 0.0) || !isfinite(pqs)) {
        // S not positive definite along p: keep the current iterate
        if (L->pcg_iterations == 0) L->linear_ok = 0;
        L->alpha = 0.0;
        L->beta = 0.0;
        L->pcg_active = 0;
        atomicSub(B.status + 3, 1);
      } else {
        L->alpha = L->rz / pqs;
      }
      __threadfence();
    }
    __syncwarp();
  }
}

// ---- phase C: one warp per camera -------------------------------------------
__device__ void phase_update_camera(const DeviceBatch &B, int c) {
  const int p = B.cam_problem[c];
  LMState *L = B.lm + p;
  const int lane = threadIdx.x & 31;
  const double alpha = __ldcg(&L->alpha);
  const size_t i = 9 * (size_t)c + (lane < 9 ? lane : 0);
  double r = 0.0, x = 0.0;
  if (lane < 9) {
    x = __ldcg(B.pcg_x + i) + alpha * __ldcg(B.pcg_p + i);
    r = __ldcg(B.pcg_r + i) - alpha * __ldcg(B.pcg_q + i);
    __stcg(B.pcg_x + i, x);
    __stcg(B.pcg_r + i, r);
  }
  double z = 0.0;
  const double *M = B.cam_Minv + 81 * (size_t)c;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const double rk = __shfl_sync(0xffffffffu, r, k);
    if (lane < 9) z += M[lane * 9 + k] * rk;
  }
  double rz = 0.0, rr = 0.0, qx = 0.0;
  if (lane < 9) {
    __stcg(B.pcg_z + i, z);
    rz = r * z;
    rr = r * r;
    qx = x * (B.pcg_v[i] + r);
  }
  rz = warp_sum(rz);
  rr = warp_sum(rr);
  qx = warp_sum(qx);
  if (lane == 0) {
    double *cp = B.cam_pcg + (size_t)kPcgScal * c;
    __stcg(cp + kPS_RZ, rz);
    __stcg(cp + kPS_RR, rr);
    __stcg(cp + kPS_QX, qx);
  }
  const ProblemInfo pi = B.prob[p];
  if (last_warp_done(B.prob_counter + 4 * p + kPC_UPDATE, (uint32_t)pi.cam_count)) {
    const int c0 = pi.cam_begin, c1 = pi.cam_begin + pi.cam_count;
    const double rzn = warp_range_sum_cg(B.cam_pcg + kPS_RZ, c0, c1, kPcgScal);
    const double rrn = warp_range_sum_cg(B.cam_pcg + kPS_RR, c0, c1, kPcgScal);
    const double qxn = warp_range_sum_cg(B.cam_pcg + kPS_QX, c0, c1, kPcgScal);
    if (lane == 0) {
      const DeviceOptions &o = B.opt;
      const double rz_old = L->rz;
      const int it = ++L->pcg_iterations;
      bool stop = false;
      if (o.pcg_criterion == GBA_PCG_QUADRATIC_MODEL) {
        // Q(x) = x'Sx - 2 v'x = -x'(v + r);  stop when i (Q_i - Q_{i-1}) / Q_i < eta
        const double Q1 = -qxn;
        const double zeta = it * (Q1 - L->q0) / Q1;
        if (zeta < o.eta && it >= o.min_pcg_iterations) stop = true;
        L->q0 = Q1;
      } else {
        if (sqrt(rrn) <= o.pcg_tolerance * L->r0_norm && it >= o.min_pcg_iterations) stop = true;
      }
      if (it >= o.max_pcg_iterations) stop = true;
      if (!isfinite(rzn) || !(rz_old != 0.0)) stop = true;
      L->rr = rrn;
      L->beta = stop ? 0.0 : rzn / rz_old;
      L->rz = rzn;
      if (stop) {
        L->pcg_active = 0;
        atomicSub(B.status + 3, 1);
      }
      __threadfence();
    }
    __syncwarp();
  }
}

// ---- bounded grid barrier (persistent driver) ------------------------------
constexpr unsigned kBarrierSpinLimit = 1u << 24;

__device__ bool grid_barrier(const DeviceBatch &B, unsigned spin_limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned *count = B.global_counter + kGC_BAR_COUNT;
    unsigned *gen = B.global_counter + kGC_BAR_GEN;
    const unsigned g = atomicAdd(gen, 0u);
    __threadfence();
    const unsigned prev = atomicAdd(count, 1u);
    ok = 1;
    if (prev == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      unsigned spins = 0;
      while (*(volatile unsigned *)gen == g) {
        if (++spins > spin_limit) {
          ok = 0;
          atomicExch(B.status + 0, (int)GBA_ERR_TIMEOUT);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// three-kernel driver
template <bool MIXED>
__global__ void __launch_bounds__(kChunkCap) k_schur_matvec(DeviceBatch B) {
  __shared__ MatvecSmem<MIXED> sm;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x)
    if (pcg_live(B.lm + B.chunk[ch].problem)) phase_matvec_chunk<MIXED>(B, ch, sm);
}

constexpr int kCamWarps = 4;  // cameras (warps) per CTA in the camera kernels

__global__ void __launch_bounds__(32 * kCamWarps) k_camera_reduce(DeviceBatch B) {
  const int c = blockIdx.x * kCamWarps + (threadIdx.x >> 5);
  if (c < B.nc && pcg_live(B.lm + B.cam_problem[c])) phase_reduce_camera(B, c);
}

__global__ void __launch_bounds__(32 * kCamWarps) k_pcg_update(DeviceBatch B) {
  __shared__ int flag;
  const int c = blockIdx.x * kCamWarps + (threadIdx.x >> 5);
  if (c < B.nc && pcg_live(B.lm + B.cam_problem[c])) phase_update_camera(B, c);
  // the grid's last CTA sets the PCG loop condition
  if (last_block_done(B.global_counter + kGC_UPDATE, gridDim.x, &flag)) {
    if (threadIdx.x == 0) {
      int any = 0;
      for (int q = 0; q < B.num_problems; ++q) any |= __ldcg(&B.lm[q].active) && __ldcg(&B.lm[q].pcg_active);
      B.status[2] = any;
      if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, any ? 1u : 0u);
    }
  }
}

// ---------------------------------------------------------------------------
// persistent cooperative driver: every PCG iteration of one LM step
template <bool MIXED>
__global__ void __launch_bounds__(kChunkCap, 2) k_pcg_persistent(DeviceBatch B) {
  __shared__ MatvecSmem<MIXED> sm;
  __shared__ int stop;
  const int G = gridDim.x;
  const int warps = G * (kChunkCap / 32);
  const int gw = blockIdx.x * (kChunkCap / 32) + (threadIdx.x >> 5);
  for (int it = 0;; ++it) {
    if (threadIdx.x == 0)
      stop = (*(volatile int *)(B.status + 3) <= 0) || (it > B.opt.max_pcg_iterations + 1) ||
             (*(volatile int *)(B.status + 0) != 0);
    __syncthreads();
    if (stop) break;
    for (int ch = blockIdx.x; ch < B.nchunks; ch += G)
      if (pcg_live(B.lm + B.chunk[ch].problem)) phase_matvec_chunk<MIXED>(B, ch, sm);
    if (!grid_barrier(B, kBarrierSpinLimit)) return;
    for (int c = gw; c < B.nc; c += warps)
      if (pcg_live(B.lm + B.cam_problem[c])) phase_reduce_camera(B, c);
    if (!grid_barrier(B, kBarrierSpinLimit)) return;
    for (int c = gw; c < B.nc; c += warps)
      if (pcg_live(B.lm + B.cam_problem[c])) phase_update_camera(B, c);
    if (!grid_barrier(B, kBarrierSpinLimit)) return;
  }
}

// Failure-path self test: a grid barrier that can never complete (it waits
// for one CTA more than the grid has) must give up after its spin limit and
// report GBA_ERR_TIMEOUT instead of hanging.
__global__ void k_barrier_timeout_probe(DeviceBatch B, unsigned spin_limit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned *count = B.global_counter + kGC_BAR_COUNT;
    unsigned *gen = B.global_counter + kGC_BAR_GEN;
    const unsigned g = atomicAdd(gen, 0u);
    atomicAdd(count, 1u);  // never reaches gridDim.x + 1
    unsigned spins = 0;
    while (*(volatile unsigned *)gen == g) {
      if (++spins > spin_limit) {
        atomicExch(B.status + 0, (int)GBA_ERR_TIMEOUT);
        break;
      }
      __nanosleep(32);
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
void launch_schur_matvec(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  if (mixed)
    k_schur_matvec<true><<<b.nchunks, kChunkCap, 0, s>>>(b);
  else
    k_schur_matvec<false><<<b.nchunks, kChunkCap, 0, s>>>(b);
}
void launch_camera_reduce(const DeviceBatch &b, cudaStream_t s) {
  k_camera_reduce<<<(b.nc + kCamWarps - 1) / kCamWarps, 32 * kCamWarps, 0, s>>>(b);
}
void launch_pcg_update(const DeviceBatch &b, cudaStream_t s) {
  k_pcg_update<<<(b.nc + kCamWarps - 1) / kCamWarps, 32 * kCamWarps, 0, s>>>(b);
}
void launch_pcg_iteration(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  launch_schur_matvec(b, mixed, s);
  launch_camera_reduce(b, s);
  launch_pcg_update(b, s);
}

int pcg_persistent_blocks_per_sm(bool mixed) {
  int n = 0;
  if (mixed)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pcg_persistent<true>, kChunkCap, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pcg_persistent<false>, kChunkCap, 0);
  return n;
}

cudaError_t launch_pcg_persistent(const DeviceBatch &b, bool mixed, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kChunkCap);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (mixed) return cudaLaunchKernelEx(&cfg, k_pcg_persistent<true>, b);
  return cudaLaunchKernelEx(&cfg, k_pcg_persistent<false>, b);
}

cudaError_t launch_barrier_timeout_probe(const DeviceBatch &b, unsigned spin_limit, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2);
  cfg.blockDim = dim3(32);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_barrier_timeout_probe, b, spin_limit);
}

}  // namespace gba
