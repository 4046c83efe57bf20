// k_pcg.cu — implicit-Schur preconditioned conjugate gradients on the
// reduced camera system  S x = v,  S = B + Dc^2 - W C^-1 W^T,  with the
// block-Jacobi preconditioner M = blockdiag(S_ii)^-1 (built by K3b).
//
// One PCG iteration is two kernels:
//   K4a k_schur_matvec  mat-vec over point-segment chunks (one CTA per chunk,
//       one thread per observation): w = J_p^T J_c p, t_j = C_j^-1 sum_j w,
//       u = J_c^T J_p t_j written at the observation's slot in the chunk's
//       camera-sorted order, summed per camera run into one partial per
//       (chunk, camera), stored at the camera's contiguous (camera-major)
//       position.  No global atomics; every sum has a fixed order.
//   K4b k_pcg_camera    everything on the camera side, one thread-block
//       cluster per problem (up to 16 CTAs, one thread per camera
//       coordinate):
//         q = (B + Dc^2) p - sum of the camera's partials;   p.q
//         alpha = r.z / p.q;  x += alpha p;  r -= alpha q;  z = M r;
//         r.z, r.r, x.(v + r);  stopping test (residual ratio or Ceres'
//         quadratic-model test);  beta;  p = z + beta p.
//       The problem-wide dot products are reduced inside the cluster (warp
//       -> CTA shared memory -> every CTA reads all CTAs' sums over
//       distributed shared memory in rank order), so every CTA holds the
//       same alpha / beta / decision without any global atomic or spin.
// GB300 runs FP64 at 1/55 of FP32 throughput and with 64-cycle dependent
// latency, so in the mixed form the matrix-like inner work (partial sums,
// (B + Dc^2) p, M r) runs in FP32 with compensated sums while the vectors
// x, r, z, p, q and every dot product stay FP64.
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
    if (!pcg_live(B.lm + ci.problem)) continue;  // uniform over the CTA
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
    // stage the direction p of the chunk's cameras
    const real *pdir = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_pf : (const void *)B.pcg_p);
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
// kPcgBlockCams cameras with one thread per camera coordinate (9 per camera,
// so a block is exactly nine full warps and no lane idles); a problem with
// more blocks than the cluster has CTAs takes several passes.
//
// Every problem-wide dot product is summed in a fixed order that depends
// only on the problem's camera count: lanes -> warp (xor butterfly); then
// the (block, warp) values of all blocks, read over distributed shared
// memory from the CTA that owns each block, strided over the lanes of one
// warp in (block, warp) order and combined by a second butterfly.  All CTAs
// therefore hold the same alpha, beta and stopping decision, and the result
// depends neither on the cluster size nor on the other problems of a batch.
//
// The three cluster barriers are split into arrive / wait so that the loads
// of the next phase overlap the wait.
constexpr int kPcgThreads = 9 * kPcgBlockCams;  // 288
constexpr int kPcgWarps = kPcgThreads / 32;     // 9

namespace {

__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// Sum of NV values per (block, warp) over all blocks of the problem: block b
// lives in CTA rank b % cs at pass slot b / cs, value v of warp w at
// blk[(slot * kPcgWarps + w) * NV + v].  Called by one whole warp; returns
// the sums in every lane.
template <int NV>
__device__ __forceinline__ void blocks_sum(cg::cluster_group &cl, const double *blk, int nblk, int cs, double *out) {
  const int lane = threadIdx.x & 31;
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = 0.0;
  const int n = nblk * kPcgWarps;
  for (int e = lane; e < n; e += 32) {
    const int b = e / kPcgWarps, w = e - kPcgWarps * b;
    const double *src = cl.map_shared_rank(blk, b % cs) + ((b / cs) * kPcgWarps + w) * NV;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += src[k];
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = warp_sum(v[k]);
}

// Loads a fixed-size batch of partials before adding them, so that several
// memory round trips overlap while the additions keep their serial order.
template <typename real, typename AccT>
__device__ __forceinline__ void sum_partials(AccT &acc, const real *part, int s0, int s1) {
  constexpr int U = 32;
  int s = s0;
  for (; s + U <= s1; s += U) {
    real v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = part[9 * (size_t)(s + u)];
#pragma unroll
    for (int u = 0; u < U; ++u) acc.add(v[u]);
  }
  for (; s < s1; ++s) acc.add(part[9 * (size_t)s]);
}

}  // namespace

template <bool MIXED>
__global__ void __launch_bounds__(kPcgThreads) k_pcg_camera(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Acc<MIXED>::type Acc;
  // per pass: kPcgWarps p.q values, then kPcgWarps x (r.z, r.r, x.(v + r))
  extern __shared__ double blk[];
  __shared__ real sv[kPcgThreads];  // the block's r, staged for z = M r
  __shared__ double tot[4];
  __shared__ int flag;
  cg::cluster_group cl = cg::this_cluster();
  const int cs = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int prob = blockIdx.x / cs;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int lc = tid / 9, q = tid - 9 * lc;  // camera in the block, coordinate
  double *blk1 = blk;
  double *blk3 = blk + kPcgWarps * B.pcg_passes;
  LMState *L = B.lm + prob;
  if (prob < B.num_problems && pcg_live(L)) {  // uniform over the cluster
    const ProblemInfo pi = B.prob[prob];
    const int nblk = (pi.cam_count + kPcgBlockCams - 1) / kPcgBlockCams;
    // every LMState field this kernel reads is read before the first cluster
    // barrier: rank 0 overwrites them after the second one
    const double rz_old = L->rz, q0 = L->q0, r0_norm = L->r0_norm;
    const int its = L->pcg_iterations;
    const real *part = reinterpret_cast<const real *>(B.seg_partial) + q;
    const real *pdir = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_pf : (const void *)B.pcg_p);
    // ---- q = (B + Dc^2) p - sum of partials, and p.q ---------------------
    for (int j = 0, b = rank; b < nblk; ++j, b += cs) {
      const int k = b * kPcgBlockCams + lc;
      const bool valid = k < pi.cam_count;
      double pq = 0.0;
      if (valid) {
        const int c = pi.cam_begin + k;
        const size_t i = 9 * (size_t)c + q;
        const double pc = B.pcg_p[i];
        const real d2 = (real)B.cam_D2[i];
        const int s0 = B.cam_seg_begin[c], s1 = B.cam_seg_begin[c + 1];
        const real *Bc = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_Bf : (const void *)B.cam_B) +
                         45 * (size_t)c;
        const real *pv = pdir + 9 * (size_t)c;
        real brow[9], prow[9];
#pragma unroll
        for (int kk = 0; kk < 9; ++kk) brow[kk] = Bc[sym9(q, kk)], prow[kk] = pv[kk];
        Acc a;
        a.init();
        sum_partials<real, Acc>(a, part, s0, s1);
        real bp = 0;
#pragma unroll
        for (int kk = 0; kk < 9; ++kk) bp += brow[kk] * prow[kk];
        const double qv = (double)(bp + d2 * (real)pc - (real)a.value());
        B.pcg_q[i] = qv;
        pq = pc * qv;
      }
      pq = warp_sum(pq);
      if (lane == 0) blk1[j * kPcgWarps + warp] = pq;
    }
    cluster_arrive();
    cluster_wait();
    if (warp == 0) {
      double t[1];
      blocks_sum<1>(cl, blk1, nblk, cs, t);
      if (lane == 0) tot[0] = t[0];
    }
    __syncthreads();
    const double pqs = tot[0];
    const bool good = pqs > 0.0 && isfinite(pqs);
    const double alpha = good ? rz_old / pqs : 0.0;
    // ---- x += alpha p, r -= alpha q, z = M r, and the three dot products ----
    if (good) {
      for (int j = 0, b = rank; b < nblk; ++j, b += cs) {
        const int k = b * kPcgBlockCams + lc;
        const bool valid = k < pi.cam_count;
        const int c = pi.cam_begin + (valid ? k : 0);
        const size_t i = 9 * (size_t)c + q;
        double x = 0.0, r = 0.0, v = 0.0;
        real mrow[9];
        if (valid) {
          const real *M = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_Minvf
                                                               : (const void *)B.cam_Minv) +
                          81 * (size_t)c + 9 * q;
#pragma unroll
          for (int kk = 0; kk < 9; ++kk) mrow[kk] = M[kk];
          x = B.pcg_x[i] + alpha * B.pcg_p[i];
          r = B.pcg_r[i] - alpha * B.pcg_q[i];
          v = B.pcg_v[i];
        }
        if (j > 0) __syncthreads();  // the previous pass has finished reading sv
        sv[tid] = (real)r;
        __syncthreads();
        double rz = 0.0, rr = 0.0, qx = 0.0;
        if (valid) {
          const real *rv = sv + 9 * lc;
          real z = 0;
#pragma unroll
          for (int kk = 0; kk < 9; ++kk) z += mrow[kk] * rv[kk];
          B.pcg_x[i] = x;
          B.pcg_r[i] = r;
          B.pcg_z[i] = (double)z;
          rz = r * (double)z;
          rr = r * r;
          qx = x * (v + r);
        }
        rz = warp_sum(rz);
        rr = warp_sum(rr);
        qx = warp_sum(qx);
        if (lane == 0) {
          double *d = blk3 + (j * kPcgWarps + warp) * 3;
          d[0] = rz, d[1] = rr, d[2] = qx;
        }
      }
    }
    cluster_arrive();
    cluster_wait();
    if (warp == 0) {
      double t[3] = {0.0, 0.0, 0.0};
      if (good) blocks_sum<3>(cl, blk3, nblk, cs, t);
      if (lane == 0) tot[1] = t[0], tot[2] = t[1], tot[3] = t[2];
    }
    __syncthreads();
    // this CTA has read all the distributed shared memory it needs
    cluster_arrive();
    const double rzn = tot[1], rrn = tot[2], qxn = tot[3];
    // ---- stopping test and the next direction (identical in every CTA) ------
    const DeviceOptions &o = B.opt;
    const int it = its + (good ? 1 : 0);
    bool stop = !good;
    double q1 = q0;
    if (good) {
      if (o.pcg_criterion == GBA_PCG_QUADRATIC_MODEL) {
        // Q(x) = x'Sx - 2 v'x = -x'(v + r);  stop when i (Q_i - Q_{i-1}) / Q_i < eta
        q1 = -qxn;
        const double zeta = it * (q1 - q0) / q1;
        if (zeta < o.eta && it >= o.min_pcg_iterations) stop = true;
      } else {
        if (sqrt(rrn) <= o.pcg_tolerance * r0_norm && it >= o.min_pcg_iterations) stop = true;
      }
      if (it >= o.max_pcg_iterations) stop = true;
      if (!isfinite(rzn) || !(rz_old != 0.0)) stop = true;
    }
    const double beta = stop ? 0.0 : rzn / rz_old;
    if (!stop) {
      for (int b = rank; b < nblk; b += cs) {
        const int k = b * kPcgBlockCams + lc;
        if (k < pi.cam_count) {
          const size_t i = 9 * (size_t)(pi.cam_begin + k) + q;
          const double pn = B.pcg_z[i] + beta * B.pcg_p[i];
          B.pcg_p[i] = pn;
          if (MIXED) B.pcg_pf[i] = (float)pn;
        }
      }
    }
    if (rank == 0 && tid == 0) {
      L->pq = pqs;
      L->alpha = alpha;
      if (good) {
        L->pcg_iterations = it;
        L->rr = rrn;
        L->rz = rzn;
        L->q0 = q1;
        L->beta = beta;
      } else if (its == 0) {
        L->linear_ok = 0;  // S not positive definite along the first direction
      }
      if (stop) L->pcg_active = 0;
      if (B.num_problems == 1) {
        // the only problem decides the loop: no cross-cluster count needed
        B.status[2] = stop ? 0 : 1;
        if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, stop ? 0u : 1u);
      }
    }
    cluster_wait();  // no CTA leaves while another may still read its shared memory
  } else if (B.num_problems == 1 && blockIdx.x == 0 && tid == 0) {
    B.status[2] = 0;
    if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, 0u);
  }
  if (B.num_problems == 1) return;
  // several problems: the last cluster to finish sets the PCG loop condition
  if (cs > 1 && (blockIdx.x % cs) != 0) return;
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
void launch_schur_matvec(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  if (mixed)
    k_schur_matvec<true><<<b.nchunks, kChunkCap, 0, s>>>(b);
  else
    k_schur_matvec<false><<<b.nchunks, kChunkCap, 0, s>>>(b);
}

cudaError_t launch_pcg_camera(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(b.num_problems * b.pcg_cluster));
  cfg.blockDim = dim3(kPcgThreads);
  cfg.dynamicSmemBytes = pcg_camera_smem(b.pcg_passes);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)b.pcg_cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (mixed) return cudaLaunchKernelEx(&cfg, k_pcg_camera<true>, b);
  return cudaLaunchKernelEx(&cfg, k_pcg_camera<false>, b);
}

void launch_pcg_iteration(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  launch_schur_matvec(b, mixed, s);
  launch_pcg_camera(b, mixed, s);
}

size_t pcg_camera_smem(int passes) { return sizeof(double) * 4 * kPcgWarps * (size_t)(passes > 0 ? passes : 1); }

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
