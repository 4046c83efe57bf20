// k_pcg_cluster.cu — the whole PCG of a problem in one launch: one thread
// block cluster per problem (mixed form, explicit Schur complement).
//
// The two-kernel PCG (k_pcg.cu, k_schur.cu) pays two kernel boundaries per
// iteration, and a batch iterates until its slowest problem's PCG ends.
// Here a cluster of cs CTAs (cs <= 16, on cs SMs of one GPC) runs every
// iteration of one problem's PCG.  CTA `rank` owns a contiguous run of the
// problem's cameras and keeps x, r, v, q and its rows of S (when they fit)
// in shared memory; every CTA keeps p of all the problem's cameras (its
// product needs p of every co-visible camera) and updates it for all of
// them with the same arithmetic, so the copies agree bitwise.  The
// direction is FP32 (the product's input) and the same FP32 values enter
// p.q and the update of x, so the curvature p.Sp and the recurrences refer
// to the direction the product used.  Per iteration:
//   1. q = S p for the owned rows (FP32 products and per-thread sums,
//      double-float across the threads of a row) and each owned camera's
//      p.q; barrier
//   2. p.q over the problem's cameras, alpha; x, r and z = M r of the owned
//      cameras, each owned camera's r.z, r.r, x.(v + r); barrier
//   3. the stopping test and beta from the cameras' values, p_{k+1} =
//      z_{k+1} + beta p_k for all cameras.
// Each CTA stores its z and per-camera values into its own shared memory;
// after the cluster barrier (release/acquire) the others read them from
// there (distributed shared memory), one load per value.  The dot products
// are summed per camera (a fixed tree over its nine coordinates) and then
// over the problem's cameras (a fixed tree over a warp), so the result
// depends neither on the cluster size nor on the batch: a problem gets the
// same bits alone and in any batch.
// GB300 issues FP64 some 64 times slower than FP32 (and with a long
// latency), so the vectors and the PCG scalars are double-float (two
// floats, about 48 bits); the mixed form's matrix (S, M) is FP32, so this
// loses nothing FP64 vectors would keep.  Every CTA takes the same decisions
// from the same values, so all reach the same cluster barriers (the
// hardware's barrier.cluster arrive/wait; there are no spin-waits).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace gba {

namespace {

constexpr int kClSub = 8;  // lanes per (camera, row triplet) of the product

// Shared-memory layout (bytes), the same on the host and the device.
struct ClLayout {
  size_t zf, ph, mo, xh, xl, rh, rl, vh, vl, qh, ql, cv, owner, boff, scol, sval, total;
};
__host__ __device__ inline size_t cl_align(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline ClLayout cl_layout(int n_max, int own_max, int cache_blocks) {
  ClLayout l;
  size_t o = 0;
  const size_t nf = 4 * 9 * (size_t)n_max, of = 4 * 9 * (size_t)own_max;
  l.zf = o, o = cl_align(o + nf);
  l.ph = o, o = cl_align(o + 4 * 12 * (size_t)n_max);  // p, 12 floats per camera (three 16-byte loads)
  l.mo = o, o = cl_align(o + 4 * 81 * (size_t)own_max);
  l.xh = o, o = cl_align(o + of);
  l.xl = o, o = cl_align(o + of);
  l.rh = o, o = cl_align(o + of);
  l.rl = o, o = cl_align(o + of);
  l.vh = o, o = cl_align(o + of);
  l.vl = o, o = cl_align(o + of);
  l.qh = o, o = cl_align(o + of);
  l.ql = o, o = cl_align(o + of);
  l.cv = o, o = cl_align(o + 8 * 4 * (size_t)n_max);  // per camera: p.q, r.z, r.r, x.(v + r) (double-float)
  l.owner = o, o = cl_align(o + 4 * (size_t)n_max);    // per camera: the rank that owns it
  // the owned rows of S (cache_blocks > 0): per owned camera its first
  // block, per block its column camera (in the problem) and its 81 values
  l.boff = o, o = cl_align(o + (cache_blocks > 0 ? 4 * ((size_t)own_max + 1) : 0));
  l.scol = o, o = cl_align(o + 4 * (size_t)cache_blocks);
  // per block three row triplets (rows g, g + 3, g + 6) of 27 values + pad
  l.sval = o, o = cl_align(o + 4 * 84 * (size_t)cache_blocks);
  l.total = o;
  return l;
}

// Sum over the 16 lanes of a half-warp group (xor butterfly: a fixed tree,
// the same bits in every lane).
__device__ __forceinline__ DF df_group16_sum(DF v, unsigned mask) {
#pragma unroll
  for (int off = 1; off < 16; off <<= 1) {
    const DF w{__shfl_xor_sync(mask, v.hi, off), __shfl_xor_sync(mask, v.lo, off)};
    v = df_add(v, w);
  }
  return v;
}

// Sum of slot j of the problem's n per-camera values (staged in shared
// memory; in one warp: lane l adds cameras l, l + 32, ... in order, then a
// butterfly); the total in every lane.
__device__ __forceinline__ DF cam_total(const float2 *camv, int j, int n) {
  const int lane = threadIdx.x & 31;
  DF s = df_zero();
  for (int c = lane; c < n; c += 32) {
    const float2 v = camv[4 * c + j];
    s = df_add(s, DF{v.x, v.y});
  }
  return df_warp_sum(s);
}

// a / b in double-float: a float quotient, one correction step
__device__ __forceinline__ DF df_div(DF a, DF b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const DF r = df_add(a, df_neg(df_mul_f(b, q1)));
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return df_fast_two_sum(q1, q2);
}
__device__ __forceinline__ bool df_le(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }

}  // namespace

__global__ void __launch_bounds__(kClThreads, 1) k_pcg_cluster(DeviceBatch B, int cs, int n_max, int own_max,
                                                            int cache_blocks) {
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char cl_smem[];
  const ClLayout lay = cl_layout(n_max, own_max, cache_blocks);
  float *zf = reinterpret_cast<float *>(cl_smem + lay.zf);
  float *ph = reinterpret_cast<float *>(cl_smem + lay.ph);
  float *Mo = reinterpret_cast<float *>(cl_smem + lay.mo);
  float *xh = reinterpret_cast<float *>(cl_smem + lay.xh);
  float *xl = reinterpret_cast<float *>(cl_smem + lay.xl);
  float *rh = reinterpret_cast<float *>(cl_smem + lay.rh);
  float *rl = reinterpret_cast<float *>(cl_smem + lay.rl);
  float *vh = reinterpret_cast<float *>(cl_smem + lay.vh);
  float *vl = reinterpret_cast<float *>(cl_smem + lay.vl);
  float *qh = reinterpret_cast<float *>(cl_smem + lay.qh);
  float *ql = reinterpret_cast<float *>(cl_smem + lay.ql);
  float2 *cvs = reinterpret_cast<float2 *>(cl_smem + lay.cv);
  int *own_of = reinterpret_cast<int *>(cl_smem + lay.owner);
  int *boff = reinterpret_cast<int *>(cl_smem + lay.boff);
  int *scol = reinterpret_cast<int *>(cl_smem + lay.scol);
  float *sval = reinterpret_cast<float *>(cl_smem + lay.sval);
  __shared__ DF scf[4];
  __shared__ int stop_s;

  const int rank = (int)cl.block_rank();
  const int prob = blockIdx.x / cs;
  const int t = threadIdx.x, T = blockDim.x;
  LMState *L = B.lm + prob;
  // uniform over the cluster: every CTA reads the same state before its
  // first barrier, and rank 0 changes it only after the last one
  if (!(L->active && L->pcg_active)) return;
  const ProblemInfo pi = B.prob[prob];
  const int n = pi.cam_count, c0 = pi.cam_begin;
  // the cameras split into cs runs of about equal blocks of S (the
  // product's work): CTA `rank` owns the cameras whose blocks before them
  // (with the diagonal ones) lie in [bound(rank), bound(rank + 1))
  // (bound(r) = ceil(r W / cs) <= before(c) exactly when r <= before(c) cs / W,
  // so camera c's owner is floor(before(c) cs / W))
  int own0 = 0, own_end = 0;
  {
    const int r0 = B.sblk_row[c0];
    const long long wtot = (long long)(B.sblk_row[c0 + n] - r0) + n;
    const long long ta = ((long long)rank * wtot + cs - 1) / cs, tb = ((long long)(rank + 1) * wtot + cs - 1) / cs;
    for (int cb = 0; cb < n; cb += T) {
      const int c = cb + t;
      const long long before = c < n ? (long long)(B.sblk_row[c0 + c] - r0) + c : wtot;
      if (c < n) own_of[c] = (int)(before * cs / wtot);
      own0 += __syncthreads_count(before < ta);
      own_end += __syncthreads_count(before < tb);
    }
  }
  const int own_n = own_end - own0;
  const int n9 = 9 * n, o9 = 9 * own_n, a9 = 9 * own0;  // a9: first owned coordinate in the problem
  const size_t g0 = 9 * (size_t)c0;                       // the problem's first coordinate (global)

  // the start (K3b): x = 0, r = v, z = M r, p_0 = z
  for (int i = t; i < n9; i += T) {
    const float z = B.pcg_zf[g0 + i];
    zf[i] = z, ph[i + 3 * (i / 9)] = z;
  }
  for (int i = t; i < o9; i += T) {
    const DF v = df_from_double(B.pcg_v[g0 + a9 + i]);
    const DF r = df_from_double(B.pcg_r[g0 + a9 + i]);
    xh[i] = 0.f, xl[i] = 0.f;
    rh[i] = r.hi, rl[i] = r.lo;
    vh[i] = v.hi, vl[i] = v.lo;
  }
  for (int i = t; i < 81 * own_n; i += T) Mo[i] = B.cam_Minvf[81 * (size_t)(c0 + own0) + i];
  const float *vals = reinterpret_cast<const float *>(B.sblk_val);
  const float *Sii = reinterpret_cast<const float *>(B.cam_Sii);
  const bool cached = cache_blocks > 0;
  if (cached) {
    // the owned rows of S, fixed during the PCG: off-diagonal blocks, then
    // the diagonal block, per owned camera
    if (t == 0) {
      int s = 0;
      for (int lc = 0; lc < own_n; ++lc) {
        boff[lc] = s;
        const int c = c0 + own0 + lc;
        s += B.sblk_row[c + 1] - B.sblk_row[c] + 1;
      }
      boff[own_n] = s;
    }
    __syncthreads();
    for (int lc = 0; lc < own_n; ++lc) {
      const int c = c0 + own0 + lc;
      const int r0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - r0, b0 = boff[lc];
      for (int v = t; v <= nb; v += T) scol[b0 + v] = (v < nb ? B.sblk_col[r0 + v] : c) - c0;
      // triplet layout: block b, triplet g, entry j = row (g + 3 (j / 9)), column j % 9
      for (int e = t; e < 84 * (nb + 1); e += T) {
        const int v = e / 84, w = e - 84 * v, g = w / 28, j = w - 28 * g;
        float x = 0.f;
        if (j < 27) {
          const int el = 9 * (g + 3 * (j / 9)) + j % 9;
          x = v < nb ? vals[81 * (size_t)(r0 + v) + el] : Sii[81 * (size_t)c + el];
        }
        sval[84 * (size_t)(b0 + v) + w] = x;
      }
    }
  }
  const DeviceOptions &o = B.opt;
  // PCG scalars (double-float in every thread; thread 0 decides)
  DF rz = df_from_double(L->rz);
  double q0 = L->q0;
  const double lim = o.pcg_tolerance * L->r0_norm;
  const DF lim2 = df_from_double(lim * lim);
  int k = 0;
  bool linear_ok = true;
  DF last_pq = df_zero(), last_beta = df_zero(), last_rr = df_from_double(L->rr);
  const int lane = t % kClSub;
  // the lanes of a row group (kClSub consecutive lanes of a warp)
  const unsigned gmask = ((1u << kClSub) - 1u) << ((t & 31) & ~(kClSub - 1));
  // camera-coordinate mapping of the per-camera sums: a half-warp per camera
  const int hq = t & 15, hc = t >> 4;
  const unsigned hmask = 0xffffu << (t & 16);
  __syncthreads();
  for (;;) {
    // 1. q = S p_k for the owned rows: a thread takes rows g, g + 3, g + 6
    // of a camera (one load of p per block for three rows) for the blocks
    // lane, lane + kClSub, ... of the row (the last one the diagonal
    // block); FP32 sums per thread, double-float over the kClSub lanes
    for (int ws = t / kClSub; ws < 3 * own_n; ws += T / kClSub) {
      const int lc = ws / 3, g = ws - 3 * lc;
      const int c = c0 + own0 + lc;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f;
      if (cached) {
        const int b0 = boff[lc], nb1 = boff[lc + 1] - b0;
        for (int v = lane; v < nb1; v += kClSub) {
          // the triplet's 27 values and the column camera's p: 16-byte loads
          const float4 *r4 = reinterpret_cast<const float4 *>(sval + 84 * (b0 + v) + 28 * g);
          const float4 *p4 = reinterpret_cast<const float4 *>(ph + 12 * scol[b0 + v]);
          float rv[28], pv[12];
#pragma unroll
          for (int u = 0; u < 7; ++u) *reinterpret_cast<float4 *>(&rv[4 * u]) = r4[u];
#pragma unroll
          for (int u = 0; u < 3; ++u) *reinterpret_cast<float4 *>(&pv[4 * u]) = p4[u];
#pragma unroll
          for (int cc = 0; cc < 9; ++cc) {
            a0 = __fmaf_rn(rv[cc], pv[cc], a0);
            a1 = __fmaf_rn(rv[9 + cc], pv[cc], a1);
            a2 = __fmaf_rn(rv[18 + cc], pv[cc], a2);
          }
        }
      } else {
        const int r0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - r0;
        for (int v = lane; v <= nb; v += kClSub) {
          const float *row = (v < nb ? vals + 81 * (size_t)(r0 + v) : Sii + 81 * (size_t)c) + 9 * g;
          const float *pc = ph + 12 * ((v < nb ? B.sblk_col[r0 + v] : c) - c0);
#pragma unroll
          for (int cc = 0; cc < 9; ++cc) {
            const float pv = pc[cc];
            a0 = __fmaf_rn(row[cc], pv, a0);
            a1 = __fmaf_rn(row[27 + cc], pv, a1);
            a2 = __fmaf_rn(row[54 + cc], pv, a2);
          }
        }
      }
      DF d0{a0, 0.f}, d1{a1, 0.f}, d2{a2, 0.f};
#pragma unroll
      for (int off = 1; off < kClSub; off <<= 1) {
        const DF w0{__shfl_xor_sync(gmask, d0.hi, off), __shfl_xor_sync(gmask, d0.lo, off)};
        const DF w1{__shfl_xor_sync(gmask, d1.hi, off), __shfl_xor_sync(gmask, d1.lo, off)};
        const DF w2{__shfl_xor_sync(gmask, d2.hi, off), __shfl_xor_sync(gmask, d2.lo, off)};
        d0 = df_add(d0, w0), d1 = df_add(d1, w1), d2 = df_add(d2, w2);
      }
      if (lane == 0) {
        const int i = 9 * lc + g;
        qh[i] = d0.hi, ql[i] = d0.lo;
        qh[i + 3] = d1.hi, ql[i + 3] = d1.lo;
        qh[i + 6] = d2.hi, ql[i + 6] = d2.lo;
      }
    }
    __syncthreads();
    // each owned camera's p.q
    for (int cb = 0; cb < own_n; cb += T / 16) {
      const int lc = cb + hc;
      DF d = df_zero();
      if (lc < own_n && hq < 9) {
        const int i = 9 * lc + hq;
        d = df_mul_f(DF{qh[i], ql[i]}, ph[12 * (own0 + lc) + hq]);
      }
      d = df_group16_sum(d, hmask);
      if (lc < own_n && hq == 0) cvs[4 * (own0 + lc)] = make_float2(d.hi, d.lo);
    }
    cl.sync();
    // 2. p.q, alpha, the owned update
    // the other CTAs' cameras' values, read from their shared memory
    for (int c = t; c < n; c += T) {
      const int r = own_of[c];
      if (r != rank) cvs[4 * c] = *cl.map_shared_rank(cvs + 4 * c, r);
    }
    __syncthreads();
    if (t < 32) {
      const DF s = cam_total(cvs, 0, n);
      if (t == 0) {
        scf[1] = s;
        scf[0] = df_div(rz, s);
      }
    }
    __syncthreads();
    const DF pq = scf[1];
    if (!(pq.hi > 0.f && isfinite(pq.hi))) {  // S not positive definite along p_k: the PCG ends with x_k
      if (k == 0) linear_ok = false;
      break;
    }
    {
      const DF alpha = scf[0], nalpha = df_neg(scf[0]);
      for (int cb = 0; cb < own_n; cb += T / 16) {
        const int lc = cb + hc;
        const bool act = lc < own_n && hq < 9;
        const int i = 9 * lc + hq;
        DF r = df_zero(), x = df_zero();
        if (act) {
          x = df_add(DF{xh[i], xl[i]}, df_mul_f(alpha, ph[12 * (own0 + lc) + hq]));
          r = df_add(DF{rh[i], rl[i]}, df_mul(nalpha, DF{qh[i], ql[i]}));
          xh[i] = x.hi, xl[i] = x.lo;
          rh[i] = r.hi, rl[i] = r.lo;
        }
        __syncwarp(hmask);  // the camera's r, for z = M r
        DF d0 = df_zero(), d1 = df_zero(), d2 = df_zero();
        if (act) {
          const float *m = Mo + 81 * lc + 9 * hq;
          const float *rr = rh + 9 * lc;
          float u = 0.f;
#pragma unroll
          for (int kk = 0; kk < 9; ++kk) u = __fmaf_rn(m[kk], rr[kk], u);
          zf[a9 + i] = u;
          d0 = df_mul_f(r, u);
          d1 = df_mul(r, r);
          d2 = df_mul(x, df_add(DF{vh[i], vl[i]}, r));
        }
        d0 = df_group16_sum(d0, hmask);
        d1 = df_group16_sum(d1, hmask);
        d2 = df_group16_sum(d2, hmask);
        if (lc < own_n && hq == 0) {
          float2 *dst = cvs + 4 * (own0 + lc);
          dst[1] = make_float2(d0.hi, d0.lo), dst[2] = make_float2(d1.hi, d1.lo), dst[3] = make_float2(d2.hi, d2.lo);
        }
      }
    }
    cl.sync();
    // 3. the stopping test on (x_{k+1}, r_{k+1}) and beta_{k+1}; the new z
    // the other CTAs' cameras' values (slots 1..3), then: warps 0-2 sum them
    // while the other warps read the other CTAs' z (both from the owners'
    // shared memory)
    for (int e = t; e < 3 * n; e += T) {
      const int c = e / 3, j = 1 + e - 3 * c, r = own_of[c];
      if (r != rank) cvs[4 * c + j] = *cl.map_shared_rank(cvs + 4 * c + j, r);
    }
    __syncthreads();
    if (t >= 96) {
      const int tz = t - 96, Tz = T - 96;
      for (int i0 = 0; i0 < n9; i0 += 4 * Tz) {
        float zv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = i0 + u * Tz + tz;
          zv[u] = 0.f;
          if (i < n9) {
            const int r = own_of[i / 9];
            if (r != rank) zv[u] = *cl.map_shared_rank(zf + i, r);
          }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = i0 + u * Tz + tz;
          if (i < n9 && own_of[i / 9] != rank) zf[i] = zv[u];
        }
      }
    }
    if (t < 96) {  // warps 0, 1, 2: r.z, r.r, x.(v + r)
      const DF sj = cam_total(cvs, 1 + (t >> 5), n);
      if ((t & 31) == 0) scf[1 + (t >> 5)] = sj;
    }
    __syncthreads();
    if (t == 0) {
      const DF rz1 = scf[1], rr1 = scf[2];
      const int k1 = k + 1;
      bool stop = false;
      if (o.pcg_criterion == GBA_PCG_QUADRATIC_MODEL) {
        const double qk = -df_value(scf[3]);  // Q(x) = x'Sx - 2 v'x = -x.(v + r)
        const double lhs = k1 * (qk - q0), rhs = o.eta * qk;
        const bool below = qk > 0.0 ? lhs < rhs : (qk < 0.0 ? lhs > rhs : q0 > 0.0);
        if (below && k1 >= o.min_pcg_iterations) stop = true;
        q0 = qk;
      } else if (df_le(rr1, lim2) && k1 >= o.min_pcg_iterations) {
        stop = true;
      }
      if (k1 >= o.max_pcg_iterations) stop = true;
      if (!(rz1.hi != 0.f && isfinite(rz1.hi))) stop = true;
      scf[0] = df_div(rz1, rz);  // beta
      stop_s = stop ? 1 : 0;
    }
    __syncthreads();
    last_beta = scf[0];
    last_rr = scf[2];
    rz = scf[1];
    last_pq = pq;
    ++k;
    if (stop_s) break;
    {
      // p_{k+1} = z_{k+1} + beta p_k, rounded once to FP32
      const DF beta = scf[0];
      for (int i = t; i < n9; i += T) {
        const int ip = i + 3 * (i / 9);
        ph[ip] = df_add(DF{zf[i], 0.f}, df_mul_f(beta, ph[ip])).hi;
      }
    }
    __syncthreads();
  }
  // results: the owned x (the camera step) and the PCG vectors; the state
  for (int i = t; i < o9; i += T) {
    const size_t gi = g0 + a9 + i;
    B.pcg_x[gi] = df_value(DF{xh[i], xl[i]});
    B.pcg_r[gi] = df_value(DF{rh[i], rl[i]});
    B.pcg_z[gi] = (double)zf[a9 + i];
    B.pcg_p[gi] = (double)ph[12 * own0 + i + 3 * (i / 9)];
  }
  if (rank == 0 && t == 0) {
    L->pcg_iterations = k;
    if (!linear_ok) L->linear_ok = 0;
    if (k > 0) {
      L->beta = df_value(last_beta);
      L->rz = df_value(rz);
      L->rr = df_value(last_rr);
      L->q0 = q0;
      L->pq = df_value(last_pq);
    }
    L->pcg_active = 0;
  }
  // no CTA leaves before the others have read what it stored for them
  cl.sync();
}

bool pcg_cluster_plan(const ProblemInfo *prob, int num_problems, const int32_t *sblk_row, int cams_per_cta,
                      ClusterPlan *plan) {
  *plan = ClusterPlan();
  int n_max = 0;
  for (int p = 0; p < num_problems; ++p) n_max = std::max(n_max, (int)prob[p].cam_count);
  if (n_max <= 0 || n_max > kClMaxCams) return false;
  // a single problem spreads over up to 16 SMs (16 cameras per CTA); a batch
  // takes fewer CTAs per problem (64 cameras per CTA) and more problems at once
  const bool single = num_problems == 1;
  const int target = cams_per_cta > 0 ? cams_per_cta : single ? 16 : 64;
  int cs = 1;
  while (cs < kClMaxCS && (n_max + cs - 1) / cs > target) cs *= 2;
  const int threads = 512;
  // the rows of S stay in shared memory when the CTAs of the launch fit on
  // the SMs one per SM and their rows fit next to the vectors
  int dev = 0, sms = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // the kernel's split of each problem's cameras (runs of about equal
  // blocks): the largest run and its blocks
  int own = 0, mb = 0;
  for (int p = 0; p < num_problems; ++p) {
    const int n = prob[p].cam_count, c0 = prob[p].cam_begin, r0 = sblk_row[c0];
    const long long wtot = (long long)(sblk_row[c0 + n] - r0) + n;
    int a = 0;
    for (int r = 0; r < cs; ++r) {
      const long long tb = ((long long)(r + 1) * wtot + cs - 1) / cs;
      int b = a;
      while (b < n && (long long)(sblk_row[c0 + b] - r0) + b < tb) ++b;
      own = std::max(own, b - a);
      mb = std::max(mb, (int)(sblk_row[c0 + b] - sblk_row[c0 + a]) + (b - a));
      a = b;
    }
  }
  if (own > kClMaxOwn) return false;
  int cache = 0;
  if ((long long)num_problems * cs <= sms && cl_layout(n_max, own, mb).total <= (size_t)optin) cache = mb;
  const ClLayout l = cl_layout(n_max, own, cache);
  if (l.total > (size_t)optin) return false;
  if (raise_smem_limit((const void *)k_pcg_cluster, l.total) != cudaSuccess ||
      (cs > 8 && cudaFuncSetAttribute(k_pcg_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cs);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = l.total;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, k_pcg_cluster, &cfg) != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    return false;
  }
  plan->cs = cs;
  plan->n_max = n_max;
  plan->own_max = own;
  plan->threads = threads;
  plan->cache_blocks = cache;
  plan->smem = l.total;
  return true;
}

cudaError_t launch_pcg_cluster(const DeviceBatch &b, const ClusterPlan &plan, cudaStream_t s) {
  if (b.num_problems == 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(b.num_problems * plan.cs));
  cfg.blockDim = dim3((unsigned)plan.threads);
  cfg.dynamicSmemBytes = plan.smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)plan.cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_pcg_cluster, b, plan.cs, plan.n_max, plan.own_max, plan.cache_blocks);
}

}  // namespace gba
