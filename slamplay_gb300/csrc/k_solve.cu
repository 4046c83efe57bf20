// k_solve.cu — linear-solve and trust-region kernels.
//
// The LM system (J^T J + D^2) y = J^T r is solved with the points eliminated
// (Schur complement on the cameras), as Ceres' SPARSE_SCHUR does for the
// reference (test_bundle_adjustment_ceres.cpp:97), but the reduced camera
// matrix S = B + Dc^2 - W C^-1 W^T is never formed: it is applied implicitly
// inside a block-Jacobi PCG.
//
//  K3a k_point_schur     per chunk: C = J_p^T J_p + Dp^2, FP64 inverse, Cinv g_p,
//                        and per (camera segment) the partial Schur diagonal
//                        block and reduced rhs of the chunk's observations
//  K3b k_camera_schur    per camera (CTA): S_ii and the reduced rhs from the
//                        partials, parallel FP64 9x9 inverse, PCG start
//                        (x = 0, r = v, z = M r)
//  K4  (k_pcg.cu)        implicit-Schur PCG: mat-vec over point-segment
//                        chunks, camera reduce, vector update
//  K5  k_back_substitute per chunk: y_p = C^-1 (g_p - W^T y_c), model cost
//                        change, candidate points
//  K6  k_decide          per problem: Ceres' accept / reject / radius update
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "kernels.cuh"
#include "kernels.h"

namespace gba {

__device__ __forceinline__ double lm_d2(double colnorm2, double radius, const DeviceOptions &o) {
  // LevenbergMarquardtStrategy: diag = clamp(|J_col|^2), D = sqrt(diag / radius);
  // g2o's Levenberg: D^2 = lambda = 1 / radius on every parameter
  const double d = o.g2o ? 1.0 : fmin(fmax(colnorm2, o.min_diagonal), o.max_diagonal);
  const double D = sqrt(d / radius);
  return D * D;
}

// ---------------------------------------------------------------------------
// K3a: one CTA per point-segment chunk.
//   1. per point (thread < pt_count): C = J_p^T J_p + Dp^2, its FP64 inverse,
//      t = C^-1 g_p (kept for the back-substitution and the reduced rhs);
//   2. per observation: the 2x2 A = J_p C^-1 J_p^T and e = J_p t, staged
//      with J_c at the observation's slot in the chunk's camera-sorted order;
//   3. per (camera segment, entry): the segment's share of the camera's
//      Schur diagonal block, sum_obs J_c^T A J_c (45 packed entries), and of
//      the reduced rhs, sum_obs J_c^T e (9), each summed over the segment's
//      observations in slot order and written to the camera-major partial
//      record of the segment (54 values).
// Observations are read coalesced in point order; no global atomics.
template <typename real>
struct PointSchurSmem {
  real jc[kChunkCap][18];  // J_c by slot (u, v interleaved per column)
  real ae[kChunkCap][5];   // A00 A01 A11 e_u e_v by slot
  real ci[kChunkCap][6];   // C^-1 by chunk point
  real tp[kChunkCap][3];   // C^-1 g_p by chunk point
  // last, and allocated only with the explicit Schur complement:
  real lc[kChunkCap][6];   // L, L L^T = C^-1: l00 l10 l11 l20 l21 l22
};

// Lower Cholesky factor of a symmetric 3x3 (packed 00 01 02 11 12 22):
// l00 l10 l11 l20 l21 l22, zero where a pivot is not positive.
__device__ __forceinline__ void chol3(const double *A, double *L) {
  const double l00 = A[0] > 0.0 ? sqrt(A[0]) : 0.0;
  const double i00 = l00 > 0.0 ? recip_nr(l00) : 0.0;
  const double l10 = A[1] * i00, l20 = A[2] * i00;
  const double d1 = A[3] - l10 * l10;
  const double l11 = d1 > 0.0 ? sqrt(d1) : 0.0;
  const double i11 = l11 > 0.0 ? recip_nr(l11) : 0.0;
  const double l21 = (A[4] - l20 * l10) * i11;
  const double d2 = A[5] - l20 * l20 - l21 * l21;
  const double l22 = d2 > 0.0 ? sqrt(d2) : 0.0;
  L[0] = l00, L[1] = l10, L[2] = l11, L[3] = l20, L[4] = l21, L[5] = l22;
}

__device__ __forceinline__ void sym9_pair(int e, int &a, int &b) {
  a = 0;
  int r = 9;
  while (e >= r) {
    e -= r;
    --r;
    ++a;
  }
  b = a + e;
}

// (the mixed form at four CTAs per SM: 64 registers a thread)
template <bool MIXED>
__global__ void __launch_bounds__(kChunkCap, MIXED ? 4 : 1) k_point_schur(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  typedef typename Acc<MIXED>::type Acc;
  extern __shared__ __align__(16) unsigned char k3_smem[];
  PointSchurSmem<real> &sm = *reinterpret_cast<PointSchurSmem<real> *>(k3_smem);
  const int t = threadIdx.x;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x) {
    const ChunkInfo ci = B.chunk[ch];
    LMState *L = B.lm + ci.problem;
    if (!L->active) continue;  // uniform over the CTA
    const bool valid = t < ci.obs_count;
    real2 Jc[9], Jp[3];
    int lp = 0, slot = 0;
    if (valid) {
      const int64_t o = ci.obs_begin + t;
#pragma unroll
      for (int q = 0; q < 9; ++q) Jc[q] = jload<real2>(B.jac, B.no, q, o);
#pragma unroll
      for (int q = 0; q < 3; ++q) Jp[q] = jload<real2>(B.jac, B.no, 9 + q, o);
      slot = B.obs_slot[o];
      lp = B.obs_pt[o] - ci.pt_begin;
    }
    if (t < ci.pt_count) {
      const int j = ci.pt_begin + t;
      const double radius = L->radius;
      double C[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) C[q] = B.pt_C[6 * (size_t)j + q];
      C[0] += lm_d2(C[0], radius, B.opt);
      C[3] += lm_d2(C[3], radius, B.opt);
      C[5] += lm_d2(C[5], radius, B.opt);
      double Ci[6];
      if (!spd_inverse3(C, Ci)) {
        L->linear_ok = 0;  // benign race: every writer stores 0
#pragma unroll
        for (int q = 0; q < 6; ++q) Ci[q] = 0.0;
      }
      real *cio = reinterpret_cast<real *>(B.pt_Cinv) + 6 * (size_t)j;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        cio[q] = (real)Ci[q];
        B.pt_Cinv64[6 * (size_t)j + q] = Ci[q];
        sm.ci[t][q] = (real)Ci[q];
      }
      const double *g = B.pt_g + 3 * (size_t)j;
      const double g0 = g[0], g1 = g[1], g2 = g[2];
      const double t0 = Ci[0] * g0 + Ci[1] * g1 + Ci[2] * g2;
      const double t1 = Ci[1] * g0 + Ci[3] * g1 + Ci[4] * g2;
      const double t2 = Ci[2] * g0 + Ci[4] * g1 + Ci[5] * g2;
      B.pt_t[3 * (size_t)j + 0] = t0;
      B.pt_t[3 * (size_t)j + 1] = t1;
      B.pt_t[3 * (size_t)j + 2] = t2;
      sm.tp[t][0] = (real)t0, sm.tp[t][1] = (real)t1, sm.tp[t][2] = (real)t2;
      if (B.explicit_schur) {
        double Lc[6];
        chol3(Ci, Lc);
#pragma unroll
        for (int q = 0; q < 6; ++q) sm.lc[t][q] = (real)Lc[q];
      }
    }
    // the first (segment, entry) task of this thread: its metadata now
    int f_b0 = 0, f_b1 = 0, f_slot = 0;
    if (t < ci.seg_count * 54) {
      const int sg = t / 54;
      f_b0 = B.seg_pos[ci.seg_begin + sg];
      f_b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
      f_slot = B.seg_slot[ci.seg_begin + sg];
    }
    __syncthreads();
    if (valid) {
      const real c0 = sm.ci[lp][0], c1 = sm.ci[lp][1], c2 = sm.ci[lp][2];
      const real c3 = sm.ci[lp][3], c4 = sm.ci[lp][4], c5 = sm.ci[lp][5];
      const real hu0 = c0 * Jp[0].x + c1 * Jp[1].x + c2 * Jp[2].x;
      const real hu1 = c1 * Jp[0].x + c3 * Jp[1].x + c4 * Jp[2].x;
      const real hu2 = c2 * Jp[0].x + c4 * Jp[1].x + c5 * Jp[2].x;
      const real hv0 = c0 * Jp[0].y + c1 * Jp[1].y + c2 * Jp[2].y;
      const real hv1 = c1 * Jp[0].y + c3 * Jp[1].y + c4 * Jp[2].y;
      const real hv2 = c2 * Jp[0].y + c4 * Jp[1].y + c5 * Jp[2].y;
      const real t0 = sm.tp[lp][0], t1 = sm.tp[lp][1], t2 = sm.tp[lp][2];
      sm.ae[slot][0] = Jp[0].x * hu0 + Jp[1].x * hu1 + Jp[2].x * hu2;
      sm.ae[slot][1] = Jp[0].x * hv0 + Jp[1].x * hv1 + Jp[2].x * hv2;
      sm.ae[slot][2] = Jp[0].y * hv0 + Jp[1].y * hv1 + Jp[2].y * hv2;
      sm.ae[slot][3] = Jp[0].x * t0 + Jp[1].x * t1 + Jp[2].x * t2;
      sm.ae[slot][4] = Jp[0].y * t0 + Jp[1].y * t1 + Jp[2].y * t2;
#pragma unroll
      for (int q = 0; q < 9; ++q) sm.jc[slot][2 * q] = Jc[q].x, sm.jc[slot][2 * q + 1] = Jc[q].y;
      if (B.explicit_schur) {
        // F = J_c^T (J_p L) (9x3) with L L^T = C^-1: the explicit
        // complement's blocks are -sum F_a F_b^T over observation pairs.
        // Stored at the observation's camera-major row, 16 bytes at a time.
        const real *Lc = sm.lc[lp];
        real P[2][3];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const real j0 = r ? Jp[0].y : Jp[0].x, j1 = r ? Jp[1].y : Jp[1].x, j2 = r ? Jp[2].y : Jp[2].x;
          P[r][0] = j0 * Lc[0] + j1 * Lc[1] + j2 * Lc[3];
          P[r][1] = j1 * Lc[2] + j2 * Lc[4];
          P[r][2] = j2 * Lc[5];
        }
        real F[kObsF];
#pragma unroll
        for (int q = 0; q < 9; ++q)
#pragma unroll
          for (int m = 0; m < 3; ++m) F[3 * q + m] = Jc[q].x * P[0][m] + Jc[q].y * P[1][m];
        F[27] = (real)0;
        typedef typename std::conditional<MIXED, float4, double2>::type vec;
        constexpr int kVec = (int)(sizeof(vec) / sizeof(real));
        vec *dst = reinterpret_cast<vec *>(reinterpret_cast<real *>(B.obs_F) +
                                           (size_t)kObsF * B.obs_fpos[ci.obs_begin + t]);
#pragma unroll
        for (int e = 0; e < kObsF / kVec; ++e) dst[e] = *reinterpret_cast<const vec *>(&F[kVec * e]);
      }
    }
    __syncthreads();
    real *part = reinterpret_cast<real *>(B.schur_partial);
    for (int i = t; i < ci.seg_count * 54; i += blockDim.x) {
      const int sg = i / 54, en = i - 54 * sg;
      int b0 = f_b0, b1 = f_b1, sl = f_slot;
      if (i != t) {
        b0 = B.seg_pos[ci.seg_begin + sg];
        b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
        sl = B.seg_slot[ci.seg_begin + sg];
      }
      Acc acc;
      acc.init();
      if (en < 45) {
        int a, b;
        sym9_pair(en, a, b);
        for (int k = b0; k < b1; ++k) {
          const real ua = sm.jc[k][2 * a], va = sm.jc[k][2 * a + 1];
          const real ub = sm.jc[k][2 * b], vb = sm.jc[k][2 * b + 1];
          const real A00 = sm.ae[k][0], A01 = sm.ae[k][1], A11 = sm.ae[k][2];
          acc.add(ua * (A00 * ub + A01 * vb) + va * (A01 * ub + A11 * vb));
        }
      } else {
        const int a = en - 45;
        for (int k = b0; k < b1; ++k) acc.add(sm.jc[k][2 * a] * sm.ae[k][3] + sm.jc[k][2 * a + 1] * sm.ae[k][4]);
      }
      part[54 * (size_t)sl + en] = (real)acc.rvalue();
    }
    __syncthreads();
  }
}

// K3a of the FP64 form with the explicit Schur complement.  Per point: C,
// its inverse, t = C^-1 g_p, the factor L (L L^T = C^-1) and u = L^-1 t;
// per observation the rows F = J_c^T (J_p L) (9x3), written for the
// formation kernel K3c and kept by slot; per (camera segment, entry) the
// segment's share of the diagonal block, sum_obs F_a . F_b over its rows
// (W C^-1 W^T = F F^T), and of the reduced rhs, sum_obs F_a . u
// (J_c^T J_p t = F L^-1 t): three FMAs an entry and observation where the
// general kernel's J_c^T A J_c takes seven, GB300's FP64 pipe being what
// bounds this kernel.
struct PointSchurEx64Smem {
  double F[kChunkCap][27];  // F by slot
  double ci[kChunkCap][6];  // C^-1 by chunk point
  double u[kChunkCap][3];   // L^-1 t by chunk point
  double lc[kChunkCap][6];  // L by chunk point
  int spt[kChunkCap];       // chunk point of each slot
};

__global__ void __launch_bounds__(kChunkCap) k_point_schur_ex64(DeviceBatch B) {
  extern __shared__ __align__(16) unsigned char k3x_smem[];
  PointSchurEx64Smem &sm = *reinterpret_cast<PointSchurEx64Smem *>(k3x_smem);
  const int t = threadIdx.x;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x) {
    const ChunkInfo ci = B.chunk[ch];
    LMState *L = B.lm + ci.problem;
    if (!L->active) continue;  // uniform over the CTA
    const bool valid = t < ci.obs_count;
    double2 Jc[9], Jp[3];
    int lp = 0, slot = 0;
    if (valid) {
      const int64_t o = ci.obs_begin + t;
#pragma unroll
      for (int q = 0; q < 9; ++q) Jc[q] = jload<double2>(B.jac, B.no, q, o);
#pragma unroll
      for (int q = 0; q < 3; ++q) Jp[q] = jload<double2>(B.jac, B.no, 9 + q, o);
      slot = B.obs_slot[o];
      lp = B.obs_pt[o] - ci.pt_begin;
      sm.spt[slot] = lp;
    }
    if (t < ci.pt_count) {
      const int j = ci.pt_begin + t;
      const double radius = L->radius;
      double C[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) C[q] = B.pt_C[6 * (size_t)j + q];
      C[0] += lm_d2(C[0], radius, B.opt);
      C[3] += lm_d2(C[3], radius, B.opt);
      C[5] += lm_d2(C[5], radius, B.opt);
      double Ci[6];
      if (!spd_inverse3(C, Ci)) {
        L->linear_ok = 0;  // benign race: every writer stores 0
#pragma unroll
        for (int q = 0; q < 6; ++q) Ci[q] = 0.0;
      }
      double *cio = reinterpret_cast<double *>(B.pt_Cinv) + 6 * (size_t)j;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        cio[q] = Ci[q];
        B.pt_Cinv64[6 * (size_t)j + q] = Ci[q];
        sm.ci[t][q] = Ci[q];
      }
      const double *g = B.pt_g + 3 * (size_t)j;
      const double g0 = g[0], g1 = g[1], g2 = g[2];
      const double t0 = Ci[0] * g0 + Ci[1] * g1 + Ci[2] * g2;
      const double t1 = Ci[1] * g0 + Ci[3] * g1 + Ci[4] * g2;
      const double t2 = Ci[2] * g0 + Ci[4] * g1 + Ci[5] * g2;
      B.pt_t[3 * (size_t)j + 0] = t0;
      B.pt_t[3 * (size_t)j + 1] = t1;
      B.pt_t[3 * (size_t)j + 2] = t2;
      double Lc[6];
      chol3(Ci, Lc);
#pragma unroll
      for (int q = 0; q < 6; ++q) sm.lc[t][q] = Lc[q];
      // u = L^-1 t (forward substitution; a zero pivot gives a zero component)
      const double i00 = Lc[0] > 0.0 ? recip_nr(Lc[0]) : 0.0;
      const double i11 = Lc[2] > 0.0 ? recip_nr(Lc[2]) : 0.0;
      const double i22 = Lc[5] > 0.0 ? recip_nr(Lc[5]) : 0.0;
      const double u0 = t0 * i00;
      const double u1 = (t1 - Lc[1] * u0) * i11;
      const double u2 = (t2 - Lc[3] * u0 - Lc[4] * u1) * i22;
      sm.u[t][0] = u0, sm.u[t][1] = u1, sm.u[t][2] = u2;
    }
    // the first (segment, entry) task of this thread: its metadata now
    int f_b0 = 0, f_b1 = 0, f_slot = 0;
    if (t < ci.seg_count * 54) {
      const int sg = t / 54;
      f_b0 = B.seg_pos[ci.seg_begin + sg];
      f_b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
      f_slot = B.seg_slot[ci.seg_begin + sg];
    }
    __syncthreads();
    if (valid) {
      const double *Lc = sm.lc[lp];
      double P[2][3];
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const double j0 = r ? Jp[0].y : Jp[0].x, j1 = r ? Jp[1].y : Jp[1].x, j2 = r ? Jp[2].y : Jp[2].x;
        P[r][0] = j0 * Lc[0] + j1 * Lc[1] + j2 * Lc[3];
        P[r][1] = j1 * Lc[2] + j2 * Lc[4];
        P[r][2] = j2 * Lc[5];
      }
      double F[kObsF];
#pragma unroll
      for (int q = 0; q < 9; ++q)
#pragma unroll
        for (int m = 0; m < 3; ++m) F[3 * q + m] = Jc[q].x * P[0][m] + Jc[q].y * P[1][m];
      F[27] = 0.0;
#pragma unroll
      for (int e = 0; e < 27; ++e) sm.F[slot][e] = F[e];
      double2 *dst = reinterpret_cast<double2 *>(reinterpret_cast<double *>(B.obs_F) +
                                                 (size_t)kObsF * B.obs_fpos[ci.obs_begin + t]);
#pragma unroll
      for (int e = 0; e < kObsF / 2; ++e) dst[e] = *reinterpret_cast<const double2 *>(&F[2 * e]);
    }
    __syncthreads();
    double *part = reinterpret_cast<double *>(B.schur_partial);
    for (int i = t; i < ci.seg_count * 54; i += blockDim.x) {
      const int sg = i / 54, en = i - 54 * sg;
      int b0 = f_b0, b1 = f_b1, sl = f_slot;
      if (i != t) {
        b0 = B.seg_pos[ci.seg_begin + sg];
        b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
        sl = B.seg_slot[ci.seg_begin + sg];
      }
      double acc = 0.0;
      if (en < 45) {
        int a, b;
        sym9_pair(en, a, b);
        for (int k = b0; k < b1; ++k) {
          const double *fa = sm.F[k] + 3 * a, *fb = sm.F[k] + 3 * b;
          acc = fma(fa[2], fb[2], fma(fa[1], fb[1], fma(fa[0], fb[0], acc)));
        }
      } else {
        const int a = en - 45;
        for (int k = b0; k < b1; ++k) {
          const double *fa = sm.F[k] + 3 * a, *u = sm.u[sm.spt[k]];
          acc = fma(fa[2], u[2], fma(fa[1], u[1], fma(fa[0], u[0], acc)));
        }
      }
      part[54 * (size_t)sl + en] = acc;
    }
    __syncthreads();
  }
}

size_t point_schur_smem(bool mixed) {
  return mixed ? sizeof(PointSchurSmem<float>) : sizeof(PointSchurSmem<double>);
}

void launch_point_prepare(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  // without the explicit Schur complement the factor rows are not allocated
  // (more CTAs per SM in the FP64 form)
  const size_t lcb = b.explicit_schur ? 0 : kChunkCap * 6 * (mixed ? sizeof(float) : sizeof(double));
  if (mixed)
    k_point_schur<true><<<b.nchunks, kChunkCap, point_schur_smem(true) - lcb, s>>>(b);
  else if (b.explicit_schur)
    k_point_schur_ex64<<<b.nchunks, kChunkCap, sizeof(PointSchurEx64Smem), s>>>(b);
  else
    k_point_schur<false><<<b.nchunks, kChunkCap, point_schur_smem(false) - lcb, s>>>(b);
}

// ---------------------------------------------------------------------------
// In-place Gauss-Jordan inverse of a 9x9 SPD matrix in shared memory, one
// thread per entry (threads 0..80; every thread of the CTA must call it).
// Diagonal pivots in order: for an SPD matrix every pivot is a Schur
// complement pivot, positive exactly when the matrix is positive definite,
// so no row exchange is needed.  Step k maps
//   a_kk -> 1/p,  a_kj -> a_kj / p,  a_ik -> -a_ik / p,
//   a_ij -> a_ij - a_ik a_kj / p  (p = a_kk);
// after nine steps the buffer holds A^-1.  Two buffers alternate so one
// barrier per step suffices.  Returns false (in every thread) when a pivot
// is not positive or an entry is not finite.
__device__ bool spd_inverse9_gj(double (*buf)[81]) {
  const int t = threadIdx.x;
  const int i = t / 9, j = t - 9 * (t / 9);
  int cur = 0;
  bool ok = true;
  for (int k = 0; k < 9; ++k) {
    const double p = buf[cur][10 * k];
    if (!(p > 0.0)) ok = false;  // uniform: every thread reads the same pivot
    if (ok && t < 81) {
      const double pinv = recip_nr(p);
      double v;
      if (i == k && j == k)
        v = pinv;
      else if (i == k)
        v = buf[cur][t] * pinv;
      else if (j == k)
        v = -buf[cur][t] * pinv;
      else
        v = fma(-(buf[cur][9 * i + k] * pinv), buf[cur][9 * k + j], buf[cur][t]);
      buf[cur ^ 1][t] = v;
    }
    __syncthreads();
    cur ^= 1;
  }
  const bool fin = t >= 81 || isfinite(buf[cur][t]);
  return __syncthreads_and(fin ? 1 : 0) && ok;
}

// ---------------------------------------------------------------------------
// K3b: one CTA per camera: S_ii = B + Dc^2 - sum of the segment partials,
// reduced rhs v = g_c - sum of the rhs partials, the FP64 inverse of S_ii
// (block-Jacobi preconditioner), and the PCG start (x = 0, r = v, z = M r).
constexpr int kSchurThreads = 96;

template <bool MIXED>
__global__ void __launch_bounds__(kSchurThreads) k_camera_schur(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Acc<MIXED>::type Acc;
  __shared__ double buf[2][81];
  __shared__ double sums[54];
  __shared__ double vec[9];
  __shared__ double red[kSchurThreads / 32];
  __shared__ int flag;
  const int c = blockIdx.x;
  const int p = B.cam_problem[c];
  LMState *L = B.lm + p;
  const int t = threadIdx.x;
  const bool work = L->active != 0;
  if (work) {
    // sums of the camera's segment partials, in segment order (FP64: four
    // interleaved accumulators, combined pairwise)
    if (t < 54) {
      const real *part = reinterpret_cast<const real *>(B.schur_partial) + t;
      const int s0 = B.cam_seg_begin[c], s1 = B.cam_seg_begin[c + 1];
      constexpr int kBatch = 16;
      constexpr int kAcc = MIXED ? 1 : 4;
      Acc a[kAcc];
#pragma unroll
      for (int u = 0; u < kAcc; ++u) a[u].init();
      for (int s = s0; s < s1; s += kBatch) {
        real v[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) v[u] = (s + u < s1) ? part[54 * (size_t)(s + u)] : (real)0;
#pragma unroll
        for (int u = 0; u < kBatch; ++u)
          if (s + u < s1) a[u % kAcc].add(v[u]);
      }
      double sum = a[0].value();
      if (kAcc == 4) sum = (a[0].value() + a[1 % kAcc].value()) + (a[2 % kAcc].value() + a[3 % kAcc].value());
      sums[t] = sum;
    }
    __syncthreads();
    const double radius = L->radius;
    if (t < 81) {
      const int a = t / 9, b = t % 9;
      double v = B.cam_B[45 * (size_t)c + sym9(a, b)] - sums[sym9(a, b)];
      if (a == b) {
        const double d2 = lm_d2(B.cam_B[45 * (size_t)c + sym9(a, a)], radius, B.opt);
        v += d2;
        B.cam_D2[9 * (size_t)c + a] = d2;
      }
      buf[0][t] = v;
      if (B.explicit_schur) reinterpret_cast<real *>(B.cam_Sii)[81 * (size_t)c + t] = (real)v;
    }
    if (t < 9) vec[t] = B.cam_g[9 * (size_t)c + t] - sums[45 + t];
    __syncthreads();
    const bool ok = spd_inverse9_gj(buf);  // result in buf[1] (nine steps)
    if (!ok) {
      if (t == 0) L->linear_ok = 0;
      if (t < 81) buf[1][t] = 0.0;
    }
    __syncthreads();
    double rz = 0.0, rr = 0.0;
    if (t < 9) {
      double z = 0.0;
      for (int k = 0; k < 9; ++k) z += buf[1][t * 9 + k] * vec[k];
      const size_t i = 9 * (size_t)c + t;
      B.pcg_v[i] = vec[t];
      B.pcg_r[i] = vec[t];
      B.pcg_x[i] = 0.0;
      B.pcg_z[i] = z;  // the first direction p_0 = z_0 is formed by the PCG kernels
      if (MIXED) B.pcg_zf[i] = (float)z;
      rz = vec[t] * z;
      rr = vec[t] * vec[t];
    }
    if (t < 81) {
      B.cam_Minv[81 * (size_t)c + t] = buf[1][t];
      if (MIXED) B.cam_Minvf[81 * (size_t)c + t] = (float)buf[1][t];
    }
    if (MIXED && t < 45) B.cam_Bf[45 * (size_t)c + t] = (float)B.cam_B[45 * (size_t)c + t];
    const double rzs = block_sum(rz, red);
    const double rrs = block_sum(rr, red);
    if (t == 0) {
      B.cam_scal[(size_t)kCamScal * c + kCC_RZ] = rzs;
      B.cam_scal[(size_t)kCamScal * c + kCC_RR] = rrs;
    }
    // the problem's last camera CTA starts its PCG
    const ProblemInfo pi = B.prob[p];
    if (last_block_done(B.prob_counter + 4 * p + kPC_SCHUR, (uint32_t)pi.cam_count, &flag)) {
      const double rz0 = block_range_sum(B.cam_scal + kCC_RZ, pi.cam_begin, pi.cam_begin + pi.cam_count, kCamScal, red);
      const double rr0 = block_range_sum(B.cam_scal + kCC_RR, pi.cam_begin, pi.cam_begin + pi.cam_count, kCamScal, red);
      if (t == 0) {
        L->rz = rz0;
        L->r0_norm = sqrt(rr0);
        L->rr = rr0;
        L->beta = 0.0;
        L->alpha = 0.0;
        L->q0 = 0.0;
        L->pcg_iterations = 0;
        L->pcg_active = (L->linear_ok && L->r0_norm > 0.0 && B.opt.max_pcg_iterations > 0) ? 1 : 0;
      }
    }
  }
  // the grid's last CTA sets the PCG loop condition
  if (last_block_done(B.global_counter + kGC_SCHUR, gridDim.x, &flag)) {
    double cnt = 0.0;
    for (int q = t; q < B.num_problems; q += blockDim.x)
      cnt += (__ldcg(&B.lm[q].active) && __ldcg(&B.lm[q].pcg_active)) ? 1.0 : 0.0;
    const int count = (int)block_sum(cnt, red);
    if (B.grid_ctl && t < 8) B.grid_ctl[t] = 0u;  // the grid PCG's control words, before its launch
    if (t == 0) {
      B.status[2] = count > 0 ? 1 : 0;
      B.status[3] = count;
      if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, count > 0 ? 1u : 0u);
    }
  }
}

void launch_camera_schur(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  if (mixed)
    k_camera_schur<true><<<b.nc, kSchurThreads, 0, s>>>(b);
  else
    k_camera_schur<false><<<b.nc, kSchurThreads, 0, s>>>(b);
}

cudaError_t raise_smem_limit(const void *func, size_t bytes) {
  static std::mutex mu;
  static auto *limits = new std::map<std::pair<const void *, int>, size_t>;  // never destroyed
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  size_t &cur = (*limits)[{func, dev}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

// Large dynamic shared memory of the point-Schur kernel (FP64 form).
void point_schur_init() {
  cudaFuncSetAttribute(k_point_schur<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)point_schur_smem(true));
  cudaFuncSetAttribute(k_point_schur<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)point_schur_smem(false));
  cudaFuncSetAttribute(k_point_schur_ex64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PointSchurEx64Smem));
}


// ---------------------------------------------------------------------------
// K5: y_p = C^-1 (g_p - W^T y_c), step = -y, model cost change
// -m.(r + m/2) with m = J step, candidate points x + step * scale.  FP64
// arithmetic in both modes (the acceptance ratio is FP64); in the mixed form
// m.r = step.g comes from the FP64 gradient (step_p.g_p here, step_c.g_c in
// K5b), and only |m|^2 from the FP32 Jacobian copies.
template <bool MIXED>
__global__ void __launch_bounds__(kChunkCap) k_back_substitute(DeviceBatch B) {
  // mixed form: the inner products with the FP32 Jacobian run in FP32; the
  // point step y = C^-1 (g_p - W^T y_c), the candidate points and the model
  // cost change stay FP64
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  __shared__ real yseg[kChunkCap][9];
  __shared__ real W[kChunkCap][3];
  __shared__ real ypt[kChunkCap][3];
  __shared__ double red[kChunkCap / 32];
  const int t = threadIdx.x;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x) {
    const ChunkInfo ci = B.chunk[ch];
    const LMState *L = B.lm + ci.problem;
    if (!L->active || !L->linear_ok) continue;
    const int parity = L->parity;
    for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
      const int s = i / 9, q = i - 9 * s;
      yseg[s][q] = (real)B.pcg_x[9 * (size_t)B.seg_cam[ci.seg_begin + s] + q];
    }
    __syncthreads();
    const bool valid = t < ci.obs_count;
    real Jpu[3], Jpv[3], zu = 0, zv = 0;
    double ru = 0.0, rv = 0.0;
    int lp = 0;
    if (valid) {
      const int64_t o = ci.obs_begin + t;
      const int s = B.obs_seg[o];
      lp = B.obs_pt[o] - ci.pt_begin;
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const real2 J = jload<real2>(B.jac, B.no, q, o);
        zu += J.x * yseg[s][q];
        zv += J.y * yseg[s][q];
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const real2 J = jload<real2>(B.jac, B.no, 9 + q, o);
        Jpu[q] = J.x;
        Jpv[q] = J.y;
        W[t][q] = Jpu[q] * zu + Jpv[q] * zv;
      }
      const real2 r = jload<real2>(B.jac, B.no, 12, o);
      ru = r.x;
      rv = r.y;
    }
    __syncthreads();
    double s2 = 0.0, ymodel = 0.0;
    if (t < ci.pt_count) {
      const int jj = ci.pt_begin + t;
      const int b0 = B.pt_obs_begin[jj] - ci.obs_begin, b1 = B.pt_obs_begin[jj + 1] - ci.obs_begin;
      real w0 = 0, w1 = 0, w2 = 0;
      for (int k = b0; k < b1; ++k) w0 += W[k][0], w1 += W[k][1], w2 += W[k][2];
      const double *g = B.pt_g + 3 * (size_t)jj;
      const double a0 = g[0] - (double)w0, a1 = g[1] - (double)w1, a2 = g[2] - (double)w2;
      const double *Ci = B.pt_Cinv64 + 6 * (size_t)jj;
      const double y0 = Ci[0] * a0 + Ci[1] * a1 + Ci[2] * a2;
      const double y1 = Ci[1] * a0 + Ci[3] * a1 + Ci[4] * a2;
      const double y2 = Ci[2] * a0 + Ci[4] * a1 + Ci[5] * a2;
      ypt[t][0] = (real)y0, ypt[t][1] = (real)y1, ypt[t][2] = (real)y2;
      const double *x = B.pt_param[parity] + 4 * (size_t)jj;
      double *xc = B.pt_param[parity ^ 1] + 4 * (size_t)jj;
      const double *sc = B.pt_scale + 3 * (size_t)jj;
      const double y[3] = {y0, y1, y2};
      const bool used = B.pt_used[jj] != 0;
      if (MIXED && used) ymodel = -(y0 * g[0] + y1 * g[1] + y2 * g[2]);  // step_p.g_p
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const double cand = used ? x[q] + (-y[q]) * sc[q] : x[q];
        const double d = x[q] - cand;
        s2 += used ? d * d : 0.0;
        xc[q] = cand;
      }
    }
    __syncthreads();
    double model = ymodel;
    if (valid) {
      const double m0 = -(double)(zu + Jpu[0] * ypt[lp][0] + Jpu[1] * ypt[lp][1] + Jpu[2] * ypt[lp][2]);
      const double m1 = -(double)(zv + Jpv[0] * ypt[lp][0] + Jpv[1] * ypt[lp][1] + Jpv[2] * ypt[lp][2]);
      // mixed form: m.r = step.g is taken from the FP64 gradient (point part
      // above, camera part in K5b); only |m|^2 / 2 comes from the FP32 copies
      model += MIXED ? (m0 * m0 + m1 * m1) / 2.0 : m0 * (ru + m0 / 2.0) + m1 * (rv + m1 / 2.0);
    }
    const double ms = block_sum(model, red);
    const double ss = block_sum(s2, red);
    if (t == 0) {
      B.chunk_scal[(size_t)kChunkScal * ch + kCS_MODEL] = ms;
      B.chunk_scal[(size_t)kChunkScal * ch + kCS_STEP2] = ss;
    }
  }
}

void launch_back_substitute(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  if (mixed)
    k_back_substitute<true><<<b.nchunks, kChunkCap, 0, s>>>(b);
  else
    k_back_substitute<false><<<b.nchunks, kChunkCap, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// K6: one CTA per problem.  Ceres' TrustRegionMinimizer step handling:
// invalid step (linear solve failed or model_cost_change <= 0), parameter
// tolerance, function tolerance, step quality vs min_relative_decrease,
// LevenbergMarquardtStrategy radius update.
__device__ __forceinline__ void terminate_(LMState *L, int type, int reason) {
  L->active = 0;
  L->termination_type = type;
  L->termination_reason = reason;
}

// g2o's Levenberg trial (OptimizationAlgorithmLevenberg, lambda = 1 / radius):
// gain rho = (chi2 - chi2') / (dx.(lambda dx + b) + 1e-3) with chi2 = 2 cost
// and dx.(lambda dx + b) = 2 model_cost_change for the solved step; accept
// when rho > 0 (lambda *= max(1/3, min(2/3, 1 - (2 rho - 1)^3))), else
// lambda *= nu, nu *= 2.  The iteration's trials end at the first accepted
// step (K7 then applies the limits at the new point) or after
// kG2oMaxTrials; a trial with rho == 0 or lambda no longer finite ends the
// solve.
__device__ void decide_g2o(const DeviceBatch &B, int p, LMState *L, int it, int pcg, bool valid, double model,
                           double cand, double bad, double step2) {
  double rho = -1.0;
  if (!valid) {
    ++L->invalid_steps;
  } else {
    const double cost = (bad != 0.0 || !isfinite(cand)) ? DBL_MAX : cand;
    L->candidate_cost = cost;
    L->step_norm = sqrt(step2);
    rho = (cost >= DBL_MAX) ? -DBL_MAX : 2.0 * (L->x_cost - cost) / (2.0 * model + 1e-3);
    L->relative_decrease = rho;
    if (rho > 0.0) {
      L->parity ^= 1;
      L->need_jacobian = 1;
      L->x_cost = cost;
      const double tq = 2.0 * rho - 1.0;
      L->radius = fmin(DBL_MAX, L->radius / fmax(1.0 / 3.0, fmin(2.0 / 3.0, 1.0 - tq * tq * tq)));
      L->decrease_factor = 2.0;
      ++L->successful_steps;
      ++L->trials;
      ++L->outer;
      return;
    }
  }
  ++L->unsuccessful_steps;
  L->radius /= L->decrease_factor;
  L->decrease_factor *= 2.0;
  trace_put(B, p, it, valid ? L->candidate_cost : L->x_cost, L->radius, pcg, 0);
  if (++L->trials >= kG2oMaxTrials || rho == 0.0 || L->radius <= 0.0)
    terminate_(L, GBA_TERMINATION_CONVERGENCE, GBA_REASON_LM_TRIALS);
}

__global__ void __launch_bounds__(256) k_decide(DeviceBatch B) {
  __shared__ double red[8 * 6];
  const int p = blockIdx.x;
  LMState *L = B.lm + p;
  if (!L->active) return;
  const ProblemInfo pi = B.prob[p];
  const int c0 = pi.chunk_begin, c1 = pi.chunk_begin + pi.chunk_count;
  const int k0 = pi.cam_begin, k1 = pi.cam_begin + pi.cam_count;
  // model cost change -(m.r + |m|^2 / 2) summed (the mixed form adds its
  // camera part of m.r = step.g), candidate cost, bad, |step|^2 (points,
  // cameras): one pass
  const double *cs = B.chunk_scal;
  const double *const a[6] = {cs + kCS_MODEL, B.cam_scal + kCC_YG, cs + kCS_COST, cs + kCS_BAD, cs + kCS_STEP2,
                              B.cam_scal + kCC_STEP2};
  const int b[6] = {c0, k0, c0, c0, c0, k0};
  const int e[6] = {c1, B.opt.mixed ? k1 : k0, c1, c1, c1, k1};
  const int st[6] = {kChunkScal, kCamScal, kChunkScal, kChunkScal, kChunkScal, kCamScal};
  const bool mx[6] = {false, false, false, true, false, false};
  double r[6];
  block_range_multi<6>(a, b, e, st, mx, r, red);
  double model = -r[0];
  if (B.opt.mixed) model -= r[1];
  const double cand = r[2], bad = r[3], s2p = r[4], s2c = r[5];
  if (threadIdx.x != 0) return;
  const DeviceOptions &o = B.opt;
  const int it = ++L->iteration;
  const int pcg = L->pcg_iterations;
  L->total_pcg_iterations += pcg;
  const bool lin_ok = L->linear_ok != 0;
  L->last_linear_ok = lin_ok ? 1 : 0;
  L->linear_ok = 1;
  L->pcg_active = 0;
  const bool valid = lin_ok && model > 0.0 && isfinite(model);
  L->model_cost_change = model;
  if (o.g2o) {
    decide_g2o(B, p, L, it, pcg, valid, model, cand, bad, s2p + s2c);
    return;
  }
  if (!valid) {
    ++L->invalid_steps;
    ++L->unsuccessful_steps;
    if (++L->invalid_run >= o.max_invalid_steps) {
      trace_put(B, p, it, L->x_cost, L->radius, pcg, 0);
      terminate_(L, GBA_TERMINATION_FAILURE, GBA_REASON_INVALID_STEPS);
      return;
    }
    L->radius /= L->decrease_factor;
    L->decrease_factor *= 2.0;
    trace_put(B, p, it, L->x_cost, L->radius, pcg, 0);
  } else {
    L->invalid_run = 0;
    const double cost = (bad != 0.0 || !isfinite(cand)) ? DBL_MAX : cand;
    L->candidate_cost = cost;
    const double step_norm = sqrt(s2p + s2c);
    L->step_norm = step_norm;
    if (step_norm <= o.parameter_tolerance * (L->x_norm + o.parameter_tolerance)) {
      ++L->unsuccessful_steps;
      trace_put(B, p, it, cost, L->radius, pcg, 0);
      terminate_(L, GBA_TERMINATION_CONVERGENCE, GBA_REASON_PARAMETER_TOLERANCE);
      return;
    }
    if (fabs(L->x_cost - cost) <= o.function_tolerance * L->x_cost) {
      ++L->unsuccessful_steps;
      trace_put(B, p, it, cost, L->radius, pcg, 0);
      terminate_(L, GBA_TERMINATION_CONVERGENCE, GBA_REASON_FUNCTION_TOLERANCE);
      return;
    }
    const double rel = (cost >= DBL_MAX) ? -DBL_MAX : (L->x_cost - cost) / model;
    L->relative_decrease = rel;
    if (rel > o.min_relative_decrease) {
      // accepted: the candidate buffer becomes current, J is re-evaluated
      // there (K0/K1/K1c), and K7 runs the post-step termination tests.
      L->parity ^= 1;
      L->need_jacobian = 1;
      L->x_cost = cost;
      const double tq = 2.0 * rel - 1.0;
      L->radius = fmin(o.max_radius, L->radius / fmax(1.0 / 3.0, 1.0 - tq * tq * tq));
      L->decrease_factor = 2.0;
      ++L->successful_steps;
      return;
    }
    ++L->unsuccessful_steps;
    L->radius /= L->decrease_factor;
    L->decrease_factor *= 2.0;
    trace_put(B, p, it, cost, L->radius, pcg, 0);
  }
  if (it >= o.max_iterations)
    terminate_(L, GBA_TERMINATION_NO_CONVERGENCE, GBA_REASON_MAX_ITERATIONS);
  else if (L->radius <= o.min_radius)
    terminate_(L, GBA_TERMINATION_CONVERGENCE, GBA_REASON_MIN_TRUST_REGION_RADIUS);
}

void launch_decide(const DeviceBatch &b, cudaStream_t s) { k_decide<<<b.num_problems, 256, 0, s>>>(b); }

}  // namespace gba
