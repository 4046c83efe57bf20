// k_eval.cu — evaluation kernels of the GB300 bundle-adjustment solver.
//
//  K0  k_camera_table   per camera: R, dR/dw (dual-number Rodrigues), t, f, k1, k2
//  K1  k_eval_chunk     per point-segment chunk, one thread per observation:
//                       residual, analytic Jacobian (== the dual-number
//                       Jacobian of SnavelyReprojectionError.h:42-87),
//                       loss corrector, Jacobi scaling, J stored SoA; point
//                       blocks J_p^T J_p and J_p^T r reduced per point in
//                       shared memory (points own contiguous observations).
//  K1c k_eval_camera    per camera (CTA): J_c^T J_c (45) and J_c^T r over the
//                       camera's observations, fixed-order CTA reduction (the
//                       mixed form's J_c^T r: a sum of K1's FP64 segment
//                       partials).
//  K7  k_post_eval      per problem: cost, gradient max-norm, |x|, Ceres'
//                       termination tests, LM-loop condition.
//  K5b k_candidate      per camera: candidate camera + its table (R only).
//  K2  k_cost_chunk     per chunk: candidate cost in FP64.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "kernels.h"

namespace gba {

// ---------------------------------------------------------------------------
__global__ void k_init_state(DeviceBatch B) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= B.num_problems) return;
  LMState L;
  memset(&L, 0, sizeof L);
  L.radius = B.opt.initial_radius;
  L.decrease_factor = 2.0;
  L.active = B.prob[p].obs_count > 0 ? 1 : 0;
  L.termination_type = L.active ? -1 : GBA_TERMINATION_CONVERGENCE;
  L.need_jacobian = 1;
  L.parity = 0;
  L.linear_ok = 1;
  L.last_linear_ok = 1;
  if (B.prob_resume && B.prob_resume[p]) {
    // a problem continued from an LM-iteration boundary of another batch:
    // its state as it was, the Jacobian to be evaluated again at its current
    // point (uploaded as this batch's initial point)
    L = B.lm_resume[p];
    L.need_jacobian = 1;
    L.parity = 0;
    L.resumed = 1;
  }
  B.lm[p] = L;
}

void launch_init_state(const DeviceBatch &b, cudaStream_t s) {
  k_init_state<<<(b.num_problems + 127) / 128, 128, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// K0
__global__ void k_camera_table(DeviceBatch B) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.nc) return;
  const LMState *L = B.lm + B.cam_problem[c];
  if (!L->active || !L->need_jacobian) return;
  double *tab = B.cam_table + (size_t)kCamTable * c;
  camera_table_entry(B.cam_param[L->parity] + 9 * (size_t)c, tab, true);
  if (B.opt.so3_left) so3_left_derivatives(tab);
  if (B.opt.mixed) {
    float *tf = B.cam_tablef + (size_t)kCamTable * c;
    float2 *td = B.cam_tabledf + (size_t)kCamTable * c;
    for (int k = 0; k < kCamTable; ++k) {
      const DF d = df_from_double(tab[k]);
      tf[k] = d.hi;
      td[k] = make_float2(d.hi, d.lo);
    }
  }
}

// One warp per block: the per-camera work is FP64 (sin, cos, the dual-number
// derivatives), and GB300's FP64 rate is per SM, so small warps spread the
// cameras over more SMs.
constexpr int kCamTableThreads = 32;

void launch_camera_table(const DeviceBatch &b, cudaStream_t s) {
  k_camera_table<<<(b.nc + kCamTableThreads - 1) / kCamTableThreads, kCamTableThreads, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// Local-BA windows: residual, the reference's Jacobian (rig_jacobian), the
// loss corrector and the Jacobi scaling of one observation, in FP64 (the
// windows are small; both precision forms take their copies from here).
__device__ __forceinline__ double eval_rig(const DeviceBatch &B, int64_t o, int c, int j, const double *X,
                                           bool unit_scale, double ju[12], double jv[12], double &ru, double &rv,
                                           bool &ok) {
  const double *tab = B.cam_table + (size_t)kCamTable * c;
  const double *rig = B.prob_rig + (size_t)kRig * B.cam_problem[c];
  rig_jacobian(tab, rig, B.obs_rig[o], X, B.obs_uv[o], ju, jv, ru, rv);
  const int loss = B.opt.loss;
  const double cost = block_cost(loss, B.opt.loss_scale, ru, rv);
  if (loss != GBA_LOSS_TRIVIAL) {
    const Corrector cr = make_corrector(loss, B.opt.loss_scale, ru, rv);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      const double rJ = ru * ju[k] + rv * jv[k];
      ju[k] = cr.sqrt_rho1 * (ju[k] - cr.alpha_sq_norm * ru * rJ);
      jv[k] = cr.sqrt_rho1 * (jv[k] - cr.alpha_sq_norm * rv * rJ);
    }
    ru *= cr.residual_scaling;
    rv *= cr.residual_scaling;
  }
  ok = isfinite(ru) && isfinite(rv) && isfinite(cost);
  if (!unit_scale) {
    const double *sc = B.cam_scale + 9 * (size_t)c, *sp = B.pt_scale + 3 * (size_t)j;
#pragma unroll
    for (int k = 0; k < 9; ++k) ju[k] *= sc[k], jv[k] *= sc[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) ju[9 + k] *= sp[k], jv[9 + k] *= sp[k];
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) ok = ok && isfinite((float)ju[k]) && isfinite((float)jv[k]);
  return cost;
}

// Residual + Jacobian of one observation.  Jc[k] = (d r_u, d r_v)/d cam_k,
// Jp[k] = (d r_u, d r_v)/d X_k, r = corrected residual; scaled by the Jacobi
// scaling.  Returns 0.5*rho(|r|^2) (FP64).  *bad = 1 on a non-finite value.
template <bool MIXED>
__device__ __forceinline__ double eval_observation(const DeviceBatch &B, int64_t o, int c, int j,
                                                   const double *X, bool unit_scale,
                                                   typename Prec<MIXED>::real2 *Jc,
                                                   typename Prec<MIXED>::real2 *Jp,
                                                   typename Prec<MIXED>::real2 &r, bool &bad) {
  typedef typename Prec<MIXED>::real real;
  if (B.opt.pinhole) {
    double jd[12], kd[12], rud, rvd;
    bool ok;
    const double cost = eval_rig(B, o, c, j, X, unit_scale, jd, kd, rud, rvd, ok);
#pragma unroll
    for (int k = 0; k < 9; ++k) Jc[k] = mk2((real)jd[k], (real)kd[k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) Jp[k] = mk2((real)jd[9 + k], (real)kd[9 + k]);
    r = mk2((real)rud, (real)rvd);
    bad = !ok;
    return cost;
  }
  const double *tab = B.cam_table + (size_t)kCamTable * c;
  // the Jacobian reads the table and the scales in its own precision (an
  // FP32 copy in the mixed form: no FP64 conversions per observation)
  const real *tr = reinterpret_cast<const real *>(MIXED ? (const void *)(B.cam_tablef + (size_t)kCamTable * c)
                                                        : (const void *)tab);
  Proj pr;
  project(tab, X, B.obs_uv[o], pr);
  // d prediction / dP = f * M * dxy  (x' = -P_x/P_z, y' = -P_y/P_z)
  const real iz = (real)pr.iz;
  const real xp = (real)pr.xp, yp = (real)pr.yp, r2 = (real)pr.r2, dist = (real)pr.dist;
  const real f = (real)pr.f, k1 = (real)pr.k1, k2 = (real)pr.k2;
  const real g = k1 + (real)2 * k2 * r2;
  const real m00 = dist + (real)2 * g * xp * xp;
  const real m01 = (real)2 * g * xp * yp;
  const real m11 = dist + (real)2 * g * yp * yp;
  const real A00 = -f * m00 * iz, A01 = -f * m01 * iz, A02 = -f * (m00 * xp + m01 * yp) * iz;
  const real A10 = -f * m01 * iz, A11 = -f * m11 * iz, A12 = -f * (m01 * xp + m11 * yp) * iz;
  real ju[12], jv[12];
  const real Xr[3] = {(real)X[0], (real)X[1], (real)X[2]};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // dP/dw_k = dR_k X
    const real *d = tr + 9 + 9 * k;
    const real q0 = d[0] * Xr[0] + d[1] * Xr[1] + d[2] * Xr[2];
    const real q1 = d[3] * Xr[0] + d[4] * Xr[1] + d[5] * Xr[2];
    const real q2 = d[6] * Xr[0] + d[7] * Xr[1] + d[8] * Xr[2];
    ju[k] = A00 * q0 + A01 * q1 + A02 * q2;
    jv[k] = A10 * q0 + A11 * q1 + A12 * q2;
    // dP/dX_k = R[:,k]
    const real c0 = tr[k], c1 = tr[3 + k], c2 = tr[6 + k];
    ju[9 + k] = A00 * c0 + A01 * c1 + A02 * c2;
    jv[9 + k] = A10 * c0 + A11 * c1 + A12 * c2;
  }
  ju[3] = A00, ju[4] = A01, ju[5] = A02;
  jv[3] = A10, jv[4] = A11, jv[5] = A12;
  ju[6] = dist * xp, jv[6] = dist * yp;
  ju[7] = f * r2 * xp, jv[7] = f * r2 * yp;
  ju[8] = f * (r2 * r2) * xp, jv[8] = f * (r2 * r2) * yp;
  // robust-loss corrector (FP64 scalars)
  const int loss = B.opt.loss;
  const double cost = block_cost(loss, B.opt.loss_scale, pr.ru, pr.rv);
  double ru = pr.ru, rv = pr.rv;
  if (loss != GBA_LOSS_TRIVIAL) {
    const Corrector cr = make_corrector(loss, B.opt.loss_scale, ru, rv);
    const real s1 = (real)cr.sqrt_rho1, al = (real)cr.alpha_sq_norm;
    const real rur = (real)ru, rvr = (real)rv;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      const real rJ = rur * ju[k] + rvr * jv[k];
      ju[k] = s1 * (ju[k] - al * rur * rJ);
      jv[k] = s1 * (jv[k] - al * rvr * rJ);
    }
    ru *= cr.residual_scaling;
    rv *= cr.residual_scaling;
  }
  bool ok = isfinite(ru) && isfinite(rv) && isfinite(cost);
  if (!unit_scale) {
    const real *sc = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_scalef : (const void *)B.cam_scale) +
                     9 * (size_t)c;
    const real *sp = reinterpret_cast<const real *>(MIXED ? (const void *)B.pt_scalef : (const void *)B.pt_scale) +
                     3 * (size_t)j;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      ju[k] *= sc[k];
      jv[k] *= sc[k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      ju[9 + k] *= sp[k];
      jv[9 + k] *= sp[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    Jc[k] = mk2(ju[k], jv[k]);
    ok = ok && isfinite(ju[k]) && isfinite(jv[k]);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    Jp[k] = mk2(ju[9 + k], jv[9 + k]);
    ok = ok && isfinite(ju[9 + k]) && isfinite(jv[9 + k]);
  }
  r = mk2((real)ru, (real)rv);
  bad = !ok;
  return cost;
}

// ---------------------------------------------------------------------------
// The same residual and Jacobian for the mixed form's gradient: the
// projection (cost, residual) in FP64, the chain rule in double-float (two
// floats, about 48 bits: GB300 issues FP32 some 64 times faster than FP64)
// from the double-float copies of the camera table and the Jacobi scales.
// Returns the FP32 Jacobian (the nearest floats) and residual, and per
// column J^T r (double-float).
__device__ __forceinline__ DF operator+(DF a, DF b) { return df_add(a, b); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ DF operator*(DF a, DF b) { return df_mul(a, b); }
__device__ __forceinline__ DF operator-(DF a) { return df_neg(a); }
// 1 / b in double-float: a float quotient and one correction step
__device__ __forceinline__ DF df_recip(DF b) {
  const float q1 = __fdiv_rn(1.f, b.hi);
  const DF r = df_add(DF{1.f, 0.f}, df_neg(df_mul_f(b, q1)));
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return df_fast_two_sum(q1, q2);
}

// cost64: the projection and the cost in FP64 (the first evaluation of a
// problem, whose cost starts the LM); otherwise the projection runs in
// double-float from the double-float camera table and the cost is not
// formed (0): the LM keeps the FP64 cost of the candidate evaluation (K2)
// that made this point current.  The residual then carries ~2^-44 of the
// predicted pixel, far below what the FP32-stored Jacobian and Schur
// products resolve.
__device__ __forceinline__ double eval_observation_df(const DeviceBatch &B, int64_t o, int c, int j,
                                                      const double *X, float2 *Jc, float2 *Jp, float2 &r,
                                                      DF *gr, bool &bad, bool cost64) {
  if (B.opt.pinhole) {
    double jd[12], kd[12], rud, rvd;
    bool ok;
    const double cost = eval_rig(B, o, c, j, X, false, jd, kd, rud, rvd, ok);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      gr[k] = df_from_double(jd[k] * rud + kd[k] * rvd);
      const float2 jk = make_float2((float)jd[k], (float)kd[k]);
      if (k < 9)
        Jc[k] = jk;
      else
        Jp[k - 9] = jk;
    }
    r = make_float2((float)rud, (float)rvd);
    bad = !ok;
    return cost;
  }
  const double *tab = B.cam_table + (size_t)kCamTable * c;
  const float2 *td = B.cam_tabledf + (size_t)kCamTable * c;
  auto T = [&](int k) {
    const float2 v = td[k];
    return DF{v.x, v.y};
  };
  const DF f = T(39), k1 = T(40), k2 = T(41);
  const DF Xd[3] = {df_from_double(X[0]), df_from_double(X[1]), df_from_double(X[2])};
  DF iz, xp, yp, r2, dist;
  double ru, rv, cost = 0.0;
  if (cost64) {
    Proj pr;
    project(tab, X, B.obs_uv[o], pr);
    iz = df_from_double(pr.iz), xp = df_from_double(pr.xp), yp = df_from_double(pr.yp);
    r2 = df_from_double(pr.r2), dist = df_from_double(pr.dist);
    ru = pr.ru, rv = pr.rv;
    cost = block_cost(B.opt.loss, B.opt.loss_scale, ru, rv);
  } else {
    DF P[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) P[i] = T(3 * i) * Xd[0] + T(3 * i + 1) * Xd[1] + T(3 * i + 2) * Xd[2] + T(36 + i);
    iz = df_recip(P[2]);
    xp = -(P[0] * iz), yp = -(P[1] * iz);
    r2 = xp * xp + yp * yp;
    dist = DF{1.f, 0.f} + r2 * (k1 + k2 * r2);
    const DF fd = f * dist;
    const double2 uv = B.obs_uv[o];
    ru = df_value(fd * xp - df_from_double(uv.x));
    rv = df_value(fd * yp - df_from_double(uv.y));
  }
  const DF two{2.f, 0.f};
  const DF g = k1 + two * k2 * r2;
  const DF m00 = dist + two * g * xp * xp;
  const DF m01 = two * g * xp * yp;
  const DF m11 = dist + two * g * yp * yp;
  const DF fiz = f * iz;
  const DF A00 = -(fiz * m00), A01 = -(fiz * m01), A02 = -(fiz * (m00 * xp + m01 * yp));
  const DF A10 = -(fiz * m01), A11 = -(fiz * m11), A12 = -(fiz * (m01 * xp + m11 * yp));
  DF ju[12], jv[12];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // dP/dw_k = dR_k X
    const int d = 9 + 9 * k;
    const DF q0 = T(d + 0) * Xd[0] + T(d + 1) * Xd[1] + T(d + 2) * Xd[2];
    const DF q1 = T(d + 3) * Xd[0] + T(d + 4) * Xd[1] + T(d + 5) * Xd[2];
    const DF q2 = T(d + 6) * Xd[0] + T(d + 7) * Xd[1] + T(d + 8) * Xd[2];
    ju[k] = A00 * q0 + A01 * q1 + A02 * q2;
    jv[k] = A10 * q0 + A11 * q1 + A12 * q2;
    // dP/dX_k = R[:,k]
    const DF c0 = T(k), c1 = T(3 + k), c2 = T(6 + k);
    ju[9 + k] = A00 * c0 + A01 * c1 + A02 * c2;
    jv[9 + k] = A10 * c0 + A11 * c1 + A12 * c2;
  }
  ju[3] = A00, ju[4] = A01, ju[5] = A02;
  jv[3] = A10, jv[4] = A11, jv[5] = A12;
  ju[6] = dist * xp, jv[6] = dist * yp;
  ju[7] = f * r2 * xp, jv[7] = f * r2 * yp;
  ju[8] = f * (r2 * r2) * xp, jv[8] = f * (r2 * r2) * yp;
  const int loss = B.opt.loss;
  if (loss != GBA_LOSS_TRIVIAL) {
    const Corrector cr = make_corrector(loss, B.opt.loss_scale, ru, rv);
    const DF s1 = df_from_double(cr.sqrt_rho1), al = df_from_double(cr.alpha_sq_norm);
    const DF rur = df_from_double(ru), rvr = df_from_double(rv);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      const DF rJ = rur * ju[k] + rvr * jv[k];
      ju[k] = s1 * (ju[k] - al * rur * rJ);
      jv[k] = s1 * (jv[k] - al * rvr * rJ);
    }
    ru *= cr.residual_scaling;
    rv *= cr.residual_scaling;
  }
  bool ok = isfinite(ru) && isfinite(rv) && isfinite(cost);
  const float2 *sc = B.cam_scaledf + 9 * (size_t)c;
  const float2 *sp = B.pt_scaledf + 3 * (size_t)j;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const DF s{sc[k].x, sc[k].y};
    ju[k] = ju[k] * s;
    jv[k] = jv[k] * s;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const DF s{sp[k].x, sp[k].y};
    ju[9 + k] = ju[9 + k] * s;
    jv[9 + k] = jv[9 + k] * s;
  }
  const DF rdu = df_from_double(ru), rdv = df_from_double(rv);
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    gr[k] = ju[k] * rdu + jv[k] * rdv;
    ok = ok && isfinite(ju[k].hi) && isfinite(jv[k].hi);
    const float2 jk = make_float2(ju[k].hi, jv[k].hi);
    if (k < 9)
      Jc[k] = jk;
    else
      Jp[k - 9] = jk;
  }
  r = make_float2(rdu.hi, rdv.hi);
  bad = !ok;
  return cost;
}

// ---------------------------------------------------------------------------
// K1
// The mixed form's gradient (G64): the Jacobian is computed in double-float
// (eval_observation_df) and only stored in FP32.  The gradient J^T r is a sum
// of large terms that cancel towards zero as the solve converges, so it is
// formed from the double-float Jacobian in double-float: per point (g_p)
// here, and per camera as one partial per (chunk, camera segment) in
// seg_grad (FP64), summed per camera by K1c.  After a problem's first
// evaluation the residual itself is projected in double-float (the cost
// then comes from the FP64 candidate evaluation), so the LM fixed point
// (g = 0) is the FP64 one to double-float rounding; the FP32 copies only
// feed the Schur products and the PCG, i.e. the accuracy of each step, not
// where the steps lead.
// The per-iteration pass (not the first evaluation's column norms) at three
// CTAs per SM (80 registers a thread, a few spilled) instead of two (122-128):
// the mixed pass waits mostly at its CTA barriers (13 % off on configuration
// 2), the FP64 pass hides more of its FP64 latency (6 % off on configuration
// 2, 1.5 % on configuration 1).
template <bool MIXED, bool NORMS>
__global__ void __launch_bounds__(kChunkCap, !NORMS ? 3 : 1) k_eval_chunk(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  typedef typename Acc<MIXED>::type Acc;
  constexpr bool G64 = MIXED && !NORMS;
  __shared__ real sm[kChunkCap][9];
  // G64: per observation its FP64 J_c^T r (9, at its camera-sorted slot) and
  // J_p^T r (3, at its position)
  __shared__ DF gsm[G64 ? kChunkCap : 1][12];
  __shared__ double red[kChunkCap / 32];
  const int t = threadIdx.x;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x) {
    const ChunkInfo ci = B.chunk[ch];
    const LMState *L = B.lm + ci.problem;
    if (!L->active || !L->need_jacobian) continue;  // uniform over the CTA
    const int parity = L->parity;
    double cost = 0.0;
    bool bad = false;
    if (t < ci.obs_count) {
      const int64_t o = ci.obs_begin + t;
      const int c = B.obs_cam[o], j = B.obs_pt[o];
      const double *Xp = B.pt_param[parity] + 4 * (size_t)j;
      const double X[3] = {Xp[0], Xp[1], Xp[2]};
      real2 Jc[9], Jp[3], r;
      if (G64) {
        float2 Jcf[9], Jpf[3], rf;
        DF gr[12];
        cost = eval_observation_df(B, o, c, j, X, Jcf, Jpf, rf, gr, bad, L->iteration == 0 && L->resumed == 0);
        const int slot = B.obs_slot[o];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          Jc[k] = mk2((real)Jcf[k].x, (real)Jcf[k].y);
          gsm[slot][k] = gr[k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          Jp[k] = mk2((real)Jpf[k].x, (real)Jpf[k].y);
          gsm[t][9 + k] = gr[9 + k];
        }
        r = mk2((real)rf.x, (real)rf.y);
      } else {
        cost = eval_observation<MIXED>(B, o, c, j, X, NORMS, Jc, Jp, r, bad);
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) jstore(B.jac, B.no, k, o, Jc[k]);
#pragma unroll
      for (int k = 0; k < 3; ++k) jstore(B.jac, B.no, 9 + k, o, Jp[k]);
      jstore(B.jac, B.no, 12, o, r);
      // point-block contributions: C (sym3) and g
#pragma unroll
      for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int b = a; b < 3; ++b) sm[t][sym3(a, b)] = Jp[a].x * Jp[b].x + Jp[a].y * Jp[b].y;
        sm[t][6 + a] = Jp[a].x * r.x + Jp[a].y * r.y;
      }
    }
    // G64: the first (segment, coordinate) camera-gradient sum of this thread
    int f_b0 = 0, f_b1 = 0, f_slot = 0;
    if (G64 && t < ci.seg_count * 9) {
      const int sg = t / 9;
      f_b0 = B.seg_pos[ci.seg_begin + sg];
      f_b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
      f_slot = B.seg_slot[ci.seg_begin + sg];
    }
    __syncthreads();
    if (G64) {
      for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
        const int sg = i / 9, q = i - 9 * sg;
        int b0 = f_b0, b1 = f_b1, slot9 = f_slot;
        if (i != t) {
          b0 = B.seg_pos[ci.seg_begin + sg];
          b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
          slot9 = B.seg_slot[ci.seg_begin + sg];
        }
        DF a = df_zero();
        for (int k = b0; k < b1; ++k) a = df_add(a, gsm[k][q]);
        B.seg_grad[9 * (size_t)slot9 + q] = df_value(a);
      }
    }
    double gmax = 0.0, xn2 = 0.0;
    if (t < ci.pt_count) {
      const int jj = ci.pt_begin + t;
      const int b0 = B.pt_obs_begin[jj] - ci.obs_begin, b1 = B.pt_obs_begin[jj + 1] - ci.obs_begin;
      Acc acc[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) acc[q].init();
      DF g64[3] = {df_zero(), df_zero(), df_zero()};
      for (int k = b0; k < b1; ++k) {
#pragma unroll
        for (int q = 0; q < (G64 ? 6 : 9); ++q) acc[q].add(sm[k][q]);
        if (G64) {
#pragma unroll
          for (int q = 0; q < 3; ++q) g64[q] = df_add(g64[q], gsm[k][9 + q]);
        }
      }
      if (NORMS) {
        B.pt_colnorm[3 * (size_t)jj + 0] = (double)acc[0].rvalue();
        B.pt_colnorm[3 * (size_t)jj + 1] = (double)acc[3].rvalue();
        B.pt_colnorm[3 * (size_t)jj + 2] = (double)acc[5].rvalue();
      } else {
#pragma unroll
        for (int q = 0; q < 6; ++q) B.pt_C[6 * (size_t)jj + q] = (double)acc[q].rvalue();
        if (B.pt_used[jj]) {
          const double *x = B.pt_param[parity] + 4 * (size_t)jj;
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const double gq = G64 ? df_value(g64[q]) : acc[6 + q].value();
            B.pt_g[3 * (size_t)jj + q] = gq;
            const double gu = gq / B.pt_scale[3 * (size_t)jj + q];
            gmax = fmax(gmax, fabs(x[q] - (x[q] - gu)));
            xn2 += x[q] * x[q];
          }
        } else {
#pragma unroll
          for (int q = 0; q < 3; ++q) B.pt_g[3 * (size_t)jj + q] = 0.0;
        }
      }
    }
    if (!NORMS) {
      // the mixed form's later evaluations form no cost (eval_observation_df)
      const bool with_cost = !G64 || (L->iteration == 0 && !L->resumed);
      const double cs = with_cost ? block_sum(cost, red) : 0.0;
      const double gm = block_max(gmax, red);
      const double xs = block_sum(xn2, red);
      const double bd = block_max(bad ? 1.0 : 0.0, red);
      if (t == 0) {
        double *cs_out = B.chunk_scal + (size_t)kChunkScal * ch;
        cs_out[kCS_COST] = cs;
        cs_out[kCS_GMAX] = gm;
        cs_out[kCS_XN2] = xs;
        cs_out[kCS_BAD] = bd;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// K1c: one CTA per camera.
constexpr int kCamThreads = 128;

template <bool MIXED, bool NORMS>
__global__ void __launch_bounds__(kCamThreads) k_eval_camera(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  typedef typename Acc<MIXED>::type Acc;
  constexpr int NV = NORMS ? 9 : 54;
  __shared__ double part[kCamThreads / 32][NV];
  __shared__ DF partf[MIXED ? kCamThreads / 32 : 1][NV];
  const int c = blockIdx.x;
  const LMState *L = B.lm + B.cam_problem[c];
  if (!L->active || !L->need_jacobian) return;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  Acc acc[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) acc[q].init();
  const int e = B.cam_obs_begin[c + 1];
  for (int k = B.cam_obs_begin[c] + t; k < e; k += kCamThreads) {
    const int64_t o = B.cam_obs_list[k];
    real2 J[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) J[q] = jload<real2>(B.jac, B.no, q, o);
    if (NORMS) {
#pragma unroll
      for (int q = 0; q < 9; ++q) acc[q].add(J[q].x * J[q].x + J[q].y * J[q].y);
    } else {
      // mixed form: J_c^T r comes in FP64 from the chunk kernel's segment
      // partials (below), not from the FP32 copies
      real2 r = mk2((real)0, (real)0);
      if (!MIXED) r = jload<real2>(B.jac, B.no, 12, o);
#pragma unroll
      for (int a = 0; a < 9; ++a) {
#pragma unroll
        for (int b = a; b < 9; ++b) acc[sym9(a, b)].add(J[a].x * J[b].x + J[a].y * J[b].y);
        if (!MIXED) acc[45 + a].add(J[a].x * r.x + J[a].y * r.y);
      }
    }
  }
  // warp sums: FP64 in the FP64 form; double-float in the mixed form (FP32
  // instructions: 54 FP64 reductions in every warp would occupy GB300's FP64
  // pipe for microseconds), converted once per value below
  if (MIXED) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const KahanF &kq = reinterpret_cast<const KahanF &>(acc[q]);
      const DF v = df_warp_sum(df_fast_two_sum(kq.s, -kq.c));
      if (lane == 0) partf[warp][q] = v;
    }
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const double v = warp_sum(acc[q].value());
      if (lane == 0) part[warp][q] = v;
    }
  }
  __syncthreads();
  if (MIXED && t < NV) {
    DF v = partf[0][t];
    for (int w = 1; w < kCamThreads / 32; ++w) v = df_add(v, partf[w][t]);
    part[0][t] = df_value(v);  // read back below by this thread only
  }
  if (t < NV) {
    double s = 0.0;
    if (MIXED && !NORMS && t >= 45) {
      // the camera's FP64 gradient: its segment partials in camera-major order
      // (four interleaved accumulators, combined pairwise: a fixed order)
      const double *gp = B.seg_grad + (t - 45);
      const int s0 = B.cam_seg_begin[c], s1 = B.cam_seg_begin[c + 1];
      double a4[4] = {0.0, 0.0, 0.0, 0.0};
      for (int sg = s0; sg < s1; sg += 16) {
        double v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) v[u] = (sg + u < s1) ? gp[9 * (size_t)(sg + u)] : 0.0;
#pragma unroll
        for (int u = 0; u < 16; ++u) a4[u % 4] += v[u];
      }
      s = (a4[0] + a4[1]) + (a4[2] + a4[3]);
    } else if (MIXED) {
      s = part[0][t];
    } else {
      for (int w = 0; w < kCamThreads / 32; ++w) s += part[w][t];
    }
    part[0][t] = s;  // each t reads its own column only before writing it
  }
  __syncthreads();
  if (t == 0) {
    if (NORMS) {
      for (int q = 0; q < 9; ++q) B.cam_colnorm[9 * (size_t)c + q] = part[0][q];
    } else {
      for (int q = 0; q < 45; ++q) B.cam_B[45 * (size_t)c + q] = part[0][q];
      double gmax = 0.0, xn2 = 0.0;
      const bool used = B.cam_used[c] != 0;
      const double *x = B.cam_param[L->parity] + 9 * (size_t)c;
      for (int q = 0; q < 9; ++q) {
        const double gq = used ? part[0][45 + q] : 0.0;
        B.cam_g[9 * (size_t)c + q] = gq;
        if (used) {
          const double gu = gq / B.cam_scale[9 * (size_t)c + q];
          gmax = fmax(gmax, fabs(x[q] - (x[q] - gu)));
          xn2 += x[q] * x[q];
        }
      }
      B.cam_scal[(size_t)kCamScal * c + kCC_GMAX] = gmax;
      B.cam_scal[(size_t)kCamScal * c + kCC_XN2] = xn2;
    }
  }
}

// ---------------------------------------------------------------------------
// K1c, FP64 form: J_c^T J_c and J_c^T r of a camera over pieces of its
// observation list (kCamPieceObs each), a CTA per piece, so the work of a
// few hundred cameras spreads over all SMs (one CTA per camera left most of
// them idle behind the cameras with the most observations).  Each thread
// sums its observations with FMA chains (2 FP64 FMAs per entry); the
// piece's sums are the threads' values added in thread order (a column per
// thread, shared memory); the camera's last piece to finish (a counter per
// camera, reset by it) adds the pieces' sums in piece order and writes the
// camera's values.  Every sum has a fixed order.
constexpr int kPieceThreads = 64;

__global__ void __launch_bounds__(kPieceThreads) k_eval_camera_pieces(DeviceBatch B) {
  __shared__ double part[kPieceThreads][55];
  __shared__ double tot[54];
  __shared__ int last;
  const int piece = blockIdx.x, t = threadIdx.x;
  // the camera of the piece: cam_piece_begin[c] <= piece < cam_piece_begin[c + 1]
  int lo = 0, hi = B.nc;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (B.cam_piece_begin[mid] <= piece)
      lo = mid;
    else
      hi = mid;
  }
  const int c = lo;
  const LMState *L = B.lm + B.cam_problem[c];
  if (!L->active || !L->need_jacobian) return;
  const int k0 = B.cam_piece_begin[c], npc = B.cam_piece_begin[c + 1] - k0;
  const int e1 = B.cam_obs_begin[c + 1];
  const int o0 = B.cam_obs_begin[c] + (piece - k0) * kCamPieceObs, o1 = min(o0 + kCamPieceObs, e1);
  double acc[54];
#pragma unroll
  for (int q = 0; q < 54; ++q) acc[q] = 0.0;
  for (int k = o0 + t; k < o1; k += kPieceThreads) {
    const int64_t o = B.cam_obs_list[k];
    double2 J[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) J[q] = jload<double2>(B.jac, B.no, q, o);
    const double2 r = jload<double2>(B.jac, B.no, 12, o);
#pragma unroll
    for (int a = 0; a < 9; ++a) {
#pragma unroll
      for (int b = a; b < 9; ++b) acc[sym9(a, b)] = fma(J[a].y, J[b].y, fma(J[a].x, J[b].x, acc[sym9(a, b)]));
      acc[45 + a] = fma(J[a].y, r.y, fma(J[a].x, r.x, acc[45 + a]));
    }
  }
#pragma unroll
  for (int q = 0; q < 54; ++q) part[t][q] = acc[q];
  __syncthreads();
  double s = 0.0;
  if (t < 54)
    for (int i = 0; i < kPieceThreads; ++i) s += part[i][t];
  if (npc > 1) {
    // the piece's sums to the camera's slots; the last piece adds them up
    if (t < 54) B.piece_part[54 * (size_t)piece + t] = s;
    __threadfence();
    __syncthreads();
    if (t == 0) last = atomicAdd(B.cam_counter + c, 1u) == (unsigned)(npc - 1);
    __syncthreads();
    if (!last) return;
    if (t < 54) {
      s = 0.0;
      for (int q = 0; q < npc; ++q) s += __ldcg(B.piece_part + 54 * (size_t)(k0 + q) + t);
    }
    if (t == 0) B.cam_counter[c] = 0u;  // ready for the next evaluation
  }
  if (t < 54) tot[t] = s;
  __syncthreads();
  if (t == 0) {
    for (int q = 0; q < 45; ++q) B.cam_B[45 * (size_t)c + q] = tot[q];
    double gmax = 0.0, xn2 = 0.0;
    const bool used = B.cam_used[c] != 0;
    const double *x = B.cam_param[L->parity] + 9 * (size_t)c;
    for (int q = 0; q < 9; ++q) {
      const double gq = used ? tot[45 + q] : 0.0;
      B.cam_g[9 * (size_t)c + q] = gq;
      if (used) {
        const double gu = gq / B.cam_scale[9 * (size_t)c + q];
        gmax = fmax(gmax, fabs(x[q] - (x[q] - gu)));
        xn2 += x[q] * x[q];
      }
    }
    B.cam_scal[(size_t)kCamScal * c + kCC_GMAX] = gmax;
    B.cam_scal[(size_t)kCamScal * c + kCC_XN2] = xn2;
  }
}

void launch_eval_jacobian(const DeviceBatch &b, bool mixed, bool norms, cudaStream_t s) {
  const int gc = b.nchunks;
  if (mixed) {
    if (norms) {
      k_eval_chunk<true, true><<<gc, kChunkCap, 0, s>>>(b);
      k_eval_camera<true, true><<<b.nc, kCamThreads, 0, s>>>(b);
    } else {
      k_eval_chunk<true, false><<<gc, kChunkCap, 0, s>>>(b);
      k_eval_camera<true, false><<<b.nc, kCamThreads, 0, s>>>(b);
    }
  } else {
    if (norms) {
      k_eval_chunk<false, true><<<gc, kChunkCap, 0, s>>>(b);
      k_eval_camera<false, true><<<b.nc, kCamThreads, 0, s>>>(b);
    } else {
      k_eval_chunk<false, false><<<gc, kChunkCap, 0, s>>>(b);
      const int npieces = b.nc > 0 ? (int)b.npieces : 0;
      if (npieces > 0) k_eval_camera_pieces<<<npieces, kPieceThreads, 0, s>>>(b);
    }
  }
}

// ---------------------------------------------------------------------------
// Jacobi scaling s = 1 / (1 + sqrt(|J_col|^2)) of the first evaluation, kept
// for the whole solve.
__global__ void k_scale_init(DeviceBatch B) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t ncam = 9 * (int64_t)B.nc, npt = 3 * (int64_t)B.np;
  if (i < ncam) {
    const bool res = B.prob_resume && B.prob_resume[B.cam_problem[i / 9]];
    B.cam_scale[i] = res ? B.cam_scale_in[i] : B.opt.jacobi_scaling ? 1.0 / (1.0 + sqrt(B.cam_colnorm[i])) : 1.0;
    const DF d = df_from_double(B.cam_scale[i]);
    B.cam_scalef[i] = d.hi;
    B.cam_scaledf[i] = make_float2(d.hi, d.lo);
  } else if (i < ncam + npt) {
    const int64_t k = i - ncam;
    const bool res = B.prob_resume && B.prob_resume[B.pt_problem[k / 3]];
    B.pt_scale[k] = res ? B.pt_scale_in[k] : B.opt.jacobi_scaling ? 1.0 / (1.0 + sqrt(B.pt_colnorm[k])) : 1.0;
    const DF d = df_from_double(B.pt_scale[k]);
    B.pt_scalef[k] = d.hi;
    B.pt_scaledf[k] = make_float2(d.hi, d.lo);
  }
}

void launch_scale_init(const DeviceBatch &b, cudaStream_t s) {
  const int64_t n = 9 * (int64_t)b.nc + 3 * (int64_t)b.np;
  k_scale_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b);
}

// Sets the LM-loop condition once every problem's CTA of this launch is
// done: any problem still active, and never more LM bodies than the
// iteration cap allows (a runaway loop cannot happen).
__device__ void finish_lm_body(const DeviceBatch &B, bool count_body) {
  __shared__ int flag;
  if (last_block_done(B.global_counter + kGC_POST, gridDim.x, &flag)) {
    if (threadIdx.x == 0) {
      int any = 0;
      for (int p = 0; p < B.num_problems; ++p) any |= __ldcg(&B.lm[p].active);
      uint32_t bodies = B.global_counter[kGC_LMBODIES];
      if (count_body) B.global_counter[kGC_LMBODIES] = ++bodies;
      if (bodies > (uint32_t)B.opt.max_bodies + 2u) {
        if (any) B.status[0] = GBA_ERR_INTERNAL;
        any = 0;
      }
      B.status[1] = any;
      // a segment run stops its loop after bodies_cap counted bodies; the
      // problems stay active for the next launch
      const bool more = any && !(B.opt.bodies_cap > 0 && bodies >= (uint32_t)B.opt.bodies_cap);
      if (B.use_cond && B.lm_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.lm_cond, more ? 1u : 0u);
    }
  }
}

// K7: one CTA per problem.
__global__ void __launch_bounds__(256) k_post_eval(DeviceBatch B, int count_body) {
  __shared__ double red[8 * 6];
  const int p = blockIdx.x;
  LMState *L = B.lm + p;
  if (L->active && L->need_jacobian) {
    const ProblemInfo pi = B.prob[p];
    const double *cs = B.chunk_scal;
    // cost, bad, max |g| (points, cameras), |x|^2 (cameras, points)
    const int h0 = pi.chunk_begin, h1 = pi.chunk_begin + pi.chunk_count;
    const int k0 = pi.cam_begin, k1 = pi.cam_begin + pi.cam_count;
    const double *const a[6] = {cs + kCS_COST, cs + kCS_BAD, cs + kCS_GMAX, B.cam_scal + kCC_GMAX,
                                B.cam_scal + kCC_XN2, cs + kCS_XN2};
    const int b[6] = {h0, h0, h0, k0, k0, h0}, e[6] = {h1, h1, h1, k1, k1, h1};
    const int st[6] = {kChunkScal, kChunkScal, kChunkScal, kCamScal, kCamScal, kChunkScal};
    const bool mx[6] = {false, true, true, true, false, false};
    double r[6];
    block_range_multi<6>(a, b, e, st, mx, r, red);
    const double cost = r[0], bad = r[1], gp = r[2], gc = r[3], xc = r[4], xp = r[5];
    // g2o's Levenberg: lambda_0 = tau max diag(J^T J) over the problem's
    // cameras and points (the column norms of the first evaluation)
    double hmax[2] = {0.0, 0.0};
    if (B.opt.g2o && L->iteration == 0) {
      const double *const ha[2] = {B.cam_colnorm, B.pt_colnorm};
      const int hb[2] = {9 * k0, 3 * pi.pt_begin}, he[2] = {9 * k1, 3 * (pi.pt_begin + pi.pt_count)};
      const int hs[2] = {1, 1};
      const bool hm[2] = {true, true};
      block_range_multi<2>(ha, hb, he, hs, hm, hmax, red);
    }
    if (threadIdx.x == 0) {
      const DeviceOptions &o = B.opt;
      const bool resumed = L->resumed != 0;
      if (o.g2o && L->iteration == 0 && !resumed) L->radius = 1.0 / (kG2oTau * fmax(hmax[0], hmax[1]));
      L->need_jacobian = 0;
      // the mixed form forms the FP64 cost only at a problem's first
      // evaluation; later the current point's cost is the FP64 cost of the
      // candidate evaluation that was accepted (already in x_cost)
      const bool cost_here = !o.mixed || (L->iteration == 0 && !resumed);
      if (cost_here) L->x_cost = cost;
      L->gradient_max_norm = fmax(gp, gc);
      L->x_norm = sqrt(xc + xp);
      L->resumed = 0;
      const int it = L->iteration;
      if (resumed) {
        // the state was carried over at an LM-iteration boundary: the same
        // point evaluated again (the same bits), nothing else to decide
      } else if (bad != 0.0 || !isfinite(L->x_cost)) {
        L->active = 0;
        L->termination_type = GBA_TERMINATION_FAILURE;
        L->termination_reason = GBA_REASON_EVALUATION_FAILED;
        if (it == 0) L->initial_cost = cost;
      } else {
        if (it == 0) {
          L->initial_cost = cost;
          L->minimum_cost = cost;
          trace_put(B, p, 0, cost, L->radius, 0, 1);
        } else {
          L->minimum_cost = L->x_cost;
          trace_put(B, p, it, L->x_cost, L->radius, L->pcg_iterations, 1);
        }
        if (o.g2o) {
          // the trials of the iteration that ended with this accepted step
          if (L->trials >= kG2oMaxTrials) {
            L->active = 0;
            L->termination_type = GBA_TERMINATION_CONVERGENCE;
            L->termination_reason = GBA_REASON_LM_TRIALS;
          } else if (L->outer >= o.max_iterations) {
            L->active = 0;
            L->termination_type = GBA_TERMINATION_NO_CONVERGENCE;
            L->termination_reason = GBA_REASON_MAX_ITERATIONS;
          }
          L->trials = 0;
        } else if (it >= o.max_iterations) {
          L->active = 0;
          L->termination_type = GBA_TERMINATION_NO_CONVERGENCE;
          L->termination_reason = GBA_REASON_MAX_ITERATIONS;
        } else if (L->gradient_max_norm <= o.gradient_tolerance) {
          L->active = 0;
          L->termination_type = GBA_TERMINATION_CONVERGENCE;
          L->termination_reason = GBA_REASON_GRADIENT_TOLERANCE;
        } else if (L->radius <= o.min_radius) {
          L->active = 0;
          L->termination_type = GBA_TERMINATION_CONVERGENCE;
          L->termination_reason = GBA_REASON_MIN_TRUST_REGION_RADIUS;
        }
      }
    }
  }
  finish_lm_body(B, count_body != 0);
}

void launch_post_eval(const DeviceBatch &b, cudaStream_t s) {
  k_post_eval<<<b.num_problems, 256, 0, s>>>(b, 1);
}

// ---------------------------------------------------------------------------
// K5b: candidate cameras x + step * scale (step = -y_c from the PCG), the
// camera part of |x - x_cand|^2, and the candidate camera tables (R only).
__global__ void k_candidate_cameras(DeviceBatch B) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.nc) return;
  const LMState *L = B.lm + B.cam_problem[c];
  if (!L->active || !L->linear_ok) return;
  const double *x = B.cam_param[L->parity] + 9 * (size_t)c;
  double *xc = B.cam_param[L->parity ^ 1] + 9 * (size_t)c;
  double cand[9];
  double s2 = 0.0;
  const bool used = B.cam_used[c] != 0;
  for (int q = 0; q < 9; ++q) {
    const double step = -B.pcg_x[9 * (size_t)c + q];
    cand[q] = used ? x[q] + step * B.cam_scale[9 * (size_t)c + q] : x[q];
  }
  if (B.opt.pinhole && used) {
    // local-BA windows: the pose moves on SE3, T <- exp(xi) T
    const double *y = B.pcg_x + 9 * (size_t)c, *sc = B.cam_scale + 9 * (size_t)c;
    const double dw[3] = {-y[0] * sc[0], -y[1] * sc[1], -y[2] * sc[2]};
    const double du[3] = {-y[3] * sc[3], -y[4] * sc[4], -y[5] * sc[5]};
    se3_compose_left(dw, du, x, cand);
  } else if (B.opt.so3_left && used) {
    const double dw[3] = {-B.pcg_x[9 * (size_t)c + 0] * B.cam_scale[9 * (size_t)c + 0],
                          -B.pcg_x[9 * (size_t)c + 1] * B.cam_scale[9 * (size_t)c + 1],
                          -B.pcg_x[9 * (size_t)c + 2] * B.cam_scale[9 * (size_t)c + 2]};
    compose_left(dw, x, cand);
  }
  for (int q = 0; q < 9; ++q) {
    const double d = x[q] - cand[q];
    s2 += d * d;
    xc[q] = cand[q];
  }
  B.cam_scal[(size_t)kCamScal * c + kCC_STEP2] = used ? s2 : 0.0;
  // the camera part of step.g (the mixed form's model cost change)
  double yg = 0.0;
  for (int q = 0; q < 9; ++q) yg += B.pcg_x[9 * (size_t)c + q] * B.cam_g[9 * (size_t)c + q];
  B.cam_scal[(size_t)kCamScal * c + kCC_YG] = used ? -yg : 0.0;
  camera_table_entry(cand, B.cam_table + (size_t)kCamTable * c, false);
}

// K2: candidate cost, FP64 in both precision modes.
__global__ void __launch_bounds__(kChunkCap) k_cost_chunk(DeviceBatch B) {
  __shared__ double red[kChunkCap / 32];
  const int t = threadIdx.x;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x) {
    const ChunkInfo ci = B.chunk[ch];
    const LMState *L = B.lm + ci.problem;
    if (!L->active || !L->linear_ok) continue;
    const int parity = L->parity ^ 1;
    double cost = 0.0;
    bool bad = false;
    if (t < ci.obs_count) {
      const int64_t o = ci.obs_begin + t;
      const int c = B.obs_cam[o], j = B.obs_pt[o];
      const double *Xp = B.pt_param[parity] + 4 * (size_t)j;
      const double X[3] = {Xp[0], Xp[1], Xp[2]};
      double ru, rv;
      if (B.opt.pinhole) {
        double Q[3];
        rig_project(B.cam_table + (size_t)kCamTable * c, B.prob_rig + (size_t)kRig * ci.problem, B.obs_rig[o], X,
                    B.obs_uv[o], Q, ru, rv);
      } else {
        Proj pr;
        project(B.cam_table + (size_t)kCamTable * c, X, B.obs_uv[o], pr);
        ru = pr.ru, rv = pr.rv;
      }
      cost = block_cost(B.opt.loss, B.opt.loss_scale, ru, rv);
      bad = !(isfinite(ru) && isfinite(rv) && isfinite(cost));
    }
    const double cs = block_sum(cost, red);
    const double bd = block_max(bad ? 1.0 : 0.0, red);
    if (t == 0) {
      B.chunk_scal[(size_t)kChunkScal * ch + kCS_COST] = cs;
      B.chunk_scal[(size_t)kChunkScal * ch + kCS_BAD] = bd;
    }
  }
}

void launch_candidate_cost(const DeviceBatch &b, cudaStream_t s) {
  k_candidate_cameras<<<(b.nc + kCamTableThreads - 1) / kCamTableThreads, kCamTableThreads, 0, s>>>(b);
  k_cost_chunk<<<b.nchunks, kChunkCap, 0, s>>>(b);
}

// Cost at the second parameter buffer with the current camera tables (the
// kernel-level evaluate entry point, where both buffers hold the same point).
void launch_cost_only(const DeviceBatch &b, cudaStream_t s) {
  if (b.nchunks > 0) k_cost_chunk<<<b.nchunks, kChunkCap, 0, s>>>(b);
}

// Busy-waits about 40 microseconds of SM clock (a fixed cycle count, so it
// always ends), used by the profiling pass only.
__global__ void k_prof_delay(long long cycles) {
  const long long t0 = clock64();
  while (clock64() - t0 < cycles) {
  }
}

void launch_prof_delay(cudaStream_t s) { k_prof_delay<<<1, 1, 0, s>>>(80000LL); }

// Fails with cudaErrorNoKernelImageForDevice when the sm_103a image cannot
// run on the current device.
cudaError_t probe_kernel_image() {
  cudaFuncAttributes a;
  return cudaFuncGetAttributes(&a, k_init_state);
}

// ---------------------------------------------------------------------------
// Starts a solve from the uploaded initial point: both working buffers get
// the initial parameters (blocks a problem never updates then hold the same
// values in both), so a solve can be re-run without a new upload.
__global__ void k_sync_params(DeviceBatch B) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nc9 = 9 * (int64_t)B.nc, np4 = 4 * (int64_t)B.np;
  if (i < nc9) {
    const double v = B.cam_init[i];
    B.cam_param[0][i] = v;
    B.cam_param[1][i] = v;
  } else if (i < nc9 + np4) {
    const double v = B.pt_init[i - nc9];
    B.pt_param[0][i - nc9] = v;
    B.pt_param[1][i - nc9] = v;
  }
}

__global__ void k_gather_results(DeviceBatch B, double *out_cam, double *out_pt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nc9 = 9 * (int64_t)B.nc, np4 = 4 * (int64_t)B.np;
  if (i < nc9) {
    const int par = B.lm[B.cam_problem[i / 9]].parity;
    out_cam[i] = B.cam_param[par][i];
  } else if (i < nc9 + np4) {
    const int64_t k = i - nc9;
    const int par = B.lm[B.pt_problem[k / 4]].parity;
    out_pt[k] = B.pt_param[par][k];
  }
}

void launch_gather_results(const DeviceBatch &b, double *out_cam, double *out_pt, cudaStream_t s) {
  const int64_t n = 9 * (int64_t)b.nc + 4 * (int64_t)b.np;
  if (n > 0) k_gather_results<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, out_cam, out_pt);
}

// Local-BA windows after the solve: camera tables at the returned estimate,
// then each observation's chi2 = |error|^2 (EdgeProjection's chi2 with the
// identity information matrix, backend.cpp:135 and :159).
__global__ void k_window_tables(DeviceBatch B, const double *out_cam) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.nc) return;
  camera_table_entry(out_cam + 9 * (size_t)c, B.cam_table + (size_t)kCamTable * c, false);
}

__global__ void k_window_chi2(DeviceBatch B, const double *out_pt) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= B.no) return;
  const int c = B.obs_cam[o], j = B.obs_pt[o];
  const double *Xp = out_pt + 4 * (size_t)j;
  const double X[3] = {Xp[0], Xp[1], Xp[2]};
  double Q[3], ru, rv;
  rig_project(B.cam_table + (size_t)kCamTable * c, B.prob_rig + (size_t)kRig * B.cam_problem[c], B.obs_rig[o], X,
              B.obs_uv[o], Q, ru, rv);
  B.obs_chi2[o] = ru * ru + rv * rv;
}

void launch_window_chi2(const DeviceBatch &b, const double *out_cam, const double *out_pt, cudaStream_t s) {
  if (b.nc > 0) k_window_tables<<<(b.nc + 127) / 128, 128, 0, s>>>(b, out_cam);
  if (b.no > 0) k_window_chi2<<<(unsigned)((b.no + 255) / 256), 256, 0, s>>>(b, out_pt);
}

void launch_sync_param_buffers(const DeviceBatch &b, cudaStream_t s) {
  const int64_t n = 9 * (int64_t)b.nc + 4 * (int64_t)b.np;
  k_sync_params<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b);
}

}  // namespace gba
