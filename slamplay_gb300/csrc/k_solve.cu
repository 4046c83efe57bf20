// k_solve.cu — linear-solve and trust-region kernels.
//
// The LM system (J^T J + D^2) y = J^T r is solved with the points eliminated
// (Schur complement on the cameras), as Ceres' SPARSE_SCHUR does for the
// reference (test_bundle_adjustment_ceres.cpp:97), but the reduced camera
// matrix S = B + Dc^2 - W C^-1 W^T is never formed: it is applied implicitly
// inside a block-Jacobi PCG.
//
//  K3a k_point_prepare   per point: C = J_p^T J_p + Dp^2, FP64 inverse, Cinv g_p
//  K3b k_camera_schur    per camera (CTA): S_ii, reduced rhs, 9x9 FP64 inverse,
//                        PCG start (x = 0, r = v, z = M r)
//  K4  (k_pcg.cu)        implicit-Schur PCG: mat-vec over point-segment
//                        chunks, camera reduce, vector update
//  K5  k_back_substitute per chunk: y_p = C^-1 (g_p - W^T y_c), model cost
//                        change, candidate points
//  K6  k_decide          per problem: Ceres' accept / reject / radius update
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "kernels.h"

namespace gba {

__device__ __forceinline__ double lm_d2(double colnorm2, double radius, const DeviceOptions &o) {
  // LevenbergMarquardtStrategy: diag = clamp(|J_col|^2), D = sqrt(diag / radius)
  const double d = fmin(fmax(colnorm2, o.min_diagonal), o.max_diagonal);
  const double D = sqrt(d / radius);
  return D * D;
}

// ---------------------------------------------------------------------------
// K3a
template <bool MIXED>
__global__ void k_point_prepare(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= B.np) return;
  LMState *L = B.lm + B.pt_problem[j];
  if (!L->active) return;
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
    for (int q = 0; q < 6; ++q) Ci[q] = 0.0;
  }
  real *cio = reinterpret_cast<real *>(B.pt_Cinv) + 6 * (size_t)j;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    cio[q] = (real)Ci[q];
    B.pt_Cinv64[6 * (size_t)j + q] = Ci[q];
  }
  const double *g = B.pt_g + 3 * (size_t)j;
  B.pt_t[3 * (size_t)j + 0] = Ci[0] * g[0] + Ci[1] * g[1] + Ci[2] * g[2];
  B.pt_t[3 * (size_t)j + 1] = Ci[1] * g[0] + Ci[3] * g[1] + Ci[4] * g[2];
  B.pt_t[3 * (size_t)j + 2] = Ci[2] * g[0] + Ci[4] * g[1] + Ci[5] * g[2];
}

void launch_point_prepare(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  if (mixed)
    k_point_prepare<true><<<(b.np + 255) / 256, 256, 0, s>>>(b);
  else
    k_point_prepare<false><<<(b.np + 255) / 256, 256, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// 9x9 SPD inverse by Cholesky, FP64, one thread.  A and Ainv row-major.
__device__ bool spd_inverse9(const double *A, double *Ainv) {
  double L[45];  // packed lower by rows: L[i][j] at i*(i+1)/2 + j
#define LL(i, j) L[(i) * ((i) + 1) / 2 + (j)]
  for (int i = 0; i < 9; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = A[i * 9 + j];
      for (int k = 0; k < j; ++k) s -= LL(i, k) * LL(j, k);
      if (i == j) {
        if (!(s > 0.0)) return false;
        LL(i, i) = sqrt(s);
      } else {
        LL(i, j) = s / LL(j, j);
      }
    }
  }
  // Y = L^{-1}, in place of L (lower)
  double Y[45];
  for (int j = 0; j < 9; ++j) {
    for (int i = j; i < 9; ++i) {
      double s = (i == j) ? 1.0 : 0.0;
      for (int k = j; k < i; ++k) s -= LL(i, k) * Y[k * (k + 1) / 2 + j];
      Y[i * (i + 1) / 2 + j] = s / LL(i, i);
    }
  }
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) {
      double s = 0.0;
      const int k0 = i > j ? i : j;
      for (int k = k0; k < 9; ++k) s += Y[k * (k + 1) / 2 + i] * Y[k * (k + 1) / 2 + j];
      Ainv[i * 9 + j] = s;
    }
#undef LL
  for (int q = 0; q < 81; ++q)
    if (!isfinite(Ainv[q])) return false;
  return true;
}

// ---------------------------------------------------------------------------
// K3b: one CTA per camera.
constexpr int kSchurThreads = 128;

template <bool MIXED>
__global__ void __launch_bounds__(kSchurThreads) k_camera_schur(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  typedef typename Acc<MIXED>::type Acc;
  __shared__ double part[kSchurThreads / 32][54];
  __shared__ double S[81];
  __shared__ double Minv[81];
  __shared__ double vec[9];
  __shared__ double red[kSchurThreads / 32];
  __shared__ int flag, okflag;
  const int c = blockIdx.x;
  const int p = B.cam_problem[c];
  LMState *L = B.lm + p;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const bool work = L->active != 0;
  if (work) {
    Acc acc[54];
#pragma unroll
    for (int q = 0; q < 54; ++q) acc[q].init();
    const int e = B.cam_obs_begin[c + 1];
    for (int k = B.cam_obs_begin[c] + t; k < e; k += kSchurThreads) {
      const int64_t o = B.cam_obs_list[k];
      const int j = B.obs_pt[o];
      real2 Jc[9], Jp[3];
#pragma unroll
      for (int q = 0; q < 9; ++q) Jc[q] = jload<real2>(B.jac, B.no, q, o);
#pragma unroll
      for (int q = 0; q < 3; ++q) Jp[q] = jload<real2>(B.jac, B.no, 9 + q, o);
      const real *Ci = reinterpret_cast<const real *>(B.pt_Cinv) + 6 * (size_t)j;
      const real c0 = Ci[0], c1 = Ci[1], c2 = Ci[2], c3 = Ci[3], c4 = Ci[4], c5 = Ci[5];
      // h = Cinv J_p^T rows
      const real hu0 = c0 * Jp[0].x + c1 * Jp[1].x + c2 * Jp[2].x;
      const real hu1 = c1 * Jp[0].x + c3 * Jp[1].x + c4 * Jp[2].x;
      const real hu2 = c2 * Jp[0].x + c4 * Jp[1].x + c5 * Jp[2].x;
      const real hv0 = c0 * Jp[0].y + c1 * Jp[1].y + c2 * Jp[2].y;
      const real hv1 = c1 * Jp[0].y + c3 * Jp[1].y + c4 * Jp[2].y;
      const real hv2 = c2 * Jp[0].y + c4 * Jp[1].y + c5 * Jp[2].y;
      const real a00 = Jp[0].x * hu0 + Jp[1].x * hu1 + Jp[2].x * hu2;
      const real a01 = Jp[0].x * hv0 + Jp[1].x * hv1 + Jp[2].x * hv2;
      const real a11 = Jp[0].y * hv0 + Jp[1].y * hv1 + Jp[2].y * hv2;
      const double *tp = B.pt_t + 3 * (size_t)j;
      const real t0 = (real)tp[0], t1 = (real)tp[1], t2 = (real)tp[2];
      const real eu = Jp[0].x * t0 + Jp[1].x * t1 + Jp[2].x * t2;
      const real ev = Jp[0].y * t0 + Jp[1].y * t1 + Jp[2].y * t2;
      real gu[9], gv[9];
#pragma unroll
      for (int b = 0; b < 9; ++b) {
        gu[b] = a00 * Jc[b].x + a01 * Jc[b].y;
        gv[b] = a01 * Jc[b].x + a11 * Jc[b].y;
      }
#pragma unroll
      for (int a = 0; a < 9; ++a) {
#pragma unroll
        for (int b = a; b < 9; ++b) acc[sym9(a, b)].add(Jc[a].x * gu[b] + Jc[a].y * gv[b]);
        acc[45 + a].add(Jc[a].x * eu + Jc[a].y * ev);
      }
    }
#pragma unroll
    for (int q = 0; q < 54; ++q) {
      const double v = warp_sum(acc[q].value());
      if (lane == 0) part[warp][q] = v;
    }
    __syncthreads();
    const double radius = L->radius;
    if (t < 81) {
      const int a = t / 9, b = t % 9;
      double s = 0.0;
      for (int w = 0; w < kSchurThreads / 32; ++w) s += part[w][sym9(a, b)];
      double v = B.cam_B[45 * (size_t)c + sym9(a, b)] - s;
      if (a == b) {
        const double d2 = lm_d2(B.cam_B[45 * (size_t)c + sym9(a, a)], radius, B.opt);
        v += d2;
        B.cam_D2[9 * (size_t)c + a] = d2;
      }
      S[t] = v;
    }
    if (t < 9) {
      double s = 0.0;
      for (int w = 0; w < kSchurThreads / 32; ++w) s += part[w][45 + t];
      vec[t] = B.cam_g[9 * (size_t)c + t] - s;
    }
    __syncthreads();
    if (t == 0) {
      okflag = spd_inverse9(S, Minv) ? 1 : 0;
      if (!okflag) {
        L->linear_ok = 0;
        for (int q = 0; q < 81; ++q) Minv[q] = 0.0;
      }
    }
    __syncthreads();
    double rz = 0.0, rr = 0.0;
    if (t < 9) {
      double z = 0.0;
      for (int k = 0; k < 9; ++k) z += Minv[t * 9 + k] * vec[k];
      const size_t i = 9 * (size_t)c + t;
      B.pcg_v[i] = vec[t];
      B.pcg_r[i] = vec[t];
      B.pcg_x[i] = 0.0;
      B.pcg_p[i] = z;  // first direction p0 = z0
      B.pcg_z[i] = z;
      if (MIXED) B.pcg_pf[i] = (float)z;
      rz = vec[t] * z;
      rr = vec[t] * vec[t];
    }
    if (t < 81) {
      B.cam_Minv[81 * (size_t)c + t] = Minv[t];
      if (MIXED) B.cam_Minvf[81 * (size_t)c + t] = (float)Minv[t];
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
    if (t == 0) {
      int any = 0, count = 0;
      for (int q = 0; q < B.num_problems; ++q) {
        const int a = __ldcg(&B.lm[q].active) && __ldcg(&B.lm[q].pcg_active);
        any |= a;
        count += a;
      }
      B.status[2] = any;
      B.status[3] = count;
      B.global_counter[kGC_BAR_COUNT] = 0u;  // persistent PCG barrier starts empty
      __threadfence();
      if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, any ? 1u : 0u);
    }
  }
}

void launch_camera_schur(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  if (mixed)
    k_camera_schur<true><<<b.nc, kSchurThreads, 0, s>>>(b);
  else
    k_camera_schur<false><<<b.nc, kSchurThreads, 0, s>>>(b);
}


// ---------------------------------------------------------------------------
// K5: y_p = C^-1 (g_p - W^T y_c), step = -y, model cost change
// -m.(r + m/2) with m = J step, candidate points x + step * scale.  FP64
// arithmetic in both modes (the acceptance ratio is FP64).
template <bool MIXED>
__global__ void __launch_bounds__(kChunkCap) k_back_substitute(DeviceBatch B) {
  typedef typename Prec<MIXED>::real2 real2;
  __shared__ double yseg[kChunkCap][9];
  __shared__ double W[kChunkCap][3];
  __shared__ double ypt[kChunkCap][3];
  __shared__ double red[kChunkCap / 32];
  const int t = threadIdx.x;
  for (int ch = blockIdx.x; ch < B.nchunks; ch += gridDim.x) {
    const ChunkInfo ci = B.chunk[ch];
    const LMState *L = B.lm + ci.problem;
    if (!L->active || !L->linear_ok) continue;
    const int parity = L->parity;
    for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
      const int s = i / 9, q = i - 9 * s;
      yseg[s][q] = B.pcg_x[9 * (size_t)B.seg_cam[ci.seg_begin + s] + q];
    }
    __syncthreads();
    const bool valid = t < ci.obs_count;
    double Jpu[3], Jpv[3], zu = 0.0, zv = 0.0, ru = 0.0, rv = 0.0;
    int lp = 0;
    if (valid) {
      const int64_t o = ci.obs_begin + t;
      const int s = B.obs_seg[o];
      lp = B.obs_pt[o] - ci.pt_begin;
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const real2 J = jload<real2>(B.jac, B.no, q, o);
        zu += (double)J.x * yseg[s][q];
        zv += (double)J.y * yseg[s][q];
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
    double s2 = 0.0;
    if (t < ci.pt_count) {
      const int jj = ci.pt_begin + t;
      const int b0 = B.pt_obs_begin[jj] - ci.obs_begin, b1 = B.pt_obs_begin[jj + 1] - ci.obs_begin;
      double w0 = 0.0, w1 = 0.0, w2 = 0.0;
      for (int k = b0; k < b1; ++k) w0 += W[k][0], w1 += W[k][1], w2 += W[k][2];
      const double *g = B.pt_g + 3 * (size_t)jj;
      const double a0 = g[0] - w0, a1 = g[1] - w1, a2 = g[2] - w2;
      const double *Ci = B.pt_Cinv64 + 6 * (size_t)jj;
      const double y0 = Ci[0] * a0 + Ci[1] * a1 + Ci[2] * a2;
      const double y1 = Ci[1] * a0 + Ci[3] * a1 + Ci[4] * a2;
      const double y2 = Ci[2] * a0 + Ci[4] * a1 + Ci[5] * a2;
      ypt[t][0] = y0, ypt[t][1] = y1, ypt[t][2] = y2;
      const double *x = B.pt_param[parity] + 4 * (size_t)jj;
      double *xc = B.pt_param[parity ^ 1] + 4 * (size_t)jj;
      const double *sc = B.pt_scale + 3 * (size_t)jj;
      const double y[3] = {y0, y1, y2};
      const bool used = B.pt_used[jj] != 0;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const double cand = used ? x[q] + (-y[q]) * sc[q] : x[q];
        const double d = x[q] - cand;
        s2 += used ? d * d : 0.0;
        xc[q] = cand;
      }
    }
    __syncthreads();
    double model = 0.0;
    if (valid) {
      const double m0 = -(zu + Jpu[0] * ypt[lp][0] + Jpu[1] * ypt[lp][1] + Jpu[2] * ypt[lp][2]);
      const double m1 = -(zv + Jpv[0] * ypt[lp][0] + Jpv[1] * ypt[lp][1] + Jpv[2] * ypt[lp][2]);
      model = m0 * (ru + m0 / 2.0) + m1 * (rv + m1 / 2.0);
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

__global__ void __launch_bounds__(256) k_decide(DeviceBatch B) {
  __shared__ double red[8];
  const int p = blockIdx.x;
  LMState *L = B.lm + p;
  if (!L->active) return;
  const ProblemInfo pi = B.prob[p];
  const int c0 = pi.chunk_begin, c1 = pi.chunk_begin + pi.chunk_count;
  const double model = -block_range_sum(B.chunk_scal + kCS_MODEL, c0, c1, kChunkScal, red);
  const double cand = block_range_sum(B.chunk_scal + kCS_COST, c0, c1, kChunkScal, red);
  const double bad = block_range_max(B.chunk_scal + kCS_BAD, c0, c1, kChunkScal, red);
  const double s2p = block_range_sum(B.chunk_scal + kCS_STEP2, c0, c1, kChunkScal, red);
  const double s2c = block_range_sum(B.cam_scal + kCC_STEP2, pi.cam_begin, pi.cam_begin + pi.cam_count, kCamScal, red);
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
