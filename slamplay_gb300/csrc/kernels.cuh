// kernels.cuh — device helpers shared by the libgba kernels.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "gba_internal.h"

namespace gba {

// ---------------------------------------------------------------------------
// Storage type of the Jacobian / Schur products per precision mode.
// ---------------------------------------------------------------------------
template <bool MIXED>
struct Prec;
template <>
struct Prec<false> {
  typedef double real;
  typedef double2 real2;
};
template <>
struct Prec<true> {
  typedef float real;
  typedef float2 real2;
};

// 1/a: the FP32 hardware reciprocal refined by two Newton-Raphson steps
// x <- x + x (1 - a x), each of which doubles the number of correct bits
// (about 23 -> 46 -> FP64 rounding).  Falls back to a division outside the
// FP32 normal range.
__device__ __forceinline__ double recip_nr(double a) {
  const double aa = fabs(a);
  if (!(aa > 1e-30 && aa < 1e30)) return 1.0 / a;
  float xf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(xf) : "f"((float)a));
  double x = (double)xf;
  double e = fma(-a, x, 1.0);
  x = fma(x, e, x);
  e = fma(-a, x, 1.0);
  return fma(x, e, x);
}

__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }

// Packed symmetric indices: 3x3 as (00 01 02 11 12 22), 9x9 upper row-major.
__host__ __device__ __forceinline__ int sym3(int i, int j) {
  if (i > j) {
    const int t = i;
    i = j;
    j = t;
  }
  return i * 3 - (i * (i - 1)) / 2 + (j - i);
}
__host__ __device__ __forceinline__ int sym9(int i, int j) {
  if (i > j) {
    const int t = i;
    i = j;
    j = t;
  }
  return i * 9 - (i * (i - 1)) / 2 + (j - i);
}

// ---------------------------------------------------------------------------
// Compensated (Kahan) summation for the FP32 segmented sums of the mixed
// form.  Written so the compiler cannot fold the compensation away (no
// fast-math is used anywhere in libgba).
// ---------------------------------------------------------------------------
struct KahanF {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f, c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
  // the sum in the working precision, without an FP64 round trip
  __device__ __forceinline__ float rvalue() const { return __fsub_rn(s, c); }
  // adds another compensated sum (its value s - c)
  __device__ __forceinline__ void merge(const KahanF &o) {
    add(o.s);
    add(-o.c);
  }
};

// Plain FP64 accumulator with the same interface.
struct SumD {
  double s;
  __device__ __forceinline__ void init() { s = 0.0; }
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
  __device__ __forceinline__ double rvalue() const { return s; }
  __device__ __forceinline__ void merge(const SumD &o) { s += o.s; }
};

// ---------------------------------------------------------------------------
// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats (|lo| <= ulp(hi) / 2), about 48 significant bits from FP32
// instructions.  GB300 issues FP32 some 55 times faster than FP64, so the
// mixed form accumulates its dot products this way and converts to FP64
// once per block.  TwoSum is Knuth's error-free addition, TwoProd the
// FMA-based error-free product (both exact under round-to-nearest).
// ---------------------------------------------------------------------------
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_zero() { return DF{0.f, 0.f}; }
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return DF{s, e};
}
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const DF s = df_two_sum(a.hi, b.hi);
  const DF t = df_two_sum(a.lo, b.lo);
  DF u = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}
__device__ __forceinline__ DF df_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return DF{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ double df_value(DF a) { return (double)a.hi + (double)a.lo; }
// a * b for a float b, and a * b: the error-free product of the high parts
// plus the cross terms, renormalised (about 2^-46 relative error)
__device__ __forceinline__ DF df_mul_f(DF a, float b) {
  const DF p = df_prod(a.hi, b);
  return df_fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const DF p = df_prod(a.hi, b.hi);
  return df_fast_two_sum(p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo)));
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
// a double as the nearest float plus the nearest float to the remainder
__device__ __forceinline__ DF df_from_double(double d) {
  const float h = __double2float_rn(d);
  return DF{h, __double2float_rn(d - (double)h)};
}
// Sum over a warp (xor butterfly, result in every lane).
__device__ __forceinline__ DF df_warp_sum(DF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DF w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = df_add(v, w);
  }
  return v;
}

template <bool MIXED>
struct Acc;
template <>
struct Acc<false> {
  typedef SumD type;
};
template <>
struct Acc<true> {
  typedef KahanF type;
};

// ---------------------------------------------------------------------------
// Deterministic reductions: fixed xor-butterfly inside a warp, then warp
// results combined in warp order.  Results depend only on blockDim.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Three warp_sum calls at once, with the same additions (and bits): the
// first two butterfly levels split the lanes between the values (after xor
// 16 lanes 0-15 hold a and b, lanes 16-31 c; after xor 8 lanes 0-7 a, 8-15
// b, 16-23 c), each lane adding only what its group keeps, so a lane issues
// 6 FP64 additions instead of 15 (GB300 issues FP64 at one warp
// instruction per 64 clocks per sub-partition).  Every lane after xor s
// holds the butterfly's value of its lane, and the butterfly ends with the
// same value in all lanes.  Every lane gets the three sums.
__device__ __forceinline__ void warp_sum3(double &a, double &b, double &c) {
  const unsigned full = 0xffffffffu;
  const int lane = (int)(threadIdx.x & 31);
  const bool lo = lane < 16, lo8 = (lane & 8) == 0;
  const double s1 = __shfl_xor_sync(full, lo ? c : a, 16);
  const double s2 = __shfl_xor_sync(full, lo ? 0.0 : b, 16);
  const double k1 = (lo ? a : c) + s1;
  const double k2 = (lo ? b : 0.0) + s2;
  double v = (lo8 ? k1 : k2) + __shfl_xor_sync(full, lo8 ? k2 : k1, 8);
  v += __shfl_xor_sync(full, v, 4);
  v += __shfl_xor_sync(full, v, 2);
  v += __shfl_xor_sync(full, v, 1);
  a = __shfl_sync(full, v, 0);
  b = __shfl_sync(full, v, 8);
  c = __shfl_sync(full, v, 16);
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// The FP64 explicit Schur product's fixed summation trees (both FP64 PCG
// forms, the two-kernel product in k_schur.cu and the grid kernel, use
// them, so they agree bitwise):
//  * a row of S times p: each block's dot over its nine columns is an FMA
//    chain in column order; the row's m block dots (the diagonal block
//    last) are summed by the pairwise tree: at level s = 1, 2, 4, ...,
//    d[i] += d[i + s] for every i that is a multiple of 2 s with
//    i + s < m; the sum is d[0];
//  * a camera's p.q from its nine rows' p_i q_i: sum9_tree;
//  * the problem's p.q from its cameras' values: chunks of 32 cameras, each
//    summed by an xor butterfly over the lanes, then the pairwise tree over
//    the chunks (cta_chunked_sum).
// Number of additions level s of the pairwise tree does on m values.
__host__ __device__ __forceinline__ int tree_adds(int m, int s) { return m > s ? (m - 1 - s) / (2 * s) + 1 : 0; }

__device__ __forceinline__ double sum9_tree(const double x[9]) {
  const double a = (x[0] + x[1]) + (x[2] + x[3]);
  const double b = (x[4] + x[5]) + (x[6] + x[7]);
  return (a + b) + x[8];
}

// The pairwise tree over x[0..m) in shared memory, levels s = 1, 2, 4, ...
// (the additions of a level spread over the CTA's threads, a barrier after
// each level); the sum ends in x[0].  Call from every thread of the CTA.
__device__ __forceinline__ void cta_pairwise_tree(double *x, int m) {
  for (int s = 1; s < m; s <<= 1) {
    for (int k = (int)threadIdx.x; k < tree_adds(m, s); k += (int)blockDim.x) x[2 * s * k] += x[2 * s * k + s];
    __syncthreads();
  }
}

// cta_pairwise_tree's additions over x[0..m), m <= 32, by one warp: lane l
// holds x[l] (0 beyond m); the sum ends in lane 0.  Call from a whole warp.
__device__ __forceinline__ double warp_pairwise_tree(double v, int m) {
  const int lane = (int)(threadIdx.x & 31);
  for (int s = 1; s < m; s <<= 1) {
    const double o = __shfl_down_sync(0xffffffffu, v, s);
    if ((lane & (2 * s - 1)) == 0 && lane + s < m) v += o;
  }
  return v;
}

// Four warp_sum calls at once, as warp_sum3 (after xor 16 lanes 0-15 hold
// a and b, lanes 16-31 c and d; after xor 8 lanes 0-7 a, 8-15 b, 16-23 c,
// 24-31 d): 6 FP64 additions a lane instead of 20.  Lanes 8 h .. 8 h + 7
// return the sum of value h.
__device__ __forceinline__ double warp_sum4_scatter(double a, double b, double c, double d) {
  const unsigned full = 0xffffffffu;
  const int lane = (int)(threadIdx.x & 31);
  const bool lo = lane < 16, lo8 = (lane & 8) == 0;
  const double k1 = (lo ? a : c) + __shfl_xor_sync(full, lo ? c : a, 16);
  const double k2 = (lo ? b : d) + __shfl_xor_sync(full, lo ? d : b, 16);
  double v = (lo8 ? k1 : k2) + __shfl_xor_sync(full, lo8 ? k2 : k1, 8);
  v += __shfl_xor_sync(full, v, 4);
  v += __shfl_xor_sync(full, v, 2);
  v += __shfl_xor_sync(full, v, 1);
  return v;
}

// The CTA's sum of v[0..n) (global memory, read with __ldcg, or shared
// memory): chunks of 32 values, each an xor butterfly over a warp's lanes
// (four chunks per warp pass, their loads in flight together and their
// butterflies at once), then the pairwise tree over the chunk sums;
// `scratch` holds (n + 31) / 32 doubles of shared memory.  Call from every
// thread of the CTA (whole warps); the total is in scratch[0] after the
// call (which ends with a barrier), 0 for n = 0.
template <bool GLOBAL>
__device__ __forceinline__ void cta_chunked_sum(const double *v, int n, double *scratch) {
  const int lane = (int)(threadIdx.x & 31), warp = (int)(threadIdx.x >> 5), nw = (int)(blockDim.x >> 5);
  const int nch = (n + 31) / 32;
  for (int j0 = 4 * warp; j0 < nch; j0 += 4 * nw) {
    double x[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int e = 32 * (j0 + h) + lane;
      x[h] = 0.0;
      if (e < n) x[h] = GLOBAL ? __ldcg(v + e) : v[e];
    }
    const double s = warp_sum4_scatter(x[0], x[1], x[2], x[3]);
    const int j = j0 + (lane >> 3);
    if ((lane & 7) == 0 && j < nch) scratch[j] = s;
  }
  if (nch == 0 && threadIdx.x == 0) scratch[0] = 0.0;
  __syncthreads();
  cta_pairwise_tree(scratch, nch);
}

// Sum over the CTA; result valid in every thread.  `red` needs blockDim/32
// doubles.  Contains __syncthreads(): call from all threads.  Thread 0 adds
// the warp sums in warp order and broadcasts the total (GB300 issues FP64 at
// about two operations per clock per SM, so the total is formed once per CTA,
// not once per thread).
__device__ __forceinline__ double block_sum(double v, double *red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w];
    red[0] = s;
  }
  __syncthreads();
  return red[0];
}
__device__ __forceinline__ double block_max(double v, double *red) {
  v = warp_max(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s = fmax(s, red[w]);
    red[0] = s;
  }
  __syncthreads();
  return red[0];
}

// Strided sum of a[begin..end) by the whole CTA in a fixed order (L2 loads:
// the values may come from other CTAs of the same kernel).
__device__ __forceinline__ double block_range_sum(const double *a, int begin, int end, int stride,
                                                  double *red) {
  double s = 0.0;
#pragma unroll 8
  for (int i = begin + threadIdx.x; i < end; i += blockDim.x) s += __ldcg(a + (size_t)i * stride);
  return block_sum(s, red);
}
__device__ __forceinline__ double block_range_max(const double *a, int begin, int end, int stride,
                                                  double *red) {
  double s = 0.0;
#pragma unroll 8
  for (int i = begin + threadIdx.x; i < end; i += blockDim.x) s = fmax(s, __ldcg(a + (size_t)i * stride));
  return block_max(s, red);
}

// N range reductions in one pass (one round of loads, one set of barriers):
// value j is the sum, or with is_max[j] the maximum (from 0), of a[j][i *
// stride[j]] over i in [begin[j], end[j]), each in exactly the order of its
// own block_range_sum / block_range_max (so the same bits).  The totals are
// valid in thread 0.  `red` needs (blockDim / 32) * N doubles.
template <int N>
__device__ __forceinline__ void block_range_multi(const double *const (&a)[N], const int (&begin)[N],
                                                  const int (&end)[N], const int (&stride)[N],
                                                  const bool (&is_max)[N], double (&out)[N], double *red) {
  double v[N];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    v[j] = 0.0;
#pragma unroll 8
    for (int i = begin[j] + threadIdx.x; i < end[j]; i += blockDim.x) {
      const double x = __ldcg(a[j] + (size_t)i * stride[j]);
      v[j] = is_max[j] ? fmax(v[j], x) : v[j] + x;
    }
  }
#pragma unroll
  for (int j = 0; j < N; ++j) v[j] = is_max[j] ? warp_max(v[j]) : warp_sum(v[j]);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < N; ++j) red[N * warp + j] = v[j];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < N; ++j) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s = is_max[j] ? fmax(s, red[N * w + j]) : s + red[N * w + j];
      out[j] = s;
    }
}

// "Last CTA done" detection without waiting: each CTA bumps a counter after
// a CTA barrier and a device-scope fence by the bumping thread (the barrier
// orders every thread's earlier writes before that fence, the pattern of a
// cooperative grid barrier); the CTA that brings the counter to `total`
// fences again, so after the final barrier all its threads see every CTA's
// results (read them with __ldcg), and resets the counter.  Returns true in
// every thread of the last CTA.
__device__ __forceinline__ bool last_block_done(uint32_t *counter, uint32_t total, int *flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const uint32_t prev = atomicAdd(counter, 1u);
    const int last = (prev == total - 1u);
    if (last) {
      *counter = 0u;
      __threadfence();
    }
    *flag = last;
  }
  __syncthreads();
  return *flag != 0;
}

// ---------------------------------------------------------------------------
// Camera table: R and dR/dw_k of the Rodrigues formula, evaluated exactly as
// utils/geometry/rotation.h:133-199 does on forward-mode duals (theta^2 >
// DBL_EPSILON branch and first-order branch), once per camera.  Per
// observation R*X and dR_k*X then reproduce the dual-number Jacobian of the
// rotation, including its rounding near the branch point.
// ---------------------------------------------------------------------------
struct J3 {
  double a, d0, d1, d2;
};
__device__ __forceinline__ J3 j3c(double a) { return J3{a, 0.0, 0.0, 0.0}; }
__device__ __forceinline__ J3 j3add(J3 x, J3 y) { return J3{x.a + y.a, x.d0 + y.d0, x.d1 + y.d1, x.d2 + y.d2}; }
__device__ __forceinline__ J3 j3sub(J3 x, J3 y) { return J3{x.a - y.a, x.d0 - y.d0, x.d1 - y.d1, x.d2 - y.d2}; }
__device__ __forceinline__ J3 j3mul(J3 x, J3 y) {
  return J3{x.a * y.a, x.a * y.d0 + x.d0 * y.a, x.a * y.d1 + x.d1 * y.a, x.a * y.d2 + x.d2 * y.a};
}

// Fills tab[0..8] = R (row-major), tab[9 + 9k + 3i + j] = dR_k[i][j].
__device__ inline void rotation_and_derivatives(const double *aa_in, double *tab) {
  const J3 aa[3] = {J3{aa_in[0], 1.0, 0.0, 0.0}, J3{aa_in[1], 0.0, 1.0, 0.0}, J3{aa_in[2], 0.0, 0.0, 1.0}};
  const J3 theta2 = j3add(j3add(j3mul(aa[0], aa[0]), j3mul(aa[1], aa[1])), j3mul(aa[2], aa[2]));
  if (theta2.a > DBL_EPSILON) {
    // theta = sqrt(theta2), c = cos, s = sin, inv = 1/theta (dual rules)
    const double th = sqrt(theta2.a);
    const double fth = 1.0 / (2.0 * th);
    const J3 theta{th, theta2.d0 * fth, theta2.d1 * fth, theta2.d2 * fth};
    double sv, cv;
    sincos(theta.a, &sv, &cv);
    const double mcs = -sv;
    const J3 c{cv, mcs * theta.d0, mcs * theta.d1, mcs * theta.d2};
    const J3 s{sv, cv * theta.d0, cv * theta.d1, cv * theta.d2};
    const double fi = -1.0 / (theta.a * theta.a);
    const J3 inv{1.0 / theta.a, theta.d0 * fi, theta.d1 * fi, theta.d2 * fi};
    const J3 w[3] = {j3mul(aa[0], inv), j3mul(aa[1], inv), j3mul(aa[2], inv)};
    const J3 omc = j3sub(j3c(1.0), c);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const J3 pt[3] = {j3c(j == 0 ? 1.0 : 0.0), j3c(j == 1 ? 1.0 : 0.0), j3c(j == 2 ? 1.0 : 0.0)};
      const J3 wx[3] = {j3sub(j3mul(w[1], pt[2]), j3mul(w[2], pt[1])),
                        j3sub(j3mul(w[2], pt[0]), j3mul(w[0], pt[2])),
                        j3sub(j3mul(w[0], pt[1]), j3mul(w[1], pt[0]))};
      const J3 dot = j3add(j3add(j3mul(w[0], pt[0]), j3mul(w[1], pt[1])), j3mul(w[2], pt[2]));
      const J3 tmp = j3mul(dot, omc);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const J3 res = j3add(j3add(j3mul(pt[i], c), j3mul(wx[i], s)), j3mul(w[i], tmp));
        tab[3 * i + j] = res.a;
        tab[9 + 0 + 3 * i + j] = res.d0;
        tab[9 + 9 + 3 * i + j] = res.d1;
        tab[9 + 18 + 3 * i + j] = res.d2;
      }
    }
  } else {
    // R X = X + w x X:  R = I + [w]_x,  dR_k X = e_k x X
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const J3 pt[3] = {j3c(j == 0 ? 1.0 : 0.0), j3c(j == 1 ? 1.0 : 0.0), j3c(j == 2 ? 1.0 : 0.0)};
      const J3 wx[3] = {j3sub(j3mul(aa[1], pt[2]), j3mul(aa[2], pt[1])),
                        j3sub(j3mul(aa[2], pt[0]), j3mul(aa[0], pt[2])),
                        j3sub(j3mul(aa[0], pt[1]), j3mul(aa[1], pt[0]))};
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const J3 res = j3add(pt[i], wx[i]);
        tab[3 * i + j] = res.a;
        tab[9 + 0 + 3 * i + j] = res.d0;
        tab[9 + 9 + 3 * i + j] = res.d1;
        tab[9 + 18 + 3 * i + j] = res.d2;
      }
    }
  }
}

// R only (candidate-point cost evaluation).  Must produce bit-identical R to
// rotation_and_derivatives, so it runs the same code and drops the rest.
__device__ inline void camera_table_entry(const double *cam, double *tab, bool derivatives) {
  double t[kCamTable];
  rotation_and_derivatives(cam, t);
  const int n = derivatives ? 36 : 9;
  for (int k = 0; k < n; ++k) tab[k] = t[k];
  tab[36] = cam[3];
  tab[37] = cam[4];
  tab[38] = cam[5];
  tab[39] = cam[6];
  tab[40] = cam[7];
  tab[41] = cam[8];
}

// ---------------------------------------------------------------------------
// Left-multiplicative rotation update R <- exp(dw) R (the g2o variant's
// VertexPoseAndIntrinsics::oplusImpl, test_bundle_adjustment_g2o.cpp:84-90).
// At dw = 0, d(exp(dw) R X)/d dw_k = e_k x (R X), so dR_k = [e_k]_x R: rows
// of R moved and negated, exact.  Replaces tab[9..35] of a camera table.
__device__ inline void so3_left_derivatives(double *tab) {
  const double *R = tab;
  double *d0 = tab + 9, *d1 = tab + 18, *d2 = tab + 27;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    d0[0 + j] = 0.0, d0[3 + j] = -R[6 + j], d0[6 + j] = R[3 + j];
    d1[0 + j] = R[6 + j], d1[3 + j] = 0.0, d1[6 + j] = -R[0 + j];
    d2[0 + j] = -R[3 + j], d2[3 + j] = R[0 + j], d2[6 + j] = 0.0;
  }
}

// Unit quaternion (s, v) of angle-axis w: (cos(|w|/2), sin(|w|/2) w / |w|);
// (1, w / 2) at w = 0.
__device__ inline void aa_quat(const double *w, double q[4]) {
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  if (th2 > 0.0) {
    const double th = sqrt(th2);
    double sh, ch;
    sincos(0.5 * th, &sh, &ch);
    const double sc = sh / th;
    q[0] = ch, q[1] = w[0] * sc, q[2] = w[1] * sc, q[3] = w[2] * sc;
  } else {
    q[0] = 1.0, q[1] = 0.5 * w[0], q[2] = 0.5 * w[1], q[3] = 0.5 * w[2];
  }
}

// out = log(exp(dw) exp(w)) in angle-axis form: Hamilton product of the two
// unit quaternions, sign fixed to s >= 0, w' = 2 atan2(|v|, s) v / |v|.
__device__ inline void compose_left(const double *dw, const double *w, double *out) {
  double a[4], b[4], q[4];
  aa_quat(dw, a);
  aa_quat(w, b);
  q[0] = a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
  q[1] = a[0] * b[1] + b[0] * a[1] + (a[2] * b[3] - a[3] * b[2]);
  q[2] = a[0] * b[2] + b[0] * a[2] + (a[3] * b[1] - a[1] * b[3]);
  q[3] = a[0] * b[3] + b[0] * a[3] + (a[1] * b[2] - a[2] * b[1]);
  const double sg = q[0] < 0.0 ? -1.0 : 1.0;
  const double s2 = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (s2 > 0.0) {
    const double sn = sqrt(s2), f = sg * 2.0 * atan2(sn, sg * q[0]) / sn;
    out[0] = q[1] * f, out[1] = q[2] * f, out[2] = q[3] * f;
  } else {
    out[0] = 0.0, out[1] = 0.0, out[2] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Snavely projection (utils/camera/SnavelyReprojectionError.h:61-87) on the
// camera table: P = R X + t; x' = -P_x/P_z; d = 1 + r2 (k1 + k2 r2);
// prediction = f d x'.  Residual = prediction - observation (:49-50).
// ---------------------------------------------------------------------------
struct Proj {
  double P[3];
  double iz;  // 1 / P_z
  double xp, yp, r2, dist, f, k1, k2;
  double ru, rv;
};

__device__ __forceinline__ void project(const double *tab, const double *X, double2 uv, Proj &o) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
    o.P[i] = tab[3 * i + 0] * X[0] + tab[3 * i + 1] * X[1] + tab[3 * i + 2] * X[2] + tab[36 + i];
  // one reciprocal of P_z (within an FP64 rounding of -P_x / P_z, -P_y / P_z)
  o.iz = recip_nr(o.P[2]);
  o.xp = -o.P[0] * o.iz;
  o.yp = -o.P[1] * o.iz;
  o.f = tab[39];
  o.k1 = tab[40];
  o.k2 = tab[41];
  o.r2 = o.xp * o.xp + o.yp * o.yp;
  o.dist = 1.0 + o.r2 * (o.k1 + o.k2 * o.r2);
  o.ru = o.f * o.dist * o.xp - uv.x;
  o.rv = o.f * o.dist * o.yp - uv.y;
}

// ---------------------------------------------------------------------------
// Local-BA windows: full_slam's stereo rig (EdgeProjection,
// full_slam/include/myslam/g2o_types.h:127-175).  The camera table holds the
// keyframe pose (R at tab[0..8], t at tab[36..38]); rig = fx, fy, cx, cy,
// then R_e (9) and t_e (3) of the two rig cameras.
//   Q = R_e (R X + t) + t_e,  pixel = (K Q) / Q_z,  error = measurement - pixel
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rig_project(const double *tab, const double *rig, int cam, const double *X,
                                            double2 uv, double Q[3], double &ru, double &rv) {
  double P[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) P[i] = tab[3 * i + 0] * X[0] + tab[3 * i + 1] * X[1] + tab[3 * i + 2] * X[2] + tab[36 + i];
  const double *Re = rig + 4 + 12 * cam;
#pragma unroll
  for (int i = 0; i < 3; ++i) Q[i] = Re[3 * i + 0] * P[0] + Re[3 * i + 1] * P[1] + Re[3 * i + 2] * P[2] + Re[9 + i];
  ru = uv.x - (rig[0] * Q[0] + rig[2] * Q[2]) / Q[2];
  rv = uv.y - (rig[1] * Q[1] + rig[3] * Q[2]) / Q[2];
}

// Residual and the reference's Jacobian (EdgeProjection::linearizeOplus,
// g2o_types.h:146-169) of one observation: with (X, Y, Z) = Q and
// zi = 1 / (Z + 1e-18), the pose columns
//   u: rotation fx X Y zi^2, -fx - fx X^2 zi^2, fx Y zi | translation -fx zi, 0, fx X zi^2
//   v: rotation fy + fy Y^2 zi^2, -fy X Y zi^2, -fy X zi | translation 0, -fy zi, fy Y zi^2
// (camera slots 0-2 rotation, 3-5 translation, 6-8 zero) and the point
// columns = the translation columns times R_e R.
__device__ __forceinline__ void rig_jacobian(const double *tab, const double *rig, int cam, const double *X,
                                             double2 uv, double ju[12], double jv[12], double &ru, double &rv) {
  double Q[3];
  rig_project(tab, rig, cam, X, uv, Q, ru, rv);
  const double fx = rig[0], fy = rig[1];
  const double zi = 1.0 / (Q[2] + 1e-18), zi2 = zi * zi;
  const double tu0 = -fx * zi, tu2 = fx * Q[0] * zi2, tv1 = -fy * zi, tv2 = fy * Q[1] * zi2;
  ju[0] = fx * Q[0] * Q[1] * zi2, ju[1] = -fx - fx * Q[0] * Q[0] * zi2, ju[2] = fx * Q[1] * zi;
  jv[0] = fy + fy * Q[1] * Q[1] * zi2, jv[1] = -fy * Q[0] * Q[1] * zi2, jv[2] = -fy * Q[0] * zi;
  ju[3] = tu0, ju[4] = 0.0, ju[5] = tu2;
  jv[3] = 0.0, jv[4] = tv1, jv[5] = tv2;
  ju[6] = ju[7] = ju[8] = 0.0;
  jv[6] = jv[7] = jv[8] = 0.0;
  const double *Re = rig + 4 + 12 * cam;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // column k of R_e R
    const double a0 = Re[0] * tab[k] + Re[1] * tab[3 + k] + Re[2] * tab[6 + k];
    const double a1 = Re[3] * tab[k] + Re[4] * tab[3 + k] + Re[5] * tab[6 + k];
    const double a2 = Re[6] * tab[k] + Re[7] * tab[3 + k] + Re[8] * tab[6 + k];
    ju[9 + k] = tu0 * a0 + tu2 * a2;
    jv[9 + k] = tv1 * a1 + tv2 * a2;
  }
}

// Rodrigues rotation of p by angle-axis w (utils/geometry/rotation.h:133-199
// form: the full formula for theta^2 > DBL_EPSILON, p + w x p below).
__device__ __forceinline__ void aa_rotate(const double *w, const double *p, double *out) {
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double wxp[3] = {w[1] * p[2] - w[2] * p[1], w[2] * p[0] - w[0] * p[2], w[0] * p[1] - w[1] * p[0]};
  if (th2 > DBL_EPSILON) {
    const double th = sqrt(th2), it = 1.0 / th;
    double s, c;
    sincos(th, &s, &c);
    const double k[3] = {w[0] * it, w[1] * it, w[2] * it};
    const double kd = k[0] * p[0] + k[1] * p[1] + k[2] * p[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = p[i] * c + wxp[i] * it * s + k[i] * kd * (1.0 - c);
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = p[i] + wxp[i];
  }
}

// T <- exp(xi) T on SE3 (VertexPose::oplusImpl, g2o_types.h:55-60), xi =
// (rotation dw, translation du): R' = exp(dw) R, t' = exp(dw) t + V(dw) du,
// V = I + (1 - cos th)/th^2 [dw]x + (th - sin th)/th^3 [dw]x^2 (series below
// th = 1e-4).  pose = angle-axis (3), translation (3).
__device__ inline void se3_compose_left(const double *dw, const double *du, const double *pose, double *out) {
  const double th2 = dw[0] * dw[0] + dw[1] * dw[1] + dw[2] * dw[2], th = sqrt(th2);
  double a, b;
  if (th < 1e-4) {
    a = 0.5 - th2 / 24.0;
    b = 1.0 / 6.0 - th2 / 120.0;
  } else {
    double s, c;
    sincos(th, &s, &c);
    a = (1.0 - c) / th2;
    b = (th - s) / (th2 * th);
  }
  const double c1[3] = {dw[1] * du[2] - dw[2] * du[1], dw[2] * du[0] - dw[0] * du[2], dw[0] * du[1] - dw[1] * du[0]};
  const double c2[3] = {dw[1] * c1[2] - dw[2] * c1[1], dw[2] * c1[0] - dw[0] * c1[2], dw[0] * c1[1] - dw[1] * c1[0]};
  double rt[3], w[3];
  aa_rotate(dw, pose + 3, rt);
  compose_left(dw, pose, w);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    out[i] = w[i];
    out[3 + i] = rt[i] + (du[i] + a * c1[i] + b * c2[i]);
  }
}

// Ceres robust-loss rho(s) (LossFunction::Evaluate) for trivial, Huber(a),
// Cauchy(a).
__device__ __forceinline__ void loss_rho(int loss, double a, double s, double rho[3]) {
  if (loss == GBA_LOSS_HUBER) {
    const double b = a * a;
    if (s > b) {
      const double r = sqrt(s);
      rho[0] = 2.0 * a * r - b;
      rho[1] = fmax(DBL_MIN, a / r);
      rho[2] = -rho[1] / (2.0 * s);
    } else {
      rho[0] = s;
      rho[1] = 1.0;
      rho[2] = 0.0;
    }
  } else if (loss == GBA_LOSS_CAUCHY) {
    const double b = a * a, c = 1.0 / b;
    const double sum = 1.0 + s * c;
    const double inv = 1.0 / sum;
    rho[0] = b * log(sum);
    rho[1] = fmax(DBL_MIN, inv);
    rho[2] = -c * (inv * inv);
  } else {
    rho[0] = s;
    rho[1] = 1.0;
    rho[2] = 0.0;
  }
}

__device__ __forceinline__ double block_cost(int loss, double a, double ru, double rv) {
  const double s = ru * ru + rv * rv;
  if (loss == GBA_LOSS_TRIVIAL) return 0.5 * s;
  double rho[3];
  loss_rho(loss, a, s, rho);
  return 0.5 * rho[0];
}

// Corrector of a residual block: r' = residual_scaling * r and
// J' = sqrt_rho1 (J - alpha_sq_norm r r^T J).
struct Corrector {
  double sqrt_rho1, residual_scaling, alpha_sq_norm;
};
__device__ __forceinline__ Corrector make_corrector(int loss, double a, double ru, double rv) {
  Corrector c{1.0, 1.0, 0.0};
  if (loss == GBA_LOSS_TRIVIAL) return c;
  const double s = ru * ru + rv * rv;
  double rho[3];
  loss_rho(loss, a, s, rho);
  c.sqrt_rho1 = sqrt(rho[1]);
  if (s == 0.0 || rho[2] <= 0.0) {
    c.residual_scaling = c.sqrt_rho1;
    c.alpha_sq_norm = 0.0;
  } else {
    const double D = 1.0 + 2.0 * s * rho[2] / rho[1];
    const double alpha = 1.0 - sqrt(D);
    c.residual_scaling = c.sqrt_rho1 / (1.0 - alpha);
    c.alpha_sq_norm = alpha / s;
  }
  return c;
}

// Loads / stores of one observation's Jacobian columns from the SoA layout:
// column k (k = 0..8 camera, 9..11 point) as a (d/du, d/dv) pair at
// jac[k * no + o]; the corrected residual pair at jac[12 * no + o].
template <typename R2>
__device__ __forceinline__ R2 jload(const void *jac, int64_t no, int k, int64_t o) {
  return reinterpret_cast<const R2 *>(jac)[(int64_t)k * no + o];
}
template <typename R2>
__device__ __forceinline__ void jstore(void *jac, int64_t no, int k, int64_t o, R2 v) {
  reinterpret_cast<R2 *>(jac)[(int64_t)k * no + o] = v;
}

// Inverse of a symmetric 3x3 block (packed 00 01 02 11 12 22) by cofactors
// and one reciprocal of the determinant (GB300 issues FP64 square roots and
// divisions slowly; a Cholesky inverse needs three and nine of them).
// Positive definiteness by Sylvester's criterion: the leading principal
// minors C00, C00 C11 - C01^2 and det C must be positive, which is exactly
// when a Cholesky factorisation succeeds.
__device__ __forceinline__ bool spd_inverse3(const double *C, double *Ci) {
  const double a = C[0], b = C[1], c = C[2], d = C[3], e = C[4], f = C[5];
  const double m00 = d * f - e * e;
  const double m01 = c * e - b * f;
  const double m02 = b * e - c * d;
  const double m11 = a * f - c * c;
  const double m12 = b * c - a * e;
  const double m22 = a * d - b * b;
  const double det = a * m00 + b * m01 + c * m02;
  if (!(a > 0.0) || !(m22 > 0.0) || !(det > 0.0)) return false;
  const double id = recip_nr(det);
  Ci[0] = m00 * id;
  Ci[1] = m01 * id;
  Ci[2] = m02 * id;
  Ci[3] = m11 * id;
  Ci[4] = m12 * id;
  Ci[5] = m22 * id;
  return isfinite(Ci[0]) && isfinite(Ci[3]) && isfinite(Ci[5]);
}

// ---------------------------------------------------------------------------
// Trace helper (LM iteration `it` of problem p).
__device__ __forceinline__ void trace_put(const DeviceBatch &B, int p, int it, double cost,
                                          double radius, int pcg, int succ) {
  if (it < 0 || it >= B.trace_cap) return;
  const size_t k = (size_t)p * B.trace_cap + it;
  B.trace_cost[k] = cost;
  B.trace_radius[k] = radius;
  B.trace_pcg[k] = pcg;
  B.trace_succ[k] = succ;
}

}  // namespace gba
