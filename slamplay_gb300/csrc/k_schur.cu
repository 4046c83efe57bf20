// k_schur.cu — the explicit Schur complement (gba_schur GBA_SCHUR_EXPLICIT).
//
// When the cameras' co-visibility is sparse, the reduced camera matrix
//   S = B + Dc^2 - W C^-1 W^T
// has few nonzero 9x9 camera-camera blocks: a 250-camera random walk has
// about 28 per camera, 2.3 MB in FP32, where the Jacobian the implicit
// mat-vec reads on every PCG iteration is 28 MB.  Then S is formed once per
// LM iteration (the points eliminated into camera-camera blocks, as Ceres'
// SPARSE_SCHUR and ITERATIVE_SCHUR with use_explicit_schur_complement do)
// and every PCG iteration multiplies by the blocks, which stay in L2.
//
// With L L^T = C_j^-1 (the point's 3x3 factor) and F_a = J_c^T J_p L of an
// observation a (9x3, formed by the point kernel K3a), the block of cameras
// (i, k) is -sum over the points both see of F_a F_b^T.
//
//  K3c k_schur_form   one CTA per block on or above the diagonal (k >= i):
//                     the F rows of 64 pairs per round staged in shared
//                     memory (the next round's loads in flight while this
//                     one is summed); the sum over the block's pairs, in a
//                     fixed order (three interleaved runs over the pairs'
//                     point order, combined in order; compensated FP32 in
//                     the mixed form), stored with its transpose as block
//                     (k, i).  The diagonal blocks B + Dc^2 - sum F_a F_a^T
//                     come from K3b; a camera that sees a point twice has a
//                     block (i, i) here for the cross terms.
//  K4a' k_schur_spmv  one CTA per camera, one warp per row of its 9x9
//                     blocks, the lanes over the row's blocks (the last
//                     one the diagonal block): q = S p_k with p_k = z_k +
//                     beta_k p_{k-1} formed on the fly exactly as the
//                     implicit mat-vec forms it, and the camera's share of
//                     p.q for the camera kernel.  The blocks are fixed
//                     during the PCG, so their loads are issued before the
//                     wait on the preceding camera kernel.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"
#include "kernels.h"

namespace gba {

namespace {

constexpr int kFormThreads = 256;
constexpr int kFormPairs = 64;  // pairs staged per round
constexpr int kFormSub = 3;     // sub-lanes per block entry (243 of the 256 threads)

__device__ __forceinline__ void pdl_wait_s() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents_s() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// 16-byte vector of the working precision
template <bool MIXED>
struct Vec16;
template <>
struct Vec16<true> {
  typedef float4 type;
};
template <>
struct Vec16<false> {
  typedef double2 type;
};

}  // namespace

// ---------------------------------------------------------------------------
// K3c
template <bool MIXED>
__global__ void __launch_bounds__(kFormThreads) k_schur_form(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Acc<MIXED>::type Acc;
  typedef typename Vec16<MIXED>::type vec;
  constexpr int kVec = (int)(sizeof(vec) / sizeof(real));
  constexpr int kRowVecs = kObsF / kVec;  // 16-byte loads per F row
  constexpr int kRoundVecs = kFormPairs * 2 * kRowVecs;
  constexpr int kPer = (kRoundVecs + kFormThreads - 1) / kFormThreads;  // loads per thread per round
  static_assert(kObsF % kVec == 0, "F rows are whole 16-byte vectors");
  __shared__ __align__(16) real Fs[kFormPairs][2][kObsF];  // F of the row's and the column's observation
  __shared__ Acc part[kFormSub][81];
  const int ub = blockIdx.x, t = threadIdx.x;
  const int blk = B.sblk_up[ub];
  const int p0 = B.sblk_pair[ub], p1 = B.sblk_pair[ub + 1];
  const LMState *L = B.lm + B.cam_problem[B.sblk_col[blk]];
  if (!L->active) return;  // uniform
  const real *F = reinterpret_cast<const real *>(B.obs_F);
  // a round's F rows: every load issued before any is stored (one L2 round
  // trip per round), the next round's loaded while this one is summed
  vec buf[kPer];
  auto load_round = [&](int g) {
    const int n = min(kFormPairs, p1 - g);
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = t + u * kFormThreads;
      if (i < n * 2 * kRowVecs) {
        const int pr = i / (2 * kRowVecs), r = i - 2 * kRowVecs * pr;
        const int side = r / kRowVecs, e = r - kRowVecs * side;
        const int2 ob = B.spair[g + pr];
        buf[u] = reinterpret_cast<const vec *>(F + (size_t)kObsF * (side ? ob.y : ob.x))[e];
      }
    }
  };
  auto store_round = [&](int g) {
    const int n = min(kFormPairs, p1 - g);
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int i = t + u * kFormThreads;
      if (i < n * 2 * kRowVecs) {
        const int pr = i / (2 * kRowVecs), r = i - 2 * kRowVecs * pr;
        const int side = r / kRowVecs, e = r - kRowVecs * side;
        *reinterpret_cast<vec *>(&Fs[pr][side][kVec * e]) = buf[u];
      }
    }
  };
  // sub-lane `sub` of entry (i, k) sums the pairs sub, sub + kFormSub, ...
  // of every round, in order
  const int sub = t / 81, en = t - 81 * sub, ei = en / 9, ek = en - 9 * ei;
  Acc acc;
  acc.init();
  load_round(p0);
  store_round(p0);
  __syncthreads();
  for (int g = p0; g < p1; g += kFormPairs) {
    const int n = min(kFormPairs, p1 - g);
    const bool more = g + kFormPairs < p1;
    if (more) load_round(g + kFormPairs);
    if (sub < kFormSub)
      for (int u = sub; u < n; u += kFormSub) {
        const real *fa = &Fs[u][0][3 * ei], *fb = &Fs[u][1][3 * ek];
        if constexpr (MIXED)
          acc.add(fa[0] * fb[0] + fa[1] * fb[1] + fa[2] * fb[2]);
        else  // FP64: one FMA chain through the accumulator (three FP64 operations a pair, not four)
          acc.s = fma(fa[2], fb[2], fma(fa[1], fb[1], fma(fa[0], fb[0], acc.s)));
      }
    __syncthreads();  // the stage is reused
    if (more) store_round(g + kFormPairs);
    __syncthreads();
  }
  if (sub < kFormSub) part[sub][en] = acc;
  __syncthreads();
  if (t < 81) {
    Acc s = part[0][t];
#pragma unroll
    for (int j = 1; j < kFormSub; ++j) s.merge(part[j][t]);
    const real v = -(real)s.rvalue();
    real *vals = reinterpret_cast<real *>(B.sblk_val);
    const int i = t / 9, k = t - 9 * i;
    vals[81 * (size_t)blk + t] = v;
    const int tr = B.sblk_tr[blk];
    if (tr != blk) vals[81 * (size_t)tr + 9 * k + i] = v;
  }
}

void launch_schur_form(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  if (!b.explicit_schur || b.nup == 0) return;
  if (mixed)
    k_schur_form<true><<<b.nup, kFormThreads, 0, s>>>(b);
  else
    k_schur_form<false><<<b.nup, kFormThreads, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// K4a'
constexpr int kSpmvThreads = 9 * 32;
constexpr int kSpmvPrefetch = 2;  // blocks per lane whose values load before the wait

template <bool MIXED>
__global__ void __launch_bounds__(kSpmvThreads) k_schur_spmv(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  __shared__ double pqs[9];
  const int c = blockIdx.x, t = threadIdx.x;
  const int q = t >> 5, lane = t & 31;
  const int prob = B.cam_problem[c];
  const int r0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - r0;
  // virtual block v of the row: v < nb the off-diagonal block r0 + v, v = nb
  // the diagonal block; lane l takes v = l, l + 32, ...
  const real *vals = reinterpret_cast<const real *>(B.sblk_val);
  const real *diag = reinterpret_cast<const real *>(B.cam_Sii) + 81 * (size_t)c + 9 * q;
  real pre[kSpmvPrefetch][9];
  int pcol[kSpmvPrefetch];
#pragma unroll
  for (int u = 0; u < kSpmvPrefetch; ++u) {
    const int v = lane + 32 * u;
    pcol[u] = -1;
#pragma unroll
    for (int cc = 0; cc < 9; ++cc) pre[u][cc] = 0;
    if (v <= nb) {
      const real *row = v < nb ? vals + 81 * (size_t)(r0 + v) + 9 * q : diag;
      pcol[u] = v < nb ? B.sblk_col[r0 + v] : c;
#pragma unroll
      for (int cc = 0; cc < 9; ++cc) pre[u][cc] = row[cc];
    }
  }
  pdl_wait_s();
  pdl_launch_dependents_s();
  const LMState *L = B.lm + prob;
  if (!(L->active && L->pcg_active)) return;  // uniform over the CTA
  const int k = L->pcg_iterations;
  const double beta = L->beta;
  const real *zv = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_zf : (const void *)B.pcg_z);
  const real *pvv = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_pf : (const void *)B.pcg_p);
  // p_k of a camera coordinate: the FP64 form evaluates the camera kernel's
  // expression, the mixed form the same recurrence in FP32 on the FP32
  // copies (as the implicit mat-vec)
  auto pdir = [&](size_t idx) -> real {
    const real z = zv[idx];
    if (k == 0) return z;
    if (MIXED) return (real)__fmaf_rn((float)beta, (float)pvv[idx], (float)z);
    return (real)fma(beta, (double)pvv[idx], (double)z);
  };
  auto row_dot = [&](const real *row, int col) -> real {
    real s = 0;
#pragma unroll
    for (int cc = 0; cc < 9; ++cc) s += row[cc] * pdir(9 * (size_t)col + cc);
    return s;
  };
  // the lane's blocks in order: FP64 sums in the FP64 form, double-float in
  // the mixed form
  DF af = df_zero();
  double ad = 0.0;
#pragma unroll
  for (int u = 0; u < kSpmvPrefetch; ++u)
    if (pcol[u] >= 0) {
      const real s = row_dot(pre[u], pcol[u]);
      if (MIXED)
        af = df_add(af, DF{(float)s, 0.f});
      else
        ad += (double)s;
    }
  for (int v = lane + 32 * kSpmvPrefetch; v <= nb; v += 32) {
    const real *row = v < nb ? vals + 81 * (size_t)(r0 + v) + 9 * q : diag;
    const real s = row_dot(row, v < nb ? B.sblk_col[r0 + v] : c);
    if (MIXED)
      af = df_add(af, DF{(float)s, 0.f});
    else
      ad += (double)s;
  }
  // the row's sum over the lanes (butterfly: a fixed order)
  double qv;
  if (MIXED) {
    af = df_warp_sum(af);
    qv = df_value(af);
  } else {
    qv = warp_sum(ad);
  }
  if (lane == 0) {
    const size_t i = 9 * (size_t)c + q;
    B.pcg_q[i] = qv;
    pqs[q] = (double)pdir(i) * qv;
  }
  __syncthreads();
  if (t == 0) {
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < 9; ++r) s += pqs[r];
    B.spmv_red[c] = s;
  }
}

// K4a' of the FP64 form: one CTA per camera; the direction p_k = z_k +
// beta_k p_{k-1} at the columns of the camera's blocks formed once into
// shared memory (`stage`; else formed at each use, nine times per block),
// the block dots of its rows (nine-column FMA chains) into shared memory,
// `rpp` rows at a time, each row summed by the pairwise tree, then the
// camera's p.q (sum9_tree of its rows' p_i q_i): the grid PCG's arithmetic,
// so both forms agree bitwise.
__global__ void __launch_bounds__(kSpmvThreads) k_schur_spmv64(DeviceBatch B, int rpp, int stage) {
  extern __shared__ double sp_smem[];  // [m][9] staged direction (stage), then [rpp][m]
  __shared__ double pqs[9];
  const int c = blockIdx.x, t = threadIdx.x;
  const int prob = B.cam_problem[c];
  pdl_wait_s();
  pdl_launch_dependents_s();
  const LMState *L = B.lm + prob;
  if (!(L->active && L->pcg_active)) return;  // uniform over the CTA
  const int k = L->pcg_iterations;
  const double beta = L->beta;
  auto pdir = [&](size_t idx) -> double {
    const double z = B.pcg_z[idx];
    if (k == 0) return z;
    return fma(beta, B.pcg_p[idx], z);
  };
  const int r0 = B.sblk_row[c], nb = B.sblk_row[c + 1] - r0, m = nb + 1;
  const double *vals = reinterpret_cast<const double *>(B.sblk_val);
  const double *diag = reinterpret_cast<const double *>(B.cam_Sii) + 81 * (size_t)c;
  double *sp_p = sp_smem, *sp_d = sp_smem + (stage ? 9 * (size_t)m : 0);
  if (stage) {  // the diagonal block's column (the camera's own) last
    for (int e = t; e < 9 * m; e += kSpmvThreads) {
      const int v = e / 9, cc = e - 9 * v;
      sp_p[e] = pdir(9 * (size_t)(v < nb ? B.sblk_col[r0 + v] : c) + cc);
    }
    __syncthreads();
  }
  for (int q0 = 0; q0 < 9; q0 += rpp) {
    const int nr = min(rpp, 9 - q0);
    for (int e = t; e < nr * m; e += kSpmvThreads) {
      const int rr = e / m, v = e - rr * m;
      const double *row = (v < nb ? vals + 81 * (size_t)(r0 + v) : diag) + 9 * (q0 + rr);
      double d = 0.0;
      if (stage) {
        const double *pp = sp_p + 9 * v;
#pragma unroll
        for (int cc = 0; cc < 9; ++cc) d = fma(row[cc], pp[cc], d);
      } else {
        const int col = v < nb ? B.sblk_col[r0 + v] : c;
#pragma unroll
        for (int cc = 0; cc < 9; ++cc) d = fma(row[cc], pdir(9 * (size_t)col + cc), d);
      }
      sp_d[e] = d;
    }
    __syncthreads();
    for (int s = 1; s < m; s <<= 1) {
      const int na = tree_adds(m, s);
      for (int e = t; e < nr * na; e += kSpmvThreads) {
        const int rr = e / na, i = 2 * s * (e - rr * na);
        sp_d[rr * m + i] += sp_d[rr * m + i + s];
      }
      __syncthreads();
    }
    if (t < nr) {
      const int q = q0 + t;
      const size_t i = 9 * (size_t)c + q;
      const double qv = sp_d[t * m];
      B.pcg_q[i] = qv;
      pqs[q] = (stage ? sp_p[9 * nb + q] : pdir(i)) * qv;
    }
    __syncthreads();
  }
  if (t == 0) B.spmv_red[c] = sum9_tree(pqs);
}

// Rows per pass of k_schur_spmv64 and its shared memory, from the longest
// row (in blocks, the diagonal one included).
static int spmv64_rows(int m_max, size_t *smem, int *stage) {
  int optin = 48 * 1024, dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t budget = (size_t)optin - 4096;
  const size_t mm = (size_t)std::max(m_max, 1);
  // the staged direction when it leaves room for one row's block dots
  *stage = 8 * 10 * mm <= budget ? 1 : 0;
  const size_t rows_budget = budget - (*stage ? 8 * 9 * mm : 0);
  int rpp = 9;
  while (rpp > 1 && 8 * (size_t)rpp * mm > rows_budget) --rpp;
  *smem = 8 * (size_t)rpp * mm + (*stage ? 8 * 9 * mm : 0);
  return rpp;
}

cudaError_t launch_schur_spmv(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl) {
  if (b.nc == 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)b.nc);
  cfg.blockDim = dim3(kSpmvThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  if (mixed) return cudaLaunchKernelEx(&cfg, k_schur_spmv<true>, b);
  size_t smem = 0;
  int stage = 0;
  const int rpp = spmv64_rows(b.sblk_max, &smem, &stage);
  if (smem > 48 * 1024) {
    const cudaError_t e = raise_smem_limit((const void *)k_schur_spmv64, smem);
    if (e != cudaSuccess) return e;
  }
  cfg.dynamicSmemBytes = smem;
  return cudaLaunchKernelEx(&cfg, k_schur_spmv64, b, rpp, stage);
}

}  // namespace gba
