// k_pcg.cu — implicit-Schur preconditioned conjugate gradients on the
// reduced camera system  S x = v,  S = B + Dc^2 - W C^-1 W^T,  with the
// block-Jacobi preconditioner M = blockdiag(S_ii)^-1 (built by K3b).
//
// The recurrence is the textbook (Hestenes-Stiefel) PCG:
//   p_k = z_k + beta_k p_{k-1}  (p_0 = z_0),   q_k = S p_k,
//   alpha_k = (r_k.z_k) / (p_k.q_k),
//   x_{k+1} = x_k + alpha_k p_k,  r_{k+1} = r_k - alpha_k q_k,  z_{k+1} = M r_{k+1},
//   beta_{k+1} = (r_{k+1}.z_{k+1}) / (r_k.z_k).
// With the mixed form's FP32 mat-vec, the single-reduction variants
// (Chronopoulos & Gear, with the shortcut denominator or with p.s expanded
// by bilinearity) drift measurably from the FP64 solve (final LM costs
// 2.5e-5 apart on the 250-camera benchmark problem); this form stays within
// 3e-7, so it pays its second reduction per iteration.
//
// One iteration is two kernels, each parallel over the whole GPU:
//   K4a k_schur_matvec  one CTA per point-segment chunk, one thread per
//       observation: forms p_k for the chunk's cameras, y = J_p^T J_c p,
//       t_j = C_j^-1 sum_j y, J_c^T J_p t_j at the observation's slot in the
//       chunk's camera-sorted order, summed per camera run into one partial
//       per (chunk, camera) at the camera's contiguous (camera-major)
//       position; and the chunk's share of p.q:
//         p.q = sum_cameras p_c.(B_c + Dc^2) p_c - sum_segments p_c.partial,
//       the camera term taken by the chunk that holds the camera's first
//       segment (problems of more than kRedDirect chunks: the last CTA of
//       each group of kRedGroup chunks also sums the group's values).
//   K4b k_pcg_camera    one CTA per block of kPcgBlockCams cameras: p.q from
//       the chunk (or group) values, summed by every CTA of the problem in
//       the same order, so all hold the same alpha_k (a non-positive
//       curvature ends the PCG); q_k = (B + Dc^2) p_k - sum of the camera's
//       partials, x, r, z = M r, and the block's r.z, r.r and x.(v + r); the
//       problem's last block sums them, runs the stopping test on
//       (x_{k+1}, r_{k+1}) and stores beta_{k+1}.  With the explicit Schur
//       complement (k_schur.cu) q_k and the cameras' shares of p.q come
//       from the block-sparse product instead.
// Every cross-CTA sum either is redundant (each CTA sums the same values in
// the same order) or is done once by the CTA that arrives last at a
// counter; there are no spin-waits and no atomics on data, so a solve is
// bitwise deterministic and independent of the other problems of a batch.
// FP64 division and square root are long instruction sequences on GB300's
// FP64 pipe (about 64 cycles per dependent operation), so the scalars are
// formed once per CTA or per problem, with Newton-refined reciprocals.
// GB300 runs FP64 at 1/55 of FP32 throughput, so in the mixed form the
// matrix-like work (the mat-vec partials, M r) runs in FP32 with compensated
// sums, while the vectors x, r, z, p, the products with B and every dot
// product stay FP64.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "kernels.h"

namespace gba {

namespace {

template <bool MIXED>
struct MatvecSmem {
  typedef typename Prec<MIXED>::real real;
  real pseg[kChunkCap][9];   // p of the chunk's cameras (working precision)
  real U[kChunkCap][9];      // first holds w (3 per obs), then u (9 per slot)
  real tpt[kChunkCap][3];
  real arow[kChunkCap][10];  // each thread's current task: row of B and Dc^2
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

// Explicit multiply-adds (no contraction left to the compiler), so the two
// mixed-form mat-vec kernels below compute bitwise the same values.
__device__ __forceinline__ float mad(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double mad(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }

// p_k of one coordinate (both kernels evaluate exactly this expression).
__device__ __forceinline__ double pcg_direction(int k, double beta, double z, double p_old) {
  return k == 0 ? z : fma(beta, p_old, z);
}

// Row q of B (the working-precision copy: FP32 in the mixed form) and Dc^2_q
// of camera c.
template <bool MIXED>
__device__ __forceinline__ void a_row(const DeviceBatch &B, int c, int q, typename Prec<MIXED>::real *row) {
  typedef typename Prec<MIXED>::real real;
  const real *Bc = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_Bf : (const void *)B.cam_B) + 45 * (size_t)c;
#pragma unroll
  for (int kk = 0; kk < 9; ++kk) row[kk] = Bc[sym9(q, kk)];
  row[9] = (real)B.cam_D2[9 * (size_t)c + q];
}

// Row q of (B + Dc^2) y in FP64, from a row given by a_row (two chains of
// five: FP64 operations have a long dependent latency on GB300).
template <typename real>
__device__ __forceinline__ double a_times(const real *row, const double *y, int q) {
  double s0 = (double)row[9] * y[q], s1 = (double)row[8] * y[8];
#pragma unroll
  for (int kk = 0; kk < 8; kk += 2) {
    s0 = fma((double)row[kk], y[kk], s0);
    s1 = fma((double)row[kk + 1], y[kk + 1], s1);
  }
  return s0 + s1;
}

// A chunk (or group) value of p.q: FP64 in the FP64 form, a double-float
// pair in the mixed form (stored in the double slot).
__device__ __forceinline__ DF chunk_value_load(const DeviceBatch &B, size_t slot) {
  const float2 v = __ldcg(reinterpret_cast<const float2 *>(B.chunk_red + slot));
  return DF{v.x, v.y};
}

// Sums the CTA's values (fixed order: warp butterflies, then thread 0 adds
// the warps in order) and stores the total at chunk_red[slot].  Call from
// every thread.
template <bool MIXED>
__device__ __forceinline__ void chunk_value_store(const DeviceBatch &B, size_t slot, double d, DF f, DF *dfred,
                                                  double *red) {
  if (MIXED) {
    f = df_warp_sum(f);
    if ((threadIdx.x & 31) == 0) dfred[threadIdx.x >> 5] = f;
    __syncthreads();
    if (threadIdx.x == 0) {
      DF s = dfred[0];
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s = df_add(s, dfred[w]);
      *reinterpret_cast<float2 *>(B.chunk_red + slot) = make_float2(s.hi, s.lo);
    }
  } else {
    const double v = block_sum(d, red);
    if (threadIdx.x == 0) B.chunk_red[slot] = v;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// K4a
template <bool MIXED>
// (four CTAs per SM in the mixed form: 1,024 threads of at most 64 registers)
__global__ void __launch_bounds__(kChunkCap, MIXED ? 4 : 2) k_schur_matvec(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Prec<MIXED>::real2 real2;
  typedef typename Acc<MIXED>::type Acc;
  extern __shared__ __align__(16) unsigned char k4_smem[];
  MatvecSmem<MIXED> &sm = *reinterpret_cast<MatvecSmem<MIXED> *>(k4_smem);
  __shared__ double red[kChunkCap / 32];
  __shared__ DF dfred[kChunkCap / 32];
  __shared__ int flag;
  const int t = threadIdx.x;
  const int ch = blockIdx.x;
  const ChunkInfo ci = B.chunk[ch];
  const bool valid = t < ci.obs_count;
  // every load that depends only on the chunk is issued before the wait, so
  // one memory round trip covers them all
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
  // the first (segment, coordinate) this thread reduces at the end; when the
  // segment is its camera's first, the row of B + Dc^2 for the camera term
  // of p.q (B and Dc^2 are fixed during the PCG)
  int f_b0 = 0, f_b1 = 0, f_slot = 0;
  size_t f_idx = 0;  // the task's entry of the camera vectors
  bool f_owner = false;
  if (t < ci.seg_count * 9) {
    const int sg = t / 9;
    f_b0 = B.seg_pos[ci.seg_begin + sg];
    f_b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
    f_slot = B.seg_slot[ci.seg_begin + sg];
    const int cam = B.seg_cam[ci.seg_begin + sg];
    f_idx = 9 * (size_t)cam + (t - 9 * sg);
    f_owner = f_slot == B.cam_seg_begin[cam];
    if (f_owner) a_row<MIXED>(B, cam, t - 9 * sg, sm.arow[t]);
  }
  const ProblemInfo pi = B.prob[ci.problem];
  // everything above is fixed during the PCG; from here on the kernel reads
  // what the previous camera-side kernel wrote (and overwrites the partials
  // it read)
  pdl_wait();
  pdl_launch_dependents();
  const LMState *L = B.lm + ci.problem;
  // the first task's z and p_{k-1} (FP32 copies in the mixed form) load
  // together with the problem state (p is only used when k > 0)
  const real *zv = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_zf : (const void *)B.pcg_z);
  const real *pvv = reinterpret_cast<const real *>(MIXED ? (const void *)B.pcg_pf : (const void *)B.pcg_p);
  real f_z = 0, f_p = 0;
  if (t < ci.seg_count * 9) f_z = zv[f_idx], f_p = pvv[f_idx];
  // uniform over the problem's CTAs: pcg_active only changes in the camera
  // kernel
  if (!pcg_live(L)) return;
  const int k = L->pcg_iterations;
  const double beta = L->beta;
  // stage p_k of the chunk's cameras: the FP64 form evaluates exactly the
  // camera kernel's expression; the mixed form the same recurrence in FP32
  // on the FP32 copies (its mat-vec input is FP32 anyway)
  for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
    const int sg = i / 9, q = i - 9 * sg;
    real z = f_z, po = f_p;
    if (i != t) {
      const size_t idx = 9 * (size_t)B.seg_cam[ci.seg_begin + sg] + q;
      z = zv[idx], po = pvv[idx];
    }
    if (MIXED)
      sm.pseg[sg][q] = k == 0 ? z : (real)__fmaf_rn((float)beta, (float)po, (float)z);
    else
      sm.pseg[sg][q] = (real)pcg_direction(k, beta, (double)z, k == 0 ? 0.0 : (double)po);
  }
  __syncthreads();
  if (valid) {
    real zu = 0, zv = 0;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const real x = sm.pseg[s][q];
      zu = mad(Jc[q].x, x, zu);
      zv = mad(Jc[q].y, x, zv);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) sm.U[t][q] = mad(Jp[q].x, zu, mul(Jp[q].y, zv));
  }
  __syncthreads();
  if (t < ci.pt_count) {
    Acc y0, y1, y2;
    y0.init(), y1.init(), y2.init();
    for (int kk = pb0; kk < pb1; ++kk) {
      y0.add(sm.U[kk][0]);
      y1.add(sm.U[kk][1]);
      y2.add(sm.U[kk][2]);
    }
    const real w0 = (real)y0.rvalue(), w1 = (real)y1.rvalue(), w2 = (real)y2.rvalue();
    sm.tpt[t][0] = mad(ci6[0], w0, mad(ci6[1], w1, mul(ci6[2], w2)));
    sm.tpt[t][1] = mad(ci6[1], w0, mad(ci6[3], w1, mul(ci6[4], w2)));
    sm.tpt[t][2] = mad(ci6[2], w0, mad(ci6[4], w1, mul(ci6[5], w2)));
  }
  __syncthreads();
  if (valid) {
    const real t0 = sm.tpt[lp][0], t1 = sm.tpt[lp][1], t2 = sm.tpt[lp][2];
    const real eu = mad(Jp[0].x, t0, mad(Jp[1].x, t1, mul(Jp[2].x, t2)));
    const real ev = mad(Jp[0].y, t0, mad(Jp[1].y, t1, mul(Jp[2].y, t2)));
#pragma unroll
    for (int q = 0; q < 9; ++q) sm.U[slot][q] = mad(Jc[q].x, eu, mul(Jc[q].y, ev));
  }
  __syncthreads();
  real *part = reinterpret_cast<real *>(B.seg_partial);
  // this thread's share of p.q: FP64 in the FP64 form, double-float in the
  // mixed form (FP32 instructions, converted once per CTA)
  double dot = 0.0;
  DF dotf = df_zero();
  for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
    const int sg = i / 9, q = i - 9 * sg;
    int b0 = f_b0, b1 = f_b1, slot9 = f_slot;
    bool owner = f_owner;
    if (i != t) {  // a chunk of more than kChunkCap / 9 segments: metadata now
      b0 = B.seg_pos[ci.seg_begin + sg];
      b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
      slot9 = B.seg_slot[ci.seg_begin + sg];
      const int cam = B.seg_cam[ci.seg_begin + sg];
      owner = slot9 == B.cam_seg_begin[cam];
      if (owner) a_row<MIXED>(B, cam, q, sm.arow[t]);  // the thread's own row, its earlier task done
    }
    Acc a;
    a.init();
    for (int kk = b0; kk < b1; ++kk) a.add(sm.U[kk][q]);
    const real pv = (real)a.rvalue();
    part[9 * (size_t)slot9 + q] = pv;
    const real *ps = sm.pseg[sg];
    if (MIXED) {
      dotf = df_add(dotf, df_prod(-(float)ps[q], (float)pv));
      if (owner) {  // the camera's (B + Dc^2) term
        const real *ar = sm.arow[t];
        float ap = __fmul_rn((float)ar[9], (float)ps[q]);
#pragma unroll
        for (int kk = 0; kk < 9; ++kk) ap = __fmaf_rn((float)ar[kk], (float)ps[kk], ap);
        dotf = df_add(dotf, df_prod((float)ps[q], ap));
      }
    } else {
      const double *p64 = reinterpret_cast<const double *>(ps);
      double d = -p64[q] * (double)pv;
      if (owner) d = fma(p64[q], a_times(sm.arow[t], p64, q), d);  // the camera's (B + Dc^2) term
      dot += d;
    }
  }
  chunk_value_store<MIXED>(B, ch, dot, dotf, dfred, red);
  if (pi.chunk_count <= kRedDirect) return;  // the camera kernel sums the chunk values itself
  // a large problem: the last CTA of each group of kRedGroup chunks sums the
  // group's values (fixed order); the camera kernel sums the group values
  const int rel = ch - pi.chunk_begin;
  const int g0 = pi.chunk_begin + (rel / kRedGroup) * kRedGroup;
  const int gn = min(kRedGroup, pi.chunk_begin + pi.chunk_count - g0);
  if (!last_block_done(B.chunk_counter + g0, (uint32_t)gn, &flag)) return;
  double gd = 0.0;
  DF gf = df_zero();
  if (t < gn) {
    if (MIXED)
      gf = chunk_value_load(B, g0 + t);
    else
      gd = __ldcg(B.chunk_red + g0 + t);
  }
  chunk_value_store<MIXED>(B, B.nchunks + g0, gd, gf, dfred, red);
}

// ---------------------------------------------------------------------------
// K4a, mixed form, lean: the same arithmetic as k_schur_matvec<true>, but
// the Jacobian is loaded after the wait (it stays in L2 between PCG
// iterations) and read again for the second product instead of being held
// in registers, so a thread needs few registers and up to kLeanCtas CTAs fit
// per SM, and a CTA whose problem's PCG has ended loads nothing at all
// (batches: the loop runs until the slowest problem's PCG ends).
constexpr int kLeanCtas = 8;

__global__ void __launch_bounds__(kChunkCap, kLeanCtas) k_schur_matvec_lean(DeviceBatch B) {
  __shared__ float pseg[kChunkCap][9];  // p of the chunk's cameras
  __shared__ float U[kChunkCap][9];     // first holds w (3 per obs), then u (9 per slot)
  __shared__ float tpt[kChunkCap][3];
  __shared__ double red[kChunkCap / 32];
  __shared__ DF dfred[kChunkCap / 32];
  __shared__ int flag;
  const int t = threadIdx.x;
  const int ch = blockIdx.x;
  const ChunkInfo ci = B.chunk[ch];
  const bool valid = t < ci.obs_count;
  // the first task's segment (fixed during the PCG)
  int f_b0 = 0, f_b1 = 0, f_slot = 0;
  size_t f_idx = 0;
  bool f_owner = false;
  if (t < ci.seg_count * 9) {
    const int sg = t / 9;
    f_b0 = B.seg_pos[ci.seg_begin + sg];
    f_b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
    f_slot = B.seg_slot[ci.seg_begin + sg];
    const int cam = B.seg_cam[ci.seg_begin + sg];
    f_idx = 9 * (size_t)cam + (t - 9 * sg);
    f_owner = f_slot == B.cam_seg_begin[cam];
  }
  pdl_wait();
  pdl_launch_dependents();
  const LMState *L = B.lm + ci.problem;
  float f_z = 0.f, f_p = 0.f;
  if (t < ci.seg_count * 9) f_z = B.pcg_zf[f_idx], f_p = B.pcg_pf[f_idx];
  if (!pcg_live(L)) return;  // uniform over the problem's CTAs
  const int k = L->pcg_iterations;
  const float beta = (float)L->beta;
  for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
    const int sg = i / 9, q = i - 9 * sg;
    float z = f_z, po = f_p;
    if (i != t) {
      const size_t idx = 9 * (size_t)B.seg_cam[ci.seg_begin + sg] + q;
      z = B.pcg_zf[idx], po = B.pcg_pf[idx];
    }
    pseg[sg][q] = k == 0 ? z : __fmaf_rn(beta, po, z);
  }
  const float2 *jac = reinterpret_cast<const float2 *>(B.jac);
  const size_t o = (size_t)ci.obs_begin + t;
  int slot = 0, lp = 0;
  __syncthreads();
  if (valid) {
    const int s = B.obs_seg[o];
    slot = B.obs_slot[o];
    lp = B.obs_pt[o] - ci.pt_begin;
    float zu = 0.f, zv = 0.f;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const float2 J = jac[(size_t)q * B.no + o];
      const float x = pseg[s][q];
      zu = mad(J.x, x, zu);
      zv = mad(J.y, x, zv);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float2 J = jac[(size_t)(9 + q) * B.no + o];
      U[t][q] = mad(J.x, zu, mul(J.y, zv));
    }
  }
  // the first task's (B + Dc^2) row, loaded now and used at the end
  float arow[10];
  if (f_owner) a_row<true>(B, (int)(f_idx / 9), (int)(f_idx % 9), arow);
  __syncthreads();
  if (t < ci.pt_count) {
    const int jj = ci.pt_begin + t;
    const int pb0 = B.pt_obs_begin[jj] - ci.obs_begin, pb1 = B.pt_obs_begin[jj + 1] - ci.obs_begin;
    const float *c6 = reinterpret_cast<const float *>(B.pt_Cinv) + 6 * (size_t)jj;
    KahanF y0, y1, y2;
    y0.init(), y1.init(), y2.init();
    for (int kk = pb0; kk < pb1; ++kk) {
      y0.add(U[kk][0]);
      y1.add(U[kk][1]);
      y2.add(U[kk][2]);
    }
    const float w0 = y0.rvalue(), w1 = y1.rvalue(), w2 = y2.rvalue();
    tpt[t][0] = mad(c6[0], w0, mad(c6[1], w1, mul(c6[2], w2)));
    tpt[t][1] = mad(c6[1], w0, mad(c6[3], w1, mul(c6[4], w2)));
    tpt[t][2] = mad(c6[2], w0, mad(c6[4], w1, mul(c6[5], w2)));
  }
  __syncthreads();
  if (valid) {
    const float t0 = tpt[lp][0], t1 = tpt[lp][1], t2 = tpt[lp][2];
    const float2 P0 = jac[(size_t)9 * B.no + o], P1 = jac[(size_t)10 * B.no + o], P2 = jac[(size_t)11 * B.no + o];
    const float eu = mad(P0.x, t0, mad(P1.x, t1, mul(P2.x, t2)));
    const float ev = mad(P0.y, t0, mad(P1.y, t1, mul(P2.y, t2)));
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const float2 J = jac[(size_t)q * B.no + o];
      U[slot][q] = mad(J.x, eu, mul(J.y, ev));
    }
  }
  __syncthreads();
  float *part = reinterpret_cast<float *>(B.seg_partial);
  DF dotf = df_zero();
  for (int i = t; i < ci.seg_count * 9; i += blockDim.x) {
    const int sg = i / 9, q = i - 9 * sg;
    int b0 = f_b0, b1 = f_b1, slot9 = f_slot;
    bool owner = f_owner;
    if (i != t) {  // a chunk of more than kChunkCap / 9 segments: metadata now
      b0 = B.seg_pos[ci.seg_begin + sg];
      b1 = (sg + 1 < ci.seg_count) ? B.seg_pos[ci.seg_begin + sg + 1] : ci.obs_count;
      slot9 = B.seg_slot[ci.seg_begin + sg];
      const int cam = B.seg_cam[ci.seg_begin + sg];
      owner = slot9 == B.cam_seg_begin[cam];
      if (owner) a_row<true>(B, cam, q, arow);
    }
    KahanF a;
    a.init();
    for (int kk = b0; kk < b1; ++kk) a.add(U[kk][q]);
    const float pv = a.rvalue();
    part[9 * (size_t)slot9 + q] = pv;
    const float *ps = pseg[sg];
    dotf = df_add(dotf, df_prod(-ps[q], pv));
    if (owner) {  // the camera's (B + Dc^2) term
      float ap = __fmul_rn(arow[9], ps[q]);
#pragma unroll
      for (int kk = 0; kk < 9; ++kk) ap = __fmaf_rn(arow[kk], ps[kk], ap);
      dotf = df_add(dotf, df_prod(ps[q], ap));
    }
  }
  chunk_value_store<true>(B, ch, 0.0, dotf, dfred, red);
  const ProblemInfo pi = B.prob[ci.problem];
  if (pi.chunk_count <= kRedDirect) return;  // the camera kernel sums the chunk values itself
  const int rel = ch - pi.chunk_begin;
  const int g0 = pi.chunk_begin + (rel / kRedGroup) * kRedGroup;
  const int gn = min(kRedGroup, pi.chunk_begin + pi.chunk_count - g0);
  if (!last_block_done(B.chunk_counter + g0, (uint32_t)gn, &flag)) return;
  DF gf = df_zero();
  if (t < gn) gf = chunk_value_load(B, g0 + t);
  chunk_value_store<true>(B, B.nchunks + g0, 0.0, gf, dfred, red);
}

// ---------------------------------------------------------------------------
// K4b: one CTA per camera block (kPcgBlockCams cameras of one problem).  Each
// camera coordinate has kPcgSub threads: sub-lane j sums the camera's
// partials j, j + kPcgSub, ... (so each thread has a fraction of the loads in
// flight), sub-lane 0 adds the kPcgSub sums in order and updates the
// coordinate.
constexpr int kPcgSub = 8;
constexpr int kPcgCoords = 9 * kPcgBlockCams;
constexpr int kPcgThreads = kPcgCoords * kPcgSub;
constexpr int kPcgWarps = kPcgThreads / 32;
static_assert(kPcgThreads % 32 == 0, "the block reductions combine whole warps");

// Two CTAs per SM (56 registers a thread, some spilled): a problem's camera
// blocks run in one wave instead of two on 1,800 cameras (20.1 instead of
// 22.7 us per PCG iteration; FP64 batches of configuration 3 +4.7 %).
template <bool MIXED>
__global__ void __launch_bounds__(kPcgThreads, 2) k_pcg_camera(DeviceBatch B) {
  typedef typename Prec<MIXED>::real real;
  typedef typename Acc<MIXED>::type Acc;
  __shared__ Acc psub[kPcgSub][kPcgCoords];  // sub-lane sums of the partials
  __shared__ double pv[kPcgCoords];          // p_k of the block, for (B + Dc^2) p
  __shared__ real rv[kPcgCoords];            // r_{k+1} of the block, for M r
  __shared__ double red[kPcgWarps];
  __shared__ DF dfred[kPcgWarps];
  __shared__ double red3[kPcgWarps][3];
  __shared__ double sc[2];
  __shared__ double chs[kPcgChunkSums];  // the explicit FP64 form's p.q chunk sums
  __shared__ int flag, sgood;
  constexpr int kLeadWarps = (kPcgCoords + 31) / 32;  // the warps holding sub-lane 0
  const int4 cb = B.camblk[blockIdx.x];  // (problem, first camera, count, 0)
  const int prob = cb.x;
  const int t = threadIdx.x, sub = t / kPcgCoords, m = t - kPcgCoords * sub;
  const int lc = m / 9, q = m - 9 * lc;
  const bool valid = lc < cb.z;
  const bool lead = valid && sub == 0;  // the thread that updates coordinate m
  const int c = cb.y + (valid ? lc : 0);
  const size_t i = 9 * (size_t)c + q;
  LMState *L = B.lm + prob;
  const ProblemInfo pi = B.prob[prob];
  // loads of what earlier kernels wrote (the previous camera-side kernel has
  // completed when this one starts; the problem state changes only in this
  // kernel's last block of the problem, after every block has read it)
  const bool live = pcg_live(L);
  const int k = L->pcg_iterations;
  const double beta = L->beta, rz_k = L->rz;
  double arow[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  real mrow[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double x = 0.0, r = 0.0, z = 0.0, p_old = 0.0, v = 0.0;
  // explicit Schur complement: q_k and the blocks' shares of p.q come from
  // the block-sparse product; no partials
  const bool ex = B.explicit_schur != 0;
  int s0 = 0, s1 = 0;
  if (valid && !ex) {
    s0 = B.cam_seg_begin[c];
    s1 = B.cam_seg_begin[c + 1];
  }
  if (lead) {
    real ar[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (!ex) a_row<MIXED>(B, c, q, ar);
#pragma unroll
    for (int kk = 0; kk < 10; ++kk) arow[kk] = (double)ar[kk];  // converted before the wait
    const real *M = reinterpret_cast<const real *>(MIXED ? (const void *)B.cam_Minvf : (const void *)B.cam_Minv) +
                    81 * (size_t)c + 9 * q;
#pragma unroll
    for (int kk = 0; kk < 9; ++kk) mrow[kk] = M[kk];
    x = B.pcg_x[i];
    r = B.pcg_r[i];
    z = B.pcg_z[i];
    v = B.pcg_v[i];
    p_old = B.pcg_p[i];  // used when k > 0
  }
  pdl_wait();  // the partials and the chunk values come from the mat-vec kernel
  double pq = 0.0, qex = 0.0;
  if (live) {
    if (ex && lead) qex = __ldcg(B.pcg_q + i);
    // p_k.q_k: the chunk values (or, for a large problem, the group values;
    // with the explicit complement the cameras' values) in a fixed order,
    // identical in every block of the problem
    const bool direct = pi.chunk_count <= kRedDirect;
    const int n = ex ? pi.cam_count : (direct ? pi.chunk_count : (pi.chunk_count + kRedGroup - 1) / kRedGroup);
    const double *cv = ex ? B.spmv_red + pi.cam_begin
                          : B.chunk_red + (direct ? pi.chunk_begin : B.nchunks + pi.chunk_begin);
    const int stride = (direct || ex) ? 1 : kRedGroup;
    // (the first kCv values per thread are loaded before the partials below,
    // so both sets of loads are in flight together); FP64 sums in the FP64
    // form and for the explicit complement's values, double-float for the
    // mixed form's chunk values
    const bool dfs = MIXED && !ex;
    constexpr int kCv = 4;
    double cvl[kCv];
    DF cvf[kCv];
#pragma unroll
    for (int j = 0; j < kCv; ++j) {
      const int e = t + j * kPcgThreads;
      cvl[j] = 0.0, cvf[j] = df_zero();
      if (e < n) {
        if (dfs)
          cvf[j] = chunk_value_load(B, (size_t)(cv - B.chunk_red) + (size_t)e * stride);
        else
          cvl[j] = __ldcg(cv + (size_t)e * stride);
      }
    }
    double psm = 0.0;
    DF psf = df_zero();
    for (int e = t + kCv * kPcgThreads; e < n; e += kPcgThreads) {
      if (dfs)
        psf = df_add(psf, chunk_value_load(B, (size_t)(cv - B.chunk_red) + (size_t)e * stride));
      else
        psm += __ldcg(cv + (size_t)e * stride);
    }
    // this sub-lane's share of the camera's partials (fixed order)
    if (valid) {
      constexpr int kBatch = 16;
      const real *part = reinterpret_cast<const real *>(B.seg_partial) + q;
      Acc a;
      a.init();
      for (int sg = s0 + sub; sg < s1; sg += kBatch * kPcgSub) {
        real pp[kBatch];
#pragma unroll
        for (int uu = 0; uu < kBatch; ++uu) {
          const int e = sg + uu * kPcgSub;
          pp[uu] = e < s1 ? part[9 * (size_t)e] : (real)0;
        }
#pragma unroll
        for (int uu = 0; uu < kBatch; ++uu)
          if (sg + uu * kPcgSub < s1) a.add(pp[uu]);
      }
      psub[sub][m] = a;
    }
    // p.q over the CTA (fixed order); thread 0 forms alpha once.  The FP64
    // form with the explicit complement sums the cameras' values in chunks
    // of 32 and a pairwise tree (cta_chunked_sum: the grid PCG's order)
    if (ex && !MIXED) {
      cta_chunked_sum<true>(cv, n, chs);
      if (t == 0) {
        const double s2 = chs[0];
        sc[0] = s2;
        sc[1] = rz_k * recip_nr(s2);
        sgood = s2 > 0.0 && isfinite(s2);
      }
    } else if (dfs) {
#pragma unroll
      for (int j = 0; j < kCv; ++j) psf = df_add(psf, cvf[j]);
      psf = df_warp_sum(psf);
      if ((t & 31) == 0) dfred[t >> 5] = psf;
    } else {
#pragma unroll
      for (int j = 0; j < kCv; ++j) psm += cvl[j];
      psm = warp_sum(psm);
      if ((t & 31) == 0) red[t >> 5] = psm;
    }
    __syncthreads();  // also publishes psub
    if (t == 0 && !(ex && !MIXED)) {
      double s2 = 0.0;
      if (dfs) {
        DF sf = dfred[0];
        for (int w = 1; w < kPcgWarps; ++w) sf = df_add(sf, dfred[w]);
        s2 = df_value(sf);
      } else {
        for (int w = 0; w < kPcgWarps; ++w) s2 += red[w];
      }
      sc[0] = s2;
      sc[1] = rz_k * recip_nr(s2);
      sgood = s2 > 0.0 && isfinite(s2);
    }
    __syncthreads();
    pq = sc[0];
  }
  // pq > 0 and finite (else S is not positive definite along p_k), tested
  // once by thread 0: an FP64 comparison in every warp would queue on the
  // FP64 pipes
  const bool good = live && sgood != 0;
  if (live && good) {
    const double alpha = sc[1];
    double p = 0.0;
    if (lead) {
      p = pcg_direction(k, beta, z, p_old);
      pv[m] = p;
    }
    __syncthreads();
    double rz = 0.0, rr = 0.0, qx = 0.0;
    if (lead) {
      // the sub-lane sums in order (compensated in the mixed form)
      Acc comb = psub[0][m];
#pragma unroll
      for (int j = 1; j < kPcgSub; ++j) comb.merge(psub[j][m]);
      const double psum = comb.value();
      const double qv = ex ? qex : a_times(arow, pv + 9 * lc, q) - psum;
      x = fma(alpha, p, x);
      r = fma(-alpha, qv, r);
      rv[m] = (real)r;
    }
    __syncthreads();
    if (lead) {
      real u = 0;
#pragma unroll
      for (int kk = 0; kk < 9; ++kk) u += mrow[kk] * rv[9 * lc + kk];
      z = (double)u;
      B.pcg_p[i] = p;
      B.pcg_x[i] = x;
      B.pcg_r[i] = r;
      B.pcg_z[i] = z;
      if (MIXED) B.pcg_pf[i] = (float)p, B.pcg_zf[i] = (float)z;
      rz = r * z, rr = r * r, qx = x * (v + r);
    }
    // the block's r.z, r.r, x.(v + r): warp butterflies in the warps that
    // hold the coordinates, then those warps in order (one value per thread)
    if ((t >> 5) < kLeadWarps) {
      warp_sum3(rz, rr, qx);
      if ((t & 31) == 0) red3[t >> 5][0] = rz, red3[t >> 5][1] = rr, red3[t >> 5][2] = qx;
    }
    __syncthreads();
    if (t < 3) {
      double b = 0.0;
      for (int w = 0; w < kLeadWarps; ++w) b += red3[w][t];
      B.blk_red[3 * (size_t)blockIdx.x + t] = b;
    }
  }
  // the next mat-vec may launch now: its early loads (the Jacobian, some 100
  // bytes per observation) would otherwise queue in front of this kernel's
  // latency-bound loads and stores above
  pdl_launch_dependents();
  if (live && last_block_done(B.prob_counter + 4 * prob + kPC_UPDATE, (uint32_t)pi.cam_block_count, &flag)) {
    // the blocks' values in block order: strided over the lanes of warp 0,
    // then a butterfly (an order fixed by the block count)
    if (t < 32) {
      double a3[3] = {0.0, 0.0, 0.0};
      if (good) {
        for (int b = t; b < pi.cam_block_count; b += 32) {
          const double *bv = B.blk_red + 3 * (size_t)(pi.cam_block_begin + b);
          a3[0] += __ldcg(bv), a3[1] += __ldcg(bv + 1), a3[2] += __ldcg(bv + 2);
        }
        warp_sum3(a3[0], a3[1], a3[2]);
      }
      if (t == 0) {
        // the stopping test on (x_{k+1}, r_{k+1}) and beta_{k+1}, without
        // FP64 division or square root (long sequences on GB300's FP64 pipe)
        const double rz1 = a3[0], rr1 = a3[1], qk = -a3[2];  // Q(x) = x'Sx - 2 v'x = -x.(v + r)
        const DeviceOptions &o = B.opt;
        const int k1 = k + 1;  // completed iterations
        bool stop = !good;     // no update: the PCG ends with x_k (a failed solve if k = 0)
        if (good) {
          if (o.pcg_criterion == GBA_PCG_QUADRATIC_MODEL) {
            // zeta = k1 (Q_k1 - Q_k) / Q_k1 < eta, multiplied through by Q_k1
            const double lhs = k1 * (qk - L->q0), rhs = o.eta * qk;
            const bool below = qk > 0.0 ? lhs < rhs : (qk < 0.0 ? lhs > rhs : L->q0 > 0.0);
            if (below && k1 >= o.min_pcg_iterations) stop = true;
          } else {
            const double lim = o.pcg_tolerance * L->r0_norm;  // |r| <= tol |r_0|
            if (rr1 <= lim * lim && k1 >= o.min_pcg_iterations) stop = true;
          }
          if (k1 >= o.max_pcg_iterations) stop = true;
          if (!(rz1 != 0.0 && isfinite(rz1))) stop = true;
          L->pcg_iterations = k1;
          L->beta = rz1 * recip_nr(rz_k);
          L->rz = rz1;
          L->rr = rr1;
          L->q0 = qk;
          L->pq = pq;
        } else if (k == 0) {
          L->linear_ok = 0;  // S not positive definite along the first direction
        }
        if (stop) {
          L->pcg_active = 0;
          atomicSub(B.status + 3, 1);
        }
        if (B.num_problems == 1) {
          // the only problem decides the loop: no grid-wide count needed
          B.status[2] = stop ? 0 : 1;
          if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, stop ? 0u : 1u);
        }
      }
    }
  } else if (!live && B.num_problems == 1 && blockIdx.x == 0 && t == 0) {
    B.status[2] = 0;
    if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, 0u);
  }
  if (B.num_problems == 1) return;
  // several problems: the grid's last CTA sets the PCG loop condition from
  // the count of problems whose PCG is still running
  if (last_block_done(B.global_counter + kGC_UPDATE, gridDim.x, &flag)) {
    if (t == 0) {
      const int any = __ldcg(B.status + 3) > 0 ? 1 : 0;
      B.status[2] = any;
      if (B.use_cond && B.pcg_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)B.pcg_cond, any ? 1u : 0u);
    }
  }
}

// ---------------------------------------------------------------------------
// pdl: launch as a programmatic dependent of the preceding kernel of the
// stream (which must be the other PCG kernel).
cudaError_t launch_schur_matvec(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl) {
  if (b.nchunks == 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)b.nchunks);
  cfg.blockDim = dim3(kChunkCap);
  cfg.dynamicSmemBytes = (mixed && b.num_problems > 1) ? 0 : (mixed ? sizeof(MatvecSmem<true>) : sizeof(MatvecSmem<false>));
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  // mixed form: a batch runs the lean kernel (chunks of problems whose PCG
  // has ended cost it nothing; the other kernel loads their Jacobian before
  // it can see that), a single problem the register-prefetching one; both
  // compute bitwise the same values
  if (b.explicit_schur) return launch_schur_spmv(b, mixed, s, pdl);
  if (mixed && b.num_problems > 1) return cudaLaunchKernelEx(&cfg, k_schur_matvec_lean, b);
  if (mixed) return cudaLaunchKernelEx(&cfg, k_schur_matvec<true>, b);
  return cudaLaunchKernelEx(&cfg, k_schur_matvec<false>, b);
}

cudaError_t launch_pcg_camera(const DeviceBatch &b, bool mixed, cudaStream_t s, bool pdl) {
  if (b.cam_blocks == 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)b.cam_blocks);
  cfg.blockDim = dim3(kPcgThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  if (mixed) return cudaLaunchKernelEx(&cfg, k_pcg_camera<true>, b);
  return cudaLaunchKernelEx(&cfg, k_pcg_camera<false>, b);
}

void launch_pcg_iteration(const DeviceBatch &b, bool mixed, cudaStream_t s) {
  launch_schur_matvec(b, mixed, s, false);
  launch_pcg_camera(b, mixed, s, false);
}

// Dynamic shared memory of the mat-vec kernel (above the 48 KB static limit).
void pcg_init() {
  cudaFuncSetAttribute(k_schur_matvec<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MatvecSmem<true>));
  cudaFuncSetAttribute(k_schur_matvec<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MatvecSmem<false>));
}

}  // namespace gba
