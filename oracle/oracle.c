/*
 * oracle.c — CPU oracle for the bundle-adjustment hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the reference the GPU solver is compared against
 * (tests/, __graft_entry__.smoke(), bench.py's CPU-baseline leg).  Never
 * linked into libgba.  See oracle.h for what it restates and where from.
 *
 * Plain C11 + OpenMP.  Every reduction runs in a fixed order, so results do
 * not depend on the thread count.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ======================================================================== */
/* Forward-mode dual numbers: value + derivative w.r.t. the 12 parameters of */
/* one residual block (9 camera, 3 point), the role Ceres' Jet<double,12>    */
/* plays for AutoDiffCostFunction<...,2,9,3> (SnavelyReprojectionError.h:89). */
/* ======================================================================== */
#define NJ 12
typedef struct {
  double a;
  double v[NJ];
} jet;

static inline jet jc(double a) {
  jet r;
  r.a = a;
  for (int k = 0; k < NJ; ++k) r.v[k] = 0.0;
  return r;
}
static inline jet jvar(double a, int idx) {
  jet r = jc(a);
  r.v[idx] = 1.0;
  return r;
}
static inline jet jadd(jet x, jet y) {
  jet r;
  r.a = x.a + y.a;
  for (int k = 0; k < NJ; ++k) r.v[k] = x.v[k] + y.v[k];
  return r;
}
static inline jet jsub(jet x, jet y) {
  jet r;
  r.a = x.a - y.a;
  for (int k = 0; k < NJ; ++k) r.v[k] = x.v[k] - y.v[k];
  return r;
}
static inline jet jneg(jet x) {
  jet r;
  r.a = -x.a;
  for (int k = 0; k < NJ; ++k) r.v[k] = -x.v[k];
  return r;
}
static inline jet jmul(jet x, jet y) {
  jet r;
  r.a = x.a * y.a;
  for (int k = 0; k < NJ; ++k) r.v[k] = x.a * y.v[k] + x.v[k] * y.a;
  return r;
}
/* quotient rule: d(x/y) = (dx - (x/y) dy) / y */
static inline jet jdiv(jet x, jet y) {
  jet r;
  const double q = x.a / y.a;
  r.a = q;
  for (int k = 0; k < NJ; ++k) r.v[k] = (x.v[k] - q * y.v[k]) / y.a;
  return r;
}
/* s / y for a constant s */
static inline jet jsdiv(double s, jet y) {
  jet r;
  r.a = s / y.a;
  const double f = -s / (y.a * y.a);
  for (int k = 0; k < NJ; ++k) r.v[k] = y.v[k] * f;
  return r;
}
static inline jet jsqrt(jet x) {
  jet r;
  const double s = sqrt(x.a);
  r.a = s;
  const double f = 1.0 / (2.0 * s);
  for (int k = 0; k < NJ; ++k) r.v[k] = x.v[k] * f;
  return r;
}
static inline jet jcos(jet x) {
  jet r;
  r.a = cos(x.a);
  const double f = -sin(x.a);
  for (int k = 0; k < NJ; ++k) r.v[k] = f * x.v[k];
  return r;
}
static inline jet jsin(jet x) {
  jet r;
  r.a = sin(x.a);
  const double f = cos(x.a);
  for (int k = 0; k < NJ; ++k) r.v[k] = f * x.v[k];
  return r;
}

/* ======================================================================== */
/* Rodrigues rotation (utils/geometry/rotation.h:133-199), double and jet.  */
/* Same branch: full formula when theta^2 > DBL_EPSILON, else pt + w x pt.   */
/* Dot products sum left to right (rotation.h:57-60), cross products as     */
/* rotation.h:62-67.                                                          */
/* ======================================================================== */
void orc_angle_axis_rotate_point(const double aa[3], const double pt[3], double out[3]) {
  const double theta2 = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
  if (theta2 > DBL_EPSILON) {
    const double theta = sqrt(theta2);
    const double c = cos(theta);
    const double s = sin(theta);
    const double inv = 1.0 / theta;
    const double w[3] = {aa[0] * inv, aa[1] * inv, aa[2] * inv};
    const double wx[3] = {w[1] * pt[2] - w[2] * pt[1], w[2] * pt[0] - w[0] * pt[2],
                          w[0] * pt[1] - w[1] * pt[0]};
    const double tmp = (w[0] * pt[0] + w[1] * pt[1] + w[2] * pt[2]) * (1.0 - c);
    for (int i = 0; i < 3; ++i) out[i] = pt[i] * c + wx[i] * s + w[i] * tmp;
  } else {
    const double wx[3] = {aa[1] * pt[2] - aa[2] * pt[1], aa[2] * pt[0] - aa[0] * pt[2],
                          aa[0] * pt[1] - aa[1] * pt[0]};
    for (int i = 0; i < 3; ++i) out[i] = pt[i] + wx[i];
  }
}

static void rotate_jet(const jet aa[3], const jet pt[3], jet out[3]) {
  const jet theta2 = jadd(jadd(jmul(aa[0], aa[0]), jmul(aa[1], aa[1])), jmul(aa[2], aa[2]));
  if (theta2.a > DBL_EPSILON) {
    const jet theta = jsqrt(theta2);
    const jet c = jcos(theta);
    const jet s = jsin(theta);
    const jet inv = jsdiv(1.0, theta);
    const jet w[3] = {jmul(aa[0], inv), jmul(aa[1], inv), jmul(aa[2], inv)};
    const jet wx[3] = {jsub(jmul(w[1], pt[2]), jmul(w[2], pt[1])),
                       jsub(jmul(w[2], pt[0]), jmul(w[0], pt[2])),
                       jsub(jmul(w[0], pt[1]), jmul(w[1], pt[0]))};
    const jet dotwp = jadd(jadd(jmul(w[0], pt[0]), jmul(w[1], pt[1])), jmul(w[2], pt[2]));
    const jet tmp = jmul(dotwp, jsub(jc(1.0), c));
    for (int i = 0; i < 3; ++i) out[i] = jadd(jadd(jmul(pt[i], c), jmul(wx[i], s)), jmul(w[i], tmp));
  } else {
    const jet wx[3] = {jsub(jmul(aa[1], pt[2]), jmul(aa[2], pt[1])),
                       jsub(jmul(aa[2], pt[0]), jmul(aa[0], pt[2])),
                       jsub(jmul(aa[0], pt[1]), jmul(aa[1], pt[0]))};
    for (int i = 0; i < 3; ++i) out[i] = jadd(pt[i], wx[i]);
  }
}

/* ======================================================================== */
/* Snavely projection (SnavelyReprojectionError.h:61-87) and residual        */
/* (:42-53): p = R(w)X + t; x' = -p/p_z; d = 1 + r2 (k1 + k2 r2);            */
/* prediction = f * d * x'; residual = prediction - observed.               */
/* ======================================================================== */
static void project_double(const double *cam, const double *pt, double pred[2]) {
  double p[3];
  orc_angle_axis_rotate_point(cam, pt, p);
  p[0] += cam[3];
  p[1] += cam[4];
  p[2] += cam[5];
  const double xp = -p[0] / p[2];
  const double yp = -p[1] / p[2];
  const double l1 = cam[7], l2 = cam[8];
  const double r2 = xp * xp + yp * yp;
  const double distortion = 1.0 + r2 * (l1 + l2 * r2);
  const double focal = cam[6];
  pred[0] = focal * distortion * xp;
  pred[1] = focal * distortion * yp;
}

/* The camera update of the g2o variant (VertexPoseAndIntrinsics::oplusImpl,
 * test_bundle_adjustment_g2o.cpp:84-90): R <- exp(dw) R, the other camera
 * parameters additive.  In angle-axis form w' = log(exp(dw) exp(w)),
 * composed through unit quaternions (q(w) = (cos |w|/2, sin(|w|/2) w/|w|),
 * q' = q(dw) q(w), w' = 2 atan2(|v'|, s') v'/|v'| with s' >= 0). */
static void aa_to_quat(const double w[3], double q[4]) {
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  if (th2 > 0.0) {
    const double th = sqrt(th2), h = 0.5 * th, sc = sin(h) / th;
    q[0] = cos(h), q[1] = w[0] * sc, q[2] = w[1] * sc, q[3] = w[2] * sc;
  } else {
    q[0] = 1.0, q[1] = 0.5 * w[0], q[2] = 0.5 * w[1], q[3] = 0.5 * w[2];
  }
}

void orc_compose_left(const double dw[3], const double w[3], double out[3]) {
  double a[4], b[4], q[4];
  aa_to_quat(dw, a);
  aa_to_quat(w, b);
  q[0] = a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
  q[1] = a[0] * b[1] + b[0] * a[1] + (a[2] * b[3] - a[3] * b[2]);
  q[2] = a[0] * b[2] + b[0] * a[2] + (a[3] * b[1] - a[1] * b[3]);
  q[3] = a[0] * b[3] + b[0] * a[3] + (a[1] * b[2] - a[2] * b[1]);
  if (q[0] < 0.0) q[0] = -q[0], q[1] = -q[1], q[2] = -q[2], q[3] = -q[3];
  const double s2 = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (s2 > 0.0) {
    const double sn = sqrt(s2), f = 2.0 * atan2(sn, q[0]) / sn;
    out[0] = q[1] * f, out[1] = q[2] * f, out[2] = q[3] * f;
  } else {
    out[0] = 0.0, out[1] = 0.0, out[2] = 0.0;
  }
}

/* Residual and Jacobian; so3_left: the rotation columns are derivatives
 * with respect to the left perturbation dw of exp(dw) R(w) at dw = 0 (the
 * jets rotate R(w) X by exp(dw) with dw = 0 + the unit parts: Rodrigues'
 * first-order branch, exact for the derivative). */
static int residual_jacobian_ex(const double cam[9], const double pt[3], const double uv[2], int so3_left,
                                double r[2], double J[24]) {
  jet c[9], X[3], p[3];
  for (int k = 0; k < 9; ++k) c[k] = jvar(cam[k], k);
  for (int k = 0; k < 3; ++k) X[k] = jvar(pt[k], 9 + k);
  if (so3_left) {
    jet w[3], dw[3], p1[3];
    for (int k = 0; k < 3; ++k) w[k] = jc(cam[k]), dw[k] = jvar(0.0, k);
    rotate_jet(w, X, p1);
    rotate_jet(dw, p1, p);
  } else {
    rotate_jet(c, X, p);
  }
  p[0] = jadd(p[0], c[3]);
  p[1] = jadd(p[1], c[4]);
  p[2] = jadd(p[2], c[5]);
  const jet xp = jdiv(jneg(p[0]), p[2]);
  const jet yp = jdiv(jneg(p[1]), p[2]);
  const jet r2 = jadd(jmul(xp, xp), jmul(yp, yp));
  const jet distortion = jadd(jc(1.0), jmul(r2, jadd(c[7], jmul(c[8], r2))));
  const jet fd = jmul(c[6], distortion);
  const jet pu = jmul(fd, xp);
  const jet pv = jmul(fd, yp);
  const jet ru = jsub(pu, jc(uv[0]));
  const jet rv = jsub(pv, jc(uv[1]));
  r[0] = ru.a;
  r[1] = rv.a;
  int ok = isfinite(r[0]) && isfinite(r[1]);
  for (int k = 0; k < NJ; ++k) {
    J[k] = ru.v[k];
    J[NJ + k] = rv.v[k];
    ok = ok && isfinite(J[k]) && isfinite(J[NJ + k]);
  }
  return ok;
}

int orc_residual_jacobian(const double cam[9], const double pt[3], const double uv[2],
                          double r[2], double J[24]) {
  return residual_jacobian_ex(cam, pt, uv, 0, r, J);
}

/* ======================================================================== */
/* Robust losses and the corrector, as Ceres documents them                  */
/* (LossFunction::Evaluate returns rho, rho', rho''; the residual-block      */
/* corrector rescales r and J so the Gauss-Newton model of 0.5*rho(|r|^2)    */
/* is the least-squares model of the corrected block).                      */
/* ======================================================================== */
static void loss_rho(int loss, double a, double s, double rho[3]) {
  if (loss == ORC_LOSS_HUBER) {
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
  } else if (loss == ORC_LOSS_CAUCHY) {
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

/* Applies the corrector to r (2) and J (2 x ncols, row stride ld). Returns
 * the block's cost 0.5*rho(s). */
static double correct_block(int loss, double a, double r[2], double *J, int ncols, int ld) {
  const double s = r[0] * r[0] + r[1] * r[1];
  if (loss == ORC_LOSS_TRIVIAL) return 0.5 * s;
  double rho[3];
  loss_rho(loss, a, s, rho);
  const double sqrt_rho1 = sqrt(rho[1]);
  double residual_scaling, alpha_sq_norm;
  if (s == 0.0 || rho[2] <= 0.0) {
    residual_scaling = sqrt_rho1;
    alpha_sq_norm = 0.0;
  } else {
    const double D = 1.0 + 2.0 * s * rho[2] / rho[1];
    const double alpha = 1.0 - sqrt(D);
    residual_scaling = sqrt_rho1 / (1.0 - alpha);
    alpha_sq_norm = alpha / s;
  }
  if (J) {
    for (int c = 0; c < ncols; ++c) {
      const double rJ = r[0] * J[c] + r[1] * J[ld + c];
      J[c] = sqrt_rho1 * (J[c] - alpha_sq_norm * r[0] * rJ);
      J[ld + c] = sqrt_rho1 * (J[ld + c] - alpha_sq_norm * r[1] * rJ);
    }
  }
  r[0] *= residual_scaling;
  r[1] *= residual_scaling;
  return 0.5 * rho[0];
}

static double block_cost(int loss, double a, const double r[2]) {
  const double s = r[0] * r[0] + r[1] * r[1];
  if (loss == ORC_LOSS_TRIVIAL) return 0.5 * s;
  double rho[3];
  loss_rho(loss, a, s, rho);
  return 0.5 * rho[0];
}

/* ======================================================================== */
/* Problem evaluation                                                        */
/* ======================================================================== */
#define SUM_BLOCK 1024

static void set_threads(const orc_options *o) {
#ifdef _OPENMP
  if (o && o->num_threads > 0) omp_set_num_threads(o->num_threads);
#else
  (void)o;
#endif
}

/* cost only at parameters x; returns 0 if any residual is non-finite */
/* ======================================================================== */
/* Rig model (local-BA window)                                              */
/* ======================================================================== */
static void aa_matrix(const double w[3], double R[9]) {
  for (int j = 0; j < 3; ++j) {
    const double e[3] = {j == 0, j == 1, j == 2};
    double c[3];
    orc_angle_axis_rotate_point(w, e, c);
    R[j] = c[0], R[3 + j] = c[1], R[6 + j] = c[2];
  }
}

static void mat_vec(const double R[9], const double x[3], double y[3]) {
  for (int i = 0; i < 3; ++i) y[i] = R[3 * i] * x[0] + R[3 * i + 1] * x[1] + R[3 * i + 2] * x[2];
}

/* pos_cam = E_k (T X): R_e (R X + t) + t_e */
static void rig_point(const double pose[9], const double pt[3], const orc_rig *rig, int cam, double R[9], double Re[9],
                      double Q[3]) {
  double P[3], RP[3];
  aa_matrix(pose, R);
  mat_vec(R, pt, P);
  for (int i = 0; i < 3; ++i) P[i] += pose[3 + i];
  aa_matrix(rig->ext[cam], Re);
  mat_vec(Re, P, RP);
  for (int i = 0; i < 3; ++i) Q[i] = RP[i] + rig->ext[cam][3 + i];
}

/* EdgeProjection::computeError (g2o_types.h:137-144): pixel = K pos_cam,
 * divided by its third entry; error = measurement - pixel. */
static void rig_residual(const double Q[3], const double uv[2], const orc_rig *rig, double r[2]) {
  const double pu = rig->fx * Q[0] + rig->cx * Q[2], pv = rig->fy * Q[1] + rig->cy * Q[2];
  r[0] = uv[0] - pu / Q[2];
  r[1] = uv[1] - pv / Q[2];
}

/* EdgeProjection::linearizeOplus (g2o_types.h:146-169), restated: with
 * (X, Y, Z) = pos_cam and zi = 1 / (Z + 1e-18), the pose columns (translation
 * first in the reference's order) are
 *   u: -fx zi, 0, fx X zi^2 | fx X Y zi^2, -fx - fx X^2 zi^2, fx Y zi
 *   v: 0, -fy zi, fy Y zi^2 | fy + fy Y^2 zi^2, -fy X Y zi^2, -fy X zi
 * (the derivative of a rotation applied in the rig camera's frame, as the
 * reference writes it), and the point columns are the translation columns
 * times R_e R.  Stored with the rotation columns in camera slots 0-2. */
int orc_rig_residual_jacobian(const double pose[9], const double pt[3], const double uv[2], const orc_rig *rig,
                              int cam, double r[2], double J[24]) {
  double R[9], Re[9], Q[3];
  rig_point(pose, pt, rig, cam, R, Re, Q);
  rig_residual(Q, uv, rig, r);
  const double fx = rig->fx, fy = rig->fy, X = Q[0], Y = Q[1], Z = Q[2];
  const double zi = 1.0 / (Z + 1e-18), zi2 = zi * zi;
  const double tu[3] = {-fx * zi, 0.0, fx * X * zi2}, tv[3] = {0.0, -fy * zi, fy * Y * zi2};
  const double ru_[3] = {fx * X * Y * zi2, -fx - fx * X * X * zi2, fx * Y * zi};
  const double rv_[3] = {fy + fy * Y * Y * zi2, -fy * X * Y * zi2, -fy * X * zi};
  double ReR[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ReR[3 * i + j] = Re[3 * i] * R[j] + Re[3 * i + 1] * R[3 + j] + Re[3 * i + 2] * R[6 + j];
  for (int k = 0; k < 3; ++k) {
    J[k] = ru_[k], J[12 + k] = rv_[k];
    J[3 + k] = tu[k], J[15 + k] = tv[k];
    J[6 + k] = 0.0, J[18 + k] = 0.0;
    J[9 + k] = tu[0] * ReR[k] + tu[1] * ReR[3 + k] + tu[2] * ReR[6 + k];
    J[21 + k] = tv[0] * ReR[k] + tv[1] * ReR[3 + k] + tv[2] * ReR[6 + k];
  }
  int ok = isfinite(r[0]) && isfinite(r[1]);
  for (int k = 0; k < 24; ++k) ok = ok && isfinite(J[k]);
  return ok;
}

/* exp(xi) on SE3 (Sophus convention, xi = (translation u, rotation w)):
 * rotation exp(w), translation V(w) u with V = I + (1 - cos t)/t^2 [w]x +
 * (t - sin t)/t^3 [w]x^2, t = |w| (series 1/2 - t^2/24, 1/6 - t^2/120 for
 * t < 1e-4).  Composed on the left: R' = exp(w) R, t' = exp(w) t + V u. */
void orc_se3_compose_left(const double dw[3], const double du[3], const double pose[6], double out[6]) {
  const double th2 = dw[0] * dw[0] + dw[1] * dw[1] + dw[2] * dw[2], th = sqrt(th2);
  double a, b;
  if (th < 1e-4) {
    a = 0.5 - th2 / 24.0;
    b = 1.0 / 6.0 - th2 / 120.0;
  } else {
    a = (1.0 - cos(th)) / th2;
    b = (th - sin(th)) / (th2 * th);
  }
  double c1[3], c2[3], rt[3];
  c1[0] = dw[1] * du[2] - dw[2] * du[1];
  c1[1] = dw[2] * du[0] - dw[0] * du[2];
  c1[2] = dw[0] * du[1] - dw[1] * du[0];
  c2[0] = dw[1] * c1[2] - dw[2] * c1[1];
  c2[1] = dw[2] * c1[0] - dw[0] * c1[2];
  c2[2] = dw[0] * c1[1] - dw[1] * c1[0];
  orc_angle_axis_rotate_point(dw, pose + 3, rt);
  double w[3];
  orc_compose_left(dw, pose, w);
  for (int i = 0; i < 3; ++i) {
    out[i] = w[i];
    out[3 + i] = rt[i] + (du[i] + a * c1[i] + b * c2[i]);
  }
}

double orc_window_outliers(const double *chi2, int no, double threshold, int max_doublings, unsigned char *outlier,
                           int *num_inliers, int *num_outliers) {
  int in = 0, out = 0;
  for (int it = 0; it < max_doublings; ++it) {
    in = out = 0;
    for (int i = 0; i < no; ++i) chi2[i] > threshold ? ++out : ++in;
    if ((double)in / (double)(in + out) > 0.5) break;
    threshold *= 2.0;
  }
  if (max_doublings <= 0)
    for (int i = 0; i < no; ++i) chi2[i] > threshold ? ++out : ++in;
  for (int i = 0; i < no; ++i)
    if (outlier) outlier[i] = chi2[i] > threshold;
  if (num_inliers) *num_inliers = in;
  if (num_outliers) *num_outliers = out;
  return threshold;
}

/* one observation under the problem's camera model */
typedef struct obs_model {
  int so3_left;
  const orc_rig *rig;
} obs_model;

static int observation_rj(const obs_model *m, const double *cam, const double *pt, const double *uv, int i,
                          double r[2], double J[24]) {
  if (m->rig) return orc_rig_residual_jacobian(cam, pt, uv, m->rig, m->rig->obs_camera[i], r, J);
  return residual_jacobian_ex(cam, pt, uv, m->so3_left, r, J);
}

static void observation_r(const obs_model *m, const double *cam, const double *pt, const double *uv, int i,
                          double r[2]) {
  if (m->rig) {
    double R[9], Re[9], Q[3];
    rig_point(cam, pt, m->rig, m->rig->obs_camera[i], R, Re, Q);
    rig_residual(Q, uv, m->rig, r);
    return;
  }
  double pred[2];
  project_double(cam, pt, pred);
  r[0] = pred[0] - uv[0];
  r[1] = pred[1] - uv[1];
}

static int eval_cost(const orc_problem *p, const obs_model *m, const double *x, int loss, double a, double *cost) {
  const int no = p->no, nb = (no + SUM_BLOCK - 1) / SUM_BLOCK;
  double *part = (double *)calloc((size_t)nb + 1, sizeof(double));
  int ok = 1;
  const double *pts = x + 9 * (size_t)p->nc;
#pragma omp parallel for schedule(static) reduction(&& : ok)
  for (int b = 0; b < nb; ++b) {
    double acc = 0.0;
    const int e = (b + 1) * SUM_BLOCK < no ? (b + 1) * SUM_BLOCK : no;
    for (int i = b * SUM_BLOCK; i < e; ++i) {
      double r[2];
      observation_r(m, x + 9 * (size_t)p->camera_index[i], pts + 3 * (size_t)p->point_index[i],
                    p->observations + 2 * i, i, r);
      if (!(isfinite(r[0]) && isfinite(r[1]))) ok = 0;
      acc += block_cost(loss, a, r);
    }
    part[b] = acc;
  }
  double c = 0.0;
  for (int b = 0; b < nb; ++b) c += part[b];
  free(part);
  *cost = c;
  return ok && isfinite(c);
}

/* residuals r (2*no) and Jacobians J (24*no), corrected for the loss; cost */
static int eval_jacobian(const orc_problem *p, const obs_model *m, const double *x, int loss, double a, double *r,
                         double *J, double *cost) {
  const int no = p->no, nb = (no + SUM_BLOCK - 1) / SUM_BLOCK;
  double *part = (double *)calloc((size_t)nb + 1, sizeof(double));
  int ok = 1;
  const double *pts = x + 9 * (size_t)p->nc;
#pragma omp parallel for schedule(static) reduction(&& : ok)
  for (int b = 0; b < nb; ++b) {
    double acc = 0.0;
    const int e = (b + 1) * SUM_BLOCK < no ? (b + 1) * SUM_BLOCK : no;
    for (int i = b * SUM_BLOCK; i < e; ++i) {
      double *ri = r + 2 * (size_t)i, *Ji = J + 24 * (size_t)i;
      if (!observation_rj(m, x + 9 * (size_t)p->camera_index[i], pts + 3 * (size_t)p->point_index[i],
                          p->observations + 2 * i, i, ri, Ji))
        ok = 0;
      acc += correct_block(loss, a, ri, Ji, 12, 12);
    }
    part[b] = acc;
  }
  double c = 0.0;
  for (int b = 0; b < nb; ++b) c += part[b];
  free(part);
  *cost = c;
  return ok && isfinite(c);
}

static int evaluate_model(const orc_problem *p, const obs_model *m, int loss, double loss_scale, double *residuals,
                          double *jacobians, double *cost) {
  const int no = p->no;
  double *r = residuals ? residuals : (double *)malloc(sizeof(double) * 2 * (size_t)no);
  double *J = jacobians ? jacobians : (double *)malloc(sizeof(double) * 24 * (size_t)no);
  int ok = 1;
  const double *pts = p->parameters + 9 * (size_t)p->nc;
  for (int i = 0; i < no; ++i)
    ok &= observation_rj(m, p->parameters + 9 * (size_t)p->camera_index[i], pts + 3 * (size_t)p->point_index[i],
                         p->observations + 2 * i, i, r + 2 * (size_t)i, J + 24 * (size_t)i);
  double c = 0.0;
  if (cost) {
    /* same blocked order as eval_cost */
    const int nb = (no + SUM_BLOCK - 1) / SUM_BLOCK;
    for (int b = 0; b < nb; ++b) {
      double acc = 0.0;
      const int e = (b + 1) * SUM_BLOCK < no ? (b + 1) * SUM_BLOCK : no;
      for (int i = b * SUM_BLOCK; i < e; ++i) acc += block_cost(loss, loss_scale, r + 2 * (size_t)i);
      c += acc;
    }
    *cost = c;
  }
  if (!residuals) free(r);
  if (!jacobians) free(J);
  return ok;
}

int orc_evaluate_ex(const orc_problem *p, int loss, double loss_scale, int camera_update, double *residuals,
                    double *jacobians, double *cost) {
  const obs_model m = {camera_update == ORC_UPDATE_SO3_LEFT, NULL};
  return evaluate_model(p, &m, loss, loss_scale, residuals, jacobians, cost);
}

int orc_evaluate_rig(const orc_problem *p, const orc_rig *rig, int loss, double loss_scale, double *residuals,
                     double *jacobians, double *cost) {
  const obs_model m = {0, rig};
  return evaluate_model(p, &m, loss, loss_scale, residuals, jacobians, cost);
}

int orc_evaluate(const orc_problem *p, int loss, double loss_scale, double *residuals,
                 double *jacobians, double *cost) {
  return orc_evaluate_ex(p, loss, loss_scale, ORC_UPDATE_ADDITIVE, residuals, jacobians, cost);
}

/* ======================================================================== */
/* Problem structure: observations grouped by point and by camera            */
/* ======================================================================== */
typedef struct {
  int nc, np, no, n;
  int *pt_begin, *pt_obs; /* CSR: observations of each point, increasing index */
  int *cam_begin, *cam_obs;
  unsigned char *cam_used, *pt_used;
} structure;

static void build_structure(const orc_problem *p, structure *s) {
  s->nc = p->nc;
  s->np = p->np;
  s->no = p->no;
  s->n = 9 * p->nc + 3 * p->np;
  s->pt_begin = (int *)calloc((size_t)p->np + 1, sizeof(int));
  s->cam_begin = (int *)calloc((size_t)p->nc + 1, sizeof(int));
  s->pt_obs = (int *)malloc(sizeof(int) * ((size_t)p->no + 1));
  s->cam_obs = (int *)malloc(sizeof(int) * ((size_t)p->no + 1));
  s->cam_used = (unsigned char *)calloc((size_t)p->nc + 1, 1);
  s->pt_used = (unsigned char *)calloc((size_t)p->np + 1, 1);
  for (int i = 0; i < p->no; ++i) {
    s->pt_begin[p->point_index[i] + 1]++;
    s->cam_begin[p->camera_index[i] + 1]++;
    s->cam_used[p->camera_index[i]] = 1;
    s->pt_used[p->point_index[i]] = 1;
  }
  for (int j = 0; j < p->np; ++j) s->pt_begin[j + 1] += s->pt_begin[j];
  for (int c = 0; c < p->nc; ++c) s->cam_begin[c + 1] += s->cam_begin[c];
  int *fp = (int *)malloc(sizeof(int) * ((size_t)p->np + 1));
  int *fc = (int *)malloc(sizeof(int) * ((size_t)p->nc + 1));
  memcpy(fp, s->pt_begin, sizeof(int) * (size_t)p->np);
  memcpy(fc, s->cam_begin, sizeof(int) * (size_t)p->nc);
  for (int i = 0; i < p->no; ++i) {
    s->pt_obs[fp[p->point_index[i]]++] = i;
    s->cam_obs[fc[p->camera_index[i]]++] = i;
  }
  free(fp);
  free(fc);
}

static void free_structure(structure *s) {
  free(s->pt_begin);
  free(s->pt_obs);
  free(s->cam_begin);
  free(s->cam_obs);
  free(s->cam_used);
  free(s->pt_used);
}

/* squared column norms of J (24 per obs) into out[n], in observation order */
static void column_norms(const orc_problem *p, const structure *st, const double *J, double *out) {
  memset(out, 0, sizeof(double) * (size_t)st->n);
  /* cameras: per camera, its observations in increasing order */
#pragma omp parallel for schedule(static)
  for (int c = 0; c < st->nc; ++c) {
    double acc[9] = {0};
    for (int k = st->cam_begin[c]; k < st->cam_begin[c + 1]; ++k) {
      const double *Ji = J + 24 * (size_t)st->cam_obs[k];
      for (int q = 0; q < 9; ++q) acc[q] += Ji[q] * Ji[q] + Ji[12 + q] * Ji[12 + q];
    }
    for (int q = 0; q < 9; ++q) out[9 * (size_t)c + q] = acc[q];
  }
#pragma omp parallel for schedule(static)
  for (int j = 0; j < st->np; ++j) {
    double acc[3] = {0};
    for (int k = st->pt_begin[j]; k < st->pt_begin[j + 1]; ++k) {
      const double *Ji = J + 24 * (size_t)st->pt_obs[k];
      for (int q = 0; q < 3; ++q) acc[q] += Ji[9 + q] * Ji[9 + q] + Ji[21 + q] * Ji[21 + q];
    }
    for (int q = 0; q < 3; ++q) out[9 * (size_t)st->nc + 3 * (size_t)j + q] = acc[q];
  }
  (void)p;
}

/* gradient g = J^T r, per parameter block in fixed order */
static void gradient(const structure *st, const double *J, const double *r, double *g) {
#pragma omp parallel for schedule(static)
  for (int c = 0; c < st->nc; ++c) {
    double acc[9] = {0};
    for (int k = st->cam_begin[c]; k < st->cam_begin[c + 1]; ++k) {
      const int i = st->cam_obs[k];
      const double *Ji = J + 24 * (size_t)i, *ri = r + 2 * (size_t)i;
      for (int q = 0; q < 9; ++q) acc[q] += Ji[q] * ri[0] + Ji[12 + q] * ri[1];
    }
    for (int q = 0; q < 9; ++q) g[9 * (size_t)c + q] = acc[q];
  }
#pragma omp parallel for schedule(static)
  for (int j = 0; j < st->np; ++j) {
    double acc[3] = {0};
    for (int k = st->pt_begin[j]; k < st->pt_begin[j + 1]; ++k) {
      const int i = st->pt_obs[k];
      const double *Ji = J + 24 * (size_t)i, *ri = r + 2 * (size_t)i;
      for (int q = 0; q < 3; ++q) acc[q] += Ji[9 + q] * ri[0] + Ji[21 + q] * ri[1];
    }
    for (int q = 0; q < 3; ++q) g[9 * (size_t)st->nc + 3 * (size_t)j + q] = acc[q];
  }
}

static void scale_columns(const orc_problem *p, double *J, const double *scale) {
  const double *sp = scale + 9 * (size_t)p->nc;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < p->no; ++i) {
    double *Ji = J + 24 * (size_t)i;
    const double *sc = scale + 9 * (size_t)p->camera_index[i];
    const double *ss = sp + 3 * (size_t)p->point_index[i];
    for (int q = 0; q < 9; ++q) {
      Ji[q] *= sc[q];
      Ji[12 + q] *= sc[q];
    }
    for (int q = 0; q < 3; ++q) {
      Ji[9 + q] *= ss[q];
      Ji[21 + q] *= ss[q];
    }
  }
}

/* ======================================================================== */
/* Small dense helpers                                                       */
/* ======================================================================== */
/* inverse of a symmetric positive-definite n x n matrix via Cholesky;
 * returns 0 when not positive definite */
static int spd_inverse(const double *A, double *Ainv, int n) {
  double L[81], Y[81];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = A[i * n + j];
      for (int k = 0; k < j; ++k) s -= L[i * n + k] * L[j * n + k];
      if (i == j) {
        if (!(s > 0.0)) return 0;
        L[i * n + i] = sqrt(s);
      } else {
        L[i * n + j] = s / L[j * n + j];
      }
    }
  /* Y = L^{-1} (lower) */
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      if (i < j) {
        Y[i * n + j] = 0.0;
        continue;
      }
      double s = (i == j) ? 1.0 : 0.0;
      for (int k = j; k < i; ++k) s -= L[i * n + k] * Y[k * n + j];
      Y[i * n + j] = s / L[i * n + i];
    }
  /* Ainv = Y^T Y */
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      const int k0 = i > j ? i : j;
      for (int k = k0; k < n; ++k) s += Y[k * n + i] * Y[k * n + j];
      Ainv[i * n + j] = s;
    }
  return 1;
}

/* Lower Cholesky of a dense row-major n x n matrix in place (blocked,
 * right-looking), restricted to the matrix's envelope: first[i] is the first
 * non-zero column of row i of the lower triangle, and every entry left of it
 * stays zero through the factorisation (no fill outside the envelope).  The
 * work skipped is exactly the terms that are products with those zeros, in
 * an unchanged order for the rest, so the factor is bitwise the one of the
 * plain dense loops; a banded reduced camera matrix (a trajectory's cameras
 * see points with their neighbours) costs about n bw^2 / 2 instead of n^3 / 6.
 * This is the role the sparse Cholesky plays in SPARSE_SCHUR.  Returns 0 when
 * not positive definite. */
static void envelope(const double *A, int n, int *first) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const double *Ai = A + (size_t)i * n;
    int f = i;
    for (int k = 0; k < i; ++k)
      if (Ai[k] != 0.0) {
        f = k;
        break;
      }
    first[i] = f;
  }
}

static int chol_dense(double *A, int n, const int *first) {
  const int NB = 48;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int k1 = (k0 + NB < n) ? k0 + NB : n;
    for (int j = k0; j < k1; ++j) {
      double d = A[(size_t)j * n + j];
      for (int k = k0; k < j; ++k) d -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
      if (!(d > 0.0) || !isfinite(d)) return 0;
      d = sqrt(d);
      A[(size_t)j * n + j] = d;
      for (int i = j + 1; i < k1; ++i) {
        double t = A[(size_t)i * n + j];
        for (int k = k0; k < j; ++k) t -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
        A[(size_t)i * n + j] = t / d;
      }
    }
#pragma omp parallel for schedule(static)
    for (int i = k1; i < n; ++i) {
      if (first[i] >= k1) continue; /* row i is zero in columns k0..k1-1 */
      for (int j = k0; j < k1; ++j) {
        double t = A[(size_t)i * n + j];
        for (int k = k0; k < j; ++k) t -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
        A[(size_t)i * n + j] = t / A[(size_t)j * n + j];
      }
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = k1; i < n; ++i) {
      if (first[i] >= k1) continue;
      const double *Li = A + (size_t)i * n;
      for (int j = k1; j <= i; ++j) {
        if (first[j] >= k1) continue;
        const double *Lj = A + (size_t)j * n;
        double t = 0.0;
        for (int k = k0; k < k1; ++k) t += Li[k] * Lj[k];
        A[(size_t)i * n + j] -= t;
      }
    }
  }
  return 1;
}

static void chol_solve(const double *L, int n, const int *first, double *b) {
  for (int i = 0; i < n; ++i) {
    double t = b[i];
    const double *Li = L + (size_t)i * n;
    for (int k = first[i]; k < i; ++k) t -= Li[k] * b[k];
    b[i] = t / Li[i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double t = b[i];
    for (int k = i + 1; k < n; ++k)
      if (first[k] <= i) t -= L[(size_t)k * n + i] * b[k];
    b[i] = t / L[(size_t)i * n + i];
  }
}

/* ======================================================================== */
/* The LM linear system (J^T J + D^2) y = J^T r, points eliminated           */
/* ======================================================================== */
typedef struct {
  const orc_problem *p;
  const structure *st;
  const orc_options *o;
  const double *J, *r; /* scaled, corrected */
  const double *D;     /* LM diagonal, n */
  double *Cinv;        /* 9 per point */
  double *W;           /* 27 per obs: W = Jc^T Jp (9 x 3) */
  double *gp;          /* 3 per point */
  double *gc;          /* 9 per camera */
  double *B;           /* 81 per camera: Jc^T Jc + Dc^2 */
} lsys;

/* point blocks, camera blocks, W */
static int lsys_build(lsys *L) {
  const structure *st = L->st;
  const double *J = L->J, *r = L->r, *D = L->D;
  const int nc = st->nc;
  int ok = 1;
#pragma omp parallel for schedule(static) reduction(&& : ok)
  for (int j = 0; j < st->np; ++j) {
    double C[9] = {0}, g[3] = {0};
    for (int k = st->pt_begin[j]; k < st->pt_begin[j + 1]; ++k) {
      const int i = st->pt_obs[k];
      const double *Ji = J + 24 * (size_t)i, *ri = r + 2 * (size_t)i;
      for (int a = 0; a < 3; ++a) {
        g[a] += Ji[9 + a] * ri[0] + Ji[21 + a] * ri[1];
        for (int b = 0; b < 3; ++b) C[a * 3 + b] += Ji[9 + a] * Ji[9 + b] + Ji[21 + a] * Ji[21 + b];
      }
    }
    for (int a = 0; a < 3; ++a) {
      const double d = D[9 * (size_t)nc + 3 * (size_t)j + a];
      C[a * 3 + a] += d * d;
      L->gp[3 * (size_t)j + a] = g[a];
    }
    if (!spd_inverse(C, L->Cinv + 9 * (size_t)j, 3)) ok = 0;
  }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    double Bc[81] = {0}, g[9] = {0};
    for (int k = st->cam_begin[c]; k < st->cam_begin[c + 1]; ++k) {
      const int i = st->cam_obs[k];
      const double *Ji = J + 24 * (size_t)i, *ri = r + 2 * (size_t)i;
      for (int a = 0; a < 9; ++a) {
        g[a] += Ji[a] * ri[0] + Ji[12 + a] * ri[1];
        for (int b = 0; b < 9; ++b) Bc[a * 9 + b] += Ji[a] * Ji[b] + Ji[12 + a] * Ji[12 + b];
      }
    }
    for (int a = 0; a < 9; ++a) {
      const double d = D[9 * (size_t)c + a];
      Bc[a * 9 + a] += d * d;
    }
    memcpy(L->B + 81 * (size_t)c, Bc, sizeof Bc);
    memcpy(L->gc + 9 * (size_t)c, g, sizeof g);
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < st->no; ++i) {
    const double *Ji = J + 24 * (size_t)i;
    double *Wi = L->W + 27 * (size_t)i;
    for (int a = 0; a < 9; ++a)
      for (int b = 0; b < 3; ++b) Wi[a * 3 + b] = Ji[a] * Ji[9 + b] + Ji[12 + a] * Ji[21 + b];
  }
  return ok;
}

/* X = W_i Cinv_j  (9x3) */
static inline void w_cinv(const double *Wi, const double *Cj, double *X) {
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 3; ++b)
      X[a * 3 + b] = Wi[a * 3 + 0] * Cj[0 * 3 + b] + Wi[a * 3 + 1] * Cj[1 * 3 + b] +
                     Wi[a * 3 + 2] * Cj[2 * 3 + b];
}

/* reduced right-hand side v = gc - sum W Cinv gp (per camera, fixed order) */
static void reduced_rhs(const lsys *L, double *v) {
  const structure *st = L->st;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < st->nc; ++c) {
    double acc[9];
    for (int a = 0; a < 9; ++a) acc[a] = L->gc[9 * (size_t)c + a];
    for (int k = st->cam_begin[c]; k < st->cam_begin[c + 1]; ++k) {
      const int i = st->cam_obs[k], j = L->p->point_index[i];
      double X[27];
      w_cinv(L->W + 27 * (size_t)i, L->Cinv + 9 * (size_t)j, X);
      const double *g = L->gp + 3 * (size_t)j;
      for (int a = 0; a < 9; ++a) acc[a] -= X[a * 3] * g[0] + X[a * 3 + 1] * g[1] + X[a * 3 + 2] * g[2];
    }
    memcpy(v + 9 * (size_t)c, acc, sizeof acc);
  }
}

/* point back-substitution y_p = Cinv (gp - W^T y_c) */
static void back_substitute(const lsys *L, const double *yc, double *yp) {
  const structure *st = L->st;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < st->np; ++j) {
    double t[3];
    for (int a = 0; a < 3; ++a) t[a] = L->gp[3 * (size_t)j + a];
    for (int k = st->pt_begin[j]; k < st->pt_begin[j + 1]; ++k) {
      const int i = st->pt_obs[k];
      const double *Wi = L->W + 27 * (size_t)i, *x = yc + 9 * (size_t)L->p->camera_index[i];
      for (int b = 0; b < 3; ++b) {
        double s = 0.0;
        for (int a = 0; a < 9; ++a) s += Wi[a * 3 + b] * x[a];
        t[b] -= s;
      }
    }
    const double *C = L->Cinv + 9 * (size_t)j;
    for (int a = 0; a < 3; ++a) yp[3 * (size_t)j + a] = C[a * 3] * t[0] + C[a * 3 + 1] * t[1] + C[a * 3 + 2] * t[2];
  }
}

/* exact: dense reduced camera matrix, Cholesky */
static int solve_dense_schur(const lsys *L, double *y) {
  const structure *st = L->st;
  const int nc = st->nc, m = 9 * nc;
  double *S = (double *)calloc((size_t)m * m, sizeof(double));
  if (!S) return 0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int c1 = 0; c1 < nc; ++c1) {
    double *rowblk = S + (size_t)9 * c1 * m;
    for (int a = 0; a < 9; ++a)
      for (int b = 0; b < 9; ++b) rowblk[(size_t)a * m + 9 * c1 + b] = L->B[81 * (size_t)c1 + a * 9 + b];
    for (int k = st->cam_begin[c1]; k < st->cam_begin[c1 + 1]; ++k) {
      const int i1 = st->cam_obs[k], j = L->p->point_index[i1];
      double X[27];
      w_cinv(L->W + 27 * (size_t)i1, L->Cinv + 9 * (size_t)j, X);
      for (int q = st->pt_begin[j]; q < st->pt_begin[j + 1]; ++q) {
        const int i2 = st->pt_obs[q], c2 = L->p->camera_index[i2];
        if (c2 > c1) continue; /* lower triangle only */
        const double *W2 = L->W + 27 * (size_t)i2;
        for (int a = 0; a < 9; ++a)
          for (int b = 0; b < 9; ++b)
            rowblk[(size_t)a * m + 9 * c2 + b] -=
                X[a * 3] * W2[b * 3] + X[a * 3 + 1] * W2[b * 3 + 1] + X[a * 3 + 2] * W2[b * 3 + 2];
      }
    }
  }
  double *v = y; /* camera part of y first holds the rhs */
  reduced_rhs(L, v);
  int *first = (int *)malloc((size_t)m * sizeof(int));
  if (!first) {
    free(S);
    return 0;
  }
  envelope(S, m, first);
  const int ok = chol_dense(S, m, first);
  if (ok) {
    chol_solve(S, m, first, v);
    back_substitute(L, v, y + m);
  }
  free(first);
  free(S);
  return ok;
}

/* implicit Schur product q = S x */
static void schur_matvec(const lsys *L, const double *x, double *q, double *tp /*3*np*/) {
  const structure *st = L->st;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < st->np; ++j) {
    double y[3] = {0, 0, 0};
    for (int k = st->pt_begin[j]; k < st->pt_begin[j + 1]; ++k) {
      const int i = st->pt_obs[k];
      const double *Wi = L->W + 27 * (size_t)i, *xc = x + 9 * (size_t)L->p->camera_index[i];
      for (int b = 0; b < 3; ++b) {
        double s = 0.0;
        for (int a = 0; a < 9; ++a) s += Wi[a * 3 + b] * xc[a];
        y[b] += s;
      }
    }
    const double *C = L->Cinv + 9 * (size_t)j;
    for (int a = 0; a < 3; ++a) tp[3 * (size_t)j + a] = C[a * 3] * y[0] + C[a * 3 + 1] * y[1] + C[a * 3 + 2] * y[2];
  }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < st->nc; ++c) {
    double acc[9];
    const double *Bc = L->B + 81 * (size_t)c, *xc = x + 9 * (size_t)c;
    for (int a = 0; a < 9; ++a) {
      double s = 0.0;
      for (int b = 0; b < 9; ++b) s += Bc[a * 9 + b] * xc[b];
      acc[a] = s;
    }
    for (int k = st->cam_begin[c]; k < st->cam_begin[c + 1]; ++k) {
      const int i = st->cam_obs[k], j = L->p->point_index[i];
      const double *Wi = L->W + 27 * (size_t)i, *t = tp + 3 * (size_t)j;
      for (int a = 0; a < 9; ++a) acc[a] -= Wi[a * 3] * t[0] + Wi[a * 3 + 1] * t[1] + Wi[a * 3 + 2] * t[2];
    }
    memcpy(q + 9 * (size_t)c, acc, sizeof acc);
  }
}

static double dotv(const double *a, const double *b, int n) {
  /* fixed blocked order */
  double s = 0.0;
  for (int i0 = 0; i0 < n; i0 += 256) {
    double t = 0.0;
    const int e = i0 + 256 < n ? i0 + 256 : n;
    for (int i = i0; i < e; ++i) t += a[i] * b[i];
    s += t;
  }
  return s;
}

/* PCG on the reduced camera system with the block-Jacobi preconditioner */
static int solve_pcg_schur(const lsys *L, double *y, int *iters) {
  const structure *st = L->st;
  const int nc = st->nc, m = 9 * nc;
  double *Minv = (double *)malloc(sizeof(double) * 81 * (size_t)nc);
  double *v = (double *)malloc(sizeof(double) * (size_t)m);
  double *r = (double *)malloc(sizeof(double) * (size_t)m);
  double *z = (double *)malloc(sizeof(double) * (size_t)m);
  double *pv = (double *)malloc(sizeof(double) * (size_t)m);
  double *q = (double *)malloc(sizeof(double) * (size_t)m);
  double *tp = (double *)malloc(sizeof(double) * 3 * ((size_t)st->np + 1));
  int ok = 1;
  /* S_ii = B_i - sum_i W Cinv W^T */
#pragma omp parallel for schedule(static) reduction(&& : ok)
  for (int c = 0; c < nc; ++c) {
    double Sii[81];
    memcpy(Sii, L->B + 81 * (size_t)c, sizeof Sii);
    for (int k = st->cam_begin[c]; k < st->cam_begin[c + 1]; ++k) {
      const int i = st->cam_obs[k], j = L->p->point_index[i];
      double X[27];
      const double *Wi = L->W + 27 * (size_t)i;
      w_cinv(Wi, L->Cinv + 9 * (size_t)j, X);
      for (int a = 0; a < 9; ++a)
        for (int b = 0; b < 9; ++b)
          Sii[a * 9 + b] -= X[a * 3] * Wi[b * 3] + X[a * 3 + 1] * Wi[b * 3 + 1] + X[a * 3 + 2] * Wi[b * 3 + 2];
    }
    if (!spd_inverse(Sii, Minv + 81 * (size_t)c, 9)) ok = 0;
  }
  reduced_rhs(L, v);
  double *x = y;
  memset(x, 0, sizeof(double) * (size_t)m);
  int it = 0;
  if (ok) {
    memcpy(r, v, sizeof(double) * (size_t)m);
    const double norm_b = sqrt(dotv(v, v, m));
    if (norm_b > 0.0) {
      double rz = 0.0, Q0 = 0.0;
      for (int c = 0; c < nc; ++c)
        for (int a = 0; a < 9; ++a) {
          double s = 0.0;
          for (int b = 0; b < 9; ++b) s += Minv[81 * (size_t)c + a * 9 + b] * r[9 * (size_t)c + b];
          z[9 * (size_t)c + a] = s;
        }
      memcpy(pv, z, sizeof(double) * (size_t)m);
      rz = dotv(r, z, m);
      const int maxit = L->o->max_linear_solver_iterations;
      while (it < maxit) {
        schur_matvec(L, pv, q, tp);
        const double pq = dotv(pv, q, m);
        if (!(pq > 0.0) || !isfinite(pq)) {
          if (it == 0) ok = 0;
          break;
        }
        const double alpha = rz / pq;
        for (int k = 0; k < m; ++k) {
          x[k] += alpha * pv[k];
          r[k] -= alpha * q[k];
        }
        ++it;
        if (L->o->pcg_criterion == ORC_PCG_QUADRATIC_MODEL) {
          /* Q(x) = x'Sx - 2 v'x = -x'(v + r) */
          double Q1 = 0.0;
          for (int k = 0; k < m; ++k) Q1 -= x[k] * (v[k] + r[k]);
          const double zeta = it * (Q1 - Q0) / Q1;
          if (zeta < L->o->eta && it >= L->o->min_linear_solver_iterations) break;
          Q0 = Q1;
        } else {
          const double rn = sqrt(dotv(r, r, m));
          if (rn <= L->o->pcg_tolerance * norm_b && it >= L->o->min_linear_solver_iterations) break;
        }
        for (int c = 0; c < nc; ++c)
          for (int a = 0; a < 9; ++a) {
            double s = 0.0;
            for (int b = 0; b < 9; ++b) s += Minv[81 * (size_t)c + a * 9 + b] * r[9 * (size_t)c + b];
            z[9 * (size_t)c + a] = s;
          }
        const double rz_new = dotv(r, z, m);
        const double beta = rz_new / rz;
        rz = rz_new;
        for (int k = 0; k < m; ++k) pv[k] = z[k] + beta * pv[k];
      }
    }
    back_substitute(L, x, y + m);
  }
  *iters = it;
  free(Minv);
  free(v);
  free(r);
  free(z);
  free(pv);
  free(q);
  free(tp);
  return ok;
}

/* Solves (J^T J + D^2) y = J^T r; returns 0 on failure. */
static int linear_solve(const orc_problem *p, const structure *st, const orc_options *o,
                        const double *J, const double *r, const double *D, double *y, int *iters) {
  lsys L;
  L.p = p;
  L.st = st;
  L.o = o;
  L.J = J;
  L.r = r;
  L.D = D;
  L.Cinv = (double *)malloc(sizeof(double) * 9 * ((size_t)st->np + 1));
  L.W = (double *)malloc(sizeof(double) * 27 * ((size_t)st->no + 1));
  L.gp = (double *)malloc(sizeof(double) * 3 * ((size_t)st->np + 1));
  L.gc = (double *)malloc(sizeof(double) * 9 * ((size_t)st->nc + 1));
  L.B = (double *)malloc(sizeof(double) * 81 * ((size_t)st->nc + 1));
  int ok = lsys_build(&L);
  *iters = 0;
  if (ok) {
    if (o->linear_solver == ORC_SOLVER_PCG_SCHUR)
      ok = solve_pcg_schur(&L, y, iters);
    else
      ok = solve_dense_schur(&L, y);
  }
  for (int k = 0; ok && k < st->n; ++k)
    if (!isfinite(y[k])) ok = 0;
  free(L.Cinv);
  free(L.W);
  free(L.gp);
  free(L.gc);
  free(L.B);
  return ok;
}

/* model_cost_change = -m.(r + m/2), m = J step (scaled J, scaled step) */
static double model_cost_change(const orc_problem *p, const double *J, const double *r,
                                const double *step) {
  const int no = p->no, nb = (no + SUM_BLOCK - 1) / SUM_BLOCK;
  double *part = (double *)calloc((size_t)nb + 1, sizeof(double));
  const double *sp = step + 9 * (size_t)p->nc;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nb; ++b) {
    double acc = 0.0;
    const int e = (b + 1) * SUM_BLOCK < no ? (b + 1) * SUM_BLOCK : no;
    for (int i = b * SUM_BLOCK; i < e; ++i) {
      const double *Ji = J + 24 * (size_t)i, *ri = r + 2 * (size_t)i;
      const double *sc = step + 9 * (size_t)p->camera_index[i], *ss = sp + 3 * (size_t)p->point_index[i];
      double m0 = 0.0, m1 = 0.0;
      for (int q = 0; q < 9; ++q) {
        m0 += Ji[q] * sc[q];
        m1 += Ji[12 + q] * sc[q];
      }
      for (int q = 0; q < 3; ++q) {
        m0 += Ji[9 + q] * ss[q];
        m1 += Ji[21 + q] * ss[q];
      }
      acc += m0 * (ri[0] + m0 / 2.0) + m1 * (ri[1] + m1 / 2.0);
    }
    part[b] = acc;
  }
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += part[b];
  free(part);
  return -s;
}

/* norm over the parameter blocks that appear in some residual block */
static double used_norm(const structure *st, const double *x) {
  double s = 0.0;
  for (int c = 0; c < st->nc; ++c)
    if (st->cam_used[c])
      for (int q = 0; q < 9; ++q) s += x[9 * (size_t)c + q] * x[9 * (size_t)c + q];
  for (int j = 0; j < st->np; ++j)
    if (st->pt_used[j])
      for (int q = 0; q < 3; ++q) {
        const double v = x[9 * (size_t)st->nc + 3 * (size_t)j + q];
        s += v * v;
      }
  return sqrt(s);
}

static double used_diff_norm(const structure *st, const double *x, const double *y) {
  double s = 0.0;
  for (int c = 0; c < st->nc; ++c)
    if (st->cam_used[c])
      for (int q = 0; q < 9; ++q) {
        const double d = x[9 * (size_t)c + q] - y[9 * (size_t)c + q];
        s += d * d;
      }
  for (int j = 0; j < st->np; ++j)
    if (st->pt_used[j])
      for (int q = 0; q < 3; ++q) {
        const size_t k = 9 * (size_t)st->nc + 3 * (size_t)j + q;
        const double d = x[k] - y[k];
        s += d * d;
      }
  return sqrt(s);
}

/* |x - (x - g)|_inf over used blocks */
static double gradient_max_norm(const structure *st, const double *x, const double *g) {
  double m = 0.0;
  for (int c = 0; c < st->nc; ++c)
    if (st->cam_used[c])
      for (int q = 0; q < 9; ++q) {
        const size_t k = 9 * (size_t)c + q;
        const double d = fabs(x[k] - (x[k] - g[k]));
        if (d > m) m = d;
      }
  for (int j = 0; j < st->np; ++j)
    if (st->pt_used[j])
      for (int q = 0; q < 3; ++q) {
        const size_t k = 9 * (size_t)st->nc + 3 * (size_t)j + q;
        const double d = fabs(x[k] - (x[k] - g[k]));
        if (d > m) m = d;
      }
  return m;
}

void orc_options_init(orc_options *o) {
  memset(o, 0, sizeof *o);
  o->max_num_iterations = 50;
  o->function_tolerance = 1e-6;
  o->gradient_tolerance = 1e-10;
  o->parameter_tolerance = 1e-8;
  o->initial_trust_region_radius = 1e4;
  o->max_trust_region_radius = 1e16;
  o->min_trust_region_radius = 1e-32;
  o->min_relative_decrease = 1e-3;
  o->min_lm_diagonal = 1e-6;
  o->max_lm_diagonal = 1e32;
  o->max_num_consecutive_invalid_steps = 5;
  o->jacobi_scaling = 1;
  o->loss = ORC_LOSS_TRIVIAL;
  o->loss_scale = 1.0;
  o->linear_solver = ORC_SOLVER_DENSE_SCHUR;
  o->pcg_criterion = ORC_PCG_RESIDUAL;
  o->max_linear_solver_iterations = 500;
  o->min_linear_solver_iterations = 0;
  o->pcg_tolerance = 1e-10;
  o->eta = 0.1;
  o->num_threads = 0;
  o->verbose = 0;
}

/* Jacobi scaling s_k = 1 / (1 + sqrt(|J_k|^2)), computed once at the first
 * Jacobian evaluation and kept for the rest of the solve. */
static void jacobi_scale(const structure *st, const double *colnorm2, int on, double *scale) {
  for (int k = 0; k < st->n; ++k) scale[k] = on ? 1.0 / (1.0 + sqrt(colnorm2[k])) : 1.0;
}

int orc_compute_step(const orc_problem *p, const orc_options *o, double radius, double *delta,
                     double *mcc_out, int *linear_iterations) {
  set_threads(o);
  const obs_model model = {o->camera_update == ORC_UPDATE_SO3_LEFT, o->rig};
  structure st;
  build_structure(p, &st);
  const int n = st.n;
  double *r = (double *)malloc(sizeof(double) * 2 * ((size_t)p->no + 1));
  double *J = (double *)malloc(sizeof(double) * 24 * ((size_t)p->no + 1));
  double *cn = (double *)malloc(sizeof(double) * (size_t)n);
  double *scale = (double *)malloc(sizeof(double) * (size_t)n);
  double *D = (double *)malloc(sizeof(double) * (size_t)n);
  double *y = (double *)malloc(sizeof(double) * (size_t)n);
  double cost;
  int ok = eval_jacobian(p, &model, p->parameters, o->loss, o->loss_scale, r, J, &cost);
  int it = 0;
  if (ok) {
    column_norms(p, &st, J, cn);
    jacobi_scale(&st, cn, o->jacobi_scaling, scale);
    scale_columns(p, J, scale);
    column_norms(p, &st, J, cn);
    for (int k = 0; k < n; ++k) {
      const double d = fmin(fmax(cn[k], o->min_lm_diagonal), o->max_lm_diagonal);
      D[k] = sqrt(d / radius);
    }
    ok = linear_solve(p, &st, o, J, r, D, y, &it);
    if (ok) {
      for (int k = 0; k < n; ++k) y[k] = -y[k];
      if (mcc_out) *mcc_out = model_cost_change(p, J, r, y);
      for (int k = 0; k < n; ++k) delta[k] = y[k] * scale[k];
    }
  }
  if (linear_iterations) *linear_iterations = it;
  free(r);
  free(J);
  free(cn);
  free(scale);
  free(D);
  free(y);
  free_structure(&st);
  return ok;
}

static void trace_put(orc_summary *s, int it, double cost, double radius, int lin, int succ) {
  if (!s || it >= s->trace_capacity) return;
  if (s->trace_cost) s->trace_cost[it] = cost;
  if (s->trace_radius) s->trace_radius[it] = radius;
  if (s->trace_linear_iterations) s->trace_linear_iterations[it] = lin;
  if (s->trace_successful) s->trace_successful[it] = succ;
  if (it + 1 > s->trace_length) s->trace_length = it + 1;
}

/* g2o's Levenberg policy (OptimizationAlgorithmLevenberg, g2o tag
 * 20230223_git, which test_bundle_adjustment_g2o.cpp:174-176 selects; the
 * library is cloned by build_thirdparty.sh:248-254 and absent here, so this
 * restates its published algorithm):
 *   damping H + lambda I on the unscaled normal equations (no Jacobi scaling);
 *   lambda_0 = tau * max diag(H) at the initial point, tau = 1e-5;
 *   gain rho = (chi2 - chi2_new) / (dx.(lambda dx + b) + 1e-3), chi2 = 2 cost,
 *     and dx.(lambda dx + b) = 2 * model_cost_change for the solved step;
 *   rho > 0: accept, lambda *= max(1/3, min(2/3, 1 - (2 rho - 1)^3)), nu = 2
 *     (Nielsen's update with the factor capped at 2/3);
 *   else: reject, lambda *= nu, nu *= 2;
 *   one outer iteration = trials until the first accepted step, at most 10;
 *   the solve stops when the 10th trial of an outer iteration has run, when a
 *   trial gives rho == 0 exactly, when lambda is no longer finite, or after
 *   max_num_iterations outer iterations.  lambda = 1 / radius below. */
#define ORC_G2O_TAU 1e-5
#define ORC_G2O_MAX_TRIALS 10

int orc_solve(const orc_problem *p, const orc_options *o, orc_summary *s) {
  set_threads(o);
  const obs_model model = {o->camera_update == ORC_UPDATE_SO3_LEFT, o->rig};
  const int g2o = o->lm_policy == ORC_LM_G2O;
  int trials = 0, outer = 0;
  structure st;
  build_structure(p, &st);
  const int n = st.n;
  const size_t no = (size_t)p->no;
  double *x = (double *)malloc(sizeof(double) * (size_t)n);
  double *xc = (double *)malloc(sizeof(double) * (size_t)n);
  double *r = (double *)malloc(sizeof(double) * 2 * (no + 1));
  double *J = (double *)malloc(sizeof(double) * 24 * (no + 1));
  double *g = (double *)malloc(sizeof(double) * (size_t)n);
  double *cn = (double *)malloc(sizeof(double) * (size_t)n);
  double *scale = (double *)malloc(sizeof(double) * (size_t)n);
  double *diag = (double *)malloc(sizeof(double) * (size_t)n);
  double *D = (double *)malloc(sizeof(double) * (size_t)n);
  double *y = (double *)malloc(sizeof(double) * (size_t)n);
  memcpy(x, p->parameters, sizeof(double) * (size_t)n);
  memcpy(xc, x, sizeof(double) * (size_t)n);

  orc_summary local;
  if (!s) {
    memset(&local, 0, sizeof local);
    s = &local;
  }
  s->num_iterations = s->num_successful_steps = s->num_unsuccessful_steps = s->num_invalid_steps = 0;
  s->num_linear_solver_iterations = 0;
  s->trace_length = 0;
  s->termination_reason = 0;

  double radius = o->initial_trust_region_radius, decrease_factor = 2.0;
  int reuse_diagonal = 0, invalid_run = 0, iteration = 0;
  double x_cost = 0.0, x_norm = used_norm(&st, x), gmax = 0.0;
  int term = -1, reason = 0;

  int ok = eval_jacobian(p, &model, x, o->loss, o->loss_scale, r, J, &x_cost);
  if (!ok) {
    term = 2;
    reason = 7;
    s->initial_cost = x_cost;
    goto done;
  }
  gradient(&st, J, r, g);
  gmax = gradient_max_norm(&st, x, g);
  column_norms(p, &st, J, cn);
  jacobi_scale(&st, cn, o->jacobi_scaling && !g2o, scale);
  scale_columns(p, J, scale);
  if (g2o) {
    double hmax = 0.0;
    for (int k = 0; k < n; ++k) hmax = fmax(hmax, cn[k]);
    radius = 1.0 / (ORC_G2O_TAU * hmax);
  }
  s->initial_cost = x_cost;
  double minimum_cost = x_cost;
  trace_put(s, 0, x_cost, radius, 0, 1);
  if (o->verbose)
    printf("iter      cost      cost_change  |gradient|   |step|    tr_ratio  tr_radius  ls_iter\n"
           "%4d %.6e %.2e %.2e %.2e %.2e %.2e %4d\n",
           0, x_cost, 0.0, gmax, 0.0, 0.0, radius, 0);
  if (o->max_num_iterations <= 0) {
    term = 1;
    reason = 1;
  } else if (g2o) {
  } else if (gmax <= o->gradient_tolerance) {
    term = 0;
    reason = 3;
  } else if (radius <= o->min_trust_region_radius) {
    term = 0;
    reason = 5;
  }

  while (term < 0) {
    ++iteration;
    if (!reuse_diagonal) {
      column_norms(p, &st, J, cn);
      for (int k = 0; k < n; ++k) diag[k] = g2o ? 1.0 : fmin(fmax(cn[k], o->min_lm_diagonal), o->max_lm_diagonal);
    }
    for (int k = 0; k < n; ++k) D[k] = sqrt(diag[k] / radius);
    int lin_it = 0;
    int lin_ok = linear_solve(p, &st, o, J, r, D, y, &lin_it);
    reuse_diagonal = 1;
    s->num_linear_solver_iterations += lin_it;
    double mcc = 0.0;
    int valid = 0;
    if (lin_ok) {
      for (int k = 0; k < n; ++k) y[k] = -y[k];
      mcc = model_cost_change(p, J, r, y);
      valid = mcc > 0.0;
    }
    int successful = 0;
    double iter_cost = x_cost, rho = -1.0;
    if (!valid) {
      ++s->num_invalid_steps;
      if (!g2o && ++invalid_run >= o->max_num_consecutive_invalid_steps) {
        term = 2;
        reason = 6;
        ++s->num_unsuccessful_steps;
        trace_put(s, iteration, x_cost, radius, lin_it, 0);
        break;
      }
      radius /= decrease_factor;
      decrease_factor *= 2.0;
      reuse_diagonal = 1;
    } else {
      invalid_run = 0;
      for (int c = 0; c < p->nc; ++c) {
        for (int q = 0; q < 9; ++q) {
          const size_t k = 9 * (size_t)c + q;
          xc[k] = st.cam_used[c] ? x[k] + y[k] * scale[k] : x[k];
        }
        if (o->rig && st.cam_used[c]) {
          /* rig model: the pose moves on SE3, T <- exp(xi) T */
          const size_t k = 9 * (size_t)c;
          const double dw[3] = {y[k] * scale[k], y[k + 1] * scale[k + 1], y[k + 2] * scale[k + 2]};
          const double du[3] = {y[k + 3] * scale[k + 3], y[k + 4] * scale[k + 4], y[k + 5] * scale[k + 5]};
          orc_se3_compose_left(dw, du, x + k, xc + k);
        } else if (o->camera_update == ORC_UPDATE_SO3_LEFT && st.cam_used[c]) {
          const size_t k = 9 * (size_t)c;
          const double dw[3] = {y[k] * scale[k], y[k + 1] * scale[k + 1], y[k + 2] * scale[k + 2]};
          orc_compose_left(dw, x + k, xc + k);
        }
      }
      for (int j = 0; j < p->np; ++j)
        for (int q = 0; q < 3; ++q) {
          const size_t k = 9 * (size_t)p->nc + 3 * (size_t)j + q;
          xc[k] = st.pt_used[j] ? x[k] + y[k] * scale[k] : x[k];
        }
      double cand_cost;
      if (!eval_cost(p, &model, xc, o->loss, o->loss_scale, &cand_cost)) cand_cost = DBL_MAX;
      const double step_norm = used_diff_norm(&st, x, xc);
      if (o->verbose)
        printf("%4d %.6e %.2e %.2e %.2e %.2e %.2e %4d\n", iteration, cand_cost, x_cost - cand_cost,
               gmax, step_norm, (x_cost - cand_cost) / mcc, radius, lin_it);
      if (!g2o && step_norm <= o->parameter_tolerance * (x_norm + o->parameter_tolerance)) {
        term = 0;
        reason = 4;
        ++s->num_unsuccessful_steps;
        trace_put(s, iteration, cand_cost, radius, lin_it, 0);
        break;
      }
      const double cost_change = x_cost - cand_cost;
      if (!g2o && fabs(cost_change) <= o->function_tolerance * x_cost) {
        term = 0;
        reason = 2;
        ++s->num_unsuccessful_steps;
        trace_put(s, iteration, cand_cost, radius, lin_it, 0);
        break;
      }
      const double rel = (cand_cost >= DBL_MAX) ? -DBL_MAX : (x_cost - cand_cost) / mcc;
      if (g2o) rho = (cand_cost >= DBL_MAX) ? -DBL_MAX : 2.0 * (x_cost - cand_cost) / (2.0 * mcc + 1e-3);
      if (g2o ? rho > 0.0 : rel > o->min_relative_decrease) {
        memcpy(x, xc, sizeof(double) * (size_t)n);
        x_norm = used_norm(&st, x);
        if (!eval_jacobian(p, &model, x, o->loss, o->loss_scale, r, J, &x_cost)) {
          term = 2;
          reason = 7;
          break;
        }
        gradient(&st, J, r, g);
        gmax = gradient_max_norm(&st, x, g);
        scale_columns(p, J, scale);
        if (g2o) {
          const double t = 2.0 * rho - 1.0;
          radius = fmin(DBL_MAX, radius / fmax(1.0 / 3.0, fmin(2.0 / 3.0, 1.0 - t * t * t)));
        } else {
          const double t = 2.0 * rel - 1.0;
          radius = radius / fmax(1.0 / 3.0, 1.0 - t * t * t);
          radius = fmin(o->max_trust_region_radius, radius);
        }
        decrease_factor = 2.0;
        reuse_diagonal = 0;
        successful = 1;
        iter_cost = x_cost;
        if (x_cost < minimum_cost) {
          minimum_cost = x_cost;
          memcpy(p->parameters, x, sizeof(double) * (size_t)n);
        }
      } else {
        radius /= decrease_factor;
        decrease_factor *= 2.0;
        reuse_diagonal = 1;
        iter_cost = cand_cost;
      }
    }
    if (successful)
      ++s->num_successful_steps;
    else
      ++s->num_unsuccessful_steps;
    trace_put(s, iteration, iter_cost, radius, lin_it, successful);
    if (g2o) {
      ++trials;
      if (trials >= ORC_G2O_MAX_TRIALS || (!successful && (rho == 0.0 || radius <= 0.0))) {
        term = 0;
        reason = 8;
      } else if (successful && ++outer >= o->max_num_iterations) {
        term = 1;
        reason = 1;
      }
      if (successful) trials = 0;
    } else if (iteration >= o->max_num_iterations) {
      term = 1;
      reason = 1;
    } else if (successful && gmax <= o->gradient_tolerance) {
      term = 0;
      reason = 3;
    } else if (radius <= o->min_trust_region_radius) {
      term = 0;
      reason = 5;
    }
  }
done:
  s->num_iterations = iteration;
  s->termination_type = term;
  s->termination_reason = reason;
  s->final_trust_region_radius = radius;
  {
    /* final cost and gradient at the returned parameters */
    double fc = 0.0;
    if (eval_jacobian(p, &model, p->parameters, o->loss, o->loss_scale, r, J, &fc)) {
      gradient(&st, J, r, g);
      s->gradient_max_norm = gradient_max_norm(&st, p->parameters, g);
    }
    s->final_cost = fc;
  }
  free(x);
  free(xc);
  free(r);
  free(J);
  free(g);
  free(cn);
  free(scale);
  free(diag);
  free(D);
  free(y);
  free_structure(&st);
  return term != 2;
}
