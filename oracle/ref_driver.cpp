// ref_driver.cpp — C entry points over the reference's OWN sources, compiled
// from where they lie in the reference tree by oracle/build_ref.sh into
// oracle/_ref/libslamplay_ref.so.
//
// TEST INFRASTRUCTURE ONLY: used by the CPU tests to pin the oracle
// restatement (oracle.c) and the product's BAL I/O against the reference:
//   - utils/camera/SnavelyReprojectionError.h:42-87 (residual functor),
//     instantiated with double and with the forward-mode dual type below (the
//     role of Ceres' Jet in AutoDiffCostFunction<...,2,9,3>, :89-92);
//   - utils/geometry/rotation.h:73-199 (rotation, quaternion conversions);
//   - utils/datasets/BALProblem.cpp:78-336 (parse, write, PLY, Normalize,
//     Perturb).
// The Ceres and Eigen headers those files include are replaced by
// declaration shims in oracle/ref_shim (Ceres' solver is not used here).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>

#include "camera/SnavelyReprojectionError.h"
#include "datasets/BALProblem.h"
#include "geometry/rotation.h"

namespace refjet {
// Value + 12 derivatives (9 camera, 3 point).
struct Jet {
  double a;
  double v[12];
  Jet() : a(0.0) { std::memset(v, 0, sizeof v); }
  Jet(double x) : a(x) { std::memset(v, 0, sizeof v); }  // NOLINT: implicit like Ceres' T(x)
  Jet &operator+=(const Jet &y) {
    a += y.a;
    for (int k = 0; k < 12; ++k) v[k] += y.v[k];
    return *this;
  }
};
inline Jet operator+(const Jet &x, const Jet &y) {
  Jet r(x.a + y.a);
  for (int k = 0; k < 12; ++k) r.v[k] = x.v[k] + y.v[k];
  return r;
}
inline Jet operator-(const Jet &x, const Jet &y) {
  Jet r(x.a - y.a);
  for (int k = 0; k < 12; ++k) r.v[k] = x.v[k] - y.v[k];
  return r;
}
inline Jet operator-(const Jet &x) {
  Jet r(-x.a);
  for (int k = 0; k < 12; ++k) r.v[k] = -x.v[k];
  return r;
}
inline Jet operator*(const Jet &x, const Jet &y) {
  Jet r(x.a * y.a);
  for (int k = 0; k < 12; ++k) r.v[k] = x.a * y.v[k] + x.v[k] * y.a;
  return r;
}
inline Jet operator/(const Jet &x, const Jet &y) {
  const double q = x.a / y.a;
  Jet r(q);
  for (int k = 0; k < 12; ++k) r.v[k] = (x.v[k] - q * y.v[k]) / y.a;
  return r;
}
inline Jet operator/(double s, const Jet &y) {
  Jet r(s / y.a);
  const double f = -s / (y.a * y.a);
  for (int k = 0; k < 12; ++k) r.v[k] = y.v[k] * f;
  return r;
}
inline bool operator>(const Jet &x, const Jet &y) { return x.a > y.a; }
inline bool operator<(const Jet &x, const Jet &y) { return x.a < y.a; }
inline Jet sqrt(const Jet &x) {
  const double s = std::sqrt(x.a);
  Jet r(s);
  const double f = 1.0 / (2.0 * s);
  for (int k = 0; k < 12; ++k) r.v[k] = x.v[k] * f;
  return r;
}
inline Jet cos(const Jet &x) {
  Jet r(std::cos(x.a));
  const double f = -std::sin(x.a);
  for (int k = 0; k < 12; ++k) r.v[k] = f * x.v[k];
  return r;
}
inline Jet sin(const Jet &x) {
  Jet r(std::sin(x.a));
  const double f = std::cos(x.a);
  for (int k = 0; k < 12; ++k) r.v[k] = f * x.v[k];
  return r;
}
}  // namespace refjet

using slamplay::BALProblem;
using slamplay::SnavelyReprojectionError;

extern "C" {

int ref_residual(const double *cam, const double *pt, const double *uv, double *r) {
  SnavelyReprojectionError f(uv[0], uv[1]);
  return f(cam, pt, r) ? 1 : 0;
}

int ref_residual_jacobian(const double *cam, const double *pt, const double *uv, double *r,
                          double *J) {
  using refjet::Jet;
  Jet c[9], X[3], res[2];
  for (int k = 0; k < 9; ++k) {
    c[k] = Jet(cam[k]);
    c[k].v[k] = 1.0;
  }
  for (int k = 0; k < 3; ++k) {
    X[k] = Jet(pt[k]);
    X[k].v[9 + k] = 1.0;
  }
  SnavelyReprojectionError f(uv[0], uv[1]);
  const bool ok = f(c, X, res);
  for (int i = 0; i < 2; ++i) {
    r[i] = res[i].a;
    for (int k = 0; k < 12; ++k) J[12 * i + k] = res[i].v[k];
  }
  return ok ? 1 : 0;
}

void ref_rotate(const double *aa, const double *pt, double *out) {
  slamplay::angleAxisRotatePoint(aa, pt, out);
}
void ref_aa_to_quat(const double *aa, double *q) { slamplay::angleAxisToQuaternion(aa, q); }
void ref_quat_to_aa(const double *q, double *aa) { slamplay::quaternionToAngleAxis(q, aa); }

// Loads a BAL file with the reference reader and copies its arrays out.
// Pass nullptr arrays to query sizes only.
int ref_bal_load(const char *path, int use_quaternions, int *nc, int *np, int *no, int *nparam,
                 int *cam_idx, int *pt_idx, double *obs, double *params) {
  BALProblem b(path, use_quaternions != 0);
  *nc = b.num_cameras();
  *np = b.num_points();
  *no = b.num_observations();
  *nparam = b.num_parameters();
  if (cam_idx) std::memcpy(cam_idx, b.camera_index(), sizeof(int) * (size_t)*no);
  if (pt_idx) std::memcpy(pt_idx, b.point_index(), sizeof(int) * (size_t)*no);
  if (obs) std::memcpy(obs, b.observations(), sizeof(double) * 2 * (size_t)*no);
  if (params) std::memcpy(params, b.parameters(), sizeof(double) * (size_t)*nparam);
  return 1;
}

// Loads `path`, runs Normalize() (if normalize) then, after srand(seed),
// Perturb(r, t, p) (if perturb) exactly as test_bundle_adjustment_ceres.cpp:48-50,
// and copies the parameters out.
int ref_bal_prepare(const char *path, int normalize, int perturb, unsigned seed, double rs,
                    double ts, double ps, double *params) {
  BALProblem b(path);
  if (normalize) b.Normalize();
  if (perturb) {
    std::srand(seed);
    b.Perturb(rs, ts, ps);
  }
  std::memcpy(params, b.parameters(), sizeof(double) * (size_t)b.num_parameters());
  return 1;
}

int ref_bal_write(const char *in_path, const char *out_path) {
  BALProblem b(in_path);
  b.WriteToFile(out_path);
  return 1;
}

int ref_bal_write_ply(const char *in_path, const char *out_path) {
  BALProblem b(in_path);
  b.WriteToPLYFile(out_path);
  return 1;
}

}  // extern "C"
