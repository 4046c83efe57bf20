// bal_io.cpp — BALProblem host functionality (utils/datasets/BALProblem.cpp)
// behind the C ABI: text reader/writer, PLY export, Normalize, Perturb, and
// the rotation helpers of utils/geometry/rotation.h.
#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gba.h"

namespace {

thread_local std::string g_io_error;

// Rodrigues rotation with the theta^2 <= DBL_EPSILON first-order branch
// (rotation.h:133-199).
void rotate(const double aa[3], const double pt[3], double out[3]) {
  const double theta2 = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
  if (theta2 > DBL_EPSILON) {
    const double theta = std::sqrt(theta2);
    const double c = std::cos(theta), s = std::sin(theta);
    const double inv = 1.0 / theta;
    const double w[3] = {aa[0] * inv, aa[1] * inv, aa[2] * inv};
    const double wx[3] = {w[1] * pt[2] - w[2] * pt[1], w[2] * pt[0] - w[0] * pt[2], w[0] * pt[1] - w[1] * pt[0]};
    const double tmp = (w[0] * pt[0] + w[1] * pt[1] + w[2] * pt[2]) * (1.0 - c);
    for (int i = 0; i < 3; ++i) out[i] = pt[i] * c + wx[i] * s + w[i] * tmp;
  } else {
    const double wx[3] = {aa[1] * pt[2] - aa[2] * pt[1], aa[2] * pt[0] - aa[0] * pt[2], aa[0] * pt[1] - aa[1] * pt[0]};
    for (int i = 0; i < 3; ++i) out[i] = pt[i] + wx[i];
  }
}

// camera -> (angle-axis, centre c = -R^T t)   (BALProblem.cpp:230-246)
void camera_to_center(const double *cam, double aa[3], double center[3]) {
  for (int i = 0; i < 3; ++i) aa[i] = cam[i];
  const double inv[3] = {-aa[0], -aa[1], -aa[2]};
  rotate(inv, cam + 3, center);
  for (int i = 0; i < 3; ++i) center[i] *= -1.0;
}

// (angle-axis, centre) -> camera, t = -R c   (BALProblem.cpp:248-261)
void center_to_camera(const double aa[3], const double center[3], double *cam) {
  for (int i = 0; i < 3; ++i) cam[i] = aa[i];
  rotate(aa, center, cam + 3);
  for (int i = 0; i < 3; ++i) cam[3 + i] *= -1.0;
}

// uniform in [0,1]: the C library's rand() as the reference draws it
// (BALProblem.cpp:39-42), or a private seeded generator.
struct Uniform {
  bool use_crand;
  uint64_t s;
  double next() {
    if (use_crand) return static_cast<double>(std::rand()) / RAND_MAX;
    // splitmix64
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740991.0);
  }
  // polar Box-Muller (BALProblem.cpp:44-54)
  double normal() {
    double x1, x2, w;
    do {
      x1 = 2.0 * next() - 1.0;
      x2 = 2.0 * next() - 1.0;
      w = x1 * x1 + x2 * x2;
    } while (w >= 1.0 || w == 0.0);
    w = std::sqrt((-2.0 * std::log(w)) / w);
    return x1 * w;
  }
};

// Buffered whitespace-separated token reader over a whole file.
struct Reader {
  std::vector<char> buf;
  size_t pos = 0;
  bool open(const char *path) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(n > 0 ? (size_t)n + 1 : 1);
    const size_t got = n > 0 ? std::fread(buf.data(), 1, (size_t)n, f) : 0;
    buf[got] = '\0';
    buf.resize(got + 1);
    std::fclose(f);
    return true;
  }
  bool next_int(int *v) {
    char *s = buf.data() + pos, *e = nullptr;
    errno = 0;
    const long x = std::strtol(s, &e, 10);
    if (e == s || errno) return false;
    pos = e - buf.data();
    *v = (int)x;
    return true;
  }
  bool next_double(double *v) {
    char *s = buf.data() + pos, *e = nullptr;
    const double x = std::strtod(s, &e);
    if (e == s) return false;
    pos = e - buf.data();
    *v = x;
    return true;
  }
};

bool write_all(FILE *f, const char *s) { return std::fputs(s, f) >= 0; }

}  // namespace

const char *gba_io_last_error(void) { return g_io_error.c_str(); }

extern "C" {

void gba_angle_axis_rotate_point(const double *angle_axis, const double *pt, double *result) {
  rotate(angle_axis, pt, result);
}

// rotation.h:72-94
void gba_angle_axis_to_quaternion(const double *aa, double *q) {
  const double a0 = aa[0], a1 = aa[1], a2 = aa[2];
  const double theta2 = a0 * a0 + a1 * a1 + a2 * a2;
  if (theta2 > DBL_EPSILON) {
    const double theta = std::sqrt(theta2);
    const double half = theta * 0.5;
    const double k = std::sin(half) / theta;
    q[0] = std::cos(half);
    q[1] = a0 * k;
    q[2] = a1 * k;
    q[3] = a2 * k;
  } else {
    q[0] = 1.0;
    q[1] = a0 * 0.5;
    q[2] = a1 * 0.5;
    q[3] = a2 * 0.5;
  }
}

// rotation.h:96-131
void gba_quaternion_to_angle_axis(const double *q, double *aa) {
  const double q1 = q[1], q2 = q[2], q3 = q[3];
  const double s2 = q1 * q1 + q2 * q2 + q3 * q3;
  if (s2 > DBL_EPSILON) {
    const double s = std::sqrt(s2);
    const double c = q[0];
    const double two_theta = 2.0 * ((c < 0.0) ? std::atan2(-s, -c) : std::atan2(s, c));
    const double k = two_theta / s;
    aa[0] = q1 * k;
    aa[1] = q2 * k;
    aa[2] = q3 * k;
  } else {
    aa[0] = q1 * 2.0;
    aa[1] = q2 * 2.0;
    aa[2] = q3 * 2.0;
  }
}

gba_status gba_bal_read_header(const char *path, int32_t *nc, int32_t *np, int32_t *no) {
  if (!path || !nc || !np || !no) return GBA_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "r");
  if (!f) {
    g_io_error = std::string("unable to open file ") + path;
    return GBA_ERR_IO;
  }
  int a, b, c;
  const int got = std::fscanf(f, "%d %d %d", &a, &b, &c);
  std::fclose(f);
  if (got != 3 || a < 0 || b < 0 || c < 0) {
    g_io_error = "invalid BAL header";
    return GBA_ERR_IO;
  }
  *nc = a;
  *np = b;
  *no = c;
  return GBA_OK;
}

gba_status gba_bal_read(const char *path, const gba_problem_view *out) {
  if (!path || !out) return GBA_ERR_INVALID_ARGUMENT;
  Reader r;
  if (!r.open(path)) {
    g_io_error = std::string("unable to open file ") + path;
    return GBA_ERR_IO;
  }
  int nc, np, no;
  if (!r.next_int(&nc) || !r.next_int(&np) || !r.next_int(&no)) {
    g_io_error = "invalid BAL header";
    return GBA_ERR_IO;
  }
  if (nc != out->num_cameras || np != out->num_points || no != out->num_observations) {
    g_io_error = "problem view sizes do not match the file header";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  if ((no > 0 && (!out->camera_index || !out->point_index || !out->observations)) ||
      (nc + np > 0 && !out->parameters))
    return GBA_ERR_INVALID_ARGUMENT;
  int32_t *ci = const_cast<int32_t *>(out->camera_index);
  int32_t *pi = const_cast<int32_t *>(out->point_index);
  double *ob = const_cast<double *>(out->observations);
  for (int i = 0; i < no; ++i) {
    int c, p;
    if (!r.next_int(&c) || !r.next_int(&p) || !r.next_double(ob + 2 * (size_t)i) ||
        !r.next_double(ob + 2 * (size_t)i + 1)) {
      g_io_error = "invalid BAL observation line " + std::to_string(i);
      return GBA_ERR_IO;
    }
    ci[i] = c;
    pi[i] = p;
  }
  const size_t npar = 9 * (size_t)nc + 3 * (size_t)np;
  for (size_t k = 0; k < npar; ++k)
    if (!r.next_double(out->parameters + k)) {
      g_io_error = "invalid BAL parameter " + std::to_string(k);
      return GBA_ERR_IO;
    }
  return GBA_OK;
}

// BALProblem::WriteToFile (BALProblem.cpp:141-183).  The reference writes the
// camera count twice in the header ("%d %d %d %d", :149), which its own
// reader cannot parse back; this writer emits the three-number header the
// reader expects and is byte-identical to the reference from line 2 on.
gba_status gba_bal_write(const char *path, const gba_problem_view *p) {
  if (!path || !p) return GBA_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "w");
  if (!f) {
    g_io_error = std::string("unable to open file ") + path;
    return GBA_ERR_IO;
  }
  char line[128];
  std::snprintf(line, sizeof line, "%d %d %d\n", p->num_cameras, p->num_points, p->num_observations);
  bool ok = write_all(f, line);
  for (int i = 0; ok && i < p->num_observations; ++i) {
    std::snprintf(line, sizeof line, "%d %d %g %g\n", p->camera_index[i], p->point_index[i],
                  p->observations[2 * (size_t)i], p->observations[2 * (size_t)i + 1]);
    ok = write_all(f, line);
  }
  const size_t npar = 9 * (size_t)p->num_cameras + 3 * (size_t)p->num_points;
  for (size_t k = 0; ok && k < npar; ++k) {
    std::snprintf(line, sizeof line, "%.16g\n", p->parameters[k]);
    ok = write_all(f, line);
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    g_io_error = "write failed";
    return GBA_ERR_IO;
  }
  return GBA_OK;
}

// BALProblem::WriteToPLYFile (BALProblem.cpp:185-228): camera centres green,
// points white, doubles printed as std::ostream does by default (%g).
gba_status gba_bal_write_ply(const char *path, const gba_problem_view *p) {
  if (!path || !p) return GBA_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "w");
  if (!f) {
    g_io_error = std::string("unable to open file ") + path;
    return GBA_ERR_IO;
  }
  std::fprintf(f,
               "ply\nformat ascii 1.0\nelement vertex %d\nproperty float x\nproperty float y\n"
               "property float z\nproperty uchar red\nproperty uchar green\nproperty uchar blue\n"
               "end_header\n",
               p->num_cameras + p->num_points);
  for (int i = 0; i < p->num_cameras; ++i) {
    double aa[3], c[3];
    camera_to_center(p->parameters + 9 * (size_t)i, aa, c);
    std::fprintf(f, "%g %g %g 0 255 0\n", c[0], c[1], c[2]);
  }
  const double *pts = p->parameters + 9 * (size_t)p->num_cameras;
  for (int i = 0; i < p->num_points; ++i)
    std::fprintf(f, "%g %g %g  255 255 255\n", pts[3 * (size_t)i], pts[3 * (size_t)i + 1], pts[3 * (size_t)i + 2]);
  if (std::fclose(f) != 0) return GBA_ERR_IO;
  return GBA_OK;
}

// BALProblem::Normalize (BALProblem.cpp:263-303): centre on the per-axis
// median, scale so the median L1 deviation is 100, move the cameras along.
gba_status gba_bal_normalize(const gba_problem_view *p) {
  if (!p || !p->parameters || p->num_points <= 0) return GBA_ERR_INVALID_ARGUMENT;
  const int np = p->num_points;
  double *pts = p->parameters + 9 * (size_t)p->num_cameras;
  std::vector<double> tmp(np);
  double median[3];
  for (int k = 0; k < 3; ++k) {
    for (int j = 0; j < np; ++j) tmp[j] = pts[3 * (size_t)j + k];
    std::nth_element(tmp.begin(), tmp.begin() + np / 2, tmp.end());
    median[k] = tmp[np / 2];
  }
  for (int j = 0; j < np; ++j) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += std::fabs(pts[3 * (size_t)j + k] - median[k]);
    tmp[j] = s;
  }
  std::nth_element(tmp.begin(), tmp.begin() + np / 2, tmp.end());
  const double mad = tmp[np / 2];
  const double scale = 100.0 / mad;
  for (int j = 0; j < np; ++j)
    for (int k = 0; k < 3; ++k) pts[3 * (size_t)j + k] = scale * (pts[3 * (size_t)j + k] - median[k]);
  for (int i = 0; i < p->num_cameras; ++i) {
    double *cam = p->parameters + 9 * (size_t)i;
    double aa[3], c[3];
    camera_to_center(cam, aa, c);
    for (int k = 0; k < 3; ++k) c[k] = scale * (c[k] - median[k]);
    center_to_camera(aa, c, cam);
  }
  return GBA_OK;
}

// BALProblem::Perturb (BALProblem.cpp:305-336).
gba_status gba_bal_perturb(const gba_problem_view *p, double rotation_sigma, double translation_sigma,
                           double point_sigma, uint64_t seed) {
  if (!p || !p->parameters || rotation_sigma < 0 || translation_sigma < 0 || point_sigma < 0)
    return GBA_ERR_INVALID_ARGUMENT;
  Uniform u{seed == 0, seed};
  double *pts = p->parameters + 9 * (size_t)p->num_cameras;
  if (point_sigma > 0)
    for (int j = 0; j < p->num_points; ++j)
      for (int k = 0; k < 3; ++k) pts[3 * (size_t)j + k] += u.normal() * point_sigma;
  for (int i = 0; i < p->num_cameras; ++i) {
    double *cam = p->parameters + 9 * (size_t)i;
    double aa[3], c[3];
    camera_to_center(cam, aa, c);
    if (rotation_sigma > 0.0)
      for (int k = 0; k < 3; ++k) aa[k] += u.normal() * rotation_sigma;
    center_to_camera(aa, c, cam);
    if (translation_sigma > 0.0)
      for (int k = 0; k < 3; ++k) cam[3 + k] += u.normal() * translation_sigma;
  }
  return GBA_OK;
}

}  // extern "C"
