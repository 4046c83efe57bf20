// synth.cpp — seeded synthetic BAL problems for the benchmark configurations.
//
// No public dataset is used: these problems stand in for BAL files with the
// shapes the benchmark names.  Snavely cameras (f = 500, k1 ~ U(-0.05,
// 0.05), k2 ~ U(-0.005, 0.005)), observations = projection + N(0, 0.5 px),
// initial guess perturbed (rotation 0.01 rad, translation 0.1, points 0.1,
// focal 1 %).  Camera layouts:
//   RING   cameras on a circle of radius 10 looking at the origin, points
//          uniform in [-2, 2]^3, each seen by U{min..max} distinct cameras;
//   WALK   random-walk trajectory (step 0.2, small yaw drift) through a
//          40 x 10 x 40 box, each point placed in front of an anchor camera
//          and seen by the nearest (in trajectory order) cameras that see it;
//   LOOPS  several closed random-walk loops starting at the same point;
//   WINDOW a short random-walk segment (local-BA window).
// The RNG is a private xoshiro256** seeded by splitmix64, so the generator
// gives the same problem on every machine with an IEEE libm.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "gba.h"

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (int i = 0; i < 4; ++i) {
      z += 0x9e3779b97f4a7c15ULL;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
      x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
      s[i] = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  int uniform_int(int a, int b) { return a + (int)(uniform() * (double)(b - a + 1)); }  // [a, b]
  double normal() {
    double x1, x2, w;
    do {
      x1 = 2.0 * uniform() - 1.0;
      x2 = 2.0 * uniform() - 1.0;
      w = x1 * x1 + x2 * x2;
    } while (w >= 1.0 || w == 0.0);
    return x1 * std::sqrt(-2.0 * std::log(w) / w);
  }
};

struct Mat3 {
  double m[9];
};

// rotation matrix (rows = camera axes in world coordinates) -> angle-axis,
// through a unit quaternion (Shepperd) and the reference's quaternion ->
// angle-axis conversion.
void matrix_to_angle_axis(const Mat3 &R, double aa[3]) {
  const double *m = R.m;
  const double tr = m[0] + m[4] + m[8];
  double q[4];
  if (tr > 0) {
    const double s = std::sqrt(tr + 1.0) * 2;
    q[0] = 0.25 * s;
    q[1] = (m[7] - m[5]) / s;
    q[2] = (m[2] - m[6]) / s;
    q[3] = (m[3] - m[1]) / s;
  } else if (m[0] > m[4] && m[0] > m[8]) {
    const double s = std::sqrt(1.0 + m[0] - m[4] - m[8]) * 2;
    q[0] = (m[7] - m[5]) / s;
    q[1] = 0.25 * s;
    q[2] = (m[1] + m[3]) / s;
    q[3] = (m[2] + m[6]) / s;
  } else if (m[4] > m[8]) {
    const double s = std::sqrt(1.0 + m[4] - m[0] - m[8]) * 2;
    q[0] = (m[2] - m[6]) / s;
    q[1] = (m[1] + m[3]) / s;
    q[2] = 0.25 * s;
    q[3] = (m[5] + m[7]) / s;
  } else {
    const double s = std::sqrt(1.0 + m[8] - m[0] - m[4]) * 2;
    q[0] = (m[3] - m[1]) / s;
    q[1] = (m[2] + m[6]) / s;
    q[2] = (m[5] + m[7]) / s;
    q[3] = 0.25 * s;
  }
  gba_quaternion_to_angle_axis(q, aa);
}

struct Cam {
  double C[3];    // centre
  double fwd[3];  // viewing direction (world)
  Mat3 R;         // world -> camera
  double cam[9];  // Snavely parameters
};

void cross(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
void normalize3(double v[3]) {
  const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= n, v[1] /= n, v[2] /= n;
}

// camera at C looking along fwd: camera z axis = -fwd (the Snavely model
// sees points with P_z < 0), x axis horizontal.
void make_camera(Cam &c, Rng &rng, double focal, double k1r, double k2r) {
  double z[3] = {-c.fwd[0], -c.fwd[1], -c.fwd[2]};
  normalize3(z);
  const double up[3] = {0.0, 1.0, 0.0};
  double x[3], y[3];
  cross(up, z, x);
  normalize3(x);
  cross(z, x, y);
  for (int k = 0; k < 3; ++k) {
    c.R.m[k] = x[k];
    c.R.m[3 + k] = y[k];
    c.R.m[6 + k] = z[k];
  }
  double aa[3];
  matrix_to_angle_axis(c.R, aa);
  c.cam[0] = aa[0], c.cam[1] = aa[1], c.cam[2] = aa[2];
  // t = -R C, evaluated through the same rotation the residual uses
  double rc[3];
  gba_angle_axis_rotate_point(aa, c.C, rc);
  c.cam[3] = -rc[0], c.cam[4] = -rc[1], c.cam[5] = -rc[2];
  c.cam[6] = focal;
  c.cam[7] = rng.uniform(-k1r, k1r);
  c.cam[8] = rng.uniform(-k2r, k2r);
}

// Snavely projection with the true camera (SnavelyReprojectionError.h:61-87)
bool project(const double *cam, const double X[3], double uv[2], double max_xy) {
  double p[3];
  gba_angle_axis_rotate_point(cam, X, p);
  p[0] += cam[3], p[1] += cam[4], p[2] += cam[5];
  if (p[2] > -0.3) return false;  // behind or too close
  const double xp = -p[0] / p[2], yp = -p[1] / p[2];
  if (std::fabs(xp) > max_xy || std::fabs(yp) > 0.75 * max_xy) return false;
  const double r2 = xp * xp + yp * yp;
  const double d = 1.0 + r2 * (cam[7] + cam[8] * r2);
  uv[0] = cam[6] * d * xp;
  uv[1] = cam[6] * d * yp;
  return true;
}

int draw_views(const gba_synth_spec &s, Rng &rng) {
  const int lo = s.min_views, hi = s.max_views;
  if (s.view_distribution == 1) {  // 2 + geometric tail
    const double p = s.view_param > 0 ? s.view_param : 0.3;
    int k = lo;
    while (k < hi && rng.uniform() > p) ++k;
    return k;
  }
  if (s.view_distribution == 2) {  // lo - 1 + Zipf(s) truncated to [1, hi - lo + 1]
    const int n = hi - lo + 1;
    const double a = s.view_param > 0 ? s.view_param : 1.5;
    // inverse CDF on the truncated support (n <= a few hundred)
    double tot = 0.0;
    for (int k = 1; k <= n; ++k) tot += std::pow((double)k, -a);
    double u = rng.uniform() * tot;
    for (int k = 1; k <= n; ++k) {
      u -= std::pow((double)k, -a);
      if (u <= 0.0) return lo - 1 + k;
    }
    return hi;
  }
  return rng.uniform_int(lo, hi);
}

struct Scene {
  std::vector<Cam> cams;
  std::vector<double> pts;
  std::vector<int> oc, op;
  std::vector<double> uv;
};

gba_status build_scene(const gba_synth_spec &s, Scene &sc) {
  Rng rng(s.seed * 0x2545F4914F6CDD1DULL + 17);
  const int nc = s.num_cameras, np = s.num_points;
  sc.cams.resize(nc);
  const double max_xy = 0.6;
  // -- trajectory
  if (s.layout == GBA_SYNTH_RING) {
    for (int i = 0; i < nc; ++i) {
      const double phi = 2.0 * M_PI * i / nc;
      Cam &c = sc.cams[i];
      c.C[0] = 10.0 * std::cos(phi), c.C[1] = 0.0, c.C[2] = 10.0 * std::sin(phi);
      c.fwd[0] = -c.C[0], c.fwd[1] = -c.C[1], c.fwd[2] = -c.C[2];
      normalize3(c.fwd);
    }
  } else {
    const int loops = s.layout == GBA_SYNTH_LOOPS ? 6 : 1;
    const int per = (nc + loops - 1) / loops;
    int idx = 0;
    for (int l = 0; l < loops && idx < nc; ++l) {
      double pos[3] = {0.0, 0.0, 0.0};
      double yaw = 2.0 * M_PI * l / loops + rng.uniform(-0.2, 0.2);
      const int n = std::min(per, nc - idx);
      // closed loop: the heading turns by 2 pi over the loop (LOOPS), or
      // drifts slowly (WALK / WINDOW)
      const double turn = (s.layout == GBA_SYNTH_LOOPS) ? 2.0 * M_PI / n : 0.0;
      for (int i = 0; i < n; ++i, ++idx) {
        Cam &c = sc.cams[idx];
        std::memcpy(c.C, pos, sizeof pos);
        c.fwd[0] = std::cos(yaw), c.fwd[1] = rng.uniform(-0.05, 0.05), c.fwd[2] = std::sin(yaw);
        normalize3(c.fwd);
        yaw += turn + rng.normal() * 0.02;
        pos[0] += 0.2 * std::cos(yaw);
        pos[2] += 0.2 * std::sin(yaw);
        pos[1] += rng.normal() * 0.01;
        if (s.layout == GBA_SYNTH_WALK) {  // stay inside the 40 x 10 x 40 box
          if (std::fabs(pos[0]) > 18.0 || std::fabs(pos[2]) > 18.0) yaw += M_PI / 2;
          pos[1] = std::max(-4.0, std::min(4.0, pos[1]));
        }
      }
    }
  }
  for (int i = 0; i < nc; ++i) make_camera(sc.cams[i], rng, s.focal, s.k1_range, s.k2_range);
  // -- points and observations
  sc.pts.resize(3 * (size_t)np);
  sc.oc.clear();
  sc.op.clear();
  sc.uv.clear();
  std::vector<int> vis, pick;
  std::vector<double> uvtmp;
  for (int j = 0; j < np; ++j) {
    int want = draw_views(s, rng);
    if (want > nc) want = nc;
    for (int attempt = 0;; ++attempt) {
      double X[3];
      int anchor = 0;
      if (s.layout == GBA_SYNTH_RING) {
        for (int k = 0; k < 3; ++k) X[k] = rng.uniform(-2.0, 2.0);
      } else {
        anchor = rng.uniform_int(0, nc - 1);
        const Cam &a = sc.cams[anchor];
        const double depth = rng.uniform(3.0, 12.0);
        const double xp = rng.uniform(-0.4, 0.4), yp = rng.uniform(-0.3, 0.3);
        // camera-frame point (xp*depth, yp*depth, -depth) -> world: R^T (P) + C
        const double P[3] = {-xp * -depth, -yp * -depth, -depth};
        for (int k = 0; k < 3; ++k)
          X[k] = a.R.m[k] * P[0] + a.R.m[3 + k] * P[1] + a.R.m[6 + k] * P[2] + a.C[k];
        (void)xp;
      }
      // visible cameras, nearest to the anchor in trajectory order first
      vis.clear();
      uvtmp.clear();
      double uv[2];
      if (s.layout == GBA_SYNTH_RING) {
        for (int i = 0; i < nc; ++i)
          if (project(sc.cams[i].cam, X, uv, max_xy)) vis.push_back(i);
      } else {
        const int window = std::max(want * 3, 24);
        for (int d = 0; d <= window && (int)vis.size() < 4 * want; ++d) {
          for (int sgn = 0; sgn < (d ? 2 : 1); ++sgn) {
            const int i = sgn ? anchor - d : anchor + d;
            if (i < 0 || i >= nc) continue;
            if (project(sc.cams[i].cam, X, uv, max_xy)) vis.push_back(i);
          }
        }
      }
      if ((int)vis.size() < std::min(want, 2) && attempt < 50) continue;
      int take = std::min(want, (int)vis.size());
      if (take < 1) {  // give up on visibility for this point: fall back to the anchor
        vis.assign(1, anchor);
        take = 1;
      }
      pick.clear();
      if (s.layout == GBA_SYNTH_RING) {
        // `take` distinct cameras uniformly (partial Fisher-Yates)
        for (int k = 0; k < take; ++k) {
          const int r = k + (int)(rng.uniform() * (double)(vis.size() - k));
          std::swap(vis[k], vis[r]);
          pick.push_back(vis[k]);
        }
      } else {
        pick.assign(vis.begin(), vis.begin() + take);
      }
      std::sort(pick.begin(), pick.end());
      for (int k = 0; k < 3; ++k) sc.pts[3 * (size_t)j + k] = X[k];
      for (int i : pick) {
        if (!project(sc.cams[i].cam, X, uv, 1e9)) continue;
        sc.oc.push_back(i);
        sc.op.push_back(j);
        sc.uv.push_back(uv[0] + rng.normal() * s.pixel_noise);
        sc.uv.push_back(uv[1] + rng.normal() * s.pixel_noise);
      }
      break;
    }
  }
  return GBA_OK;
}

}  // namespace

extern "C" {

gba_status gba_synth_preset(int32_t config, int32_t index, uint64_t seed, gba_synth_spec *s) {
  if (!s) return GBA_ERR_INVALID_ARGUMENT;
  std::memset(s, 0, sizeof *s);
  s->focal = 500.0;
  s->k1_range = 0.05;
  s->k2_range = 0.005;
  s->pixel_noise = 0.5;
  s->rotation_noise = 0.01;
  s->translation_noise = 0.1;
  s->point_noise = 0.1;
  s->focal_noise = 0.01;
  s->seed = seed + 1000003ULL * (uint64_t)config + 7919ULL * (uint64_t)index;
  switch (config) {
    case 0:
      s->layout = GBA_SYNTH_RING;
      s->num_cameras = 16;
      s->num_points = 2000;
      s->min_views = 4, s->max_views = 10;
      s->view_distribution = 0;
      return GBA_OK;
    case 1:
      s->layout = GBA_SYNTH_WALK;
      s->num_cameras = 250;
      s->num_points = 60000;
      s->min_views = 2, s->max_views = 15;
      s->view_distribution = 1;
      s->view_param = 0.25;  // mean ~5 views
      return GBA_OK;
    case 2:
      s->layout = GBA_SYNTH_LOOPS;
      s->num_cameras = 1800;
      s->num_points = 1000000;
      s->min_views = 2, s->max_views = 40;
      s->view_distribution = 2;
      s->view_param = 1.5;
      return GBA_OK;
    case 3: {
      Rng r(s->seed);
      s->layout = GBA_SYNTH_WINDOW;
      s->num_cameras = r.uniform_int(5, 40);
      s->num_points = r.uniform_int(200, 5000);
      s->min_views = 2, s->max_views = 8;
      s->view_distribution = 0;
      return GBA_OK;
    }
    case 4: {
      Rng r(s->seed);
      s->layout = GBA_SYNTH_WALK;
      s->num_cameras = (int)std::lround(std::exp(r.uniform(std::log(10.0), std::log(400.0))));
      s->num_points = (int)std::lround(std::exp(r.uniform(std::log(1000.0), std::log(150000.0))));
      s->min_views = 2, s->max_views = 15;
      s->view_distribution = 1;
      s->view_param = 0.25;
      return GBA_OK;
    }
    default:
      return GBA_ERR_INVALID_ARGUMENT;
  }
}

gba_status gba_synth_size(const gba_synth_spec *s, int32_t *nc, int32_t *np, int32_t *no) {
  if (!s || !nc || !np || !no || s->num_cameras <= 0 || s->num_points < 0 || s->min_views < 1 ||
      s->max_views < s->min_views)
    return GBA_ERR_INVALID_ARGUMENT;
  Scene sc;
  build_scene(*s, sc);
  *nc = s->num_cameras;
  *np = s->num_points;
  *no = (int32_t)sc.oc.size();
  return GBA_OK;
}

gba_status gba_synth_generate(const gba_synth_spec *s, const gba_problem_view *out, double *truth) {
  if (!s || !out) return GBA_ERR_INVALID_ARGUMENT;
  Scene sc;
  build_scene(*s, sc);
  if (out->num_cameras != s->num_cameras || out->num_points != s->num_points ||
      out->num_observations != (int32_t)sc.oc.size())
    return GBA_ERR_INVALID_ARGUMENT;
  const int nc = s->num_cameras, np = s->num_points;
  for (size_t i = 0; i < sc.oc.size(); ++i) {
    const_cast<int32_t *>(out->camera_index)[i] = sc.oc[i];
    const_cast<int32_t *>(out->point_index)[i] = sc.op[i];
    const_cast<double *>(out->observations)[2 * i] = sc.uv[2 * i];
    const_cast<double *>(out->observations)[2 * i + 1] = sc.uv[2 * i + 1];
  }
  double *par = out->parameters;
  for (int i = 0; i < nc; ++i) std::memcpy(par + 9 * (size_t)i, sc.cams[i].cam, 9 * sizeof(double));
  std::memcpy(par + 9 * (size_t)nc, sc.pts.data(), 3 * (size_t)np * sizeof(double));
  if (truth) std::memcpy(truth, par, sizeof(double) * (9 * (size_t)nc + 3 * (size_t)np));
  // initial guess: perturb rotation, translation, points and focal length
  Rng rng(s->seed ^ 0x5DEECE66DULL);
  for (int i = 0; i < nc; ++i) {
    double *c = par + 9 * (size_t)i;
    for (int k = 0; k < 3; ++k) c[k] += rng.normal() * s->rotation_noise;
    for (int k = 3; k < 6; ++k) c[k] += rng.normal() * s->translation_noise;
    c[6] *= 1.0 + rng.normal() * s->focal_noise;
  }
  for (int j = 0; j < np; ++j)
    for (int k = 0; k < 3; ++k) par[9 * (size_t)nc + 3 * (size_t)j + k] += rng.normal() * s->point_noise;
  return GBA_OK;
}

}  // extern "C"
