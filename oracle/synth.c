/*
 * synth.c — the benchmark configurations' synthetic problems, generated on
 * the oracle's side.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference ships one real BAL file and no
 * generator; the benchmark workloads are seeded synthetic BAL problems that
 * the product library also generates (slamplay_gb300/csrc/synth.cpp,
 * gba_synth_*).  This is a second, independent implementation of the same
 * recipe in C, so that the CPU baseline builds its input without loading the
 * product library.  tests/test_oracle_synth.py checks that both give the
 * same bytes (camera and point indices, observations, parameters).
 *
 * The recipe: Snavely cameras (BAL layout, utils/datasets/BALProblem.h:55-98:
 * angle-axis, translation, f, k1, k2) with f = 500, k1 ~ U(-0.05, 0.05),
 * k2 ~ U(-0.005, 0.005); observations = the Snavely projection
 * (utils/camera/SnavelyReprojectionError.h:61-87) of the true scene plus
 * N(0, 0.5 px); the initial guess perturbs rotation by 0.01 rad,
 * translation by 0.1, points by 0.1 and f by 1 %.  Layouts: a 16-camera ring
 * (configuration 0), a 250-camera random walk through a 40 x 10 x 40 box
 * (1), six loops with coincident starts (2), short random-walk windows (3)
 * and log-uniform serving requests (4).  The random stream is xoshiro256**
 * seeded by splitmix64; normals are the polar Box-Muller method.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define SYN_PI 3.14159265358979323846

/* ---- random stream --------------------------------------------------- */
typedef struct {
  uint64_t s[4];
} rng_t;

static void rng_seed(rng_t *r, uint64_t seed) {
  uint64_t z = seed;
  for (int i = 0; i < 4; ++i) {
    z += 0x9e3779b97f4a7c15ULL;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    r->s[i] = x ^ (x >> 31);
  }
}
static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t rng_next(rng_t *r) {
  uint64_t *s = r->s;
  const uint64_t out = rotl64(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return out;
}
static double rng_u(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static double rng_ab(rng_t *r, double a, double b) { return a + (b - a) * rng_u(r); }
static int rng_int(rng_t *r, int a, int b) { return a + (int)(rng_u(r) * (double)(b - a + 1)); }
static double rng_normal(rng_t *r) {
  double x1, x2, w;
  do {
    x1 = 2.0 * rng_u(r) - 1.0;
    x2 = 2.0 * rng_u(r) - 1.0;
    w = x1 * x1 + x2 * x2;
  } while (w >= 1.0 || w == 0.0);
  return x1 * sqrt(-2.0 * log(w) / w);
}

/* ---- the configurations ------------------------------------------------ */
enum { LAY_RING = 0, LAY_WALK = 1, LAY_LOOPS = 2, LAY_WINDOW = 3 };

typedef struct {
  int layout, nc, np, min_views, max_views, view_dist;
  double view_param, focal, k1r, k2r, pixel_noise, rot_noise, trans_noise, point_noise, focal_noise;
  uint64_t seed;
} spec_t;

static int make_spec(int config, int index, uint64_t seed, spec_t *s) {
  memset(s, 0, sizeof *s);
  s->focal = 500.0;
  s->k1r = 0.05;
  s->k2r = 0.005;
  s->pixel_noise = 0.5;
  s->rot_noise = 0.01;
  s->trans_noise = 0.1;
  s->point_noise = 0.1;
  s->focal_noise = 0.01;
  s->seed = seed + 1000003ULL * (uint64_t)config + 7919ULL * (uint64_t)index;
  rng_t r;
  switch (config) {
    case 0:
      s->layout = LAY_RING, s->nc = 16, s->np = 2000, s->min_views = 4, s->max_views = 10;
      return 1;
    case 1:
      s->layout = LAY_WALK, s->nc = 250, s->np = 60000, s->min_views = 2, s->max_views = 15;
      s->view_dist = 1, s->view_param = 0.25;
      return 1;
    case 2:
      s->layout = LAY_LOOPS, s->nc = 1800, s->np = 1000000, s->min_views = 2, s->max_views = 40;
      s->view_dist = 2, s->view_param = 1.5;
      return 1;
    case 3:
      rng_seed(&r, s->seed);
      s->layout = LAY_WINDOW;
      s->nc = rng_int(&r, 5, 40);
      s->np = rng_int(&r, 200, 5000);
      s->min_views = 2, s->max_views = 8;
      return 1;
    case 4:
      rng_seed(&r, s->seed);
      s->layout = LAY_WALK;
      s->nc = (int)lround(exp(rng_ab(&r, log(10.0), log(400.0))));
      s->np = (int)lround(exp(rng_ab(&r, log(1000.0), log(150000.0))));
      s->min_views = 2, s->max_views = 15;
      s->view_dist = 1, s->view_param = 0.25;
      return 1;
    default:
      return 0;
  }
}

/* ---- geometry ------------------------------------------------------------ */
/* quaternion -> angle-axis as utils/geometry/rotation.h:96-131 */
static void quat_to_aa(const double q[4], double aa[3]) {
  const double q1 = q[1], q2 = q[2], q3 = q[3];
  const double s2 = q1 * q1 + q2 * q2 + q3 * q3;
  if (s2 > DBL_EPSILON) {
    const double s = sqrt(s2);
    const double c = q[0];
    const double two_theta = 2.0 * ((c < 0.0) ? atan2(-s, -c) : atan2(s, c));
    const double k = two_theta / s;
    aa[0] = q1 * k, aa[1] = q2 * k, aa[2] = q3 * k;
  } else {
    aa[0] = q1 * 2.0, aa[1] = q2 * 2.0, aa[2] = q3 * 2.0;
  }
}

/* rotation matrix (rows = camera axes in world coordinates) -> unit
 * quaternion (Shepperd's branches) -> angle-axis */
static void mat_to_aa(const double *m, double aa[3]) {
  const double tr = m[0] + m[4] + m[8];
  double q[4];
  if (tr > 0) {
    const double s = sqrt(tr + 1.0) * 2;
    q[0] = 0.25 * s, q[1] = (m[7] - m[5]) / s, q[2] = (m[2] - m[6]) / s, q[3] = (m[3] - m[1]) / s;
  } else if (m[0] > m[4] && m[0] > m[8]) {
    const double s = sqrt(1.0 + m[0] - m[4] - m[8]) * 2;
    q[0] = (m[7] - m[5]) / s, q[1] = 0.25 * s, q[2] = (m[1] + m[3]) / s, q[3] = (m[2] + m[6]) / s;
  } else if (m[4] > m[8]) {
    const double s = sqrt(1.0 + m[4] - m[0] - m[8]) * 2;
    q[0] = (m[2] - m[6]) / s, q[1] = (m[1] + m[3]) / s, q[2] = 0.25 * s, q[3] = (m[5] + m[7]) / s;
  } else {
    const double s = sqrt(1.0 + m[8] - m[0] - m[4]) * 2;
    q[0] = (m[3] - m[1]) / s, q[1] = (m[2] + m[6]) / s, q[2] = (m[5] + m[7]) / s, q[3] = 0.25 * s;
  }
  quat_to_aa(q, aa);
}

static void cross3(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
static void unit3(double v[3]) {
  const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= n, v[1] /= n, v[2] /= n;
}

typedef struct {
  double C[3], fwd[3], R[9], cam[9];
} cam_t;

/* camera at C looking along fwd; camera z axis = -fwd (Snavely cameras see
 * points with P_z < 0), x axis horizontal; t = -R C through the rotation the
 * residual uses */
static void make_camera(cam_t *c, rng_t *r, double focal, double k1r, double k2r) {
  double z[3] = {-c->fwd[0], -c->fwd[1], -c->fwd[2]};
  unit3(z);
  const double up[3] = {0.0, 1.0, 0.0};
  double x[3], y[3];
  cross3(up, z, x);
  unit3(x);
  cross3(z, x, y);
  for (int k = 0; k < 3; ++k) c->R[k] = x[k], c->R[3 + k] = y[k], c->R[6 + k] = z[k];
  double aa[3], rc[3];
  mat_to_aa(c->R, aa);
  c->cam[0] = aa[0], c->cam[1] = aa[1], c->cam[2] = aa[2];
  orc_angle_axis_rotate_point(aa, c->C, rc);
  c->cam[3] = -rc[0], c->cam[4] = -rc[1], c->cam[5] = -rc[2];
  c->cam[6] = focal;
  c->cam[7] = rng_ab(r, -k1r, k1r);
  c->cam[8] = rng_ab(r, -k2r, k2r);
}

/* projection with the true camera; 0 when behind, too close or outside the
 * image window */
static int project(const double *cam, const double X[3], double uv[2], double max_xy) {
  double p[3];
  orc_angle_axis_rotate_point(cam, X, p);
  p[0] += cam[3], p[1] += cam[4], p[2] += cam[5];
  if (p[2] > -0.3) return 0;
  const double xp = -p[0] / p[2], yp = -p[1] / p[2];
  if (fabs(xp) > max_xy || fabs(yp) > 0.75 * max_xy) return 0;
  const double r2 = xp * xp + yp * yp;
  const double d = 1.0 + r2 * (cam[7] + cam[8] * r2);
  uv[0] = cam[6] * d * xp;
  uv[1] = cam[6] * d * yp;
  return 1;
}

static int draw_views(const spec_t *s, rng_t *r) {
  const int lo = s->min_views, hi = s->max_views;
  if (s->view_dist == 1) { /* lo + geometric tail */
    const double p = s->view_param > 0 ? s->view_param : 0.3;
    int k = lo;
    while (k < hi && rng_u(r) > p) ++k;
    return k;
  }
  if (s->view_dist == 2) { /* lo - 1 + Zipf(s) on [1, hi - lo + 1], inverse CDF */
    const int n = hi - lo + 1;
    const double a = s->view_param > 0 ? s->view_param : 1.5;
    double tot = 0.0;
    for (int k = 1; k <= n; ++k) tot += pow((double)k, -a);
    double u = rng_u(r) * tot;
    for (int k = 1; k <= n; ++k) {
      u -= pow((double)k, -a);
      if (u <= 0.0) return lo - 1 + k;
    }
    return hi;
  }
  return rng_int(r, lo, hi);
}

static int cmp_int(const void *a, const void *b) {
  const int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

typedef struct {
  cam_t *cams;
  double *pts;
  int *oc, *op;
  double *uv;
  size_t no, cap;
} scene_t;

static int push_obs(scene_t *sc, int c, int j, double u, double v) {
  if (sc->no == sc->cap) {
    const size_t cap = sc->cap ? 2 * sc->cap : 4096;
    int *oc = (int *)realloc(sc->oc, cap * sizeof(int));
    if (oc) sc->oc = oc;
    int *op = (int *)realloc(sc->op, cap * sizeof(int));
    if (op) sc->op = op;
    double *uv = (double *)realloc(sc->uv, 2 * cap * sizeof(double));
    if (uv) sc->uv = uv;
    if (!oc || !op || !uv) return 0;
    sc->cap = cap;
  }
  sc->oc[sc->no] = c, sc->op[sc->no] = j;
  sc->uv[2 * sc->no] = u, sc->uv[2 * sc->no + 1] = v;
  ++sc->no;
  return 1;
}

static void free_scene(scene_t *sc) {
  free(sc->cams), free(sc->pts), free(sc->oc), free(sc->op), free(sc->uv);
  memset(sc, 0, sizeof *sc);
}

static int build_scene(const spec_t *s, scene_t *sc) {
  memset(sc, 0, sizeof *sc);
  rng_t rng;
  rng_seed(&rng, s->seed * 0x2545F4914F6CDD1DULL + 17);
  const int nc = s->nc, np = s->np;
  const double max_xy = 0.6;
  sc->cams = (cam_t *)calloc((size_t)nc, sizeof(cam_t));
  sc->pts = (double *)calloc(3 * (size_t)np + 1, sizeof(double));
  int *vis = (int *)malloc(((size_t)nc + 1) * sizeof(int));
  int *pick = (int *)malloc(((size_t)nc + 1) * sizeof(int));
  if (!sc->cams || !sc->pts || !vis || !pick) {
    free(vis), free(pick);
    return 0;
  }
  /* trajectory */
  if (s->layout == LAY_RING) {
    for (int i = 0; i < nc; ++i) {
      const double phi = 2.0 * SYN_PI * i / nc;
      cam_t *c = &sc->cams[i];
      c->C[0] = 10.0 * cos(phi), c->C[1] = 0.0, c->C[2] = 10.0 * sin(phi);
      c->fwd[0] = -c->C[0], c->fwd[1] = -c->C[1], c->fwd[2] = -c->C[2];
      unit3(c->fwd);
    }
  } else {
    const int loops = s->layout == LAY_LOOPS ? 6 : 1;
    const int per = (nc + loops - 1) / loops;
    int idx = 0;
    for (int l = 0; l < loops && idx < nc; ++l) {
      double pos[3] = {0.0, 0.0, 0.0};
      double yaw = 2.0 * SYN_PI * l / loops + rng_ab(&rng, -0.2, 0.2);
      const int n = per < nc - idx ? per : nc - idx;
      const double turn = (s->layout == LAY_LOOPS) ? 2.0 * SYN_PI / n : 0.0;
      for (int i = 0; i < n; ++i, ++idx) {
        cam_t *c = &sc->cams[idx];
        memcpy(c->C, pos, sizeof pos);
        c->fwd[0] = cos(yaw), c->fwd[1] = rng_ab(&rng, -0.05, 0.05), c->fwd[2] = sin(yaw);
        unit3(c->fwd);
        yaw += turn + rng_normal(&rng) * 0.02;
        pos[0] += 0.2 * cos(yaw);
        pos[2] += 0.2 * sin(yaw);
        pos[1] += rng_normal(&rng) * 0.01;
        if (s->layout == LAY_WALK) { /* stay inside the 40 x 10 x 40 box */
          if (fabs(pos[0]) > 18.0 || fabs(pos[2]) > 18.0) yaw += SYN_PI / 2;
          pos[1] = fmax(-4.0, fmin(4.0, pos[1]));
        }
      }
    }
  }
  for (int i = 0; i < nc; ++i) make_camera(&sc->cams[i], &rng, s->focal, s->k1r, s->k2r);
  /* points and observations */
  for (int j = 0; j < np; ++j) {
    int want = draw_views(s, &rng);
    if (want > nc) want = nc;
    for (int attempt = 0;; ++attempt) {
      double X[3], uv[2];
      int anchor = 0, nvis = 0;
      if (s->layout == LAY_RING) {
        for (int k = 0; k < 3; ++k) X[k] = rng_ab(&rng, -2.0, 2.0);
      } else {
        anchor = rng_int(&rng, 0, nc - 1);
        const cam_t *a = &sc->cams[anchor];
        const double depth = rng_ab(&rng, 3.0, 12.0);
        const double xp = rng_ab(&rng, -0.4, 0.4), yp = rng_ab(&rng, -0.3, 0.3);
        const double P[3] = {-xp * -depth, -yp * -depth, -depth};
        for (int k = 0; k < 3; ++k) X[k] = a->R[k] * P[0] + a->R[3 + k] * P[1] + a->R[6 + k] * P[2] + a->C[k];
      }
      /* visible cameras: all (ring), or the nearest to the anchor in
       * trajectory order first */
      if (s->layout == LAY_RING) {
        for (int i = 0; i < nc; ++i)
          if (project(sc->cams[i].cam, X, uv, max_xy)) vis[nvis++] = i;
      } else {
        const int window = want * 3 > 24 ? want * 3 : 24;
        for (int d = 0; d <= window && nvis < 4 * want; ++d)
          for (int sgn = 0; sgn < (d ? 2 : 1); ++sgn) {
            const int i = sgn ? anchor - d : anchor + d;
            if (i < 0 || i >= nc) continue;
            if (project(sc->cams[i].cam, X, uv, max_xy)) vis[nvis++] = i;
          }
      }
      if (nvis < (want < 2 ? want : 2) && attempt < 50) continue;
      int take = want < nvis ? want : nvis;
      if (take < 1) { /* no camera sees it: keep the anchor */
        vis[0] = anchor;
        nvis = 1;
        take = 1;
      }
      int npick = 0;
      if (s->layout == LAY_RING) { /* `take` distinct cameras (partial Fisher-Yates) */
        for (int k = 0; k < take; ++k) {
          const int r = k + (int)(rng_u(&rng) * (double)(nvis - k));
          const int t = vis[k];
          vis[k] = vis[r];
          vis[r] = t;
          pick[npick++] = vis[k];
        }
      } else {
        for (int k = 0; k < take; ++k) pick[npick++] = vis[k];
      }
      qsort(pick, (size_t)npick, sizeof(int), cmp_int);
      for (int k = 0; k < 3; ++k) sc->pts[3 * (size_t)j + k] = X[k];
      for (int q = 0; q < npick; ++q) {
        const int i = pick[q];
        if (!project(sc->cams[i].cam, X, uv, 1e9)) continue;
        const double u = uv[0] + rng_normal(&rng) * s->pixel_noise;
        const double v = uv[1] + rng_normal(&rng) * s->pixel_noise;
        if (!push_obs(sc, i, j, u, v)) {
          free(vis), free(pick);
          return 0;
        }
      }
      break;
    }
  }
  free(vis), free(pick);
  return 1;
}

int orc_synth_size(int config, int index, uint64_t seed, int *nc, int *np, int *no) {
  spec_t s;
  scene_t sc;
  if (!make_spec(config, index, seed, &s)) return 0;
  if (!build_scene(&s, &sc)) {
    free_scene(&sc);
    return 0;
  }
  *nc = s.nc, *np = s.np, *no = (int)sc.no;
  free_scene(&sc);
  return 1;
}

int orc_synth_generate(int config, int index, uint64_t seed, int nc, int np, int no, int *camera_index,
                       int *point_index, double *observations, double *parameters) {
  spec_t s;
  scene_t sc;
  if (!make_spec(config, index, seed, &s)) return 0;
  if (!build_scene(&s, &sc)) {
    free_scene(&sc);
    return 0;
  }
  if (nc != s.nc || np != s.np || no != (int)sc.no) {
    free_scene(&sc);
    return 0;
  }
  memcpy(camera_index, sc.oc, sc.no * sizeof(int));
  memcpy(point_index, sc.op, sc.no * sizeof(int));
  memcpy(observations, sc.uv, 2 * sc.no * sizeof(double));
  for (int i = 0; i < nc; ++i) memcpy(parameters + 9 * (size_t)i, sc.cams[i].cam, 9 * sizeof(double));
  memcpy(parameters + 9 * (size_t)nc, sc.pts, 3 * (size_t)np * sizeof(double));
  /* initial guess: perturbed rotation, translation, points and focal length */
  rng_t rng;
  rng_seed(&rng, s.seed ^ 0x5DEECE66DULL);
  for (int i = 0; i < nc; ++i) {
    double *c = parameters + 9 * (size_t)i;
    for (int k = 0; k < 3; ++k) c[k] += rng_normal(&rng) * s.rot_noise;
    for (int k = 3; k < 6; ++k) c[k] += rng_normal(&rng) * s.trans_noise;
    c[6] *= 1.0 + rng_normal(&rng) * s.focal_noise;
  }
  for (int j = 0; j < np; ++j)
    for (int k = 0; k < 3; ++k) parameters[9 * (size_t)nc + 3 * (size_t)j + k] += rng_normal(&rng) * s.point_noise;
  free_scene(&sc);
  return 1;
}
