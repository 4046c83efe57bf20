// prep.cpp — host-side layout of a batch of BAL problems.
//
// Input: the BALProblem arrays of each problem (utils/datasets/BALProblem.h:
// 109-118), in any observation order.  Output: observations sorted by
// (internal point, camera, input index) — point-major as BAL files usually
// are (data/bal/ladybug49.txt) — with every point's observations contiguous;
// chunks of whole points; per chunk the camera-sorted order of its
// observations and its camera segments; per camera its segments and its
// observations.  All orderings are deterministic functions of the input.
#include "prep.h"

#include <functional>
#include <thread>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace gba {

static std::string fmt(const char *f, long long a, long long b = 0, long long c = 0) {
  char buf[256];
  std::snprintf(buf, sizeof buf, f, a, b, c);
  return buf;
}

gba_status validate_problem(const gba_problem_view *v, std::string *err) {
  if (!v) {
    *err = "null problem view";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  if (v->num_cameras < 0 || v->num_points < 0 || v->num_observations < 0) {
    *err = "negative problem size";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  if (v->num_observations > 0 &&
      (!v->camera_index || !v->point_index || !v->observations))
    return *err = "null observation array", GBA_ERR_INVALID_ARGUMENT;
  if ((v->num_cameras > 0 || v->num_points > 0) && !v->parameters)
    return *err = "null parameter array", GBA_ERR_INVALID_ARGUMENT;
  const int nc = v->num_cameras, np = v->num_points;
  for (int i = 0; i < v->num_observations; ++i) {
    const int c = v->camera_index[i], p = v->point_index[i];
    if (c < 0 || c >= nc) {
      *err = fmt("observation %lld: camera index %lld out of range [0, %lld)", i, c, nc);
      return GBA_ERR_INVALID_ARGUMENT;
    }
    if (p < 0 || p >= np) {
      *err = fmt("observation %lld: point index %lld out of range [0, %lld)", i, p, np);
      return GBA_ERR_INVALID_ARGUMENT;
    }
    if (!std::isfinite(v->observations[2 * i]) || !std::isfinite(v->observations[2 * i + 1])) {
      *err = fmt("observation %lld is not finite", i);
      return GBA_ERR_NON_FINITE;
    }
  }
  const long long npar = 9LL * nc + 3LL * np;
  for (long long k = 0; k < npar; ++k)
    if (!std::isfinite(v->parameters[k])) {
      *err = fmt("parameter %lld is not finite", k);
      return GBA_ERR_NON_FINITE;
    }
  return GBA_OK;
}

// Runs fn(begin, end) over [0, n) in runs on host threads (one run when n
// is small); fn must write disjoint outputs per index.
static void parallel_runs(long long n, long long min_per_thread, const std::function<void(long long, long long)> &fn) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const long long nth = std::min<long long>(std::min(hw, 32u), std::max<long long>(1, n / std::max(1LL, min_per_thread)));
  if (nth <= 1) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  for (long long w = 0; w < nth; ++w) th.emplace_back([&, w] { fn(n * w / nth, n * (w + 1) / nth); });
  for (auto &x : th) x.join();
}

// The explicit Schur complement's structure, row camera by row camera: the
// row's co-visible cameras (sorted; the row's own camera when it observes a
// point more than once), the transpose of every block, and for the blocks
// on and above the diagonal (column camera >= row camera: the formation
// kernel forms those and writes each transpose) the ordered observation
// pairs (a of the row camera, b of the column camera, a != b, same point;
// stored as the two observations' camera-major positions) in point order,
// so the formation sums have a fixed order.  A camera's observations
// (cam_obs_list) are in point order, so walking them and each point's
// observations lists every block's pairs in that order.  O(pairs) with a
// per-row lookup table; the rows are independent, so host threads take runs
// of rows (the result does not depend on the thread count).
static void build_schur_structure(HostBatch *hbp) {
  HostBatch &hb = *hbp;
  const int nc = hb.nc;
  // F rows are stored camera-major (a camera's observations together, in
  // point order): the pairs of a block read two cameras' runs of rows
  hb.obs_fpos.resize(hb.no);
  for (int i = 0; i < hb.no; ++i) hb.obs_fpos[hb.cam_obs_list[i]] = i;
  std::vector<std::vector<int32_t>> rows(nc), cnts(nc);  // per row: columns; pair counts of its upper blocks
  std::vector<int32_t> first_up(nc, 0);                  // per row: index of its first column >= the row
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nth = (int)std::min<long long>(std::min(hw, 32u), std::max<long long>(1, (long long)hb.no / 20000));
  auto for_rows = [&](const std::function<void(int, int, std::vector<int32_t> &, std::vector<int32_t> &)> &fn) {
    std::vector<std::thread> th;
    for (int w = 0; w < nth; ++w) {
      const int c0 = (int)((long long)nc * w / nth), c1 = (int)((long long)nc * (w + 1) / nth);
      th.emplace_back([&, c0, c1] {
        std::vector<int32_t> mark(nc, -1), pos(nc, 0);
        fn(c0, c1, mark, pos);
      });
    }
    for (auto &x : th) x.join();
  };
  // 1. per row: sorted co-visible cameras, pair counts of the upper blocks
  for_rows([&](int c0, int c1, std::vector<int32_t> &mark, std::vector<int32_t> &pos) {
    for (int c = c0; c < c1; ++c) {
      const int a0 = hb.cam_obs_begin[c], a1 = hb.cam_obs_begin[c + 1];
      std::vector<int32_t> &row = rows[c];
      for (int ia = a0; ia < a1; ++ia) {
        const int a = hb.cam_obs_list[ia], j = hb.obs_pt[a];
        for (int b = hb.pt_obs_begin[j]; b < hb.pt_obs_begin[j + 1]; ++b) {
          const int k = hb.obs_cam[b];
          if (b != a && mark[k] != c) mark[k] = c, row.push_back(k);
        }
      }
      std::sort(row.begin(), row.end());
      const int nb = (int)row.size();
      const int u0 = (int)(std::lower_bound(row.begin(), row.end(), c) - row.begin());
      first_up[c] = u0;
      std::vector<int32_t> &cnt = cnts[c];
      cnt.assign(nb - u0, 0);
      for (int u = u0; u < nb; ++u) pos[row[u]] = u - u0;
      for (int ia = a0; ia < a1; ++ia) {
        const int a = hb.cam_obs_list[ia], j = hb.obs_pt[a];
        for (int b = hb.pt_obs_begin[j]; b < hb.pt_obs_begin[j + 1]; ++b)
          if (b != a && hb.obs_cam[b] >= c) ++cnt[pos[hb.obs_cam[b]]];
      }
    }
  });
  // 2. prefix sums: the CSR, the upper blocks, their pair ranges
  hb.sblk_row.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) hb.sblk_row[c + 1] = hb.sblk_row[c] + (int32_t)rows[c].size();
  hb.nblk = hb.sblk_row[nc];
  hb.sblk_col.resize(hb.nblk);
  hb.sblk_up.clear();
  hb.sblk_pair.assign(1, 0);
  std::vector<long long> up_begin(nc + 1, 0);  // per row: its first upper block (index into sblk_up)
  for (int c = 0; c < nc; ++c) {
    std::copy(rows[c].begin(), rows[c].end(), hb.sblk_col.begin() + hb.sblk_row[c]);
    up_begin[c] = (long long)hb.sblk_up.size();
    for (size_t u = 0; u < cnts[c].size(); ++u) {
      hb.sblk_up.push_back(hb.sblk_row[c] + first_up[c] + (int32_t)u);
      hb.sblk_pair.push_back(hb.sblk_pair.back() + cnts[c][u]);
    }
  }
  up_begin[nc] = (long long)hb.sblk_up.size();
  hb.nup = (long long)hb.sblk_up.size();
  hb.npairs = hb.sblk_pair.back();
  hb.spair.resize(2 * (size_t)hb.npairs);
  // 3. the pairs, in point order per block
  for_rows([&](int c0, int c1, std::vector<int32_t> &mark, std::vector<int32_t> &pos) {
    (void)mark;
    std::vector<int32_t> next;
    for (int c = c0; c < c1; ++c) {
      const std::vector<int32_t> &row = rows[c];
      const int u0 = first_up[c], nu = (int)row.size() - u0;
      next.resize(nu);
      for (int u = 0; u < nu; ++u) {
        pos[row[u0 + u]] = u;
        next[u] = hb.sblk_pair[up_begin[c] + u];
      }
      for (int ia = hb.cam_obs_begin[c]; ia < hb.cam_obs_begin[c + 1]; ++ia) {
        const int a = hb.cam_obs_list[ia], j = hb.obs_pt[a];
        for (int b = hb.pt_obs_begin[j]; b < hb.pt_obs_begin[j + 1]; ++b)
          if (b != a && hb.obs_cam[b] >= c) {
            const size_t k = (size_t)next[pos[hb.obs_cam[b]]]++;
            hb.spair[2 * k] = hb.obs_fpos[a];
            hb.spair[2 * k + 1] = hb.obs_fpos[b];
          }
      }
    }
  });
  // 4. the transpose of block (c, k) is block (k, c), in row k
  hb.sblk_tr.resize(hb.nblk);
  for_rows([&](int c0, int c1, std::vector<int32_t> &, std::vector<int32_t> &) {
    for (int c = c0; c < c1; ++c)
      for (int e = hb.sblk_row[c]; e < hb.sblk_row[c + 1]; ++e) {
        const int k = hb.sblk_col[e];
        const auto b0 = hb.sblk_col.begin() + hb.sblk_row[k], b1 = hb.sblk_col.begin() + hb.sblk_row[k + 1];
        hb.sblk_tr[e] = (int32_t)(std::lower_bound(b0, b1, c) - hb.sblk_col.begin());
      }
  });
}

void HostBatch::reset() {
  P = nc = np = no = nchunks = nseg = cam_blocks = 0;
  explicit_schur = false;
  nblk = nup = npairs = 0;
  for (auto *v : {&obs_cam, &obs_pt, &pt_obs_begin, &pt_problem, &cam_problem, &seg_cam, &cam_seg_begin, &seg_slot,
                  &cam_obs_begin, &cam_obs_list, &sblk_row, &sblk_col, &sblk_tr, &sblk_up, &sblk_pair, &spair,
                  &obs_fpos, &obs_orig, &pt_orig})
    v->clear();
  for (auto *v : {&obs_seg, &obs_slot, &seg_pos}) v->clear();
  for (auto *v : {&obs_uv, &cam_param, &pt_param}) v->clear();
  pt_used.clear();
  cam_used.clear();
  obs_rig.clear();
  prob_rig.clear();
  prob.clear();
  chunk.clear();
  camblk.clear();
}

gba_status prepare_batch(const gba_problem_view *views, int n, const PrepOptions &opt, HostBatch *out,
                         std::string *err) {
  HostBatch &hb = *out;
  hb.reset();
  if (n <= 0 || !views) {
    *err = "empty batch";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  const int cap = opt.chunk_cap;
  long long tc = 0, tp = 0, to = 0;
  for (int p = 0; p < n; ++p) {
    const gba_status st = validate_problem(&views[p], err);
    if (st != GBA_OK) {
      if (n > 1) *err = fmt("problem %lld: ", p) + *err;
      return st;
    }
    tc += views[p].num_cameras;
    tp += views[p].num_points;
    to += views[p].num_observations;
  }
  if (tc > (1LL << 30) || tp > (1LL << 30) || to > (1LL << 30)) {
    *err = "batch too large for 32-bit indices";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  hb.P = n;
  hb.nc = (int)tc;
  hb.np = (int)tp;
  hb.no = (int)to;
  hb.prob.resize(n);
  hb.obs_cam.resize(to);
  hb.obs_pt.resize(to);
  hb.obs_uv.resize(2 * to);
  hb.obs_seg.resize(to);
  hb.obs_slot.resize(to);
  hb.obs_orig.resize(to);
  hb.pt_obs_begin.assign(tp + 1, 0);
  hb.pt_problem.resize(tp);
  hb.cam_problem.resize(tc);
  hb.pt_used.assign(tp, 0);
  hb.cam_used.assign(tc, 0);
  hb.pt_orig.resize(tp);
  hb.cam_param.resize(9 * tc);
  hb.pt_param.assign(4 * tp, 0.0);
  hb.cam_obs_begin.assign(tc + 1, 0);
  hb.cam_obs_list.resize(to);

  int cam0 = 0, pt0 = 0, obs0 = 0;
  std::vector<int32_t> deg, key, order, inv, fill, cams;
  // per camera of the batch, for the chunks' camera-sorted orders: the
  // chunk that last saw it, its count, next position, segment
  std::vector<int32_t> cmark(tc, -1), ccount(tc), cstart(tc), cseg(tc), distinct;
  for (int p = 0; p < n; ++p) {
    const gba_problem_view &v = views[p];
    const int nc = v.num_cameras, np = v.num_points, no = v.num_observations;
    ProblemInfo &pi = hb.prob[p];
    pi.cam_begin = cam0;
    pi.cam_count = nc;
    pi.pt_begin = pt0;
    pi.pt_count = np;
    pi.obs_begin = obs0;
    pi.obs_count = no;
    pi.chunk_begin = (int)hb.chunk.size();
    pi.seg_begin = (int)hb.seg_cam.size();
    // degrees, first camera of each point
    deg.assign(np, 0);
    key.assign(np, nc);
    for (int i = 0; i < no; ++i) {
      const int c = v.camera_index[i], j = v.point_index[i];
      ++deg[j];
      if (c < key[j]) key[j] = c;
      hb.cam_used[cam0 + c] = 1;
    }
    // internal point order: by first camera (locality of the camera
    // segments in the chunk kernels), stable in the input index
    order.resize(np);
    if (opt.reorder_points) {
      fill.assign(nc + 2, 0);
      for (int j = 0; j < np; ++j) ++fill[key[j] + 1];
      for (int c = 0; c <= nc; ++c) fill[c + 1] += fill[c];
      for (int j = 0; j < np; ++j) order[fill[key[j]]++] = j;
    } else {
      for (int j = 0; j < np; ++j) order[j] = j;
    }
    inv.resize(np);
    for (int ji = 0; ji < np; ++ji) inv[order[ji]] = ji;
    // CSR by internal point, observations stable in input index
    for (int ji = 0; ji < np; ++ji) {
      const int j = order[ji];
      hb.pt_orig[pt0 + ji] = j;
      hb.pt_problem[pt0 + ji] = p;
      hb.pt_used[pt0 + ji] = deg[j] > 0;
      hb.pt_obs_begin[pt0 + ji + 1] = deg[j];
      for (int q = 0; q < 3; ++q) hb.pt_param[4 * (size_t)(pt0 + ji) + q] = v.parameters[9 * (size_t)nc + 3 * (size_t)j + q];
    }
    hb.pt_obs_begin[pt0] = obs0;
    for (int ji = 0; ji < np; ++ji) hb.pt_obs_begin[pt0 + ji + 1] += hb.pt_obs_begin[pt0 + ji];
    fill.assign(hb.pt_obs_begin.begin() + pt0, hb.pt_obs_begin.begin() + pt0 + np + 1);
    for (int i = 0; i < no; ++i) hb.obs_orig[fill[inv[v.point_index[i]]]++] = i;
    // within a point: by camera, then input index (insertion sort, stable);
    // points and observations are independent (host threads)
    parallel_runs(np, 20000, [&](long long j0, long long j1) {
      for (int ji = (int)j0; ji < (int)j1; ++ji) {
        const int b = hb.pt_obs_begin[pt0 + ji], e = hb.pt_obs_begin[pt0 + ji + 1];
        for (int k = b + 1; k < e; ++k) {
          const int x = hb.obs_orig[k];
          const int cx = v.camera_index[x];
          int m = k - 1;
          while (m >= b && v.camera_index[hb.obs_orig[m]] > cx) {
            hb.obs_orig[m + 1] = hb.obs_orig[m];
            --m;
          }
          hb.obs_orig[m + 1] = x;
        }
      }
    });
    parallel_runs(no, 50000, [&](long long k0, long long k1) {
      for (int k = obs0 + (int)k0; k < obs0 + (int)k1; ++k) {
        const int i = hb.obs_orig[k];
        hb.obs_cam[k] = cam0 + v.camera_index[i];
        hb.obs_pt[k] = pt0 + inv[v.point_index[i]];
        hb.obs_uv[2 * (size_t)k] = v.observations[2 * (size_t)i];
        hb.obs_uv[2 * (size_t)k + 1] = v.observations[2 * (size_t)i + 1];
      }
    });
    for (int c = 0; c < nc; ++c) {
      hb.cam_problem[cam0 + c] = p;
      for (int q = 0; q < 9; ++q) hb.cam_param[9 * (size_t)(cam0 + c) + q] = v.parameters[9 * (size_t)c + q];
    }
    // chunks of whole points
    int ji = 0;
    while (ji < np) {
      ChunkInfo ci;
      std::memset(&ci, 0, sizeof ci);
      ci.problem = p;
      ci.pt_begin = pt0 + ji;
      ci.obs_begin = hb.pt_obs_begin[pt0 + ji];
      int nobs = 0, npts = 0;
      while (ji < np && npts < cap) {
        const int d = hb.pt_obs_begin[pt0 + ji + 1] - hb.pt_obs_begin[pt0 + ji];
        if (d > cap) {
          *err = fmt("point %lld is observed %lld times; at most %lld observations per point are supported",
                     order[ji], d, cap);
          return GBA_ERR_INVALID_ARGUMENT;
        }
        if (nobs + d > cap) break;
        nobs += d;
        ++npts;
        ++ji;
      }
      ci.obs_count = nobs;
      ci.pt_count = npts;
      // camera-sorted order of the chunk's observations, stable: the
      // chunk's distinct cameras (a stamped table), sorted, then each
      // observation's position from its camera's running count
      const int stamp = (int)hb.chunk.size();
      distinct.clear();
      for (int k = 0; k < nobs; ++k) {
        const int cam = hb.obs_cam[ci.obs_begin + k];
        if (cmark[cam] != stamp) cmark[cam] = stamp, ccount[cam] = 0, distinct.push_back(cam);
        ++ccount[cam];
      }
      std::sort(distinct.begin(), distinct.end());
      ci.seg_begin = (int)hb.seg_cam.size();
      const int segs = (int)distinct.size();
      for (int sg = 0, pos = 0; sg < segs; ++sg) {
        const int cam = distinct[sg];
        hb.seg_pos.push_back((uint16_t)pos);
        hb.seg_cam.push_back(cam);
        cstart[cam] = pos;
        cseg[cam] = sg;
        pos += ccount[cam];
      }
      for (int k = 0; k < nobs; ++k) {
        const int cam = hb.obs_cam[ci.obs_begin + k];
        hb.obs_slot[ci.obs_begin + k] = (uint16_t)cstart[cam]++;
        hb.obs_seg[ci.obs_begin + k] = (uint16_t)cseg[cam];
      }
      ci.seg_count = segs;
      hb.chunk.push_back(ci);
    }
    pi.chunk_count = (int)hb.chunk.size() - pi.chunk_begin;
    pi.seg_count = (int)hb.seg_cam.size() - pi.seg_begin;
    // camera blocks of the PCG kernels
    pi.cam_block_begin = (int)hb.camblk.size();
    for (int c = 0; c < nc; c += kPcgBlockCams) {
      int4 b;
      b.x = p;
      b.y = cam0 + c;
      b.z = std::min(kPcgBlockCams, nc - c);
      b.w = 0;
      hb.camblk.push_back(b);
    }
    pi.cam_block_count = (int)hb.camblk.size() - pi.cam_block_begin;
    cam0 += nc;
    pt0 += np;
    obs0 += no;
  }
  hb.nchunks = (int)hb.chunk.size();
  hb.nseg = (int)hb.seg_cam.size();
  hb.cam_blocks = (int)hb.camblk.size();
  // per camera: its segments (chunk order) and its observations (internal order)
  hb.cam_seg_begin.assign(hb.nc + 1, 0);
  for (int s = 0; s < hb.nseg; ++s) ++hb.cam_seg_begin[hb.seg_cam[s] + 1];
  for (int c = 0; c < hb.nc; ++c) hb.cam_seg_begin[c + 1] += hb.cam_seg_begin[c];
  // each segment's partial goes to its camera-major position, so a camera's
  // partials are contiguous for the camera reduce
  hb.seg_slot.resize(hb.nseg);
  fill.assign(hb.cam_seg_begin.begin(), hb.cam_seg_begin.end());
  for (int s = 0; s < hb.nseg; ++s) hb.seg_slot[s] = fill[hb.seg_cam[s]]++;
  // explicit Schur complement: chosen by the option, AUTO when a point's
  // ordered observation pairs (sum over points of m (m - 1)) are at most
  // kExplicitPairsPerObs per observation (forming S then costs less than the
  // implicit mat-vec saves over a PCG solve)
  {
    long long pairs = 0;
    for (int j = 0; j < hb.np; ++j) {
      const long long m = hb.pt_obs_begin[j + 1] - hb.pt_obs_begin[j];
      pairs += m * (m - 1);
    }
    hb.explicit_schur = opt.schur == GBA_SCHUR_EXPLICIT ||
                        (opt.schur == GBA_SCHUR_AUTO && pairs <= kExplicitPairsPerObs * (long long)hb.no);
    if (hb.explicit_schur && pairs > kExplicitPairsMax) {
      *err = fmt("the explicit Schur complement needs %lld observation pairs; at most %lld are supported", pairs,
                 (long long)kExplicitPairsMax);
      return GBA_ERR_INVALID_ARGUMENT;
    }
  }
  for (int k = 0; k < hb.no; ++k) ++hb.cam_obs_begin[hb.obs_cam[k] + 1];
  for (int c = 0; c < hb.nc; ++c) hb.cam_obs_begin[c + 1] += hb.cam_obs_begin[c];
  fill.assign(hb.cam_obs_begin.begin(), hb.cam_obs_begin.end());
  for (int k = 0; k < hb.no; ++k) hb.cam_obs_list[fill[hb.obs_cam[k]]++] = k;
  if (hb.explicit_schur) build_schur_structure(&hb);
  return GBA_OK;
}

void scatter_parameters(const HostBatch &hb, int p, const double *cam_param, const double *pt_param,
                        double *out) {
  const ProblemInfo &pi = hb.prob[p];
  std::memcpy(out, cam_param + 9 * (size_t)pi.cam_begin, sizeof(double) * 9 * (size_t)pi.cam_count);
  double *pts = out + 9 * (size_t)pi.cam_count;
  for (int ji = 0; ji < pi.pt_count; ++ji) {
    const int j = hb.pt_orig[pi.pt_begin + ji];
    for (int q = 0; q < 3; ++q) pts[3 * (size_t)j + q] = pt_param[4 * (size_t)(pi.pt_begin + ji) + q];
  }
}

}  // namespace gba
