// Host-logic check of prepare_batch (prep.cpp) against brute force:
//  - the explicit Schur complement's structure: every co-visible camera
//    pair is a block, each block's transpose, the blocks on and above the
//    diagonal with their observation pairs (camera-major F positions) in
//    point order;
//  - each chunk's camera-sorted observation order is stable and its
//    segments are the chunk's distinct cameras in increasing order;
//  - each camera's observation list in pieces of kCamPieceObs (at least
//    one piece a camera);
//  - a resumed problem's state: the Jacobi scales gathered to user order
//    and set back into a batch land where they were (set_resume inverts
//    gather_scales), the LM state carried.
// Usage: check_prep <num_cameras> <num_points> <seed>; prints "ok" or the
// first mismatch and exits non-zero.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <vector>

#include "prep.h"

using namespace gba;

int main(int argc, char **argv) {
  const int nc = argc > 1 ? atoi(argv[1]) : 9, np = argc > 2 ? atoi(argv[2]) : 60;
  std::mt19937 rng(argc > 3 ? atoi(argv[3]) : 1);
  std::vector<int32_t> ci, pi;
  std::vector<double> obs;
  for (int j = 0; j < np; ++j) {
    const int m = 2 + (int)(rng() % 5);
    for (int u = 0; u < m; ++u) {  // cameras drawn with repetition: some points seen twice by a camera
      ci.push_back((int32_t)(rng() % nc));
      pi.push_back(j);
      obs.push_back(1.0);
      obs.push_back(2.0);
    }
  }
  std::vector<double> par(9 * (size_t)nc + 3 * (size_t)np, 0.1);
  gba_problem_view v{};
  v.num_cameras = nc;
  v.num_points = np;
  v.num_observations = (int)ci.size();
  v.camera_index = ci.data();
  v.point_index = pi.data();
  v.observations = obs.data();
  v.parameters = par.data();
  PrepOptions po;
  po.schur = GBA_SCHUR_EXPLICIT;
  HostBatch hb;
  std::string err;
  for (int pass = 0; pass < 2; ++pass) {  // the second pass reuses the batch's storage
    if (prepare_batch(&v, 1, po, &hb, &err) != GBA_OK) {
      printf("prepare_batch failed: %s\n", err.c_str());
      return 1;
    }
  }
  // structure
  std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> ref;
  for (int j = 0; j < hb.np; ++j)
    for (int a = hb.pt_obs_begin[j]; a < hb.pt_obs_begin[j + 1]; ++a)
      for (int b = hb.pt_obs_begin[j]; b < hb.pt_obs_begin[j + 1]; ++b)
        if (a != b) ref[{hb.obs_cam[a], hb.obs_cam[b]}].push_back({a, b});
  if ((long long)ref.size() != hb.nblk) {
    printf("block count %zu vs %lld\n", ref.size(), hb.nblk);
    return 1;
  }
  long long nup = 0, npairs = 0;
  for (auto &kv : ref)
    if (kv.first.second >= kv.first.first) ++nup, npairs += (long long)kv.second.size();
  if (nup != hb.nup || npairs != hb.npairs) {
    printf("upper blocks %lld/%lld pairs %lld/%lld\n", nup, hb.nup, npairs, hb.npairs);
    return 1;
  }
  for (int c = 0; c < hb.nc; ++c)
    for (int e = hb.sblk_row[c]; e < hb.sblk_row[c + 1]; ++e) {
      const int k = hb.sblk_col[e], tr = hb.sblk_tr[e];
      if (!ref.count({c, k}) || (e > hb.sblk_row[c] && k <= hb.sblk_col[e - 1]) || tr < hb.sblk_row[k] ||
          tr >= hb.sblk_row[k + 1] || hb.sblk_col[tr] != c) {
        printf("row %d block %d\n", c, e);
        return 1;
      }
    }
  for (long long u = 0; u < hb.nup; ++u) {
    const int e = hb.sblk_up[u];
    const int c = (int)(std::upper_bound(hb.sblk_row.begin(), hb.sblk_row.end(), e) - hb.sblk_row.begin()) - 1;
    const auto &r = ref[{c, hb.sblk_col[e]}];
    if (hb.sblk_col[e] < c || (int)r.size() != hb.sblk_pair[u + 1] - hb.sblk_pair[u]) {
      printf("upper block %lld\n", u);
      return 1;
    }
    for (size_t w = 0; w < r.size(); ++w) {
      const size_t q = (size_t)hb.sblk_pair[u] + w;
      if (hb.spair[2 * q] != hb.obs_fpos[r[w].first] || hb.spair[2 * q + 1] != hb.obs_fpos[r[w].second]) {
        printf("pair %zu of upper block %lld\n", w, u);
        return 1;
      }
    }
  }
  // chunks: stable camera-sorted order and segments
  for (int ch = 0; ch < hb.nchunks; ++ch) {
    const ChunkInfo &k = hb.chunk[ch];
    std::vector<std::pair<int, int>> ord(k.obs_count);
    for (int i = 0; i < k.obs_count; ++i) ord[i] = {hb.obs_cam[k.obs_begin + i], i};
    std::stable_sort(ord.begin(), ord.end(), [](auto &a, auto &b) { return a.first < b.first; });
    for (int pos = 0; pos < k.obs_count; ++pos)
      if (hb.obs_slot[k.obs_begin + ord[pos].second] != pos) {
        printf("chunk %d slot %d\n", ch, pos);
        return 1;
      }
    int sg = -1;
    for (int pos = 0; pos < k.obs_count; ++pos) {
      if (pos == 0 || ord[pos].first != ord[pos - 1].first) {
        ++sg;
        if (hb.seg_cam[k.seg_begin + sg] != ord[pos].first || hb.seg_pos[k.seg_begin + sg] != pos) {
          printf("chunk %d segment %d\n", ch, sg);
          return 1;
        }
      }
      if (hb.obs_seg[k.obs_begin + ord[pos].second] != sg) {
        printf("chunk %d observation segment\n", ch);
        return 1;
      }
    }
    if (sg + 1 != k.seg_count) {
      printf("chunk %d segment count\n", ch);
      return 1;
    }
  }
  // pieces of the cameras' observation lists
  if ((int)hb.cam_piece_begin.size() != hb.nc + 1 || hb.cam_piece_begin[0] != 0) {
    printf("piece table size\n");
    return 1;
  }
  for (int c = 0; c < hb.nc; ++c) {
    const int n = hb.cam_obs_begin[c + 1] - hb.cam_obs_begin[c];
    const int want = std::max(1, (n + kCamPieceObs - 1) / kCamPieceObs);
    if (hb.cam_piece_begin[c + 1] - hb.cam_piece_begin[c] != want) {
      printf("camera %d pieces\n", c);
      return 1;
    }
  }
  // resume: gather_scales then set_resume is the identity on the scales
  {
    std::vector<double> cs(9 * (size_t)hb.nc), ps(3 * (size_t)hb.np);
    for (size_t i = 0; i < cs.size(); ++i) cs[i] = 1.0 + 0.001 * (double)i;
    for (size_t i = 0; i < ps.size(); ++i) ps[i] = 2.0 + 0.001 * (double)i;
    ProblemState st;
    gather_scales(hb, 0, cs.data(), ps.data(), &st);
    st.lm.iteration = 7;
    st.lm.radius = 123.5;
    set_resume(hb, 0, st);
    if (hb.resume.size() != 1 || hb.resume[0] != 1 || hb.resume_lm[0].iteration != 7 ||
        hb.resume_lm[0].radius != 123.5 || hb.resume_cam_scale != cs || hb.resume_pt_scale != ps) {
      printf("resume round trip\n");
      return 1;
    }
    // user order: point j of the input is internal point inv(j)
    for (int ji = 0; ji < hb.np; ++ji)
      for (int q = 0; q < 3; ++q)
        if (st.pt_scale[3 * (size_t)hb.pt_orig[ji] + q] != ps[3 * (size_t)ji + q]) {
          printf("resume point order\n");
          return 1;
        }
  }
  printf("ok nblk %lld nup %lld npairs %lld chunks %d\n", hb.nblk, hb.nup, hb.npairs, hb.nchunks);
  return 0;
}
