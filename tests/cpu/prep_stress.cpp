// Host-logic check of prepare_batch (prep.cpp) under concurrency: the
// layout of a problem is the same bytes when prepared alone, when several
// host threads prepare at once (the pool is then busy and a prepare runs on
// its own thread), when the input observations come in another order after
// a point-major sort of the same set (the internal order depends only on
// (point, camera, input index)), and in a forked child.
// Usage: prep_stress; prints "ok" or the first failure and exits non-zero.
#include <sys/wait.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <stdexcept>
#include <cstdio>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

#include "prep.h"

using namespace gba;

struct Problem {
  std::vector<int32_t> ci, pi;
  std::vector<double> obs, par;
  gba_problem_view view() {
    return gba_problem_view{(int32_t)(par.size() - 3 * np) / 9, np, (int32_t)ci.size(), ci.data(), pi.data(),
                            obs.data(), par.data()};
  }
  int np = 0;
};

static Problem make(int nc, int np, unsigned seed, int maxv) {
  std::mt19937 rng(seed);
  Problem p;
  p.np = np;
  for (int j = 0; j < np; ++j) {
    const int m = 2 + (int)(rng() % (unsigned)(maxv - 1));
    for (int u = 0; u < m; ++u) {  // repeated cameras allowed
      p.ci.push_back((int32_t)(rng() % (unsigned)nc));
      p.pi.push_back(j);
      p.obs.push_back((double)(rng() % 1000));
      p.obs.push_back((double)(rng() % 1000));
    }
  }
  p.par.resize(9 * (size_t)nc + 3 * (size_t)np);
  for (auto &x : p.par) x = (double)(rng() % 997) * 0.01;
  return p;
}

template <typename T>
static bool eq(const std::vector<T> &a, const std::vector<T> &b) {
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}

static bool same(const HostBatch &a, const HostBatch &b) {
  bool ok = a.no == b.no && a.nchunks == b.nchunks && a.nseg == b.nseg && a.npairs == b.npairs &&
            a.nblk == b.nblk && a.explicit_schur == b.explicit_schur;
  ok = ok && eq(a.obs_cam, b.obs_cam) && eq(a.obs_pt, b.obs_pt) && eq(a.obs_uv, b.obs_uv) &&
       eq(a.obs_seg, b.obs_seg) && eq(a.obs_slot, b.obs_slot) && eq(a.pt_obs_begin, b.pt_obs_begin) &&
       eq(a.seg_cam, b.seg_cam) && eq(a.seg_pos, b.seg_pos) && eq(a.seg_slot, b.seg_slot) &&
       eq(a.cam_obs_begin, b.cam_obs_begin) && eq(a.cam_obs_list, b.cam_obs_list) &&
       eq(a.cam_piece_begin, b.cam_piece_begin) && eq(a.pt_param, b.pt_param) &&
       eq(a.cam_param, b.cam_param) && eq(a.cam_used, b.cam_used) && eq(a.pt_used, b.pt_used) &&
       eq(a.pt_orig, b.pt_orig);
  if (ok && a.explicit_schur)
    ok = eq(a.spair, b.spair) && eq(a.sblk_row, b.sblk_row) && eq(a.sblk_col, b.sblk_col) &&
         eq(a.sblk_tr, b.sblk_tr) && eq(a.sblk_up, b.sblk_up) && eq(a.sblk_pair, b.sblk_pair) &&
         eq(a.obs_fpos, b.obs_fpos);
  return ok;
}

int main() {
  // one large problem (parallel paths), a batch of small ones, a shuffled copy
  std::vector<Problem> big{make(120, 30000, 7, 8)};
  std::vector<Problem> batch;
  for (int i = 0; i < 24; ++i) batch.push_back(make(5 + i % 7, 300 + 37 * i, 100 + i, 5));
  Problem shuf = big[0];
  {
    std::mt19937 rng(3);
    std::vector<size_t> perm(shuf.ci.size());
    for (size_t i = 0; i < perm.size(); ++i) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), rng);
    std::vector<int32_t> ci(perm.size()), pi(perm.size());
    std::vector<double> ob(2 * perm.size());
    for (size_t i = 0; i < perm.size(); ++i) {
      ci[i] = big[0].ci[perm[i]], pi[i] = big[0].pi[perm[i]];
      ob[2 * i] = big[0].obs[2 * perm[i]], ob[2 * i + 1] = big[0].obs[2 * perm[i] + 1];
    }
    shuf.ci = ci, shuf.pi = pi, shuf.obs = ob;
  }
  std::vector<std::vector<gba_problem_view>> sets(2);
  sets[0].push_back(big[0].view());
  for (auto &p : batch) sets[1].push_back(p.view());
  PrepOptions po;
  po.schur = GBA_SCHUR_EXPLICIT;
  std::string err;
  std::vector<HostBatch> ref(2);
  for (int s = 0; s < 2; ++s)
    if (prepare_batch(sets[s].data(), (int)sets[s].size(), po, &ref[s], &err) != GBA_OK) {
      printf("prepare failed: %s\n", err.c_str());
      return 1;
    }
  // the shuffled input: same (point, camera) multiset, so the same camera and
  // point sequences and structure counts
  {
    HostBatch hs;
    gba_problem_view v = shuf.view();
    if (prepare_batch(&v, 1, po, &hs, &err) != GBA_OK || !eq(hs.obs_cam, ref[0].obs_cam) ||
        !eq(hs.obs_pt, ref[0].obs_pt) || !eq(hs.spair, ref[0].spair) || hs.nseg != ref[0].nseg) {
      printf("shuffled input: different internal layout\n");
      return 1;
    }
  }
  int fails = 0;
  std::vector<std::thread> th;
  std::vector<int> f(6, 0);
  for (int t = 0; t < 6; ++t)
    th.emplace_back([&, t] {
      HostBatch hb;
      std::string e;
      for (int r = 0; r < 8; ++r) {
        const int s = (t + r) % 2;
        if (prepare_batch(sets[s].data(), (int)sets[s].size(), po, &hb, &e) != GBA_OK || !same(hb, ref[s])) ++f[t];
      }
    });
  for (auto &x : th) x.join();
  for (int x : f) fails += x;
  if (fails) {
    printf("concurrent prepares: %d differ\n", fails);
    return 1;
  }
  // a task that throws: the loop's other tasks stop early, run() rethrows
  // once every worker has left, and the pool keeps working afterwards
  {
    std::atomic<int> ran{0};
    bool caught = false;
    try {
      gba::host_parallel(64, [&](int t) {
        ran.fetch_add(1);
        if (t == 3) throw std::runtime_error("task 3");
      });
    } catch (const std::runtime_error &) {
      caught = true;
    }
    std::atomic<int> after{0};
    gba::host_parallel(64, [&](int) { after.fetch_add(1); });
    if (!caught || ran.load() < 1 || after.load() != 64) {
      printf("pool exception: caught %d ran %d after %d\n", (int)caught, ran.load(), after.load());
      return 1;
    }
  }
  const pid_t pid = fork();
  if (pid == 0) {
    HostBatch hb;
    std::string e;
    int bad = 0;
    for (int s = 0; s < 2; ++s)
      if (prepare_batch(sets[s].data(), (int)sets[s].size(), po, &hb, &e) != GBA_OK || !same(hb, ref[s])) ++bad;
    exit(bad ? 1 : 0);  // through the static destructors: the pool holds no threads here
  }
  int status = 0;
  if (pid < 0 || waitpid(pid, &status, 0) != pid || !WIFEXITED(status) || WEXITSTATUS(status) != 0) {
    printf("forked child failed\n");
    return 1;
  }
  printf("ok\n");
  return 0;
}
