// engine.cpp — device workspace, uploads, the LM loop as one CUDA graph
// (conditional WHILE nodes for the LM loop and the nested PCG loop, set from
// the kernels themselves), a host-driven variant with per-kernel event
// timing, and result download.
#include "engine.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "kernels.h"

namespace gba {

cudaError_t probe_kernel_image();
void launch_cost_only(const DeviceBatch &b, cudaStream_t s);

namespace {

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Carver {
  char *base;
  size_t off;
  template <typename T>
  T *take(size_t n) {
    off = align_up(off, 256);
    T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
    off += n * sizeof(T);
    return p;
  }
};

enum ProfSlot {
  PF_EVAL = 0,
  PF_POST,
  PF_POINT,
  PF_SCHUR,
  PF_MATVEC,
  PF_PCGCAM,
  PF_BACKSUB,
  PF_CANDIDATE,
  PF_DECIDE,
  PF_TABLE,
  PF_SETUP_MISC,
  PF_FORM,
  PF_CLUSTER,
  PF_GRID,
  PF_COUNT
};
const char *kProfNames[PF_COUNT] = {"eval_jacobian",  "post_eval", "point_schur",  "camera_schur",
                                    "schur_matvec",   "pcg_camera", "back_substitute", "candidate_cost",
                                    "decide",         "camera_table", "setup_misc", "schur_form",
                                    "pcg_cluster",    "pcg_grid"};

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

Engine::Engine(const gba_options &o) : o_(o) {
  mixed_ = o.precision == GBA_PRECISION_MIXED;
  device_ = o.device;
  trace_cap_ = std::max(1, max_lm_bodies() + 1);
  profile_.resize(PF_COUNT);
  for (int i = 0; i < PF_COUNT; ++i) profile_[i].name = kProfNames[i];
}

Engine::~Engine() {
  cudaSetDevice(device_);
  destroy_graph();
  if (d_arena_) cudaFree(d_arena_);
  if (h_stage_) cudaFreeHost(h_stage_);
  for (cudaStream_t &s : cap_)
    if (s) cudaStreamDestroy(s);
  if (own_stream_ && stream_) cudaStreamDestroy(stream_);
  for (cudaEvent_t e : {ev_start_, ev_stop_, pev_[0], pev_[1]})
    if (e) cudaEventDestroy(e);
}

gba_status Engine::check(cudaError_t e, const char *what, std::string *err) {
  if (e == cudaSuccess) return GBA_OK;
  *err = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return GBA_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice ||
      e == cudaErrorInvalidDevice)
    return GBA_ERR_NO_DEVICE;
  return GBA_ERR_CUDA;
}

gba_status Engine::init(std::string *err) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    *err = "no CUDA device available";
    return GBA_ERR_NO_DEVICE;
  }
  if (device_ < 0 || device_ >= n) {
    *err = "device ordinal out of range";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  gba_status st;
  if ((st = check(cudaSetDevice(device_), "cudaSetDevice", err)) != GBA_OK) return st;
  {
    const char *e = std::getenv("GBA_TEST_GRID_WAIT");
    grid_wait_test_ = e && e[0] == '1';
  }
  if ((st = check(probe_kernel_image(), "loading the sm_103a kernels", err)) != GBA_OK) return st;
  if (o_.stream) {
    stream_ = static_cast<cudaStream_t>(o_.stream);
  } else {
    if ((st = check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream", err)) != GBA_OK) return st;
    own_stream_ = true;
  }
  for (cudaStream_t &s : cap_)
    if ((st = check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream", err)) != GBA_OK) return st;
  for (cudaEvent_t *e : {&ev_start_, &ev_stop_, &pev_[0], &pev_[1]})
    if ((st = check(cudaEventCreate(e), "event", err)) != GBA_OK) return st;
  if ((st = check(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_), "SM count", err)) !=
      GBA_OK)
    return st;
  point_schur_init();
  pcg_init();
  return GBA_OK;
}

PrepOptions Engine::prep_options() const {
  PrepOptions po;
  po.reorder_points = o_.reorder_points != 0;
  if (o_.chunk_observations > 0) po.chunk_cap = std::max(32, std::min(kChunkCap, (int)o_.chunk_observations));
  po.schur = o_.schur;
  return po;
}

void Engine::set_tuning(int chunk_observations, int pcg_unroll, int cluster_cams, int pcg_cap, int grid_ctas) {
  o_.chunk_observations = chunk_observations;
  o_.pcg_unroll = pcg_unroll;
  cluster_cams_ = std::max(0, cluster_cams);
  grid_ctas_ = std::max(0, grid_ctas);
  if (pcg_cap > 0) o_.max_linear_solver_iterations = pcg_cap;
  destroy_graph();
  cur_key_.clear();
}

// Arena order: [upload | download | work].  The pinned host staging buffer
// mirrors [upload | download] at the same offsets, so one H2D copy uploads
// a whole batch and one D2H copy returns its results.
size_t Engine::layout(const HostBatch &hb, char *base, DeviceBatch *db, size_t *upload_bytes,
                      size_t *download_off, size_t *download_bytes) {
  Carver cv{base, 0};
  DeviceBatch &b = *db;
  const size_t P = hb.P, nc = hb.nc, np = hb.np, no = hb.no, nch = hb.nchunks, ns = hb.nseg;
  const size_t nb = hb.cam_blocks;
  b.num_problems = hb.P;
  b.nc = hb.nc;
  b.np = hb.np;
  b.no = hb.no;
  b.nchunks = hb.nchunks;
  b.nseg = hb.nseg;
  b.cam_blocks = hb.cam_blocks;
  // upload
  b.prob = cv.take<ProblemInfo>(P);
  b.chunk = cv.take<ChunkInfo>(nch);
  b.obs_cam = cv.take<int32_t>(no);
  b.obs_pt = cv.take<int32_t>(no);
  b.obs_uv = cv.take<double2>(no);
  b.obs_seg = cv.take<uint16_t>(no);
  b.obs_slot = cv.take<uint16_t>(no);
  b.pt_obs_begin = cv.take<int32_t>(np + 1);
  b.pt_problem = cv.take<int32_t>(np);
  b.cam_problem = cv.take<int32_t>(nc);
  b.pt_used = cv.take<uint8_t>(np);
  b.cam_used = cv.take<uint8_t>(nc);
  b.seg_pos = cv.take<uint16_t>(ns);
  b.seg_cam = cv.take<int32_t>(ns);
  b.cam_seg_begin = cv.take<int32_t>(nc + 1);
  b.seg_slot = cv.take<int32_t>(ns);
  b.cam_obs_begin = cv.take<int32_t>(nc + 1);
  b.cam_obs_list = cv.take<int32_t>(no);
  const int npieces = hb.cam_piece_begin.empty() ? 0 : hb.cam_piece_begin.back();
  b.cam_piece_begin = cv.take<int32_t>(hb.cam_piece_begin.size());
  b.npieces = npieces;
  b.camblk = cv.take<int4>(nb);
  b.cam_init = cv.take<double>(9 * nc);
  b.pt_init = cv.take<double>(4 * np);
  const bool ex = hb.explicit_schur;
  const size_t nsb = ex ? (size_t)hb.nblk : 0, nup = ex ? (size_t)hb.nup : 0;
  b.explicit_schur = ex ? 1 : 0;
  b.nblk = (int32_t)nsb;
  b.nup = (int32_t)nup;
  b.npairs = ex ? hb.npairs : 0;
  b.sblk_row = cv.take<int32_t>(ex ? nc + 1 : 0);
  b.sblk_max = 0;
  if (ex)
    for (size_t c = 0; c < nc; ++c) b.sblk_max = std::max(b.sblk_max, hb.sblk_row[c + 1] - hb.sblk_row[c] + 1);
  b.sblk_col = cv.take<int32_t>(nsb);
  b.sblk_tr = cv.take<int32_t>(nsb);
  b.sblk_up = cv.take<int32_t>(nup);
  b.sblk_pair = cv.take<int32_t>(ex ? nup + 1 : 0);
  b.spair = cv.take<int2>(ex ? (size_t)hb.npairs : 0);
  b.obs_fpos = cv.take<int32_t>(ex ? no : 0);
  const bool rig = !hb.obs_rig.empty();
  b.obs_rig = cv.take<uint8_t>(rig ? no : 0);
  b.prob_rig = cv.take<double>(rig ? (size_t)kRig * P : 0);
  const bool res = !hb.resume.empty();
  b.prob_resume = cv.take<int32_t>(res ? P : 0);
  b.lm_resume = cv.take<LMState>(res ? P : 0);
  b.cam_scale_in = cv.take<double>(res ? 9 * nc : 0);
  b.pt_scale_in = cv.take<double>(res ? 3 * np : 0);
  if (!res) b.prob_resume = nullptr, b.lm_resume = nullptr, b.cam_scale_in = nullptr, b.pt_scale_in = nullptr;
  *upload_bytes = align_up(cv.off, 256);
  // download
  cv.off = *upload_bytes;
  *download_off = cv.off;
  double *out_cam = cv.take<double>(9 * nc);
  double *out_pt = cv.take<double>(4 * np);
  (void)out_cam;
  (void)out_pt;
  b.lm = cv.take<LMState>(P);
  b.trace_cap = trace_cap_;
  b.trace_cost = cv.take<double>(P * trace_cap_);
  b.trace_radius = cv.take<double>(P * trace_cap_);
  b.trace_pcg = cv.take<int32_t>(P * trace_cap_);
  b.trace_succ = cv.take<int32_t>(P * trace_cap_);
  b.status = cv.take<int32_t>(8);
  b.obs_chi2 = cv.take<double>(rig ? no : 0);
  *download_bytes = align_up(cv.off, 256) - *download_off;
  cv.off = *download_off + *download_bytes;
  // work
  const size_t rs = mixed_ ? sizeof(float) : sizeof(double);
  b.cam_param[0] = cv.take<double>(9 * nc);
  b.cam_param[1] = cv.take<double>(9 * nc);
  b.pt_param[0] = cv.take<double>(4 * np);
  b.pt_param[1] = cv.take<double>(4 * np);
  b.cam_table = cv.take<double>(kCamTable * nc);
  b.cam_tablef = cv.take<float>(kCamTable * nc);
  b.cam_tabledf = cv.take<float2>(kCamTable * nc);
  b.jac = cv.take<char>(13 * no * 2 * rs);
  b.pt_C = cv.take<double>(6 * np);
  b.pt_g = cv.take<double>(3 * np);
  b.pt_scale = cv.take<double>(3 * np);
  b.pt_scalef = cv.take<float>(3 * np);
  b.pt_scaledf = cv.take<float2>(3 * np);
  b.pt_t = cv.take<double>(3 * np);
  b.pt_Cinv = cv.take<char>(6 * np * rs);
  b.pt_Cinv64 = cv.take<double>(6 * np);
  b.pt_colnorm = cv.take<double>(3 * np);
  b.cam_B = cv.take<double>(45 * nc);
  b.cam_g = cv.take<double>(9 * nc);
  b.cam_scale = cv.take<double>(9 * nc);
  b.cam_scalef = cv.take<float>(9 * nc);
  b.cam_scaledf = cv.take<float2>(9 * nc);
  b.cam_Minv = cv.take<double>(81 * nc);
  b.cam_Minvf = cv.take<float>(81 * nc);
  b.cam_Bf = cv.take<float>(45 * nc);
  b.cam_D2 = cv.take<double>(9 * nc);
  b.pcg_x = cv.take<double>(9 * nc);
  b.pcg_r = cv.take<double>(9 * nc);
  b.pcg_z = cv.take<double>(9 * nc);
  b.pcg_p = cv.take<double>(9 * nc);
  b.pcg_v = cv.take<double>(9 * nc);
  b.pcg_zf = cv.take<float>(9 * nc);
  b.pcg_pf = cv.take<float>(9 * nc);
  b.cam_colnorm = cv.take<double>(9 * nc);
  b.piece_part = cv.take<double>(mixed_ ? 0 : 54 * (size_t)npieces);
  b.cam_counter = cv.take<uint32_t>(mixed_ ? 0 : nc);
  b.seg_partial = cv.take<double>(9 * ns);
  b.schur_partial = cv.take<char>(54 * ns * rs);
  b.seg_grad = cv.take<double>(mixed_ ? 9 * ns : 0);
  b.chunk_scal = cv.take<double>(kChunkScal * nch);
  b.cam_scal = cv.take<double>(kCamScal * nc);
  b.chunk_red = cv.take<double>(2 * nch);
  b.blk_red = cv.take<double>(3 * nb);
  b.obs_F = cv.take<char>(ex ? (size_t)kObsF * no * rs : 0);
  b.sblk_val = cv.take<char>(81 * nsb * rs);
  b.cam_Sii = cv.take<char>(ex ? 81 * nc * rs : 0);
  b.pcg_q = cv.take<double>(ex ? 9 * nc : 0);
  b.spmv_red = cv.take<double>(ex ? nc : 0);
  b.pcg_p2 = cv.take<double>(ex ? 9 * nc : 0);
  b.pq_row = cv.take<double>(ex ? 9 * nc : 0);
  b.grid_ctl = cv.take<uint32_t>(8);
  b.prob_counter = cv.take<uint32_t>(4 * P);
  b.global_counter = cv.take<uint32_t>(8);
  b.chunk_counter = cv.take<uint32_t>(nch);
  b.opt.function_tolerance = o_.function_tolerance;
  b.opt.gradient_tolerance = o_.gradient_tolerance;
  b.opt.parameter_tolerance = o_.parameter_tolerance;
  b.opt.initial_radius = o_.initial_trust_region_radius;
  b.opt.max_radius = o_.max_trust_region_radius;
  b.opt.min_radius = o_.min_trust_region_radius;
  b.opt.min_relative_decrease = o_.min_relative_decrease;
  b.opt.min_diagonal = o_.min_lm_diagonal;
  b.opt.max_diagonal = o_.max_lm_diagonal;
  b.opt.loss_scale = o_.loss_scale;
  b.opt.pcg_tolerance = o_.pcg_tolerance;
  b.opt.eta = o_.eta;
  b.opt.max_iterations = o_.max_num_iterations;
  b.opt.max_invalid_steps = o_.max_num_consecutive_invalid_steps;
  b.opt.jacobi_scaling = o_.jacobi_scaling;
  b.opt.loss = o_.loss;
  b.opt.pcg_criterion = o_.pcg_criterion;
  b.opt.max_pcg_iterations = o_.max_linear_solver_iterations;
  b.opt.min_pcg_iterations = o_.min_linear_solver_iterations;
  b.opt.mixed = mixed_ ? 1 : 0;
  b.opt.so3_left = o_.camera_update == GBA_CAMERA_UPDATE_SO3_LEFT ? 1 : 0;
  b.opt.g2o = o_.lm_policy == GBA_LM_POLICY_G2O ? 1 : 0;
  if (b.opt.g2o) b.opt.jacobi_scaling = 0;
  b.opt.max_bodies = max_lm_bodies();
  b.opt.bodies_cap = 0;  // set per graph by the segment runs
  b.opt.grid_wait_test = grid_wait_test_ ? 1 : 0;
  b.opt.pinhole = rig ? 1 : 0;
  b.lm_cond = 0;
  b.pcg_cond = 0;
  b.use_cond = 0;
  return align_up(cv.off, 256);
}

gba_status Engine::ensure_capacity(size_t dev_bytes, size_t host_bytes, std::string *err) {
  gba_status st;
  if (dev_bytes > d_cap_) {
    destroy_graph();
    if (d_arena_) cudaFree(d_arena_);
    d_arena_ = nullptr;
    d_cap_ = 0;
    const size_t want = align_up(dev_bytes + dev_bytes / 8, 1 << 20);
    if ((st = check(cudaMalloc(&d_arena_, want), "device workspace", err)) != GBA_OK) {
      d_arena_ = nullptr;
      return st;
    }
    d_cap_ = want;
  }
  if (host_bytes > h_cap_) {
    if (h_stage_) cudaFreeHost(h_stage_);
    h_stage_ = nullptr;
    h_cap_ = 0;
    const size_t want = align_up(host_bytes + host_bytes / 8, 1 << 20);
    if ((st = check(cudaMallocHost(&h_stage_, want), "pinned staging", err)) != GBA_OK) {
      h_stage_ = nullptr;
      return st;
    }
    h_cap_ = want;
  }
  return GBA_OK;
}

// The staging copies of an upload, run together in 1 MiB pieces on the
// host threads (a batch stages tens of MB into pinned memory).
struct StageCopies {
  struct Piece {
    void *dst;
    const void *src;
    size_t bytes;
  };
  std::vector<Piece> pieces;
  size_t total = 0;
  void add(void *dst, const void *src, size_t bytes) {
    constexpr size_t kPiece = 1 << 20;
    total += bytes;
    for (size_t o = 0; o < bytes; o += kPiece)
      pieces.push_back({static_cast<char *>(dst) + o, static_cast<const char *>(src) + o, std::min(kPiece, bytes - o)});
  }
  template <typename T, typename U>
  void put(const T *dst, const std::vector<U> &src) {
    if (!src.empty()) add(const_cast<T *>(dst), src.data(), src.size() * sizeof(U));
  }
  void run() {
    auto copy = [&](int i) { std::memcpy(pieces[i].dst, pieces[i].src, pieces[i].bytes); };
    if (total < (4u << 20)) {
      for (int i = 0; i < (int)pieces.size(); ++i) copy(i);
    } else {
      host_parallel((int)pieces.size(), copy);
    }
  }
};

gba_status Engine::upload(const HostBatch &hb, std::string *err) {
  gba_status st;
  if ((st = check(cudaSetDevice(device_), "cudaSetDevice", err)) != GBA_OK) return st;
  DeviceBatch probe{};
  size_t ub, doff, dbytes;
  const size_t total = layout(hb, nullptr, &probe, &ub, &doff, &dbytes);
  if ((st = ensure_capacity(total, doff + dbytes, err)) != GBA_OK) return st;
  upload_bytes_ = ub;
  download_off_ = doff;
  download_bytes_ = dbytes;
  layout(hb, d_arena_, &db_, &ub, &doff, &dbytes);
  DeviceBatch hdb{};
  layout(hb, h_stage_, &hdb, &ub, &doff, &dbytes);
  StageCopies sc;
  sc.put(hdb.prob, hb.prob);
  sc.put(hdb.chunk, hb.chunk);
  sc.put(hdb.obs_cam, hb.obs_cam);
  sc.put(hdb.obs_pt, hb.obs_pt);
  sc.put(hdb.obs_uv, hb.obs_uv);
  sc.put(hdb.obs_seg, hb.obs_seg);
  sc.put(hdb.obs_slot, hb.obs_slot);
  sc.put(hdb.pt_obs_begin, hb.pt_obs_begin);
  sc.put(hdb.pt_problem, hb.pt_problem);
  sc.put(hdb.cam_problem, hb.cam_problem);
  sc.put(hdb.pt_used, hb.pt_used);
  sc.put(hdb.cam_used, hb.cam_used);
  sc.put(hdb.seg_pos, hb.seg_pos);
  sc.put(hdb.seg_cam, hb.seg_cam);
  sc.put(hdb.cam_seg_begin, hb.cam_seg_begin);
  sc.put(hdb.seg_slot, hb.seg_slot);
  sc.put(hdb.cam_obs_begin, hb.cam_obs_begin);
  sc.put(hdb.cam_obs_list, hb.cam_obs_list);
  sc.put(hdb.cam_piece_begin, hb.cam_piece_begin);
  sc.put(hdb.camblk, hb.camblk);
  if (hb.explicit_schur) {
    sc.put(hdb.sblk_row, hb.sblk_row);
    sc.put(hdb.sblk_col, hb.sblk_col);
    sc.put(hdb.sblk_tr, hb.sblk_tr);
    sc.put(hdb.sblk_up, hb.sblk_up);
    sc.put(hdb.sblk_pair, hb.sblk_pair);
    sc.put(hdb.obs_fpos, hb.obs_fpos);
    sc.put(hdb.spair, hb.spair);
  }
  if (!hb.obs_rig.empty()) {
    sc.put(hdb.obs_rig, hb.obs_rig);
    sc.put(hdb.prob_rig, hb.prob_rig);
  }
  if (!hb.resume.empty()) {
    sc.put(hdb.prob_resume, hb.resume);
    sc.put(hdb.lm_resume, hb.resume_lm);
    sc.put(hdb.cam_scale_in, hb.resume_cam_scale);
    sc.put(hdb.pt_scale_in, hb.resume_pt_scale);
  }
  sc.put(hdb.cam_init, hb.cam_param);
  sc.put(hdb.pt_init, hb.pt_param);
  sc.run();
  if ((st = check(cudaMemcpyAsync(d_arena_, h_stage_, upload_bytes_, cudaMemcpyHostToDevice, stream_),
                  "upload", err)) != GBA_OK)
    return st;
  // the PCG as one cluster launch per LM iteration: mixed form, explicit
  // Schur complement, every problem small enough
  cl_plan_ = ClusterPlan();
  if (mixed_ && hb.explicit_schur && o_.persistent_pcg &&
      !pcg_cluster_plan(hb.prob.data(), (int)hb.prob.size(), hb.sblk_row.data(), cluster_cams_, &cl_plan_))
    cl_plan_ = ClusterPlan();
  // the PCG as one grid-wide launch per LM iteration: FP64 form, explicit
  // Schur complement, one problem
  gr_plan_ = GridPlan();
  if (o_.persistent_pcg && !pcg_grid_plan((int)hb.prob.size(), mixed_, hb.explicit_schur, hb.nc,
                                          hb.explicit_schur ? hb.sblk_row.data() : nullptr, grid_ctas_, &gr_plan_))
    gr_plan_ = GridPlan();
  // current batch shape + pointers + options + PCG form = graph key
  DeviceBatch k = db_;
  cur_key_.assign(reinterpret_cast<const char *>(&k), reinterpret_cast<const char *>(&k) + sizeof k);
  cur_key_.push_back(cl_plan_.cs);
  cur_key_.push_back(cl_plan_.threads);
  cur_key_.push_back(cl_plan_.cache_blocks);
  cur_key_.push_back(gr_plan_.grid);
  cur_key_.push_back(gr_plan_.cap_blocks);
  cur_key_.push_back(gr_plan_.cap_pairs);
  return GBA_OK;
}

void Engine::destroy_graph() {
  if (exec_) cudaGraphExecDestroy(exec_);
  if (graph_) cudaGraphDestroy(graph_);
  exec_ = nullptr;
  graph_ = nullptr;
  graph_key_.clear();
  if (exec_c_) cudaGraphExecDestroy(exec_c_);
  if (graph_c_) cudaGraphDestroy(graph_c_);
  exec_c_ = nullptr;
  graph_c_ = nullptr;
  graph_c_key_.clear();
}

// Profiling runs one launch at a time and waits for it, so the GPU is idle
// when the next launch is queued.  A short delay kernel ahead of the start
// event keeps the GPU busy while the host queues the event and the measured
// kernel: the event pair then brackets the kernel's device time only, not
// the host's launch latency.
void Engine::prof_begin(cudaStream_t s) {
  if (!profiling_) return;
  launch_prof_delay(s);
  cudaEventRecord(pev_[0], s);
}
void Engine::prof_end(cudaStream_t s, int entry, double bytes) {
  if (!profiling_) return;
  cudaEventRecord(pev_[1], s);
  cudaEventSynchronize(pev_[1]);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, pev_[0], pev_[1]);
  profile_[entry].launches += 1;
  profile_[entry].total_ms += ms;
  profile_[entry].bytes += bytes;
}

// Algorithmic bytes of one launch of the main kernels (what the kernel
// must read and write at least once; cached gathers counted once per
// distinct item).  Used for the achieved-bandwidth figures.
static double bytes_spmv(const DeviceBatch &b) {
  // the blocks' values and columns, the diagonal blocks, z and p_{k-1} of
  // every camera (working precision), S p and the p.q shares out (FP64)
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  return (double)b.nblk * (81.0 * rs + 4.0) + (double)b.nc * (81.0 * rs + 18.0 * rs + 72.0 + 8.0 + 8.0);
}
static double bytes_matvec(const DeviceBatch &b) {
  if (b.explicit_schur) return bytes_spmv(b);
  // J_c, J_p (12 pairs) + segment / slot / point indices per observation;
  // C^-1 + CSR per point; per segment its position, slot, camera and the
  // camera's first-segment index, the camera's z and p_{k-1} (working
  // precision) and its partial out; per camera the B + Dc^2 row of the
  // chunk that owns it; per chunk its record and its value of p.q
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  return (double)b.no * (24.0 * rs + 8.0) + (double)b.np * (4.0 + 6.0 * rs) +
         (double)b.nseg * (14.0 + 27.0 * rs) + (double)b.nc * 90.0 * rs + (double)b.nchunks * 40.0;
}
static double bytes_schur_form(const DeviceBatch &b) {
  // the pairs, every observation's F once (a cached gather), per formed
  // block its index, pair range and transpose index, and every block's 81
  // values out
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  return (double)b.npairs * 8.0 + (double)b.no * kObsF * rs + (double)b.nup * 12.0 + (double)b.nblk * 81.0 * rs;
}
static double bytes_pcg_camera(const DeviceBatch &b) {
  // partials and chunk values read once; per camera x, r, z, v, p in and
  // x, r, z, p out (FP64; FP32 copies of z and p in the mixed form), the
  // rows of B and M^-1, Dc^2 and the segment range
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  return (double)b.nseg * 9.0 * rs + (double)b.nchunks * 8.0 +
         (double)b.nc * (9.0 * 8.0 * 9.0 + (b.opt.mixed ? 72.0 : 0.0) + (45.0 + 81.0) * rs + 72.0 + 8.0);
}
static double bytes_eval(const DeviceBatch &b) {
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  // K1: uv, cam, pt in; 13 pairs out; points in/out; K1c: list, 10 pairs in.
  // Mixed form: K1 also reads the slot per observation and writes 9 FP64
  // gradient partials per segment, which K1c reads instead of r.
  const double seg = b.opt.mixed ? (double)b.nseg * (2.0 + 4.0 + 2.0 * 72.0) + (double)b.no * (2.0 - 2.0 * rs) : 0.0;
  return (double)b.no * (24.0 + 26.0 * rs) + (double)b.np * (32.0 + 72.0 + 4.0 + 24.0) +
         (double)b.nc * (kCamTable * 8.0) + (double)b.no * (4.0 + 20.0 * rs) + (double)b.nc * (54.0 * 8.0) + seg;
}
static double bytes_point_schur(const DeviceBatch &b) {
  // J_c, J_p, slot and point index per observation; C, g in and C^-1 (both
  // precisions), t out per point; 54 partials per segment
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  // (+ F per observation with the explicit Schur complement)
  return (double)b.no * (24.0 * rs + 2.0 + 4.0) + (double)b.np * (48.0 + 24.0 + 6.0 * rs + 48.0 + 24.0) +
         (double)b.nseg * (54.0 * rs + 8.0) + (b.explicit_schur ? (double)b.no * kObsF * rs : 0.0);
}
static double bytes_schur(const DeviceBatch &b) {
  // partials in; B, g in; D^2, M^-1 (both precisions), PCG start vectors out
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  return (double)b.nseg * 54.0 * rs + (double)b.nc * ((45.0 + 9.0) * 8.0 + 9.0 * 8.0 + 81.0 * (8.0 + rs) + 5.0 * 72.0);
}
static double bytes_backsub(const DeviceBatch &b) {
  const double rs = b.opt.mixed ? 4.0 : 8.0;
  return (double)b.no * (26.0 * rs + 8.0) + (double)b.np * (24.0 + 48.0 + 24.0 + 64.0);
}
static double bytes_cost(const DeviceBatch &b) {
  return (double)b.no * 24.0 + (double)b.np * 32.0 + (double)b.nc * 15.0 * 8.0;
}

// Every completion counter starts at zero (the last CTA at a counter resets
// it, so they stay zero between kernels).
void Engine::zero_counters(cudaStream_t s) {
  cudaMemsetAsync(db_.prob_counter, 0, 4 * sizeof(uint32_t) * (size_t)db_.num_problems, s);
  cudaMemsetAsync(db_.global_counter, 0, 8 * sizeof(uint32_t), s);
  if (db_.nchunks > 0) cudaMemsetAsync(db_.chunk_counter, 0, sizeof(uint32_t) * (size_t)db_.nchunks, s);
  if (!mixed_ && db_.nc > 0) cudaMemsetAsync(db_.cam_counter, 0, sizeof(uint32_t) * (size_t)db_.nc, s);
}

void Engine::enqueue_setup(cudaStream_t s) {
  zero_counters(s);
  cudaMemsetAsync(db_.status, 0, 8 * sizeof(int32_t), s);
  launch_sync_param_buffers(db_, s);
  launch_init_state(db_, s);
  launch_camera_table(db_, s);
  launch_eval_jacobian(db_, mixed_, true, s);
  launch_scale_init(db_, s);
  launch_eval_jacobian(db_, mixed_, false, s);
  launch_post_eval(db_, s);
}

void Engine::enqueue_lm_head(cudaStream_t s) {
  prof_begin(s);
  launch_point_prepare(db_, mixed_, s);
  prof_end(s, PF_POINT, bytes_point_schur(db_));
  prof_begin(s);
  launch_camera_schur(db_, mixed_, s);
  prof_end(s, PF_SCHUR, bytes_schur(db_));
  if (db_.explicit_schur) {
    prof_begin(s);
    launch_schur_form(db_, mixed_, s);
    prof_end(s, PF_FORM, bytes_schur_form(db_));
  }
}

void Engine::enqueue_lm_tail(cudaStream_t s) {
  prof_begin(s);
  launch_back_substitute(db_, mixed_, s);
  prof_end(s, PF_BACKSUB, bytes_backsub(db_));
  prof_begin(s);
  launch_candidate_cost(db_, s);
  prof_end(s, PF_CANDIDATE, bytes_cost(db_));
  prof_begin(s);
  launch_decide(db_, s);
  prof_end(s, PF_DECIDE, 0.0);
  prof_begin(s);
  launch_camera_table(db_, s);
  prof_end(s, PF_TABLE, (double)db_.nc * (72.0 + kCamTable * 8.0));
  prof_begin(s);
  launch_eval_jacobian(db_, mixed_, false, s);
  prof_end(s, PF_EVAL, bytes_eval(db_));
  prof_begin(s);
  launch_post_eval(db_, s);
  prof_end(s, PF_POST, 0.0);
}

// The solve as one graph: setup, WHILE(LM) { head; PCG; tail }, gather.
// cont: the continue graph of segment runs (counters zeroed, no setup).
// With a segment length k the loop of one launch stops after k LM bodies
// (k + 1 counted bodies with the setup's evaluation).
gba_status Engine::build_graph(std::string *err, bool cont) {
  cudaGraph_t &graph = cont ? graph_c_ : graph_;
  cudaGraphExec_t &exec = cont ? exec_c_ : exec_;
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
  gba_status st;
  cudaGraphConditionalHandle lmh = 0, pcgh = 0;
  cudaGetLastError();  // the launches below report their own errors only
  if ((st = check(cudaGraphCreate(&graph, 0), "cudaGraphCreate", err)) != GBA_OK) return st;
  if ((st = check(cudaGraphConditionalHandleCreate(&lmh, graph, 1, cudaGraphCondAssignDefault),
                  "conditional handle", err)) != GBA_OK)
    return st;
  const DeviceBatch saved = db_;
  db_.use_cond = 1;
  db_.lm_cond = lmh;
  db_.pcg_cond = 0;
  db_.opt.bodies_cap = segment_bodies_ > 0 ? segment_bodies_ + (cont ? 0 : 1) : 0;
  const bool prof = profiling_;
  profiling_ = false;
  // a failed build: the captures are ended and the graph is dropped, not
  // destroyed (a capture that failed may have left it unusable)
  auto fail = [&](cudaError_t e, const char *what) {
    profiling_ = prof;
    end_captures();
    cudaGetLastError();
    const gba_status r = check(e, what, err);
    exec = nullptr;
    graph = nullptr;
    db_ = saved;
    return r;
  };
  auto add_while = [&](cudaStream_t s, cudaGraphConditionalHandle h, cudaGraph_t *body) -> cudaError_t {
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &np);
    if (e != cudaSuccess) return e;
    *body = np.conditional.phGraph_out[0];
    return cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  };
  // setup, then WHILE(LM) { head; WHILE(PCG) { mat-vec; camera side } tail }, then gather
  cudaError_t e = cudaStreamBeginCaptureToGraph(stream_, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(e, "capture setup");
  if (cont)
    zero_counters(stream_);
  else
    enqueue_setup(stream_);
  cudaGraph_t lmbody = nullptr, pcgbody = nullptr, tmp = nullptr;
  if ((e = add_while(stream_, lmh, &lmbody)) != cudaSuccess) return fail(e, "LM conditional node");
  // (a conditional handle must belong to a node: none for the cluster PCG)
  const bool one_launch = cl_plan_.cs > 0 || gr_plan_.grid > 0;
  if (!one_launch &&
      (e = cudaGraphConditionalHandleCreate(&pcgh, lmbody, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
    return fail(e, "PCG conditional handle");
  db_.pcg_cond = one_launch ? 0 : pcgh;
  e = cudaStreamBeginCaptureToGraph(cap_[0], lmbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(e, "capture LM body");
  enqueue_lm_head(cap_[0]);
  if (cl_plan_.cs > 0) {
    // the whole PCG of every problem in one cluster launch
    if ((e = launch_pcg_cluster(db_, cl_plan_, cap_[0])) != cudaSuccess) return fail(e, "PCG cluster kernel");
  } else if (gr_plan_.grid > 0) {
    // the whole PCG of the problem in one grid-wide launch
    if ((e = launch_pcg_grid(db_, gr_plan_, cap_[0])) != cudaSuccess) return fail(e, "PCG grid kernel");
  } else {
    if ((e = add_while(cap_[0], pcgh, &pcgbody)) != cudaSuccess) return fail(e, "PCG conditional node");
    e = cudaStreamBeginCaptureToGraph(cap_[1], pcgbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(e, "capture PCG body");
    // pcg_unroll (default kPcgUnroll) PCG iterations per body (a finished PCG turns the extra
    // launches into early exits); inside the body each kernel is a
    // programmatic dependent of the one before it
    const int unroll = o_.pcg_unroll > 0 ? std::min(o_.pcg_unroll, 8) : kPcgUnroll;
    for (int u = 0; u < unroll; ++u) {
      if ((e = launch_schur_matvec(db_, mixed_, cap_[1], pdl_ && u > 0)) != cudaSuccess)
        return fail(e, "mat-vec kernel");
      if ((e = launch_pcg_camera(db_, mixed_, cap_[1], pdl_)) != cudaSuccess) return fail(e, "PCG camera kernel");
    }
    if ((e = cudaStreamEndCapture(cap_[1], &tmp)) != cudaSuccess) return fail(e, "end capture PCG body");
  }
  enqueue_lm_tail(cap_[0]);
  if ((e = cudaStreamEndCapture(cap_[0], &tmp)) != cudaSuccess) return fail(e, "end capture LM body");
  enqueue_gather(stream_);
  if ((e = cudaStreamEndCapture(stream_, &tmp)) != cudaSuccess) return fail(e, "end capture");
  if ((e = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) return fail(e, "cudaGraphInstantiate");
  profiling_ = prof;
  if (cont) {
    graph_c_key_ = cur_key_;
    graph_c_segment_ = segment_bodies_;
  } else {
    graph_key_ = cur_key_;
    graph_segment_ = segment_bodies_;
  }
  db_ = saved;
  return GBA_OK;
}

// Ends the captures a failed graph build left open.  Every capture goes
// into a graph that is already owned (the graph being built, or a body of
// one of its conditional nodes), so nothing returned here is destroyed: the
// caller destroys the graph being built, which owns the bodies.
void Engine::end_captures() {
  cudaStreamCaptureStatus cs;
  for (cudaStream_t s : {cap_[1], cap_[0], stream_}) {
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
    }
  }
}

void Engine::enqueue_gather(cudaStream_t s) {
  char *out = d_arena_ + download_off_;
  double *out_cam = reinterpret_cast<double *>(out);
  double *out_pt = reinterpret_cast<double *>(out + align_up(sizeof(double) * 9 * (size_t)db_.nc, 256));
  launch_gather_results(db_, out_cam, out_pt, s);
  if (db_.opt.pinhole) launch_window_chi2(db_, out_cam, out_pt, s);
}

gba_status Engine::run_host_driven(std::string *err) {
  gba_status st;
  db_.use_cond = 0;
  db_.lm_cond = 0;
  db_.pcg_cond = 0;
  int32_t *hstat = reinterpret_cast<int32_t *>(h_stage_ + (reinterpret_cast<char *>(db_.status) - d_arena_));
  auto read_status = [&]() -> gba_status {
    gba_status s2 = check(cudaMemcpyAsync(hstat, db_.status, 8 * sizeof(int32_t), cudaMemcpyDeviceToHost, stream_),
                          "status read", err);
    if (s2 != GBA_OK) return s2;
    return check(cudaStreamSynchronize(stream_), "solver kernels", err);
  };
  prof_begin(stream_);
  zero_counters(stream_);
  cudaMemsetAsync(db_.status, 0, 8 * sizeof(int32_t), stream_);
  launch_sync_param_buffers(db_, stream_);
  launch_init_state(db_, stream_);
  prof_end(stream_, PF_SETUP_MISC, 0.0);
  prof_begin(stream_);
  launch_camera_table(db_, stream_);
  prof_end(stream_, PF_TABLE, (double)db_.nc * (72.0 + kCamTable * 8.0));
  prof_begin(stream_);
  launch_eval_jacobian(db_, mixed_, true, stream_);
  launch_scale_init(db_, stream_);
  prof_end(stream_, PF_SETUP_MISC, 0.0);
  prof_begin(stream_);
  launch_eval_jacobian(db_, mixed_, false, stream_);
  prof_end(stream_, PF_EVAL, bytes_eval(db_));
  prof_begin(stream_);
  launch_post_eval(db_, stream_);
  prof_end(stream_, PF_POST, 0.0);
  if ((st = read_status()) != GBA_OK) return st;
  int bodies = 0;
  while (hstat[1] && hstat[0] == 0) {
    if (++bodies > max_lm_bodies() + 2) break;
    enqueue_lm_head(stream_);
    if (cl_plan_.cs > 0 || gr_plan_.grid > 0) {
      if ((st = enqueue_pcg_one_launch(stream_, err)) != GBA_OK) return st;
      enqueue_lm_tail(stream_);
      if ((st = read_status()) != GBA_OK) return st;
      continue;
    }
    if ((st = read_status()) != GBA_OK) return st;
    int pcg = 0;
    while (hstat[2] && pcg <= o_.max_linear_solver_iterations) {
      ++pcg;
      prof_begin(stream_);
      if ((st = check(launch_schur_matvec(db_, mixed_, stream_, false), "mat-vec kernel", err)) != GBA_OK) return st;
      prof_end(stream_, PF_MATVEC, bytes_matvec(db_));
      prof_begin(stream_);
      if ((st = check(launch_pcg_camera(db_, mixed_, stream_, false), "PCG camera kernel", err)) != GBA_OK) return st;
      prof_end(stream_, PF_PCGCAM, bytes_pcg_camera(db_));
      if ((st = read_status()) != GBA_OK) return st;
    }
    enqueue_lm_tail(stream_);
    if ((st = read_status()) != GBA_OK) return st;
  }
  enqueue_gather(stream_);
  return check(cudaGetLastError(), "kernel launch", err);
}

// Algorithmic bytes of one cluster-PCG launch: the blocks of S (off-diagonal
// and diagonal) and M^-1 once (FP32), v, r, z in and x, r, z, p out per
// camera coordinate (FP64), z in FP32; the exchanges between the CTAs stay
// in L2.
static double bytes_pcg_cluster(const DeviceBatch &b) {
  return ((double)b.nblk + b.nc) * 81.0 * 4.0 + (double)b.nc * 81.0 * 4.0 + (double)b.nc * 9.0 * (3 * 8.0 + 4.0 + 4 * 8.0);
}

// Algorithmic bytes of one grid-PCG launch: the blocks of S (off-diagonal
// and diagonal) and M^-1 once (FP64), v, r, z, x in and x, r, z, p out per
// camera coordinate; the per-iteration exchanges stay in L2.
static double bytes_pcg_grid(const DeviceBatch &b) {
  return ((double)b.nblk + b.nc) * 81.0 * 8.0 + (double)b.nc * 81.0 * 8.0 + (double)b.nc * 9.0 * 8 * 8.0;
}

gba_status Engine::enqueue_pcg_one_launch(cudaStream_t s, std::string *err) {
  prof_begin(s);
  if (gr_plan_.grid > 0) {
    const gba_status st = check(launch_pcg_grid(db_, gr_plan_, s), "PCG grid kernel", err);
    prof_end(s, PF_GRID, bytes_pcg_grid(db_));
    return st;
  }
  const gba_status st = check(launch_pcg_cluster(db_, cl_plan_, s), "PCG cluster kernel", err);
  prof_end(s, PF_CLUSTER, bytes_pcg_cluster(db_));
  return st;
}

gba_status Engine::rerun(std::string *err) {
  if (!d_arena_ || cur_key_.empty()) {
    *err = "no problem has been uploaded on this handle";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  return run_solve(err);
}

gba_status Engine::run_solve(std::string *err) {
  gba_status st;
  if ((st = check(cudaEventRecord(ev_start_, stream_), "event", err)) != GBA_OK) return st;
  if (o_.use_graphs && !profiling_) {
    if (!exec_ || graph_key_ != cur_key_ || graph_segment_ != segment_bodies_) {
      st = build_graph(err);
      if (st != GBA_OK && pdl_) {
        pdl_ = false;  // a driver without programmatic edges in conditional bodies
        st = build_graph(err);
      }
      if (st != GBA_OK) return st;
    }
    if ((st = check(cudaGraphLaunch(exec_, stream_), "cudaGraphLaunch", err)) != GBA_OK) return st;
  } else {
    if ((st = run_host_driven(err)) != GBA_OK) return st;
  }
  return check(cudaEventRecord(ev_stop_, stream_), "event", err);
}

gba_status Engine::prepare_continue(std::string *err) {
  if (exec_c_ && graph_c_key_ == cur_key_ && graph_c_segment_ == segment_bodies_) return GBA_OK;
  gba_status st = build_graph(err, true);
  if (st != GBA_OK && pdl_) {
    pdl_ = false;
    st = build_graph(err, true);
  }
  return st;
}

gba_status Engine::run_segment(bool cont, std::string *err) {
  if (!cont) return run_solve(err);
  const gba_status st = prepare_continue(err);
  if (st != GBA_OK) return st;
  return check(cudaGraphLaunch(exec_c_, stream_), "cudaGraphLaunch", err);
}

gba_status Engine::fetch_states(std::string *err) {
  const size_t off = reinterpret_cast<char *>(db_.lm) - d_arena_;
  const size_t soff = reinterpret_cast<char *>(db_.status) - d_arena_;
  gba_status st = check(cudaMemcpyAsync(h_stage_ + off, db_.lm, sizeof(LMState) * (size_t)db_.num_problems,
                                        cudaMemcpyDeviceToHost, stream_),
                        "state read", err);
  if (st != GBA_OK) return st;
  return check(cudaMemcpyAsync(h_stage_ + soff, db_.status, 8 * sizeof(int32_t), cudaMemcpyDeviceToHost, stream_),
               "status read", err);
}

const LMState *Engine::states(const HostBatch &hb) {
  (void)hb;
  return reinterpret_cast<const LMState *>(h_stage_ + (reinterpret_cast<char *>(db_.lm) - d_arena_));
}

// The device-side error word of the batch (as last downloaded or fetched).
gba_status Engine::device_status(std::string *err) {
  const int32_t s0 = *reinterpret_cast<const int32_t *>(h_stage_ + (reinterpret_cast<char *>(db_.status) - d_arena_));
  if (s0 == GBA_ERR_TIMEOUT) {
    *err = "a bounded device-side wait of the grid PCG ran out (the solve was stopped)";
    return GBA_ERR_TIMEOUT;
  }
  if (s0 != 0) {
    *err = "device-side loop guard tripped (internal error)";
    return GBA_ERR_INTERNAL;
  }
  return GBA_OK;
}

void Engine::summarize(const DeviceBatch &hdb, int p, double solve_s, gba_summary *out) {
  const LMState &L = hdb.lm[p];
  gba_summary &S = *out;
  S.initial_cost = L.initial_cost;
  S.final_cost = L.x_cost;
  S.num_iterations = L.iteration;
  S.num_successful_steps = L.successful_steps;
  S.num_unsuccessful_steps = L.unsuccessful_steps;
  S.num_invalid_steps = L.invalid_steps;
  S.num_linear_solver_iterations = L.total_pcg_iterations;
  S.termination_type = L.termination_type < 0 ? GBA_TERMINATION_NO_CONVERGENCE : L.termination_type;
  S.termination_reason = L.termination_reason;
  S.final_trust_region_radius = L.radius;
  S.gradient_max_norm = L.gradient_max_norm;
  S.solve_time_s = solve_s;
  const int n = std::min(L.iteration + 1, trace_cap_);
  S.trace_length = std::min(n, S.trace_capacity > 0 ? S.trace_capacity : 0);
  for (int k = 0; k < S.trace_length; ++k) {
    const size_t i = (size_t)p * trace_cap_ + k;
    if (S.trace_cost) S.trace_cost[k] = hdb.trace_cost[i];
    if (S.trace_radius) S.trace_radius[k] = hdb.trace_radius[i];
    if (S.trace_linear_iterations) S.trace_linear_iterations[k] = hdb.trace_pcg[i];
    if (S.trace_successful) S.trace_successful[k] = hdb.trace_succ[i];
  }
}

gba_status Engine::deliver(const HostBatch &hb, const std::vector<int> &probs, const gba_problem_view *v,
                           gba_summary *s, std::string *err) {
  if (probs.empty()) return GBA_OK;
  const size_t cam_off = download_off_;
  const size_t pt_off = download_off_ + align_up(sizeof(double) * 9 * (size_t)hb.nc, 256);
  gba_status st;
  for (int p : probs) {
    const ProblemInfo &pi = hb.prob[p];
    const size_t oc = cam_off + sizeof(double) * 9 * (size_t)pi.cam_begin;
    const size_t op = pt_off + sizeof(double) * 4 * (size_t)pi.pt_begin;
    if ((st = check(cudaMemcpyAsync(h_stage_ + oc, d_arena_ + oc, sizeof(double) * 9 * (size_t)pi.cam_count,
                                    cudaMemcpyDeviceToHost, stream_),
                    "result read", err)) != GBA_OK ||
        (st = check(cudaMemcpyAsync(h_stage_ + op, d_arena_ + op, sizeof(double) * 4 * (size_t)pi.pt_count,
                                    cudaMemcpyDeviceToHost, stream_),
                    "result read", err)) != GBA_OK)
      return st;
  }
  if ((st = check(cudaStreamSynchronize(stream_), "solver kernels", err)) != GBA_OK) return st;
  DeviceBatch hdb{};
  size_t ub, doff, dbytes;
  layout(hb, h_stage_, &hdb, &ub, &doff, &dbytes);
  const double *out_cam = reinterpret_cast<const double *>(h_stage_ + cam_off);
  const double *out_pt = reinterpret_cast<const double *>(h_stage_ + pt_off);
  for (int p : probs) {
    if (v[p].parameters) scatter_parameters(hb, p, out_cam, out_pt, v[p].parameters);
    if (s) summarize(hdb, p, 0.0, &s[p]);
  }
  return GBA_OK;
}

gba_status Engine::download_states(const HostBatch &hb, std::vector<ProblemState> *out, std::string *err) {
  std::vector<double> cs(9 * (size_t)hb.nc), ps(3 * (size_t)hb.np);
  gba_status st;
  if (hb.nc && (st = check(cudaMemcpyAsync(cs.data(), db_.cam_scale, cs.size() * sizeof(double),
                                           cudaMemcpyDeviceToHost, stream_),
                           "scale read", err)) != GBA_OK)
    return st;
  if (hb.np && (st = check(cudaMemcpyAsync(ps.data(), db_.pt_scale, ps.size() * sizeof(double),
                                           cudaMemcpyDeviceToHost, stream_),
                           "scale read", err)) != GBA_OK)
    return st;
  if ((st = check(cudaStreamSynchronize(stream_), "scale read", err)) != GBA_OK) return st;
  const LMState *lm = states(hb);
  out->resize((size_t)hb.P);
  for (int p = 0; p < hb.P; ++p) {
    (*out)[p].lm = lm[p];
    gather_scales(hb, p, cs.data(), ps.data(), &(*out)[p]);
  }
  return GBA_OK;
}

gba_status Engine::download(const HostBatch &hb, const gba_problem_view *v, gba_summary *s, std::string *err) {
  gba_status st;
  if ((st = check(cudaMemcpyAsync(h_stage_ + download_off_, d_arena_ + download_off_, download_bytes_,
                                  cudaMemcpyDeviceToHost, stream_),
                  "download", err)) != GBA_OK)
    return st;
  if ((st = check(cudaStreamSynchronize(stream_), "solver kernels", err)) != GBA_OK) return st;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev_start_, ev_stop_);
  last_solve_ms_ = ms;
  DeviceBatch hdb{};
  size_t ub, doff, dbytes;
  layout(hb, h_stage_, &hdb, &ub, &doff, &dbytes);
  const int32_t *hstat = hdb.status;
  if (hstat[0] == GBA_ERR_TIMEOUT) {
    *err = "a bounded device-side wait of the grid PCG ran out (the solve was stopped)";
    return GBA_ERR_TIMEOUT;
  }
  if (hstat[0] != 0) {
    *err = "device-side loop guard tripped (internal error)";
    return GBA_ERR_INTERNAL;
  }
  const double *out_cam = reinterpret_cast<const double *>(h_stage_ + download_off_);
  const double *out_pt =
      reinterpret_cast<const double *>(h_stage_ + download_off_ + align_up(sizeof(double) * 9 * (size_t)hb.nc, 256));
  for (int p = 0; p < hb.P; ++p) {
    if (v[p].parameters) scatter_parameters(hb, p, out_cam, out_pt, v[p].parameters);
    if (s) summarize(hdb, p, ms * 1e-3, &s[p]);
  }
  return GBA_OK;
}

gba_status Engine::solve(const gba_problem_view *v, int n, gba_summary *s, std::string *err) {
  const double t0 = now_s();
  PrepOptions po = prep_options();
  HostBatch &hb = hb_;  // kept between solves: its storage is reused
  gba_status st = prepare_batch(v, n, po, &hb, err);
  if (st != GBA_OK) return st;
  if ((st = upload(hb, err)) != GBA_OK) return st;
  const double t1 = now_s();
  if ((st = run_solve(err)) != GBA_OK) return st;
  if ((st = download(hb, v, s, err)) != GBA_OK) return st;
  const double t2 = now_s();
  if (s)
    for (int p = 0; p < n; ++p) {
      s[p].setup_time_s = t1 - t0;
      s[p].total_time_s = t2 - t0;
    }
  if (o_.minimizer_progress_to_stdout && s) {
    for (int p = 0; p < n; ++p) {
      std::printf("problem %d: iter  cost  tr_radius  pcg  success\n", p);
      for (int k = 0; k < s[p].trace_length; ++k)
        std::printf("%4d % .6e % .2e %4d %d\n", k, s[p].trace_cost ? s[p].trace_cost[k] : 0.0,
                    s[p].trace_radius ? s[p].trace_radius[k] : 0.0,
                    s[p].trace_linear_iterations ? s[p].trace_linear_iterations[k] : 0,
                    s[p].trace_successful ? s[p].trace_successful[k] : 0);
    }
  }
  return GBA_OK;
}

gba_status Engine::solve_windows(gba_window_view *w, int n, gba_summary *s, gba_window_result *res,
                                 std::string *err) {
  const double t0 = now_s();
  if (n <= 0 || !w) {
    *err = "empty batch";
    return GBA_ERR_INVALID_ARGUMENT;
  }
  // each window as a BAL-layout problem: a pose in a 9-slot camera block
  // (angle-axis, translation, three unused zeros), then the landmarks
  std::vector<std::vector<double>> par(n);
  std::vector<gba_problem_view> v(n);
  for (int p = 0; p < n; ++p) {
    const gba_window_view &x = w[p];
    if (x.num_keyframes < 0 || x.num_landmarks < 0 || x.num_observations < 0 ||
        (x.num_keyframes > 0 && !x.poses) || (x.num_landmarks > 0 && !x.landmarks) ||
        (x.num_observations > 0 && !x.rig_camera)) {
      *err = "window " + std::to_string(p) + ": missing arrays";
      return GBA_ERR_INVALID_ARGUMENT;
    }
    const double *k = &x.rig.fx;
    bool fin = std::isfinite(x.chi2_threshold) && x.max_threshold_doublings >= 0;
    for (int q = 0; q < 4 + 12; ++q) fin = fin && std::isfinite(k[q]);
    if (!fin) {
      *err = "window " + std::to_string(p) + ": non-finite rig or threshold";
      return GBA_ERR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < x.num_observations; ++i)
      if (x.rig_camera[i] > 1) {
        *err = "window " + std::to_string(p) + ": rig_camera must be 0 or 1";
        return GBA_ERR_INVALID_ARGUMENT;
      }
    par[p].assign(9 * (size_t)x.num_keyframes + 3 * (size_t)x.num_landmarks, 0.0);
    for (int c = 0; c < x.num_keyframes; ++c)
      for (int q = 0; q < 6; ++q) par[p][9 * (size_t)c + q] = x.poses[6 * (size_t)c + q];
    if (x.num_landmarks > 0)
      std::memcpy(par[p].data() + 9 * (size_t)x.num_keyframes, x.landmarks, sizeof(double) * 3 * (size_t)x.num_landmarks);
    v[p] = gba_problem_view{x.num_keyframes, x.num_landmarks, x.num_observations, x.keyframe_index,
                            x.landmark_index, x.observations, par[p].data()};
  }
  PrepOptions po = prep_options();
  HostBatch &hb = hb_;
  gba_status st = prepare_batch(v.data(), n, po, &hb, err);
  if (st != GBA_OK) return st;
  hb.obs_rig.resize(hb.no);
  hb.prob_rig.assign((size_t)kRig * n, 0.0);
  for (int p = 0; p < n; ++p) {
    const ProblemInfo &pi = hb.prob[p];
    for (int k = pi.obs_begin; k < pi.obs_begin + pi.obs_count; ++k) hb.obs_rig[k] = w[p].rig_camera[hb.obs_orig[k]];
    double *r = hb.prob_rig.data() + (size_t)kRig * p;
    r[0] = w[p].rig.fx, r[1] = w[p].rig.fy, r[2] = w[p].rig.cx, r[3] = w[p].rig.cy;
    for (int e = 0; e < 2; ++e) {
      double *R = r + 4 + 12 * e;
      const double *aa = w[p].rig.extrinsic[e];
      for (int j = 0; j < 3; ++j) {
        const double ej[3] = {j == 0 ? 1.0 : 0.0, j == 1 ? 1.0 : 0.0, j == 2 ? 1.0 : 0.0};
        double col[3];
        gba_angle_axis_rotate_point(aa, ej, col);
        R[j] = col[0], R[3 + j] = col[1], R[6 + j] = col[2];
      }
      R[9] = aa[3], R[10] = aa[4], R[11] = aa[5];
    }
  }
  if ((st = upload(hb, err)) != GBA_OK) return st;
  const double t1 = now_s();
  if ((st = run_solve(err)) != GBA_OK) return st;
  if ((st = download(hb, v.data(), s, err)) != GBA_OK) return st;
  // results: poses and landmarks back, then the outlier test of
  // backend.cpp:156-187 on each window's chi2 (GPU-evaluated at the returned
  // estimate, internal order -> the window's own order)
  DeviceBatch hdb{};
  size_t ub, doff, dbytes;
  layout(hb, h_stage_, &hdb, &ub, &doff, &dbytes);
  std::vector<double> chi2;
  for (int p = 0; p < n; ++p) {
    gba_window_view &x = w[p];
    for (int c = 0; c < x.num_keyframes; ++c)
      for (int q = 0; q < 6; ++q) x.poses[6 * (size_t)c + q] = par[p][9 * (size_t)c + q];
    if (x.num_landmarks > 0)
      std::memcpy(x.landmarks, par[p].data() + 9 * (size_t)x.num_keyframes, sizeof(double) * 3 * (size_t)x.num_landmarks);
    const ProblemInfo &pi = hb.prob[p];
    chi2.assign(x.num_observations, 0.0);
    for (int k = pi.obs_begin; k < pi.obs_begin + pi.obs_count; ++k) chi2[hb.obs_orig[k]] = hdb.obs_chi2[k];
    double th = x.chi2_threshold;
    int in = 0, out = 0;
    for (int it = 0; it < x.max_threshold_doublings; ++it) {
      in = out = 0;
      for (double c2 : chi2) c2 > th ? ++out : ++in;
      if ((double)in / (double)(in + out) > 0.5) break;
      th *= 2.0;
    }
    if (x.max_threshold_doublings <= 0)
      for (double c2 : chi2) c2 > th ? ++out : ++in;
    if (x.outlier)
      for (int i = 0; i < x.num_observations; ++i) x.outlier[i] = chi2[i] > th ? 1 : 0;
    if (res) {
      res[p].num_inliers = in;
      res[p].num_outliers = out;
      res[p].chi2_threshold = th;
    }
  }
  const double t2 = now_s();
  if (s)
    for (int p = 0; p < n; ++p) {
      s[p].setup_time_s = t1 - t0;
      s[p].total_time_s = t2 - t0;
    }
  return GBA_OK;
}

gba_status Engine::evaluate(const gba_problem_view *v, double *residuals, double *jacobians, double *cost,
                            std::string *err) {
  PrepOptions po = prep_options();
  HostBatch hb;
  gba_status st = prepare_batch(v, 1, po, &hb, err);
  if (st != GBA_OK) return st;
  if ((st = upload(hb, err)) != GBA_OK) return st;
  const int loss = db_.opt.loss;
  db_.opt.loss = GBA_LOSS_TRIVIAL;
  db_.use_cond = 0;
  zero_counters(stream_);
  cudaMemsetAsync(db_.status, 0, 8 * sizeof(int32_t), stream_);
  launch_sync_param_buffers(db_, stream_);
  launch_init_state(db_, stream_);
  launch_camera_table(db_, stream_);
  launch_eval_jacobian(db_, mixed_, true, stream_);
  db_.opt.loss = loss;
  launch_cost_only(db_, stream_);
  if ((st = check(cudaStreamSynchronize(stream_), "evaluate kernels", err)) != GBA_OK) return st;
  const size_t no = hb.no;
  const size_t pair = mixed_ ? sizeof(float2) : sizeof(double2);
  std::vector<char> jac(13 * no * pair);
  std::vector<double> cs((size_t)kChunkScal * hb.nchunks);
  if (no && (st = check(cudaMemcpy(jac.data(), db_.jac, jac.size(), cudaMemcpyDeviceToHost), "download", err)) != GBA_OK)
    return st;
  if (!cs.empty() && (st = check(cudaMemcpy(cs.data(), db_.chunk_scal, cs.size() * sizeof(double), cudaMemcpyDeviceToHost),
                                 "download", err)) != GBA_OK)
    return st;
  auto get = [&](int k, size_t o, int comp) -> double {
    if (mixed_) {
      const float2 f = reinterpret_cast<const float2 *>(jac.data())[k * no + o];
      return comp ? f.y : f.x;
    }
    const double2 d = reinterpret_cast<const double2 *>(jac.data())[k * no + o];
    return comp ? d.y : d.x;
  };
  for (size_t o = 0; o < no; ++o) {
    const size_t i = hb.obs_orig[o];
    for (int row = 0; row < 2; ++row) {
      if (residuals) residuals[2 * i + row] = get(12, o, row);
      if (jacobians)
        for (int k = 0; k < 12; ++k) jacobians[24 * i + 12 * row + k] = get(k, o, row);
    }
  }
  if (cost) {
    double c = 0.0;
    for (int ch = 0; ch < hb.nchunks; ++ch) c += cs[(size_t)kChunkScal * ch + kCS_COST];
    *cost = c;
  }
  return GBA_OK;
}

gba_status Engine::compute_step(const gba_problem_view *v, double radius, double *delta, double *model,
                                int *pcg_iterations, std::string *err) {
  PrepOptions po = prep_options();
  HostBatch hb;
  gba_status st = prepare_batch(v, 1, po, &hb, err);
  if (st != GBA_OK) return st;
  if ((st = upload(hb, err)) != GBA_OK) return st;
  db_.use_cond = 0;
  int32_t *hstat = reinterpret_cast<int32_t *>(h_stage_ + (reinterpret_cast<char *>(db_.status) - d_arena_));
  auto read_status = [&]() -> gba_status {
    gba_status s2 = check(cudaMemcpyAsync(hstat, db_.status, 8 * sizeof(int32_t), cudaMemcpyDeviceToHost, stream_),
                          "status read", err);
    if (s2 != GBA_OK) return s2;
    return check(cudaStreamSynchronize(stream_), "kernels", err);
  };
  zero_counters(stream_);
  cudaMemsetAsync(db_.status, 0, 8 * sizeof(int32_t), stream_);
  launch_sync_param_buffers(db_, stream_);
  launch_init_state(db_, stream_);
  launch_camera_table(db_, stream_);
  launch_eval_jacobian(db_, mixed_, true, stream_);
  launch_scale_init(db_, stream_);
  launch_eval_jacobian(db_, mixed_, false, stream_);
  launch_post_eval(db_, stream_);
  if ((st = read_status()) != GBA_OK) return st;
  // force the problem active with the requested radius
  LMState L;
  if ((st = check(cudaMemcpy(&L, db_.lm, sizeof L, cudaMemcpyDeviceToHost), "state", err)) != GBA_OK) return st;
  L.radius = radius;
  L.active = 1;
  if ((st = check(cudaMemcpy(db_.lm, &L, sizeof L, cudaMemcpyHostToDevice), "state", err)) != GBA_OK) return st;
  launch_point_prepare(db_, mixed_, stream_);
  launch_camera_schur(db_, mixed_, stream_);
  launch_schur_form(db_, mixed_, stream_);
  if ((st = read_status()) != GBA_OK) return st;
  if (cl_plan_.cs > 0 || gr_plan_.grid > 0) {
    if ((st = enqueue_pcg_one_launch(stream_, err)) != GBA_OK) return st;
  } else {
    int pcg = 0;
    while (hstat[2] && pcg <= o_.max_linear_solver_iterations) {
      ++pcg;
      launch_pcg_iteration(db_, mixed_, stream_);
      if ((st = read_status()) != GBA_OK) return st;
    }
  }
  launch_back_substitute(db_, mixed_, stream_);
  launch_candidate_cost(db_, stream_);
  launch_decide(db_, stream_);
  if ((st = check(cudaStreamSynchronize(stream_), "step kernels", err)) != GBA_OK) return st;
  if ((st = check(cudaMemcpy(&L, db_.lm, sizeof L, cudaMemcpyDeviceToHost), "state", err)) != GBA_OK) return st;
  std::vector<double> c0(9 * (size_t)hb.nc), c1(9 * (size_t)hb.nc), p0(4 * (size_t)hb.np), p1(4 * (size_t)hb.np);
  if (hb.nc) {
    cudaMemcpy(c0.data(), db_.cam_param[0], c0.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(c1.data(), db_.cam_param[1], c1.size() * 8, cudaMemcpyDeviceToHost);
  }
  if (hb.np) {
    cudaMemcpy(p0.data(), db_.pt_param[0], p0.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(p1.data(), db_.pt_param[1], p1.size() * 8, cudaMemcpyDeviceToHost);
  }
  if ((st = check(cudaGetLastError(), "download", err)) != GBA_OK) return st;
  const size_t n = 9 * (size_t)hb.nc + 3 * (size_t)hb.np;
  std::vector<double> x0(n), x1(n);
  scatter_parameters(hb, 0, c0.data(), p0.data(), x0.data());
  scatter_parameters(hb, 0, c1.data(), p1.data(), x1.data());
  for (size_t k = 0; k < n; ++k) delta[k] = x1[k] - x0[k];
  if (model) *model = L.model_cost_change;
  if (pcg_iterations) *pcg_iterations = L.pcg_iterations;
  if (!L.last_linear_ok) {
    *err = "linear solve failed";
    return GBA_ERR_INTERNAL;
  }
  return GBA_OK;
}

}  // namespace gba
