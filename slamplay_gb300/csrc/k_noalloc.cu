// k_noalloc.cu — gba_evaluate_noalloc: residuals and cost of a problem whose
// arrays already live on the device, without allocating anything.
//
// Who needs it: callers that cannot call cudaMalloc — a real-time tracking
// thread that must not take cudaMalloc's implicit device synchronisation and
// unbounded latency, or a host framework that owns all
// device memory through its own pool and forbids a library from allocating
// outside it.  They pass device inputs and outputs; the only scratch this
// entry point needs (per-camera rotation tables and per-CTA partial costs)
// lives in the file-scope array below, which the CUDA runtime loads with the
// module: every GPU that loads libgba holds it until the process exits.
//
// Limits: at most kNoAllocMaxCameras cameras and kNoAllocMaxObservations
// observations per call; larger problems are rejected with
// GBA_ERR_INVALID_ARGUMENT before any GPU work.
//
// Sharing: every call uses the same array.  Each call overwrites all of the
// scratch it reads (tables and partials are written before they are read),
// so no state leaks from one call to the next when calls are ordered; calls
// that may overlap on the GPU (different streams without ordering between
// them) race on the array and must not be issued.
//
// Set-up: the first call on a device (with that device current) looks up the
// device address of the array with cudaGetSymbolAddress and caches it per
// device; make that first call before any stream capture starts.  The cached
// address is the one of the module loaded in that device's primary context:
// after a cudaDeviceReset the module is loaded again and the array may move,
// so the entry point must not be used across a device reset.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "kernels.cuh"

namespace gba {

namespace {

constexpr int kNoAllocMaxCameras = 16384;
constexpr int kNoAllocMaxObservations = 1 << 24;
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = kNoAllocMaxObservations / kNoAllocThreads;
constexpr size_t kNoAllocScratchDoubles = (size_t)kNoAllocMaxCameras * kCamTable + kNoAllocMaxBlocks;  // ~6.3 MB

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double *g_scratch_ptr[kMaxDevices] = {nullptr};

gba_status fail(gba_status st, const std::string &msg);

// Per-camera table (R, t, f, k1, k2) of the rotation the residual uses.
__global__ void k_na_tables(const double *cameras, int nc, double *tables) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  camera_table_entry(cameras + 9 * (size_t)c, tables + (size_t)kCamTable * c, false);
}

// Per observation: residual (pred - observed) and the block's cost partial.
// Out-of-range indices give NaN residuals (and a NaN cost) instead of a read
// outside the arrays.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_na_residuals(gba_device_problem p, const double *tables, int loss, double loss_scale, double *residuals,
                   double *partials) {
  __shared__ double red[kNoAllocThreads / 32];
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double cost = 0.0;
  if (o < p.num_observations) {
    const int c = p.camera_index[o], j = p.point_index[o];
    double ru = __longlong_as_double(0x7ff8000000000000LL), rv = ru;
    if (c >= 0 && c < p.num_cameras && j >= 0 && j < p.num_points) {
      const double X[3] = {p.points[3 * (size_t)j], p.points[3 * (size_t)j + 1], p.points[3 * (size_t)j + 2]};
      const double2 uv = make_double2(p.observations[2 * o], p.observations[2 * o + 1]);
      Proj pr;
      project(tables + (size_t)kCamTable * c, X, uv, pr);
      ru = pr.ru;
      rv = pr.rv;
    }
    if (residuals) {
      residuals[2 * o] = ru;
      residuals[2 * o + 1] = rv;
    }
    cost = block_cost(loss, loss_scale, ru, rv);
  }
  const double s = block_sum(cost, red);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// Fixed-order sum of the partials (same result for the same problem).
__global__ void __launch_bounds__(kNoAllocThreads) k_na_reduce(const double *partials, int n, double *cost) {
  __shared__ double red[kNoAllocThreads / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partials[i];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *cost = s;
}

}  // namespace

// The calling thread's handle-less error message, read by gba_last_error(NULL).
std::string &thread_error_message();

namespace {
gba_status fail(gba_status st, const std::string &msg) {
  thread_error_message() = msg;
  return st;
}
}  // namespace

}  // namespace gba

extern "C" gba_status gba_evaluate_noalloc(const gba_device_problem *p, int32_t loss, double loss_scale,
                                           double *residuals, double *cost, void *stream) {
  using namespace gba;
  if (!p || !cost) return fail(GBA_ERR_INVALID_ARGUMENT, "null problem or cost pointer");
  if (p->num_cameras < 0 || p->num_points < 0 || p->num_observations < 0)
    return fail(GBA_ERR_INVALID_ARGUMENT, "negative problem size");
  if (p->num_cameras > kNoAllocMaxCameras)
    return fail(GBA_ERR_INVALID_ARGUMENT, "gba_evaluate_noalloc: more than 16384 cameras (fixed scratch limit)");
  if (p->num_observations > kNoAllocMaxObservations)
    return fail(GBA_ERR_INVALID_ARGUMENT,
                "gba_evaluate_noalloc: more than 16777216 observations (fixed scratch limit)");
  if (loss < GBA_LOSS_TRIVIAL || loss > GBA_LOSS_CAUCHY || !(loss_scale > 0.0))
    return fail(GBA_ERR_INVALID_ARGUMENT, "invalid loss");
  if (p->num_observations > 0 && (!p->camera_index || !p->point_index || !p->observations || !p->cameras ||
                                  (p->num_points > 0 && !p->points)))
    return fail(GBA_ERR_INVALID_ARGUMENT, "null device array");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(GBA_ERR_NO_DEVICE, "no current CUDA device");
  }
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        cudaGetLastError();
        return fail(e == cudaErrorNoKernelImageForDevice ? GBA_ERR_NO_DEVICE : GBA_ERR_CUDA,
                    std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
      g_scratch_ptr[dev] = static_cast<double *>(ptr);
    }
    scratch = g_scratch_ptr[dev];
  }
  double *tables = scratch;
  double *partials = scratch + (size_t)kNoAllocMaxCameras * kCamTable;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblocks = (p->num_observations + kNoAllocThreads - 1) / kNoAllocThreads;
  if (p->num_cameras > 0) k_na_tables<<<(p->num_cameras + 127) / 128, 128, 0, s>>>(p->cameras, p->num_cameras, tables);
  if (nblocks > 0)
    k_na_residuals<<<nblocks, kNoAllocThreads, 0, s>>>(*p, tables, loss, loss_scale, residuals, partials);
  k_na_reduce<<<1, kNoAllocThreads, 0, s>>>(partials, nblocks, cost);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GBA_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return GBA_OK;
}
