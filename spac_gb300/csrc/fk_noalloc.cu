// Point solves that allocate nothing (fk_solve_points_noalloc).
//
// Some callers cannot call cudaMalloc at solve time: code running while a
// CUDA stream is being captured, embedders that pre-reserve all device memory
// and forbid later allocations, or hosts with a strict real-time budget where
// an allocation (and the device synchronisation it may imply) is not
// acceptable.  This entry point runs the same path and finalize kernels as
// fk_solve_points, but every piece of scratch memory it needs -- the BVP
// record, the per-point item records, the work chunks, the work counter and
// the per-point FP64 sums -- lives in one file-scope __device__ array of
// kNoAllocBytes (4 MiB), which every GPU that loads the library holds until
// the process exits.  Inputs and outputs are device buffers owned by the
// caller; there is no context, no stream creation and no host staging buffer.
//
// The array's host-side name is only a stand-in for the device symbol, so
// its device address is obtained once per device with cudaGetSymbolAddress
// (on the first call made on that device, which should therefore happen
// before any stream capture) and cached.  All calls share the array: the
// parts that must start at zero are cleared on every call, and two calls
// whose kernels overlap on the GPU (different streams, no ordering) race on
// it and give wrong results.
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/spac_fk.h"
#include "fk_device.cuh"
#include "fk_internal.h"

namespace fk {
namespace {

constexpr size_t kNoAllocBytes = 4u << 20;
constexpr size_t kBvpOff = 0;
constexpr size_t kQueueOff = 256;
constexpr size_t kItemsOff = 512;
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kChunksOff = align256(kItemsOff + sizeof(ItemDev) * FK_NOALLOC_MAX_POINTS);
constexpr size_t kStatsOff = align256(kChunksOff + sizeof(ChunkDev) * FK_NOALLOC_MAX_POINTS);
constexpr size_t kEnd = kStatsOff + sizeof(double) * kNumStats * FK_NOALLOC_MAX_POINTS;
static_assert(kEnd <= kNoAllocBytes, "no-alloc scratch layout exceeds the reserved array");
static_assert(sizeof(BvpDev) <= kQueueOff - kBvpOff, "BVP record does not fit its slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device (set-up once per device).
cudaError_t scratch_address(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

// Writes the BVP record, one item and one chunk per point (a point's paths
// form one chunk), from the caller's device inputs.
__global__ void noalloc_prepare(BvpDev bvp, int n, const double* xy, const unsigned* paths, const double* h,
                                BvpDev* d_bvp, ItemDev* items, ChunkDev* chunks) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *d_bvp = bvp;
  if (i >= n) return;
  ItemDev it;
  it.x = xy[2 * i];
  it.y = xy[2 * i + 1];
  it.h = h[i];
  it.sqrth = sqrt(h[i]);
  for (int q = 0; q < 4; ++q) it.sub[q] = 0.0;
  it.paths = paths[i];
  it.stencil = -1;
  it.frontera = 0;
  it.sub_shape = -1;
  it.cv_region = 0;
  it.bvp = 0;
  it.acc_off = 0;
  items[i] = it;
  chunks[i] = ChunkDev{i, 0u, paths[i]};
}

}  // namespace
}  // namespace fk

extern "C" int fk_solve_points_noalloc(const fk_bvp_desc* d, unsigned long long seed, unsigned stream_id, int n,
                                       const double* d_xy, const unsigned* d_paths, const double* d_h, int precision,
                                       int max_steps, void* cuda_stream, fk_stats* d_out) {
  using namespace fk;
  if (!d || n < 0 || (n > 0 && (!d_xy || !d_paths || !d_h || !d_out))) return FK_ERR_ARG;
  if (n > FK_NOALLOC_MAX_POINTS) return FK_ERR_CAPACITY;  // beyond the reserved scratch array
  if (d->problem < 0 || d->problem > 4 || d->cv < FK_CV_NONE || d->cv > FK_CV_EXACT) return FK_ERR_ARG;
  if (d->problem == FK_PROBLEM_ROBIN &&
      !(d->prob[0] >= 0 && d->prob[0] <= 15 && d->prob[0] == std::floor(d->prob[0]) && d->prob[2] >= 0))
    return FK_ERR_ARG;
  if (d->dom_shape != ((d->problem == FK_PROBLEM_DISK) ? FK_SHAPE_CIRCLE : FK_SHAPE_RECT)) return FK_ERR_ARG;
  if (precision != FK_FP64 && precision != FK_FP32) return FK_ERR_ARG;
  if (max_steps < 1 || max_steps > (1 << 30)) return FK_ERR_ARG;
  for (int i = 0; i < 4; ++i)
    if (!std::isfinite(d->dom[i]) || !std::isfinite(d->prob[i])) return FK_ERR_ARG;
  if (n == 0) return FK_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FK_ERR_NO_DEVICE;
  unsigned char* base = nullptr;
  if (scratch_address(dev, &base) != cudaSuccess) return FK_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  BvpDev b;
  std::memset(&b, 0, sizeof(b));
  b.problem = d->problem;
  b.cv = d->cv;
  b.dom_shape = d->dom_shape;
  b.mlp = -1;
  for (int i = 0; i < 4; ++i) { b.dom[i] = d->dom[i]; b.prob[i] = d->prob[i]; }
  BvpDev* d_bvp = reinterpret_cast<BvpDev*>(base + kBvpOff);
  int* d_queue = reinterpret_cast<int*>(base + kQueueOff);
  ItemDev* d_items = reinterpret_cast<ItemDev*>(base + kItemsOff);
  ChunkDev* d_chunks = reinterpret_cast<ChunkDev*>(base + kChunksOff);
  double* d_stats = reinterpret_cast<double*>(base + kStatsOff);
  // the work counter and the FP64 sums start at zero on every call
  if (cudaMemsetAsync(d_queue, 0, 2 * sizeof(int), s) != cudaSuccess) return FK_ERR_CUDA;
  if (cudaMemsetAsync(d_stats, 0, sizeof(double) * kNumStats * n, s) != cudaSuccess) return FK_ERR_CUDA;
  noalloc_prepare<<<(n + 127) / 128, 128, 0, s>>>(b, n, d_xy, d_paths, d_h, d_bvp, d_items, d_chunks);
  if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;

  LaunchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.acc_zeroed = 1;  // (point solves: no stencil moments)
  a.bvp = d_bvp;
  a.items = d_items;
  a.chunks = d_chunks;
  a.n_chunks = n;
  a.queue = d_queue;
  a.stats = d_stats;
  a.key0 = static_cast<uint32_t>(seed);
  a.key1 = static_cast<uint32_t>(seed >> 32);
  a.stream = stream_id;
  a.max_steps = max_steps;
  a.cv = (d->cv == FK_CV_EXACT) ? 1 : 0;
  a.stencil_kind = 0;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FK_ERR_CUDA;
  const int block = 256;
  const int occ = paths_kernel_occupancy(d->problem, precision, 0, a.cv, block, 0);
  if (launch_paths(a, d->problem, precision, sms * occ, block, 0, s) != cudaSuccess) return FK_ERR_CUDA;

  FinalizeArgs f;
  std::memset(&f, 0, sizeof(f));
  f.bvp = d_bvp;
  f.items = d_items;
  f.n_items = n;
  f.stats = d_stats;
  f.stencil_kind = 0;
  f.item_stats = reinterpret_cast<double*>(d_out);
  if (launch_finalize(f, d->problem, s) != cudaSuccess) return FK_ERR_CUDA;
  return FK_OK;
}
