// Point solves that allocate nothing (fk_solve_points_noalloc).
//
// Some callers cannot call cudaMalloc when they solve: embedders that reserve
// all device memory up front and forbid later allocations (a framework's
// caching allocator owns the GPU), and hosts with a strict real-time budget,
// where an allocation and the device synchronisation it may imply are not
// acceptable.  This entry point runs the same path and finalize kernels as
// fk_solve_points, but every piece of scratch memory it needs -- the BVP
// record, the per-point item records, the work chunks and their count, the
// work counter and status words, and the per-point FP64 sums -- lives in one
// file-scope __device__ array of kNoAllocBytes (4 MiB), which every GPU that
// loads the library holds until the process exits.  Inputs and outputs are
// device buffers owned by the caller; there is no context, no stream creation
// and no host staging buffer.
//
// The array's host-side name is only a stand-in for the device symbol, so its
// device address is looked up with cudaGetSymbolAddress on the first call
// made in each CUDA context (once per device for the usual primary context;
// again after cudaDeviceReset) and cached with that context's id.  All calls
// share the array: the parts that must start at zero are cleared on every
// call, and two calls whose kernels overlap on the GPU (different streams, no
// ordering) race on it and give wrong results.
//
// The work chunks are built on the device from the caller's path counts (the
// host never sees them): every point is split into chunks of equal size so
// that one point with many paths spreads over the whole persistent grid, as
// in fk_solve_points, with the chunk size raised where needed to keep the
// chunk count within the array's kNoAllocMaxChunks.
#include <cuda.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/spac_fk.h"
#include "fk_device.cuh"
#include "fk_internal.h"

namespace fk {
namespace {

constexpr size_t kNoAllocBytes = 4u << 20;
constexpr int kNoAllocMaxChunks = 65536;
constexpr int kPrepThreads = 1024;
constexpr size_t kBvpOff = 0;
constexpr size_t kQueueOff = 256;  // [0] chunk counter, [1] error word, [2..3] result flags, [4] chunk count
constexpr size_t kItemsOff = 512;
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kChunksOff = align256(kItemsOff + sizeof(ItemDev) * FK_NOALLOC_MAX_POINTS);
constexpr size_t kStatsOff = align256(kChunksOff + sizeof(ChunkDev) * kNoAllocMaxChunks);
constexpr size_t kEnd = kStatsOff + sizeof(double) * kNumStats * FK_NOALLOC_MAX_POINTS;
static_assert(kEnd <= kNoAllocBytes, "no-alloc scratch layout exceeds the reserved array");
static_assert(sizeof(BvpDev) <= kQueueOff - kBvpOff, "BVP record does not fit its slot");
static_assert(FK_NOALLOC_MAX_POINTS <= 16 * kPrepThreads, "prepare kernel covers at most 16 points per thread");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Scratch address per CUDA context, keyed by the context's unique id (a
// context created after cudaDeviceReset gets a new id, and the module, with
// the array, may load at another address there).
constexpr int kMaxDevices = 64;
struct ScratchCache {
  unsigned long long ctx_id = 0;
  unsigned char* ptr = nullptr;
};
ScratchCache g_scratch[kMaxDevices];
std::mutex g_scratch_mu;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Id of the current CUDA context (0 if it cannot be read: then the address
// is looked up on every call).
unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
    cudaGetLastError();
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the scratch array in the current context (set-up once per
// context; the device must already be current).  cudaGetSymbolAddress also
// makes the device's primary context current if no context is yet, so the
// context id is read after it.
cudaError_t scratch_address(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  ScratchCache& c = g_scratch[dev];
  const unsigned long long id = current_ctx_id();
  if (id == 0 || c.ctx_id != id || !c.ptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    c.ptr = static_cast<unsigned char*>(p);
    c.ctx_id = current_ctx_id();
  }
  *out = c.ptr;
  return cudaSuccess;
}

// One CTA of kPrepThreads threads writes the BVP record, one item per point
// and the work chunks: every point's paths in equal chunks of at most `chunk`
// paths (as fk_solve_points splits them), where `chunk` is about a quarter of
// the paths per CTA of the grid, 256..32768, and large enough that the chunk
// count stays within kNoAllocMaxChunks.  Thread t covers points
// [t*per, (t+1)*per): their chunk counts are scanned across the CTA.
__global__ void __launch_bounds__(kPrepThreads) noalloc_prepare(BvpDev bvp, int n, const double* xy,
                                                                const unsigned* paths, const double* h, int grid,
                                                                BvpDev* d_bvp, ItemDev* items, ChunkDev* chunks,
                                                                int* n_chunks) {
  __shared__ unsigned long long s_total[kPrepThreads / 32];
  __shared__ int s_cnt[kPrepThreads / 32];
  __shared__ long long s_chunk;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int per = (n + kPrepThreads - 1) / kPrepThreads;
  const int i0 = min(n, t * per), i1 = min(n, i0 + per);
  unsigned long long mine = 0;
  for (int i = i0; i < i1; ++i) mine += paths[i];
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if (lane == 0) s_total[warp] = mine;
  __syncthreads();
  if (t == 0) {
    unsigned long long total = 0;
    for (int w = 0; w < kPrepThreads / 32; ++w) total += s_total[w];
    long long c = static_cast<long long>(total / (4ull * static_cast<unsigned long long>(grid)));
    c = c < 256 ? 256 : (c > 32768 ? 32768 : c);
    // each point gives at most paths/chunk + 1 chunks
    const long long room = kNoAllocMaxChunks - n;
    const long long need = static_cast<long long>((total + room - 1) / room);
    s_chunk = c > need ? c : need;
    *d_bvp = bvp;
  }
  __syncthreads();
  const long long chunk = s_chunk;
  // chunk counts of this thread's points, then an exclusive scan over the CTA
  int cnt = 0;
  for (int i = i0; i < i1; ++i) {
    const long long np = paths[i];
    if (np == 0) continue;
    const long long pieces = (np + chunk - 1) / chunk;
    const long long each = (np + pieces - 1) / pieces;
    cnt += static_cast<int>((np + each - 1) / each);
  }
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_cnt[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = s_cnt[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += v;
    }
    s_cnt[lane] = w;  // inclusive totals per warp
  }
  __syncthreads();
  int base = incl - cnt + (warp > 0 ? s_cnt[warp - 1] : 0);
  if (t == kPrepThreads - 1) *n_chunks = base + cnt;
  for (int i = i0; i < i1; ++i) {
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
    const long long np = paths[i];
    if (np == 0) continue;
    const long long pieces = (np + chunk - 1) / chunk;
    const long long each = (np + pieces - 1) / pieces;
    for (long long p0 = 0; p0 < np; p0 += each) {
      const long long p1 = p0 + each < np ? p0 + each : np;
      chunks[base++] = ChunkDev{i, static_cast<unsigned>(p0), static_cast<unsigned>(p1)};
    }
  }
}

}  // namespace
}  // namespace fk

extern "C" int fk_solve_points_noalloc(const fk_bvp_desc* d, unsigned long long seed, unsigned stream_id, int n,
                                       const double* d_xy, const unsigned* d_paths, const double* d_h, int precision,
                                       int max_steps, void* cuda_stream, fk_stats* d_out) {
  using namespace fk;
  if (!d || n < 0 || (n > 0 && (!d_xy || !d_paths || !d_h || !d_out))) return FK_ERR_ARG;
  if (n > FK_NOALLOC_MAX_POINTS) return FK_ERR_CAPACITY;  // beyond the reserved scratch array
  if (d->problem < 0 || d->problem >= kNumProblems || d->cv < FK_CV_NONE || d->cv > FK_CV_EXACT) return FK_ERR_ARG;
  if (d->problem == FK_PROBLEM_ROBIN &&
      !(d->prob[0] >= 0 && d->prob[0] <= 15 && d->prob[0] == std::floor(d->prob[0]) && d->prob[2] >= 0))
    return FK_ERR_ARG;
  if (d->dom_shape != problem_domain_shape(d->problem)) return FK_ERR_ARG;
  if (precision != FK_FP64 && precision != FK_FP32) return FK_ERR_ARG;
  if (max_steps < 1 || max_steps > (1 << 30)) return FK_ERR_ARG;
  for (int i = 0; i < 4; ++i)
    if (!std::isfinite(d->dom[i]) || !std::isfinite(d->prob[i])) return FK_ERR_ARG;
  // as fk_register_bvp: a domain with no inside would run every path to max_steps
  if (d->dom_shape == FK_SHAPE_RECT && !(d->dom[2] > d->dom[0] && d->dom[3] > d->dom[1])) return FK_ERR_ARG;
  if (d->dom_shape == FK_SHAPE_CIRCLE && !(d->dom[0] > 0)) return FK_ERR_ARG;
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
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FK_ERR_CUDA;
  const int block = 256;
  const int cvm = (d->cv == FK_CV_EXACT) ? 1 : 0;
  const int grid = sms * paths_kernel_occupancy(d->problem, precision, 0, cvm, block, 0);
  // the work counter, the status words and the FP64 sums start at zero on every call
  if (cudaMemsetAsync(d_queue, 0, 4 * sizeof(int), s) != cudaSuccess) return FK_ERR_CUDA;
  if (cudaMemsetAsync(d_stats, 0, sizeof(double) * kNumStats * n, s) != cudaSuccess) return FK_ERR_CUDA;
  noalloc_prepare<<<1, kPrepThreads, 0, s>>>(b, n, d_xy, d_paths, d_h, grid, d_bvp, d_items, d_chunks, d_queue + 4);
  if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;

  LaunchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.acc_zeroed = 1;  // (point solves: no stencil moments)
  a.bvp = d_bvp;
  a.items = d_items;
  a.chunks = d_chunks;
  a.n_chunks = 0;
  a.n_chunks_dev = d_queue + 4;
  a.queue = d_queue;
  a.stats = d_stats;
  a.key0 = static_cast<uint32_t>(seed);
  a.key1 = static_cast<uint32_t>(seed >> 32);
  set_round_keys(a);
  a.stream = stream_id;
  a.max_steps = max_steps;
  a.cv = cvm;
  a.any_cv = d->cv != FK_CV_NONE ? 1 : 0;
  a.stencil_kind = 0;
  if (launch_paths(a, d->problem, precision, grid, block, 0, s) != cudaSuccess) return FK_ERR_CUDA;

  FinalizeArgs f;
  std::memset(&f, 0, sizeof(f));
  f.bvp = d_bvp;
  f.items = d_items;
  f.n_items = n;
  f.stats = d_stats;
  f.stencil_kind = 0;
  f.item_stats = reinterpret_cast<double*>(d_out);
  f.flags = d_queue + 2;
  if (launch_finalize(f, d->problem, s) != cudaSuccess) return FK_ERR_CUDA;
  return FK_OK;
}
