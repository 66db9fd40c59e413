// noalloc.cu -- spreading entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: frameworks whose device memory all belongs to
// their own pool allocator (a side allocation can fail once the pool has reserved the
// device, or fragment it), real-time loops that must not pay an allocation's latency
// or risk its failure mid-run, and host applications that forbid allocation inside
// their plug-in callbacks.  For them cunfft_x_spread_noalloc bins the nodes and
// spreads them with the same kernels as cunfft_x_spread, but keeps all of its scratch
// (the sorted node records, per-tile counts and offsets, work items, queue counters
// and the device status word) in one fixed file-scope device array instead of
// plan-owned allocations.
//
// That array is part of the library's device image: every GPU on which the library
// is loaded holds it (about 58 MB) until the process exits.  All calls share it, so
// calls that overlap on the GPU (concurrent streams, or host threads driving the same
// device) race on it and must be serialised by the caller.  Every call rewrites all
// scratch it reads: the per-tile counts, the work-queue counters and the status word
// are cleared on the stream before use.
//
// The array's device address is looked up once per device and cached; a device reset
// (cudaDeviceReset) unloads the module, after which the cached address is stale, so
// the entry point must not be used across a device reset.
#include <mutex>
#include <stdio.h>

#include "runtime.h"

namespace cg {
namespace {

constexpr int64_t kNaMaxNodes = int64_t(1) << 20;   // nodes per call
constexpr int64_t kNaMaxTiles = int64_t(1) << 16;   // grid tiles per call
constexpr int kNaChunk = 1024;                      // nodes per work item
constexpr int64_t kNaMaxItems = kNaMaxTiles + kNaMaxNodes / kNaChunk + 1;

// byte offsets of the scratch regions (each 256-byte aligned)
constexpr size_t na_align(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kOffSidx = 0;
constexpr size_t kOffSoff = na_align(kOffSidx + sizeof(int32_t) * kNaMaxNodes);
constexpr size_t kOffSfrac = na_align(kOffSoff + sizeof(int32_t) * kNaMaxNodes);
constexpr size_t kOffRank = na_align(kOffSfrac + sizeof(double) * 3 * kNaMaxNodes);
constexpr size_t kOffFperm = na_align(kOffRank + sizeof(int2) * kNaMaxNodes);
constexpr size_t kOffCount = na_align(kOffFperm + sizeof(double) * 2 * kNaMaxNodes);
constexpr size_t kOffTileOff = na_align(kOffCount + sizeof(int32_t) * (kNaMaxTiles + 1));
constexpr size_t kOffItemOff = na_align(kOffTileOff + sizeof(int32_t) * (kNaMaxTiles + 1));
constexpr size_t kOffItems = na_align(kOffItemOff + sizeof(int32_t) * (kNaMaxTiles + 1));
constexpr size_t kOffNumItems = na_align(kOffItems + sizeof(int4) * kNaMaxItems);
constexpr size_t kOffWork = na_align(kOffNumItems + sizeof(int32_t));
constexpr size_t kOffInstOff = na_align(kOffWork + 2 * sizeof(int32_t));
constexpr size_t kOffStatus = na_align(kOffInstOff + 2 * sizeof(int32_t));
constexpr size_t kOffFmax = na_align(kOffStatus + sizeof(int32_t));
constexpr size_t kNaBytes = na_align(kOffFmax + sizeof(uint32_t));

}  // namespace

// The scratch array.  In host code this name is only a stand-in for the device
// object; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

namespace {

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
unsigned char* g_na_ptr[kNaMaxDevices] = {nullptr};

// Device address of the scratch array on the current device, looked up once
// per device (with that device current).
cudaError_t na_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNaMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_na_ptr[dev] = static_cast<unsigned char*>(ptr);
  }
  *out = g_na_ptr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace cg

extern "C" int cunfft_x_spread_noalloc(int d, const int64_t* N, const int64_t* n, int m, int precision, int64_t M,
                                       const double* x, const void* f, void* g, void* stream, int32_t* status) {
  using namespace cg;
  if (!N || M < 0 || (M > 0 && (!x || !f)) || !g) {
    fprintf(stderr, "cunfft_x_spread_noalloc: invalid argument (NULL pointer or M < 0)\n");
    return CUNFFT_X_INVALID_ARGUMENT;
  }
  if (M > kNaMaxNodes) {
    fprintf(stderr, "cunfft_x_spread_noalloc: M = %lld exceeds the fixed scratch limit of %lld nodes\n",
            (long long)M, (long long)kNaMaxNodes);
    return CUNFFT_X_INVALID_ARGUMENT;
  }
  Plan p;  // host-side description only: no stream, grid, FFT plan or buffers are created
  int s = geom_init(&p, d, N, n, m, precision, 1);
  if (s != CUNFFT_X_SUCCESS) {
    fprintf(stderr, "cunfft_x_spread_noalloc: %s\n", p.last_msg);
    return s;
  }
  const int T0[3] = {0, 0, 0};
  s = plan_choose_tiling(&p, T0, kNaChunk);
  if (s != CUNFFT_X_SUCCESS) {
    fprintf(stderr, "cunfft_x_spread_noalloc: %s\n", p.last_msg);
    return s;
  }
  p.tl.sub_on = 0;  // spreading needs the nodes in tile order only: no sub-bins, no room for them
  p.tl.sub_items = 0;
  p.tl.ns = 1;
  if (p.tl.tiles_total > kNaMaxTiles) {
    fprintf(stderr, "cunfft_x_spread_noalloc: the grid needs %lld tiles, beyond the fixed scratch limit of %lld\n",
            (long long)p.tl.tiles_total, (long long)kNaMaxTiles);
    return CUNFFT_X_INVALID_ARGUMENT;
  }
  unsigned char* base = nullptr;
  cudaError_t e = na_scratch(&base);
  if (e != cudaSuccess) {
    fprintf(stderr, "cunfft_x_spread_noalloc: scratch address lookup failed: %s\n", cudaGetErrorString(e));
    return CUNFFT_X_CUDA_ERROR;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the kernels' device status word: the caller's, or the scratch copy; cleared per call
  int32_t* status_word = status ? status : reinterpret_cast<int32_t*>(base + kOffStatus);
  if ((e = cudaMemsetAsync(status_word, 0, sizeof(int32_t), st)) != cudaSuccess) {
    fprintf(stderr, "cunfft_x_spread_noalloc: clearing the status word failed: %s\n", cudaGetErrorString(e));
    return CUNFFT_X_CUDA_ERROR;
  }
  if (M == 0) return CUNFFT_X_SUCCESS;  // nothing to spread: g stays as it is
  Bins& B = p.bins;
  B.sidx = reinterpret_cast<int32_t*>(base + kOffSidx);
  B.soff = reinterpret_cast<int32_t*>(base + kOffSoff);
  B.sfrac = base + kOffSfrac;
  B.tile_rank = reinterpret_cast<int2*>(base + kOffRank);
  B.fperm = base + kOffFperm;
  B.count = reinterpret_cast<int32_t*>(base + kOffCount);
  B.tile_off = reinterpret_cast<int32_t*>(base + kOffTileOff);
  B.item_off = reinterpret_cast<int32_t*>(base + kOffItemOff);
  B.items = reinterpret_cast<int4*>(base + kOffItems);
  B.num_items = reinterpret_cast<int32_t*>(base + kOffNumItems);
  B.work = reinterpret_cast<int32_t*>(base + kOffWork);
  B.inst_off = reinterpret_cast<int32_t*>(base + kOffInstOff);  // unused for one instance
  B.status = status_word;
  B.fmax = reinterpret_cast<uint32_t*>(base + kOffFmax);
  B.M = M;
  B.max_items = kNaMaxItems;
  B.valid = 1;
  p.M = M;
  p.x = x;
  if ((e = launch_binning(p, x, st)) != cudaSuccess || (e = launch_spread(p, f, g, st)) != cudaSuccess) {
    fprintf(stderr, "cunfft_x_spread_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return CUNFFT_X_CUDA_ERROR;
  }
  return CUNFFT_X_SUCCESS;
}
