// Liquid volume without any device allocation.
//
// Some hosts cannot let this library call cudaMalloc: an engine integration in which every GPU
// buffer is created by the engine (e.g. a Godot RenderingDevice that shares its buffers with the
// renderer and owns their lifetime), and real-time callers that size all device memory at start-up
// and must not allocate inside a frame, because cudaMalloc can synchronise the whole device.
// waves_liquid_volume_noalloc serves them: the caller passes the fraction field and the result
// slot in its own device memory, and the reduction's scratch (per-block partial sums and the
// last-block counter) lives in the file-scope array below, which every GPU that loads the library
// holds until the process exits (64 KiB of partials plus one counter).
//
// The arithmetic and the order of every addition are those of the solver's initial-volume
// reduction (ops 41/42, coupled_motion.glslinc:356-357; k_init_volume through last_block_reduce):
// per cell double(F) * (double(hx)*double(hy)*double(hz)), 256 cells per block reduced by
// block_reduce_k, the last block to finish adding the partials with the same strided loop and
// block_reduce_k — so the result is bit-identical to the solver's initial_volume_m3 for the same F.
#include <mutex>

#include "../../include/waves.h"
#include "common.cuh"

namespace wg {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 8192;  // => at most 2,097,152 cells per call

// Shared by every call on a device: partial sums, then the last-block counter.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxBlocks + 32];

__global__ void __launch_bounds__(kNoAllocThreads)
k_volume_noalloc(const float* __restrict__ F, long long n, double cell, double* out, double* part,
                 unsigned int* counter) {
  __shared__ double sh[kNoAllocThreads];
  __shared__ double tot[1];
  __shared__ bool am_last;
  const int ops[1] = {0};
  const int nb = gridDim.x;
  long long i = (long long)blockIdx.x * kNoAllocThreads + threadIdx.x;
  double v[1] = {0};
  if (i < n) v[0] = (double)F[i] * cell;
  block_reduce_k<kNoAllocThreads, 1>(v, ops, sh, tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot[0];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = atomicAdd(counter, 1u) == (unsigned)nb - 1;
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double acc[1] = {0.0};
  for (int b = threadIdx.x; b < nb; b += kNoAllocThreads) acc[0] = acc[0] + __ldcg(&part[b]);
  block_reduce_k<kNoAllocThreads, 1>(acc, ops, sh, tot);
  if (threadIdx.x == 0) {
    *out = tot[0];
    *counter = 0;
  }
}

// The scratch address is a property of a CUDA context (the module is loaded per context), so the
// cache is keyed by device ordinal and the driver's context id, which is never reused within a
// process: after cudaDeviceReset, or with another context current on the device, the address is
// fetched again.  The driver's entry points are looked up through the runtime, so the library
// does not link libcuda.  Where the driver offers no context id, the key is the ordinal alone.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

struct ScratchEntry {
  int dev;
  unsigned long long ctx_id;
  double* ptr;
};
constexpr int kCacheSlots = 64;

std::mutex g_noalloc_mutex;
ScratchEntry g_cache[kCacheSlots];
int g_cache_used = 0, g_cache_next = 0;
bool g_entry_points_tried = false;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

void* driver_entry(const char* name) {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return f;
}

// Id of the context current on this thread (0 when none is current or the driver has no ids).
unsigned long long current_context_id() {
  if (!g_entry_points_tried) {
    g_entry_points_tried = true;
    g_ctx_get_current = (CtxGetCurrentFn)driver_entry("cuCtxGetCurrent");
    g_ctx_get_id = (CtxGetIdFn)driver_entry("cuCtxGetId");
  }
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != 0 || !ctx) return 0;
  if (g_ctx_get_id(ctx, &id) != 0) return 0;
  return id;
}

// Device address of g_noalloc_scratch in the current context of device `dev` (null on error).
double* scratch_address(int dev) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  unsigned long long id = current_context_id();
  if (id != 0) {
    for (int k = 0; k < g_cache_used; k++)
      if (g_cache[k].dev == dev && g_cache[k].ctx_id == id) return g_cache[k].ptr;
  }
  // Set-up: with the device current, fetch the device address of the array.  The host-side name
  // of the array is not a device address.  This also makes the primary context current if no
  // context was, so the id is read again afterwards.
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
    cudaGetLastError();
    return nullptr;
  }
  if (id == 0) id = current_context_id();
  int slot;
  if (g_cache_used < kCacheSlots) slot = g_cache_used++;
  else slot = g_cache_next = (g_cache_next + 1) % kCacheSlots;
  g_cache[slot] = ScratchEntry{dev, id, (double*)p};
  return (double*)p;
}

}  // namespace
}  // namespace wg

extern "C" waves_status waves_liquid_volume_noalloc(const float* F, int32_t nx, int32_t ny, int32_t nz, float hx, float hy,
                                                    float hz, double* out, void* stream) {
  using namespace wg;
  if (!F || !out || nx < 1 || ny < 1 || nz < 1 || !(hx > 0) || !(hy > 0) || !(hz > 0)) return WAVES_INVALID_ARG;
  long long n = (long long)nx * ny * nz;
  long long blocks = (n + kNoAllocThreads - 1) / kNoAllocThreads;
  if (blocks > kNoAllocMaxBlocks) return WAVES_INVALID_ARG;  // more than 2,097,152 cells
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
    cudaGetLastError();
    return WAVES_NO_DEVICE;
  }
  double* scratch = scratch_address(dev);
  if (!scratch) return WAVES_CUDA_ERROR;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int* counter = (unsigned int*)(scratch + kNoAllocMaxBlocks);
  // The counter must start at zero; the partials are all overwritten before they are read.
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned int), s) != cudaSuccess) return WAVES_CUDA_ERROR;
  double cell = double(hx) * double(hy) * double(hz);
  k_volume_noalloc<<<(unsigned)blocks, kNoAllocThreads, 0, s>>>(F, n, cell, out, scratch, counter);
  return cudaGetLastError() == cudaSuccess ? WAVES_OK : WAVES_CUDA_ERROR;
}
