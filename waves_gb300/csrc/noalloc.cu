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
// The arithmetic is that of the initial-volume reduction of the solver (ops 41/42,
// coupled_motion.glslinc:356-357): sum over cells of double(F) * (double(hx)*double(hy)*double(hz)),
// 256 cells per block, blocks reduced in a fixed tree, the last block to finish adding the
// partials in block order — so the result is bit-identical to the solver's initial_volume_m3 for
// the same F.
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
  __shared__ double sh[32];
  __shared__ bool am_last;
  long long i = (long long)blockIdx.x * kNoAllocThreads + threadIdx.x;
  double v = i < n ? (double)F[i] * cell : 0.0;
  double r = block_reduce<kNoAllocThreads>(v, AddD(), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double acc = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kNoAllocThreads) acc += __ldcg(&part[b]);
  double total = block_reduce<kNoAllocThreads>(acc, AddD(), sh);
  if (threadIdx.x == 0) {
    *out = total;
    *counter = 0;
  }
}

std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[64] = {nullptr};

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
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return WAVES_NO_DEVICE;
  double* scratch;
  {
    // Set-up on the first call per device, with that device current: the host-side name of the
    // array is not a device address, so fetch the device address once and keep it.
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return WAVES_CUDA_ERROR;
      }
      g_noalloc_ptr[dev] = (double*)p;
    }
    scratch = g_noalloc_ptr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int* counter = (unsigned int*)(scratch + kNoAllocMaxBlocks);
  // The counter must start at zero; the partials are all overwritten before they are read.
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned int), s) != cudaSuccess) return WAVES_CUDA_ERROR;
  double cell = double(hx) * double(hy) * double(hz);
  k_volume_noalloc<<<(unsigned)blocks, kNoAllocThreads, 0, s>>>(F, n, cell, out, scratch, counter);
  return cudaGetLastError() == cudaSuccess ? WAVES_OK : WAVES_CUDA_ERROR;
}
