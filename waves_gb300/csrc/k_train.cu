// Training of the learned warm start on the GPU (no reference counterpart): forward, backward and
// Adam kernels for the 4-layer 3x3x3 convolution network of k_net.cu (3 -> 16 -> 16 -> 16 -> 1
// channels, ReLU after the first three layers), on a batch of crops with zero padding at the crop
// edge.  Inputs, weights and the activations between layers are rounded to BF16 as in the
// inference kernels; products accumulate in FP32 in the forward pass and in FP64 in the weight and
// input gradients (the gradient passes through the roundings unchanged).
//
// Layout (one crop after another): x[b][3][z][y][x]; activations and pre-activations [b][c][z][y][x];
// weights [co][27][ci] with tap t = (kz * 3 + ky) * 3 + kx at offset (kx - 1, ky - 1, kz - 1).
// Loss: sum mask (y - target)^2 / max(sum mask, 1).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/waves.h"

namespace {

constexpr int NTT = 256;
constexpr int kLayers = 4;
constexpr int kIn[kLayers] = {3, 16, 16, 16};
constexpr int kOut[kLayers] = {16, 16, 16, 1};

struct Crop {
  int B, nz, ny, nx;
  long long C;  // cells per crop
  __host__ __device__ long long at(int x, int y, int z) const { return ((long long)z * ny + y) * nx + x; }
};

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__global__ void __launch_bounds__(NTT) k_tr_round(const float* src, float* dst, long long n) {
  const long long i = (long long)blockIdx.x * NTT + threadIdx.x;
  if (i < n) dst[i] = bf16r(src[i]);
}

// z[b][co][cell] = bias + sum_t sum_ci w[co][t][ci] a[b][ci][cell + off_t]; with a_next, also the
// BF16-rounded ReLU activation.  One thread per output element.
__global__ void __launch_bounds__(NTT) k_tr_forward(const Crop S, int ci_n, int co_n, const float* __restrict__ a,
                                                   const float* __restrict__ wb, const float* __restrict__ bias,
                                                   float* __restrict__ z, float* __restrict__ a_next) {
  const long long idx = (long long)blockIdx.x * NTT + threadIdx.x;
  if (idx >= (long long)S.B * co_n * S.C) return;
  const long long cell = idx % S.C, bc = idx / S.C;
  const int co = (int)(bc % co_n), b = (int)(bc / co_n);
  const int xx = (int)(cell % S.nx), yy = (int)((cell / S.nx) % S.ny), zz = (int)(cell / ((long long)S.nx * S.ny));
  float acc = bias[co];
  for (int t = 0; t < 27; t++) {
    const int qx = xx + t % 3 - 1, qy = yy + (t / 3) % 3 - 1, qz = zz + t / 9 - 1;
    if (qx < 0 || qy < 0 || qz < 0 || qx >= S.nx || qy >= S.ny || qz >= S.nz) continue;
    const float* w = wb + ((long long)co * 27 + t) * ci_n;
    const float* in = a + (long long)b * ci_n * S.C + S.at(qx, qy, qz);
    for (int ci = 0; ci < ci_n; ci++) acc += w[ci] * in[(long long)ci * S.C];
  }
  z[idx] = acc;
  if (a_next) a_next[idx] = bf16r(acc > 0.f ? acc : 0.f);
}

// dL/dy = 2 mask (y - target) / norm per cell; the loss sum in FP64 (one atomic per block).
__global__ void __launch_bounds__(NTT) k_tr_loss(long long n, const float* __restrict__ y, const float* __restrict__ t,
                                                const float* __restrict__ m, double norm, float* __restrict__ g,
                                                double* loss) {
  __shared__ double part[NTT];
  const long long i = (long long)blockIdx.x * NTT + threadIdx.x;
  double l = 0.0;
  if (i < n) {
    const double d = (double)y[i] - (double)t[i];
    l = (double)m[i] * d * d;
    g[i] = (float)(2.0 * (double)m[i] * d / norm);
  }
  part[threadIdx.x] = l;
  __syncthreads();
  for (int s = NTT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, part[0] / norm);
}

// dL/dW[co][t][ci] = sum_b sum_cell g[b][co][cell] a[b][ci][cell + off_t]: one block per weight;
// blockIdx.x == co_n * 27 * ci_n + co gives dL/db[co] = sum g[b][co][cell].
__global__ void __launch_bounds__(NTT) k_tr_grad_w(const Crop S, int ci_n, int co_n, const float* __restrict__ g,
                                                  const float* __restrict__ a, float* __restrict__ gw,
                                                  float* __restrict__ gb) {
  __shared__ double part[NTT];
  const int nw = co_n * 27 * ci_n;
  const int k = blockIdx.x;
  const bool is_bias = k >= nw;
  const int co = is_bias ? k - nw : k / (27 * ci_n);
  const int t = is_bias ? 13 : (k / ci_n) % 27, ci = is_bias ? 0 : k % ci_n;
  const int ox = t % 3 - 1, oy = (t / 3) % 3 - 1, oz = t / 9 - 1;
  double s = 0.0;
  const long long n = (long long)S.B * S.C;
  for (long long j = threadIdx.x; j < n; j += NTT) {
    const long long cell = j % S.C;
    const int b = (int)(j / S.C);
    const float gv = g[((long long)b * co_n + co) * S.C + cell];
    if (is_bias) {
      s += gv;
      continue;
    }
    const int xx = (int)(cell % S.nx), yy = (int)((cell / S.nx) % S.ny), zz = (int)(cell / ((long long)S.nx * S.ny));
    const int qx = xx + ox, qy = yy + oy, qz = zz + oz;
    if (qx < 0 || qy < 0 || qz < 0 || qx >= S.nx || qy >= S.ny || qz >= S.nz) continue;
    s += (double)gv * (double)a[((long long)b * ci_n + ci) * S.C + S.at(qx, qy, qz)];
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int h = NTT / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (is_bias) gb[co] = (float)part[0];
    else gw[k] = (float)part[0];
  }
}

// dL/da[b][ci][cell] = sum_t sum_co w[co][t][ci] g[b][co][cell - off_t], through the ReLU of the
// layer below (zero where its pre-activation z_prev <= 0).
__global__ void __launch_bounds__(NTT) k_tr_grad_a(const Crop S, int ci_n, int co_n, const float* __restrict__ g,
                                                  const float* __restrict__ wb, const float* __restrict__ z_prev,
                                                  float* __restrict__ ga) {
  const long long idx = (long long)blockIdx.x * NTT + threadIdx.x;
  if (idx >= (long long)S.B * ci_n * S.C) return;
  if (!(z_prev[idx] > 0.f)) {
    ga[idx] = 0.f;
    return;
  }
  const long long cell = idx % S.C, bc = idx / S.C;
  const int ci = (int)(bc % ci_n), b = (int)(bc / ci_n);
  const int xx = (int)(cell % S.nx), yy = (int)((cell / S.nx) % S.ny), zz = (int)(cell / ((long long)S.nx * S.ny));
  double s = 0.0;
  for (int t = 0; t < 27; t++) {
    const int ox = xx - (t % 3 - 1), oy = yy - ((t / 3) % 3 - 1), oz = zz - (t / 9 - 1);
    if (ox < 0 || oy < 0 || oz < 0 || ox >= S.nx || oy >= S.ny || oz >= S.nz) continue;
    const float* gsrc = g + (long long)b * co_n * S.C + S.at(ox, oy, oz);
    for (int co = 0; co < co_n; co++)
      s += (double)wb[((long long)co * 27 + t) * ci_n + ci] * (double)gsrc[(long long)co * S.C];
  }
  ga[idx] = (float)s;
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected) on the FP32 master parameters.
__global__ void __launch_bounds__(NTT) k_tr_adam(long long n, float* __restrict__ w, const float* __restrict__ g,
                                                float* __restrict__ m, float* __restrict__ v, float lr, float c1,
                                                float c2) {
  const long long i = (long long)blockIdx.x * NTT + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = 0.9f * m[i] + 0.1f * gi, vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

unsigned blocks(long long n) { return (unsigned)((n + NTT - 1) / NTT); }

// Device state of one training run: the batch, the FP32 master parameters with their BF16
// roundings, gradients and Adam moments, and the per-layer activations.
struct Trainer {
  Crop S{};
  double norm = 1.0;
  std::vector<void*> allocs;
  float *x = nullptr, *t = nullptr, *m = nullptr, *g = nullptr, *ga = nullptr;
  float *w[kLayers] = {}, *wb[kLayers] = {}, *b[kLayers] = {}, *gw[kLayers] = {}, *gb[kLayers] = {};
  float *mw[kLayers] = {}, *vw[kLayers] = {}, *mb[kLayers] = {}, *vb[kLayers] = {};
  float *a[kLayers] = {}, *z[kLayers] = {};
  double* loss = nullptr;
  cudaError_t err = cudaSuccess;

  template <class T> T* alloc(size_t count) {
    void* p = nullptr;
    if (err == cudaSuccess) err = cudaMalloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 16);
    if (err == cudaSuccess) {
      allocs.push_back(p);
      err = cudaMemset(p, 0, count * sizeof(T));
    }
    return (T*)p;
  }
  ~Trainer() {
    for (void* p : allocs) cudaFree(p);
  }
  static size_t nw(int l) { return (size_t)kOut[l] * 27 * kIn[l]; }

  waves_status setup(const waves_net_batch* bt, const float* const* weights, const float* const* bias) {
    S = Crop{bt->crops, bt->nz, bt->ny, bt->nx, (long long)bt->nz * bt->ny * bt->nx};
    const size_t cells = (size_t)S.B * S.C;
    x = alloc<float>(3 * cells);
    t = alloc<float>(cells);
    m = alloc<float>(cells);
    g = alloc<float>(16 * cells);
    ga = alloc<float>(16 * cells);
    loss = alloc<double>(1);
    a[0] = alloc<float>(3 * cells);
    for (int l = 0; l < kLayers; l++) {
      if (l > 0) a[l] = alloc<float>(16 * cells);
      z[l] = alloc<float>((size_t)kOut[l] * cells);
      w[l] = alloc<float>(nw(l));
      wb[l] = alloc<float>(nw(l));
      gw[l] = alloc<float>(nw(l));
      mw[l] = alloc<float>(nw(l));
      vw[l] = alloc<float>(nw(l));
      b[l] = alloc<float>(kOut[l]);
      gb[l] = alloc<float>(kOut[l]);
      mb[l] = alloc<float>(kOut[l]);
      vb[l] = alloc<float>(kOut[l]);
    }
    if (err != cudaSuccess) return err == cudaErrorMemoryAllocation ? WAVES_OUT_OF_MEMORY : WAVES_CUDA_ERROR;
    double msum = 0.0;
    for (size_t k = 0; k < cells; k++) msum += bt->mask[k];
    norm = msum > 1.0 ? msum : 1.0;
    cudaMemcpy(x, bt->x, 3 * cells * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(t, bt->target, cells * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m, bt->mask, cells * sizeof(float), cudaMemcpyHostToDevice);
    for (int l = 0; l < kLayers; l++) {
      cudaMemcpy(w[l], weights[l], nw(l) * sizeof(float), cudaMemcpyHostToDevice);
      cudaMemcpy(b[l], bias[l], kOut[l] * sizeof(float), cudaMemcpyHostToDevice);
    }
    k_tr_round<<<blocks(3 * cells), NTT>>>(x, a[0], (long long)(3 * cells));
    return cudaGetLastError() == cudaSuccess ? WAVES_OK : WAVES_CUDA_ERROR;
  }
  // forward + loss + backward: gradients in gw/gb, the loss in *loss
  void pass() {
    const long long cells = (long long)S.B * S.C;
    for (int l = 0; l < kLayers; l++) k_tr_round<<<blocks((long long)nw(l)), NTT>>>(w[l], wb[l], (long long)nw(l));
    for (int l = 0; l < kLayers; l++)
      k_tr_forward<<<blocks(cells * kOut[l]), NTT>>>(S, kIn[l], kOut[l], a[l], wb[l], b[l], z[l],
                                                      l + 1 < kLayers ? a[l + 1] : nullptr);
    cudaMemsetAsync(loss, 0, sizeof(double));
    k_tr_loss<<<blocks(cells), NTT>>>(cells, z[kLayers - 1], t, m, norm, g, loss);
    for (int l = kLayers - 1; l >= 0; l--) {
      k_tr_grad_w<<<(unsigned)(nw(l) + kOut[l]), NTT>>>(S, kIn[l], kOut[l], g, a[l], gw[l], gb[l]);
      if (l == 0) break;
      k_tr_grad_a<<<blocks(cells * kIn[l]), NTT>>>(S, kIn[l], kOut[l], g, wb[l], z[l - 1], ga);
      std::swap(g, ga);
    }
  }
  void adam(int step, float lr) {
    const float c1 = 1.f - powf(0.9f, (float)step), c2 = 1.f - powf(0.999f, (float)step);
    for (int l = 0; l < kLayers; l++) {
      k_tr_adam<<<blocks((long long)nw(l)), NTT>>>((long long)nw(l), w[l], gw[l], mw[l], vw[l], lr, c1, c2);
      k_tr_adam<<<blocks(kOut[l]), NTT>>>(kOut[l], b[l], gb[l], mb[l], vb[l], lr, c1, c2);
    }
  }
};

bool batch_ok(const waves_net_batch* bt) {
  return bt && bt->crops >= 1 && bt->nz >= 1 && bt->ny >= 1 && bt->nx >= 1 && bt->x && bt->target && bt->mask &&
         (double)bt->crops * bt->nz * bt->ny * bt->nx * 16 < 2e9;
}

}  // namespace

extern "C" {

waves_status waves_net_gradients(const waves_net_batch* batch, const float* const* weights, const float* const* bias,
                                 double* loss, float* const* grad_w, float* const* grad_b, float* y, int32_t device) {
  if (!batch_ok(batch) || !weights || !bias || !loss || !grad_w || !grad_b) return WAVES_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return WAVES_NO_DEVICE;
  }
  Trainer tr;
  waves_status st = tr.setup(batch, weights, bias);
  if (st != WAVES_OK) return st;
  tr.pass();
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return WAVES_CUDA_ERROR;
  cudaMemcpy(loss, tr.loss, sizeof(double), cudaMemcpyDeviceToHost);
  for (int l = 0; l < kLayers; l++) {
    cudaMemcpy(grad_w[l], tr.gw[l], Trainer::nw(l) * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(grad_b[l], tr.gb[l], kOut[l] * sizeof(float), cudaMemcpyDeviceToHost);
  }
  if (y) cudaMemcpy(y, tr.z[kLayers - 1], (size_t)tr.S.B * tr.S.C * sizeof(float), cudaMemcpyDeviceToHost);
  return cudaGetLastError() == cudaSuccess ? WAVES_OK : WAVES_CUDA_ERROR;
}

waves_status waves_net_train(const waves_net_batch* batch, float* const* weights, float* const* bias, int32_t iterations,
                             float learning_rate, double* loss_history, int32_t device) {
  if (!batch_ok(batch) || !weights || !bias || iterations < 0 || !(learning_rate > 0.f)) return WAVES_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return WAVES_NO_DEVICE;
  }
  Trainer tr;
  waves_status st = tr.setup(batch, weights, bias);
  if (st != WAVES_OK) return st;
  for (int it = 0; it < iterations; it++) {
    tr.pass();
    if (loss_history) cudaMemcpy(&loss_history[it], tr.loss, sizeof(double), cudaMemcpyDeviceToHost);
    tr.adam(it + 1, learning_rate);
  }
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return WAVES_CUDA_ERROR;
  for (int l = 0; l < kLayers; l++) {
    cudaMemcpy(weights[l], tr.w[l], Trainer::nw(l) * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(bias[l], tr.b[l], kOut[l] * sizeof(float), cudaMemcpyDeviceToHost);
  }
  return cudaGetLastError() == cudaSuccess ? WAVES_OK : WAVES_CUDA_ERROR;
}

}  // extern "C"
