// Training of the learned warm start on the GPU (no reference counterpart): forward, backward and
// Adam kernels for the 4-layer 3x3x3 convolution network of k_net.cu (3 -> 16 -> 16 -> 16 -> 1
// channels, ReLU after the first three layers), on a batch of crops with zero padding at the crop
// edge.  Inputs, weights and the activations between layers are rounded to BF16 as in the
// inference kernels.  WAVES_NET_EXACT: products accumulate in FP32 in the forward pass (the CPU
// oracle's order) and in FP64 in the weight and input gradients (the gradient passes through the
// roundings unchanged).  WAVES_NET_TENSOR: every convolution and the weight gradient are implicit
// GEMMs on the tensor cores (below).
//
// Layout (one crop after another): x[b][3][z][y][x]; activations and pre-activations [b][c][z][y][x];
// weights [co][27][ci] with tap t = (kz * 3 + ky) * 3 + kx at offset (kx - 1, ky - 1, kz - 1).
// Loss: sum mask (y - target)^2 / max(sum mask, 1).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/waves.h"
#include "mma_bf16.cuh"

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

// dL/dy = 2 mask (y - target) / norm per cell; the loss in FP64: each block writes its partial sum,
// k_tr_loss_sum adds the partials in a fixed order, so the loss is the same bits on every run.
__global__ void __launch_bounds__(NTT) k_tr_loss(long long n, const float* __restrict__ y, const float* __restrict__ t,
                                                const float* __restrict__ m, double norm, float* __restrict__ g,
                                                double* __restrict__ loss_part) {
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
  if (threadIdx.x == 0) loss_part[blockIdx.x] = part[0];
}

// One block: thread j adds partials j, j + NTT, ... in turn, then a fixed tree; loss = sum / norm.
__global__ void __launch_bounds__(NTT) k_tr_loss_sum(long long nparts, const double* __restrict__ loss_part,
                                                    double norm, double* __restrict__ loss) {
  __shared__ double part[NTT];
  double s = 0.0;
  for (long long b = threadIdx.x; b < nparts; b += NTT) s += loss_part[b];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int k = NTT / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) part[threadIdx.x] += part[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = part[0] / norm;
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

// ---- WAVES_NET_TENSOR: implicit GEMM on the tensor cores ----
//
// Operands are BF16 channel-last, [b * C + cell][16] (32 B per cell, absent channels zero); the
// FP32 pre-activations and input gradients stay [b][c][cell] for the ReLU masks and bias sums.
// The convolutions use the tiling of the inference kernels (k_net.cu): a block stages the
// 34 x 6 x 3 halo of 32 x 4 cells of one plane of one crop with a 48-byte cell stride.
constexpr int TX = 32, TY = 4, HX = TX + 2, HY = TY + 2, HZ = 3;
constexpr int kStride = 24;             // bf16 per staged cell: 16 channels + 8 padding
constexpr int kHalo = HX * HY * HZ;     // 612 staged cells
constexpr int kFragWords = 27 * 2 * 64; // B fragments of one layer: [tap][n-tile][lane][2]
constexpr int kPadW = 16 * 27 * 16;     // a weight gradient padded to [16 co][27][16 ci]
constexpr int kSplits = 32;             // FP64 partial sums of the weight-gradient reduction
constexpr int kZChunk = 4;              // planes per block of the weight gradient

// x[b][3][cell] -> BF16 [b * C + cell][16] (channels 3..15 zero)
__global__ void __launch_bounds__(NTT) k_tc_pack_x(const Crop S, const float* __restrict__ x, uint4* __restrict__ act) {
  const long long j = (long long)blockIdx.x * NTT + threadIdx.x;
  if (j >= (long long)S.B * S.C) return;
  const long long b = j / S.C, cell = j % S.C;
  const float* src = x + b * 3 * S.C + cell;
  act[2 * j] = make_uint4(wg::pack_bf16(src[0], src[S.C]), wg::pack_bf16(src[2 * S.C], 0.f), 0u, 0u);
  act[2 * j + 1] = make_uint4(0u, 0u, 0u, 0u);
}

// one-channel g[j] -> BF16 [j][16] (channels 1..15 zero)
__global__ void __launch_bounds__(NTT) k_tc_pack_g1(long long n, const float* __restrict__ g, uint4* __restrict__ g16) {
  const long long j = (long long)blockIdx.x * NTT + threadIdx.x;
  if (j >= n) return;
  g16[2 * j] = make_uint4(wg::pack_bf16(g[j], 0.f), 0u, 0u, 0u);
  g16[2 * j + 1] = make_uint4(0u, 0u, 0u, 0u);
}

// B fragments (layout of include/waves.h's inference weights, always two n-tiles) of one layer:
// transpose 0, the forward pass (n = output channel, k = input channel, tap t); transpose 1, the
// input gradient (n = input channel, k = output channel, tap 26 - t: the mirrored offset).
__global__ void __launch_bounds__(NTT) k_tc_frag(const float* __restrict__ w, int ci_n, int co_n, int transpose,
                                                uint32_t* __restrict__ frag) {
  const int k = blockIdx.x * NTT + threadIdx.x;  // (tap * 2 + j) * 32 + lane
  if (k >= 27 * 2 * 32) return;
  const int lane = k & 31, j = (k >> 5) & 1, tap = k >> 6;
  const int n = 8 * j + (lane >> 2), t = lane & 3;
  auto val = [&](int kk) -> float {
    if (transpose) return (n < ci_n && kk < co_n) ? w[((size_t)kk * 27 + (26 - tap)) * ci_n + n] : 0.f;
    return (n < co_n && kk < ci_n) ? w[((size_t)n * 27 + tap) * ci_n + kk] : 0.f;
  };
  frag[2 * k] = wg::pack_bf16(val(2 * t), val(2 * t + 1));
  frag[2 * k + 1] = wg::pack_bf16(val(2 * t + 8), val(2 * t + 9));
}

// Stage the 34 x 6 x 3 halo of the block's 32 x 4 cells around plane z of one crop.
__device__ __forceinline__ void stage_halo(const Crop& S, const __nv_bfloat16* src_b, int x0, int y0, int z,
                                           __nv_bfloat16* tile) {
  for (int c = threadIdx.x; c < kHalo; c += NTT) {
    const int hx = c % HX, hy = (c / HX) % HY, hz = c / (HX * HY);
    const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z + hz - 1;
    uint4 lo = make_uint4(0u, 0u, 0u, 0u), hi = lo;
    if (gx >= 0 && gx < S.nx && gy >= 0 && gy < S.ny && gz >= 0 && gz < S.nz) {
      const uint4* src = reinterpret_cast<const uint4*>(src_b + (size_t)S.at(gx, gy, gz) * 16);
      lo = src[0];
      hi = src[1];
    }
    uint4* dst = reinterpret_cast<uint4*>(tile + c * kStride);
    dst[0] = lo;
    dst[1] = hi;
  }
}

// Implicit-GEMM 3x3x3 convolution over a batch of crops: a warp owns 16 consecutive x cells and
// issues per tap one ldmatrix.x4 (cells x input channels) and NTILES mma.sync against the tap's
// B fragments.  Grid (ceil(nx / 32), ceil(ny / 4), crops * nz).
//   MODE 0  hidden layer: z = acc + bias, FP32 [b][16][cell], and the BF16 ReLU activation;
//   MODE 1  last layer: y = acc + bias of output channel 0, FP32 [b][cell];
//   MODE 2  input gradient: acc where the layer below's pre-activation z_prev > 0, else 0, FP32
//           [b][16][cell] and BF16.
template <int NTILES, int MODE>
__global__ void __launch_bounds__(NTT) k_tc_conv(const Crop S, const __nv_bfloat16* __restrict__ in,
                                                const uint32_t* __restrict__ frag, const float* __restrict__ bias,
                                                int n_bias, const float* __restrict__ z_prev, float* __restrict__ out,
                                                __nv_bfloat16* __restrict__ out16) {
  __shared__ __align__(16) __nv_bfloat16 tile[kHalo * kStride];
  __shared__ __align__(16) uint32_t wfrag[kFragWords];
  __shared__ float sb[16];
  const int z = blockIdx.z % S.nz, b = blockIdx.z / S.nz;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  for (int k = threadIdx.x; k < kFragWords; k += NTT) wfrag[k] = frag[k];
  if (threadIdx.x < 16) sb[threadIdx.x] = (MODE != 2 && (int)threadIdx.x < n_bias) ? bias[threadIdx.x] : 0.f;
  stage_halo(S, in + (size_t)b * S.C * 16, x0, y0, z, tile);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wx = (warp & 1) * 16, wy = warp >> 1;
  const int row = (lane & 7) + ((lane >> 3) & 1) * 8, half = (lane >> 4) * 8;
  float acc[NTILES][4];
#pragma unroll
  for (int j = 0; j < NTILES; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll 3
  for (int tap = 0; tap < 27; tap++) {
    const int kx = tap % 3, ky = (tap / 3) % 3, kz = tap / 9;
    const int cell = (kz * HY + wy + ky) * HX + wx + kx + row;
    uint32_t a0, a1, a2, a3;
    wg::ldmatrix_x4(a0, a1, a2, a3, tile + cell * kStride + half);
#pragma unroll
    for (int j = 0; j < NTILES; j++) {
      const uint2 bf = *reinterpret_cast<const uint2*>(&wfrag[((tap * 2 + j) * 32 + lane) * 2]);
      wg::mma_bf16(acc[j], a0, a1, a2, a3, bf.x, bf.y);
    }
  }
  const int g = lane >> 2, t = lane & 3;
  const int y = y0 + wy;
#pragma unroll
  for (int hrow = 0; hrow < 2; hrow++) {
    const int x = x0 + wx + g + 8 * hrow;
    if (x >= S.nx || y >= S.ny) continue;
    const long long cell = S.at(x, y, z);
    if constexpr (MODE == 1) {
      if (t == 0) out[(long long)b * S.C + cell] = acc[0][2 * hrow] + sb[0];
    } else {
#pragma unroll
      for (int j = 0; j < NTILES; j++) {
        const int n = j * 8 + 2 * t;
        float v0 = acc[j][2 * hrow] + sb[n], v1 = acc[j][2 * hrow + 1] + sb[n + 1];
        float* o = out + ((long long)b * 16 + n) * S.C + cell;
        uint32_t* o16 = reinterpret_cast<uint32_t*>(out16 + ((long long)b * S.C + cell) * 16 + n);
        if constexpr (MODE == 2) {
          const float* zp = z_prev + ((long long)b * 16 + n) * S.C + cell;
          v0 = zp[0] > 0.f ? v0 : 0.f;
          v1 = zp[S.C] > 0.f ? v1 : 0.f;
          *o16 = wg::pack_bf16(v0, v1);
        } else {
          *o16 = wg::pack_bf16(v0 > 0.f ? v0 : 0.f, v1 > 0.f ? v1 : 0.f);
        }
        o[0] = v0;
        o[S.C] = v1;
      }
    }
  }
}

// dL/dW on the tensor cores: per tap, D[co][ci] += sum over cells of g[cell][co] a[cell + off][ci],
// one m16n8k16 product per 16 cells (the cells are k; both operands are loaded transposed by
// ldmatrix.trans from their channel-last rows).  A block covers 32 x 4 cells of kZChunk planes of
// one crop; warp w accumulates taps w, w + 8, w + 16 (and w + 24 for w < 3) over the block's eight
// 16-cell rows and writes those taps of the block's partial [co][27][ci] (padded to 16 x 27 x 16).
// Grid (ceil(nx / 32), ceil(ny / 4), crops * ceil(nz / kZChunk)).
__global__ void __launch_bounds__(NTT) k_tc_grad_w(const Crop S, const __nv_bfloat16* __restrict__ g16,
                                                  const __nv_bfloat16* __restrict__ act, float* __restrict__ part) {
  __shared__ __align__(16) __nv_bfloat16 tile[kHalo * kStride];
  __shared__ __align__(16) __nv_bfloat16 gt[TX * TY * kStride];
  const int chunks = (S.nz + kZChunk - 1) / kZChunk;
  const int b = blockIdx.z / chunks, z0 = (blockIdx.z % chunks) * kZChunk;
  const int z1 = z0 + kZChunk < S.nz ? z0 + kZChunk : S.nz;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntaps = warp < 3 ? 4 : 3;
  // ldmatrix.trans row addresses, block q = lane / 8.  A (g, m = co, k = cell): cells
  // (lane & 7) + 8 (q >> 1), channels 8 (q & 1) -> a0..a3.  B (activations, k = cell, n = ci):
  // cells (lane & 7) + 8 (q & 1), channels 8 (q >> 1) -> b0, b1 of n-tile 0, then of n-tile 1.
  const int arow = (lane & 7) + (lane >> 4) * 8, ach = ((lane >> 3) & 1) * 8;
  const int brow = (lane & 7) + ((lane >> 3) & 1) * 8, bch = (lane >> 4) * 8;
  float acc[4][2][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
  const __nv_bfloat16* ab = act + (size_t)b * S.C * 16;
  const __nv_bfloat16* gb = g16 + (size_t)b * S.C * 16;
  for (int z = z0; z < z1; z++) {
    __syncthreads();  // the previous plane's operands are no longer read
    stage_halo(S, ab, x0, y0, z, tile);
    for (int c = threadIdx.x; c < TX * TY; c += NTT) {
      const int gx = x0 + c % TX, gy = y0 + c / TX;
      uint4 lo = make_uint4(0u, 0u, 0u, 0u), hi = lo;
      if (gx < S.nx && gy < S.ny) {
        const uint4* src = reinterpret_cast<const uint4*>(gb + (size_t)S.at(gx, gy, z) * 16);
        lo = src[0];
        hi = src[1];
      }
      uint4* dst = reinterpret_cast<uint4*>(gt + c * kStride);
      dst[0] = lo;
      dst[1] = hi;
    }
    __syncthreads();
    for (int seg = 0; seg < 8; seg++) {
      const int wx = (seg & 1) * 16, wy = seg >> 1;
      uint32_t a0, a1, a2, a3;
      wg::ldmatrix_x4_trans(a0, a1, a2, a3, gt + (wy * TX + wx + arow) * kStride + ach);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        if (i < ntaps) {
          const int tap = warp + 8 * i;
          const int kx = tap % 3, ky = (tap / 3) % 3, kz = tap / 9;
          const int cell = (kz * HY + wy + ky) * HX + wx + kx + brow;
          uint32_t b0, b1, b2, b3;
          wg::ldmatrix_x4_trans(b0, b1, b2, b3, tile + cell * kStride + bch);
          wg::mma_bf16(acc[i][0], a0, a1, a2, a3, b0, b1);
          wg::mma_bf16(acc[i][1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
  const size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
  float* pb = part + blk * kPadW;
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (i >= ntaps) continue;
    const int tap = warp + 8 * i;
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int ci = j * 8 + 2 * t;
      pb[(g * 27 + tap) * 16 + ci] = acc[i][j][0];
      pb[(g * 27 + tap) * 16 + ci + 1] = acc[i][j][1];
      pb[((g + 8) * 27 + tap) * 16 + ci] = acc[i][j][2];
      pb[((g + 8) * 27 + tap) * 16 + ci + 1] = acc[i][j][3];
    }
  }
}

// part2[s][k] = sum of part[blk][k] over blk = s, s + kSplits, ... (FP64); grid (kPadW / NTT, kSplits)
__global__ void __launch_bounds__(NTT) k_tc_reduce(const float* __restrict__ part, long long nblk,
                                                  double* __restrict__ part2) {
  const int k = blockIdx.x * NTT + threadIdx.x;
  if (k >= kPadW) return;
  double s = 0.0;
  for (long long blk = blockIdx.y; blk < nblk; blk += kSplits) s += (double)part[blk * kPadW + k];
  part2[(size_t)blockIdx.y * kPadW + k] = s;
}

// gw[co][t][ci] = sum over the kSplits partial sums, for the layer's real channels
__global__ void __launch_bounds__(NTT) k_tc_finish(const double* __restrict__ part2, int ci_n, int co_n,
                                                  float* __restrict__ gw) {
  const int k = blockIdx.x * NTT + threadIdx.x;
  if (k >= kPadW) return;
  const int co = k / (27 * 16), tap = (k / 16) % 27, ci = k % 16;
  if (co >= co_n || ci >= ci_n) return;
  double s = 0.0;
  for (int j = 0; j < kSplits; j++) s += part2[(size_t)j * kPadW + k];
  gw[((size_t)co * 27 + tap) * ci_n + ci] = (float)s;
}

// dL/db[co] = sum over the batch of g[b][co][cell] (FP64), one block per output channel
__global__ void __launch_bounds__(NTT) k_tc_grad_b(const Crop S, int co_n, const float* __restrict__ g,
                                                  float* __restrict__ gb) {
  __shared__ double part[NTT];
  const int co = blockIdx.x;
  double s = 0.0;
  for (long long j = threadIdx.x; j < (long long)S.B * S.C; j += NTT) {
    const long long b = j / S.C, cell = j % S.C;
    s += g[(b * co_n + co) * S.C + cell];
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int h = NTT / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) gb[co] = (float)part[0];
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
  double* loss_part = nullptr;  // per-block partial sums of the loss
  cudaError_t err = cudaSuccess;
  // WAVES_NET_TENSOR operands: BF16 activations and gradients, B fragments, weight-gradient partials
  bool tc = false;
  __nv_bfloat16 *act16[kLayers] = {}, *g16 = nullptr, *ga16 = nullptr;
  uint32_t *fw[kLayers] = {}, *ft[kLayers] = {};
  float* part = nullptr;
  double* part2 = nullptr;
  long long nblk = 0;
  dim3 conv_grid, gw_grid;

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
    tc = bt->arithmetic == WAVES_NET_TENSOR;
    const size_t cells = (size_t)S.B * S.C;
    x = alloc<float>(3 * cells);
    t = alloc<float>(cells);
    m = alloc<float>(cells);
    g = alloc<float>(16 * cells);
    ga = alloc<float>(16 * cells);
    loss = alloc<double>(1);
    loss_part = alloc<double>(blocks((long long)cells));
    if (tc) {
      const unsigned bx = (unsigned)((S.nx + TX - 1) / TX), by = (unsigned)((S.ny + TY - 1) / TY);
      const unsigned chunks = (unsigned)((S.nz + kZChunk - 1) / kZChunk);
      conv_grid = dim3(bx, by, (unsigned)(S.B * S.nz));
      gw_grid = dim3(bx, by, (unsigned)S.B * chunks);
      nblk = (long long)bx * by * S.B * chunks;
      g16 = alloc<__nv_bfloat16>(16 * cells);
      ga16 = alloc<__nv_bfloat16>(16 * cells);
      part = alloc<float>((size_t)nblk * kPadW);
      part2 = alloc<double>((size_t)kSplits * kPadW);
    } else {
      a[0] = alloc<float>(3 * cells);
    }
    for (int l = 0; l < kLayers; l++) {
      if (tc) {
        act16[l] = alloc<__nv_bfloat16>(16 * cells);
        fw[l] = alloc<uint32_t>(kFragWords);
        ft[l] = alloc<uint32_t>(kFragWords);
      } else if (l > 0) {
        a[l] = alloc<float>(16 * cells);
      }
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
    if (tc) k_tc_pack_x<<<blocks((long long)cells), NTT>>>(S, x, reinterpret_cast<uint4*>(act16[0]));
    else k_tr_round<<<blocks(3 * cells), NTT>>>(x, a[0], (long long)(3 * cells));
    return cudaGetLastError() == cudaSuccess ? WAVES_OK : WAVES_CUDA_ERROR;
  }
  // forward + loss + backward: gradients in gw/gb, the loss in *loss
  void pass() {
    if (tc) return pass_tc();
    const long long cells = (long long)S.B * S.C;
    for (int l = 0; l < kLayers; l++) k_tr_round<<<blocks((long long)nw(l)), NTT>>>(w[l], wb[l], (long long)nw(l));
    for (int l = 0; l < kLayers; l++)
      k_tr_forward<<<blocks(cells * kOut[l]), NTT>>>(S, kIn[l], kOut[l], a[l], wb[l], b[l], z[l],
                                                      l + 1 < kLayers ? a[l + 1] : nullptr);
    k_tr_loss<<<blocks(cells), NTT>>>(cells, z[kLayers - 1], t, m, norm, g, loss_part);
    k_tr_loss_sum<<<1, NTT>>>((long long)blocks(cells), loss_part, norm, loss);
    for (int l = kLayers - 1; l >= 0; l--) {
      k_tr_grad_w<<<(unsigned)(nw(l) + kOut[l]), NTT>>>(S, kIn[l], kOut[l], g, a[l], gw[l], gb[l]);
      if (l == 0) break;
      k_tr_grad_a<<<blocks(cells * kIn[l]), NTT>>>(S, kIn[l], kOut[l], g, wb[l], z[l - 1], ga);
      std::swap(g, ga);
    }
  }
  void pass_tc() {
    const long long cells = (long long)S.B * S.C;
    for (int l = 0; l < kLayers; l++) {
      k_tc_frag<<<blocks(27 * 2 * 32), NTT>>>(w[l], kIn[l], kOut[l], 0, fw[l]);
      if (l > 0) k_tc_frag<<<blocks(27 * 2 * 32), NTT>>>(w[l], kIn[l], kOut[l], 1, ft[l]);
    }
    for (int l = 0; l + 1 < kLayers; l++)
      k_tc_conv<2, 0><<<conv_grid, NTT>>>(S, act16[l], fw[l], b[l], kOut[l], nullptr, z[l], act16[l + 1]);
    k_tc_conv<1, 1><<<conv_grid, NTT>>>(S, act16[kLayers - 1], fw[kLayers - 1], b[kLayers - 1], kOut[kLayers - 1],
                                        nullptr, z[kLayers - 1], nullptr);
    k_tr_loss<<<blocks(cells), NTT>>>(cells, z[kLayers - 1], t, m, norm, g, loss_part);
    k_tr_loss_sum<<<1, NTT>>>((long long)blocks(cells), loss_part, norm, loss);
    k_tc_pack_g1<<<blocks(cells), NTT>>>(cells, g, reinterpret_cast<uint4*>(g16));
    for (int l = kLayers - 1; l >= 0; l--) {
      k_tc_grad_b<<<(unsigned)kOut[l], NTT>>>(S, kOut[l], g, gb[l]);
      k_tc_grad_w<<<gw_grid, NTT>>>(S, g16, act16[l], part);
      k_tc_reduce<<<dim3(kPadW / NTT, kSplits), NTT>>>(part, nblk, part2);
      k_tc_finish<<<kPadW / NTT, NTT>>>(part2, kIn[l], kOut[l], gw[l]);
      if (l == 0) break;
      k_tc_conv<2, 2><<<conv_grid, NTT>>>(S, g16, ft[l], nullptr, 0, z[l - 1], ga, ga16);
      std::swap(g, ga);
      std::swap(g16, ga16);
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
         (double)bt->crops * bt->nz * bt->ny * bt->nx * 16 < 2e9 &&
         (bt->arithmetic == WAVES_NET_EXACT ||
          (bt->arithmetic == WAVES_NET_TENSOR && (long long)bt->crops * bt->nz <= 65535 && bt->ny <= 4 * 65535));
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
