// Learned warm start (no reference counterpart): a 4-layer 3x3x3 convolution network
// (3 -> 16 -> 16 -> 16 -> 1 channels, ReLU after the first three layers, zero padding at the
// domain edge) that predicts the initial pressure of the first CG round from the candidate volume
// fraction F, the right-hand side b and the warm-start pressure p_prev of op 2
// (pressure_pass.glslinc:33-34): p_net = p_prev + output_scale * y on wet cells.
//
// Each layer is a direct convolution on the tensor cores: a warp owns 16 consecutive x cells and
// all 16 output channels, and for each of the 27 taps multiplies the 16 x 16 tile (cells x input
// channels, BF16) by the tap's 16 x 16 weight block with mma.sync m16n8k16 (BF16 in, FP32
// accumulate).  A block stages the 34 x 6 x 3 halo of its 32 x 4 x 1 cells in shared memory with a
// 48-byte cell stride, so the ldmatrix rows of a tap fall in distinct banks.  Activations between
// layers are BF16, channel-last (32 bytes per cell).
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.h"
#include "mma_bf16.cuh"

namespace wg {

namespace {
constexpr int NT = 256;
constexpr int TX = 32, TY = 4;                 // block tile: 32 x 4 cells of one z plane
constexpr int HX = TX + 2, HY = TY + 2, HZ = 3;  // halo tile
constexpr int kStride = 24;                    // bf16 per staged cell (16 channels + 8 padding)
constexpr int kHalo = HX * HY * HZ;

DI bool warm_on(const Dev& D) { return D.c[kNetLoaded] > .5 && D.c[5] > .5 && D.c[7] < .5; }

// One layer.  LAYER 0 reads (F, b, p_prev) scaled by input_scale (channels 3..15 zero); layers 1
// and 2 read the previous BF16 activations; layer 3 (one output channel, one n-tile) writes p_net.
// Weights arrive in mma fragment order: [tap][n-tile][lane][2] packed BF16 pairs.
template <int LAYER>
__global__ void __launch_bounds__(NT) k_net_layer(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!warm_on(D)) return;
  constexpr int NTILES = LAYER == 3 ? 1 : 2;
  __shared__ __align__(16) __nv_bfloat16 tile[kHalo * kStride];
  __shared__ __align__(16) uint32_t wfrag[27 * NTILES * 64];
  __shared__ float bias[16];
  const int nx = D.nx, ny = D.ny, nz = D.nz;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z = blockIdx.z;
  const uint32_t* wsrc = D.net_w + LAYER * kNetLayerWords;
  for (int k = threadIdx.x; k < 27 * NTILES * 64; k += NT) wfrag[k] = wsrc[k];
  if (threadIdx.x < 16) bias[threadIdx.x] = D.net_b[LAYER * 16 + threadIdx.x];
  const float* Cb = bank_ptr(D, 1 - acc_bank(D));
  const __nv_bfloat16* act = reinterpret_cast<const __nv_bfloat16*>(D.net_act);
  const __nv_bfloat16* in = LAYER == 0 ? nullptr : act + (size_t)((LAYER - 1) & 1) * D.N * 16;
  for (int c = threadIdx.x; c < kHalo; c += NT) {
    const int hx = c % HX, hy = (c / HX) % HY, hz = c / (HX * HY);
    const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z + hz - 1;
    uint4 lo = make_uint4(0u, 0u, 0u, 0u), hi = lo;
    if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && gz >= 0 && gz < nz) {
      const int i = gx + nx * (gy + ny * gz);
      if constexpr (LAYER == 0) {
        const float f = Cb[i] * D.net_scale[0], b = D.b[i] * D.net_scale[1];
        const float p = Cb[D.N + D.NF + i] * D.net_scale[2];
        lo.x = pack_bf16(f, b);
        lo.y = pack_bf16(p, 0.f);
      } else {
        const uint4* src = reinterpret_cast<const uint4*>(in + (size_t)i * 16);
        lo = src[0];
        hi = src[1];
      }
    }
    uint4* dst = reinterpret_cast<uint4*>(tile + c * kStride);
    dst[0] = lo;
    dst[1] = hi;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wx = (warp & 1) * 16, wy = warp >> 1;
  // ldmatrix x4: lanes 0-7 / 8-15 give rows 0-7 / 8-15 of channels 0-7, lanes 16-31 the same rows
  // of channels 8-15 -- the A fragments a0..a3 of m16n8k16
  const int row = (lane & 7) + ((lane >> 3) & 1) * 8, half = (lane >> 4) * 8;
  float acc[NTILES][4];
#pragma unroll
  for (int j = 0; j < NTILES; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll 3
  for (int tap = 0; tap < 27; tap++) {
    const int kx = tap % 3, ky = (tap / 3) % 3, kz = tap / 9;
    const int cell = (kz * HY + wy + ky) * HX + wx + kx + row;
    uint32_t a0, a1, a2, a3;
    ldmatrix_x4(a0, a1, a2, a3, tile + cell * kStride + half);
#pragma unroll
    for (int j = 0; j < NTILES; j++) {
      const uint2 b = *reinterpret_cast<const uint2*>(&wfrag[((tap * NTILES + j) * 32 + lane) * 2]);
      mma_bf16(acc[j], a0, a1, a2, a3, b.x, b.y);
    }
  }
  // D fragment: lane (g = lane / 4, t = lane % 4) holds cells g and g + 8, channels 2t, 2t + 1
  // of each n-tile
  const int g = lane >> 2, t = lane & 3;
  const int y = y0 + wy;
#pragma unroll
  for (int hrow = 0; hrow < 2; hrow++) {
    const int x = x0 + wx + g + 8 * hrow;
    if (x >= nx || y >= ny) continue;
    const int i = x + nx * (y + ny * z);
    if constexpr (LAYER < 3) {
      __nv_bfloat16* out = reinterpret_cast<__nv_bfloat16*>(D.net_act) + (size_t)(LAYER & 1) * D.N * 16 + (size_t)i * 16;
#pragma unroll
      for (int j = 0; j < NTILES; j++) {
        const int co = j * 8 + 2 * t;
        const float v0 = fmaxf(acc[j][2 * hrow] + bias[co], 0.f), v1 = fmaxf(acc[j][2 * hrow + 1] + bias[co + 1], 0.f);
        *reinterpret_cast<uint32_t*>(out + co) = pack_bf16(v0, v1);
      }
    } else if (t == 0) {
      const float p = Cb[D.N + D.NF + i];
      D.net_p[i] = D.kind[i] > 0 ? p + D.net_scale[3] * (acc[0][2 * hrow] + bias[0]) : p;
    }
  }
}

}  // namespace

void launch_warm_network(const Dev& D, cudaStream_t s) {
  const dim3 grid((unsigned)((D.nx + TX - 1) / TX), (unsigned)((D.ny + TY - 1) / TY), (unsigned)D.nz);
  pdl_launch(k_net_layer<0>, grid, NT, 0, s, D);
  pdl_launch(k_net_layer<1>, grid, NT, 0, s, D);
  pdl_launch(k_net_layer<2>, grid, NT, 0, s, D);
  pdl_launch(k_net_layer<3>, grid, NT, 0, s, D);
}

}  // namespace wg
