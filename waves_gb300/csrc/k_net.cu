// Learned warm start (no reference counterpart): a 4-layer 3x3x3 convolution network
// (3 -> 16 -> 16 -> 16 -> 1 channels, ReLU after the first three layers, zero padding at the
// domain edge) that predicts the initial pressure of the first CG round from the candidate volume
// fraction F, the right-hand side b and the warm-start pressure p_prev of op 2
// (pressure_pass.glslinc:33-34): p_net = p_prev + output_scale * y on wet cells.
//
// Two forms of each layer.  The tcgen05 form (the default) is described at k_net_layer_tc.  The
// mma.sync form is a direct convolution on the warp-level tensor-core path: a warp owns 16 consecutive x cells and
// all 16 output channels, and for each of the 27 taps multiplies the 16 x 16 tile (cells x input
// channels, BF16) by the tap's 16 x 16 weight block with mma.sync m16n8k16 (BF16 in, FP32
// accumulate).  A block stages the 34 x 6 x 3 halo of its 32 x 4 x 1 cells in shared memory with a
// 48-byte cell stride, so the ldmatrix rows of a tap fall in distinct banks.  Activations between
// layers are BF16, channel-last (32 bytes per cell).
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.h"
#include "mma_bf16.cuh"
#include "tcgen05.cuh"

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

// ---------------------------------------------------------------- tcgen05 form
// The same layer on the fifth-generation tensor cores.  A block owns 128 consecutive x cells of
// four (y) rows of one z plane: four M = 128 tiles.  It stages the 130 x 6 x 3 halo (BF16,
// channel-last) as two 16-byte planes (channels 0-7, 8-15) and the layer's weights as
// [tap][channel half][output channel][8 channels]; for each tile, one thread issues 27
// tcgen05.mma (M = 128, N = 16, K = 16), one per tap, whose A operand is the halo row of the tap
// shifted by kx cells -- the descriptor's start address moves by kx rows, no im2col copy -- and
// whose accumulator is 16 FP32 columns of tensor memory.  After the commit's mbarrier completes,
// each warp reads its 32 lanes (cells) of two tiles with tcgen05.ld and writes bias + ReLU as
// BF16 (or, in the last layer, p_net).
constexpr int TCX = 128, TCY = 4;
constexpr int TCHX = TCX + 2, TCHY = TCY + 2, TCHZ = 3;
constexpr int kTcHalo = TCHX * TCHY * TCHZ;
constexpr int kTcPlane = kTcHalo * 16;     // bytes of one channel half of the halo
constexpr int kTcWeights = 27 * 512;       // bytes of one layer's weights
constexpr int kTcSmem = 2 * kTcPlane + kTcWeights;
constexpr uint32_t kTcCols = 64;           // tensor-memory columns: four 16-column accumulators
constexpr uint32_t kTcWaitLimit = 1u << 22;

template <int LAYER>
__global__ void __launch_bounds__(NT) k_net_layer_tc(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!warm_on(D)) return;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* plane0 = smem;
  unsigned char* plane1 = smem + kTcPlane;
  unsigned char* wts = smem + 2 * kTcPlane;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  __shared__ float bias[16];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nx = D.nx, ny = D.ny, nz = D.nz;
  const int x0 = blockIdx.x * TCX, y0 = blockIdx.y * TCY, z = blockIdx.z;
  if (warp == 0) tc05::alloc(&tmem_slot, kTcCols);
  if (threadIdx.x == 0) tc05::mbar_init(&mbar, 1);
  {
    const uint4* wsrc = reinterpret_cast<const uint4*>(D.net_wt) + (size_t)LAYER * (kTcWeights / 16);
    for (int k = threadIdx.x; k < kTcWeights / 16; k += NT) reinterpret_cast<uint4*>(wts)[k] = wsrc[k];
  }
  if (threadIdx.x < 16) bias[threadIdx.x] = D.net_b[LAYER * 16 + threadIdx.x];
  const float* Cb = bank_ptr(D, 1 - acc_bank(D));
  const __nv_bfloat16* act = reinterpret_cast<const __nv_bfloat16*>(D.net_act);
  const __nv_bfloat16* in = LAYER == 0 ? nullptr : act + (size_t)((LAYER - 1) & 1) * D.N * 16;
  for (int c = threadIdx.x; c < kTcHalo; c += NT) {
    const int hx = c % TCHX, hy = (c / TCHX) % TCHY, hz = c / (TCHX * TCHY);
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
    reinterpret_cast<uint4*>(plane0)[c] = lo;
    reinterpret_cast<uint4*>(plane1)[c] = hi;
  }
  tc05::fence_proxy_async();
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  if (threadIdx.x == 0) {
    constexpr uint32_t idesc = tc05::idesc_bf16_f32(128, 16);
    const uint32_t a_base = tc05::smem_u32(plane0), b_base = tc05::smem_u32(wts);
    for (int ty = 0; ty < TCY; ty++)
      for (int tap = 0; tap < 27; tap++) {
        const int kx = tap % 3, ky = (tap / 3) % 3, kz = tap / 9;
        const int cell0 = (kz * TCHY + ty + ky) * TCHX + kx;
        const uint64_t adesc = tc05::smem_desc(a_base + (uint32_t)cell0 * 16u, kTcPlane, 128);
        const uint64_t bdesc = tc05::smem_desc(b_base + (uint32_t)tap * 512u, 256, 128);
        tc05::mma_bf16(tmem + (uint32_t)ty * 16u, adesc, bdesc, idesc, tap > 0);
      }
    tc05::commit(&mbar);
  }
  bool ok = tc05::mbar_wait(&mbar, 0, kTcWaitLimit);
  tc05::fence_after_sync();
  const int q = warp & 3;
#pragma unroll
  for (int tt = 0; tt < 2; tt++) {
    const int ty = (warp >> 2) * 2 + tt;
    float v[16];
    tc05::ld_32x32b_x16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)ty * 16u, v);
    const int x = x0 + 32 * q + lane, y = y0 + ty;
    if (!ok || x >= nx || y >= ny) continue;
    const int i = x + nx * (y + ny * z);
    if constexpr (LAYER < 3) {
      uint32_t packed[8];
#pragma unroll
      for (int k = 0; k < 8; k++) packed[k] = pack_bf16(fmaxf(v[2 * k] + bias[2 * k], 0.f), fmaxf(v[2 * k + 1] + bias[2 * k + 1], 0.f));
      uint4* out = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(D.net_act) + (size_t)(LAYER & 1) * D.N * 16 + (size_t)i * 16);
      out[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
      out[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    } else {
      const float p = Cb[D.N + D.NF + i];
      D.net_p[i] = D.kind[i] > 0 ? p + D.net_scale[3] * (v[0] + bias[0]) : p;
    }
  }
  if (!ok) {
    // the accumulators did not arrive in time: record the failure, give the tensor cores a second
    // bounded wait before the columns are released
    if (threadIdx.x == 0) D.c[7] = 98;
    tc05::mbar_wait(&mbar, 0, kTcWaitLimit);
  }
  tc05::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc05::fence_after_sync();
    tc05::dealloc(tmem, kTcCols);
  }
}

}  // namespace

void setup_warm_network() {
  cudaFuncSetAttribute(k_net_layer_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  cudaFuncSetAttribute(k_net_layer_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  cudaFuncSetAttribute(k_net_layer_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  cudaFuncSetAttribute(k_net_layer_tc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
}

void launch_warm_network(const Dev& D, cudaStream_t s) {
  if (D.net_tc05) {
    const dim3 grid((unsigned)((D.nx + TCX - 1) / TCX), (unsigned)((D.ny + TCY - 1) / TCY), (unsigned)D.nz);
    pdl_launch(k_net_layer_tc<0>, grid, NT, kTcSmem, s, D);
    pdl_launch(k_net_layer_tc<1>, grid, NT, kTcSmem, s, D);
    pdl_launch(k_net_layer_tc<2>, grid, NT, kTcSmem, s, D);
    pdl_launch(k_net_layer_tc<3>, grid, NT, kTcSmem, s, D);
    return;
  }
  const dim3 grid((unsigned)((D.nx + TX - 1) / TX), (unsigned)((D.ny + TY - 1) / TY), (unsigned)D.nz);
  pdl_launch(k_net_layer<0>, grid, NT, 0, s, D);
  pdl_launch(k_net_layer<1>, grid, NT, 0, s, D);
  pdl_launch(k_net_layer<2>, grid, NT, 0, s, D);
  pdl_launch(k_net_layer<3>, grid, NT, 0, s, D);
}

}  // namespace wg
