// Warp-level BF16 tensor-core helpers shared by the warm-start network (k_net.cu) and its training
// kernels (k_train.cu): ldmatrix loads of 8x8 BF16 blocks from shared memory and mma.sync
// m16n8k16 with BF16 operands and FP32 accumulation.
//
// Fragment layout of m16n8k16 (g = lane / 4, t = lane % 4): A (16 x 16, row-major) a0 = rows 0-7
// x k 0-7, a1 = rows 8-15 x k 0-7, a2 = rows 0-7 x k 8-15, a3 = rows 8-15 x k 8-15, each lane
// holding row g, k 2t and 2t + 1 of its block; B (16 x 8) b0 = k 2t, 2t + 1 and b1 = k 2t + 8,
// 2t + 9 of column g; D (16 x 8) d0, d1 = row g, columns 2t, 2t + 1 and d2, d3 = row g + 8.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace wg {

// Four 8x8 blocks; lanes 8q..8q+7 give the row addresses of block q.  Lane L receives row L / 4,
// columns 2 (L % 4) and 2 (L % 4) + 1 of each block.
__device__ __forceinline__ void ldmatrix_x4(uint32_t& a0, uint32_t& a1, uint32_t& a2, uint32_t& a3,
                                            const void* smem_row) {
  const unsigned addr = (unsigned)__cvta_generic_to_shared(smem_row);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3)
               : "r"(addr));
}

// The same blocks transposed: lane L receives rows 2 (L % 4) and 2 (L % 4) + 1 of column L / 4.
__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t& a0, uint32_t& a1, uint32_t& a2, uint32_t& a3,
                                                  const void* smem_row) {
  const unsigned addr = (unsigned)__cvta_generic_to_shared(smem_row);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3)
               : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Two floats rounded to BF16 (nearest even), the first in the low half.
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

}  // namespace wg
