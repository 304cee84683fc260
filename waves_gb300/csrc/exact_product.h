// The FP64 product of two FP32 values, formed with integer instructions.
//
// A float has a 24-bit significand, so the product of two floats has at most 48 significant bits
// and (double)a * (double)b is exact.  This GPU issues FP64 instructions at a small fraction of
// the FP32 and integer rates, and the FP64 dot products of the solver (r.z, r.r, b.b, d.q) spent
// most of their time converting and multiplying; here the 24 x 24-bit significand product is one
// wide integer multiply and the double is assembled from its bits: sign, exponent sum, the 47 or
// 48 product bits normalised into the 52-bit fraction.  For normal finite operands the result is
// the same double, bit for bit, that the FP64 multiply gives (both are the exact product); zeros,
// subnormals, infinities and NaNs take the FP64 multiply.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define WG_HD __host__ __device__ __forceinline__
#else
#define WG_HD inline
#endif

namespace wg {

WG_HD double exact_product(float a, float b) {
  uint32_t ua, ub;
  std::memcpy(&ua, &a, 4);
  std::memcpy(&ub, &b, 4);
  const uint32_t ea = (ua >> 23) & 0xffu, eb = (ub >> 23) & 0xffu;
  if (ea == 0u || eb == 0u || ea == 0xffu || eb == 0xffu) return (double)a * (double)b;
  const uint64_t p = (uint64_t)((ua & 0x7fffffu) | 0x800000u) * (uint64_t)((ub & 0x7fffffu) | 0x800000u);
  // p in [2^46, 2^48): value = p * 2^(ea + eb - 254 - 46)
  const bool top = (p >> 47) != 0u;
  const uint64_t frac = (top ? (p << 5) : (p << 6)) & 0xfffffffffffffull;
  const uint64_t exp = (uint64_t)((int)ea + (int)eb - (top ? 253 : 254) + 1023);
  const uint64_t bits = ((uint64_t)((ua ^ ub) >> 31) << 63) | (exp << 52) | frac;
  double r;
  std::memcpy(&r, &bits, 8);
  return r;
}

}  // namespace wg
