// TEST INFRASTRUCTURE ONLY — part of the CPU oracle of the waves solver step.
//
// The oracle is a literal CPU restatement of the reference's GLSL compute shaders
// (neuron-forest/waves, water/shaders/compute/*.glslinc) and of the GDScript command order
// (water/coupled_gpu.gd:34-56, water/coastal_gpu.gd:26-33, water/pressure_multigrid.gd:121-176,
// water/pressure_hierarchy_state.gd:36-41).  It is templated on the element type R:
//   R = float  — the decision-parity instantiation: the same FP32 operations in the same order as
//                the CUDA kernels (compiled with -ffp-contract=off, the kernels with -fmad=false);
//   R = double — the error reference ("FP64 oracle") for F, u and p.
// Reductions always accumulate in double.  Transcendentals are evaluated in double and rounded
// to R, in the oracle and in the kernels alike.
//
// Parity status: the reference has no tests, golden vectors or fixtures.  This oracle is pinned to
// the reference's own GLSL compute shaders, translated to C++ and run on the host beside it, op by
// op (oracle/glsl/, tests/test_cpu_reference_pin.py), and to the analytic known answers the shaders
// encode (PLIC identities, still-water hydrostatics, dispersion relation, Stokes probe formulas) in
// tests/test_cpu_oracle.py.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may build or call this.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/waves.h"

namespace wo {

// min/max as plain comparisons so that the CUDA kernels can use the identical definition.
template <class R> inline R mn(R a, R b) { return (b < a) ? b : a; }
template <class R> inline R mx(R a, R b) { return (a < b) ? b : a; }
template <class R> inline R clampr(R x, R lo, R hi) { return mn(mx(x, lo), hi); }
template <class R> inline R fract_(R x) { return x - std::floor(x); }
template <class R> inline R sgn(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }
// Transcendentals: double evaluation rounded to R.
template <class R> inline R tcos(R x) { return R(std::cos(double(x))); }
template <class R> inline R tsin(R x) { return R(std::sin(double(x))); }
template <class R> inline R ttanh(R x) { return R(std::tanh(double(x))); }
template <class R> inline R tsinh(R x) { return R(std::sinh(double(x))); }
template <class R> inline R tcosh(R x) { return R(std::cosh(double(x))); }
template <class R> inline R texp(R x) { return R(std::exp(double(x))); }
// pow(s, 4) of coastal_target.glslinc:17 as a double product.
template <class R> inline R tpow4(R x) { double d = double(x); return R(d * d * d * d); }

struct I3 {
  int x = 0, y = 0, z = 0;
  I3() = default;
  I3(int a, int b, int c) : x(a), y(b), z(c) {}
  int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  bool operator==(const I3& o) const { return x == o.x && y == o.y && z == o.z; }
  bool operator!=(const I3& o) const { return !(*this == o); }
};
inline I3 operator+(I3 a, I3 b) { return I3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline I3 operator-(I3 a, I3 b) { return I3(a.x - b.x, a.y - b.y, a.z - b.z); }

template <class R> struct V3 {
  R x = 0, y = 0, z = 0;
  V3() = default;
  V3(R a, R b, R c) : x(a), y(b), z(c) {}
  R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> struct V4 {
  R x = 0, y = 0, z = 0, w = 0;
  V4() = default;
  V4(R a, R b, R c, R d) : x(a), y(b), z(c), w(d) {}
  R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  V3<R> xyz() const { return V3<R>(x, y, z); }
};
// GLSL dot/length in left-to-right order.
template <class R> inline R dot3(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline R len3(V3<R> a) { return std::sqrt(dot3(a, a)); }
template <class R> inline V3<R> sub3(V3<R> a, V3<R> b) { return V3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> inline V3<R> add3(V3<R> a, V3<R> b) { return V3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> inline V3<R> mul3(V3<R> a, V3<R> b) { return V3<R>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> inline V3<R> div3(V3<R> a, V3<R> b) { return V3<R>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <class R> inline V3<R> scl3(V3<R> a, R s) { return V3<R>(a.x * s, a.y * s, a.z * s); }
template <class R> inline V3<R> abs3(V3<R> a) { return V3<R>(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }
// GLSL dot(abs(v), vec3(1)).
template <class R> inline R l1(V3<R> a) { return std::fabs(a.x) * R(1) + std::fabs(a.y) * R(1) + std::fabs(a.z) * R(1); }
// GLSL dot(v, vec3(.5)).
template <class R> inline R half_dot(V3<R> a) { return a.x * R(.5) + a.y * R(.5) + a.z * R(.5); }

// periodic_index.glslinc:3-6.
inline int periodic_index(int q, int n) {
  if (q >= 0) return q % n;
  return n - 1 - ((-1 - q) % n);
}

// BF16 round-to-nearest-even of a float (storage precision of the BF16 multigrid).
inline float bf16_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) {  // inf / nan: keep (quiet nan)
    if (u & 0x007fffffu) u |= 0x00400000u;
    u &= 0xffff0000u;
  } else {
    uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;
    u &= 0xffff0000u;
  }
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

}  // namespace wo
