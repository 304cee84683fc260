// TEST INFRASTRUCTURE ONLY — a GLSL 4.50 compute-shader environment in C++ so that the
// reference's own shader sources (translated by oracle/glsl/translate.py, which only rewrites
// syntax C++ lacks) run on the host and pin the oracle's restatement op by op.
//
// What GLSL leaves to the implementation is given one IEEE-754 FP32 realisation here, the one
// the oracle and the CUDA kernels use:
//   - +, -, *, / and sqrt are correctly rounded FP32 operations, never contracted into an FMA
//     (the translation units are compiled with -ffp-contract=off); fma() is the fused operation;
//   - sin, cos, tan, tanh, sinh, cosh, exp are evaluated in double and rounded to float;
//   - pow(x, y) with a float exponent of exactly 3 is x*x*x in float (cube_volume,
//     plic_math.glslinc:20); with an integer exponent it is a double product rounded to float
//     (coastal_target.glslinc:17); otherwise double pow rounded to float;
//   - length(v) = sqrt(dot(v, v)), normalize(v) = v / length(v), dot sums left to right;
//   - round() rounds half away from zero.
// Workgroups of 128 invocations run one after the other; the invocations of a workgroup that
// calls barrier() run as cooperative fibers (glsl_runtime.cpp), otherwise one after the other.
// Atomics are plain read-modify-writes (one invocation runs at a time).
#pragma once
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace glsl {

typedef unsigned int uint;

// ------------------------------------------------------------------ scalar helpers
template <class T> struct is_scalar : std::integral_constant<bool, std::is_arithmetic<T>::value> {};

template <class T> struct tvec2;
template <class T> struct tvec3;
template <class T> struct tvec4;

// A swizzle of N components of a vector lvalue as an assignment target: writes go through to the
// components.
template <class T, int N> struct swz {
  T* p[N];
  typedef typename std::conditional<N == 2, tvec2<T>, typename std::conditional<N == 3, tvec3<T>, tvec4<T>>::type>::type V;
  operator V() const;
  V get() const { return V(*this); }
  swz& operator=(const V& v);
  swz& operator=(const swz& o) { return *this = o.get(); }
  swz& operator+=(const V& v);
  swz& operator-=(const V& v);
  swz& operator*=(const V& v);
  swz& operator/=(const V& v);
  swz& operator*=(T s);
  swz& operator/=(T s);
  T& operator[](int i) { return *p[i]; }
};

// Swizzles: name() reads (a vector value), name_w() is the write target of an assignment.
#define GLSL_SWZ2(name, a, b) \
  tvec2<T> name() const { return tvec2<T>(a, b); } \
  swz<T, 2> name##_w() { return swz<T, 2>{{&a, &b}}; }
#define GLSL_SWZ3(name, a, b, c) \
  tvec3<T> name() const { return tvec3<T>(a, b, c); } \
  swz<T, 3> name##_w() { return swz<T, 3>{{&a, &b, &c}}; }

template <class T> struct tvec2 {
  T x, y;
  tvec2() : x(0), y(0) {}
  template <class S, class = typename std::enable_if<is_scalar<S>::value>::type> explicit tvec2(S s) : x(T(s)), y(T(s)) {}
  template <class A, class B> tvec2(A a, B b) : x(T(a)), y(T(b)) {}
  template <class U> explicit tvec2(const tvec2<U>& o) : x(T(o.x)), y(T(o.y)) {}
  template <class U> explicit tvec2(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)) {}
  template <class U> explicit tvec2(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)) {}
  tvec2(const swz<T, 2>& s) : x(*s.p[0]), y(*s.p[1]) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  const T& operator[](int i) const { return i == 0 ? x : y; }
  GLSL_SWZ2(xy, x, y)
  GLSL_SWZ2(yx, y, x)
};
template <class T> struct tvec3 {
  T x, y, z;
  tvec3() : x(0), y(0), z(0) {}
  template <class S, class = typename std::enable_if<is_scalar<S>::value>::type> explicit tvec3(S s) : x(T(s)), y(T(s)), z(T(s)) {}
  template <class A, class B, class C> tvec3(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
  template <class U, class B> tvec3(const tvec2<U>& a, B b) : x(T(a.x)), y(T(a.y)), z(T(b)) {}
  template <class A, class U> tvec3(A a, const tvec2<U>& b) : x(T(a)), y(T(b.x)), z(T(b.y)) {}
  template <class U> explicit tvec3(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  template <class U> explicit tvec3(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  tvec3(const swz<T, 3>& s) : x(*s.p[0]), y(*s.p[1]), z(*s.p[2]) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  GLSL_SWZ2(xy, x, y)
  GLSL_SWZ2(yz, y, z)
  GLSL_SWZ2(xz, x, z)
  GLSL_SWZ3(xyz, x, y, z)
};
template <class T> struct tvec4 {
  T x, y, z, w;
  tvec4() : x(0), y(0), z(0), w(0) {}
  template <class S, class = typename std::enable_if<is_scalar<S>::value>::type> explicit tvec4(S s) : x(T(s)), y(T(s)), z(T(s)), w(T(s)) {}
  template <class A, class B, class C, class D> tvec4(A a, B b, C c, D d) : x(T(a)), y(T(b)), z(T(c)), w(T(d)) {}
  template <class U, class D> tvec4(const tvec3<U>& a, D d) : x(T(a.x)), y(T(a.y)), z(T(a.z)), w(T(d)) {}
  template <class A, class U> tvec4(A a, const tvec3<U>& b) : x(T(a)), y(T(b.x)), z(T(b.y)), w(T(b.z)) {}
  template <class U, class V> tvec4(const tvec2<U>& a, const tvec2<V>& b) : x(T(a.x)), y(T(a.y)), z(T(b.x)), w(T(b.y)) {}
  template <class U, class C, class D> tvec4(const tvec2<U>& a, C c, D d) : x(T(a.x)), y(T(a.y)), z(T(c)), w(T(d)) {}
  template <class U> explicit tvec4(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
  tvec4(const swz<T, 4>& s) : x(*s.p[0]), y(*s.p[1]), z(*s.p[2]), w(*s.p[3]) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  GLSL_SWZ2(xy, x, y)
  GLSL_SWZ2(zw, z, w)
  GLSL_SWZ2(yz, y, z)
  GLSL_SWZ3(xyz, x, y, z)
  GLSL_SWZ3(yzw, y, z, w)
};
#undef GLSL_SWZ2
#undef GLSL_SWZ3

template <class T, int N> swz<T, N>::operator V() const {
  V v;
  for (int i = 0; i < N; i++) v[i] = *p[i];
  return v;
}
template <class T, int N> swz<T, N>& swz<T, N>::operator=(const V& v) {
  V copy = v;  // the right-hand side may alias the components
  for (int i = 0; i < N; i++) *p[i] = copy[i];
  return *this;
}
template <class T, int N> swz<T, N>& swz<T, N>::operator+=(const V& v) { return *this = get() + v; }
template <class T, int N> swz<T, N>& swz<T, N>::operator-=(const V& v) { return *this = get() - v; }
template <class T, int N> swz<T, N>& swz<T, N>::operator*=(const V& v) { return *this = get() * v; }
template <class T, int N> swz<T, N>& swz<T, N>::operator/=(const V& v) { return *this = get() / v; }
template <class T, int N> swz<T, N>& swz<T, N>::operator*=(T s) { return *this = get() * s; }
template <class T, int N> swz<T, N>& swz<T, N>::operator/=(T s) { return *this = get() / s; }

typedef tvec2<float> vec2;
typedef tvec3<float> vec3;
typedef tvec4<float> vec4;
typedef tvec2<int> ivec2;
typedef tvec3<int> ivec3;
typedef tvec4<int> ivec4;
typedef tvec2<uint> uvec2;
typedef tvec3<uint> uvec3;
typedef tvec4<uint> uvec4;
typedef tvec2<bool> bvec2;
typedef tvec3<bool> bvec3;
typedef tvec4<bool> bvec4;

// ------------------------------------------------------------------ component-wise operators
// Defined per concrete vector type (non-template functions), so that swizzle proxies and the
// implicit int -> float conversions of GLSL arguments resolve through ordinary conversions.
#define GLSL_VEC_OPS(V, T, N)                                                                    \
  inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + b[i]; return r; } \
  inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - b[i]; return r; } \
  inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * b[i]; return r; } \
  inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / b[i]; return r; } \
  inline V operator+(const V& a, T s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + s; return r; }           \
  inline V operator-(const V& a, T s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - s; return r; }           \
  inline V operator*(const V& a, T s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * s; return r; }           \
  inline V operator/(const V& a, T s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / s; return r; }           \
  inline V operator+(T s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s + a[i]; return r; }           \
  inline V operator-(T s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s - a[i]; return r; }           \
  inline V operator*(T s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s * a[i]; return r; }           \
  inline V operator/(T s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s / a[i]; return r; }           \
  inline V operator-(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = -a[i]; return r; }                     \
  inline V& operator+=(V& a, const V& b) { a = a + b; return a; }                                               \
  inline V& operator-=(V& a, const V& b) { a = a - b; return a; }                                               \
  inline V& operator*=(V& a, const V& b) { a = a * b; return a; }                                               \
  inline V& operator/=(V& a, const V& b) { a = a / b; return a; }                                               \
  inline V& operator+=(V& a, T s) { a = a + s; return a; }                                                      \
  inline V& operator-=(V& a, T s) { a = a - s; return a; }                                                      \
  inline V& operator*=(V& a, T s) { a = a * s; return a; }                                                      \
  inline V& operator/=(V& a, T s) { a = a / s; return a; }                                                      \
  inline bool operator==(const V& a, const V& b) { for (int i = 0; i < N; i++) if (!(a[i] == b[i])) return false; return true; } \
  inline bool operator!=(const V& a, const V& b) { return !(a == b); }
GLSL_VEC_OPS(vec2, float, 2)
GLSL_VEC_OPS(vec3, float, 3)
GLSL_VEC_OPS(vec4, float, 4)
GLSL_VEC_OPS(ivec2, int, 2)
GLSL_VEC_OPS(ivec3, int, 3)
GLSL_VEC_OPS(ivec4, int, 4)
GLSL_VEC_OPS(uvec2, uint, 2)
GLSL_VEC_OPS(uvec3, uint, 3)
GLSL_VEC_OPS(uvec4, uint, 4)
#undef GLSL_VEC_OPS
inline ivec3 operator%(const ivec3& a, const ivec3& b) { return ivec3(a.x % b.x, a.y % b.y, a.z % b.z); }
// ------------------------------------------------------------------ built-in functions
inline float abs(float x) { return x < 0.f ? -x : (x == 0.f ? 0.f : x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float sign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
template <class T, class = typename std::enable_if<std::is_same<T, int>::value || std::is_same<T, uint>::value>::type>
inline T min(T a, T b) { return b < a ? b : a; }
template <class T, class = typename std::enable_if<std::is_same<T, int>::value || std::is_same<T, uint>::value>::type>
inline T max(T a, T b) { return a < b ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
template <class T, class = typename std::enable_if<std::is_same<T, int>::value || std::is_same<T, uint>::value>::type>
inline T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float fract(float x) { return x - floor(x); }
inline float round(float x) { return __builtin_roundf(x); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float fma(float a, float b, float c) { return __builtin_fmaf(a, b, c); }
inline float mix(float a, float b, float t) { return a * (1.f - t) + b * t; }
inline float step(float edge, float x) { return x < edge ? 0.f : 1.f; }
inline float cos(float x) { return (float)__builtin_cos((double)x); }
inline float sin(float x) { return (float)__builtin_sin((double)x); }
inline float tan(float x) { return (float)__builtin_tan((double)x); }
inline float tanh(float x) { return (float)__builtin_tanh((double)x); }
inline float sinh(float x) { return (float)__builtin_sinh((double)x); }
inline float cosh(float x) { return (float)__builtin_cosh((double)x); }
inline float exp(float x) { return (float)__builtin_exp((double)x); }
inline float pow(float x, float y) {
  if (y == 3.f) return x * x * x;
  return (float)__builtin_pow((double)x, (double)y);
}
inline float pow(float x, int k) {
  double d = (double)x, r = 1.0;
  for (int i = 0; i < k; i++) r *= d;
  return (float)r;
}
inline bool isnan(float x) { return x != x; }
inline bool isinf(float x) { return x == __builtin_inff() || x == -__builtin_inff(); }
inline uint floatBitsToUint(float x) { uint u; std::memcpy(&u, &x, 4); return u; }
inline int floatBitsToInt(float x) { int u; std::memcpy(&u, &x, 4); return u; }
inline float uintBitsToFloat(uint u) { float x; std::memcpy(&x, &u, 4); return x; }
inline float intBitsToFloat(int u) { float x; std::memcpy(&x, &u, 4); return x; }

#define GLSL_VEC_FUNCS(V, N)                                                                            \
  inline V abs(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = abs(a[i]); return r; }             \
  inline V floor(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = floor(a[i]); return r; }         \
  inline V fract(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = fract(a[i]); return r; }         \
  inline V sign(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = sign(a[i]); return r; }           \
  inline V min(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = min(a[i], b[i]); return r; } \
  inline V max(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = max(a[i], b[i]); return r; } \
  inline V min(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = min(a[i], b); return r; } \
  inline V max(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = max(a[i], b); return r; } \
  inline V clamp(const V& x, const V& lo, const V& hi) { V r; for (int i = 0; i < N; i++) r[i] = clamp(x[i], lo[i], hi[i]); return r; } \
  inline V clamp(const V& x, float lo, float hi) { V r; for (int i = 0; i < N; i++) r[i] = clamp(x[i], lo, hi); return r; } \
  inline V mix(const V& a, const V& b, const V& t) { V r; for (int i = 0; i < N; i++) r[i] = mix(a[i], b[i], t[i]); return r; } \
  inline V mix(const V& a, const V& b, float t) { V r; for (int i = 0; i < N; i++) r[i] = mix(a[i], b[i], t); return r; } \
  inline float dot(const V& a, const V& b) { float s = a[0] * b[0]; for (int i = 1; i < N; i++) s = s + a[i] * b[i]; return s; } \
  inline float length(const V& a) { return sqrt(dot(a, a)); }                                            \
  inline V normalize(const V& a) { return a / length(a); }
GLSL_VEC_FUNCS(vec2, 2)
GLSL_VEC_FUNCS(vec3, 3)
GLSL_VEC_FUNCS(vec4, 4)
#undef GLSL_VEC_FUNCS
inline ivec3 abs(const ivec3& a) { return ivec3(abs(a.x), abs(a.y), abs(a.z)); }
inline ivec3 min(const ivec3& a, const ivec3& b) { return ivec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline ivec3 max(const ivec3& a, const ivec3& b) { return ivec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline ivec3 clamp(const ivec3& x, const ivec3& lo, const ivec3& hi) { return min(max(x, lo), hi); }
inline uvec4 max(const uvec4& a, const uvec4& b) { return uvec4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
// relational vector functions
#define GLSL_REL(name, op)                                                                           \
  template <class T> inline bvec3 name(const tvec3<T>& a, const tvec3<T>& b) { return bvec3(a.x op b.x, a.y op b.y, a.z op b.z); } \
  template <class T> inline bvec2 name(const tvec2<T>& a, const tvec2<T>& b) { return bvec2(a.x op b.x, a.y op b.y); } \
  template <class T> inline bvec4 name(const tvec4<T>& a, const tvec4<T>& b) { return bvec4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w); }
GLSL_REL(greaterThanEqual, >=)
GLSL_REL(greaterThan, >)
GLSL_REL(lessThanEqual, <=)
GLSL_REL(lessThan, <)
GLSL_REL(equal, ==)
GLSL_REL(notEqual, !=)
#undef GLSL_REL
inline bool all(const bvec2& b) { return b.x && b.y; }
inline bool all(const bvec3& b) { return b.x && b.y && b.z; }
inline bool all(const bvec4& b) { return b.x && b.y && b.z && b.w; }
inline bool any(const bvec2& b) { return b.x || b.y; }
inline bool any(const bvec3& b) { return b.x || b.y || b.z; }
inline bool any(const bvec4& b) { return b.x || b.y || b.z || b.w; }
inline bvec4 isnan(const vec4& v) { return bvec4(isnan(v.x), isnan(v.y), isnan(v.z), isnan(v.w)); }
inline bvec4 isinf(const vec4& v) { return bvec4(isinf(v.x), isinf(v.y), isinf(v.z), isinf(v.w)); }

// ------------------------------------------------------------------ invocation state
struct Invocation {
  uvec3 global, local, group, groups;
};
extern Invocation* current;  // the running invocation (glsl_runtime.cpp)
void barrier();              // workgroup barrier: yields to the scheduler
inline void memoryBarrierShared() {}
inline void memoryBarrier() {}
inline void groupMemoryBarrier() {}
inline uint atomicAdd(uint& m, uint v) { uint o = m; m = o + v; return o; }
inline int atomicAdd(int& m, int v) { int o = m; m = o + v; return o; }
inline uint atomicMax(uint& m, uint v) { uint o = m; m = o < v ? v : o; return o; }
inline uint atomicCompSwap(uint& m, uint compare, uint value) { uint o = m; if (o == compare) m = value; return o; }

// 3-D image of the accepted-surface export (imageStore targets), x fastest.
struct Image3D {
  float* data = nullptr;
  int channels = 4, nx = 0, ny = 0, nz = 0;
};
inline void imageStore(Image3D& img, const ivec3& q, const vec4& v) {
  if (!img.data || q.x < 0 || q.y < 0 || q.z < 0 || q.x >= img.nx || q.y >= img.ny || q.z >= img.nz) return;
  float* p = img.data + (size_t)img.channels * ((size_t)q.x + (size_t)img.nx * ((size_t)q.y + (size_t)img.ny * (size_t)q.z));
  for (int k = 0; k < img.channels; k++) p[k] = v[k];
}

// Runs `body` for every invocation of a dispatch of groups.x x groups.y workgroups of 128.
void dispatch(void (*body)(), uvec3 groups);

}  // namespace glsl

#define gl_GlobalInvocationID (glsl::current->global)
#define gl_LocalInvocationID (glsl::current->local)
#define gl_WorkGroupID (glsl::current->group)
#define gl_NumWorkGroups (glsl::current->groups)
