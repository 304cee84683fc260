// Device arithmetic of the waves solver step, shared by all kernels.
//
// Every function restates the reference shader function named in its comment
// (neuron-forest/waves water/shaders/compute/*.glslinc) with the same FP32 operations in the same
// order.  The translation units are compiled with -fmad=false so that no multiply-add is fused
// unless the reference writes fma(); min/max are plain comparisons; transcendentals are evaluated
// in double and rounded to float.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>

#include "dev.h"
#include "exact_product.h"

namespace wg {

#define DI __device__ __forceinline__

struct I3 {
  int x, y, z;
  DI int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  DI int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
DI I3 mk(int x, int y, int z) { I3 q; q.x = x; q.y = y; q.z = z; return q; }
DI I3 addI(I3 a, I3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
DI I3 subI(I3 a, I3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
DI bool eqI(I3 a, I3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
DI I3 ax(I3 q, int axis, int delta) { q[axis] += delta; return q; }

struct F3 {
  float x, y, z;
  DI float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  DI float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
DI F3 mf(float x, float y, float z) { F3 v; v.x = x; v.y = y; v.z = z; return v; }
DI float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DI float len3(F3 a) { return sqrtf(dot3(a, a)); }
DI F3 sub3(F3 a, F3 b) { return mf(a.x - b.x, a.y - b.y, a.z - b.z); }
DI F3 add3(F3 a, F3 b) { return mf(a.x + b.x, a.y + b.y, a.z + b.z); }
DI F3 mul3(F3 a, F3 b) { return mf(a.x * b.x, a.y * b.y, a.z * b.z); }
DI F3 div3(F3 a, F3 b) { return mf(a.x / b.x, a.y / b.y, a.z / b.z); }
DI F3 scl3(F3 a, float s) { return mf(a.x * s, a.y * s, a.z * s); }
DI F3 abs3(F3 a) { return mf(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
DI float l1(F3 a) { return fabsf(a.x) * 1.f + fabsf(a.y) * 1.f + fabsf(a.z) * 1.f; }
DI float half_dot(F3 a) { return a.x * .5f + a.y * .5f + a.z * .5f; }

DI float mnf(float a, float b) { return (b < a) ? b : a; }
DI float mxf(float a, float b) { return (a < b) ? b : a; }
DI float clampf_(float x, float lo, float hi) { return mnf(mxf(x, lo), hi); }
DI float fract_(float x) { return x - floorf(x); }
DI float sgnf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
// griddepcontrol.wait: returns once the grid this one depends on (programmatic launch) has
// completed and its memory is visible (immediate for a normally launched kernel).  With `early`,
// griddepcontrol.launch_dependents then lets the next kernel be scheduled as soon as every block
// of this grid is resident; without it the next kernel launches as this grid exits.  On the beach
// the exit trigger is the faster (13.23 vs 13.86 ms per step; 13.48 without programmatic launch).
DI void grid_dep_wait(int early) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (early) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
DI float tcos(float x) { return (float)cos((double)x); }
DI float tsin(float x) { return (float)sin((double)x); }
DI float ttanh(float x) { return (float)tanh((double)x); }
DI float tsinh(float x) { return (float)sinh((double)x); }
DI float tcosh(float x) { return (float)cosh((double)x); }
DI float texp(float x) { return (float)exp((double)x); }
DI float tpow4(float x) { double d = (double)x; return (float)(d * d * d * d); }
// periodic_index.glslinc:3-6
DI int pidx(int q, int n) {
  if (q >= 0 && q < n) return q;
  if (q < 0 && q >= -n) return q + n;
  if (q >= n && q < 2 * n) return q - n;
  return q >= 0 ? q % n : n - 1 - ((-1 - q) % n);
}

// ---------------------------------------------------------------- grid helpers
struct Grid {
  const Dev& D;
  DI explicit Grid(const Dev& d) : D(d) {}
  DI float h(int a) const { return a == 0 ? D.hx : (a == 1 ? D.hy : D.hz); }
  DI long long index3(I3 q) const { return (long long)q.x + (long long)D.nx * ((long long)q.y + (long long)D.ny * q.z); }
  // cell and face counts stay below 2^31, so the index arithmetic runs in 32-bit unsigned integers
  DI I3 coord(long long i) const {
    const unsigned u = (unsigned)i, nx = (unsigned)D.nx, row = u / nx;
    return mk(int(u - row * nx), int(row % (unsigned)D.ny), int(row / (unsigned)D.ny));
  }
  DI I3 wrap_cell(I3 q) const {
    q.z = pidx(q.z, D.nz);
    if (D.px) q.x = pidx(q.x, D.nx);
    return q;
  }
  DI bool outside(I3 q) const { return q.x < 0 || q.x >= D.nx || q.y < 0 || q.y >= D.ny; }
  DI F3 center(I3 q) const {
    return mf(D.ox + ((float)q.x + 0.5f) * D.hx, D.oy + ((float)q.y + 0.5f) * D.hy, D.oz + ((float)q.z + 0.5f) * D.hz);
  }
  // solid (pressure_core.glslinc:87-96), tabulated over (x, y) with a margin
  DI bool solid_direct(I3 q) const {
    q = wrap_cell(q);
    if (q.y < 0 || q.x >= D.nx) return true;
    if (!D.coastal && q.x < 0) return true;
    if (q.y >= D.ny) return false;
    if (D.slope > 0.f) {
      float x = center(q).x;
      float bed = -0.45f + mxf(0.f, x - 1.5f) / D.slope;
      return center(q).y <= bed;
    }
    return false;
  }
  DI bool solid(I3 q) const {
    q = wrap_cell(q);
    int x = q.x + kSolidPad, y = q.y + kSolidPad;
    if (x >= 0 && y >= 0 && x < D.tab_w && y < D.tab_h) return D.solid_tab[y * D.tab_w + x] != 0;
    return solid_direct(q);
  }
  DI bool wet(I3 q) const {
    q = wrap_cell(q);
    return !outside(q) && D.kind[index3(q)] > 0;
  }
  // eta (pressure_core.glslinc:73-83)
  DI float eta(I3 q) const {
    if (D.shape == 5) {
      float phase = D.wave[1] * (D.ox + ((float)q.x + .5f) * D.hx);
      float sigma = ttanh(D.wave[1] * D.wave[3]);
      float second = D.stokes2 ? D.wave[1] * D.wave[0] * D.wave[0] * (3.f - sigma * sigma) / (4.f * sigma * sigma * sigma) : 0.f;
      return D.eta0 + D.wave[0] * tcos(phase) + second * tcos(2.f * phase);
    }
    return D.eta0 + D.corr * tcos(6.28318530718f * ((float)q.x + 0.5f) / (float)D.nx + D.corr_phase);
  }
  DI float phi(I3 q) const {
    q = wrap_cell(q);
    return outside(q) ? center(q).y - eta(q) : D.phi[index3(q)];
  }
  // face_index (pressure_core.glslinc:129-133), local to the face block (minus U())
  DI long long face_local(I3 q, int axis) const {
    if (axis == 2 && q.z == D.nz) q.z = 0;
    if (axis == 0 && D.px && q.x == D.nx) q.x = 0;
    if (axis == 0) return (long long)q.x + (long long)(D.nx + 1) * ((long long)q.y + (long long)D.ny * q.z);
    if (axis == 1) return D.NU + (long long)q.x + (long long)D.nx * ((long long)q.y + (long long)(D.ny + 1) * q.z);
    return D.NU + D.NV + (long long)q.x + (long long)D.nx * ((long long)q.y + (long long)D.ny * q.z);
  }
  DI long long face_index(I3 q, int axis) const { return D.N + face_local(q, axis); }
  // lattice index of face (q, axis) without folding periodic duplicates
  DI long long face_local_raw(I3 q, int axis) const {
    if (axis == 0) return (long long)q.x + (long long)(D.nx + 1) * ((long long)q.y + (long long)D.ny * q.z);
    if (axis == 1) return D.NU + (long long)q.x + (long long)D.nx * ((long long)q.y + (long long)(D.ny + 1) * q.z);
    return D.NU + D.NV + (long long)q.x + (long long)D.nx * ((long long)q.y + (long long)D.ny * q.z);
  }
  DI void unpack_face(long long f, I3& q, int& axis) const {
    long long base;
    int mx_, my_;
    if (f < D.NU) { axis = 0; base = 0; mx_ = D.nx + 1; my_ = D.ny; }
    else if (f < D.NU + D.NV) { axis = 1; base = D.NU; mx_ = D.nx; my_ = D.ny + 1; }
    else { axis = 2; base = D.NU + D.NV; mx_ = D.nx; my_ = D.ny; }
    const unsigned u = (unsigned)(f - base), row = u / (unsigned)mx_;
    q = mk(int(u - row * (unsigned)mx_), int(row % (unsigned)my_), int(row / (unsigned)my_));
  }
  DI bool wall_face(I3 q, int axis) const { return solid(q) || solid(ax(q, axis, -1)); }
  DI bool face_in_bounds(I3 q, int axis) const {
    int mx_ = D.nx + (axis == 0), my_ = D.ny + (axis == 1), mz_ = D.nz + (axis == 2);
    return q.x >= 0 && q.y >= 0 && q.z >= 0 && q.x < mx_ && q.y < my_ && q.z < mz_;
  }
  DI I3 wrap_face(I3 q) const {
    q.z = pidx(q.z, D.nz);
    if (D.px) q.x = pidx(q.x, D.nx);
    return q;
  }
  // d - round(d / n) * n on the periodic axes (coupled_motion.glslinc periodic_delta).  For the
  // integer differences here (|d| <= n) round(d / n) is -1, 0 or 1, and |d / n| >= 1/2 exactly
  // when |2d| >= n: the float quotient of two small integers never rounds onto 1/2.  So the
  // shift is decided in integers and the result is the same float.
  DI F3 periodic_delta(I3 a, I3 b) const {
    int dx = a.x - b.x, dz = a.z - b.z;
    if (2 * dz >= D.nz) dz -= D.nz;
    else if (2 * dz <= -D.nz) dz += D.nz;
    if (D.px) {
      if (2 * dx >= D.nx) dx -= D.nx;
      else if (2 * dx <= -D.nx) dx += D.nx;
    }
    return mf((float)dx * D.hx, (float)(a.y - b.y) * D.hy, (float)dz * D.hz);
  }
};

// ---------------------------------------------------------------- plic_math.glslinc
DI float cube_volume(F3 normal, float alpha) {
  alpha -= mnf(normal.x, 0.f) + mnf(normal.y, 0.f) + mnf(normal.z, 0.f);
  F3 v = abs3(normal);
  float total = v.x + v.y + v.z;
  if (alpha <= 0.f) return 0.f;
  if (alpha >= total) return 1.f;
  float t;
  if (v.x > v.y) { t = v.x; v.x = v.y; v.y = t; }
  if (v.y > v.z) { t = v.y; v.y = v.z; v.z = t; }
  if (v.x > v.y) { t = v.x; v.x = v.y; v.y = t; }
  bool complement = alpha > 0.5f * total;
  t = complement ? total - alpha : alpha;
  float x = v.x, y = v.y, z = v.z, result;
  if (x < 1e-6f * total) {
    t -= x * 0.5f;
    if (y < 1e-6f * total) result = (t - y * 0.5f) / z;
    else if (t < y) result = t * t / (2.f * y * z);
    else result = (t - 0.5f * y) / z;
  } else if (t < x) result = t * t * t / (6.f * x * y * z);
  else if (t < y) result = (3.f * t * t - 3.f * t * x + x * x) / (6.f * y * z);
  else if (x + y < z && t >= x + y) result = (t - 0.5f * (x + y)) / z;
  else {
    float ty = mxf(t - y, 0.f), tz = mxf(t - z, 0.f);
    float numerator = x * (3.f * t * t - 3.f * t * x + x * x) - ty * ty * ty - tz * tz * tz;
    result = numerator / (6.f * x * y * z);
  }
  return complement ? 1.0f - result : result;
}
DI float inverse_volume(F3 normal, float fraction) {
  float lo = mnf(normal.x, 0.f) + mnf(normal.y, 0.f) + mnf(normal.z, 0.f);
  float hi = mxf(normal.x, 0.f) + mxf(normal.y, 0.f) + mxf(normal.z, 0.f);
  for (int it = 0; it < 25; it++) {
    float mid = 0.5f * (lo + hi);
    if (cube_volume(normal, mid) < fraction) lo = mid;
    else hi = mid;
  }
  float alpha = 0.5f * (lo + hi), cen = half_dot(normal);
  if (fraction == .5f) return cen;
  if (fraction < .5f) return mnf(alpha, cen);
  if (alpha <= cen) alpha = cen + 5.96046448e-8f * l1(normal);
  return alpha;
}

// ---------------------------------------------------------------- coastal_target.glslinc
struct Coast {
  const Dev& D;
  DI explicit Coast(const Dev& d) : D(d) {}
  DI static float smooth_ramp(float q) {
    q = clampf_(q, 0.f, 1.f);
    return q * q * q * (10.f + q * (-15.f + 6.f * q));
  }
  DI float ramped_amplitude(float time) const {
    return D.wave[0] * smooth_ramp(time * D.wave[2] / (6.28318530718f * D.forcing[3]));
  }
  DI void surface(float x, float time, float& s0, float& s1) const {
    float a = ramped_amplitude(time), k = D.wave[1], w = D.wave[2], hh = D.wave[3];
    float sigma = ttanh(k * hh), second = k * a * a * (3.f - sigma * sigma) / (4.f * sigma * sigma * sigma);
    if (!D.stokes2) second = 0.f;
    float phase = k * (x - D.forcing[0]) - w * time;
    s0 = a * tcos(phase) + second * tcos(2.f * phase);
    s1 = -k * a * tsin(phase) - 2.f * k * second * tsin(2.f * phase);
  }
  DI F3 velocity(F3 world, float time) const {
    float a = ramped_amplitude(time), k = D.wave[1], w = D.wave[2], hh = D.wave[3];
    float s = tsinh(k * hh), phase = k * (world.x - D.forcing[0]) - w * time, y = world.y + hh;
    float first = a * w / s, second = D.stokes2 ? .75f * a * a * w * k / tpow4(s) : 0.f;
    return mf(first * tcosh(k * y) * tcos(phase) + second * tcosh(2.f * k * y) * tcos(2.f * phase),
              first * tsinh(k * y) * tsin(phase) + second * tsinh(2.f * k * y) * tsin(2.f * phase), 0.f);
  }
  // single velocity component (avoids the unused transcendentals)
  DI float velocity_c(F3 world, float time, int axis) const {
    if (axis == 2) return 0.f;
    float a = ramped_amplitude(time), k = D.wave[1], w = D.wave[2], hh = D.wave[3];
    float s = tsinh(k * hh), phase = k * (world.x - D.forcing[0]) - w * time, y = world.y + hh;
    float first = a * w / s, second = D.stokes2 ? .75f * a * a * w * k / tpow4(s) : 0.f;
    if (axis == 0) return first * tcosh(k * y) * tcos(phase) + second * tcosh(2.f * k * y) * tcos(2.f * phase);
    return first * tsinh(k * y) * tsin(phase) + second * tsinh(2.f * k * y) * tsin(2.f * phase);
  }
  DI F3 face_position(const Grid& g, I3 q, int axis) const {
    F3 p = g.center(q);
    p[axis] -= .5f * g.h(axis);
    return p;
  }
  // Tabulated forms (entries are these same functions of the same arguments, so a lookup and a
  // direct evaluation give identical bits).
  DI int slot_of(float time) const {
    const float* s = D.wstamp;
    if (!s) return -1;
    return time == s[0] ? 0 : (time == s[1] ? 1 : (time == s[2] ? 2 : -1));
  }
  // surface() at the centre of cell column x
  DI void surface_col(const Grid& g, int x, float time, float& s0, float& s1) const {
    const int j = x - D.wt_x0;
    int sl;
    if (j >= 0 && j < D.wt_w && (sl = slot_of(time)) >= 0) {
      const float2 v = D.wsurf[sl * D.wt_w + j];
      s0 = v.x;
      s1 = v.y;
      return;
    }
    surface(g.center(mk(x, 0, 0)).x, time, s0, s1);
  }
  // velocity_c() at the position of face (q, axis); z does not enter the wave target.  Not inlined
  // (nor plane, fraction): most kernels call these only for the ghost columns left of the domain,
  // and inlined copies of the wave target's arithmetic made their code several times larger.
  __device__ __noinline__ float velocity_face(const Grid& g, I3 q, int axis, float time) const {
    if (axis == 2) return 0.f;
    const int j = q.x - D.wt_x0;
    int sl;
    if (j >= 0 && j < D.wt_w && q.y >= 0 && q.y < D.wt_h && (sl = slot_of(time)) >= 0)
      return D.wvel[((sl * 2 + axis) * D.wt_h + q.y) * D.wt_w + j];
    return velocity_c(face_position(g, q, axis), time, axis);
  }
  // relaxation factor 1 - exp(-rate dt) at a cell centre (axis < 0) or a face position
  DI float relax(const Grid& g, I3 q, int axis, float dt) const {
    const int j = q.x - D.wt_x0;
    if (D.wstamp && dt == D.wstamp[3] && j >= 0 && j < D.wt_w) return D.wdecay[(axis == 0 ? D.wt_w : 0) + j];
    const F3 p = axis < 0 ? g.center(q) : face_position(g, q, axis);
    return 1.f - texp(-rate(p.x) * dt);
  }
  __device__ __noinline__ float4 plane(const Grid& g, I3 q, float time) const {
    float s0, s1;
    F3 cq = g.center(q);
    surface_col(g, q.x, time, s0, s1);
    F3 normal = mf(-s1 * D.hx, D.hy, 0.f);
    return make_float4(normal.x, normal.y, normal.z, half_dot(normal) + s0 - cq.y);
  }
  __device__ __noinline__ float fraction(const Grid& g, I3 q, float time) const {
    float4 eq = plane(g, q, time);
    return clampf_(cube_volume(mf(eq.x, eq.y, eq.z), eq.w), 0.f, 1.f);
  }
  DI float rate(float x) const {
    float left = 1.f - smooth_ramp((x - D.forcing[0]) / D.forcing[1]);
    float right = D.shape == 6 ? smooth_ramp((x - (D.ox + (float)D.nx * D.hx - D.forcing[1])) / D.forcing[1]) : 0.f;
    return D.forcing[2] * mxf(left, D.right_abs * right);
  }
  DI bool offshore(float x) const { return x < D.forcing[0] + D.forcing[1]; }
};

// ---------------------------------------------------------------- PLIC reconstruction
// Normal from a gradient and the plane constant (pressure_geometry.glslinc:58-60,
// coupled_motion.glslinc:54-55).
DI float4 plane_from_gradient(const Dev& D, F3 g, float f) {
  if (len3(g) < 1e-9f) g = mf(0.f, 1.f, 0.f);
  float L = len3(g);
  F3 normal = mf(g.x / L * D.hx, g.y / L * D.hy, g.z / L * D.hz);
  float s = l1(normal);
  normal = mf(normal.x / s, normal.y / s, normal.z / s);
  return make_float4(normal.x, normal.y, normal.z, inverse_volume(normal, f));
}

// Weighted Youngs gradient (pressure_geometry.glslinc:35-53) over a fraction lookup `Fr`.
template <class Fr> DI F3 interface_gradient(const Grid& g, I3 q, const Fr& fr) {
  F3 grad = mf(0.f, 0.f, 0.f);
  for (int axis = 0; axis < 3; axis++) {
    int b = (axis + 1) % 3, d = (axis + 2) % 3, weights = 0;
    float acc = 0.f;
    float hh = g.h(axis);
    for (int j = -1; j <= 1; j++)
      for (int k = -1; k <= 1; k++) {
        I3 middle = q;
        middle[b] += j;
        middle[d] += k;
        if (g.solid(middle)) continue;
        I3 l = ax(middle, axis, -1), r = ax(middle, axis, 1);
        bool left = !g.solid(l), right = !g.solid(r);
        if (!left && !right) continue;
        float difference;
        if (left && right) difference = fr(l) - fr(r);
        else if (left) difference = 2.f * (fr(l) - fr(middle));
        else difference = 2.f * (fr(middle) - fr(r));
        int weight = (j == 0 ? 2 : 1) * (k == 0 ? 2 : 1);
        weights += weight;
        acc += (float)weight * difference / (32.f * hh);
      }
    if (weights > 0) acc *= 16.0f / (float)weights;
    grad[axis] = acc;
  }
  return grad;
}

// Height-function normal (height_normal.glslinc:6-34), flag bit 0.
template <class Fr> DI F3 height_normal(const Grid& g, I3 q, F3 youngs, const Fr& fr) {
  F3 sp = mf(g.D.hx, g.D.hy, g.D.hz);
  F3 scaled = mul3(abs3(youngs), sp);
  int axis = scaled.x > scaled.y ? 0 : 1;
  if (scaled.z > scaled[axis]) axis = 2;
  if (scaled[axis] < 1e-12f) return youngs;
  int b = (axis + 1) % 3, d = (axis + 2) % 3;
  float orientation = sgnf(youngs[axis]);
  float heights[5];
  for (int column = 0; column < 5; column++) {
    I3 base = q;
    if (column == 1) base[b]--;
    if (column == 2) base[b]++;
    if (column == 3) base[d]--;
    if (column == 4) base[d]++;
    float sum = 0.f, previous = orientation > 0.f ? 1.f : 0.f;
    for (int t = -4; t <= 4; t++) {
      I3 cell = ax(base, axis, t);
      I3 w = g.wrap_cell(cell);
      if (g.outside(w) || g.solid(w)) return youngs;
      float f = fr(cell);
      if (isnan(f) || isinf(f) || f < 0.f || f > 1.f) return youngs;
      if (orientation * (f - previous) > 2e-6f) return youngs;
      if (t == -4 && f != (orientation > 0.f ? 1.f : 0.f)) return youngs;
      if (t == 4 && f != (orientation > 0.f ? 0.f : 1.f)) return youngs;
      sum += f;
      previous = f;
    }
    heights[column] = sum * sp[axis];
  }
  F3 result = mf(0.f, 0.f, 0.f);
  result[axis] = orientation;
  result[b] = -(heights[2] - heights[1]) / (2.f * sp[b]);
  result[d] = -(heights[4] - heights[3]) / (2.f * sp[d]);
  return result;
}

// ---------------------------------------------------------------- deterministic reductions
// Block-wide reduction in a fixed tree; result valid in thread 0.
template <int NT, class T, class Op> DI T block_reduce(T v, Op op, T* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_down_sync(0xffffffffu, v, o));
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    v = sh[0];
    for (int w = 1; w < NT / 32; w++) v = op(v, sh[w]);
  }
  __syncthreads();
  return v;
}
struct AddD { DI double operator()(double a, double b) const { return a + b; } };
struct MaxD { DI double operator()(double a, double b) const { return a < b ? b : a; } };
struct MinF { DI float operator()(float a, float b) const { return (b < a) ? b : a; } };
struct MaxF { DI float operator()(float a, float b) const { return (a < b) ? b : a; } };

// K values per thread reduced over the block in FP64 with few FP64 instructions: every thread
// stores its values (one barrier), then warp w reduces value k = w, w + NT/32, ...: lane j
// combines entries j, j + 32, j + 64, ... in that order, then a shuffle tree over the lanes.
// The order is fixed, so the result is deterministic.  Totals land in tot[] (all threads).
// A value whose entries are all +0.0 in the block totals +0.0 (sum or maximum) without FP64
// instructions: each warp records which values it holds other bits of.
template <int NT, int K>
DI void block_reduce_k(const double (&vals)[K], const int (&ops)[K], double* sh, double* tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ unsigned nonzero[NT / 32];
  unsigned mine = 0;
#pragma unroll
  for (int k = 0; k < K; k++) {
    sh[k * NT + threadIdx.x] = vals[k];
    if (__any_sync(0xffffffffu, __double_as_longlong(vals[k]) != 0)) mine |= 1u << k;
  }
  if (lane == 0) nonzero[warp] = mine;
  __syncthreads();
  unsigned any = 0;
#pragma unroll
  for (int w = 0; w < NT / 32; w++) any |= nonzero[w];
  for (int k = warp; k < K; k += NT / 32) {
    if (!((any >> k) & 1u)) {
      if (lane == 0) tot[k] = 0.0;
      continue;
    }
    const bool mx = ops[k] != 0;
    double acc = sh[k * NT + lane];
#pragma unroll
    for (int i = 1; i < NT / 32; i++) {
      const double v = sh[k * NT + lane + 32 * i];
      acc = mx ? (acc < v ? v : acc) : acc + v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v = __shfl_down_sync(0xffffffffu, acc, o);
      acc = mx ? (acc < v ? v : acc) : acc + v;
    }
    if (lane == 0) tot[k] = acc;
  }
  __syncthreads();
}

// The last block's pass over nb per-block partials of one component: thread t combines partials
// t, t + NT, t + 2 NT, ... in that order (sum, op 0, or maximum), with kPartU loads issued before
// their additions, so the thread waits out one memory latency per kPartU partials, not per partial.
constexpr int kPartU = 4;
template <int NT> DI double partials_in_order(const double* part, int nb, int op) {
  double acc = op == 0 ? 0.0 : -1e300;
  for (int b0 = threadIdx.x; b0 < nb; b0 += kPartU * NT) {
    double p[kPartU];
#pragma unroll
    for (int u = 0; u < kPartU; u++) p[u] = b0 + u * NT < nb ? __ldcg(&part[b0 + u * NT]) : 0.0;
#pragma unroll
    for (int u = 0; u < kPartU; u++)
      if (b0 + u * NT < nb) acc = op == 0 ? acc + p[u] : (acc < p[u] ? p[u] : acc);
  }
  return acc;
}

// Write `K` per-block partials (double), then let the last block to finish reduce all partials
// in a fixed order.  Returns true in every thread of the last block, with the totals in `out`.
// `ops[k]` selects 0 = sum, 1 = max for each component.
template <int NT, int K>
DI bool last_block_reduce(const Dev& D, int site, double (&vals)[K], const int (&ops)[K], double (&out)[K]) {
  __shared__ double sh[K * NT];
  __shared__ double tot[K];
  __shared__ bool am_last;
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  double* part = D.part;
  block_reduce_k<NT, K>(vals, ops, sh, tot);
  if (threadIdx.x < K) part[(size_t)threadIdx.x * nb + bid] = tot[threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int prev = atomicAdd(&D.count[site], 1u);
    am_last = (prev == (unsigned)nb - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; k++) acc[k] = partials_in_order<NT>(part + (size_t)k * nb, nb, ops[k]);
  block_reduce_k<NT, K>(acc, ops, sh, tot);
#pragma unroll
  for (int k = 0; k < K; k++) out[k] = tot[k];
  if (threadIdx.x == 0) D.count[site] = 0;
  return true;
}


// Block maxima of K FP32 values: shuffle trees per warp, one barrier, the warps combined by
// threads 0..K-1.  Maxima are independent of the order of combination.
template <int NT, int K> DI void block_max_f(const float (&vals)[K], float (*shw)[NT / 32], float* tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    float m = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float x = __shfl_down_sync(0xffffffffu, m, o);
      m = m < x ? x : m;
    }
    if (lane == 0) shw[k][warp] = m;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    float m = shw[threadIdx.x][0];
    for (int w = 1; w < NT / 32; w++) m = m < shw[threadIdx.x][w] ? shw[threadIdx.x][w] : m;
    tot[threadIdx.x] = m;
  }
  __syncthreads();
}

// last_block_reduce with KD FP64 components (sums or maxima, `ops`) and KF FP32 maxima (the
// maxima of FP32 values need no FP64 instructions: the same value results in either precision).
// The FP32 partials follow the FP64 ones in D.part (KD + KF <= 9).
template <int NT, int KD, int KF>
DI bool last_block_reduce_mf(const Dev& D, int site, const double* vals, const int* ops, const float (&fvals)[KF],
                             double* out, float (&fout)[KF]) {
  static_assert(KD + KF <= 9, "partials buffer holds 9 values per block");
  __shared__ double sh[(KD > 0 ? KD : 1) * NT];
  __shared__ double tot[KD > 0 ? KD : 1];
  __shared__ float shw[KF][NT / 32];
  __shared__ float totf[KF];
  __shared__ bool am_last;
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  double* part = D.part;
  float* partf = (float*)(D.part + (size_t)KD * nb);
  int opk[KD > 0 ? KD : 1];
  if constexpr (KD > 0) {
    double v[KD];
#pragma unroll
    for (int k = 0; k < KD; k++) {
      v[k] = vals[k];
      opk[k] = ops[k];
    }
    block_reduce_k<NT, KD>(v, opk, sh, tot);
  }
  block_max_f<NT, KF>(fvals, shw, totf);
  if constexpr (KD > 0)
    if (threadIdx.x < KD) part[(size_t)threadIdx.x * nb + bid] = tot[threadIdx.x];
  if (threadIdx.x < KF) partf[(size_t)threadIdx.x * nb + bid] = totf[threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int prev = atomicAdd(&D.count[site], 1u);
    am_last = (prev == (unsigned)nb - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  if constexpr (KD > 0) {
    double acc[KD];
#pragma unroll
    for (int k = 0; k < KD; k++) acc[k] = partials_in_order<NT>(part + (size_t)k * nb, nb, opk[k]);
    block_reduce_k<NT, KD>(acc, opk, sh, tot);
#pragma unroll
    for (int k = 0; k < KD; k++) out[k] = tot[k];
  }
  float accf[KF];
#pragma unroll
  for (int k = 0; k < KF; k++) {
    accf[k] = -INFINITY;
    // kPartU loads in flight per thread; maxima do not depend on the order anyway
    for (int b0 = threadIdx.x; b0 < nb; b0 += kPartU * NT) {
      float p[kPartU];
#pragma unroll
      for (int u = 0; u < kPartU; u++) p[u] = b0 + u * NT < nb ? __ldcg(&partf[(size_t)k * nb + b0 + u * NT]) : -INFINITY;
#pragma unroll
      for (int u = 0; u < kPartU; u++) accf[k] = accf[k] < p[u] ? p[u] : accf[k];
    }
  }
  block_max_f<NT, KF>(accf, shw, totf);
#pragma unroll
  for (int k = 0; k < KF; k++) fout[k] = totf[k];
  if (threadIdx.x == 0) D.count[site] = 0;
  return true;
}

// ---------------------------------------------------------------- PCG control (pressure_core.glslinc:156-179)
DI bool solving(const Dev& D) { return D.c[4] > 0.5 && D.c[6] < 0.5 && D.c[7] < 0.5; }
DI bool pressure_setup(const Dev& D) { return D.c[5] > .5 || D.c[57] == 2; }

// pressure_norm_converged / residual_converged (pressure_core.glslinc:173-178)
DI double scaled_norm(const Dev& D, double sq) {
  double d = D.c[20];
  return d * d / 1000 * sqrt(sq > 0 ? sq : 0.0);
}
DI bool norm_converged(const Dev& D, double res2, double rhs2) {
  double t = (double)D.tol;
  return res2 <= t * t * rhs2 || (scaled_norm(D, rhs2) <= 1e-5 && scaled_norm(D, res2) <= 1e-8);
}
DI bool residual_converged(const Dev& D, const double* s, double rhs2) {
  double d = D.c[20];
  return norm_converged(D, s[1], rhs2) && d * d / 1000 * s[3] < 5e-5;
}

// op 4 finalisation (pressure_iterations.glslinc:332-337)
DI void finalize_op4(const Dev& D, const double* s) {
  double* c = D.c;
  c[9] = s[0];
  c[10] = s[2];
  c[13] = sqrt(s[1] / (s[2] > 1e-30 ? s[2] : 1e-30));
  if (residual_converged(D, s, s[2])) c[6] = 1;
  if (c[58] == 0) c[59] = s[2];
  c[57] = 0;
}
// op 9 finalisation (pressure_iterations.glslinc:349)
DI void finalize_op9(const Dev& D, const double* s) {
  double* c = D.c;
  c[12] = s[0] / (c[9] > 1e-30 ? c[9] : 1e-30);
  c[9] = s[0];
  c[8] += 1;
  c[18] += 1;
  c[13] = sqrt(s[1] / (c[10] > 1e-30 ? c[10] : 1e-30));
  if (isnan(c[13]) || isinf(c[13])) c[7] = 2;
  else if (residual_converged(D, s, c[10])) c[6] = 1;
  else if (c[8] > 4096) c[7] = 3;
  // The reference runs ipb iterations per batch and every batch starts with op 1, which clears
  // the set-up flag (pressure_pass.glslinc:20-24); a trial still solving after a whole batch
  // continues in the next one.
  if (c[6] < .5 && c[7] < .5 && D.ipb > 0 && (long long)c[8] % D.ipb == 0) c[5] = 0;
}


// Multigrid storage: FP32 or BF16 values with FP32 arithmetic.
template <class T> DI T st_val(float x);
template <> DI float st_val<float>(float x) { return x; }
template <> DI __nv_bfloat16 st_val<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
DI float ld_val(float x) { return x; }
DI float ld_val(__nv_bfloat16 x) { return __bfloat162float(x); }

// Read the accepted/candidate bank pointers.
DI float* bank_ptr(const Dev& D, int b) { return b == 0 ? D.bank0 : D.bank1; }
DI int acc_bank(const Dev& D) { return (int)D.c[0]; }

}  // namespace wg
