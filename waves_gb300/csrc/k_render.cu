// Headless presentation of the exported PLIC surface: one ray per pixel, marched cell by cell
// through the op-19 planes and kinds (neuron-forest/waves water/presentation/water.gdshader:21-176,
// water/presentation/daylight.gdshaderinc:1-16, water/shaders/render/clay.gdshader:8-66).
//
// The reference runs these as Godot fragment shaders over a volume proxy; here the camera rays are
// generated in the kernel and the colour goes to a float RGBA buffer.  What the fragment shader
// reads from the rendered scene (screen and depth textures) is replaced by an analytic scene: the
// sky of daylight() and the sand bed y = -0.45 + max(0, x - 1.5) / slope.  Every FP32 operation is
// spelled out in the shader's order (the library is built without multiply-add contraction);
// transcendentals are evaluated in FP64 and rounded to FP32.
#include "kernels.h"

namespace wg {

namespace {

#define RD __device__ __forceinline__

struct V3 {
  float x, y, z;
};
RD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
RD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
RD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
RD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
RD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
RD V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
RD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
RD V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
RD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RD float length(V3 a) { return __fsqrt_rn(dot(a, a)); }
RD V3 normalize(V3 a) {
  const float l = length(a);
  return v3(a.x / l, a.y / l, a.z / l);
}
RD V3 vmin(V3 a, V3 b) { return v3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
RD V3 vmax(V3 a, V3 b) { return v3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
RD V3 mix(V3 a, V3 b, float t) { return a * (1.f - t) + b * t; }
RD float sgn(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
RD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
RD float smoothstep(float e0, float e1, float x) {
  const float t = clampf((x - e0) / (e1 - e0), 0.f, 1.f);
  return t * t * (3.f - 2.f * t);
}
RD float powd(float x, float y) { return (float)pow((double)x, (double)y); }
RD float expd(float x) { return (float)exp((double)x); }
RD float sind(float x) { return (float)sin((double)x); }
RD float cosd(float x) { return (float)cos((double)x); }
RD V3 expd(V3 a) { return v3(expd(a.x), expd(a.y), expd(a.z)); }
RD V3 xyz(float4 p) { return v3(p.x, p.y, p.z); }
// GLSL floor-then-int, with the float clamped first so that the conversion stays in range
RD int cell_index(float x, int n) { return (int)floorf(clampf(x, -1.f, (float)n)); }

struct Scene {
  const RenderArgs& A;
  V3 bmin, bmax, h, sun;
  int n[3];
  RD explicit Scene(const RenderArgs& a) : A(a) {
    bmin = v3(a.bmin[0], a.bmin[1], a.bmin[2]);
    bmax = v3(a.bmax[0], a.bmax[1], a.bmax[2]);
    n[0] = a.nx;
    n[1] = a.ny;
    n[2] = a.nz;
    h = (bmax - bmin) / v3((float)a.nx, (float)a.ny, (float)a.nz);
    sun = normalize(v3(a.sun[0], a.sun[1], a.sun[2]));
  }
  RD long long at(int x, int y, int z) const { return ((long long)z * n[1] + y) * n[0] + x; }
  RD float kind(int x, int y, int z) const { return __ldg(A.kinds + at(x, y, z)); }
  RD float4 plane(int x, int y, int z) const { return __ldg(A.planes + at(x, y, z)); }

  // daylight_reflection / daylight (daylight.gdshaderinc:3-16)
  RD V3 sky_reflection(V3 d) const {
    const float up = clampf(d.y, 0.f, 1.f);
    V3 sky = mix(v3(0.24f, 0.43f, 0.55f), v3(0.065f, 0.19f, 0.35f), powd(up, 0.45f));
    if (d.y < 0.f) sky = mix(v3(0.43f, 0.34f, 0.21f), v3(0.24f, 0.43f, 0.55f), expd(d.y * 12.f));
    const float s = fmaxf(dot(sun, d), 0.f);
    return sky + v3(1.f, 0.87f, 0.65f) * 0.035f * powd(s, 32.f);
  }
  RD V3 sky(V3 d) const {
    const float s = fmaxf(dot(sun, d), 0.f);
    return sky_reflection(d) + v3(1.f, 0.87f, 0.65f) * 2.f * powd(s, 1800.f);
  }
  // Distance along the ray to the sand bed over the domain's x-z footprint (the bed mesh of
  // presentation.gd:94-112), or -1.  The bed is linear on each side of x = 1.5.
  RD float bed_hit(V3 o, V3 d) const {
    if (!(A.slope > 0.f)) return -1.f;
    float best = -1.f;
    for (int piece = 0; piece < 2; piece++) {
      const float g = piece == 0 ? 0.f : 1.f / A.slope;
      // o.y + t d.y = -0.45 + g (o.x + t d.x - 1.5)
      const float rate = d.y - g * d.x;
      if (fabsf(rate) < 1e-10f) continue;
      const float t = (-0.45f + g * (o.x - 1.5f) - o.y) / rate;
      if (!(t > 0.f)) continue;
      const V3 p = o + d * t;
      if (piece == 0 ? p.x > 1.5f : p.x <= 1.5f) continue;
      if (p.x < bmin.x || p.x > bmax.x || p.z < bmin.z || p.z > bmax.z) continue;
      if (best < 0.f || t < best) best = t;
    }
    return best;
  }
  // The opaque scene behind the water (stand-in for the screen texture): lit sand with the
  // base colours of sand.gdshader:6-9 (grain at its mean), else the sky with its sun disk.
  RD V3 opaque(V3 o, V3 d, float t_bed) const {
    if (t_bed < 0.f) return sky(d);
    const V3 w = o + d * t_bed;
    const float ribbons = sind(w.x * 19.f + sind(w.z * 4.f) * 1.8f) * 0.006f;
    const float damp = 1.f - smoothstep(-0.02f, 0.20f, w.y);
    const V3 sand = mix(v3(0.88f, 0.69f, 0.42f), v3(0.56f, 0.41f, 0.23f), damp * 0.55f) * (0.98f + 0.02f + ribbons);
    const V3 nb = normalize(v3(w.x > 1.5f ? -1.f / A.slope : 0.f, 1.f, 0.f));
    const float lit = fmaxf(dot(nb, sun), 0.f) * 1.1f;
    return sand * (v3(0.35f, 0.35f, 0.35f) + v3(1.f, 0.94f, 0.83f) * lit);
  }

  // trace_water (water.gdshader:23-91): the summed occupied PLIC intervals, the first entry, the
  // exit of the first connected interval, and the texture queries.
  RD float4 trace_water(V3 o, V3 d, float limit, V3& first_normal, float& first_exit, bool& complete) const {
    const V3 sd = v3(fabsf(d.x) < 1e-8f ? 1e-8f : d.x, fabsf(d.y) < 1e-8f ? 1e-8f : d.y, fabsf(d.z) < 1e-8f ? 1e-8f : d.z);
    const V3 a = (bmin - o) / sd, b = (bmax - o) / sd, lo = vmin(a, b), hi = vmax(a, b);
    const float start = fmaxf(0.f, fmaxf(lo.x, fmaxf(lo.y, lo.z)));
    const float finish = fminf(limit, fminf(hi.x, fminf(hi.y, hi.z)));
    float first = -1.f, occupied = 0.f, last_end = -1.f;
    first_exit = -1.f;
    complete = true;
    first_normal = v3(0.f, 1.f, 0.f);
    V3 entry;
    if (lo.x >= lo.y && lo.x >= lo.z) entry = v3(-sgn(d.x), 0.f, 0.f);
    else if (lo.y >= lo.z) entry = v3(0.f, -sgn(d.y), 0.f);
    else entry = v3(0.f, 0.f, -sgn(d.z));
    if (finish <= start) return make_float4(-1.f, 0.f, 0.f, 0.f);
    const bool contact = A.contact && A.slope > 0.f;
    float t = start;
    int queries = 0;
    bool open_first = false;
    for (int step = 0; step < 640; step++) {
      if (t >= finish - 1e-7f) break;
      const V3 probe = o + d * (t + 1e-6f);
      const V3 r = (probe - bmin) / h;
      const int cx = min(max(cell_index(r.x, n[0]), 0), n[0] - 1);
      const int cy = min(max(cell_index(r.y, n[1]), 0), n[1] - 1);
      const int cz = min(max(cell_index(r.z, n[2]), 0), n[2] - 1);
      const V3 corner = bmin + v3((float)cx, (float)cy, (float)cz) * h;
      const V3 next = corner + v3(d.x >= 0.f ? h.x : 0.f, d.y >= 0.f ? h.y : 0.f, d.z >= 0.f ? h.z : 0.f);
      const V3 exits = (next - o) / sd;
      const float end = fminf(finish, fminf(exits.x, fminf(exits.y, exits.z)));
      if (end <= t + 1e-8f) {
        t += 1e-6f;
        continue;
      }
      float kind = kind_at(cx, cy, cz);
      queries++;
      float4 plane = make_float4(0.f, 0.f, 0.f, 0.f);
      if (kind > 1.5f) plane = this->plane(cx, cy, cz);
      float bed_x = 0.f, bed_center = 0.f;
      if (contact) {
        // extend the wet footprint from the voxel top to the smooth bed (water.gdshader:46-57)
        bed_x = bmin.x + ((float)cx + 0.5f) * h.x;
        bed_center = -0.45f + fmaxf(0.f, bed_x - 1.5f) / A.slope;
        int bottom = cell_index((bed_center - bmin.y) / h.y - 0.5f, n[1] + 2) + 1;
        if (bmin.y + ((float)bottom + 0.5f) * h.y <= bed_center) bottom++;
        if (bmin.y + ((float)bottom - 0.5f) * h.y > bed_center) bottom--;
        if (cy == bottom - 1 && bottom >= 0 && bottom < n[1]) {
          kind = kind_at(cx, bottom, cz);
          if (kind > 1.5f) {
            plane = this->plane(cx, bottom, cz);
            plane.y = 0.f;
          }
        }
      }
      float enter = t, leave = end;
      V3 normal = entry;
      if (kind > 1.5f) {
        queries++;
        const V3 pn = xyz(plane);
        const float rate = dot(pn, d / h), value = dot(pn, (o - corner) / h) - plane.w;
        if (fabsf(rate) < 1e-10f) {
          if (value > 0.f) leave = enter;
        } else if (rate < 0.f) {
          const float crossing = -value / rate;
          if (crossing > enter) {
            enter = crossing;
            normal = normalize(pn / h);
          }
        } else {
          leave = fminf(leave, -value / rate);
        }
      } else if (kind < 0.5f) {
        leave = enter;
      }
      if (contact) {
        // clip buried PLIC water against the continuous bed (water.gdshader:66-75)
        const float gradient = bed_x > 1.5f ? 1.f / A.slope : 0.f;
        const float value = o.y - bed_center - gradient * (o.x - bed_x);
        const float rate = d.y - gradient * d.x;
        if (fabsf(rate) < 1e-10f) {
          if (value < 0.f) leave = enter;
        } else if (rate > 0.f) {
          const float crossing = -value / rate;
          if (crossing > enter) {
            enter = crossing;
            normal = normalize(v3(gradient, -1.f, 0.f));
          }
        } else {
          leave = fminf(leave, -value / rate);
        }
      }
      enter = fmaxf(t, enter);
      leave = fminf(end, leave);
      if (leave > enter + 1e-7f) {
        occupied += leave - enter;
        if (first < 0.f) {
          first = enter;
          first_normal = normal;
          open_first = true;
        } else if (enter > last_end + 4e-6f) {
          open_first = false;
        }
        if (open_first) first_exit = leave;
        last_end = leave;
      } else if (first >= 0.f) {
        open_first = false;
      }
      if (exits.x <= exits.y && exits.x <= exits.z) entry = v3(-sgn(d.x), 0.f, 0.f);
      else if (exits.y <= exits.z) entry = v3(0.f, -sgn(d.y), 0.f);
      else entry = v3(0.f, 0.f, -sgn(d.z));
      t = end;
      if (step == 639 && t < finish - 1e-6f) complete = false;
    }
    return make_float4(first, occupied, finish, (float)queries);
  }
  RD float kind_at(int x, int y, int z) const { return kind(x, y, z); }

  // normal_weight (water.gdshader:92-95); the square is written as a product
  RD static float normal_weight(float x) {
    x = fabsf(x);
    if (x < 0.5f) return 0.75f - x * x;
    const float r = fmaxf(0.f, 1.5f - x);
    return 0.5f * (r * r);
  }
  // optical_normal (water.gdshader:96-124)
  RD V3 optical_normal(V3 hit, V3 geometric) const {
    const V3 rel = (hit - bmin) / h;
    const V3 local = rel - v3(0.5f, 0.5f, 0.5f);
    const int lx = cell_index(local.x, n[0] + 2), ly = cell_index(local.y, n[1] + 2), lz = cell_index(local.z, n[2] + 2);
    const float hmin = fminf(h.x, h.y);
    V3 anchor = geometric;
    float closest = 1e10f;
    for (int z = 0; z < 2; z++)
      for (int y = 0; y < 2; y++)
        for (int x = 0; x < 2; x++) {
          const int qx = lx + x, qy = ly + y, qz = lz + z;
          if (qx < 0 || qy < 0 || qz < 0 || qx >= n[0] || qy >= n[1] || qz >= n[2]) continue;
          if (kind(qx, qy, qz) < 1.5f) continue;
          const float4 p = plane(qx, qy, qz);
          const V3 raw = xyz(p) / h;
          const float ln = length(raw);
          if (ln < 1e-8f) continue;
          const V3 nrm = v3(raw.x / ln, raw.y / ln, raw.z / ln);
          const V3 q = v3((float)qx, (float)qy, (float)qz);
          const float distance = fabsf(dot(xyz(p), rel - q) - p.w) / ln;
          const float score = distance / hmin + 0.15f * length(local - q);
          if (distance < 0.8f * hmin && score < closest) {
            closest = score;
            anchor = nrm;
          }
        }
    V3 sum = v3(0.f, 0.f, 0.f);
    float weights = 0.f;
    const int cx = cell_index(rel.x, n[0] + 2), cy = cell_index(rel.y, n[1] + 2), cz = cell_index(rel.z, n[2] + 2);
    for (int z = -1; z <= 1; z++)
      for (int y = -1; y <= 1; y++)
        for (int x = -2; x <= 2; x++) {
          const int qx = cx + x, qy = cy + y, qz = cz + z;
          if (qx < 0 || qy < 0 || qz < 0 || qx >= n[0] || qy >= n[1] || qz >= n[2]) continue;
          if (kind(qx, qy, qz) < 1.5f) continue;
          const float4 p = plane(qx, qy, qz);
          const V3 raw = xyz(p) / h;
          const float ln = length(raw);
          if (ln < 1e-8f) continue;
          const V3 nrm = v3(raw.x / ln, raw.y / ln, raw.z / ln);
          const V3 q = v3((float)qx, (float)qy, (float)qz);
          const float distance = fabsf(dot(xyz(p), rel - q) - p.w) / ln;
          const V3 delta = local - q;
          const float w = normal_weight(delta.x * 0.6f) * normal_weight(delta.y) * normal_weight(delta.z) *
                          smoothstep(0.15f, 0.8f, dot(nrm, anchor)) * (1.f - smoothstep(0.7f, 1.5f, distance / hmin));
          sum = sum + nrm * w;
          weights += w;
        }
    return weights > 0.001f ? normalize(sum) : anchor;
  }

  // fragment() of water.gdshader:125-176 with the scene stand-ins
  RD float4 water(V3 o, V3 d, float4& trace) const {
    const float t_bed = bed_hit(o, d);
    const V3 behind = opaque(o, d, t_bed);
    V3 gn;
    float first_exit;
    bool complete;
    trace = trace_water(o, d, t_bed >= 0.f ? t_bed : 10000.f, gn, first_exit, complete);
    const float first = trace.x, occupied = trace.y;
    trace.z = first_exit;
    if (first < 0.f || !complete) return make_float4(behind.x, behind.y, behind.z, 1.f);
    const V3 hit = o + d * first;
    V3 nrm = optical_normal(hit, gn);
    if (dot(nrm, -d) < 0.f) nrm = -nrm;
    const V3 smooth = nrm;
    const float time = A.clock_ready ? (float)A.c[1] : 0.f;
    V3 ripple = v3(cosd(hit.x * 75.f + hit.z * 31.f - time * 2.5f), 0.f, sind(hit.z * 103.f - hit.x * 22.f + time * 3.1f));
    ripple = ripple + 0.35f * v3(sind(hit.z * 160.f + time * 4.f), cosd(hit.x * 95.f + time), cosd(hit.x * 140.f - time * 3.f));
    nrm = normalize(nrm + A.ripple * (ripple - nrm * dot(ripple, nrm)));
    const float nv = clampf(dot(smooth, -d), 0.f, 1.f);
    const float fresnel = 0.02037f + (0.97963f - A.roughness * 0.35f) * powd(1.f - nv, 5.f);
    const V3 rd = d - nrm * (2.f * dot(nrm, d));  // reflect(d, n)
    const V3 reflection = sky_reflection(rd);
    const float att = fmaxf(A.attenuation, 0.01f);
    const V3 absorption = v3(1.4f / att, 1.f / att, 0.85f / att);
    const V3 transmission = expd(-absorption * occupied);
    const float deeper = 1.f - expd(-occupied / 0.45f);
    V3 scatter = v3(A.tint[0], A.tint[1], A.tint[2]) * mix(v3(0.65f, 1.18f, 1.f), v3(0.4f, 0.65f, 0.92f), deeper);
    scatter = scatter * (0.55f + 0.45f * fmaxf(dot(smooth, sun), 0.f));
    const V3 body = behind * transmission + scatter * (v3(1.f, 1.f, 1.f) - transmission);
    const V3 half_vector = normalize(sun - d);
    const float nh = fmaxf(dot(nrm, half_vector), 0.f), a = A.roughness * A.roughness, a2 = a * a;
    const float den = fmaxf(nh * nh * (a2 - 1.f) + 1.f, 0.001f);
    const float distribution = a2 / (3.14159265f * (den * den));
    const float nl = fmaxf(dot(nrm, sun), 0.f);
    const V3 sunc = v3(1.f, 0.90f, 0.74f) * fminf(0.6f, distribution * 0.007f) * nl;
    const V3 color = mix(body, reflection, fresnel) + sunc;
    return make_float4(color.x, color.y, color.z, 1.f);
  }

  // fragment() of clay.gdshader:8-66: first liquid entry, Lambert shading, magenta on overflow
  RD float4 clay(V3 o, V3 d, float4& trace) const {
    const V3 sd = v3(fabsf(d.x) < 1e-8f ? 1e-8f : d.x, fabsf(d.y) < 1e-8f ? 1e-8f : d.y, fabsf(d.z) < 1e-8f ? 1e-8f : d.z);
    const V3 t0 = (bmin - o) / sd, t1 = (bmax - o) / sd, lo = vmin(t0, t1), hi = vmax(t0, t1);
    const float start = fmaxf(0.f, fmaxf(lo.x, fmaxf(lo.y, lo.z))), finish = fminf(hi.x, fminf(hi.y, hi.z));
    trace = make_float4(-1.f, 0.f, finish, 0.f);
    if (finish <= start) return make_float4(0.f, 0.f, 0.f, 0.f);
    float t = start + 1e-6f, first = -1.f, occupied = 0.f;
    V3 first_normal = v3(0.f, 1.f, 0.f), entry_normal = v3(0.f, 1.f, 0.f);
    int queries = 0;
    bool overflow = true;
    for (int step = 0; step < 512; step++) {
      if (t >= finish - 1e-6f) {
        overflow = false;
        break;
      }
      const V3 x = o + d * t;
      const V3 r = (x - bmin) / h;
      const int cx = min(max(cell_index(r.x, n[0]), 0), n[0] - 1);
      const int cy = min(max(cell_index(r.y, n[1]), 0), n[1] - 1);
      const int cz = min(max(cell_index(r.z, n[2]), 0), n[2] - 1);
      const V3 corner = bmin + v3((float)cx, (float)cy, (float)cz) * h;
      const V3 next = corner + v3(d.x >= 0.f ? h.x : 0.f, d.y >= 0.f ? h.y : 0.f, d.z >= 0.f ? h.z : 0.f);
      const V3 exits = (next - o) / sd;
      float end = fminf(finish, fminf(exits.x, fminf(exits.y, exits.z)));
      end = fmaxf(t + 1e-7f, end);
      const float kind = this->kind(cx, cy, cz);
      queries++;
      float enter = t, leave = end;
      V3 normal = entry_normal;
      if (kind > 1.5f) {
        const float4 p = plane(cx, cy, cz);
        queries++;
        const V3 pn = xyz(p);
        const float rate = dot(pn, d / h), value = dot(pn, (o - corner) / h) - p.w;
        if (fabsf(rate) < 1e-10f) {
          if (value > 0.f) leave = enter;
        } else {
          const float crossing = -value / rate;
          if (rate < 0.f) {
            if (crossing > enter) {
              enter = crossing;
              normal = normalize(pn / h);
            }
          } else {
            leave = fminf(leave, crossing);
          }
        }
      } else if (kind < 0.5f) {
        leave = enter;
      }
      enter = fmaxf(t, enter);
      leave = fminf(end, leave);
      if (leave > enter + 1e-7f) {
        occupied += leave - enter;
        if (first < 0.f) {
          first = enter;
          first_normal = normal;
          overflow = false;
          break;
        }
      }
      if (exits.x <= exits.y && exits.x <= exits.z) entry_normal = v3(-sgn(d.x), 0.f, 0.f);
      else if (exits.y <= exits.z) entry_normal = v3(0.f, -sgn(d.y), 0.f);
      else entry_normal = v3(0.f, 0.f, -sgn(d.z));
      t = end + 1e-6f;
    }
    trace = make_float4(first, occupied, finish, (float)queries);
    if (first < 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
    if (overflow) return make_float4(1.f, 0.f, 1.f, 1.f);
    const float diffuse = 0.28f + 0.72f * fmaxf(0.f, dot(first_normal, normalize(v3(-0.4f, 0.8f, 0.5f))));
    const float g = 0.54f * diffuse;
    return make_float4(g, g, g, 1.f);
  }
};

// One thread per pixel, 16 x 8 pixel tiles (neighbouring rays walk neighbouring cells).
__global__ void __launch_bounds__(128) k_render(const __grid_constant__ RenderArgs A) {
  const int px = blockIdx.x * 16 + (threadIdx.x & 15), py = blockIdx.y * 8 + (threadIdx.x >> 4);
  if (px >= A.width || py >= A.height) return;
  const Scene S(A);
  // camera ray: pixel centres, row 0 at the top
  const float sx = ((float)px + 0.5f) / (float)A.width * 2.f - 1.f;
  const float sy = 1.f - ((float)py + 0.5f) / (float)A.height * 2.f;
  const V3 eye = v3(A.eye[0], A.eye[1], A.eye[2]), f = v3(A.fwd[0], A.fwd[1], A.fwd[2]);
  const V3 r = v3(A.right[0], A.right[1], A.right[2]), u = v3(A.up[0], A.up[1], A.up[2]);
  V3 o, d;
  if (A.ortho) {
    o = eye + r * (sx * A.half_w) + u * (sy * A.half_h);
    d = f;
  } else {
    o = eye;
    d = normalize(f + r * (sx * A.half_w) + u * (sy * A.half_h));
  }
  float4 trace;
  const float4 rgba = A.mode == 0 ? S.clay(o, d, trace) : S.water(o, d, trace);
  const long long i = (long long)py * A.width + px;
  A.rgba[i] = rgba;
  if (A.trace) A.trace[i] = trace;
}

}  // namespace

void launch_render(const RenderArgs& A, cudaStream_t s) {
  const dim3 grid((unsigned)((A.width + 15) / 16), (unsigned)((A.height + 7) / 8));
  k_render<<<grid, 128, 0, s>>>(A);
}

}  // namespace wg
