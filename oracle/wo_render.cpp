// TEST INFRASTRUCTURE ONLY: CPU restatement of the presentation ray-march, against which the tests
// compare the library's waves_render.  Follows neuron-forest/waves water/presentation/water.gdshader:21-176
// (trace_water, normal_weight, optical_normal, fragment), water/presentation/
// daylight.gdshaderinc:1-16 and water/shaders/render/clay.gdshader:8-66 statement by statement,
// in FP32 with no contraction (-ffp-contract=off); transcendentals in FP64 rounded to FP32.
//
// Where the fragment shaders read the rendered scene (screen and depth textures), this restatement
// uses the analytic scene the library documents: the sky of daylight(), and the sand bed
// y = -0.45 + max(0, x - 1.5) / slope over the domain footprint (presentation.gd:94-112), lit by
// the directional light of presentation.gd:26 plus a constant ambient term.
//
// Parity is unpinned for this file: the reference's shaders need Godot's renderer and cannot run
// here, so there are no reference images to compare against.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../include/waves.h"

namespace {

struct F3 {
  float x, y, z;
};
F3 f3(float x, float y, float z) { return F3{x, y, z}; }
F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
F3 neg(F3 a) { return f3(-a.x, -a.y, -a.z); }
F3 mul(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
F3 div(F3 a, F3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
F3 scale(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float len(F3 a) { return std::sqrt(dot(a, a)); }
F3 unit(F3 a) {
  const float l = len(a);
  return f3(a.x / l, a.y / l, a.z / l);
}
// GLSL mix(a, b, t) = a (1 - t) + b t
F3 mix(F3 a, F3 b, float t) { return add(scale(a, 1.f - t), scale(b, t)); }
float sign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
float smoothstep(float e0, float e1, float x) {
  const float t = clamp((x - e0) / (e1 - e0), 0.f, 1.f);
  return t * t * (3.f - 2.f * t);
}
float p64(float x, float y) { return (float)std::pow((double)x, (double)y); }
float e64(float x) { return (float)std::exp((double)x); }
float s64(float x) { return (float)std::sin((double)x); }
float c64(float x) { return (float)std::cos((double)x); }
int ifloor(float x) { return (int)std::floor(x); }
F3 safe_ray(F3 d) {
  return f3(std::fabs(d.x) < 1e-8f ? 1e-8f : d.x, std::fabs(d.y) < 1e-8f ? 1e-8f : d.y, std::fabs(d.z) < 1e-8f ? 1e-8f : d.z);
}

struct Volume {
  const float* planes;
  const float* kinds;
  int n[3];
  F3 bmin, bmax, h;
  float slope;
  size_t at(int x, int y, int z) const { return ((size_t)z * n[1] + y) * n[0] + x; }
  float kind(int x, int y, int z) const { return kinds[at(x, y, z)]; }
  void plane(int x, int y, int z, float p[4]) const { std::memcpy(p, planes + 4 * at(x, y, z), 4 * sizeof(float)); }
  bool inside(int x, int y, int z) const { return x >= 0 && y >= 0 && z >= 0 && x < n[0] && y < n[1] && z < n[2]; }
  int clampc(int v, int k) const { return v < 0 ? 0 : (v > n[k] - 1 ? n[k] - 1 : v); }
};

struct Look {
  F3 tint, sun;
  float attenuation, ripple, roughness;
  bool contact, clock_ready;
  float time;
};

// daylight_reflection (daylight.gdshaderinc:3-10)
F3 daylight_reflection(F3 d, F3 sun_n) {
  const float up = clamp(d.y, 0.f, 1.f);
  F3 sky = mix(f3(0.24f, 0.43f, 0.55f), f3(0.065f, 0.19f, 0.35f), p64(up, 0.45f));
  if (d.y < 0.f) sky = mix(f3(0.43f, 0.34f, 0.21f), f3(0.24f, 0.43f, 0.55f), e64(d.y * 12.f));
  const float sun = std::fmax(dot(sun_n, d), 0.f);
  return add(sky, scale(scale(f3(1.f, 0.87f, 0.65f), 0.035f), p64(sun, 32.f)));
}
// daylight (daylight.gdshaderinc:11-16)
F3 daylight(F3 d, F3 sun_n) {
  const float sun = std::fmax(dot(sun_n, d), 0.f);
  return add(daylight_reflection(d, sun_n), scale(scale(f3(1.f, 0.87f, 0.65f), 2.f), p64(sun, 1800.f)));
}

// First crossing of the ray with the two linear pieces of the bed inside the footprint, or -1.
float bed_distance(const Volume& V, F3 o, F3 d) {
  if (!(V.slope > 0.f)) return -1.f;
  float best = -1.f;
  for (int piece = 0; piece < 2; piece++) {
    const float g = piece == 0 ? 0.f : 1.f / V.slope;
    const float rate = d.y - g * d.x;
    if (std::fabs(rate) < 1e-10f) continue;
    const float t = (-0.45f + g * (o.x - 1.5f) - o.y) / rate;
    if (!(t > 0.f)) continue;
    const F3 p = add(o, scale(d, t));
    if (piece == 0 ? p.x > 1.5f : p.x <= 1.5f) continue;
    if (p.x < V.bmin.x || p.x > V.bmax.x || p.z < V.bmin.z || p.z > V.bmax.z) continue;
    if (best < 0.f || t < best) best = t;
  }
  return best;
}
// Scene colour along the ray: lit sand (sand.gdshader:6-9, grain at its mean) or the sky.
F3 scene(const Volume& V, F3 o, F3 d, float t_bed, F3 sun_n) {
  if (t_bed < 0.f) return daylight(d, sun_n);
  const F3 w = add(o, scale(d, t_bed));
  const float ribbons = s64(w.x * 19.f + s64(w.z * 4.f) * 1.8f) * 0.006f;
  const float damp = 1.f - smoothstep(-0.02f, 0.20f, w.y);
  const F3 sand = scale(mix(f3(0.88f, 0.69f, 0.42f), f3(0.56f, 0.41f, 0.23f), damp * 0.55f), 0.98f + 0.02f + ribbons);
  const F3 nb = unit(f3(w.x > 1.5f ? -1.f / V.slope : 0.f, 1.f, 0.f));
  const float lit = std::fmax(dot(nb, sun_n), 0.f) * 1.1f;
  return mul(sand, add(f3(0.35f, 0.35f, 0.35f), scale(f3(1.f, 0.94f, 0.83f), lit)));
}

// trace_water (water.gdshader:23-91); returns (first, occupied, finish, queries)
void trace_water(const Volume& V, const Look& L, F3 origin, F3 dir, float opaque_limit, F3& first_normal,
                 float& first_exit, bool& complete, float out[4]) {
  const F3 sd = safe_ray(dir), h = V.h;
  const F3 a = div(sub(V.bmin, origin), sd), b = div(sub(V.bmax, origin), sd);
  const F3 lo = f3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z));
  const F3 hi = f3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z));
  const float start = std::fmax(0.f, std::fmax(lo.x, std::fmax(lo.y, lo.z)));
  const float finish = std::fmin(opaque_limit, std::fmin(hi.x, std::fmin(hi.y, hi.z)));
  float first = -1.f, occupied = 0.f, last_end = -1.f;
  first_exit = -1.f;
  complete = true;
  first_normal = f3(0, 1, 0);
  F3 entry = f3(0, 1, 0);
  if (lo.x >= lo.y && lo.x >= lo.z) entry = f3(-sign(dir.x), 0, 0);
  else if (lo.y >= lo.z) entry = f3(0, -sign(dir.y), 0);
  else entry = f3(0, 0, -sign(dir.z));
  if (finish <= start) {
    out[0] = -1.f;
    out[1] = out[2] = out[3] = 0.f;
    return;
  }
  const bool contact = L.contact && V.slope > 0.f;
  float t = start;
  int queries = 0;
  bool open_first = false;
  for (int step = 0; step < 640; step++) {
    if (t >= finish - 1e-7f) break;
    const F3 probe = add(origin, scale(dir, t + 1e-6f));
    const F3 rel = div(sub(probe, V.bmin), h);
    const int cx = V.clampc(ifloor(rel.x), 0), cy = V.clampc(ifloor(rel.y), 1), cz = V.clampc(ifloor(rel.z), 2);
    const F3 corner = add(V.bmin, mul(f3((float)cx, (float)cy, (float)cz), h));
    const F3 next = add(corner, f3(dir.x >= 0.f ? h.x : 0.f, dir.y >= 0.f ? h.y : 0.f, dir.z >= 0.f ? h.z : 0.f));
    const F3 exits = div(sub(next, origin), sd);
    const float end = std::fmin(finish, std::fmin(exits.x, std::fmin(exits.y, exits.z)));
    if (end <= t + 1e-8f) {
      t += 1e-6f;
      continue;
    }
    float kind = V.kind(cx, cy, cz);
    queries++;
    float plane[4] = {0, 0, 0, 0};
    if (kind > 1.5f) V.plane(cx, cy, cz, plane);
    float bed_x = 0.f, bed_center = 0.f;
    if (contact) {
      bed_x = V.bmin.x + ((float)cx + 0.5f) * h.x;
      bed_center = -0.45f + std::fmax(0.f, bed_x - 1.5f) / V.slope;
      int bottom = ifloor((bed_center - V.bmin.y) / h.y - 0.5f) + 1;
      if (V.bmin.y + ((float)bottom + 0.5f) * h.y <= bed_center) bottom++;
      if (V.bmin.y + ((float)bottom - 0.5f) * h.y > bed_center) bottom--;
      if (cy == bottom - 1 && bottom >= 0 && bottom < V.n[1]) {
        kind = V.kind(cx, bottom, cz);
        if (kind > 1.5f) {
          V.plane(cx, bottom, cz, plane);
          plane[1] = 0.f;
        }
      }
    }
    float enter = t, leave = end;
    F3 normal = entry;
    if (kind > 1.5f) {
      queries++;
      const F3 pn = f3(plane[0], plane[1], plane[2]);
      const float rate = dot(pn, div(dir, h)), value = dot(pn, div(sub(origin, corner), h)) - plane[3];
      if (std::fabs(rate) < 1e-10f) {
        if (value > 0.f) leave = enter;
      } else if (rate < 0.f) {
        const float crossing = -value / rate;
        if (crossing > enter) {
          enter = crossing;
          normal = unit(div(pn, h));
        }
      } else {
        leave = std::fmin(leave, -value / rate);
      }
    } else if (kind < 0.5f) {
      leave = enter;
    }
    if (contact) {
      const float gradient = bed_x > 1.5f ? 1.f / V.slope : 0.f;
      const float value = origin.y - bed_center - gradient * (origin.x - bed_x);
      const float rate = dir.y - gradient * dir.x;
      if (std::fabs(rate) < 1e-10f) {
        if (value < 0.f) leave = enter;
      } else if (rate > 0.f) {
        const float crossing = -value / rate;
        if (crossing > enter) {
          enter = crossing;
          normal = unit(f3(gradient, -1.f, 0.f));
        }
      } else {
        leave = std::fmin(leave, -value / rate);
      }
    }
    enter = std::fmax(t, enter);
    leave = std::fmin(end, leave);
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
    if (exits.x <= exits.y && exits.x <= exits.z) entry = f3(-sign(dir.x), 0, 0);
    else if (exits.y <= exits.z) entry = f3(0, -sign(dir.y), 0);
    else entry = f3(0, 0, -sign(dir.z));
    t = end;
    if (step == 639 && t < finish - 1e-6f) complete = false;
  }
  out[0] = first;
  out[1] = occupied;
  out[2] = finish;
  out[3] = (float)queries;
}

// normal_weight (water.gdshader:92-95): pow(., 2.0) as a product
float normal_weight(float x) {
  x = std::fabs(x);
  if (x < 0.5f) return 0.75f - x * x;
  const float r = std::fmax(0.f, 1.5f - x);
  return 0.5f * (r * r);
}

// optical_normal (water.gdshader:96-124)
F3 optical_normal(const Volume& V, F3 hit, F3 geometric) {
  const F3 h = V.h, rel = div(sub(hit, V.bmin), h), local = sub(rel, f3(0.5f, 0.5f, 0.5f));
  const int lx = ifloor(local.x), ly = ifloor(local.y), lz = ifloor(local.z);
  const float hmin = std::fmin(h.x, h.y);
  F3 anchor = geometric;
  float closest = 1e10f;
  for (int z = 0; z < 2; z++)
    for (int y = 0; y < 2; y++)
      for (int x = 0; x < 2; x++) {
        const int qx = lx + x, qy = ly + y, qz = lz + z;
        if (!V.inside(qx, qy, qz) || V.kind(qx, qy, qz) < 1.5f) continue;
        float p[4];
        V.plane(qx, qy, qz, p);
        const F3 raw = div(f3(p[0], p[1], p[2]), h);
        const float ln = len(raw);
        if (ln < 1e-8f) continue;
        const F3 nrm = f3(raw.x / ln, raw.y / ln, raw.z / ln), q = f3((float)qx, (float)qy, (float)qz);
        const float distance = std::fabs(dot(f3(p[0], p[1], p[2]), sub(rel, q)) - p[3]) / ln;
        const float score = distance / hmin + 0.15f * len(sub(local, q));
        if (distance < 0.8f * hmin && score < closest) {
          closest = score;
          anchor = nrm;
        }
      }
  F3 sum = f3(0, 0, 0);
  float weights = 0.f;
  const int cx = ifloor(rel.x), cy = ifloor(rel.y), cz = ifloor(rel.z);
  for (int z = -1; z <= 1; z++)
    for (int y = -1; y <= 1; y++)
      for (int x = -2; x <= 2; x++) {
        const int qx = cx + x, qy = cy + y, qz = cz + z;
        if (!V.inside(qx, qy, qz) || V.kind(qx, qy, qz) < 1.5f) continue;
        float p[4];
        V.plane(qx, qy, qz, p);
        const F3 raw = div(f3(p[0], p[1], p[2]), h);
        const float ln = len(raw);
        if (ln < 1e-8f) continue;
        const F3 nrm = f3(raw.x / ln, raw.y / ln, raw.z / ln), q = f3((float)qx, (float)qy, (float)qz);
        const float distance = std::fabs(dot(f3(p[0], p[1], p[2]), sub(rel, q)) - p[3]) / ln;
        const F3 delta = sub(local, q);
        const float w = normal_weight(delta.x * 0.6f) * normal_weight(delta.y) * normal_weight(delta.z) *
                        smoothstep(0.15f, 0.8f, dot(nrm, anchor)) * (1.f - smoothstep(0.7f, 1.5f, distance / hmin));
        sum = add(sum, scale(nrm, w));
        weights += w;
      }
  return weights > 0.001f ? unit(sum) : anchor;
}

// fragment() of water.gdshader:125-176 (refraction offset of the screen lookup left out: the
// scene colour is taken along the view ray)
void water_pixel(const Volume& V, const Look& L, F3 origin, F3 dir, float rgba[4], float tr[4]) {
  const float t_bed = bed_distance(V, origin, dir);
  const F3 behind = scene(V, origin, dir, t_bed, L.sun);
  F3 gn;
  float first_exit;
  bool complete;
  trace_water(V, L, origin, dir, t_bed >= 0.f ? t_bed : 10000.f, gn, first_exit, complete, tr);
  tr[2] = first_exit;
  const float first = tr[0], occupied = tr[1];
  if (first < 0.f || !complete) {
    rgba[0] = behind.x;
    rgba[1] = behind.y;
    rgba[2] = behind.z;
    rgba[3] = 1.f;
    return;
  }
  const F3 hit = add(origin, scale(dir, first));
  F3 n = optical_normal(V, hit, gn);
  if (dot(n, neg(dir)) < 0.f) n = neg(n);
  const F3 smooth_normal = n;
  const float time = L.clock_ready ? L.time : 0.f;
  F3 ripple = f3(c64(hit.x * 75.f + hit.z * 31.f - time * 2.5f), 0.f, s64(hit.z * 103.f - hit.x * 22.f + time * 3.1f));
  const F3 r2 = f3(s64(hit.z * 160.f + time * 4.f), c64(hit.x * 95.f + time), c64(hit.x * 140.f - time * 3.f));
  ripple = add(ripple, f3(0.35f * r2.x, 0.35f * r2.y, 0.35f * r2.z));
  const F3 tang = sub(ripple, scale(n, dot(ripple, n)));
  n = unit(add(n, f3(L.ripple * tang.x, L.ripple * tang.y, L.ripple * tang.z)));
  const float nv = clamp(dot(smooth_normal, neg(dir)), 0.f, 1.f);
  const float fresnel = 0.02037f + (0.97963f - L.roughness * 0.35f) * p64(1.f - nv, 5.f);
  // reflect(I, N) = I - 2 dot(N, I) N
  const F3 reflection = daylight_reflection(sub(dir, scale(n, 2.f * dot(n, dir))), L.sun);
  const float att = std::fmax(L.attenuation, 0.01f);
  const F3 absorption = f3(1.4f / att, 1.f / att, 0.85f / att);
  const F3 transmission = f3(e64(-absorption.x * occupied), e64(-absorption.y * occupied), e64(-absorption.z * occupied));
  const float deeper = 1.f - e64(-occupied / 0.45f);
  F3 scatter = mul(L.tint, mix(f3(0.65f, 1.18f, 1.f), f3(0.4f, 0.65f, 0.92f), deeper));
  scatter = scale(scatter, 0.55f + 0.45f * std::fmax(dot(smooth_normal, L.sun), 0.f));
  const F3 body = add(mul(behind, transmission), mul(scatter, sub(f3(1, 1, 1), transmission)));
  const F3 half_vector = unit(sub(L.sun, dir));
  const float nh = std::fmax(dot(n, half_vector), 0.f), a = L.roughness * L.roughness, a2 = a * a;
  const float den = std::fmax(nh * nh * (a2 - 1.f) + 1.f, 0.001f);
  const float distribution = a2 / (3.14159265f * (den * den));
  const float nl = std::fmax(dot(n, L.sun), 0.f);
  const F3 sun = scale(scale(f3(1.f, 0.90f, 0.74f), std::fmin(0.6f, distribution * 0.007f)), nl);
  const F3 color = add(mix(body, reflection, fresnel), sun);
  rgba[0] = color.x;
  rgba[1] = color.y;
  rgba[2] = color.z;
  rgba[3] = 1.f;
}

// fragment() of clay.gdshader:8-66
void clay_pixel(const Volume& V, F3 origin, F3 dir, float rgba[4], float tr[4]) {
  const F3 sd = safe_ray(dir), h = V.h;
  const F3 t0 = div(sub(V.bmin, origin), sd), t1 = div(sub(V.bmax, origin), sd);
  const F3 lo = f3(std::fmin(t0.x, t1.x), std::fmin(t0.y, t1.y), std::fmin(t0.z, t1.z));
  const F3 hi = f3(std::fmax(t0.x, t1.x), std::fmax(t0.y, t1.y), std::fmax(t0.z, t1.z));
  const float start = std::fmax(0.f, std::fmax(lo.x, std::fmax(lo.y, lo.z)));
  const float finish = std::fmin(hi.x, std::fmin(hi.y, hi.z));
  rgba[0] = rgba[1] = rgba[2] = rgba[3] = 0.f;
  tr[0] = -1.f;
  tr[1] = 0.f;
  tr[2] = finish;
  tr[3] = 0.f;
  if (finish <= start) return;
  float t = start + 1e-6f, first = -1.f, occupied = 0.f;
  F3 first_normal = f3(0, 1, 0), entry_normal = f3(0, 1, 0);
  int queries = 0;
  bool overflow = true;
  for (int step = 0; step < 512; step++) {
    if (t >= finish - 1e-6f) {
      overflow = false;
      break;
    }
    const F3 x = add(origin, scale(dir, t));
    const F3 rel = div(sub(x, V.bmin), h);
    const int cx = V.clampc(ifloor(rel.x), 0), cy = V.clampc(ifloor(rel.y), 1), cz = V.clampc(ifloor(rel.z), 2);
    const F3 corner = add(V.bmin, mul(f3((float)cx, (float)cy, (float)cz), h));
    const F3 next = add(corner, f3(dir.x >= 0.f ? h.x : 0.f, dir.y >= 0.f ? h.y : 0.f, dir.z >= 0.f ? h.z : 0.f));
    const F3 exits = div(sub(next, origin), sd);
    float end = std::fmin(finish, std::fmin(exits.x, std::fmin(exits.y, exits.z)));
    end = std::fmax(t + 1e-7f, end);
    const float kind = V.kind(cx, cy, cz);
    queries++;
    float enter = t, leave = end;
    F3 normal = entry_normal;
    if (kind > 1.5f) {
      float p[4];
      V.plane(cx, cy, cz, p);
      queries++;
      const F3 pn = f3(p[0], p[1], p[2]);
      const float rate = dot(pn, div(dir, h)), value = dot(pn, div(sub(origin, corner), h)) - p[3];
      if (std::fabs(rate) < 1e-10f) {
        if (value > 0.f) leave = enter;
      } else {
        const float crossing = -value / rate;
        if (rate < 0.f) {
          if (crossing > enter) {
            enter = crossing;
            normal = unit(div(pn, h));
          }
        } else {
          leave = std::fmin(leave, crossing);
        }
      }
    } else if (kind < 0.5f) {
      leave = enter;
    }
    enter = std::fmax(t, enter);
    leave = std::fmin(end, leave);
    if (leave > enter + 1e-7f) {
      occupied += leave - enter;
      if (first < 0.f) {
        first = enter;
        first_normal = normal;
        overflow = false;
        break;
      }
    }
    if (exits.x <= exits.y && exits.x <= exits.z) entry_normal = f3(-sign(dir.x), 0, 0);
    else if (exits.y <= exits.z) entry_normal = f3(0, -sign(dir.y), 0);
    else entry_normal = f3(0, 0, -sign(dir.z));
    t = end + 1e-6f;
  }
  tr[0] = first;
  tr[1] = occupied;
  tr[3] = (float)queries;
  if (first < 0.f) return;
  rgba[3] = 1.f;
  if (overflow) {
    rgba[0] = 1.f;
    rgba[1] = 0.f;
    rgba[2] = 1.f;
    return;
  }
  const float diffuse = 0.28f + 0.72f * std::fmax(0.f, dot(first_normal, unit(f3(-0.4f, 0.8f, 0.5f))));
  rgba[0] = rgba[1] = rgba[2] = 0.54f * diffuse;
}

}  // namespace

extern "C" {

// Renders planes[4N]/kinds[N] (the op-19 export) with the camera and look of `p` over the box
// origin .. origin + n spacing of `cfg`; `clock_time` is the surface clock (accepted time).
void wo_render(const float* planes, const float* kinds, const waves_config* cfg, const waves_render_params* p,
               float clock_time, float* rgba, float* trace) {
  Volume V;
  V.planes = planes;
  V.kinds = kinds;
  for (int k = 0; k < 3; k++) V.n[k] = cfg->n[k];
  V.bmin = f3(cfg->origin[0], cfg->origin[1], cfg->origin[2]);
  V.bmax = f3(cfg->origin[0] + (float)cfg->n[0] * cfg->spacing[0], cfg->origin[1] + (float)cfg->n[1] * cfg->spacing[1],
              cfg->origin[2] + (float)cfg->n[2] * cfg->spacing[2]);
  V.h = div(sub(V.bmax, V.bmin), f3((float)V.n[0], (float)V.n[1], (float)V.n[2]));
  V.slope = cfg->slope;
  Look L;
  L.tint = f3(p->water_tint[0], p->water_tint[1], p->water_tint[2]);
  L.sun = unit(f3(p->sun_direction[0], p->sun_direction[1], p->sun_direction[2]));
  L.attenuation = p->attenuation_distance;
  L.ripple = p->ripple_strength;
  L.roughness = p->surface_roughness;
  L.contact = p->contact_correction != 0;
  L.clock_ready = p->clock_ready != 0;
  L.time = clock_time;
  // camera: forward, right = forward x up, up' = right x forward
  const F3 eye = f3(p->eye[0], p->eye[1], p->eye[2]), upv = f3(p->up[0], p->up[1], p->up[2]);
  const F3 f = unit(sub(f3(p->target[0], p->target[1], p->target[2]), eye));
  const F3 r = unit(f3(f.y * upv.z - f.z * upv.y, f.z * upv.x - f.x * upv.z, f.x * upv.y - f.y * upv.x));
  const F3 u = f3(r.y * f.z - r.z * f.y, r.z * f.x - r.x * f.z, r.x * f.y - r.y * f.x);
  const float half_h = p->orthographic ? p->size * 0.5f : (float)std::tan((double)p->fov_y_deg * M_PI / 360.0);
  const float half_w = half_h * ((float)p->width / (float)p->height);
#pragma omp parallel for schedule(dynamic, 4)
  for (int py = 0; py < p->height; py++)
    for (int px = 0; px < p->width; px++) {
      const float sx = ((float)px + 0.5f) / (float)p->width * 2.f - 1.f;
      const float sy = 1.f - ((float)py + 0.5f) / (float)p->height * 2.f;
      F3 o, d;
      if (p->orthographic) {
        o = add(add(eye, scale(r, sx * half_w)), scale(u, sy * half_h));
        d = f;
      } else {
        o = eye;
        d = unit(add(add(f, scale(r, sx * half_w)), scale(u, sy * half_h)));
      }
      const size_t i = (size_t)py * p->width + px;
      float tr[4];
      if (p->mode == 0) clay_pixel(V, o, d, rgba + 4 * i, tr);
      else water_pixel(V, L, o, d, rgba + 4 * i, tr);
      if (trace) std::memcpy(trace + 4 * i, tr, sizeof(tr));
    }
}

}  // extern "C"
