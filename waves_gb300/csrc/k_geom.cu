// Geometry, projection set-up / gradient apply, air-velocity extension, acceptance and coastal
// forcing kernels (neuron-forest/waves water/shaders/compute/pressure_pass.glslinc ops 2, 11-19,
// pressure_geometry.glslinc, coupled_motion.glslinc ops 30-36, 47/48, 62-66, coastal_pass.glslinc).
#include "common.cuh"
#include "kernels.h"

namespace wg {

namespace {
constexpr int NT = 256;

struct Geo {
  const Dev& D;
  Grid g;
  Coast cs;
  int acc, cand, gbank;
  const float* A;
  float* Cb;
  const float* Gb;  // geometry bank
  float dt;
  double c1;
  // op selects geometry_bank (pressure_core.glslinc:66-72)
  DI Geo(const Dev& d, int op) : D(d), g(d), cs(d) {
    acc = acc_bank(d);
    cand = 1 - acc;
    A = bank_ptr(d, acc);
    Cb = bank_ptr(d, cand);
    gbank = (op == 19 || d.c[4] < .5) ? acc : cand;
    Gb = bank_ptr(d, gbank);
    dt = (float)d.c[20];
    c1 = d.c[1];
  }
  // geometry_fraction (pressure_geometry.glslinc:2-10)
  DI float gfrac(I3 q) const {
    q = g.wrap_cell(q);
    if (D.coastal && q.x < 0 && !g.solid(q)) return cs.fraction(g, q, (float)(c1 + (gbank == cand ? (double)D.c[20] : 0.0)));
    if (g.solid(q)) {
      q.x = min(max(q.x, 0), D.nx - 1);
      q.y = min(max(q.y, 0), D.ny - 1);
      q.z = min(max(q.z, 0), D.nz - 1);
    }
    if (g.outside(q)) return 0.f;
    return Gb[g.index3(q)];
  }
  DI float4 reconstruct(I3 q) const {
    float f = gfrac(q);
    if (f <= 0.f || f >= 1.f) return make_float4(0.f, 1.f, 0.f, f);
    auto fr = [&](I3 p) { return gfrac(p); };
    F3 grad = interface_gradient(g, q, fr);
    if (D.flags & 1) grad = height_normal(g, q, grad, fr);
    return plane_from_gradient(D, grad, f);
  }
  DI F3 hvec() const { return mf(D.hx, D.hy, D.hz); }
  DI float segment_distance(F3 point, F3 a, F3 b) const {
    F3 ab = sub3(b, a);
    float t = clampf_(dot3(sub3(point, a), ab) / mxf(dot3(ab, ab), 1e-30f), 0.f, 1.f);
    return len3(sub3(point, add3(a, scl3(ab, t))));
  }
  // polygon_distance (pressure_geometry.glslinc:68-83)
  DI float polygon_distance(F3 point, float4 eq) const {
    F3 hh = hvec();
    F3 n = div3(mf(eq.x, eq.y, eq.z), hh);
    float norm2 = dot3(n, n);
    float s = dot3(n, point) - eq.w;
    float signed_d = s / sqrtf(norm2);
    F3 pr = mf(point.x - n.x * s / norm2, point.y - n.y * s / norm2, point.z - n.z * s / norm2);
    if (pr.x >= 0.f && pr.y >= 0.f && pr.z >= 0.f && pr.x <= hh.x && pr.y <= hh.y && pr.z <= hh.z) return fabsf(signed_d);
    F3 vertices[12];
    int count = 0;
    F3 e3 = mf(eq.x, eq.y, eq.z);
    for (int axis = 0; axis < 3; axis++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) {
          F3 a = mf(0.f, 0.f, 0.f);
          a[(axis + 1) % 3] = (float)j;
          a[(axis + 2) % 3] = (float)k;
          float den = e3[axis];
          if (fabsf(den) < 1e-15f) continue;
          float t = (eq.w - dot3(e3, a)) / den;
          if (t >= 0.f && t <= 1.f) {
            a[axis] = t;
            vertices[count++] = mul3(a, hh);
          }
        }
    float best = 1e10f;
    for (int j = 0; j < count; j++) {
      best = mnf(best, len3(sub3(point, vertices[j])));
      for (int k = 0; k < j; k++) best = mnf(best, segment_distance(point, vertices[j], vertices[k]));
    }
    return best;
  }
  DI static int clip_polygon(F3* poly, int count, float4 eq) {
    F3 result[12];
    int size = 0;
    F3 e3 = mf(eq.x, eq.y, eq.z);
    for (int j = 0; j < count; j++) {
      F3 a = poly[j], b = poly[(j + 1) % count];
      float da = dot3(e3, a) - eq.w, db = dot3(e3, b) - eq.w;
      if (da <= 0.f) result[size++] = a;
      if ((da < 0.f && db > 0.f) || (da > 0.f && db < 0.f)) {
        float t = da / (da - db);
        result[size++] = mf(a.x * (1.f - t) + b.x * t, a.y * (1.f - t) + b.y * t, a.z * (1.f - t) + b.z * t);
      }
    }
    for (int j = 0; j < size; j++) poly[j] = result[j];
    return size;
  }
  // transition_distance (pressure_geometry.glslinc:96-119)
  DI float transition_distance(F3 point, I3 left, int axis) const {
    I3 right = ax(left, axis, 1);
    I3 l = g.wrap_cell(left), r = g.wrap_cell(right);
    if (g.outside(l) || g.outside(r) || g.solid(l) || g.solid(r)) return 1e10f;
    float fl = gfrac(l), fr = gfrac(r);
    if ((fl <= 0.f && fr <= 0.f) || (fl >= 1.f && fr >= 1.f)) return 1e10f;
    float4 a = D.plane[g.index3(l)], b = D.plane[g.index3(r)];
    if (fl <= 0.f) a = make_float4(0.f, 0.f, 0.f, -1.f);
    if (fl >= 1.f) a = make_float4(0.f, 0.f, 0.f, 1.f);
    if (fr <= 0.f) b = make_float4(0.f, 0.f, 0.f, -1.f);
    if (fr >= 1.f) b = make_float4(0.f, 0.f, 0.f, 1.f);
    b.w += axis == 0 ? b.x : (axis == 1 ? b.y : b.z);
    float best = 1e10f;
    F3 hh = hvec();
    for (int side = 0; side < 2; side++) {
      F3 poly[12];
      int j = (axis + 1) % 3, k = (axis + 2) % 3;
      for (int v = 0; v < 4; v++) {
        poly[v] = mf(0.f, 0.f, 0.f);
        poly[v][axis] = 1.f;
        poly[v][j] = (v == 1 || v == 2) ? 1.f : 0.f;
        poly[v][k] = v >= 2 ? 1.f : 0.f;
      }
      float4 first = side == 0 ? a : b;
      float4 second = side == 0 ? make_float4(-b.x, -b.y, -b.z, -b.w) : make_float4(-a.x, -a.y, -a.z, -a.w);
      int count = clip_polygon(poly, 4, first);
      count = clip_polygon(poly, count, second);
      if (count == 0) continue;
      F3 projected = point;
      projected[axis] = hh[axis];
      F3 local = div3(projected, hh);
      if (local.x >= 0.f && local.y >= 0.f && local.z >= 0.f && local.x <= 1.f && local.y <= 1.f && local.z <= 1.f &&
          dot3(mf(first.x, first.y, first.z), local) <= first.w && dot3(mf(second.x, second.y, second.z), local) <= second.w)
        best = mnf(best, fabsf(point[axis] - hh[axis]));
      for (int v = 0; v < count; v++) best = mnf(best, segment_distance(point, mul3(poly[v], hh), mul3(poly[(v + 1) % count], hh)));
    }
    return best;
  }
  // geometry_distance (pressure_geometry.glslinc:120-145) up to the neighbourhood search: the
  // distance, or *search = true where the cell needs the 27-neighbour search (seed_terms and the
  // ordered replay in k_geom_seed finish it)
  DI float distance_or_search(I3 q, bool* search) const {
    float f = gfrac(q);
    F3 hh = hvec();
    *search = false;
    if (f > 0.f && f < 1.f) {
      float4 eq = D.plane[g.index3(q)];
      F3 e3 = mf(eq.x, eq.y, eq.z);
      return (half_dot(e3) - eq.w) / len3(div3(e3, hh));
    }
    bool needs_seed = false;
    for (int axis = 0; axis < 3; axis++)
      for (int sign = -1; sign <= 1; sign += 2) {
        I3 nb = g.wrap_cell(ax(q, axis, sign));
        if (g.solid(nb) || g.outside(nb)) continue;
        float other = gfrac(nb);
        bool inside = other >= 1.f;
        if (other > 0.f && other < 1.f) {
          float4 eq = D.plane[g.index3(nb)];
          inside = half_dot(mf(eq.x, eq.y, eq.z)) < eq.w;
        }
        if (inside != (f >= 1.f)) needs_seed = true;
      }
    if (!needs_seed) return (f >= 1.f ? -1.f : 1.f) * len3(hh) * 4.f;
    *search = true;
    return 0.f;
  }
  // One neighbour (x, y, z) of the search of geometry_distance: false where it is skipped (outside
  // the domain or solid); else its lower bound lb (the distance to its box) and the values the
  // search takes the minimum of, in its order: the polygon distance (where the neighbour holds an
  // interface, has_poly) and the three transition distances.
  DI bool seed_terms(I3 q, int x, int y, int z, float& lb, bool& has_poly, float v[4]) const {
    const F3 hh = hvec();
    const I3 neighbor = addI(q, mk(x, y, z)), wrapped = g.wrap_cell(neighbor);
    if (g.outside(wrapped) || g.solid(wrapped)) return false;
    const float fraction = gfrac(wrapped);
    const I3 dq = subI(q, neighbor);
    const F3 point = mf(((float)dq.x + .5f) * hh.x, ((float)dq.y + .5f) * hh.y, ((float)dq.z + .5f) * hh.z);
    const F3 cl = mf(clampf_(point.x, 0.f, hh.x), clampf_(point.y, 0.f, hh.y), clampf_(point.z, 0.f, hh.z));
    lb = len3(sub3(point, cl));
    has_poly = fraction > 0.f && fraction < 1.f;
    v[0] = has_poly ? polygon_distance(point, D.plane[g.index3(wrapped)]) : 0.f;
    for (int axis = 0; axis < 3; axis++) v[1 + axis] = transition_distance(point, neighbor, axis);
    return true;
  }
  // geometry_distance (pressure_geometry.glslinc:120-145), the sequential form
  DI float distance(I3 q) const {
    float f = gfrac(q);
    F3 hh = hvec();
    if (f > 0.f && f < 1.f) {
      float4 eq = D.plane[g.index3(q)];
      F3 e3 = mf(eq.x, eq.y, eq.z);
      return (half_dot(e3) - eq.w) / len3(div3(e3, hh));
    }
    bool needs_seed = false;
    for (int axis = 0; axis < 3; axis++)
      for (int sign = -1; sign <= 1; sign += 2) {
        I3 nb = g.wrap_cell(ax(q, axis, sign));
        if (g.solid(nb) || g.outside(nb)) continue;
        float other = gfrac(nb);
        bool inside = other >= 1.f;
        if (other > 0.f && other < 1.f) {
          float4 eq = D.plane[g.index3(nb)];
          inside = half_dot(mf(eq.x, eq.y, eq.z)) < eq.w;
        }
        if (inside != (f >= 1.f)) needs_seed = true;
      }
    if (!needs_seed) return (f >= 1.f ? -1.f : 1.f) * len3(hh) * 4.f;
    float best = len3(hh) * 4.f;
    for (int x = -1; x <= 1; x++)
      for (int y = -1; y <= 1; y++)
        for (int z = -1; z <= 1; z++) {
          I3 neighbor = addI(q, mk(x, y, z)), wrapped = g.wrap_cell(neighbor);
          if (g.outside(wrapped) || g.solid(wrapped)) continue;
          float fraction = gfrac(wrapped);
          I3 dq = subI(q, neighbor);
          F3 point = mf(((float)dq.x + .5f) * hh.x, ((float)dq.y + .5f) * hh.y, ((float)dq.z + .5f) * hh.z);
          F3 cl = mf(clampf_(point.x, 0.f, hh.x), clampf_(point.y, 0.f, hh.y), clampf_(point.z, 0.f, hh.z));
          if (len3(sub3(point, cl)) >= best) continue;
          if (fraction > 0.f && fraction < 1.f) best = mnf(best, polygon_distance(point, D.plane[g.index3(wrapped)]));
          for (int axis = 0; axis < 3; axis++) best = mnf(best, transition_distance(point, neighbor, axis));
        }
    return (f >= 1.f ? -1.f : 1.f) * best;
  }
  // press (pressure_core.glslinc:99), candidate bank
  DI float press(I3 q) const {
    q = g.wrap_cell(q);
    return g.wet(q) ? Cb[D.N + D.NU + D.NV + D.NW + g.index3(q)] : 0.f;
  }
  // distance_face (pressure_core.glslinc:100-109)
  DI float distance_face(I3 l, I3 r, int axis) const {
    float hh = g.h(axis);
    if (axis == 1 && (l.y >= D.ny || r.y >= D.ny)) return .5f * hh;
    bool wl = g.wet(l), wr = g.wet(r);
    if (wl && wr) return hh;
    float pl = fabsf(g.phi(l)), pr = fabsf(g.phi(r));
    return hh * mxf((wl ? pl : pr) / mxf(pl + pr, 1e-30f), 1e-6f);
  }
  DI float coefficient(I3 q, I3 nb, int axis) const {
    if (g.solid(nb)) return 0.f;
    if (D.coastal && axis == 0 && nb.x < 0) return 0.f;
    return 1.0f / (g.h(axis) * distance_face(q, nb, axis));
  }
  DI float divergence(I3 q) const {
    float d = 0.f;
    for (int axis = 0; axis < 3; axis++) {
      I3 right = ax(q, axis, 1);
      d += (Cb[g.face_index(right, axis)] - Cb[g.face_index(q, axis)]) / g.h(axis);
    }
    return d;
  }
};

// Source faces of the extension are stored as packed lattice coordinates z<<22 | y<<11 | x; within
// one component lattice this orders exactly like the face index (the tie-break of
// coupled_motion.glslinc:441).
DI int pack_face(I3 q) { return (q.z << 22) | (q.y << 11) | q.x; }
DI I3 unpack_coords(int p) { return mk(p & 2047, (p >> 11) & 2047, p >> 22); }

DI bool geometry_on(const Dev& D) { return !(D.c[4] > .5 && D.c[5] < .5); }
DI bool setup_on(const Dev& D) { return D.c[5] > .5 && D.c[7] < .5; }
DI bool post_on(const Dev& D) { return D.c[4] > .5 && D.c[6] > .5 && D.c[7] < .5; }

// ---------------------------------------------------------------- op 17 (+ coastal op 87/88)
__global__ void __launch_bounds__(NT) k_geom_plane(const __grid_constant__ Dev D, int op, int with_bounds) {
  grid_dep_wait(D.pdl_early);
  bool on = op == 19 ? !(D.c[4] > .5) : geometry_on(D);
  bool bounds = with_bounds && setup_on(D);
  if (!on && !bounds) return;
  Geo G(D, op);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  float v[2] = {-INFINITY, -INFINITY};
  if (op == 17 && on && i == 0) D.geo_qcount[0] = 0u;  // the search queue of k_geom_phi
  if (i < D.N) {
    if (on) D.plane[i] = G.reconstruct(G.g.coord(i));
    if (bounds) {
      float f = G.Cb[i];
      float a = f, b = f;
      if (isnan(f) || isinf(f)) { a = -1e30f; b = 1e30f; }
      v[0] = -a;
      v[1] = b;
    }
  }
  if (!bounds) return;
  float out[2];
  if (last_block_reduce_mf<NT, 0, 2>(D, kSiteBounds, nullptr, nullptr, v, nullptr, out) && threadIdx.x == 0) {
    float minimum = mnf(1.f, -out[0]), maximum = mxf(0.f, out[1]);
    D.c[88] = minimum;
    D.c[89] = maximum;
    if (minimum < 0.f || maximum > 1.f) { D.c[7] = 23; D.c[3] += 1; }
  }
}

// ---------------------------------------------------------------- op 18
// Every cell but those that need the neighbourhood search, which are queued for k_geom_seed (the
// queue's count is reset by k_geom_plane, op 17, which runs first).  A warp of this pass would
// otherwise wait for its few searching lanes.
__global__ void __launch_bounds__(NT, 6) k_geom_phi(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!geometry_on(D)) return;
  Geo G(D, 18);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  bool search = false;
  if (i < D.N) {
    I3 q = G.g.coord(i);
    float ph = G.distance_or_search(q, &search);
    if (!search) {
      D.phi[i] = ph;
      D.kind[i] = G.g.solid(q) ? -1 : (ph < 0.f ? 1 : 0);
    }
  }
  const unsigned ballot = __ballot_sync(0xffffffffu, search);
  const int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (lane == 0 && ballot) base = atomicAdd(D.geo_qcount, (unsigned)__popc(ballot));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (search) D.geo_queue[base + __popc(ballot & ((1u << lane) - 1u))] = (int)i;
}
// The neighbourhood search of the queued cells, one warp per cell: lane n < 27 evaluates
// neighbour n (x, y, z from -1 to 1, z fastest: the search's own order); lane 0 then replays the
// search in that order with the same pruning test and the same minimum operations, so the
// distance is the sequential search's bit for bit.
constexpr int kSeedWarps = NT / 32;
__global__ void __launch_bounds__(NT) k_geom_seed(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!geometry_on(D)) return;
  __shared__ float sv[kSeedWarps][27][5];
  __shared__ unsigned char sflag[kSeedWarps][27];  // bit 0: evaluated, bit 1: has a polygon
  Geo G(D, 18);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned total = *D.geo_qcount;
  for (unsigned k = blockIdx.x * kSeedWarps + w; k < total; k += gridDim.x * kSeedWarps) {  // uniform over the warp
    const int i = D.geo_queue[k];
    const I3 q = G.g.coord(i);
    if (lane < 27) {
      float lb = 0.f, v[4] = {0.f, 0.f, 0.f, 0.f};
      bool hp = false;
      const bool ok = G.seed_terms(q, lane / 9 - 1, (lane / 3) % 3 - 1, lane % 3 - 1, lb, hp, v);
      sv[w][lane][0] = lb;
      for (int j = 0; j < 4; j++) sv[w][lane][1 + j] = v[j];
      sflag[w][lane] = (ok ? 1 : 0) | (hp ? 2 : 0);
    }
    __syncwarp();
    if (lane == 0) {
      const float f = G.gfrac(q);
      const F3 hh = G.hvec();
      float best = len3(hh) * 4.f;
      for (int n = 0; n < 27; n++) {
        const unsigned fl = sflag[w][n];
        if (!(fl & 1u)) continue;
        if (sv[w][n][0] >= best) continue;
        if (fl & 2u) best = mnf(best, sv[w][n][1]);
        for (int axis = 0; axis < 3; axis++) best = mnf(best, sv[w][n][2 + axis]);
      }
      const float ph = (f >= 1.f ? -1.f : 1.f) * best;
      D.phi[i] = ph;
      D.kind[i] = G.g.solid(q) ? -1 : (ph < 0.f ? 1 : 0);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- op 16
__global__ void __launch_bounds__(NT) k_geom_coef(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!geometry_on(D)) return;
  Geo G(D, 16);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i >= D.N) return;
  I3 q = G.g.coord(i);
  bool w = D.kind[i] > 0;
  float diag = 0.f;
  int face = 0;
  for (int axis = 0; axis < 3; axis++)
    for (int sign = -1; sign <= 1; sign += 2) {
      float k = w ? G.coefficient(q, ax(q, axis, sign), axis) : 0.f;
      D.coef[(long long)face * D.N + i] = k;
      diag += k;
      face++;
    }
  D.diag[i] = w ? diag : 1.0f;
}

// ---------------------------------------------------------------- op 2 + op 47
__global__ void __launch_bounds__(NT) k_proj_setup(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!(D.c[5] > .5)) return;
  Geo G(D, 2);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i >= D.S) return;
  const long long P = D.N + D.NF;
  if (i < D.N) {
    D.pbase[i] = 0.f;
    return;
  }
  if (i >= P) {
    G.Cb[i] = G.g.wet(G.g.coord(i - P)) ? G.A[i] : 0.f;
    return;
  }
  I3 r;
  int axis;
  G.g.unpack_face(i - D.N, r, axis);
  long long canonical = G.g.face_index(r, axis);
  bool sync = D.c[4] > .5 && D.c[7] < .5;  // op 47 follows op 2
  long long src = (sync && canonical != i) ? canonical : i;
  float val = G.Cb[src];
  I3 l = ax(r, axis, -1);
  if (G.g.solid(l) || G.g.solid(r) || (!G.g.wet(l) && !G.g.wet(r))) val = 0.f;
  else if (axis == 1) val -= 9.81f * G.dt * (float)D.c[31];
  G.Cb[i] = val;
}

// ---------------------------------------------------------------- op 11 (gradient apply)
__global__ void __launch_bounds__(NT) k_grad_apply(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!post_on(D)) return;
  Geo G(D, 11);
  long long f = (long long)blockIdx.x * NT + threadIdx.x;
  if (f >= D.NF) return;
  long long i = D.N + f;
  I3 r;
  int axis;
  G.g.unpack_face(f, r, axis);
  I3 l = ax(r, axis, -1);
  float value = 0.f;
  float cur = G.Cb[i];
  if (!G.g.solid(l) && !G.g.solid(r) && (G.g.wet(l) || G.g.wet(r)))
    value = cur - G.dt / 1000.0f * (G.press(r) - G.press(l)) / G.distance_face(l, r, axis);
  if (D.coastal && axis == 0 && r.x == 0 && !G.g.solid(r)) value = cur;
  G.Cb[i] = value;
}

// ---------------------------------------------------------------- ops 30-33 (nearest sources)
__global__ void __launch_bounds__(NT) k_ext_init(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!post_on(D)) return;
  Grid g(D);
  long long f = (long long)blockIdx.x * NT + threadIdx.x;
  if (f >= D.NF) return;
  I3 q;
  int axis;
  g.unpack_face(f, q, axis);
  I3 l = ax(q, axis, -1);
  D.src0[f] = (!g.wall_face(q, axis) && (g.wet(q) || g.wet(l))) ? pack_face(q) : -1;
}
// Static neighbourhood of every face for the extension hops: bit 6 set for a wall face, bit
// 2a + (sign > 0) set when the neighbour along axis a is in bounds and not a wall face.
__global__ void __launch_bounds__(NT) k_ext_masks(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  Grid g(D);
  long long f = (long long)blockIdx.x * NT + threadIdx.x;
  if (f >= D.NF) return;
  I3 q;
  int axis;
  g.unpack_face(f, q, axis);
  unsigned bits = g.wall_face(q, axis) ? 64u : 0u;
  for (int a = 0; a < 3; a++)
    for (int sign = -1; sign <= 1; sign += 2) {
      I3 nb = g.wrap_face(ax(q, a, sign));
      if (g.face_in_bounds(nb, axis) && !g.wall_face(nb, axis)) bits |= 1u << (2 * a + (sign > 0));
    }
  D.ext_nb[f] = (unsigned char)bits;
}
__global__ void __launch_bounds__(NT) k_ext_step(const __grid_constant__ Dev D, int rb) {
  grid_dep_wait(D.pdl_early);
  if (!post_on(D)) return;
  Grid g(D);
  long long f = (long long)blockIdx.x * NT + threadIdx.x;
  if (f >= D.NF) return;
  const int* in = rb == 0 ? D.src0 : D.src1;
  int* out = rb == 0 ? D.src1 : D.src0;
  I3 q;
  int axis;
  g.unpack_face(f, q, axis);
  int source = in[f];
  float best = 1e20f;
  const unsigned bits = D.ext_nb[f];
  if (!(bits & 64u)) {
    if (source >= 0) {
      F3 dl = g.periodic_delta(q, unpack_coords(source));
      best = dot3(dl, dl);
      // a face that is its own source keeps it: no neighbour's source is nearer, and one at the
      // same distance is this face, not a smaller index
      if (best == 0.f) {
        out[f] = source;
        return;
      }
    }
    for (int a = 0; a < 3; a++)
      for (int sign = -1; sign <= 1; sign += 2) {
        if (!(bits & (1u << (2 * a + (sign > 0))))) continue;
        I3 nb = g.wrap_face(ax(q, a, sign));
        int cs = in[g.face_local(nb, axis)];
        if (cs < 0) continue;
        F3 delta = g.periodic_delta(q, unpack_coords(cs));
        float distance = dot3(delta, delta);
        if (distance < best || (distance == best && cs < source)) {
          best = distance;
          source = cs;
        }
      }
  } else
    source = -1;
  out[f] = source;
}

// extended_value (coupled_motion.glslinc:212-230)
DI bool projected_face(const Grid& g, I3 q, int axis) {
  q = g.wrap_face(q);
  if (!g.face_in_bounds(q, axis) || g.wall_face(q, axis)) return false;
  return g.wet(q) || g.wet(ax(q, axis, -1));
}
DI float extended_value(const Dev& D, const Grid& g, const float* Cb, int packed, int component, I3 target) {
  I3 q = unpack_coords(packed);
  float value = Cb[D.N + g.face_local_raw(q, component)];
  if (!D.linear_air) return value;
  F3 gradient = mf(0.f, 0.f, 0.f);
  for (int axis = 0; axis < 3; axis++) {
    I3 l = g.wrap_face(ax(q, axis, -1)), r = g.wrap_face(ax(q, axis, 1));
    bool left = projected_face(g, l, component), right = projected_face(g, r, component);
    float dl = left ? value - Cb[g.face_index(l, component)] : 0.f;
    float dr = right ? Cb[g.face_index(r, component)] - value : 0.f;
    if (left && right) gradient[axis] = dl * dr > 0.f ? sgnf(dl) * mnf(fabsf(dl), fabsf(dr)) : 0.f;
    else gradient[axis] = left ? dl : (right ? dr : 0.f);
  }
  F3 pd = g.periodic_delta(target, q);
  F3 off = mf(clampf_(pd.x / D.hx, -1.f, 1.f), clampf_(pd.y / D.hy, -1.f, 1.f), clampf_(pd.z / D.hz, -1.f, 1.f));
  return value + dot3(gradient, off);
}

// ---------------------------------------------------------------- op 34 + 47 + 48
__global__ void __launch_bounds__(NT) k_ext_write(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!post_on(D)) return;
  Grid g(D);
  int cand = 1 - acc_bank(D);
  float* Cb = bank_ptr(D, cand);
  long long f = (long long)blockIdx.x * NT + threadIdx.x;
  if (f < D.N) (cand == 0 ? D.pmask0 : D.pmask1)[f] = D.kind[f] > 0 ? 1.f : 0.f;
  if (f >= D.NF) return;
  I3 q;
  int axis;
  g.unpack_face(f, q, axis);
  (cand == 0 ? D.vband0 : D.vband1)[f] = D.src1[f] >= 0 ? 1.f : 0.f;
  long long canonical = g.face_local(q, axis);
  I3 cq = q;
  if (canonical != f) g.unpack_face(canonical, cq, axis);  // op 47: the duplicate takes the canonical value
  bool air = !(g.wet(cq) || g.wet(ax(cq, axis, -1)));
  if (canonical != f) {
    float value;
    if (air) {
      int source = D.src1[canonical];
      value = source < 0 ? 0.f : extended_value(D, g, Cb, source, axis, cq);
    } else
      value = Cb[D.N + canonical];
    Cb[D.N + f] = value;
  } else if (air) {
    int source = D.src1[f];
    Cb[D.N + f] = source < 0 ? 0.f : extended_value(D, g, Cb, source, axis, q);
  }
}

// ---------------------------------------------------------------- ops 35/36, 62/66, 65, 12/13
__global__ void __launch_bounds__(NT) k_accept(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!post_on(D)) return;
  Geo G(D, 12);
  const Grid& g = G.g;
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  // FP64 sums: 0 res^2, 1 volume; FP32 maxima: 0 courant dt, 1 dt|div|, 2 speed, 3 hydro error
  double v[2] = {0, 0};
  float fv[4] = {0.f, 0.f, 0.f, 0.f};
  if (i < D.N) {
    I3 q = g.coord(i);
    const long long P = D.N + D.NF;
    float p = G.Cb[P + i] + D.pbase[i];  // op 65
    G.Cb[P + i] = p;
    float s[3];
    float speed = 0.f;
    for (int axis = 0; axis < 3; axis++) {
      I3 r = ax(q, axis, 1);
      float a = fabsf(G.Cb[g.face_index(q, axis)]), b = fabsf(G.Cb[g.face_index(r, axis)]);
      s[axis] = mxf(a, b);
      speed = mxf(speed, mxf(a, b));
    }
    float cr = D.max_face_cfl ? mxf(s[0] / D.hx, mxf(s[1] / D.hy, s[2] / D.hz))
                              : (s[0] / D.hx) * 1.f + (s[1] / D.hy) * 1.f + (s[2] / D.hz) * 1.f;
    fv[0] = cr * G.dt;
    bool w = D.kind[i] > 0;
    float dv = w ? G.divergence(q) : 0.f;
    float rr = w ? 1000.f / G.dt * dv : 0.f;
    if (rr != 0.f) v[0] = (double)rr * (double)rr;
    float div = w ? G.dt * fabsf(dv) : 0.f;
    float err = w ? fabsf(p - 9810.0f * (g.eta(q) - g.center(q).y)) : 0.f;
    float f = G.Cb[i];
    double vol = f != 0.f ? (double)f * D.cell_d : 0.0;
    if (isnan(div) || isnan(speed) || isnan(err) || isnan(f) || isinf(div) || isinf(speed) || isinf(err) || isinf(f)) {
      div = speed = err = 1e30f;
      vol = 1e30;
    }
    fv[1] = div;
    fv[2] = speed;
    fv[3] = err;
    v[1] = vol;
  }
  const int ops[2] = {0, 0};
  double out[2];
  float fout[4];
  if (last_block_reduce_mf<NT, 2, 4>(D, kSiteAccept, v, ops, fv, out, fout) && threadIdx.x == 0) {
    double* c = D.c;
    double dtd = (double)G.dt;
    // op 36
    c[27] = (double)fout[0];
    // op 66
    double r2 = out[0];
    auto scaled = [&](double sq) { return dtd * dtd / 1000 * sqrt(sq > 0 ? sq : 0.0); };
    double tol = (double)D.tol;
    auto conv = [&](double res2, double rhs2) {
      return res2 <= tol * tol * rhs2 || (scaled(rhs2) <= 1e-5 && scaled(res2) <= 1e-8);
    };
    c[60] = sqrt(r2 / (c[59] > 1e-30 ? c[59] : 1e-30));
    c[62] = scaled(c[59]);
    c[63] = scaled(r2);
    c[61] = conv(r2, c[59]) ? 1 : 0;
    // op 13
    float vx = fout[1], vy = fout[2], vz = fout[3];
    double vw = out[1];
    c[14] = vx; c[15] = vy; c[16] = vz; c[17] = vw;
    if ((vx >= 1e-4f || c[61] < .5) && vy < 1e20f && c[19] < .5 && c[58] < 4) {
      c[57] = 1; c[58] += 1; c[6] = 0;
      return;
    }
    if (c[61] < .5) { c[3] += 1; c[7] = 4; return; }
    if (vx >= 1e-4f || vy >= 1e20f || c[19] > .5) { c[3] += 1; c[7] = 4; return; }
    c[28] = vw + c[40] + c[39] - c[26] - c[24] - c[22];
    if (D.coastal) c[28] += c[74] + c[66] - c[73] - c[65] - c[72] - c[64];
    c[kConservation] = vw - c[26] - (c[kRoundCommit] + c[kSweepRound]) - (c[kCompCommit] + c[kSweepComp]) + (c[40] + c[39]) -
                       (c[73] + c[65]) + (c[74] + c[66]) - (c[72] + c[64]);
    if (fabs(c[28]) > 1e-3 * (c[26] > 1e-20 ? c[26] : 1e-20)) { c[3] += 1; c[7] = 21; return; }
    if (c[27] > (double)D.cfl + 1e-6) { c[3] += 1; c[7] = 20; return; }
    c[24] += c[22]; c[25] += c[23]; c[40] += c[39]; c[29] = 0; c[30] = 0;
    c[kRoundCommit] += c[kSweepRound];
    c[kCompCommit] += c[kSweepComp];
    if (D.coastal) {
      for (int k = 0; k < 6; k++) c[72 + k] += c[64 + k];
      c[90] = c[20];
    }
    c[0] = 1 - c[0];
    c[1] += c[20];
    c[2] += 1;
    c[4] = 0;
  }
}

// ---------------------------------------------------------------- ops 44, 85, 89 (one block)
// One block of kTrialEndThreads threads.  Op 85 (gauges of the accepted state): for each of the
// eight gauge columns x, the column heights oy + sum_y (solid ? 1 : F) hy of every z, each summed
// in y order, then the gauge's mean over z in z order.  The terms of kGaugeZ planes at a time are
// loaded by the whole block into shared memory (every load independent), then summed in that order.
constexpr int kTrialEndThreads = 1024, kGaugeVals = 10240, kGaugeMaxZ = 128;
__global__ void __launch_bounds__(kTrialEndThreads) k_trial_end(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  __shared__ float vals[kGaugeVals];
  __shared__ float cols[8 * kGaugeMaxZ];
  __shared__ int gx[8];
  Grid g(D);
  const float* A = bank_ptr(D, acc_bank(D));
  double* c = D.c;
  if (D.coastal) {
    if (threadIdx.x < 8) {
      float begin = D.forcing[0] + D.forcing[1] + .4f;
      float end = D.ox + (float)D.nx * D.hx - (D.shape == 6 ? D.forcing[1] + .4f : 1.0f);
      float tt = (float)threadIdx.x / 7.f;
      float pos = begin * (1.f - tt) + end * tt;
      gx[threadIdx.x] = min(max((int)((pos - D.ox) / D.hx), 0), D.nx - 1);
    }
    __syncthreads();
    const int ny = D.ny;
    const int zc = min(kGaugeMaxZ, max(1, kGaugeVals / (8 * ny)));
    const bool staged = 8 * ny <= kGaugeVals;
    float height = 0.f;
    for (int z0 = 0; z0 < D.nz; z0 += zc) {
      const int nzc = min(zc, D.nz - z0);
      if (staged) {
        for (int t = threadIdx.x; t < 8 * nzc * ny; t += kTrialEndThreads) {
          const int gi = t / (nzc * ny), r = t - gi * (nzc * ny), zl = r / ny, y = r - zl * ny;
          const I3 q = mk(gx[gi], y, z0 + zl);
          vals[t] = (g.solid(q) ? 1.f : A[g.index3(q)]) * D.hy;
        }
        __syncthreads();
        if (threadIdx.x < 8 * nzc) {
          const float* v = vals + threadIdx.x * ny;  // gauge threadIdx.x / nzc, plane threadIdx.x % nzc
          float column = D.oy;
          for (int y = 0; y < ny; y++) column += v[y];
          cols[threadIdx.x] = column;
        }
      } else if (threadIdx.x < 8 * nzc) {
        const int gi = threadIdx.x / nzc, z = z0 + threadIdx.x % nzc;
        float column = D.oy;
        for (int y = 0; y < ny; y++) {
          const I3 q = mk(gx[gi], y, z);
          column += (g.solid(q) ? 1.f : A[g.index3(q)]) * D.hy;
        }
        cols[threadIdx.x] = column;
      }
      __syncthreads();
      if (threadIdx.x < 8)
        for (int zl = 0; zl < nzc; zl++) height += cols[threadIdx.x * nzc + zl];
      __syncthreads();
    }
    if (threadIdx.x < 8) c[80 + threadIdx.x] = (double)(height / (float)D.nz);
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  // op 44
  if (c[32] > 0 && c[32] <= D.hist_cap) {
    long long row = (long long)(c[32] - 1) * 4 + 3;
    D.history[row] = make_float4((float)c[1], (float)c[20], c[7] > 0 ? (float)(-c[7]) : (c[4] < .5 ? 1.f : 0.f), (float)c[2]);
  }
  // op 89
  if (D.coastal && !(c[2] <= c[91] || c[2] > D.hist_cap)) {
    long long row = (long long)(c[2] - 1) * 5;
    float4* h = D.chistory;
    h[row] = make_float4((float)c[1], (float)c[90], (float)c[17], (float)c[72]);
    h[row + 1] = make_float4((float)c[73], (float)c[74], (float)c[40], (float)c[24]);
    h[row + 2] = make_float4((float)c[80], (float)c[81], (float)c[82], (float)c[83]);
    h[row + 3] = make_float4((float)c[84], (float)c[85], (float)c[86], (float)c[87]);
    h[row + 4] = make_float4((float)c[75], (float)c[76], (float)c[77], (float)c[28]);
    c[91] = c[2];
  }
}

// ---------------------------------------------------------------- coastal ops 80-84
__global__ void __launch_bounds__(NT) k_coast_cells(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Geo G(D, 80);
  const Grid& g = G.g;
  long long cells = (long long)D.zone_x_end * D.ny * D.nz;
  long long t = (long long)blockIdx.x * NT + threadIdx.x;
  double v[4] = {0, 0, 0, 0};
  if (t < cells) {
    const unsigned zx = (unsigned)D.zone_x_end, rest = (unsigned)t / zx;
    I3 q = mk(int((unsigned)t - rest * zx), int(rest % (unsigned)D.ny), int(rest / (unsigned)D.ny));
    if (!g.solid(q)) {
      long long i = g.index3(q);
      float time = (float)(D.c[1] + D.c[20]);
      F3 cq = g.center(q);
      float old = G.Cb[i];
      float target = G.cs.offshore(cq.x) ? G.cs.fraction(g, q, time) : clampf_(.5f - cq.y / D.hy, 0.f, 1.f);
      float value = old + G.cs.relax(g, q, -1, G.dt) * (target - old);
      G.Cb[i] = value;
      v[0] = ((double)value - (double)old) * D.cell_d;
      float vel[3];
      for (int axis = 0; axis < 3; axis++) {
        I3 r = ax(q, axis, 1);
        vel[axis] = .5f * (G.Cb[g.face_index(q, axis)] + G.Cb[g.face_index(r, axis)]);
      }
      double m = (double)(1000.f * (value - old)) * D.cell_d;
      v[1] = m * (double)vel[0];
      v[2] = m * (double)vel[1];
      v[3] = m * (double)vel[2];
    }
  }
  const int ops[4] = {0, 0, 0, 0};
  double out[4];
  if (last_block_reduce<NT, 4>(D, kSiteCoastF, v, ops, out) && threadIdx.x == 0) {
    D.c[64] += out[0];
    D.c[67] += out[1];
    D.c[68] += out[2];
    D.c[69] += out[3];
  }
}
__global__ void __launch_bounds__(NT) k_coast_faces(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Geo G(D, 82);
  const Grid& g = G.g;
  long long t = (long long)blockIdx.x * NT + threadIdx.x;
  // faces with x <= zone_x_end of the three lattices, in lattice order
  int zx = D.zone_x_end + 1;
  long long nu = (long long)zx * D.ny * D.nz, nv = (long long)zx * (D.ny + 1) * D.nz, nw = (long long)zx * D.ny * (D.nz + 1);
  if (t >= nu + nv + nw) return;
  int axis;
  long long rest;
  int my_;
  if (t < nu) { axis = 0; rest = t; my_ = D.ny; }
  else if (t < nu + nv) { axis = 1; rest = t - nu; my_ = D.ny + 1; }
  else { axis = 2; rest = t - nu - nv; my_ = D.ny; }
  const unsigned ur = (unsigned)rest, row = ur / (unsigned)zx;
  I3 q = mk(int(ur - row * (unsigned)zx), int(row % (unsigned)my_), int(row / (unsigned)my_));
  int mxl = D.nx + (axis == 0);
  if (q.x >= mxl) return;
  long long f;
  if (axis == 0) f = (long long)q.x + (long long)(D.nx + 1) * ((long long)q.y + (long long)D.ny * q.z);
  else if (axis == 1) f = D.NU + (long long)q.x + (long long)D.nx * ((long long)q.y + (long long)(D.ny + 1) * q.z);
  else f = D.NU + D.NV + (long long)q.x + (long long)D.nx * ((long long)q.y + (long long)D.ny * q.z);
  float time = (float)(D.c[1] + D.c[20]);
  F3 position = G.cs.face_position(g, q, axis);
  float old = G.Cb[D.N + f], value = old;
  if (!g.wall_face(q, axis)) {
    float target = G.cs.offshore(position.x) ? G.cs.velocity_face(g, q, axis, time) : 0.f;
    float a = G.cs.relax(g, q, axis, G.dt);
    value = old * (1.f - a) + target * a;
    if (axis == 0 && q.x == 0) value = target;
  }
  G.Cb[D.N + f] = value;
  D.fwd[f] = value - old;
}
__global__ void __launch_bounds__(NT) k_coast_momentum(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Geo G(D, 83);
  const Grid& g = G.g;
  long long cells = (long long)D.zone_x_end * D.ny * D.nz;
  long long t = (long long)blockIdx.x * NT + threadIdx.x;
  double v[3] = {0, 0, 0};
  if (t < cells) {
    const unsigned zx = (unsigned)D.zone_x_end, rest = (unsigned)t / zx;
    I3 q = mk(int((unsigned)t - rest * zx), int(rest % (unsigned)D.ny), int(rest / (unsigned)D.ny));
    long long i = g.index3(q);
    float m = G.Cb[i] * 1000.f;
    for (int axis = 0; axis < 3; axis++) {
      I3 r = ax(q, axis, 1);
      float ch = .5f * (D.fwd[g.face_local(q, axis)] + D.fwd[g.face_local(r, axis)]);
      v[axis] = (double)ch * (double)m * D.cell_d;
    }
  }
  const int ops[3] = {0, 0, 0};
  double out[3];
  if (last_block_reduce<NT, 3>(D, kSiteCoastM, v, ops, out) && threadIdx.x == 0) {
    for (int a = 0; a < 3; a++) D.c[67 + a] += out[a];
  }
}

// ---------------------------------------------------------------- export (op 19) into buffers
// Op 19 (pressure_pass.glslinc:127-130) and, when `clock` is given, the surface clock of
// surface_clock.glsl:7: the committed (accepted time, accepted steps) read after the export.
__global__ void __launch_bounds__(NT) k_export(const __grid_constant__ Dev D, float4* planes, float* kinds,
                                               float4* clock) {
  grid_dep_wait(D.pdl_early);
  Geo G(D, 19);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i == 0 && clock) *clock = make_float4((float)D.c[1], (float)D.c[2], 0.f, 0.f);
  if (i >= D.N) return;
  float f = G.A[i];
  planes[i] = G.reconstruct(G.g.coord(i));
  kinds[i] = f <= 0.f ? 0.f : (f >= 1.f ? 1.f : 2.f);
}

}  // namespace

static unsigned grid_for(long long n) { return (unsigned)((n + NT - 1) / NT); }

void launch_coastal(const Dev& D, cudaStream_t s) {
  long long cells = (long long)D.zone_x_end * D.ny * D.nz;
  int zx = D.zone_x_end + 1;
  long long faces = (long long)zx * D.ny * D.nz + (long long)zx * (D.ny + 1) * D.nz + (long long)zx * D.ny * (D.nz + 1);
  pdl_launch(k_coast_cells, grid_for(cells), NT, 0, s, D);
  pdl_launch(k_coast_faces, grid_for(faces), NT, 0, s, D);
  pdl_launch(k_coast_momentum, grid_for(cells), NT, 0, s, D);
}
void launch_geometry(const Dev& D, cudaStream_t s) {
  pdl_launch(k_geom_plane, grid_for(D.N), NT, 0, s, D, 17, D.coastal);
  pdl_launch(k_geom_phi, grid_for(D.N), NT, 0, s, D);
  pdl_launch(k_geom_seed, D.geo_seed_grid, NT, 0, s, D);
  pdl_launch(k_geom_coef, grid_for(D.N), NT, 0, s, D);
}
void launch_proj_setup(const Dev& D, cudaStream_t s) { pdl_launch(k_proj_setup, grid_for(D.S), NT, 0, s, D); }
void launch_post(const Dev& D, cudaStream_t s) {
  pdl_launch(k_grad_apply, grid_for(D.NF), NT, 0, s, D);
  pdl_launch(k_ext_init, grid_for(D.NF), NT, 0, s, D);
  pdl_launch(k_ext_step, grid_for(D.NF), NT, 0, s, D, 0);
  pdl_launch(k_ext_step, grid_for(D.NF), NT, 0, s, D, 1);
  pdl_launch(k_ext_step, grid_for(D.NF), NT, 0, s, D, 0);
  pdl_launch(k_ext_write, grid_for(D.NF > D.N ? D.NF : D.N), NT, 0, s, D);
  pdl_launch(k_accept, grid_for(D.N), NT, 0, s, D);
}
void launch_ext_masks(const Dev& D, cudaStream_t s) { pdl_launch(k_ext_masks, grid_for(D.NF), NT, 0, s, D); }
void launch_trial_end(const Dev& D, cudaStream_t s) { pdl_launch(k_trial_end, 1, kTrialEndThreads, 0, s, D); }
void launch_export(const Dev& D, cudaStream_t s, float4* planes, float* kinds, float4* clock) {
  pdl_launch(k_export, grid_for(D.N), NT, 0, s, D, planes, kinds, clock);
}

}  // namespace wg
