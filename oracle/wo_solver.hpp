// TEST INFRASTRUCTURE ONLY — CPU oracle of the waves solver step (see wo_common.hpp).
//
// Solver<R> holds the reference's buffers (pressure_gpu.gd:92-117, coupled_gpu.gd:23-33,
// coastal_gpu.gd:9-20) and executes its dispatch list op by op with the shaders' own gating, so a
// "batch" here is exactly one pass of coupled_gpu.gd:_record_commands (+ coastal additions).
// The control block c[] follows the reference index map (pressure_core.glslinc:24,
// coupled_motion.glslinc:6-7, coastal_pass.glslinc:36-37) but is stored in double.
#pragma once
#include "wo_common.hpp"

namespace wo {

template <class R> struct Solver;

// Multigrid hierarchy state (pressure_multigrid.gd, pressure_multigrid.glslinc,
// pressure_mg_coarse.glslinc, pressure_hierarchy_state.{gd,glsl}).
template <class R> struct MG {
  struct Level {
    I3 n;
    int count = 0;
    I3 f;
    bool aggregate = false;
    std::vector<I3> stencil;
    int twidth = 1;  // transfer-cache width (md(l,14))
  };
  std::vector<Level> levels;
  std::vector<std::vector<R>> v;              // 8 fields x count per level
  std::vector<std::vector<R>> matrix;         // canonical 125-slot rows (l >= 1)
  std::vector<R> ap;                          // A P of the Galerkin product's first stage (125 per fine row)
  std::vector<std::vector<R>> ellv;           // ELL values [k][i] (l >= 1)
  std::vector<std::vector<int>> ellc;         // ELL columns [k][i]
  std::vector<std::vector<int>> tid;          // transfer cache ids [k][i] (l < L-1)
  std::vector<std::vector<R>> tw;             // transfer cache weights
  std::vector<R> linv;                        // dense L^-1 of the last level
  std::vector<R> snapshot, previous;          // 9N each
  std::vector<uint32_t> state;                // audit state, 64 + 32 * capacity
  std::vector<R> c0bf;                        // BF16 copies of the 6 level-0 face coefficients
};

template <class R> struct Solver {
  // ---- parameters (push constants, pressure_core.glslinc:34-43) ----
  I3 n;
  R h[3];
  R dtcfg;
  V3<R> org;
  R eta0;
  bool px = false;
  R slope, corr, corr_phase;
  R shape, grav;
  bool max_face_cfl = false;
  int hist_cap = 0;
  R wave[4];
  R tol;
  bool linear_air = false, stokes2 = false;
  int flags = 0;
  bool coastal = true;
  R forcing[4];
  R right_abs;
  R cfl;
  int iters_per_batch = 8;
  int mg_smoother = 1, mg_smoothing = 3, mg_mode = 2, mg_lag = 8, mg_aggr = 2;
  bool bf16 = false;

  // ---- sizes ----
  size_t N = 0, NU = 0, NV = 0, NW = 0, S = 0, NF = 0;

  // ---- buffers ----
  std::vector<R> bank[2];
  std::vector<R> work;  // 14 N: r, z, d, q, diag, b, coef[6], diag, defect base
  std::vector<R> gphi, gkind;
  std::vector<V4<R>> plane;
  std::vector<R> mF, mci, flux, fwd;
  std::vector<int32_t> src[2];
  std::vector<R> vband[2], pmask[2];
  std::vector<R> tcache[6];
  std::vector<V4<R>> history, chistory;
  V4<R> probe[8];
  double c[WAVES_CONTROL_SIZE];
  double red[4];  // contents of the reduction partials, as the final reduce would see them
  double quota = 0;
  MG<R> mg;

  // ---------------------------------------------------------------- set-up
  explicit Solver(const waves_config& k) {
    n = I3(k.n[0], k.n[1], k.n[2]);
    for (int a = 0; a < 3; a++) h[a] = R(k.spacing[a]);
    dtcfg = R(k.dt);
    org = V3<R>(R(k.origin[0]), R(k.origin[1]), R(k.origin[2]));
    eta0 = R(k.eta);
    px = k.periodic_x != 0;
    slope = R(k.slope);
    corr = R(k.corrugation);
    corr_phase = R(k.corrugation_phase);
    shape = R(k.shape);
    grav = R(k.gravity);
    max_face_cfl = k.max_face_cfl != 0;
    hist_cap = k.history_capacity;
    for (int a = 0; a < 4; a++) wave[a] = R(k.wave[a]);
    tol = R(k.pressure_tolerance);
    linear_air = k.linear_air != 0;
    stokes2 = k.stokes_second != 0;
    flags = (k.height_normals ? 1 : 0) + (k.active_advection ? 2 : 0) + (k.transport_cache ? 4 : 0) +
            (k.transport_interior ? 8 : 0);
    coastal = k.coastal != 0;
    forcing[0] = R(k.origin[0]);
    forcing[1] = R(k.zone_length);
    forcing[2] = R(k.damping_rate);
    forcing[3] = R(k.ramp_periods);
    right_abs = R(k.right_absorption);
    cfl = R(k.cfl);
    iters_per_batch = k.iterations_per_batch;
    mg_smoother = k.mg_smoother;
    mg_smoothing = k.mg_smoothing;
    mg_mode = k.mg_maintenance;
    mg_lag = k.mg_lag;
    mg_aggr = k.mg_aggregate_from;
    bf16 = (k.mg_precision == 16);
    N = size_t(n.x) * n.y * n.z;
    NU = size_t(n.x + 1) * n.y * n.z;
    NV = size_t(n.x) * (n.y + 1) * n.z;
    NW = size_t(n.x) * n.y * (n.z + 1);
    S = 2 * N + NU + NV + NW;
    NF = NU + NV + NW;
    for (int b = 0; b < 2; b++) {
      bank[b].assign(S, R(0));
      src[b].assign(NF, -1);
      vband[b].assign(NF, R(0));
      pmask[b].assign(N, R(0));
    }
    work.assign(14 * N, R(0));
    gphi.assign(N, R(0));
    gkind.assign(N, R(0));
    plane.assign(N, V4<R>());
    mF.assign(N, R(0));
    mci.assign(N, R(0));
    flux.assign(NF, R(0));
    fwd.assign(NF, R(0));
    for (int f = 0; f < 6; f++) tcache[f].assign(NF, R(0));
    history.assign(size_t(std::max(hist_cap, 0)) * 4, V4<R>());
    chistory.assign(size_t(std::max(hist_cap, 0)) * 5, V4<R>());
    std::fill(c, c + WAVES_CONTROL_SIZE, 0.0);
    for (double& r : red) r = 0;
    build_solid_table();
    mg_initialize();
  }

  // ---------------------------------------------------------------- pressure_core.glslinc
  size_t U() const { return N; }
  size_t V() const { return N + NU; }
  size_t W() const { return N + NU + NV; }
  size_t P() const { return N + NU + NV + NW; }
  static size_t index3(I3 q, I3 m) { return size_t(q.x) + size_t(m.x) * (size_t(q.y) + size_t(m.y) * size_t(q.z)); }
  static I3 coord(size_t i, I3 m) { return I3(int(i % m.x), int((i / m.x) % m.y), int(i / (size_t(m.x) * m.y))); }
  R dt() const { return R(c[20]); }  // timestep() (pressure_core.glslinc:58-64), coupled
  int accepted() const { return int(c[0]); }
  int candidate() const { return 1 - accepted(); }
  // geometry_bank (pressure_core.glslinc:66-72)
  int geometry_bank(int op) const { return (op == 19 || c[4] < .5) ? accepted() : candidate(); }
  // eta (pressure_core.glslinc:73-83)
  R eta(I3 q) const {
    if (shape == R(5)) {
      R phase = wave[1] * (org.x + (R(q.x) + R(.5)) * h[0]);
      R sigma = ttanh(wave[1] * wave[3]);
      R second = stokes2 ? wave[1] * wave[0] * wave[0] * (R(3) - sigma * sigma) / (R(4) * sigma * sigma * sigma) : R(0);
      return eta0 + wave[0] * tcos(phase) + second * tcos(R(2) * phase);
    }
    return eta0 + corr * tcos(R(6.28318530718) * (R(q.x) + R(0.5)) / R(n.x) + corr_phase);
  }
  V3<R> center(I3 q) const {
    return V3<R>(org.x + (R(q.x) + R(0.5)) * h[0], org.y + (R(q.y) + R(0.5)) * h[1], org.z + (R(q.z) + R(0.5)) * h[2]);
  }
  I3 wrap_cell(I3 q) const {
    q.z = periodic_index(q.z, n.z);
    if (px) q.x = periodic_index(q.x, n.x);
    return q;
  }
  bool outside(I3 q) const { return q.x < 0 || q.x >= n.x || q.y < 0 || q.y >= n.y; }
  // solid (pressure_core.glslinc:87-96).  A pure function of the wrapped (x, y): tabulated on a
  // margin of kPad cells around the domain, evaluated directly beyond it.
  static constexpr int kPad = 16;
  std::vector<char> solid_tab;
  void build_solid_table() {
    int wx = n.x + 2 * kPad, wy = n.y + 2 * kPad;
    solid_tab.assign(size_t(wx) * wy, 0);
    for (int y = 0; y < wy; y++)
      for (int x = 0; x < wx; x++) solid_tab[size_t(y) * wx + x] = solid_direct(I3(x - kPad, y - kPad, 0)) ? 1 : 0;
  }
  bool solid(I3 q) const {
    q = wrap_cell(q);
    int x = q.x + kPad, y = q.y + kPad;
    if (x >= 0 && y >= 0 && x < n.x + 2 * kPad && y < n.y + 2 * kPad) return solid_tab[size_t(y) * (n.x + 2 * kPad) + x] != 0;
    return solid_direct(q);
  }
  bool solid_direct(I3 q) const {
    q = wrap_cell(q);
    if (q.y < 0 || q.x >= n.x) return true;
    if (!coastal && q.x < 0) return true;
    if (q.y >= n.y) return false;
    if (slope > R(0)) {
      R x = center(q).x;
      R bed = R(-0.45) + mx(R(0), x - R(1.5)) / slope;
      return center(q).y <= bed;
    }
    return false;
  }
  bool wet(I3 q) const {
    q = wrap_cell(q);
    return !outside(q) && gkind[index3(q, n)] > R(0.5);
  }
  R phi(I3 q) const {
    q = wrap_cell(q);
    return outside(q) ? center(q).y - eta(q) : gphi[index3(q, n)];
  }
  R press(I3 q) const {
    q = wrap_cell(q);
    return wet(q) ? bank[candidate()][P() + index3(q, n)] : R(0);
  }
  // distance_face (pressure_core.glslinc:100-109)
  R distance_face(I3 l, I3 r, int axis) const {
    R hh = h[axis];
    if (axis == 1 && (l.y >= n.y || r.y >= n.y)) return R(.5) * hh;
    bool wl = wet(l), wr = wet(r);
    if (wl && wr) return hh;
    R pl = std::fabs(phi(l)), pr = std::fabs(phi(r));
    return hh * mx((wl ? pl : pr) / mx(pl + pr, R(1e-30)), R(1e-6));
  }
  // coefficient (pressure_core.glslinc:110-118)
  R coefficient(I3 q, I3 nb, int axis) const {
    if (solid(nb)) return R(0);
    if (coastal && axis == 0 && nb.x < 0) return R(0);
    return R(1.0) / (h[axis] * distance_face(q, nb, axis));
  }
  R vector_at(I3 q, int which) const {
    q = wrap_cell(q);
    if (!wet(q)) return R(0);
    size_t i = index3(q, n);
    return which == 0 ? press(q) : work[2 * N + i];
  }
  // operator_at (pressure_core.glslinc:120-125)
  R operator_at(I3 q, int which) const {
    R result = 0, here = vector_at(q, which);
    size_t i = index3(q, n);
    int face = 0;
    for (int axis = 0; axis < 3; axis++)
      for (int sign = -1; sign <= 1; sign += 2) {
        I3 nb = q;
        nb[axis] += sign;
        R k = work[size_t(6 + face) * N + i];
        result += k * (here - vector_at(nb, which));
        face++;
      }
    return result;
  }
  R diagonal(I3 q) const { return work[12 * N + index3(q, n)]; }
  // face_index (pressure_core.glslinc:129-133)
  size_t face_index(I3 q, int axis) const {
    I3 m = n;
    if (axis == 2 && q.z == m.z) q.z = 0;
    if (axis == 0 && px && q.x == m.x) q.x = 0;
    m[axis]++;
    return (axis == 0 ? U() : (axis == 1 ? V() : W())) + index3(q, m);
  }
  R divergence(I3 q) const {
    R d = 0;
    const std::vector<R>& b = bank[candidate()];
    for (int axis = 0; axis < 3; axis++) {
      I3 right = q;
      right[axis]++;
      d += (b[face_index(right, axis)] - b[face_index(q, axis)]) / h[axis];
    }
    return d;
  }
  bool pressure_setup() const { return c[5] > .5 || c[57] == 2; }
  double pressure_scaled_norm(double squared) const {
    double d = double(dt());
    return d * d / 1000 * std::sqrt(std::max(squared, 0.0));
  }
  bool pressure_norm_converged(double residual2, double rhs2) const {
    double t = double(tol);
    return residual2 <= t * t * rhs2 || (pressure_scaled_norm(rhs2) <= 1e-5 && pressure_scaled_norm(residual2) <= 1e-8);
  }
  bool residual_converged(const double s[4], double rhs2) const {
    double d = double(dt());
    return pressure_norm_converged(s[1], rhs2) && d * d / 1000 * s[3] < 5e-5;
  }
  bool solving() const { return c[4] > 0.5 && c[6] < 0.5 && c[7] < 0.5; }

  // ---------------------------------------------------------------- plic_math.glslinc
  static R cube_volume(V3<R> normal, R alpha) {
    alpha -= mn(normal.x, R(0)) + mn(normal.y, R(0)) + mn(normal.z, R(0));
    V3<R> v = abs3(normal);
    R total = v.x + v.y + v.z;
    if (alpha <= R(0)) return R(0);
    if (alpha >= total) return R(1);
    if (v.x > v.y) std::swap(v.x, v.y);
    if (v.y > v.z) std::swap(v.y, v.z);
    if (v.x > v.y) std::swap(v.x, v.y);
    bool complement = alpha > R(0.5) * total;
    R t = complement ? total - alpha : alpha;
    R x = v.x, y = v.y, z = v.z, result;
    if (x < R(1e-6) * total) {
      t -= x * R(0.5);
      if (y < R(1e-6) * total) result = (t - y * R(0.5)) / z;
      else if (t < y) result = t * t / (R(2) * y * z);
      else result = (t - R(0.5) * y) / z;
    } else if (t < x) result = t * t * t / (R(6) * x * y * z);
    else if (t < y) result = (R(3) * t * t - R(3) * t * x + x * x) / (R(6) * y * z);
    else if (x + y < z && t >= x + y) result = (t - R(0.5) * (x + y)) / z;
    else {
      R ty = mx(t - y, R(0)), tz = mx(t - z, R(0));
      R numerator = x * (R(3) * t * t - R(3) * t * x + x * x) - ty * ty * ty - tz * tz * tz;
      result = numerator / (R(6) * x * y * z);
    }
    return complement ? R(1.0) - result : result;
  }
  static R inverse_volume(V3<R> normal, R fraction) {
    R lo = mn(normal.x, R(0)) + mn(normal.y, R(0)) + mn(normal.z, R(0));
    R hi = mx(normal.x, R(0)) + mx(normal.y, R(0)) + mx(normal.z, R(0));
    for (int it = 0; it < 25; it++) {
      R mid = R(0.5) * (lo + hi);
      if (cube_volume(normal, mid) < fraction) lo = mid;
      else hi = mid;
    }
    R alpha = R(0.5) * (lo + hi), cen = half_dot(normal);
    if (fraction == R(.5)) return cen;
    if (fraction < R(.5)) return mn(alpha, cen);
    if (alpha <= cen) alpha = cen + R(5.96046448e-8) * l1(normal);
    return alpha;
  }

  // ---------------------------------------------------------------- coastal_target.glslinc
  static R smooth_ramp(R q) {
    q = clampr(q, R(0), R(1));
    return q * q * q * (R(10) + q * (R(-15) + R(6) * q));
  }
  R ramped_amplitude(R time) const {
    return wave[0] * smooth_ramp(time * wave[2] / (R(6.28318530718) * forcing[3]));
  }
  void coastal_surface(R x, R time, R& s0, R& s1) const {
    R a = ramped_amplitude(time), k = wave[1], w = wave[2], hh = wave[3];
    R sigma = ttanh(k * hh), second = k * a * a * (R(3) - sigma * sigma) / (R(4) * sigma * sigma * sigma);
    if (!stokes2) second = 0;
    R phase = k * (x - forcing[0]) - w * time;
    s0 = a * tcos(phase) + second * tcos(R(2) * phase);
    s1 = -k * a * tsin(phase) - R(2) * k * second * tsin(R(2) * phase);
  }
  V3<R> coastal_velocity(V3<R> world, R time) const {
    R a = ramped_amplitude(time), k = wave[1], w = wave[2], hh = wave[3];
    R s = tsinh(k * hh), phase = k * (world.x - forcing[0]) - w * time, y = world.y + hh;
    R first = a * w / s, second = stokes2 ? R(.75) * a * a * w * k / tpow4(s) : R(0);
    return V3<R>(first * tcosh(k * y) * tcos(phase) + second * tcosh(R(2) * k * y) * tcos(R(2) * phase),
                 first * tsinh(k * y) * tsin(phase) + second * tsinh(R(2) * k * y) * tsin(R(2) * phase), R(0));
  }
  V3<R> coastal_face_position(I3 q, int axis) const {
    V3<R> p = center(q);
    p[axis] -= R(.5) * h[axis];
    return p;
  }
  V4<R> coastal_plane(I3 q, R time) const {
    R s0, s1;
    coastal_surface(center(q).x, time, s0, s1);
    V3<R> normal(-s1 * h[0], h[1], R(0));
    return V4<R>(normal.x, normal.y, normal.z, half_dot(normal) + s0 - center(q).y);
  }
  R coastal_fraction(I3 q, R time) const {
    V4<R> eq = coastal_plane(q, time);
    return clampr(cube_volume(eq.xyz(), eq.w), R(0), R(1));
  }
  R coastal_rate(R x) const {
    R left = R(1) - smooth_ramp((x - forcing[0]) / forcing[1]);
    R right = shape == R(6) ? smooth_ramp((x - (org.x + R(n.x) * h[0] - forcing[1])) / forcing[1]) : R(0);
    return forcing[2] * mx(left, right_abs * right);
  }
  bool offshore_zone(R x) const { return x < forcing[0] + forcing[1]; }
  R time_plus_dt() const { return R(c[1] + c[20]); }  // c[1]+timestep()

  // ---------------------------------------------------------------- pressure_geometry.glslinc
  R geometry_fraction(I3 q, int op) const {
    q = wrap_cell(q);
    if (coastal && q.x < 0 && !solid(q))
      return coastal_fraction(q, R(c[1] + (geometry_bank(op) == candidate() ? c[20] : 0.0)));
    if (solid(q)) {
      q.x = std::min(std::max(q.x, 0), n.x - 1);
      q.y = std::min(std::max(q.y, 0), n.y - 1);
      q.z = std::min(std::max(q.z, 0), n.z - 1);
    }
    if (outside(q)) return R(0);
    return bank[geometry_bank(op)][index3(q, n)];
  }
  // transport_f (coupled_motion.glslinc:36-44)
  R transport_f(I3 q) const {
    q = wrap_cell(q);
    if (coastal && q.x < 0 && !solid(q)) return coastal_fraction(q, R(c[1]));
    if (outside(q) || solid(q)) return R(0);
    size_t i = index3(q, n);
    int sweep = int(c[21]);
    return sweep == 0 ? bank[accepted()][i] : (sweep == 1 ? bank[candidate()][i] : mF[i]);
  }
  R hf_fraction(I3 q, int source, int op) const { return source == 1 ? transport_f(q) : geometry_fraction(q, op); }
  bool hf_valid(I3 q) const {
    q = wrap_cell(q);
    return !outside(q) && !solid(q);
  }
  V3<R> interface_gradient(I3 q, int source, int op) const {
    V3<R> g(0, 0, 0);
    for (int axis = 0; axis < 3; axis++) {
      int b = (axis + 1) % 3, d = (axis + 2) % 3, weights = 0;
      for (int j = -1; j <= 1; j++)
        for (int k = -1; k <= 1; k++) {
          I3 middle = q;
          middle[b] += j;
          middle[d] += k;
          if (solid(middle)) continue;
          I3 l = middle, r = middle;
          l[axis]--;
          r[axis]++;
          bool left = !solid(l), right = !solid(r);
          if (!left && !right) continue;
          R difference;
          if (left && right) difference = hf_fraction(l, source, op) - hf_fraction(r, source, op);
          else if (left) difference = R(2) * (hf_fraction(l, source, op) - hf_fraction(middle, source, op));
          else difference = R(2) * (hf_fraction(middle, source, op) - hf_fraction(r, source, op));
          int weight = (j == 0 ? 2 : 1) * (k == 0 ? 2 : 1);
          weights += weight;
          g[axis] += R(weight) * difference / (R(32) * h[axis]);
        }
      if (weights > 0) g[axis] *= R(16.0) / R(weights);
    }
    return g;
  }
  // height_normal.glslinc:6-34
  V3<R> height_normal(I3 q, V3<R> youngs, int source, int op) const {
    V3<R> sp(h[0], h[1], h[2]);
    V3<R> scaled = mul3(abs3(youngs), sp);
    int axis = scaled.x > scaled.y ? 0 : 1;
    if (scaled.z > scaled[axis]) axis = 2;
    if (scaled[axis] < R(1e-12)) return youngs;
    int b = (axis + 1) % 3, d = (axis + 2) % 3;
    R orientation = sgn(youngs[axis]);
    R heights[5];
    for (int column = 0; column < 5; column++) {
      I3 base = q;
      if (column == 1) base[b]--;
      if (column == 2) base[b]++;
      if (column == 3) base[d]--;
      if (column == 4) base[d]++;
      R sum = 0, previous = orientation > R(0) ? R(1) : R(0);
      for (int t = -4; t <= 4; t++) {
        I3 cell = base;
        cell[axis] += t;
        if (!hf_valid(cell)) return youngs;
        R f = hf_fraction(cell, source, op);
        if (std::isnan(f) || std::isinf(f) || f < R(0) || f > R(1)) return youngs;
        if (orientation * (f - previous) > R(2e-6)) return youngs;
        if (t == -4 && f != (orientation > R(0) ? R(1) : R(0))) return youngs;
        if (t == 4 && f != (orientation > R(0) ? R(0) : R(1))) return youngs;
        sum += f;
        previous = f;
      }
      heights[column] = sum * sp[axis];
    }
    V3<R> result(0, 0, 0);
    result[axis] = orientation;
    result[b] = -(heights[2] - heights[1]) / (R(2) * sp[b]);
    result[d] = -(heights[4] - heights[3]) / (R(2) * sp[d]);
    return result;
  }
  V4<R> plane_from_gradient(V3<R> g, R f) const {
    if (len3(g) < R(1e-9)) g = V3<R>(0, 1, 0);
    R L = len3(g);
    V3<R> normal(g.x / L * h[0], g.y / L * h[1], g.z / L * h[2]);
    R s = l1(normal);
    normal = V3<R>(normal.x / s, normal.y / s, normal.z / s);
    return V4<R>(normal.x, normal.y, normal.z, inverse_volume(normal, f));
  }
  // reconstruct_pressure (pressure_geometry.glslinc:54-61)
  V4<R> reconstruct_pressure(I3 q, int op) const {
    R f = geometry_fraction(q, op);
    if (f <= R(0) || f >= R(1)) return V4<R>(0, 1, 0, f);
    V3<R> g = interface_gradient(q, 0, op);
    if (flags & 1) g = height_normal(q, g, 0, op);
    return plane_from_gradient(g, f);
  }
  // transport_plane (coupled_motion.glslinc:50-56)
  V4<R> transport_plane(I3 q) const {
    R f = transport_f(q);
    if (f <= R(0) || f >= R(1)) return V4<R>(0, 1, 0, f);
    V3<R> g = interface_gradient(q, 1, 23);
    if (flags & 1) g = height_normal(q, g, 1, 23);
    return plane_from_gradient(g, f);
  }
  R segment_distance(V3<R> point, V3<R> a, V3<R> b) const {
    V3<R> ab = sub3(b, a);
    R t = clampr(dot3(sub3(point, a), ab) / mx(dot3(ab, ab), R(1e-30)), R(0), R(1));
    return len3(sub3(point, add3(a, scl3(ab, t))));
  }
  R polygon_distance(V3<R> point, V4<R> eq) const {
    V3<R> hh(h[0], h[1], h[2]);
    V3<R> normal = div3(eq.xyz(), hh);
    R norm2 = dot3(normal, normal);
    R s = dot3(normal, point) - eq.w;
    R signed_d = s / std::sqrt(norm2);
    V3<R> projected(point.x - normal.x * s / norm2, point.y - normal.y * s / norm2, point.z - normal.z * s / norm2);
    if (projected.x >= R(0) && projected.y >= R(0) && projected.z >= R(0) && projected.x <= hh.x && projected.y <= hh.y &&
        projected.z <= hh.z)
      return std::fabs(signed_d);
    V3<R> vertices[12];
    int count = 0;
    for (int axis = 0; axis < 3; axis++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) {
          V3<R> a(0, 0, 0);
          a[(axis + 1) % 3] = R(j);
          a[(axis + 2) % 3] = R(k);
          R den = eq[axis];
          if (std::fabs(den) < R(1e-15)) continue;
          R t = (eq.w - dot3(eq.xyz(), a)) / den;
          if (t >= R(0) && t <= R(1)) {
            a[axis] = t;
            vertices[count++] = mul3(a, hh);
          }
        }
    R best = R(1e10);
    for (int j = 0; j < count; j++) {
      best = mn(best, len3(sub3(point, vertices[j])));
      for (int k = 0; k < j; k++) best = mn(best, segment_distance(point, vertices[j], vertices[k]));
    }
    return best;
  }
  static int clip_polygon(V3<R> poly[12], int count, V4<R> eq) {
    V3<R> result[12];
    int size = 0;
    for (int j = 0; j < count; j++) {
      V3<R> a = poly[j], b = poly[(j + 1) % count];
      R da = dot3(eq.xyz(), a) - eq.w, db = dot3(eq.xyz(), b) - eq.w;
      if (da <= R(0)) result[size++] = a;
      if ((da < R(0) && db > R(0)) || (da > R(0) && db < R(0))) {
        R t = da / (da - db);
        result[size++] = V3<R>(a.x * (R(1) - t) + b.x * t, a.y * (R(1) - t) + b.y * t, a.z * (R(1) - t) + b.z * t);
      }
    }
    for (int j = 0; j < size; j++) poly[j] = result[j];
    return size;
  }
  R transition_distance(V3<R> point, I3 left, int axis, int op) const {
    I3 right = left;
    right[axis]++;
    I3 l = wrap_cell(left), r = wrap_cell(right);
    if (outside(l) || outside(r) || solid(l) || solid(r)) return R(1e10);
    R fl = geometry_fraction(l, op), fr = geometry_fraction(r, op);
    if ((fl <= R(0) && fr <= R(0)) || (fl >= R(1) && fr >= R(1))) return R(1e10);
    V4<R> a = plane[index3(l, n)], b = plane[index3(r, n)];
    if (fl <= R(0)) a = V4<R>(0, 0, 0, -1);
    if (fl >= R(1)) a = V4<R>(0, 0, 0, 1);
    if (fr <= R(0)) b = V4<R>(0, 0, 0, -1);
    if (fr >= R(1)) b = V4<R>(0, 0, 0, 1);
    b.w += b[axis];
    R best = R(1e10);
    V3<R> hh(h[0], h[1], h[2]);
    for (int side = 0; side < 2; side++) {
      V3<R> poly[12];
      int j = (axis + 1) % 3, k = (axis + 2) % 3;
      for (int v = 0; v < 4; v++) {
        poly[v] = V3<R>(0, 0, 0);
        poly[v][axis] = R(1);
        poly[v][j] = (v == 1 || v == 2) ? R(1) : R(0);
        poly[v][k] = v >= 2 ? R(1) : R(0);
      }
      V4<R> first = side == 0 ? a : b;
      V4<R> second = side == 0 ? V4<R>(-b.x, -b.y, -b.z, -b.w) : V4<R>(-a.x, -a.y, -a.z, -a.w);
      int count = clip_polygon(poly, 4, first);
      count = clip_polygon(poly, count, second);
      if (count == 0) continue;
      V3<R> projected = point;
      projected[axis] = hh[axis];
      V3<R> local = div3(projected, hh);
      if (local.x >= R(0) && local.y >= R(0) && local.z >= R(0) && local.x <= R(1) && local.y <= R(1) &&
          local.z <= R(1) && dot3(first.xyz(), local) <= first.w && dot3(second.xyz(), local) <= second.w)
        best = mn(best, std::fabs(point[axis] - hh[axis]));
      for (int v = 0; v < count; v++)
        best = mn(best, segment_distance(point, mul3(poly[v], hh), mul3(poly[(v + 1) % count], hh)));
    }
    return best;
  }
  R geometry_distance(I3 q, int op) const {
    R f = geometry_fraction(q, op);
    V3<R> hh(h[0], h[1], h[2]);
    if (f > R(0) && f < R(1)) {
      V4<R> eq = plane[index3(q, n)];
      return (half_dot(eq.xyz()) - eq.w) / len3(div3(eq.xyz(), hh));
    }
    bool needs_seed = false;
    for (int axis = 0; axis < 3; axis++)
      for (int sign = -1; sign <= 1; sign += 2) {
        I3 nb = q;
        nb[axis] += sign;
        nb = wrap_cell(nb);
        if (solid(nb) || outside(nb)) continue;
        R other = geometry_fraction(nb, op);
        bool inside = other >= R(1);
        if (other > R(0) && other < R(1)) {
          V4<R> eq = plane[index3(nb, n)];
          inside = half_dot(eq.xyz()) < eq.w;
        }
        if (inside != (f >= R(1))) needs_seed = true;
      }
    if (!needs_seed) return (f >= R(1) ? R(-1) : R(1)) * len3(hh) * R(4);
    R best = len3(hh) * R(4);
    for (int x = -1; x <= 1; x++)
      for (int y = -1; y <= 1; y++)
        for (int z = -1; z <= 1; z++) {
          I3 neighbor = q + I3(x, y, z), wrapped = wrap_cell(neighbor);
          if (outside(wrapped) || solid(wrapped)) continue;
          R fraction = geometry_fraction(wrapped, op);
          I3 dq = q - neighbor;
          V3<R> point((R(dq.x) + R(.5)) * hh.x, (R(dq.y) + R(.5)) * hh.y, (R(dq.z) + R(.5)) * hh.z);
          V3<R> cl(clampr(point.x, R(0), hh.x), clampr(point.y, R(0), hh.y), clampr(point.z, R(0), hh.z));
          if (len3(sub3(point, cl)) >= best) continue;
          if (fraction > R(0) && fraction < R(1)) best = mn(best, polygon_distance(point, plane[index3(wrapped, n)]));
          for (int axis = 0; axis < 3; axis++) best = mn(best, transition_distance(point, neighbor, axis, op));
        }
    return (f >= R(1) ? R(-1) : R(1)) * best;
  }

  // ---------------------------------------------------------------- coupled_motion.glslinc helpers
  size_t faces() const { return NF; }
  size_t face_local(I3 q, int axis) const { return face_index(q, axis) - U(); }
  void unpack_face(size_t f, I3& q, int& axis) const {
    axis = f < NU ? 0 : (f < NU + NV ? 1 : 2);
    size_t base = axis == 0 ? 0 : (axis == 1 ? NU : NU + NV);
    I3 m = n;
    m[axis]++;
    q = coord(f - base, m);
  }
  V3<R> periodic_delta(I3 a, I3 b) const {
    V3<R> d(R(a.x - b.x), R(a.y - b.y), R(a.z - b.z));
    d.z -= std::round(d.z / R(n.z)) * R(n.z);
    if (px) d.x -= std::round(d.x / R(n.x)) * R(n.x);
    return V3<R>(d.x * h[0], d.y * h[1], d.z * h[2]);
  }
  bool wall_face(I3 q, int axis) const {
    I3 l = q;
    l[axis]--;
    return solid(q) || solid(l);
  }
  bool face_in_bounds(I3 q, int axis) const {
    I3 m = n;
    m[axis]++;
    return q.x >= 0 && q.y >= 0 && q.z >= 0 && q.x < m.x && q.y < m.y && q.z < m.z;
  }
  I3 wrap_face(I3 q, int) const {
    q.z = periodic_index(q.z, n.z);
    if (px) q.x = periodic_index(q.x, n.x);
    return q;
  }
  R old_face(I3 q, int axis) const {
    q = wrap_face(q, axis);
    if (coastal && q.x < 0 && !wall_face(q, axis)) return coastal_velocity(coastal_face_position(q, axis), R(c[1]))[axis];
    if (!face_in_bounds(q, axis) || wall_face(q, axis)) return R(0);
    return bank[accepted()][face_index(q, axis)];
  }
  R face_courant(I3 q, int axis) const { return old_face(q, axis) * dt() / h[axis]; }

  // reflect_voxel_donor (coupled_motion.glslinc:66-85)
  bool reflect_voxel_donor(I3& q, int component, R& parity) const {
    R best = R(1e20);
    I3 selected = q;
    parity = 1;
    for (int axis = 0; axis < 3; axis++)
      for (int sign = -1; sign <= 1; sign += 2) {
        for (int layer = 1; layer <= 3; layer++) {
          I3 edge = q;
          edge[axis] += sign * layer;
          edge = wrap_face(edge, component);
          if (!face_in_bounds(edge, component)) break;
          I3 left = edge;
          left[component]--;
          bool sl = solid(left), sr = solid(edge);
          bool boundary = axis == component ? (sl != sr) : (!sl && !sr);
          if (!boundary) continue;
          I3 mirror = q;
          mirror[axis] += sign * (2 * layer - (axis == component ? 0 : 1));
          mirror = wrap_face(mirror, component);
          R distance = (R(layer) - (axis == component ? R(0) : R(.5))) * h[axis];
          if (face_in_bounds(mirror, component) && !wall_face(mirror, component) && distance < best) {
            selected = mirror;
            best = distance;
            parity = axis == component ? R(-1) : R(1);
          }
          break;
        }
      }
    q = selected;
    return best < R(1e19);
  }
  // velocity_donor (coupled_motion.glslinc:86-111)
  R velocity_donor(I3 q, int axis, bool forward, bool& valid) const {
    R parity = 1;
    if (q.y < 0) {
      q.y = -q.y - (axis == 1 ? 0 : 1);
      if (axis == 1) parity = -parity;
    }
    if (!px) {
      if (!coastal && q.x < 0) {
        q.x = -q.x - (axis == 0 ? 0 : 1);
        if (axis == 0) parity = -parity;
      }
      if (q.x >= n.x + (axis == 0 ? 1 : 0)) {
        q.x = 2 * n.x - q.x - (axis == 0 ? 0 : 1);
        if (axis == 0) parity = -parity;
      }
    }
    q = wrap_face(q, axis);
    if (coastal && q.x < 0 && q.y >= 0 && q.y < n.y && !wall_face(q, axis)) {
      valid = true;
      return parity * coastal_velocity(coastal_face_position(q, axis), R(c[1]))[axis];
    }
    if (!face_in_bounds(q, axis)) {
      valid = false;
      return 0;
    }
    I3 l = q;
    l[axis]--;
    bool left = solid(l), right = solid(q);
    if (left != right) {
      valid = true;
      return 0;
    }
    if (left && right) {
      R reflection;
      if (!reflect_voxel_donor(q, axis, reflection)) {
        valid = false;
        return 0;
      }
      parity *= reflection;
    }
    size_t f = face_local(q, axis);
    valid = vband[accepted()][f] > R(.5);
    return parity * (forward ? fwd[f] : bank[accepted()][face_index(q, axis)]);
  }
  // sampled_component (coupled_motion.glslinc:112-137)
  R sampled_component(V3<R> x, int axis, bool forward, bool& valid, R& lim0, R& lim1) const {
    V3<R> lattice(x.x / h[0] - R(.5), x.y / h[1] - R(.5), x.z / h[2] - R(.5));
    lattice[axis] += R(.5);
    I3 lo(int(std::floor(lattice.x)), int(std::floor(lattice.y)), int(std::floor(lattice.z)));
    V3<R> t(fract_(lattice.x), fract_(lattice.y), fract_(lattice.z));
    lim0 = R(1e20);
    lim1 = R(-1e20);
    valid = true;
    bool interior = (flags & 8) != 0 && lo.x >= 1 && lo.y >= 1 && lo.z >= 1 && lo.x + 1 < n.x && lo.y + 1 < n.y &&
                    lo.z + 1 < n.z && !solid(I3(lo.x + 1, lo.y - 1, lo.z));
    I3 fn = n;
    fn[axis]++;
    R values[8];
    for (int z = 0; z < 2; z++)
      for (int y = 0; y < 2; y++)
        for (int xx = 0; xx < 2; xx++) {
          bool supported;
          R value;
          if (interior) {
            size_t base = face_local(lo, axis);
            size_t f = base + size_t(xx + fn.x * (y + fn.y * z));
            supported = vband[accepted()][f] > R(.5);
            value = forward ? fwd[f] : bank[accepted()][U() + f];
          } else
            value = velocity_donor(lo + I3(xx, y, z), axis, forward, supported);
          values[xx + 2 * y + 4 * z] = value;
          R wx = xx ? t.x : R(1) - t.x, wy = y ? t.y : R(1) - t.y, wz = z ? t.z : R(1) - t.z;
          if (wx * wy * wz > R(0)) {
            valid = valid && supported;
            lim0 = mn(lim0, value);
            lim1 = mx(lim1, value);
          }
        }
    R a = std::fma(t.x, values[1] - values[0], values[0]), b = std::fma(t.x, values[3] - values[2], values[2]);
    R d = std::fma(t.x, values[5] - values[4], values[4]), e = std::fma(t.x, values[7] - values[6], values[6]);
    R lower = std::fma(t.y, b - a, a), upper = std::fma(t.y, e - d, d);
    return std::fma(t.z, upper - lower, lower);
  }
  V3<R> sampled_velocity(V3<R> x) const {
    V3<R> v;
    for (int axis = 0; axis < 3; axis++) {
      bool valid;
      R l0, l1v;
      v[axis] = sampled_component(x, axis, false, valid, l0, l1v);
    }
    return v;
  }
  V3<R> trace(V3<R> x, R d) const {
    V3<R> s = sampled_velocity(x);
    R hd = R(.5) * d;
    V3<R> mid(x.x - hd * s.x, x.y - hd * s.y, x.z - hd * s.z);
    V3<R> s2 = sampled_velocity(mid);
    return V3<R>(x.x - d * s2.x, x.y - d * s2.y, x.z - d * s2.z);
  }
  bool solid_at(V3<R> p) const {
    return solid(I3(int(std::floor(p.x / h[0])), int(std::floor(p.y / h[1])), int(std::floor(p.z / h[2]))));
  }
  bool trace_supported(V3<R> x, R d) const {
    V3<R> s = sampled_velocity(x);
    R hd = R(.5) * d;
    V3<R> mid(x.x - hd * s.x, x.y - hd * s.y, x.z - hd * s.z);
    V3<R> s2 = sampled_velocity(mid);
    V3<R> end(x.x - d * s2.x, x.y - d * s2.y, x.z - d * s2.z);
    for (int stage = 0; stage < 3; stage++) {
      V3<R> point = stage == 0 ? x : (stage == 1 ? mid : end);
      if (solid_at(point)) return false;
      for (int axis = 0; axis < 3; axis++) {
        bool valid;
        R l0, l1v;
        sampled_component(point, axis, false, valid, l0, l1v);
        if (!valid) return false;
      }
    }
    return true;
  }
  V3<R> sampled_velocity_checked(V3<R> x, bool& supported) const {
    V3<R> value;
    supported = true;
    for (int axis = 0; axis < 3; axis++) {
      bool valid;
      R l0, l1v;
      value[axis] = sampled_component(x, axis, false, valid, l0, l1v);
      supported = supported && valid;
    }
    return value;
  }
  R checked_endpoint(V3<R> x, int component, bool forward, bool& supported, R& lim0, R& lim1) const {
    R value = 0;
    supported = true;
    lim0 = 0;
    lim1 = 0;
    for (int axis = 0; axis < 3; axis++) {
      bool valid;
      R d0, d1;
      R dv = sampled_component(x, axis, axis == component && forward, valid, d0, d1);
      supported = supported && valid;
      if (axis == component) {
        value = dv;
        lim0 = d0;
        lim1 = d1;
      }
    }
    return value;
  }
  bool trace_points_clear(V3<R> x, V3<R> mid, V3<R> end) const {
    return !solid_at(x) && !solid_at(mid) && !solid_at(end);
  }
  // cached_advection (coupled_motion.glslinc:168-188)
  R cached_advection(size_t i, V3<R> x, int axis, R d, bool correct) {
    if (!correct) {
      bool vs, vm, ve;
      R l0, l1v;
      V3<R> sv = sampled_velocity_checked(x, vs);
      R hd = R(.5) * d;
      V3<R> mid(x.x - hd * sv.x, x.y - hd * sv.y, x.z - hd * sv.z);
      V3<R> s2 = sampled_velocity_checked(mid, vm);
      V3<R> end(x.x - d * s2.x, x.y - d * s2.y, x.z - d * s2.z);
      R value = checked_endpoint(end, axis, false, ve, l0, l1v);
      tcache[0][i] = l0;
      tcache[1][i] = l1v;
      tcache[2][i] = (vs && vm && ve && trace_points_clear(x, mid, end)) ? R(1) : R(0);
      for (int k = 0; k < 3; k++) tcache[3 + k][i] = sv[k];
      return value;
    }
    R forward = fwd[i];
    if (tcache[2][i] < R(.5)) return forward;
    V3<R> sv(tcache[3][i], tcache[4][i], tcache[5][i]);
    bool vm, ve;
    R u0, u1;
    R rd = -d;
    R hd = R(.5) * rd;
    V3<R> mid(x.x - hd * sv.x, x.y - hd * sv.y, x.z - hd * sv.z);
    V3<R> s2 = sampled_velocity_checked(mid, vm);
    V3<R> end(x.x - rd * s2.x, x.y - rd * s2.y, x.z - rd * s2.z);
    R backward = checked_endpoint(end, axis, true, ve, u0, u1);
    R value = forward + R(.5) * (bank[accepted()][U() + i] - backward);
    return (vm && ve && trace_points_clear(x, mid, end) && value >= tcache[0][i] && value <= tcache[1][i]) ? value : forward;
  }
  // courant_at (coupled_motion.glslinc:189-202)
  R courant_at(I3 q, int b, bool accelerate) const {
    V3<R> speed(0, 0, 0);
    for (int axis = 0; axis < 3; axis++) {
      I3 r = q;
      r[axis]++;
      speed[axis] = mx(std::fabs(bank[b][face_index(q, axis)]), std::fabs(bank[b][face_index(r, axis)]));
    }
    if (coastal && accelerate) {
      V3<R> cq = center(q);
      R tt = R(c[1] + double(dtcfg));
      R s0, s1;
      coastal_surface(cq.x, tt, s0, s1);
      if (coastal_rate(cq.x) > R(0) && cq.y < s0 + R(3) * h[1]) {
        for (int axis = 0; axis < 3; axis++) {
          I3 r = q;
          r[axis]++;
          speed[axis] = mx(speed[axis], mx(std::fabs(coastal_velocity(coastal_face_position(q, axis), tt)[axis]),
                                           std::fabs(coastal_velocity(coastal_face_position(r, axis), tt)[axis])));
        }
      }
    }
    if (accelerate) speed.y += R(9.81) * dtcfg * grav;
    speed = div3(speed, V3<R>(h[0], h[1], h[2]));
    return max_face_cfl ? mx(speed.x, mx(speed.y, speed.z)) : speed.x * R(1) + speed.y * R(1) + speed.z * R(1);
  }
  R linear_streamfunction(V3<R> x) const {
    R value = wave[0] * wave[2] / (wave[1] * tsinh(wave[1] * wave[3])) * tsinh(wave[1] * (x.y + wave[3])) * tcos(wave[1] * x.x);
    if (stokes2)
      value += R(.375) * wave[0] * wave[0] * wave[2] / tpow4(tsinh(wave[1] * wave[3])) * tsinh(R(2) * wave[1] * (x.y + wave[3])) *
               tcos(R(2) * wave[1] * x.x);
    return value;
  }
  bool projected_face(I3 q, int axis) const {
    q = wrap_face(q, axis);
    if (!face_in_bounds(q, axis) || wall_face(q, axis)) return false;
    I3 l = q;
    l[axis]--;
    return wet(q) || wet(l);
  }
  R extended_value(size_t source, I3 target) const {
    const std::vector<R>& cb = bank[candidate()];
    R value = cb[U() + source];
    if (!linear_air) return value;
    I3 q;
    int component;
    unpack_face(source, q, component);
    V3<R> gradient(0, 0, 0);
    for (int axis = 0; axis < 3; axis++) {
      I3 l = q, r = q;
      l[axis]--;
      r[axis]++;
      l = wrap_face(l, component);
      r = wrap_face(r, component);
      bool left = projected_face(l, component), right = projected_face(r, component);
      R dl = left ? value - cb[face_index(l, component)] : R(0);
      R dr = right ? cb[face_index(r, component)] - value : R(0);
      if (left && right) gradient[axis] = dl * dr > R(0) ? sgn(dl) * mn(std::fabs(dl), std::fabs(dr)) : R(0);
      else gradient[axis] = left ? dl : (right ? dr : R(0));
    }
    V3<R> pd = periodic_delta(target, q);
    V3<R> off(clampr(pd.x / h[0], R(-1), R(1)), clampr(pd.y / h[1], R(-1), R(1)), clampr(pd.z / h[2], R(-1), R(1)));
    return value + dot3(gradient, off);
  }
  V3<R> cell_velocity(int b, I3 q) const {
    V3<R> vel;
    for (int axis = 0; axis < 3; axis++) {
      I3 r = q;
      r[axis]++;
      vel[axis] = R(.5) * (bank[b][face_index(q, axis)] + bank[b][face_index(r, axis)]);
    }
    return vel;
  }
  R cellvol() const { return h[0] * h[1] * h[2]; }

#include "wo_ops.inc"
#include "wo_mg.inc"
};

}  // namespace wo
