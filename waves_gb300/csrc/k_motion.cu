// Motion phase of the solver step: CFL time step, compression pre-check, the three directional
// PLIC/Weymouth-Yue VOF sweeps and limited MacCormack advection
// (neuron-forest/waves water/shaders/compute/coupled_motion.glslinc ops 20-28, 45/46, 55/56).
#include "common.cuh"
#include "kernels.h"

namespace wg {

namespace {
constexpr int NT = 256;

struct Motion {
  const Dev& D;
  Grid g;
  Coast cs;
  int acc, cand;
  const float* A;  // accepted bank
  float* Cb;       // candidate bank
  float dt;
  double c1;
  DI explicit Motion(const Dev& d) : D(d), g(d), cs(d) {
    acc = acc_bank(d);
    cand = 1 - acc;
    A = bank_ptr(d, acc);
    Cb = bank_ptr(d, cand);
    dt = (float)d.c[20];
    c1 = d.c[1];
  }
  // old_face (coupled_motion.glslinc:28-35)
  DI float old_face(I3 q, int axis) const {
    q = g.wrap_face(q);
    if (D.coastal && q.x < 0 && !g.wall_face(q, axis)) return cs.velocity_face(g, q, axis, (float)c1);
    if (!g.face_in_bounds(q, axis) || g.wall_face(q, axis)) return 0.f;
    return A[g.face_index(q, axis)];
  }
  // transport_f (coupled_motion.glslinc:36-44)
  DI float transport_f(I3 q) const {
    q = g.wrap_cell(q);
    if (D.coastal && q.x < 0 && !g.solid(q)) return cs.fraction(g, q, (float)c1);
    if (g.outside(q) || g.solid(q)) return 0.f;
    long long i = g.index3(q);
    int sweep = (int)D.c[21];
    return sweep == 0 ? A[i] : (sweep == 1 ? Cb[i] : D.mF[i]);
  }
  // courant_at (coupled_motion.glslinc:189-202)
  DI float courant_at(I3 q, const float* B, bool accelerate) const {
    float s[3];
    for (int axis = 0; axis < 3; axis++) {
      I3 r = ax(q, axis, 1);
      s[axis] = mxf(fabsf(B[g.face_index(q, axis)]), fabsf(B[g.face_index(r, axis)]));
    }
    if (D.coastal && accelerate) {
      F3 cq = g.center(q);
      float tt = (float)(c1 + (double)D.dtcfg);
      if (cs.rate(cq.x) > 0.f) {
        float s0, s1;
        cs.surface_col(g, q.x, tt, s0, s1);
        if (cq.y < s0 + 3.f * D.hy) {
          for (int axis = 0; axis < 3; axis++) {
            I3 r = ax(q, axis, 1);
            s[axis] = mxf(s[axis], mxf(fabsf(cs.velocity_face(g, q, axis, tt)), fabsf(cs.velocity_face(g, r, axis, tt))));
          }
        }
      }
    }
    if (accelerate) s[1] += 9.81f * D.dtcfg * D.grav;
    s[0] = s[0] / D.hx;
    s[1] = s[1] / D.hy;
    s[2] = s[2] / D.hz;
    return D.max_face_cfl ? mxf(s[0], mxf(s[1], s[2])) : s[0] * 1.f + s[1] * 1.f + s[2] * 1.f;
  }
};

DI bool setup_on(const Dev& D) { return D.c[5] > .5 && D.c[7] < .5; }

// ---------------------------------------------------------------- wave-target tables
// which 0: the accepted time and the CFL look-ahead time (before op 20); which 1: the new time
// c1 + dt and the relaxation factors at dt (after op 20 has set dt).  One thread per (column, row).
__global__ void __launch_bounds__(NT) k_wave_tables(const __grid_constant__ Dev D, int which) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  const Grid g(D);
  const Coast cs(D);
  const int t = blockIdx.x * NT + threadIdx.x;
  if (t >= D.wt_w * D.wt_h) return;
  const int j = t % D.wt_w, y = t / D.wt_w, x = D.wt_x0 + j;
  const double c1 = D.c[1];
  const float times[3] = {(float)c1, (float)(c1 + (double)D.dtcfg), (float)(c1 + D.c[20])};
  for (int sl = which == 0 ? 0 : 2; sl <= (which == 0 ? 1 : 2); sl++) {
    const float time = times[sl];
    if (y == 0) {
      float s0, s1;
      cs.surface(g.center(mk(x, 0, 0)).x, time, s0, s1);
      D.wsurf[sl * D.wt_w + j] = make_float2(s0, s1);
    }
    for (int axis = 0; axis < 2; axis++)
      D.wvel[((sl * 2 + axis) * D.wt_h + y) * D.wt_w + j] = cs.velocity_c(cs.face_position(g, mk(x, y, 0), axis), time, axis);
    if (t == 0) D.wstamp[sl] = time;
  }
  if (which == 1 && y == 0) {
    const float dt = (float)D.c[20];
    D.wdecay[j] = 1.f - texp(-cs.rate(g.center(mk(x, 0, 0)).x) * dt);
    D.wdecay[D.wt_w + j] = 1.f - texp(-cs.rate(cs.face_position(g, mk(x, 0, 0), 0).x) * dt);
    if (t == 0) D.wstamp[3] = dt;
  }
}

// ---------------------------------------------------------------- op 20/21
__global__ void __launch_bounds__(NT) k_cfl(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Motion m(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  float v[1] = {0.f};
  if (i < D.N) v[0] = m.courant_at(m.g.coord(i), m.A, true);
  float out[1];
  if (last_block_reduce_mf<NT, 0, 1>(D, kSiteCFL, nullptr, nullptr, v, nullptr, out) && threadIdx.x == 0) {
    double* c = D.c;
    float rate = mxf(0.f, out[0]);
    float d = mnf(D.dtcfg, D.cfl / mxf(rate, 1e-20f));
    if (c[29] > 0) d = mnf(d, (float)c[30]);
    c[20] = (double)d;
    c[21] = 0; c[22] = 0; c[23] = 0; c[39] = 0; c[kSweepRound] = 0; c[kSweepComp] = 0;
    if (D.coastal)
      for (int f = 64; f < 70; f++) c[f] = 0;
  }
}

// ---------------------------------------------------------------- op 45/46 + c_i of op 22
__global__ void __launch_bounds__(NT) k_compress(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Motion m(D);
  const float* pmA = m.acc == 0 ? D.pmask0 : D.pmask1;
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  double v[4] = {0, 0, 0, 0};
  if (i < D.N) {
    I3 q = m.g.coord(i);
    float f = m.A[i];
    float dv = 0.f, raw = 0.f;
    for (int axis = 0; axis < 3; axis++) {
      I3 r = ax(q, axis, 1);
      float h = m.g.h(axis);
      dv += (m.old_face(r, axis) - m.old_face(q, axis)) / h;
      raw += (m.A[m.g.face_index(r, axis)] - m.A[m.g.face_index(q, axis)]) / h;
    }
    if (f > .5f) v[0] = (double)(m.dt * dv) * D.cell_d;
    if (f > .5f && pmA[i] < .5f) v[1] = 1.0;
    if (f != 0.f) v[2] = (double)f * D.cell_d;
    if (f > .5f) v[3] = (double)(m.dt * raw) * D.cell_d;
    D.mci[i] = f > .5f ? 1.f : 0.f;
  }
  const int ops[4] = {0, 0, 0, 0};
  double out[4];
  if (last_block_reduce<NT, 4>(D, kSiteCompress, v, ops, out) && threadIdx.x == 0) {
    double* c = D.c;
    c[35] = out[0]; c[36] = out[1]; c[37] = out[2]; c[38] = out[3];
    if (out[1] > 0) { c[7] = 22; c[3] += 1; }
  }
}

// ---------------------------------------------------------------- op 22 (faces and pressure)
// candidate <- accepted (coupled_motion.glslinc:370-373).  The sweeps rewrite every F, so only the
// faces and the pressure are copied; in an accepted trial MacCormack and op 2 overwrite them too,
// but a trial that fails before them (CFL, compression, sweep bounds) leaves this copy, as the
// reference does.  c_i is set by k_compress.
__global__ void __launch_bounds__(NT) k_stage_candidate(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  const int acc = acc_bank(D);
  const float4* src = reinterpret_cast<const float4*>(bank_ptr(D, acc) + D.N);
  float4* dst = reinterpret_cast<float4*>(bank_ptr(D, 1 - acc) + D.N);
  const long long n = D.NF + D.N, n4 = (D.N % 4 == 0 && n % 4 == 0) ? n / 4 : 0;  // 16-byte aligned, whole
  const long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (n4) {
    if (i < n4) dst[i] = src[i];
  } else if (i < n) {
    bank_ptr(D, 1 - acc)[D.N + i] = bank_ptr(D, acc)[D.N + i];
  }
}

// ---------------------------------------------------------------- op 23
// 6 resident blocks per SM (40 registers): measured on the beach equal to or faster than the
// register-rich forms for this and the update kernel (k_sweep_update 187 vs 195-213 us)
__global__ void __launch_bounds__(NT, 6) k_sweep_plane(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Motion m(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i >= D.N) return;
  I3 q = m.g.coord(i);
  float f = m.transport_f(q);
  float4 out;
  if (f <= 0.f || f >= 1.f) out = make_float4(0.f, 1.f, 0.f, f);
  else {
    auto fr = [&](I3 p) { return m.transport_f(p); };
    F3 grad = interface_gradient(m.g, q, fr);
    if (D.flags & 1) grad = height_normal(m.g, q, grad, fr);
    out = plane_from_gradient(D, grad, f);
  }
  D.plane[i] = out;
}

// op 24 flux of one sweep-axis face (coupled_motion.glslinc:375-388); `courant` returns the face's
// Courant number old_face * dt / h (the face_courant expression), which the update needs as well.
DI float sweep_flux(const Motion& m, I3 q, int axis, float& courant) {
  const Dev& D = m.D;
  const float velocity = m.old_face(q, axis);
  courant = velocity * m.dt / m.g.h(axis);
  if (m.g.wall_face(q, axis)) return 0.f;
  I3 donor = q;
  if (velocity > 0.f) donor[axis]--;
  donor = m.g.wrap_cell(donor);
  float f = m.transport_f(donor), width = fabsf(courant);
  float amount = f * width;
  if (f > 0.f && f < 1.f && width > 0.f) {
    float4 eq = (D.coastal && donor.x < 0) ? m.cs.plane(m.g, donor, (float)m.c1) : D.plane[m.g.index3(donor)];
    F3 n = mf(eq.x, eq.y, eq.z);
    F3 low = mf(0.f, 0.f, 0.f), extent = mf(1.f, 1.f, 1.f);
    extent[axis] = width;
    if (velocity > 0.f) low[axis] = 1.f - width;
    amount = width * cube_volume(mul3(n, extent), eq.w - dot3(n, low));
  }
  return amount * sgnf(velocity);
}

// ---------------------------------------------------------------- op 24 + 55/56 + 25/26
__global__ void __launch_bounds__(NT, 6) k_sweep_update(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Motion m(D);
  int sa = ((int)D.c[2] + (int)D.c[21]) % 3;
  int sweep = (int)D.c[21];
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  // FP32 maxima: -min f, max f; FP64 sums: change, |change|, rounding ledger, compression, top,
  // in, out
  float fv[2] = {-1e20f, -1e20f};
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  if (i < D.N) {
    I3 q = m.g.coord(i), r = ax(q, sa, 1);
    float cq, cr;
    float fq = sweep_flux(m, q, sa, cq), fr_ = sweep_flux(m, r, sa, cr);
    float net = fq - fr_;
    float correction = D.mci[i] * (cr - cq);
    float increment = net + correction;
    float fin = m.transport_f(q);
    float f = fin + increment;
    float change = 0.f;
    if (f >= -1e-6f && f <= 1.f + 1e-6f) change = clampf_(f, 0.f, 1.f) - f;
    float out = f + change;
    if (sweep == 1) D.mF[i] = out;
    else m.Cb[i] = out;
    float a = f, b = f;
    if (isnan(f) || isinf(f)) { a = -1e30f; b = 1e30f; }
    fv[0] = -a;
    fv[1] = b;
    // the FP64 ledger terms only where they can be other than zero
    if (change != 0.f) {
      v[0] = (double)change;
      v[1] = (double)fabsf(change);
    }
    if (out != fin || net != 0.f || correction != 0.f)
      v[2] = ((double)out - (double)fin - (double)net - (double)correction) * D.cell_d;
    if (correction != 0.f) v[3] = (double)correction * D.cell_d;
    if (sa == 1 && q.y == D.ny - 1) v[4] = (double)fr_ * D.cell_d;
    if (D.coastal && sa == 0 && q.x == 0) {
      double fl = (double)fq * D.cell_d;
      v[5] = fl > 0 ? fl : 0.0;
      v[6] = -fl > 0 ? -fl : 0.0;
    }
  }
  const int ops[7] = {0, 0, 0, 0, 0, 0, 0};
  double out[7];
  float fout[2];
  if (last_block_reduce_mf<NT, 7, 2>(D, kSiteSweep, v, ops, fv, out, fout) && threadIdx.x == 0) {
    double* c = D.c;
    float vmin = -fout[0], vmax = fout[1];
    long long step = (long long)c[32] - 1;
    if (c[32] >= 1 && step < D.hist_cap) D.history[step * 4 + sweep] = make_float4(vmin, vmax, (float)out[0], (float)out[1]);
    c[22] += out[0] * D.cell_d;
    c[23] += out[1] * D.cell_d;
    c[kSweepRound] += out[2];
    c[kSweepComp] += out[3];
    c[39] += out[4];
    if (D.coastal) { c[65] += out[5]; c[66] += out[6]; }
    if (vmin < -1e-6f || vmax > 1.f + 1e-6f) { c[7] = 10 + c[21]; c[3] += 1; }
    c[21] += 1;
  }
}

// ---------------------------------------------------------------- MacCormack
struct Mac {
  const Motion& m;
  const float* vb;  // valid band of the accepted bank
  DI explicit Mac(const Motion& mm) : m(mm) { vb = mm.acc == 0 ? mm.D.vband0 : mm.D.vband1; }
  // reflect_voxel_donor (coupled_motion.glslinc:66-85)
  __device__ __noinline__ bool reflect(I3& q, int component, float& parity) const {
    const Grid& g = m.g;
    float best = 1e20f;
    I3 selected = q;
    parity = 1.f;
    for (int axis = 0; axis < 3; axis++)
      for (int sign = -1; sign <= 1; sign += 2) {
        for (int layer = 1; layer <= 3; layer++) {
          I3 edge = g.wrap_face(ax(q, axis, sign * layer));
          if (!g.face_in_bounds(edge, component)) break;
          I3 left = ax(edge, component, -1);
          bool sl = g.solid(left), sr = g.solid(edge);
          bool boundary = axis == component ? (sl != sr) : (!sl && !sr);
          if (!boundary) continue;
          I3 mirror = g.wrap_face(ax(q, axis, sign * (2 * layer - (axis == component ? 0 : 1))));
          float distance = ((float)layer - (axis == component ? 0.f : .5f)) * g.h(axis);
          if (g.face_in_bounds(mirror, component) && !g.wall_face(mirror, component) && distance < best) {
            selected = mirror;
            best = distance;
            parity = axis == component ? -1.f : 1.f;
          }
          break;
        }
      }
    q = selected;
    return best < 1e19f;
  }
  // velocity_donor (coupled_motion.glslinc:86-111)
  __device__ __noinline__ float donor(I3 q, int axis, bool forward, bool& valid) const {
    const Grid& g = m.g;
    const Dev& D = m.D;
    float parity = 1.f;
    if (q.y < 0) {
      q.y = -q.y - (axis == 1 ? 0 : 1);
      if (axis == 1) parity = -parity;
    }
    if (!D.px) {
      if (!D.coastal && q.x < 0) {
        q.x = -q.x - (axis == 0 ? 0 : 1);
        if (axis == 0) parity = -parity;
      }
      if (q.x >= D.nx + (axis == 0 ? 1 : 0)) {
        q.x = 2 * D.nx - q.x - (axis == 0 ? 0 : 1);
        if (axis == 0) parity = -parity;
      }
    }
    q = g.wrap_face(q);
    if (D.coastal && q.x < 0 && q.y >= 0 && q.y < D.ny && !g.wall_face(q, axis)) {
      valid = true;
      return parity * m.cs.velocity_face(g, q, axis, (float)m.c1);
    }
    if (!g.face_in_bounds(q, axis)) {
      valid = false;
      return 0.f;
    }
    // the face's solid neighbourhood, tabulated once from the static geometry (k_mac_donor_table:
    // the same tests and the same reflect_voxel_donor search)
    const int code = D.mac_dtab[g.face_local(q, axis)];
    if (code == kDonorWall) {  // a solid cell on one side only
      valid = true;
      return 0.f;
    }
    if (code == kDonorNone) {  // solid on both sides and no mirror face
      valid = false;
      return 0.f;
    }
    if (code & 1) parity = -parity;  // the mirror across a face normal to the component
    const long long f = code >> 1;
    valid = vb[f] > .5f;
    return parity * (forward ? D.fwd[f] : m.A[D.N + f]);
  }
  // The donor-table entry of in-bounds face (q, axis): kDonorWall where exactly one side is solid;
  // where both are, the reflect_voxel_donor mirror (2 f' + 1 when its parity is -1) or kDonorNone;
  // else the face itself (2 f).
  DI int donor_code(I3 q, int axis) const {
    const Grid& g = m.g;
    const bool left = g.solid(ax(q, axis, -1)), right = g.solid(q);
    if (left != right) return kDonorWall;
    if (!left) return (int)(2 * g.face_local(q, axis));
    float reflection;
    if (!reflect(q, axis, reflection)) return kDonorNone;
    return (int)(2 * g.face_local(q, axis)) + (reflection < 0.f ? 1 : 0);
  }
  // sampled_component (coupled_motion.glslinc:112-137).  Fast path: when the donor block's corner
  // lo is inside the domain and no solid cell lies in the 3x3 (x, y) window around it, every
  // donor is a plain stored face (no reflection, ghost or wall branch applies, parity 1), so the
  // donor lookups reduce to two loads each; the arithmetic is unchanged.
  // With want_value false only `valid` is produced (the value and limits are not needed): the
  // fast path then skips the eight value loads.
  // A sample point in units of the cell size, x / h per axis: the lattice coordinates of every
  // component and the solid test of the point start from the same three quotients, so a point's
  // three samples and its solid test divide once.
  DI F3 scaled(F3 x) const { return mf(x.x / m.D.hx, x.y / m.D.hy, x.z / m.D.hz); }
  template <bool FAST = false>
  DI float sample(F3 x, int axis, bool forward, bool& valid, float& lim0, float& lim1, bool want_value = true,
                  bool* fail = nullptr) const {
    return sample_s<FAST>(scaled(x), axis, forward, valid, lim0, lim1, want_value, fail);
  }
  // FAST: only the fast path is compiled in; where its precondition fails, `fail` is set and the
  // result is left undefined (the caller hands the face to the general kernel).
  template <bool FAST = false>
  DI float sample_s(F3 xs, int axis, bool forward, bool& valid, float& lim0, float& lim1, bool want_value = true,
                    bool* fail = nullptr) const {
    const Dev& D = m.D;
    F3 lattice = mf(xs.x - .5f, xs.y - .5f, xs.z - .5f);
    lattice[axis] += .5f;
    I3 lo = mk((int)floorf(lattice.x), (int)floorf(lattice.y), (int)floorf(lattice.z));
    if ((D.flags & 8) == 0 && !D.px && lo.x >= 0 && lo.y >= 0 && lo.x + 1 < D.nx + (axis == 0) &&
        lo.y + 1 < D.ny + (axis == 1) && lo.x + kSolidPad < D.tab_w && lo.y + kSolidPad < D.tab_h &&
        D.clear_tab[(lo.y + kSolidPad) * D.tab_w + lo.x + kSolidPad]) {
      F3 t = mf(fract_(lattice.x), fract_(lattice.y), fract_(lattice.z));
      lim0 = 1e20f;
      lim1 = -1e20f;
      valid = true;
      // face indices of the 2 x 2 x 2 donors: rows (y, z) of the block, z wrapped (a face at
      // z = nz is the canonical z = 0); every index fits 32 bits
      const int mx_ = D.nx + (axis == 0), my_ = D.ny + (axis == 1);
      const int base = axis == 0 ? 0 : (axis == 1 ? (int)D.NU : (int)(D.NU + D.NV));
      const int qz0 = pidx(lo.z, D.nz), qz1 = qz0 + 1 == D.nz ? 0 : qz0 + 1;
      const int r00 = base + lo.x + mx_ * (lo.y + my_ * qz0), r01 = base + lo.x + mx_ * (lo.y + my_ * qz1);
      const float* src = forward ? D.fwd : m.A + D.N;
      float values[8];
#pragma unroll
      for (int c = 0; c < 8; c++) {
        int xx = c & 1, y = (c >> 1) & 1, z = c >> 2;
        const int f = (z ? r01 : r00) + y * mx_ + xx;
        bool supported = vb[f] > .5f;
        float value = want_value ? src[f] : 0.f;
        values[c] = value;
        float wx = xx ? t.x : 1.f - t.x, wy = y ? t.y : 1.f - t.y, wz = z ? t.z : 1.f - t.z;
        if (wx * wy * wz > 0.f) {
          valid = valid && supported;
          lim0 = mnf(lim0, value);
          lim1 = mxf(lim1, value);
        }
      }
      float a = __fmaf_rn(t.x, values[1] - values[0], values[0]), b = __fmaf_rn(t.x, values[3] - values[2], values[2]);
      float d = __fmaf_rn(t.x, values[5] - values[4], values[4]), e = __fmaf_rn(t.x, values[7] - values[6], values[6]);
      float lower = __fmaf_rn(t.y, b - a, a), upper = __fmaf_rn(t.y, e - d, d);
      return __fmaf_rn(t.z, upper - lower, lower);
    }
    if constexpr (FAST) {
      *fail = true;
      valid = false;
      lim0 = lim1 = 0.f;
      return 0.f;
    } else {
      return sample_slow(xs, axis, forward, valid, lim0, lim1);
    }
  }
  __device__ __noinline__ float sample_slow(F3 xs, int axis, bool forward, bool& valid, float& lim0, float& lim1) const {
    const Grid& g = m.g;
    const Dev& D = m.D;
    F3 lattice = mf(xs.x - .5f, xs.y - .5f, xs.z - .5f);
    lattice[axis] += .5f;
    I3 lo = mk((int)floorf(lattice.x), (int)floorf(lattice.y), (int)floorf(lattice.z));
    F3 t = mf(fract_(lattice.x), fract_(lattice.y), fract_(lattice.z));
    lim0 = 1e20f;
    lim1 = -1e20f;
    valid = true;
    bool interior = (D.flags & 8) != 0 && lo.x >= 1 && lo.y >= 1 && lo.z >= 1 && lo.x + 1 < D.nx && lo.y + 1 < D.ny &&
                    lo.z + 1 < D.nz && !g.solid(mk(lo.x + 1, lo.y - 1, lo.z));
    int fnx = D.nx + (axis == 0), fny = D.ny + (axis == 1);
    float values[8];
    for (int c = 0; c < 8; c++) {
      int xx = c & 1, y = (c >> 1) & 1, z = c >> 2;
      bool supported;
      float value;
      if (interior) {
        long long base = g.face_local(lo, axis);
        long long f = base + (long long)(xx + fnx * (y + fny * z));
        supported = vb[f] > .5f;
        value = forward ? D.fwd[f] : m.A[D.N + f];
      } else
        value = donor(addI(lo, mk(xx, y, z)), axis, forward, supported);
      values[c] = value;
      float wx = xx ? t.x : 1.f - t.x, wy = y ? t.y : 1.f - t.y, wz = z ? t.z : 1.f - t.z;
      if (wx * wy * wz > 0.f) {
        valid = valid && supported;
        lim0 = mnf(lim0, value);
        lim1 = mxf(lim1, value);
      }
    }
    float a = __fmaf_rn(t.x, values[1] - values[0], values[0]), b = __fmaf_rn(t.x, values[3] - values[2], values[2]);
    float d = __fmaf_rn(t.x, values[5] - values[4], values[4]), e = __fmaf_rn(t.x, values[7] - values[6], values[6]);
    float lower = __fmaf_rn(t.y, b - a, a), upper = __fmaf_rn(t.y, e - d, d);
    return __fmaf_rn(t.z, upper - lower, lower);
  }
  DI F3 velocity(F3 x) const {
    F3 v;
    bool valid;
    float l0, l1v;
    for (int axis = 0; axis < 3; axis++) v[axis] = sample(x, axis, false, valid, l0, l1v);
    return v;
  }
  DI bool solid_at(F3 p) const { return solid_at_s(scaled(p)); }
  DI bool solid_at_s(F3 ps) const { return m.g.solid(mk((int)floorf(ps.x), (int)floorf(ps.y), (int)floorf(ps.z))); }
  DI F3 trace(F3 x, float d) const {
    F3 s = velocity(x);
    float hd = .5f * d;
    F3 mid = mf(x.x - hd * s.x, x.y - hd * s.y, x.z - hd * s.z);
    F3 s2 = velocity(mid);
    return mf(x.x - d * s2.x, x.y - d * s2.y, x.z - d * s2.z);
  }
  DI bool trace_supported(F3 x, float d) const {
    F3 s = velocity(x);
    float hd = .5f * d;
    F3 mid = mf(x.x - hd * s.x, x.y - hd * s.y, x.z - hd * s.z);
    F3 s2 = velocity(mid);
    F3 end = mf(x.x - d * s2.x, x.y - d * s2.y, x.z - d * s2.z);
    for (int stage = 0; stage < 3; stage++) {
      F3 p = stage == 0 ? x : (stage == 1 ? mid : end);
      if (solid_at(p)) return false;
      for (int axis = 0; axis < 3; axis++) {
        bool valid;
        float l0, l1v;
        sample(p, axis, false, valid, l0, l1v);
        if (!valid) return false;
      }
    }
    return true;
  }
};

// The donor table of every face (static geometry), built once at set-up.
__global__ void __launch_bounds__(NT) k_mac_donor_table(const __grid_constant__ Dev D) {
  const long long f = (long long)blockIdx.x * NT + threadIdx.x;
  if (f >= D.NF) return;
  Motion m(D);
  Mac mc(m);
  I3 q;
  int axis;
  m.g.unpack_face(f, q, axis);
  D.mac_dtab[f] = mc.donor_code(q, axis);
}

// ---------------------------------------------------------------- op 27 / op 28
// Face position of face (q, axis) in local coordinates (coupled_motion.glslinc:411).
DI F3 face_x(const Dev& D, const Grid& g, I3 q, int axis) {
  F3 x = mf(((float)q.x + .5f) * D.hx, ((float)q.y + .5f) * D.hy, ((float)q.z + .5f) * D.hz);
  x[axis] -= .5f * g.h(axis);
  return x;
}
// cached_advection, forward pass (coupled_motion.glslinc:170-179); dbg (optional) gets 16 floats.
// The nine samples (three components at x, at the midpoint and at the end point) come from one
// sampler call site in a loop that is not unrolled, so the sampler is emitted once per kernel.
template <bool FAST = false>
DI float mac_forward(const Mac& mc, F3 x, int axis, float d, long long i, float* dbg, bool* fail = nullptr) {
  const Dev& D = mc.m.D;
  const long long nf = D.NF;
  const float hd = .5f * d;
  F3 p = x, sv = mf(0.f, 0.f, 0.f), mid = x, end = x;
  F3 ps[3];  // the three points in units of the cell size
  float value = 0.f, l0 = 0.f, l1v = 0.f;
  unsigned ok = 7u;  // bit s: every sample of stage s supported
#pragma unroll 1
  for (int stage = 0; stage < 3; stage++) {
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    ps[stage] = mc.scaled(p);
#pragma unroll 1
    for (int a = 0; a < 3; a++) {
      bool valid;
      float lo, hi;
      const float s = mc.template sample_s<FAST>(ps[stage], a, false, valid, lo, hi, stage < 2 || a == axis, fail);
      if (!valid) ok &= ~(1u << stage);
      if (a == 0) v0 = s;
      else if (a == 1) v1 = s;
      else v2 = s;
      if (stage == 2 && a == axis) {
        value = s;
        l0 = lo;
        l1v = hi;
      }
    }
    if (stage == 0) {
      sv = mf(v0, v1, v2);
      mid = mf(x.x - hd * sv.x, x.y - hd * sv.y, x.z - hd * sv.z);
      p = mid;
    } else if (stage == 1) {
      end = mf(x.x - d * v0, x.y - d * v1, x.z - d * v2);
      p = end;
    }
  }
  if constexpr (FAST) {
    if (*fail) return 0.f;  // nothing written: the general kernel takes the face
  }
  const bool vs = ok & 1u, vm = ok & 2u, ve = ok & 4u;
  bool clear = !mc.solid_at_s(ps[0]) && !mc.solid_at_s(ps[1]) && !mc.solid_at_s(ps[2]);
  if (dbg) {
    float t[16] = {x.x, x.y, x.z, sv.x, sv.y, sv.z, (float)vs, mid.x, mid.y, mid.z, (float)vm, end.x, end.y, end.z, (float)ve, (float)clear};
    for (int k = 0; k < 16; k++) dbg[k] = t[k];
    return value;
  }
  D.tcache[i] = l0;
  D.tcache[nf + i] = l1v;
  D.tcache[2 * nf + i] = (vs && vm && ve && clear) ? 1.f : 0.f;
  D.tcache[3 * nf + i] = sv.x;
  D.tcache[4 * nf + i] = sv.y;
  D.tcache[5 * nf + i] = sv.z;
  return value;
}
// cached_advection, corrected pass (coupled_motion.glslinc:180-187): the reverse trace from the
// cached start velocity, six samples from one call site.
template <bool FAST = false>
DI float mac_correct(const Mac& mc, F3 x, int axis, float d, long long i, bool* fail = nullptr) {
  const Dev& D = mc.m.D;
  const long long nf = D.NF;
  const float forward = D.fwd[i];
  if (D.tcache[2 * nf + i] < .5f) return forward;
  const F3 sv = mf(D.tcache[3 * nf + i], D.tcache[4 * nf + i], D.tcache[5 * nf + i]);
  const float rd = -d;
  const float hd = .5f * rd;
  const F3 mid = mf(x.x - hd * sv.x, x.y - hd * sv.y, x.z - hd * sv.z);
  F3 p = mid, end = mid;
  F3 ps[2];  // mid and end in units of the cell size
  float backward = 0.f;
  bool ok = true;
#pragma unroll 1
  for (int stage = 0; stage < 2; stage++) {
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    ps[stage] = mc.scaled(p);
#pragma unroll 1
    for (int a = 0; a < 3; a++) {
      bool valid;
      float lo, hi;
      const float s = mc.template sample_s<FAST>(ps[stage], a, stage == 1 && a == axis, valid, lo, hi, stage == 0 || a == axis, fail);
      ok = ok && valid;
      if (a == 0) v0 = s;
      else if (a == 1) v1 = s;
      else v2 = s;
      if (stage == 1 && a == axis) backward = s;
    }
    if (stage == 0) {
      end = mf(x.x - rd * v0, x.y - rd * v1, x.z - rd * v2);
      p = end;
    }
  }
  float corrected = forward + .5f * (mc.m.A[D.N + i] - backward);
  if constexpr (FAST) {
    if (*fail) return 0.f;
  }
  return (ok && !mc.solid_at(x) && !mc.solid_at_s(ps[0]) && !mc.solid_at_s(ps[1]) && corrected >= D.tcache[i] &&
          corrected <= D.tcache[nf + i])
             ? corrected
             : forward;
}
// One advecting face of op 27 (forward pass) or op 28 (corrected pass).
template <int op, bool cached> DI void mac_face(const Dev& D, const Motion& m, const Mac& mc, long long i) {
  I3 q;
  int axis;
  m.g.unpack_face(i, q, axis);
  F3 x = face_x(D, m.g, q, axis);
  float value;
  float d = m.dt;
  if constexpr (cached) {
    if constexpr (op == 27) value = mac_forward(mc, x, axis, d, i, nullptr);
    else value = mac_correct(mc, x, axis, d, i);
  } else if constexpr (op == 27) {
    bool valid;
    float l0, l1v;
    value = mc.sample(mc.trace(x, d), axis, false, valid, l0, l1v);
  } else {
    bool valid, vf;
    float l0, l1v, d0, d1;
    float backward = mc.sample(mc.trace(x, -d), axis, true, valid, l0, l1v);
    mc.sample(mc.trace(x, d), axis, false, vf, d0, d1);
    float forward = D.fwd[i], corrected = forward + .5f * (m.A[D.N + i] - backward);
    value = (valid && vf && mc.trace_supported(x, d) && mc.trace_supported(x, -d) && corrected >= d0 && corrected <= d1)
                ? corrected
                : forward;
  }
  if constexpr (op == 27) D.fwd[i] = value;
  else m.Cb[D.N + i] = value;
}

// Work list of ops 27/28, rebuilt every trial.  The faces that advect (not wall faces; inside the
// valid band when flag 2 is set) are listed, those within three cells (x, y) of a solid cell or of
// the domain edge (the donor slow path) at the back of the list, the rest at the front; every
// warp appends its faces contiguously.  A face that does not advect gets its op 27/28 results
// (zero) here.  mac_ctr: [0] interior count, [1] boundary count, [2]/[3] op 27/28 work cursors.
__global__ void k_mac_reset(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (threadIdx.x < kMacCounters) D.mac_ctr[threadIdx.x] = 0u;
}
__global__ void __launch_bounds__(NT) k_mac_list(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  Motion m(D);
  const float* vb = m.acc == 0 ? D.vband0 : D.vband1;
  const long long i = (long long)blockIdx.x * NT + threadIdx.x;
  bool act = false, edge = false;
  if (i < D.NF) {
    I3 q;
    int axis;
    m.g.unpack_face(i, q, axis);
    act = !m.g.wall_face(q, axis) && ((D.flags & 2) == 0 || vb[i] > .5f);
    if (act) edge = D.mac_class[(axis * (D.ny + 1) + q.y) * (D.nx + 1) + q.x] != 0;
    else {
      D.fwd[i] = 0.f;
      m.Cb[D.N + i] = 0.f;
    }
  }
  const unsigned be = __ballot_sync(0xffffffffu, act && edge), bi = __ballot_sync(0xffffffffu, act && !edge);
  const int lane = threadIdx.x & 31;
  unsigned base_e = 0, base_i = 0;
  if (lane == 0) {
    if (be) base_e = atomicAdd(&D.mac_ctr[1], (unsigned)__popc(be));
    if (bi) base_i = atomicAdd(&D.mac_ctr[0], (unsigned)__popc(bi));
  }
  base_e = __shfl_sync(0xffffffffu, base_e, 0);
  base_i = __shfl_sync(0xffffffffu, base_i, 0);
  if (act) {
    const unsigned below = (unsigned)__popc((edge ? be : bi) & ((1u << lane) - 1u));
    if (edge) D.mac_list[D.NF - 1 - (long long)(base_e + below)] = (int)i;
    else D.mac_list[base_i + below] = (int)i;
  }
}
// Persistent pass over the work list: each warp takes 32 consecutive entries at a time, boundary
// faces first, so a slow warp never holds idle lanes of a finished block.  With `split`, the
// interior faces were taken by k_mac_fast and this pass covers the boundary faces and the faces
// k_mac_fast handed over (mac_ovf).
template <int op, bool cached, int MINB = 2>
__global__ void __launch_bounds__(NT, MINB) k_mac(const __grid_constant__ Dev D, int split) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  const unsigned n_edge = D.mac_ctr[1];
  const unsigned n_rest = split ? D.mac_ctr[op == 27 ? 6 : 7] : D.mac_ctr[0];
  const unsigned total = n_edge + n_rest;
  unsigned* cursor = D.mac_ctr + (op == 27 ? 2 : 3);
  const int lane = threadIdx.x & 31;
  while (true) {
    __syncwarp();
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(cursor, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const unsigned k = base + lane;
    if (k < total) {
      const long long i = k < n_edge ? (long long)D.mac_list[D.NF - 1 - (long long)k]
                                     : (long long)(split ? D.mac_ovf[k - n_edge] : D.mac_list[k - n_edge]);
      Motion m(D);  // views of the parameter block, rebuilt per face so none of it stays live
      Mac mc(m);
      mac_face<op, cached>(D, m, mc, i);
    }
  }
}
// The interior faces of the work list (no solid cell or domain edge within three cells, so every
// donor of every trace is a plain stored face) with the sampler's fast path alone: no boundary
// code in the kernel, so fewer registers and more resident warps.  A face whose trace leaves the
// fast path's region is handed over to the general pass untouched.
template <int op>
__global__ void __launch_bounds__(NT, 4) k_mac_fast(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!setup_on(D)) return;
  const unsigned total = D.mac_ctr[0];
  unsigned* cursor = D.mac_ctr + (op == 27 ? 4 : 5);
  const int lane = threadIdx.x & 31;
  while (true) {
    __syncwarp();
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(cursor, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const unsigned k = base + lane;
    if (k < total) {
      const long long i = (long long)D.mac_list[k];
      Motion m(D);
      Mac mc(m);
      I3 q;
      int axis;
      m.g.unpack_face(i, q, axis);
      const F3 x = face_x(D, m.g, q, axis);
      bool fail = false;
      if constexpr (op == 27) {
        const float value = mac_forward<true>(mc, x, axis, m.dt, i, nullptr, &fail);
        if (!fail) D.fwd[i] = value;
      } else {
        const float value = mac_correct<true>(mc, x, axis, m.dt, i, &fail);
        if (!fail) m.Cb[D.N + i] = value;
      }
      if (fail) D.mac_ovf[atomicAdd(D.mac_ctr + (op == 27 ? 6 : 7), 1u)] = (int)i;
    }
  }
}
// Debug probe: the op-27 forward trace of one face (16 floats + value).
__global__ void k_debug_face(const __grid_constant__ Dev D, long long i, float* out) {
  Motion m(D);
  Mac mc(m);
  I3 q;
  int axis;
  m.g.unpack_face(i, q, axis);
  F3 x = face_x(D, m.g, q, axis);
  out[16] = mac_forward(mc, x, axis, m.dt, i, out);
  out[17] = (float)axis;
  out[18] = (float)q.x;
  out[19] = (float)q.y;
}

// Debug probe: one sampled component with its eight donors (include/waves_debug.h).
__global__ void k_debug_sample(const __grid_constant__ Dev D, float x, float y, float z, int axis, int forward, float* out) {
  Motion m(D);
  Mac mc(m);
  bool valid;
  float l0, l1;
  F3 p = mf(x, y, z);
  out[0] = mc.sample(p, axis, forward != 0, valid, l0, l1);
  out[1] = valid;
  out[2] = l0;
  out[3] = l1;
  F3 lattice = mf(p.x / D.hx - .5f, p.y / D.hy - .5f, p.z / D.hz - .5f);
  lattice[axis] += .5f;
  out[4] = lattice.x;
  out[5] = lattice.y;
  out[6] = lattice.z;
  I3 lo = mk((int)floorf(lattice.x), (int)floorf(lattice.y), (int)floorf(lattice.z));
  for (int c = 0; c < 8; c++) {
    bool sup;
    I3 q = addI(lo, mk(c & 1, (c >> 1) & 1, c >> 2));
    out[8 + 4 * c] = mc.donor(q, axis, forward != 0, sup);
    out[9 + 4 * c] = sup;
    out[10 + 4 * c] = m.g.solid(q);
    out[11 + 4 * c] = m.g.wall_face(q, axis);
  }
}

}  // namespace

static unsigned grid_for(long long n) { return (unsigned)((n + NT - 1) / NT); }

void launch_debug_sample(const Dev& D, cudaStream_t s, const float* x, int axis, int forward, float* out) {
  if (axis < 0) k_debug_face<<<1, 1, 0, s>>>(D, (long long)x[0], out);
  else k_debug_sample<<<1, 1, 0, s>>>(D, x[0], x[1], x[2], axis, forward, out);
}

void launch_motion_cfl(const Dev& D, cudaStream_t s) {
  const unsigned wt = grid_for((long long)D.wt_w * D.wt_h);
  if (D.coastal) pdl_launch(k_wave_tables, wt, NT, 0, s, D, 0);
  pdl_launch(k_cfl, grid_for(D.N), NT, 0, s, D);
  if (D.coastal) pdl_launch(k_wave_tables, wt, NT, 0, s, D, 1);
  pdl_launch(k_compress, grid_for(D.N), NT, 0, s, D);
  const long long staged = D.NF + D.N;
  pdl_launch(k_stage_candidate, grid_for(D.N % 4 == 0 && staged % 4 == 0 ? staged / 4 : staged), NT, 0, s, D);
}
void launch_sweep(const Dev& D, cudaStream_t s) {
  pdl_launch(k_sweep_plane, grid_for(D.N), NT, 0, s, D);
  // reads F, the plane field (16 B), the sweep-axis faces and c_i; writes F
  probed(kProbeSweepVof, s, 32.0 * (double)D.N, [&] { pdl_launch(k_sweep_update, grid_for(D.N), NT, 0, s, D); });
}
int mac_blocks2() {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mac<28, true>, NT, 0) != cudaSuccess)
    return 0;
  return sms * (per_sm > 0 ? per_sm : 1);
}
int mac_blocks() {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mac<28, true, 3>, NT, 0) != cudaSuccess)
    return 0;
  return sms * (per_sm > 0 ? per_sm : 1);
}
void launch_mac_donor_table(const Dev& D, cudaStream_t s) { k_mac_donor_table<<<grid_for(D.NF), NT, 0, s>>>(D); }
void launch_maccormack(const Dev& D, cudaStream_t s) {
  pdl_launch(k_mac_reset, 1, 32, 0, s, D);
  pdl_launch(k_mac_list, grid_for(D.NF), NT, 0, s, D);
  // op 27 reads the accepted faces and valid band, writes the forward values (and, with the trace
  // cache, its six fields); op 28 reads those, the faces and the band, and writes the candidate.
  const double nf = (double)D.NF, cache = (D.flags & 4) ? 6.0 : 0.0;
  if (D.flags & 4) {
    // interior faces on the fast-path kernel, then boundary and handed-over faces
    const int split = D.mac_split ? 1 : 0;
    if (split) probed(kProbeMac, s, 4.0 * nf * (3.0 + cache), [&] { pdl_launch((k_mac_fast<27>), D.mac_fast_grid, NT, 0, s, D); });
    if (D.mac_minb == 3)
      probed(kProbeMac, s, split ? 0.0 : 4.0 * nf * (3.0 + cache), [&] { pdl_launch((k_mac<27, true, 3>), D.mac_grid, NT, 0, s, D, split); });
    else
      probed(kProbeMac, s, split ? 0.0 : 4.0 * nf * (3.0 + cache), [&] { pdl_launch((k_mac<27, true>), D.mac_grid2, NT, 0, s, D, split); });
    if (split) probed(kProbeMac, s, 4.0 * nf * (4.0 + cache), [&] { pdl_launch((k_mac_fast<28>), D.mac_fast_grid, NT, 0, s, D); });
    if (D.mac_minb == 3)
      probed(kProbeMac, s, split ? 0.0 : 4.0 * nf * (4.0 + cache), [&] { pdl_launch((k_mac<28, true, 3>), D.mac_grid, NT, 0, s, D, split); });
    else
      probed(kProbeMac, s, split ? 0.0 : 4.0 * nf * (4.0 + cache), [&] { pdl_launch((k_mac<28, true>), D.mac_grid2, NT, 0, s, D, split); });
  } else {
    probed(kProbeMac, s, 4.0 * nf * (3.0 + cache), [&] { pdl_launch((k_mac<27, false>), D.mac_grid, NT, 0, s, D, 0); });
    probed(kProbeMac, s, 4.0 * nf * (4.0 + cache), [&] { pdl_launch((k_mac<28, false>), D.mac_grid, NT, 0, s, D, 0); });
  }
}
int mac_fast_blocks() {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mac_fast<28>, NT, 0) != cudaSuccess)
    return 0;
  return sms * (per_sm > 0 ? per_sm : 1);
}

}  // namespace wg
