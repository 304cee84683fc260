// TEST INFRASTRUCTURE ONLY — pins the oracle to the reference's own shaders, op by op.
//
// The reference's GLSL compute programs, translated by oracle/glsl/translate.py and compiled
// against the host GLSL environment (glsl.hpp), run beside the FP32 oracle (wo::Solver<float>).
// For every dispatch unit of the reference's command lists -- coupled_gpu.gd:38-56 (+
// coastal_gpu.gd:26-33), the multigrid commands of pressure_multigrid.gd:121-176 and the hierarchy
// audit of pressure_hierarchy_state.gd:36-41 -- the harness
//   1. copies the oracle's whole state into the reference's buffers (bindings of
//      pressure_gpu.gd:92-117, coupled_gpu.gd:23-33, coastal_gpu.gd:9-20, pressure_multigrid.gd:
//      71-98, pressure_hierarchy_state.gd:13-26), so every unit starts from the same state;
//   2. dispatches the unit's ops through the reference's shader code;
//   3. runs the oracle's method for the same ops;
//   4. compares every buffer.  Banks, geometry, planes, masks, bands, sources, trace caches,
//      multigrid vectors, rows, transfers, audit words and the export must agree bit for bit.
//      Control-block entries written by the reference's FP32 workgroup reductions (sums) are
//      compared to the oracle's FP64 sums within a relative bound, and every decision entry
//      (accept/reject, failure codes, counters, convergence flags, dt) must agree exactly.  The
//      Galerkin products are compared within a relative bound: the reference adds them with float
//      atomics in dispatch order, the oracle in its fixed gather order.
// The oracle stays authoritative between units, so a difference of a reduction's last bits never
// carries into the next unit.  The GDScript dispatch lists are restated below with their group
// counts; the arithmetic of every op is the reference's own shader code.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../wo_solver.hpp"
#include "glsl.hpp"

#define REF_PROGRAM(ns)                \
  namespace ns {                       \
  void bind(int binding, void* ptr);   \
  void* push_constants();              \
  unsigned push_constant_bytes();      \
  void run(unsigned gx, unsigned gy);  \
  }
REF_PROGRAM(ref_coastal)
REF_PROGRAM(ref_coupled)
REF_PROGRAM(ref_mg_vectors)
REF_PROGRAM(ref_mg_build)
REF_PROGRAM(ref_mg_coarse)
REF_PROGRAM(ref_mg_arguments)
REF_PROGRAM(ref_hierarchy)

namespace {

struct Program {
  void (*bind)(int, void*);
  void* (*pc)();
  unsigned (*pcb)();
  void (*run)(unsigned, unsigned);
};
#define PROGRAM_OF(ns) Program{ns::bind, ns::push_constants, ns::push_constant_bytes, ns::run}

using glsl::uint;
typedef wo::Solver<float> Oracle;

// Control entries that are decisions, counters or maxima: equal in any precision.
bool exact_control(int k) {
  static const int ks[] = {0, 2, 3, 4, 5, 6, 7, 8, 14, 15, 16, 18, 19, 20, 21, 27, 29, 30, 31, 32, 33, 34, 36, 57, 58, 61, 88, 89, 90, 91};
  for (int e : ks)
    if (e == k) return true;
  return false;
}

struct Stat {
  long units = 0, exact = 0, within = 0, mismatched = 0;
  double max_rel = 0;
  std::string first;
};

struct Lockstep {
  Oracle o;
  bool coastal;
  Program fluid, mg_vec, mg_build, mg_coarse, mg_args, hier;
  size_t N, NF, S;
  unsigned cg, sg, fg;
  int cap, L;
  // reference buffers
  std::vector<float> a, b, work, geo, partial, c, plane, motion, history, chistory, probe, img_planes, img_kinds;
  glsl::vec4 boundary;
  glsl::Image3D planes_img, kinds_img;
  std::vector<int> meta;
  std::vector<uint> matrix, state, args;
  std::vector<float> v, rows, tcache, snap, prev;
  std::vector<size_t> node_off, mat_off, row_off, tr_off;
  size_t linv_off = 0;
  std::vector<std::vector<int>> mg_build_commands, mg_cycle_commands;
  std::map<std::string, Stat> stats;
  std::vector<std::string> order;
  std::string log;
  double rel_bound = 1e-4;

  explicit Lockstep(const waves_config& k)
      : o(k), coastal(k.coastal != 0), fluid(k.coastal ? PROGRAM_OF(ref_coastal) : PROGRAM_OF(ref_coupled)),
        mg_vec(PROGRAM_OF(ref_mg_vectors)), mg_build(PROGRAM_OF(ref_mg_build)), mg_coarse(PROGRAM_OF(ref_mg_coarse)),
        mg_args(PROGRAM_OF(ref_mg_arguments)), hier(PROGRAM_OF(ref_hierarchy)) {
    N = o.N;
    NF = o.NF;
    S = o.S;
    cg = unsigned((N + 127) / 128);
    sg = unsigned((S + 127) / 128);
    fg = unsigned((NF + 127) / 128);
    cap = std::max(k.history_capacity, 0);
    a.assign(S, 0.f);
    b.assign(S, 0.f);
    work.assign(14 * N, 0.f);
    geo.assign(2 * N, 0.f);
    partial.assign(4 * (std::max(N, NF) / 128 + 2), 0.f);
    c.assign(128, 0.f);
    plane.assign(4 * N, 0.f);
    motion.assign(4 * N + 12 * NF, 0.f);
    history.assign(16 * size_t(cap), 0.f);
    chistory.assign(20 * size_t(cap), 0.f);
    probe.assign(32, 0.f);
    img_planes.assign(4 * N, 0.f);
    img_kinds.assign(N, 0.f);
    boundary = glsl::vec4(k.right_absorption, 0, 0, 0);
    planes_img = glsl::Image3D{img_planes.data(), 4, k.n[0], k.n[1], k.n[2]};
    kinds_img = glsl::Image3D{img_kinds.data(), 1, k.n[0], k.n[1], k.n[2]};
    build_metadata();
    build_commands();
  }

  // ------------------------------------------------------------ multigrid layout
  // pressure_multigrid.gd:36-69: per level 16 ints (n, node offset, matrix offset, factors,
  // count, dense factor offset, stencil table offset, stencil size, row offset, transfer offset,
  // transfer width, aggregate), then the stencil offsets.
  void build_metadata() {
    L = o.L();
    meta.assign(16 * size_t(L), 0);
    size_t nodes = 0, mats = 0, rowc = 0, trc = 0;
    node_off.assign(L, 0);
    mat_off.assign(L, 0);
    row_off.assign(L, 0);
    tr_off.assign(L, 0);
    for (int l = 0; l < L; l++) {
      const auto& lv = o.mg.levels[l];
      int* m = &meta[16 * l];
      m[0] = lv.n.x; m[1] = lv.n.y; m[2] = lv.n.z;
      m[3] = int(nodes); m[4] = int(mats);
      m[5] = lv.f.x; m[6] = lv.f.y; m[7] = lv.f.z;
      m[8] = lv.count;
      m[15] = lv.aggregate ? 1 : 0;
      node_off[l] = nodes;
      mat_off[l] = mats;
      nodes += size_t(lv.count);
      if (l >= 1) mats += size_t(lv.count) * 125;
    }
    for (int l = 0; l < L; l++) {
      const auto& lv = o.mg.levels[l];
      int* m = &meta[16 * l];
      m[10] = int(meta.size());
      m[11] = int(lv.stencil.size());
      m[12] = int(rowc);
      m[13] = int(trc);
      m[14] = lv.aggregate ? 1 : lv.f.x * lv.f.y * lv.f.z;
      row_off[l] = rowc;
      tr_off[l] = trc;
      if (l + 1 < L) trc += size_t(lv.count) * size_t(m[14]);
      if (l > 0) rowc += size_t(lv.count) * lv.stencil.size();
      for (const auto& off : lv.stencil) {
        meta.push_back(off.x);
        meta.push_back(off.y);
        meta.push_back(off.z);
        m = &meta[16 * l];  // push_back may move the storage
      }
    }
    meta[16 * (L - 1) + 9] = int(mats);
    linv_off = mats;
    mats += size_t(o.mcount(L - 1)) * size_t(o.mcount(L - 1));
    matrix.assign(mats, 0u);
    v.assign(8 * nodes, 0.f);
    rows.assign(2 * std::max<size_t>(rowc, 1), 0.f);
    tcache.assign(2 * std::max<size_t>(trc, 1), 0.f);
    snap.assign(9 * N, 0.f);
    prev.assign(9 * N, 0.f);
    state.assign(64 + 32 * size_t(cap), 0u);
    args.assign(18 * size_t(L), 0u);
  }
  // pressure_multigrid.gd:121-135 (build) and :129-154 (cycle): [op, level, field, kind]
  void build_commands() {
    auto& B = mg_build_commands;
    B.push_back({0, 0, 0, -1});
    for (int l = 0; l < L; l++) B.push_back({1, l, 0, 3});
    B.push_back({0, 0, 0, -1});
    for (int l = 0; l + 1 < L; l++) B.push_back({16, l, 0, 4});
    B.push_back({4, 0, 0, 0});
    for (int l = 1; l < L; l++) {
      B.push_back({2, l, 0, 1});
      B.push_back({3, l - 1, 0, 2});
      B.push_back({4, l, 0, 0});
    }
    for (int l = 1; l < L; l++) B.push_back({13, l, 0, 0});
    if (o.mcount(L - 1) <= 64) B.push_back({11, L - 1, 0, 5});
    auto& C = mg_cycle_commands;
    C.push_back({0, 0, 0, -1});
    C.push_back({5, 0, 0, 0});
    int final_field = cycle(0);
    C.push_back({10, 0, final_field, 0});
  }
  int smooth(int l, int field, bool zero) {
    for (int sweep = 0; sweep < o.mg_smoothing; sweep++) {
      if (o.mg_smoother == 1) mg_cycle_commands.push_back({15, l, field + 4 * (sweep + 1), 0});
      else mg_cycle_commands.push_back({zero && sweep == 0 ? 14 : 6, l, field, 0});
      field = 3 - field;
    }
    return field;
  }
  int cycle(int l) {
    if (l == L - 1) {
      if (o.mcount(l) <= 64) {
        mg_cycle_commands.push_back({12, l, 0, -1});
        return 1;
      }
      int terminal = 1;
      for (int sweep = 0; sweep < 32; sweep++) {
        mg_cycle_commands.push_back({sweep == 0 ? 14 : 6, l, terminal, 0});
        terminal = 3 - terminal;
      }
      return terminal;
    }
    int field = smooth(l, 1, true);
    mg_cycle_commands.push_back({7, l, field, 0});
    mg_cycle_commands.push_back({8, l + 1, 0, 0});
    int coarse = cycle(l + 1);
    mg_cycle_commands.push_back({9, l, field + 4 * coarse, 0});
    return smooth(l, field, false);
  }

  // ------------------------------------------------------------ state transfer
  void to_ref() {
    a = o.bank[0];
    b = o.bank[1];
    work = o.work;
    for (size_t i = 0; i < N; i++) {
      geo[2 * i] = o.gphi[i];
      geo[2 * i + 1] = o.gkind[i];
      for (int k = 0; k < 4; k++) plane[4 * i + k] = o.plane[i][k];
    }
    for (int k = 0; k < 128; k++) c[k] = float(o.c[k]);
    float* m = motion.data();
    std::copy(o.mF.begin(), o.mF.end(), m);
    std::copy(o.mci.begin(), o.mci.end(), m + N);
    std::copy(o.flux.begin(), o.flux.end(), m + 2 * N);
    std::copy(o.fwd.begin(), o.fwd.end(), m + 2 * N + NF);
    for (int bk = 0; bk < 2; bk++) {
      for (size_t i = 0; i < NF; i++) m[2 * N + (2 + bk) * NF + i] = float(o.src[bk][i]);
      std::copy(o.vband[bk].begin(), o.vband[bk].end(), m + 2 * N + (4 + bk) * NF);
      std::copy(o.pmask[bk].begin(), o.pmask[bk].end(), m + 2 * N + 6 * NF + bk * N);
    }
    for (int f = 0; f < 6; f++) std::copy(o.tcache[f].begin(), o.tcache[f].end(), m + 4 * N + (6 + f) * NF);
    for (size_t r = 0; r < o.history.size(); r++)
      for (int k = 0; k < 4; k++) history[4 * r + k] = o.history[r][k];
    for (size_t r = 0; r < o.chistory.size(); r++)
      for (int k = 0; k < 4; k++) chistory[4 * r + k] = o.chistory[r][k];
    for (int r = 0; r < 8; r++)
      for (int k = 0; k < 4; k++) probe[4 * r + k] = o.probe[r][k];
    if (o.exp_plane.size() == N)
      for (size_t i = 0; i < N; i++) {
        for (int k = 0; k < 4; k++) img_planes[4 * i + k] = o.exp_plane[i][k];
        img_kinds[i] = o.exp_kind[i];
      }
    for (int l = 0; l < L; l++) {
      const size_t cnt = size_t(o.mcount(l));
      std::copy(o.mg.v[l].begin(), o.mg.v[l].end(), v.begin() + 8 * node_off[l]);
      if (l >= 1) {
        for (size_t e = 0; e < cnt * 125; e++) matrix[mat_off[l] + e] = glsl::floatBitsToUint(o.mg.matrix[l][e]);
        const size_t w = o.mg.levels[l].stencil.size();
        for (size_t e = 0; e < w * cnt; e++) {
          rows[2 * (row_off[l] + e)] = o.mg.ellv[l][e];
          rows[2 * (row_off[l] + e) + 1] = glsl::intBitsToFloat(o.mg.ellc[l][e]);
        }
      }
      if (l + 1 < L) {
        const size_t w = size_t(o.mg.levels[l].twidth);
        for (size_t e = 0; e < w * cnt; e++) {
          tcache[2 * (tr_off[l] + e)] = glsl::intBitsToFloat(o.mg.tid[l][e]);
          tcache[2 * (tr_off[l] + e) + 1] = o.mg.tw[l][e];
        }
      }
    }
    for (size_t e = 0; e < o.mg.linv.size(); e++) matrix[linv_off + e] = glsl::floatBitsToUint(o.mg.linv[e]);
    snap = o.mg.snapshot;
    prev = o.mg.previous;
    state = o.mg.state;
  }

  // ------------------------------------------------------------ comparison
  bool reduction_unit = false, galerkin_unit = false;
  std::string unit_name;
  Stat* cur = nullptr;
  bool unit_bad = false, unit_tol = false;

  void mismatch(const std::string& what) {
    unit_bad = true;
    if (cur->first.empty()) cur->first = what;
    if (log.size() < 20000) log += unit_name + ": " + what + "\n";
  }
  template <class T> void same(const char* name, const T* ref, const T* ora, size_t n) {
    for (size_t i = 0; i < n; i++) {
      if (std::memcmp(&ref[i], &ora[i], sizeof(T)) != 0) {
        char buf[256];
        std::snprintf(buf, sizeof buf, "%s[%zu]: reference %.9g oracle %.9g (%zu of %zu differ from here)", name, i,
                      double(ref[i]), double(ora[i]), count_diff(ref + i, ora + i, n - i), n);
        mismatch(buf);
        return;
      }
    }
  }
  template <class T> static size_t count_diff(const T* x, const T* y, size_t n) {
    size_t k = 0;
    for (size_t i = 0; i < n; i++) k += std::memcmp(&x[i], &y[i], sizeof(T)) != 0;
    return k;
  }
  void close(const char* name, int k, double ref, double ora) { close_scaled(name, k, ref, ora, std::fabs(ora)); }
  void close_scaled(const char* name, int k, double ref, double ora, double scale) {
    if (float(ref) == float(ora)) return;
    double rel = std::fabs(ref - ora) / std::max(scale, 1e-30);
    if (std::fabs(ref - ora) <= 1e-12) rel = 0;
    cur->max_rel = std::max(cur->max_rel, rel);
    unit_tol = true;
    if (rel > rel_bound) {
      char buf[256];
      std::snprintf(buf, sizeof buf, "%s[%d]: reference %.9g oracle %.9g (relative %.3g)", name, k, ref, ora, rel);
      mismatch(buf);
    }
  }
  void compare() {
    // oracle state after the unit, in the reference layout
    Lockstep& s = *this;
    std::vector<float> ta = a, tb = b, twork = work, tgeo = geo, tplane = plane, tmotion = motion, thist = history,
                       tch = chistory, tprobe = probe, tip = img_planes, tik = img_kinds, tv = v, trows = rows,
                       ttc = tcache, tsnap = snap, tprev = prev, tc = c;
    std::vector<uint> tmatrix = matrix, tstate = state;
    s.to_ref();
    // now (a, b, ...) hold the oracle's state, (ta, tb, ...) the reference's
    same("bank0", ta.data(), a.data(), S);
    same("bank1", tb.data(), b.data(), S);
    same("work", twork.data(), work.data(), work.size());
    same("geo", tgeo.data(), geo.data(), geo.size());
    same("geometry_plane", tplane.data(), plane.data(), plane.size());
    same("motion", tmotion.data(), motion.data(), motion.size());
    same("probe", tprobe.data(), probe.data(), probe.size());
    same("planes", tip.data(), img_planes.data(), img_planes.size());
    same("kinds", tik.data(), img_kinds.data(), img_kinds.size());
    same("mg_vectors", tv.data(), v.data(), v.size());
    same("mg_rows", trows.data(), rows.data(), rows.size());
    same("mg_transfers", ttc.data(), tcache.data(), tcache.size());
    same("mg_snapshot", tsnap.data(), snap.data(), snap.size());
    same("mg_previous", tprev.data(), prev.data(), prev.size());
    same("mg_audit", tstate.data(), state.data(), state.size());
    same("coastal_history", tch.data(), chistory.data(), chistory.size());
    if (reduction_unit) {  // per-trial sweep rows hold FP32 workgroup sums
      for (size_t i = 0; i < history.size(); i++)
        if (std::memcmp(&thist[i], &history[i], 4) != 0) close("history", int(i), thist[i], history[i]);
    } else {
      same("history", thist.data(), history.data(), history.size());
    }
    if (galerkin_unit) {
      // relative to the row's diagonal: the entries are sums of terms of either sign, and float
      // additions in another order differ by rounding of the terms, not of the sum
      for (int l = 1; l < L; l++)
        for (size_t e = mat_off[l]; e < mat_off[l] + size_t(o.mcount(l)) * 125; e++) {
          if (tmatrix[e] == matrix[e]) continue;
          const size_t row = mat_off[l] + ((e - mat_off[l]) / 125) * 125;
          const double diag = std::fabs(glsl::uintBitsToFloat(matrix[row + 62]));
          const double ref = glsl::uintBitsToFloat(tmatrix[e]), ora = glsl::uintBitsToFloat(matrix[e]);
          close_scaled("mg_matrix", int(e), ref, ora, std::max(std::fabs(ora), diag));
        }
      same("mg_matrix dense factor", tmatrix.data() + linv_off, matrix.data() + linv_off, matrix.size() - linv_off);
    } else {
      same("mg_matrix", tmatrix.data(), matrix.data(), matrix.size());
    }
    for (int k = 0; k < 96; k++) {  // the reference's control block (slots from 96 are the build's own)
      const double ref = tc[k], ora = o.c[k];
      if (float(ora) == tc[k]) continue;
      if (exact_control(k) || !reduction_unit) {
        char buf[256];
        std::snprintf(buf, sizeof buf, "c[%d]: reference %.9g oracle %.17g", k, ref, ora);
        mismatch(buf);
      } else {
        // volume-ledger entries are differences of volume sums: their rounding is that of the
        // liquid volume, so they are bounded relative to it
        const bool ledger = k == 17 || (k >= 22 && k <= 28) || (k >= 35 && k <= 40) || (k >= 64 && k <= 77);
        const double scale = ledger ? std::max(std::fabs(ora), std::max(std::fabs(o.c[26]), std::fabs(o.c[17]))) : std::fabs(ora);
        close_scaled("c", k, ref, ora, scale);
      }
    }
  }

  // ------------------------------------------------------------ dispatch
  void bind_fluid() {
    Program& p = fluid;
    p.bind(0, a.data());
    p.bind(1, b.data());
    p.bind(2, work.data());
    p.bind(3, geo.data());
    p.bind(4, partial.data());
    p.bind(5, c.data());
    p.bind(6, &planes_img);
    p.bind(7, &kinds_img);
    p.bind(8, plane.data());
    p.bind(9, motion.data());
    p.bind(10, history.data());
    if (coastal) {
      p.bind(11, &boundary);
      p.bind(12, probe.data());
      p.bind(13, chistory.data());
    }
  }
  // pressure_gpu.gd:67-68, coupled_gpu.gd:16-22, coastal_gpu.gd:21-25
  void fluid_params(int op) {
    float* pc = static_cast<float*>(fluid.pc());
    const waves_config& k = cfg;
    float v32[32] = {float(k.n[0]), float(k.n[1]), float(k.n[2]), float(op), k.spacing[0], k.spacing[1], k.spacing[2], k.dt,
                     k.origin[0], k.origin[1], k.origin[2], k.eta, float(k.periodic_x ? 1 : 0), k.slope, k.corrugation, float(o.quota),
                     float(k.shape), k.gravity, float(k.max_face_cfl ? 1 : 0), float(k.history_capacity),
                     k.wave[0], k.wave[1], k.wave[2], k.wave[3],
                     k.pressure_tolerance, float(k.linear_air ? 1 : 0), float(k.stokes_second ? 1 : 0),
                     float((k.height_normals ? 1 : 0) + (k.active_advection ? 2 : 0) + (k.transport_cache ? 4 : 0) + (k.transport_interior ? 8 : 0)),
                     k.origin[0], k.zone_length, k.damping_rate, k.ramp_periods};
    std::memcpy(pc, v32, fluid.pcb());
  }
  waves_config cfg;
  void fluid_op(int op, unsigned groups) {
    bind_fluid();
    fluid_params(op);
    fluid.run(groups, 1);
  }
  void bind_mg(Program& p, int selected) {
    if (selected == 0) {  // the argument producer: control, levels, arguments, audit
      p.bind(0, c.data());
      p.bind(1, meta.data());
      p.bind(2, args.data());
      p.bind(3, state.data());
      return;
    }
    p.bind(0, work.data());
    p.bind(1, geo.data());
    p.bind(2, c.data());
    p.bind(3, meta.data());
    p.bind(4, matrix.data());
    p.bind(5, v.data());
    p.bind(7, partial.data());
    p.bind(8, rows.data());
    p.bind(9, snap.data());
    p.bind(10, tcache.data());
    p.bind(11, state.data());
  }
  // pressure_multigrid.gd:155-176: one command through its pipeline, indirect groups from the
  // argument buffer (kind >= 0) or one group.
  void mg_command(const std::vector<int>& cmd, int phase) {
    const int op = cmd[0], l = cmd[1], field = cmd[2], kind = cmd[3];
    const bool build = phase == 2;
    const int selected = op == 0 ? 0 : ((op == 11 || op == 12) ? 3 : (build ? 1 : 2));
    Program& p = selected == 0 ? mg_args : (selected == 3 ? mg_coarse : (selected == 1 ? mg_build : mg_vec));
    bind_mg(p, selected);
    int* pc = static_cast<int*>(p.pc());
    int payload[8] = {op, l, phase, field, L, cfg.periodic_x ? 1 : 0, o.mg_smoothing, 1};
    std::memcpy(pc, payload, p.pcb());
    unsigned gx = 1, gy = 1;
    if (kind >= 0) {
      gx = args[18 * l + 3 * kind];
      gy = args[18 * l + 3 * kind + 1];
    }
    if (gx > 0 && gy > 0) p.run(gx, gy);
  }
  // pressure_hierarchy_state.gd:36-41
  void hierarchy_op(int op) {
    hier.bind(0, work.data());
    hier.bind(1, geo.data());
    hier.bind(2, c.data());
    hier.bind(3, snap.data());
    hier.bind(4, prev.data());
    hier.bind(5, state.data());
    int payload[8] = {cfg.n[0], cfg.n[1], cfg.n[2], op, cfg.periodic_x ? 1 : 0, cfg.mg_maintenance, cfg.mg_lag, cfg.history_capacity};
    std::memcpy(hier.pc(), payload, hier.pcb());
    hier.run((op == 1 || op == 3) ? cg : 1u, 1);
  }

  // ------------------------------------------------------------ units
  // false: the reference runs on its own state (its FP32 control block and workgroup sums) and
  // the oracle is not stepped
  bool sync = true;

  template <class RefFn, class OracleFn>
  void unit(const std::string& name, bool reduction, RefFn ref_fn, OracleFn oracle_fn, bool galerkin = false) {
    if (!sync) {
      ref_fn();
      return;
    }
    if (!stats.count(name)) order.push_back(name);
    cur = &stats[name];
    unit_name = name;
    reduction_unit = reduction;
    galerkin_unit = galerkin;
    unit_bad = unit_tol = false;
    to_ref();
    ref_fn();
    oracle_fn();
    compare();
    cur->units++;
    if (unit_bad) cur->mismatched++;
    else if (unit_tol) cur->within++;
    else cur->exact++;
  }
  void op(int k, unsigned groups, void (Oracle::*m)()) {
    unit("op " + std::to_string(k), false, [&] { fluid_op(k, groups); }, [&] { (o.*m)(); });
  }
  void pair(int k1, unsigned g1, int k2, void (Oracle::*m)()) {
    unit("ops " + std::to_string(k1) + "+" + std::to_string(k2), true, [&] { fluid_op(k1, g1); fluid_op(k2, 1); },
         [&] { (o.*m)(); });
  }

  void initial_commands() {
    unit("op 0", false, [&] { fluid_op(0, sg); }, [&] { o.op0(); });
    unit("op 40", false, [&] { fluid_op(40, sg); }, [&] { o.op40(); });
    op(17, cg, &Oracle::op17);
    op(18, cg, &Oracle::op18);
    op(16, cg, &Oracle::op16);
    op(19, cg, &Oracle::op19);
    pair(41, cg, 42, &Oracle::op41_42);
    unit("op 49", false, [&] { fluid_op(49, sg); }, [&] { o.op48_49(true); });
    if (coastal) {
      op(85, 1, &Oracle::op85);
      op(86, 1, &Oracle::op86);
    }
  }

  void mg_build_unit() {
    if (!sync) {
      for (int k = 0; k < 4; k++) hierarchy_op(k);
      for (const auto& cmd : mg_build_commands) mg_command(args_for(cmd, 2), 2);
      hierarchy_op(4);
      return;
    }
    unit("hierarchy ops 0-3", false, [&] { for (int k = 0; k < 4; k++) hierarchy_op(k); }, [&] { o.hs_ops0_3(); });
    const auto& s = o.mg.state;
    for (size_t ci = 0; ci < mg_build_commands.size(); ci++) {
      const auto& cmd = mg_build_commands[ci];
      const int op = cmd[0], l = cmd[1];
      if (op == 0) {
        mg_command(cmd, 2);  // argument producer: no oracle counterpart (its gating is inline)
        continue;
      }
      if (op == 2) {  // zeroing + scatter (ops 2 and 3) against the oracle's gather
        const auto next = mg_build_commands[ci + 1];
        unit("mg build ops 2+3 (Galerkin)", false,
             [&] {
               mg_command(args_for(cmd, 2), 2);
               mg_command(args_for(next, 2), 2);
             },
             [&] {
               if (o.build_enabled() && s[8] != 0) o.mg_galerkin(l - 1);
             },
             true);
        ci++;
        continue;
      }
      std::string name = "mg build op " + std::to_string(op);
      unit(name, false, [&] { mg_command(args_for(cmd, 2), 2); }, [&] {
        if (!o.build_enabled()) return;
        if (op == 1 && s[9] != 0) o.mg_op1(l);
        if (op == 16 && (s[14] == 0 || s[20 + l + 1] != 0)) o.mg_op16(l);
        if (op == 4 && s[8] != 0) o.mg_op4(l);
        if (op == 13 && s[8] != 0) o.mg_op13(l);
        if (op == 11 && s[8] != 0) o.mg_op11(l);
      });
    }
    unit("hierarchy op 4", false, [&] { hierarchy_op(4); }, [&] { o.hs_op4(); });
  }
  // the argument producer runs before the command (its output is the group count)
  std::vector<int> args_for(const std::vector<int>& cmd, int phase) {
    if (cmd[3] >= 0) {
      to_ref_args(phase);
    }
    return cmd;
  }
  void to_ref_args(int phase) {
    std::vector<int> produce = {0, 0, 0, -1};
    mg_command(produce, phase);
  }

  // One V-cycle (phase 0 before op 4, phase 1 before op 9), command by command.
  void mg_cycle_units(int phase) {
    if (!sync) {
      for (const auto& cmd : mg_cycle_commands) mg_command(args_for(cmd, phase), phase);
      return;
    }
    if (!o.mg_cycle_on(phase)) {
      // every command of the cycle is gated off: run them on the reference and expect no change
      unit("mg cycle (gated off)", false, [&] { for (const auto& cmd : mg_cycle_commands) mg_command(args_for(cmd, phase), phase); }, [] {});
      return;
    }
    int final_field = 1;
    for (const auto& cmd : mg_cycle_commands) {
      const int op = cmd[0], l = cmd[1], field = cmd[2];
      if (op == 0) continue;
      std::string name = "mg cycle op " + std::to_string(op);
      unit(name, false, [&] { mg_command(args_for(cmd, phase), phase); }, [&] {
        switch (op) {
          case 5: o.mg_op5(); break;
          case 15: o.mg_op15(l, field % 4, field / 4); break;
          case 14: o.mg_op14(l); break;
          case 6: o.mg_op6(l, field); break;
          case 7: o.mg_op7(l, field); break;
          case 8: o.mg_op8(l); break;
          case 9: o.mg_op9(l, field % 4, field / 4); break;
          case 12: o.mg_op12(l); break;
          case 10: final_field = field; o.mg_op10(phase, field); break;
        }
      });
    }
    (void)final_field;
  }

  // coupled_gpu.gd:38-56 (+ coastal_gpu.gd:28-33), with the multigrid injected before ops 4 and 9
  // (pressure_gpu.gd:70-74)
  void batch() {
    op(43, 1, &Oracle::op43);
    op(1, 1, &Oracle::op1);
    pair(20, cg, 21, &Oracle::op20_21);
    pair(45, cg, 46, &Oracle::op45_46);
    op(22, sg, &Oracle::op22);
    for (int axis = 0; axis < 3; axis++) {
      op(23, cg, &Oracle::op23);
      op(24, fg, &Oracle::op24);
      pair(55, cg, 56, &Oracle::op55_56);
      pair(25, cg, 26, &Oracle::op25_26);
    }
    unit("op 27", false, [&] { fluid_op(27, fg); }, [&] { o.op27_28(27); });
    unit("op 28", false, [&] { fluid_op(28, fg); }, [&] { o.op27_28(28); });
    if (coastal) {
      pair(80, cg, 81, &Oracle::op80_81);
      op(82, fg, &Oracle::op82);
      pair(83, cg, 84, &Oracle::op83_84);
      pair(87, cg, 88, &Oracle::op87_88);
    }
    op(17, cg, &Oracle::op17);
    op(18, cg, &Oracle::op18);
    op(16, cg, &Oracle::op16);
    op(2, sg, &Oracle::op2);
    op(47, fg, &Oracle::op47);
    op(63, 1, &Oracle::op63);
    op(64, cg, &Oracle::op64);
    mg_build_unit();
    unit("op 3", false, [&] { fluid_op(3, cg); }, [&] { o.op3(); });
    mg_cycle_units(0);
    unit("op 4", true, [&] { fluid_op(4, 1); }, [&] { o.op4(); });
    for (int it = 0; it < o.iters_per_batch; it++) {
      op(5, cg, &Oracle::op5);
      pair(6, cg, 7, &Oracle::op6_7);
      unit("op 8", false, [&] { fluid_op(8, cg); }, [&] { o.op8(); });
      mg_cycle_units(1);
      unit("op 9", true, [&] { fluid_op(9, 1); }, [&] { o.op9(); });
      op(10, cg, &Oracle::op10);
    }
    op(11, sg, &Oracle::op11);
    op(65, cg, &Oracle::op65);
    op(47, fg, &Oracle::op47);
    op(30, fg, &Oracle::op30);
    unit("op 31", false, [&] { fluid_op(31, fg); }, [&] { o.op31_33(31); });
    unit("op 32", false, [&] { fluid_op(32, fg); }, [&] { o.op31_33(32); });
    unit("op 33", false, [&] { fluid_op(33, fg); }, [&] { o.op31_33(33); });
    op(34, fg, &Oracle::op34);
    op(47, fg, &Oracle::op47);
    unit("op 48", false, [&] { fluid_op(48, fg); }, [&] { o.op48_49(false); });
    pair(35, cg, 36, &Oracle::op35_36);
    pair(62, cg, 66, &Oracle::op62_66);
    pair(12, cg, 13, &Oracle::op12_13);
    op(44, 1, &Oracle::op44);
    op(19, cg, &Oracle::op19);
    if (coastal) {
      op(85, 1, &Oracle::op85);
      op(89, 1, &Oracle::op89);
    }
  }
};

}  // namespace

extern "C" {

void* ref_create(const waves_config* cfg) {
  Lockstep* s = new Lockstep(*cfg);
  s->cfg = *cfg;
  s->initial_commands();
  return s;
}
void ref_destroy(void* h) { delete static_cast<Lockstep*>(h); }
void ref_set_quota(void* h, double quota) { static_cast<Lockstep*>(h)->o.quota = quota; }
// Batches in lockstep until the oracle's run loop would stop; returns the batches run.
int ref_run(void* h, int max_batches) {
  Lockstep* s = static_cast<Lockstep*>(h);
  Oracle& o = s->o;
  int b = 0;
  for (; b < max_batches; b++) {
    if (o.c[7] > .5 && !(o.c[7] == 20 || (o.c[7] >= 10 && o.c[7] <= 12))) break;
    if (o.c[7] > .5 && o.c[29] >= 2) break;
    if (o.quota_met() && o.c[4] < .5 && o.c[7] < .5) break;
    s->batch();
  }
  return b;
}
// The reference alone, on its own state from its own initial commands (its FP32 control block,
// its workgroup sums in dispatch order): the run the reference's shaders make by themselves.
void* ref_free_create(const waves_config* cfg) {
  Lockstep* s = new Lockstep(*cfg);
  s->cfg = *cfg;
  s->sync = false;
  s->initial_commands();
  return s;
}
// Batches of the reference alone until its own control block shows the quota met with no trial
// pending, or a halt (the stopping rule of work_scheduler.gd:43-46 on the reference's telemetry).
int ref_free_run(void* h, double quota, int max_batches) {
  Lockstep* s = static_cast<Lockstep*>(h);
  s->o.quota = quota;
  int b = 0;
  for (; b < max_batches; b++) {
    const float* c = s->c.data();
    const bool recoverable = (c[7] == 20 || (c[7] >= 10 && c[7] <= 12)) && c[29] < 2;
    if (c[7] > .5f && !recoverable) break;
    const bool met = quota >= 0 ? c[2] >= float(quota) : c[1] >= float(-quota);
    if (met && c[4] < .5f && c[7] < .5f) break;
    s->batch();
  }
  return b;
}
void ref_free_control(void* h, float* out) {
  Lockstep* s = static_cast<Lockstep*>(h);
  for (int k = 0; k < 96; k++) out[k] = s->c[k];
}
void ref_free_bank(void* h, int which, float* out) {
  Lockstep* s = static_cast<Lockstep*>(h);
  const std::vector<float>& b = which == 0 ? s->a : s->b;
  std::copy(b.begin(), b.end(), out);
}
void ref_get_control(void* h, double* out) {
  Lockstep* s = static_cast<Lockstep*>(h);
  for (int k = 0; k < WAVES_CONTROL_SIZE; k++) out[k] = s->o.c[k];
}
// Per unit kind: units run, bit-exact units, units within the bounds, mismatched units, the
// largest relative difference of a bounded entry, and the first mismatch.
int ref_report(void* h, char* buf, int cap) {
  Lockstep* s = static_cast<Lockstep*>(h);
  std::string r;
  long bad = 0;
  for (const auto& name : s->order) {
    const Stat& st = s->stats[name];
    char line[512];
    std::snprintf(line, sizeof line, "%-30s units %6ld  exact %6ld  within %6ld  mismatched %4ld  max_rel %.3g%s%s\n", name.c_str(),
                  st.units, st.exact, st.within, st.mismatched, st.max_rel, st.first.empty() ? "" : "  first: ", st.first.c_str());
    r += line;
    bad += st.mismatched;
  }
  if (buf && cap > 0) {
    std::snprintf(buf, size_t(cap), "%s", r.c_str());
  }
  return int(bad);
}
// Totals over every unit: [units, exact, within, mismatched].
void ref_totals(void* h, long* out) {
  Lockstep* s = static_cast<Lockstep*>(h);
  out[0] = out[1] = out[2] = out[3] = 0;
  for (const auto& kv : s->stats) {
    out[0] += kv.second.units;
    out[1] += kv.second.exact;
    out[2] += kv.second.within;
    out[3] += kv.second.mismatched;
  }
}

}  // extern "C"
