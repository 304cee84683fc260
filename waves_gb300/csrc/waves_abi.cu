// C ABI of the GB300-native waves solver step (include/waves.h).
//
// One handle owns one simulation on one device.  A solver trial (the reference's
// coupled_gpu.gd:_record_commands + coastal_gpu.gd additions, with the multigrid injected as in
// pressure_gpu.gd:70-74) is either
//   * captured once into a CUDA graph whose control flow is device-driven: an IF node on "trial
//     begun" (op 1), a WHILE node over defect-correction rounds (op 13 -> op 63) and, inside it, a
//     WHILE node over CG iterations (op 9) — the reference's per-kernel early-exit flags become
//     graph conditionals set by the kernels that decide them; or
//   * run from the host, reading the control block between phases (the debugging path).
// Both paths enqueue the same kernels; results are identical.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <chrono>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/waves.h"
#include "../../include/waves_debug.h"
#include "dev.h"
#include "kernels.h"

using wg::Dev;

namespace wg {
thread_local std::vector<ProbeRec>* g_probe = nullptr;
bool g_pdl = true;
}

namespace {

thread_local std::string g_create_error;

struct Alloc {
  void* ptr;
  size_t bytes;
  bool persistent;  // part of a checkpoint
  const char* name;
};

struct HLevel {
  int n[3];
  int count;
  int f[3];
  bool aggregate;
  std::vector<int> stencil;  // 3 ints per offset
};

}  // namespace

struct waves_handle {
  waves_config cfg;
  cudaStream_t stream = nullptr;
  Dev D;
  std::vector<Alloc> allocs;
  std::vector<HLevel> levels;
  std::vector<int> stencil_tab;
  float4* probes = nullptr;
  float4* export_planes = nullptr;
  float* export_kinds = nullptr;
  float4* render_buf = nullptr;  // waves_render: image and trace
  size_t render_px = 0;
  double* host_c = nullptr;  // pinned
  double* host_quota = nullptr;  // pinned
  std::atomic<double> quota{0.0};
  cudaGraph_t graph = nullptr, graph_p = nullptr;
  cudaGraphExec_t exec = nullptr, exec_p = nullptr;  // motion part, pressure part
  bool graph_mode = true;
  std::string err;
  // device timing of submitted trials: events (before motion, between, after pressure)
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::array<cudaEvent_t, 3>> ev_pending;
  double motion_ms = 0, pressure_ms = 0;
  int64_t timed_trials = 0;
  // kernels per phase: begin, setup-motion, setup-pressure, cg round set-up, cg iteration, post, end
  int32_t launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // frame-budgeted submission (waves_frame): running trial cost, unfinished submissions, each with
  // its pinned control-block copy
  struct Submission {
    cudaEvent_t done;
    int slot;
    int trials;
  };
  static constexpr int kFrameSlots = 8;
  double trial_cost_ms = 0;
  double gpu_ms_total = 0;
  std::vector<Submission> inflight;
  double* frame_c = nullptr;  // pinned, kFrameSlots x WAVES_CONTROL_SIZE
  double last_c[WAVES_CONTROL_SIZE] = {};
  bool have_last = false;
  int64_t last_mg_builds = 0, last_mg_structure_builds = 0;  // hierarchy counters of the last waves_stats
  int64_t serial = 0, retired = 0;
};

namespace {

#define CK(expr)                                                          \
  do {                                                                    \
    cudaError_t e_ = (expr);                                              \
    if (e_ != cudaSuccess) {                                              \
      h->err = std::string(#expr) + ": " + cudaGetErrorString(e_);        \
      return WAVES_CUDA_ERROR;                                            \
    }                                                                     \
  } while (0)

waves_status alloc(waves_handle* h, void** p, size_t bytes, bool persistent, const char* name) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    h->err = std::string("cudaMalloc ") + name + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? WAVES_OUT_OF_MEMORY : WAVES_CUDA_ERROR;
  }
  h->allocs.push_back({*p, bytes, persistent, name});
  return cudaMemsetAsync(*p, 0, bytes, h->stream) == cudaSuccess ? WAVES_OK : WAVES_CUDA_ERROR;
}
template <class T> waves_status alloc_t(waves_handle* h, T** p, size_t count, bool persistent, const char* name) {
  return alloc(h, (void**)p, count * sizeof(T), persistent, name);
}

// Level plan of pressure_multigrid.gd:37-69 with _basis/_coarse_stencil (:181-198).
std::vector<int> basis(const int q[3], const int f[3], bool aggregate) {
  auto fl = [](double a) { return (int)std::floor(a); };
  std::vector<int> out;
  if (aggregate) {
    out = {fl(double(q[0]) / f[0]), fl(double(q[1]) / f[1]), fl(double(q[2]) / f[2])};
    return out;
  }
  int base[3];
  for (int a = 0; a < 3; a++) base[a] = fl((q[a] + .5) / f[a] - .5);
  for (int z = 0; z < f[2]; z++)
    for (int y = 0; y < f[1]; y++)
      for (int x = 0; x < f[0]; x++) {
        out.push_back(base[0] + x);
        out.push_back(base[1] + y);
        out.push_back(base[2] + z);
      }
  return out;
}
std::vector<int> coarse_stencil(const std::vector<int>& st, const int f[3], bool aggregate) {
  std::vector<int> result;
  for (int z = 0; z < f[2]; z++)
    for (int y = 0; y < f[1]; y++)
      for (int x = 0; x < f[0]; x++) {
        int q[3] = {x, y, z};
        std::vector<int> left = basis(q, f, aggregate);
        for (size_t o = 0; o < st.size(); o += 3)
          for (size_t a = 0; a < left.size(); a += 3) {
            int qo[3] = {q[0] + st[o], q[1] + st[o + 1], q[2] + st[o + 2]};
            std::vector<int> right = basis(qo, f, aggregate);
            for (size_t b = 0; b < right.size(); b += 3) {
              int d[3] = {right[b] - left[a], right[b + 1] - left[a + 1], right[b + 2] - left[a + 2]};
              bool seen = false;
              for (size_t r = 0; r < result.size(); r += 3)
                if (result[r] == d[0] && result[r + 1] == d[1] && result[r + 2] == d[2]) { seen = true; break; }
              if (!seen) result.insert(result.end(), d, d + 3);
            }
          }
      }
  return result;
}
void plan_levels_of(const waves_config& k, std::vector<HLevel>& levels) {
  int n[3] = {k.n[0], k.n[1], k.n[2]};
  double hh[3] = {double(k.spacing[0]), double(k.spacing[1]), double(k.spacing[2])};
  std::vector<int> st = {0, 0, 0, -1, 0, 0, 1, 0, 0, 0, -1, 0, 0, 1, 0, 0, 0, -1, 0, 0, 1};
  levels.clear();
  while (true) {
    int count = n[0] * n[1] * n[2];
    int f[3] = {1, 1, 1};
    if (count > 64) {
      double smallest = INFINITY;
      for (int a = 0; a < 3; a++)
        if (n[a] > 2) smallest = std::min(smallest, hh[a]);
      for (int a = 0; a < 3; a++)
        if (n[a] > 2 && hh[a] < 1.8 * smallest) f[a] = 2;
      if (k.periodic_x && n[0] % 2) f[0] = 1;
      if (n[2] % 2) f[2] = 1;
    }
    HLevel lv;
    std::memcpy(lv.n, n, sizeof(n));
    lv.count = count;
    std::memcpy(lv.f, f, sizeof(f));
    lv.aggregate = int(levels.size()) >= k.mg_aggregate_from;
    lv.stencil = st;
    levels.push_back(lv);
    if (count <= 64 || (f[0] == 1 && f[1] == 1 && f[2] == 1)) break;
    st = coarse_stencil(st, f, lv.aggregate);
    for (int a = 0; a < 3; a++) {
      n[a] = (n[a] + f[a] - 1) / f[a];
      hh[a] *= f[a];
    }
  }
}
void plan_levels(waves_handle* h) { plan_levels_of(h->cfg, h->levels); }

// solid() of pressure_core.glslinc:87-96 over (x, y) with a margin (z-independent geometry).
bool solid_host(const waves_config& k, int x, int y) {
  if (k.periodic_x) x = x >= 0 ? x % k.n[0] : k.n[0] - 1 - ((-1 - x) % k.n[0]);
  if (y < 0 || x >= k.n[0]) return true;
  if (!k.coastal && x < 0) return true;
  if (y >= k.n[1]) return false;
  if (k.slope > 0.f) {
    float cx = k.origin[0] + ((float)x + 0.5f) * k.spacing[0];
    float cy = k.origin[1] + ((float)y + 0.5f) * k.spacing[1];
    float m = cx - 1.5f;
    float bed = -0.45f + ((0.f < m) ? m : 0.f) / k.slope;
    return cy <= bed;
  }
  return false;
}

// Columns [0, zone_x_end) contain every cell and face with a nonzero relaxation rate
// (coastal_target.glslinc:28-33).
int coastal_zone_end(const waves_config& k) {
  if (!k.coastal) return 0;
  if (k.shape == 6) return k.n[0];
  auto ramp = [](float q) {
    q = q < 0.f ? 0.f : (q > 1.f ? 1.f : q);
    return q * q * q * (10.f + q * (-15.f + 6.f * q));
  };
  int last = 0;
  for (int x = 0; x <= k.n[0]; x++) {
    float cx = k.origin[0] + ((float)x + 0.5f) * k.spacing[0];
    float fx = cx - .5f * k.spacing[0];
    float rc = k.damping_rate * (1.f - ramp((cx - k.origin[0]) / k.zone_length));
    float rf = k.damping_rate * (1.f - ramp((fx - k.origin[0]) / k.zone_length));
    bool off = cx < k.origin[0] + k.zone_length || fx < k.origin[0] + k.zone_length;
    if (rc > 0.f || rf > 0.f || off) last = x + 1;
  }
  return std::min(k.n[0], last + 2);
}

waves_status setup_device(waves_handle* h) {
  const waves_config& k = h->cfg;
  Dev& D = h->D;
  std::memset(&D, 0, sizeof(D));
  D.nx = k.n[0]; D.ny = k.n[1]; D.nz = k.n[2];
  D.N = (long long)D.nx * D.ny * D.nz;
  D.NU = (long long)(D.nx + 1) * D.ny * D.nz;
  D.NV = (long long)D.nx * (D.ny + 1) * D.nz;
  D.NW = (long long)D.nx * D.ny * (D.nz + 1);
  D.NF = D.NU + D.NV + D.NW;
  D.S = 2 * D.N + D.NF;
  D.hx = k.spacing[0]; D.hy = k.spacing[1]; D.hz = k.spacing[2];
  D.dtcfg = k.dt;
  D.ox = k.origin[0]; D.oy = k.origin[1]; D.oz = k.origin[2];
  D.eta0 = k.eta;
  D.px = k.periodic_x != 0;
  D.slope = k.slope;
  D.corr = k.corrugation;
  D.corr_phase = k.corrugation_phase;
  D.shape = k.shape;
  D.grav = k.gravity;
  D.max_face_cfl = k.max_face_cfl != 0;
  D.hist_cap = k.history_capacity;
  for (int a = 0; a < 4; a++) D.wave[a] = k.wave[a];
  D.tol = k.pressure_tolerance;
  D.linear_air = k.linear_air != 0;
  D.stokes2 = k.stokes_second != 0;
  D.flags = (k.height_normals ? 1 : 0) + (k.active_advection ? 2 : 0) + (k.transport_cache ? 4 : 0) + (k.transport_interior ? 8 : 0);
  D.coastal = k.coastal != 0;
  D.forcing[0] = k.origin[0];
  D.forcing[1] = k.zone_length;
  D.forcing[2] = k.damping_rate;
  D.forcing[3] = k.ramp_periods;
  D.right_abs = k.right_absorption;
  D.cfl = k.cfl;
  D.cell_d = double(k.spacing[0]) * double(k.spacing[1]) * double(k.spacing[2]);
  D.zone_x_end = coastal_zone_end(k);
  D.ipb = k.iterations_per_batch;
  D.mg_smoother = k.mg_smoother;
  D.mg_smoothing = k.mg_smoothing;
  D.mg_mode = k.mg_maintenance;
  D.mg_lag = k.mg_lag;
  D.mg_aggr = k.mg_aggregate_from;
  D.bf16 = k.mg_precision == 16;

  const long long N = D.N, NF = D.NF, S = D.S;
  const int cap = std::max(k.history_capacity, 1);
  waves_status st;
#define AL(p, n, pers, name) \
  if ((st = alloc_t(h, &p, (size_t)(n), pers, name)) != WAVES_OK) return st
  AL(D.bank0, S, true, "bank0");
  AL(D.bank1, S, true, "bank1");
  AL(D.r, N, false, "r");
  AL(D.z, N, false, "z");
  AL(D.d, N, false, "d");
  AL(D.q, N, false, "q");
  AL(D.diag, N, true, "diag");
  AL(D.b, N, false, "b");
  AL(D.coef, 6 * N, true, "coef");
  AL(D.pbase, N, true, "pbase");
  AL(D.phi, N, true, "phi");
  AL(D.kind, N, true, "kind");
  AL(D.plane, N, false, "plane");
  AL(D.mF, N, false, "mF");
  AL(D.mci, N, false, "mci");
  AL(D.fwd, NF, false, "fwd");
  AL(D.tcache, 6 * NF, false, "tcache");
  AL(D.src0, NF, false, "src0");
  AL(D.src1, NF, true, "src1");
  AL(D.vband0, NF, true, "vband0");
  AL(D.vband1, NF, true, "vband1");
  AL(D.pmask0, N, true, "pmask0");
  AL(D.pmask1, N, true, "pmask1");
  AL(D.history, 4 * (size_t)cap, true, "history");
  AL(D.chistory, 5 * (size_t)cap, true, "chistory");
  AL(D.c, WAVES_CONTROL_SIZE, true, "control");
  // every grid that writes reduction partials: one block per 256 entries, or the level-0 tiles
  // of 32 x 8 cells per z plane
  long long tiles0 = (long long)((D.nx + 31) / 32) * ((D.ny + 7) / 8) * D.nz;
  long long maxblocks = std::max((std::max(std::max(N, NF), S) + 255) / 256 + 1, tiles0);
  AL(D.part, 9 * maxblocks, false, "partials");
  AL(D.count, wg::kSiteCount, false, "counters");
  AL(h->probes, 8, true, "probes");
  // solid table
  D.tab_w = D.nx + 2 * wg::kSolidPad;
  D.tab_h = D.ny + 2 * wg::kSolidPad;
  {
    std::vector<signed char> tab((size_t)D.tab_w * D.tab_h);
    for (int y = 0; y < D.tab_h; y++)
      for (int x = 0; x < D.tab_w; x++) tab[(size_t)y * D.tab_w + x] = solid_host(k, x - wg::kSolidPad, y - wg::kSolidPad) ? 1 : 0;
    signed char* dtab;
    AL(dtab, tab.size(), false, "solid_table");
    CK(cudaMemcpyAsync(dtab, tab.data(), tab.size(), cudaMemcpyHostToDevice, h->stream));
    D.solid_tab = dtab;
    std::vector<signed char> clear(tab.size(), 0);
    for (int y = 1; y + 1 < D.tab_h; y++)
      for (int x = 1; x + 1 < D.tab_w; x++) {
        bool any = false;
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) any = any || tab[(size_t)(y + dy) * D.tab_w + x + dx] != 0;
        clear[(size_t)y * D.tab_w + x] = any ? 0 : 1;
      }
    signed char* dclear;
    AL(dclear, clear.size(), false, "clear_table");
    CK(cudaMemcpyAsync(dclear, clear.data(), clear.size(), cudaMemcpyHostToDevice, h->stream));
    D.clear_tab = dclear;
    // MacCormack face class per (axis, y, x) column: 1 within WAVES_MAC_BAND cells (default 1) of a
    // solid cell or of the domain edge (where donors take the boundary path), every column when x
    // is periodic.  On the beach at t = 5 s (ms per step): band 3 14.85, 2 14.48, 1 14.36, 0 14.43.
    const int cx = D.nx + 1, cy = D.ny + 1;
    std::vector<unsigned char> cls((size_t)3 * cx * cy, 1);
    // faces within `band` cells of a solid cell or the domain edge go straight to the general
    // pass; the others try the fast pass, which hands over every face whose samples leave the
    // fast path (so the band only moves work between the passes; the results do not depend on it)
    int band = 1;
    if (const char* e = getenv("WAVES_MAC_BAND")) band = std::max(0, std::min(3, atoi(e)));
    if (!D.px)
      for (int y = 0; y < cy; y++)
        for (int x = 0; x < cx; x++) {
          bool edge = x < band || x > D.nx - 1 - band || y < band || y > D.ny - 1 - band;
          for (int dy = -band; dy <= band && !edge; dy++)
            for (int dx = -band; dx <= band && !edge; dx++) edge = solid_host(k, x + dx, y + dy);
          for (int a = 0; a < 3; a++) cls[((size_t)a * cy + y) * cx + x] = edge ? 1 : 0;
        }
    unsigned char* dcls;
    AL(dcls, cls.size(), false, "mac_class");
    CK(cudaMemcpyAsync(dcls, cls.data(), cls.size(), cudaMemcpyHostToDevice, h->stream));
    D.mac_class = dcls;
    CK(cudaStreamSynchronize(h->stream));
  }
  // wave-target tables: columns from 4 ghost columns left of x = 0 to the last face column of the
  // forcing zone, rows 0..ny; the stamps start as NaN, which no time equals
  D.wt_x0 = -4;
  D.wt_w = D.coastal ? D.zone_x_end + 2 - D.wt_x0 : 0;
  D.wt_h = D.coastal ? D.ny + 1 : 0;
  if (D.coastal) {
    AL(D.wsurf, (size_t)3 * D.wt_w, false, "wave_surface");
    AL(D.wvel, (size_t)6 * D.wt_h * D.wt_w, false, "wave_velocity");
    AL(D.wdecay, (size_t)2 * D.wt_w, false, "wave_relaxation");
    AL(D.wstamp, 4, false, "wave_stamps");
    const float nan4[4] = {NAN, NAN, NAN, NAN};
    CK(cudaMemcpyAsync(D.wstamp, nan4, sizeof(nan4), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  if (k.warm_start) {
    D.net_on = 1;
    AL(D.net_w, (size_t)WAVES_NET_LAYERS * wg::kNetLayerWords, false, "net_weights");
    AL(D.net_wt, (size_t)WAVES_NET_LAYERS * 27 * 256, false, "net_weights_tcgen05");
    // the layers on tcgen05 unless WAVES_NET_MMA=sync asks for the warp-level mma.sync form
    D.net_tc05 = 1;
    if (const char* e = getenv("WAVES_NET_MMA")) D.net_tc05 = std::strcmp(e, "sync") != 0;
    wg::setup_warm_network();
    AL(D.net_b, (size_t)WAVES_NET_LAYERS * 16, false, "net_bias");
    AL(D.net_scale, 4, false, "net_scale");
    AL(D.net_act, (size_t)2 * N * 16, false, "net_activations");
    AL(D.net_p, N, false, "net_pressure");
  }
  AL(D.ext_nb, NF, false, "ext_neighbours");
  AL(D.mac_list, NF, false, "mac_list");
  AL(D.mac_ctr, wg::kMacCounters, false, "mac_counters");
  AL(D.mac_ovf, NF, false, "mac_handover");
  if (NF >= (1LL << 30)) {  // donor-table entries hold 2 f + 1 in an int
    h->err = "too many faces for the MacCormack donor table";
    return WAVES_INVALID_ARG;
  }
  AL(D.mac_dtab, NF, false, "mac_donor_table");
  AL(D.geo_queue, N, false, "geometry_search_queue");
  AL(D.geo_qcount, 1, false, "geometry_search_count");
  {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 152;
    D.geo_seed_grid = 8 * std::max(sms, 1);
  }
  D.mac_grid = wg::mac_blocks();
  D.mac_fast_grid = wg::mac_fast_blocks();
  if (D.mac_fast_grid <= 0) D.mac_fast_grid = 4 * 152;
  // interior faces on the fast-path pass where the fast path exists (not periodic in x, the
  // interior fast path of flag 8 off); WAVES_MAC_SPLIT=0 runs every face on the general pass
  D.mac_split = (!D.px && (D.flags & 8) == 0) ? 1 : 0;
  if (const char* e = getenv("WAVES_MAC_SPLIT")) D.mac_split = D.mac_split && atoi(e) != 0;
  D.pdl_early = 0;
  if (const char* e = getenv("WAVES_PDL")) D.pdl_early = atoi(e) == 2;
  if (D.mac_grid <= 0) D.mac_grid = 2 * 152;
  D.mac_grid2 = wg::mac_blocks2();
  if (D.mac_grid2 <= 0) D.mac_grid2 = 2 * 152;
  // MacCormack: 3 blocks per SM (80 registers, a few spills) beats 2 (128 registers): 935 vs
  // 1032 us per pass on the beach; 4 measured the same as 3
  D.mac_minb = 3;
  if (const char* e = getenv("WAVES_MAC_BLOCKS")) D.mac_minb = atoi(e) == 2 ? 2 : 3;
  // multigrid
  plan_levels(h);
  if ((int)h->levels.size() > wg::kMaxLevels) {
    h->err = "multigrid hierarchy deeper than 12 levels";
    return WAVES_INVALID_ARG;
  }
  D.L = (int)h->levels.size();
  long long nodes = 0, moff = 0, eoff = 0, toff = 0;
  int soff = 0;
  h->stencil_tab.clear();
  for (int l = 0; l < D.L; l++) {
    const HLevel& hl = h->levels[l];
    wg::MGLevelDev& lv = D.lv[l];
    lv.nx = hl.n[0]; lv.ny = hl.n[1]; lv.nz = hl.n[2];
    lv.count = hl.count;
    lv.fx = hl.f[0]; lv.fy = hl.f[1]; lv.fz = hl.f[2];
    lv.aggregate = hl.aggregate;
    lv.stencil = (int)hl.stencil.size() / 3;
    lv.twidth = hl.aggregate ? 1 : hl.f[0] * hl.f[1] * hl.f[2];
    lv.off = (int)nodes;
    lv.moff = moff;
    lv.eoff = eoff;
    lv.toff = toff;
    lv.soff = soff;
    nodes += hl.count;
    if (l > 0) {
      moff += (long long)hl.count * 125;
      eoff += (long long)hl.count * lv.stencil;
    }
    if (l + 1 < D.L) toff += (long long)hl.count * lv.twidth;
    soff += lv.stencil;
    h->stencil_tab.insert(h->stencil_tab.end(), hl.stencil.begin(), hl.stencil.end());
  }
  D.mg_nodes = nodes;
  size_t tsz = D.bf16 ? 2 : 4;
  {
    void* p;
    if ((st = alloc(h, &p, (size_t)(8 * nodes) * tsz, true, "mg_vectors")) != WAVES_OK) return st;
    D.mgv = p;
  }
  {
    int* dst;
    AL(dst, h->stencil_tab.size(), false, "stencils");
    CK(cudaMemcpyAsync(dst, h->stencil_tab.data(), h->stencil_tab.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    D.stencil_tab = dst;
    // linear offsets of the stencil entries, per level (valid for cells two cells from every edge)
    std::vector<int> lin(h->stencil_tab.size() / 3);
    for (int l = 0; l < D.L; l++)
      for (int k = 0; k < D.lv[l].stencil; k++) {
        const int* o = &h->stencil_tab[3 * (D.lv[l].soff + k)];
        lin[D.lv[l].soff + k] = o[0] + D.lv[l].nx * (o[1] + D.lv[l].ny * o[2]);
      }
    int* dlin;
    AL(dlin, lin.size(), false, "stencil_linear");
    CK(cudaMemcpyAsync(dlin, lin.data(), lin.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    D.stencil_lin = dlin;
    // Galerkin partials per stencil entry for the coarse levels with small stencils.  A product
    // term's offset d is a difference of two transfer targets; the transfers clamp at the bottom
    // and the sides (moving d one step toward zero on that axis) and fold short periodic axes to
    // the minimum image, so the stencil must be closed under both for every term to find its slot.
    std::vector<signed char> cslot((size_t)wg::kMaxLevels * 125, -1);
    for (int l = 1; l < D.L; l++) {
      wg::MGLevelDev& lv = D.lv[l];
      lv.gal_slots = 0;
      const int S = lv.stencil;
      if (S > 48) continue;
      const int* st = &h->stencil_tab[3 * lv.soff];
      const int n[3] = {lv.nx, lv.ny, lv.nz};
      auto find = [&](int x, int y, int z) {
        for (int k = 0; k < S; k++)
          if (st[3 * k] == x && st[3 * k + 1] == y && st[3 * k + 2] == z) return k;
        return -1;
      };
      bool closed = true;
      for (int k = 0; k < S && closed; k++)
        for (int a = 0; a < 3 && closed; a++) {
          int d[3] = {st[3 * k], st[3 * k + 1], st[3 * k + 2]};
          const bool periodic = a == 2 || (a == 0 && D.px);
          if (periodic) {
            const int m = n[a];
            d[a] = ((d[a] + m / 2) % m + m) % m - m / 2;
          } else if (d[a] != 0) {
            d[a] -= d[a] > 0 ? 1 : -1;
          }
          closed = find(d[0], d[1], d[2]) >= 0;
        }
      if (!closed) continue;
      lv.gal_slots = S;
      for (int k = 0; k < S; k++) {
        const int* o = &st[3 * k];
        if (o[0] < -2 || o[0] > 2 || o[1] < -2 || o[1] > 2 || o[2] < -2 || o[2] > 2) {
          lv.gal_slots = 0;
          break;
        }
        cslot[(size_t)l * 125 + (o[0] + 2) + 5 * ((o[1] + 2) + 5 * (o[2] + 2))] = (signed char)k;
      }
    }
    signed char* dcs;
    AL(dcs, cslot.size(), false, "galerkin_slots");
    CK(cudaMemcpyAsync(dcs, cslot.data(), cslot.size(), cudaMemcpyHostToDevice, h->stream));
    D.gal_cslot = dcs;
    CK(cudaStreamSynchronize(h->stream));
  }
  // Restriction tables (pressure_multigrid.glslinc:208-221): for coarse level l, axis a, coarse
  // index X, up to four fine coordinates and the axis weight, with the same float arithmetic.
  {
    std::vector<int> ridx;
    std::vector<float> rw;
    auto pm = [](int x, int m) { return x >= 0 ? x % m : (m - 1) - ((-1 - x) % m); };
    for (int l = 1; l < D.L; l++) {
      wg::MGLevelDev& cv = D.lv[l];
      const wg::MGLevelDev& pv = D.lv[l - 1];
      int nc[3] = {cv.nx, cv.ny, cv.nz}, nf[3] = {pv.nx, pv.ny, pv.nz}, fa[3] = {pv.fx, pv.fy, pv.fz};
      for (int a = 0; a < 3; a++) {
        bool periodic = a == 2 || (a == 0 && D.px);
        int f = fa[a];
        int ext = f > 1 ? ((periodic && nf[a] <= 4) ? nf[a] : 4) : 1;
        cv.roff[a] = (int)ridx.size();
        cv.rext[a] = ext;
        for (int X = 0; X < nc[a]; X++) {
          int lo = f > 1 ? ((periodic && nf[a] <= 4) ? 0 : X * f - 1) : X * f;
          for (int t = 0; t < 4; t++) {
            int q = lo + t, idx = -1;
            float w = 0.f;
            if (t < ext) {
              if (periodic) q = pm(q, nf[a]);
              if (q >= 0 && q < nf[a]) {
                idx = q;
                volatile float pos = ((float)q + .5f) / (float)f;
                pos = pos - .5f;
                int base = (int)std::floor((float)pos);
                float tt = (float)pos - std::floor((float)pos);
                for (int bit = 0; bit < f; bit++) {
                  int nb = base + bit;
                  if (periodic) nb = pm(nb, nc[a]);
                  else if (a == 0) nb = std::min(std::max(nb, 0), nc[a] - 1);
                  else nb = std::max(nb, 0);
                  if (nb == X) w += f == 1 ? 1.f : (bit == 1 ? tt : 1.f - tt);
                }
              }
            }
            ridx.push_back(idx);
            rw.push_back(w);
          }
        }
      }
    }
    if (ridx.empty()) {
      ridx.push_back(-1);
      rw.push_back(0.f);
    }
    int* di;
    float* dw;
    AL(di, ridx.size(), false, "restrict_idx");
    AL(dw, rw.size(), false, "restrict_w");
    CK(cudaMemcpyAsync(di, ridx.data(), ridx.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(dw, rw.data(), rw.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    D.rt_idx = di;
    D.rt_w = dw;
    CK(cudaStreamSynchronize(h->stream));
  }
  AL(D.mgnb0, N, true, "mg_level0_neighbours");
  AL(D.mg_rowlist, nodes, false, "mg_active_rows");
  AL(D.mg_rowcount, wg::kMaxLevels, false, "mg_active_counts");
  AL(D.mgcol, eoff, false, "mg_ell_columns");
  // Levels from mg_bottom down run inside one thread block (latency-bound sizes).
  D.mg_bottom = D.L - 1;
  for (int l = 1; l < D.L; l++)
    if (D.lv[l].count <= 1024) {
      D.mg_bottom = l;
      break;
    }
  if (const char* e = getenv("WAVES_MG_BOTTOM")) {
    int v = atoi(e);
    if (v >= 1 && v < D.L) D.mg_bottom = v;
  }
  // Levels with fewer rows than this use the product-parallel apply (both forms give the same bits).
  D.mg_rows_below = 65536;
  if (const char* e = getenv("WAVES_MG_ROWS_BELOW")) D.mg_rows_below = std::max(0, atoi(e));
  // launch shapes of the level >= 1 sweeps (measured on the beach, ms per step over 120 steps:
  // 16 rows per product-parallel block 13.45-13.48, 8 rows 13.67-13.70, 32 rows 13.72, 64 rows
  // 14.52; 128-thread one-row-per-thread blocks 0.2 % faster than 256)
  D.mg_thread_nt = 128;
  if (const char* e = getenv("WAVES_MG_THREAD_NT")) D.mg_thread_nt = atoi(e) == 256 ? 256 : 128;
  // four lanes per active row in the sweeps of the large levels (k_mgl4); WAVES_MG_LANES=1 keeps one
  // thread per row (k_mgl).  Both give the same bits.
  D.mg_lanes = 4;
  if (const char* e = getenv("WAVES_MG_LANES")) D.mg_lanes = atoi(e) == 1 ? 1 : 4;
  D.mg_rows_rr = 16;
  if (const char* e = getenv("WAVES_MG_ROWS_RR")) {
    const int v = atoi(e);
    D.mg_rows_rr = (v == 8 || v == 32 || v == 64) ? v : 16;
  }
  {
    // levels mg_bottom..L-1 staged in shared memory when their fields and rows fit
    const int lb = D.mg_bottom, Lc = D.L - 1;
    const size_t span = (size_t)D.lv[Lc].off + D.lv[Lc].count - D.lv[lb].off;
    const size_t rows = (size_t)(D.lv[Lc].eoff + (long long)D.lv[Lc].stencil * D.lv[Lc].count - D.lv[lb].eoff);
    const size_t nc = (size_t)D.lv[Lc].count;
    const size_t bytes = ((8 * span * tsz + 15) & ~(size_t)15) + ((rows * tsz + 15) & ~(size_t)15) +
                         ((rows * 2 + 15) & ~(size_t)15) + (nc <= 64 ? nc * nc * sizeof(float) : 0);
    bool narrow = true;  // every staged level indexable in 16 bits
    for (int l = lb; l <= Lc; l++) narrow = narrow && D.lv[l].count <= 65536;
    D.mg_bottom_smem = lb >= 1 && narrow && bytes <= (size_t)wg::kBottomSmemMax ? (int)bytes : 0;
    if (getenv("WAVES_MG_BOTTOM_GLOBAL")) D.mg_bottom_smem = 0;
  }
  {
    // WAVES_MG_COARSE=1: the coarse levels (fewer than 65536 rows) above the bottom run as one
    // cooperative launch.  Off by default: on the beach it removes about 230 launches per trial
    // but is no faster than the per-level launches (14.05 vs 13.93 ms per step).
    D.mg_coarse_from = 0;
    if (const char* e = getenv("WAVES_MG_COARSE"))
      if (atoi(e) != 0)
        for (int l = 1; l < D.mg_bottom; l++)
          if (D.lv[l].count < 65536) {
            D.mg_coarse_from = l;
            break;
          }
    if (D.mg_coarse_from > 0) {
      wg::mg_kernel_attributes();
      const size_t smem = std::max((size_t)wg::kMaxStencil * 64 * sizeof(float), (size_t)D.mg_bottom_smem);
      D.coarse_blocks = wg::coarse_blocks(smem);
      if (D.coarse_blocks <= 0) D.mg_coarse_from = 0;
    }
    AL(D.gbar, 2, false, "grid_barrier");
  }
  {
    // WAVES_MG_LEG=1: the coarse leg (the levels with at most kLegRowsFrom rows above the
    // bottom, and the bottom) runs as one launch of one thread-block cluster instead of a launch
    // per sweep, restriction and prolongation.  Off by default: on the beach (leg = level 3,
    // 4,680 rows, and the bottom) it is slower than the per-level launches (17.32 vs 16.98 ms per
    // step at t = 5 s): each of its ten phases waits out several dependent global-memory round
    // trips on eight SMs, about 98 us per V-cycle in all.
    D.mg_leg_from = 0;
    D.mg_leg_smem = 0;
    bool want = false;
    if (const char* e = getenv("WAVES_MG_LEG")) want = D.mg_coarse_from == 0 && atoi(e) != 0;
    int from = 0;
    for (int l = 1; want && l < D.mg_bottom; l++)
      if (D.lv[l].count <= wg::kLegRowsFrom) {
        from = l;
        break;
      }
    if (from > 0) {
      wg::mg_kernel_attributes();
      const size_t smem = std::max(wg::kLegSmemMin, (size_t)D.mg_bottom_smem);
      if (wg::leg_available(smem)) {
        D.mg_leg_from = from;
        D.mg_leg_smem = (int)smem;
      }
    }
  }
  AL(D.mgmat, moff, true, "mg_matrix");
  {
    // A P of the two-stage Galerkin product, 125 slots per row of the largest fine level >= 1
    // that is coarsened (dense by fine cell; only active rows are written and read)
    long long ap_rows = 1;
    for (int l = 1; l + 1 < D.L; l++) ap_rows = std::max(ap_rows, (long long)D.lv[l].count);
    AL(D.gal_ap, (size_t)ap_rows * 125, false, "galerkin_ap");
  }
  {
    void* p;
    if ((st = alloc(h, &p, (size_t)eoff * tsz, true, "mg_ell")) != WAVES_OK) return st;
    D.mgell = p;
  }
  AL(D.mgtid, toff, true, "mg_transfer_ids");
  AL(D.mgtw, toff, true, "mg_transfer_weights");
  AL(D.mgtq, toff, true, "mg_transfer_coarse_coordinates");
  AL(D.mglinv, 64 * 64, true, "mg_linv");
  AL(D.snapshot, 9 * N, true, "mg_snapshot");
  AL(D.previous, 9 * N, true, "mg_previous");
  if (D.bf16) {
    void* p;
    if ((st = alloc(h, &p, (size_t)6 * N * 2, true, "mg_c0_bf16")) != WAVES_OK) return st;
    D.c0 = p;
  } else
    D.c0 = D.snapshot;
  AL(D.hstate, 64 + 32 * (size_t)cap, true, "mg_audit");
#undef AL
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}

// ---------------------------------------------------------------- step enqueue
// Motion part of the set-up: CFL, VOF sweeps, MacCormack, coastal forcing.
void enqueue_motion(waves_handle* h, cudaStream_t s) {
  const Dev& D = h->D;
  wg::launch_motion_cfl(D, s);
  for (int sweep = 0; sweep < 3; sweep++) wg::launch_sweep(D, s);
  wg::launch_maccormack(D, s);
  if (D.coastal) wg::launch_coastal(D, s);
}
// Pressure set-up: geometry, coefficients, projection set-up, multigrid build.
void enqueue_pressure_setup(waves_handle* h, cudaStream_t s) {
  const Dev& D = h->D;
  wg::launch_geometry(D, s);
  wg::launch_proj_setup(D, s);
  wg::launch_warm_start(D, s);
  wg::launch_mg_build(D, s);
}
void enqueue_setup(waves_handle* h, cudaStream_t s) {
  enqueue_motion(h, s);
  enqueue_pressure_setup(h, s);
}
void enqueue_cg_begin(waves_handle* h, cudaStream_t s) {
  const Dev& D = h->D;
  wg::launch_defect_begin(D, s);
  wg::launch_cg_init(D, s);
  wg::launch_mg_vcycle(D, s, 0);
}
void enqueue_cg_iteration(waves_handle* h, cudaStream_t s, cudaGraphConditionalHandle hc, int use_handle) {
  const Dev& D = h->D;
  wg::launch_cg_matvec(D, s);
  wg::launch_cg_update(D, s);
  wg::launch_mg_vcycle(D, s, 1);
  wg::launch_cg_direction(D, s, hc, use_handle);
}

// Add a conditional node at the current capture point of `s`; returns its body graph.
waves_status add_conditional(waves_handle* h, cudaStream_t s, cudaGraphConditionalNodeType type, int cond_kind,
                             cudaGraphConditionalHandle* out_handle, cudaGraph_t* body) {
  cudaStreamCaptureStatus status;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CK(cudaStreamGetCaptureInfo(s, &status, nullptr, &graph, &deps, nullptr, &ndeps));
  cudaGraphConditionalHandle hc;
  CK(cudaGraphConditionalHandleCreate(&hc, graph, 0, cudaGraphCondAssignDefault));
  wg::launch_set_cond(h->D, s, hc, cond_kind);
  CK(cudaStreamGetCaptureInfo(s, &status, nullptr, &graph, &deps, nullptr, &ndeps));
  cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
  p.conditional.handle = hc;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &p));
  *body = p.conditional.phGraph_out[0];
  *out_handle = hc;
  CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return WAVES_OK;
}

// Kernel nodes enqueued by `fn` (captured into a scratch graph and counted).
template <class Fn> int32_t count_kernels(waves_handle* h, Fn fn) {
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return -1;
  cudaGraph_t g = nullptr;
  int32_t n = -1;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    fn(s);
    if (cudaStreamEndCapture(s, &g) == cudaSuccess) {
      size_t count = 0;
      cudaGraphGetNodes(g, nullptr, &count);
      n = (int32_t)count;
      cudaGraphDestroy(g);
    }
  }
  cudaStreamDestroy(s);
  cudaGetLastError();
  return n;
}
void count_launches(waves_handle* h) {
  const Dev& D = h->D;
  h->launches[0] = count_kernels(h, [&](cudaStream_t s) { wg::launch_begin(D, s); });
  h->launches[1] = count_kernels(h, [&](cudaStream_t s) { enqueue_motion(h, s); });
  h->launches[2] = count_kernels(h, [&](cudaStream_t s) { enqueue_pressure_setup(h, s); });
  h->launches[3] = count_kernels(h, [&](cudaStream_t s) { enqueue_cg_begin(h, s); });
  h->launches[4] = count_kernels(h, [&](cudaStream_t s) { enqueue_cg_iteration(h, s, 0, 0); });
  h->launches[5] = count_kernels(h, [&](cudaStream_t s) { wg::launch_post(D, s); });
  h->launches[6] = count_kernels(h, [&](cudaStream_t s) { wg::launch_trial_end(D, s); });
  h->launches[7] = 1;  // condition-setting kernel
}

// Motion graph: begin (ops 43, 1) and, if a trial is active, CFL/VOF/MacCormack/forcing.
// Pressure graph: if active, geometry .. multigrid build, then WHILE(defect round) { CG set-up,
// WHILE(solving) { CG iteration }, projection/extension/acceptance }, trial end.
waves_status build_graph(waves_handle* h) {
  cudaStream_t s0 = h->stream, s1 = nullptr, s2 = nullptr, s3 = nullptr;
  CK(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking));
  waves_status st = WAVES_OK;
  do {
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle hc;
    cudaGraph_t body;
    // --- motion graph
    CK(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
    wg::launch_begin(h->D, s0);
    if ((st = add_conditional(h, s0, cudaGraphCondTypeIf, wg::kCondActive, &hc, &body)) != WAVES_OK) break;
    CK(cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    enqueue_motion(h, s1);
    CK(cudaStreamEndCapture(s1, &body));
    CK(cudaStreamEndCapture(s0, &graph));
    CK(cudaGraphInstantiate(&h->exec, graph, 0));
    h->graph = graph;
    // --- pressure graph
    graph = nullptr;
    cudaGraphConditionalHandle h_active, h_defect, h_cg;
    cudaGraph_t body_active, body_defect, body_cg;
    CK(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
    if ((st = add_conditional(h, s0, cudaGraphCondTypeIf, wg::kCondActive, &h_active, &body_active)) != WAVES_OK) break;
    CK(cudaStreamBeginCaptureToGraph(s1, body_active, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    enqueue_pressure_setup(h, s1);
    if ((st = add_conditional(h, s1, cudaGraphCondTypeWhile, wg::kCondDefectFirst, &h_defect, &body_defect)) != WAVES_OK) break;
    CK(cudaStreamBeginCaptureToGraph(s2, body_defect, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    enqueue_cg_begin(h, s2);
    if ((st = add_conditional(h, s2, cudaGraphCondTypeWhile, wg::kCondSolving, &h_cg, &body_cg)) != WAVES_OK) break;
    CK(cudaStreamBeginCaptureToGraph(s3, body_cg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    enqueue_cg_iteration(h, s3, h_cg, 1);
    CK(cudaStreamEndCapture(s3, &body_cg));
    wg::launch_post(h->D, s2);
    wg::launch_set_cond(h->D, s2, h_defect, wg::kCondDefect);
    CK(cudaStreamEndCapture(s2, &body_defect));
    wg::launch_trial_end(h->D, s1);
    CK(cudaStreamEndCapture(s1, &body_active));
    CK(cudaStreamEndCapture(s0, &graph));
    CK(cudaGraphInstantiate(&h->exec_p, graph, 0));
    h->graph_p = graph;
  } while (0);
  cudaStreamDestroy(s1);
  cudaStreamDestroy(s2);
  cudaStreamDestroy(s3);
  if (st != WAVES_OK) {
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(s0, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(s0, &junk);
      if (junk) cudaGraphDestroy(junk);
    }
    cudaGetLastError();
  }
  return st;
}

cudaEvent_t take_event(waves_handle* h) {
  if (!h->ev_pool.empty()) {
    cudaEvent_t e = h->ev_pool.back();
    h->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
// One finished trial: totals and the running per-trial cost (work_scheduler.gd:31: weight .25,
// floor 2 us).
void fold_trial(waves_handle* h, float motion, float pressure) {
  h->motion_ms += motion;
  h->pressure_ms += pressure;
  h->timed_trials++;
  const double ms = (double)motion + (double)pressure;
  h->gpu_ms_total += ms;
  h->trial_cost_ms = h->trial_cost_ms <= 0 ? ms : h->trial_cost_ms + .25 * (std::max(ms, 0.002) - h->trial_cost_ms);
}
// Fold completed trial timings into the totals (called after a stream synchronisation).
void collect_timing(waves_handle* h) {
  for (auto& t : h->ev_pending) {
    float a = 0, b = 0;
    if (cudaEventElapsedTime(&a, t[0], t[1]) == cudaSuccess && cudaEventElapsedTime(&b, t[1], t[2]) == cudaSuccess)
      fold_trial(h, a, b);
    for (cudaEvent_t e : t) h->ev_pool.push_back(e);
  }
  h->ev_pending.clear();
  cudaGetLastError();
}
// The same for the trials already finished, without waiting (stream order: stop at the first
// unfinished one).
void collect_timing_ready(waves_handle* h) {
  size_t k = 0;
  for (; k < h->ev_pending.size(); k++) {
    auto& t = h->ev_pending[k];
    if (cudaEventQuery(t[2]) != cudaSuccess) break;
    float a = 0, b = 0;
    if (cudaEventElapsedTime(&a, t[0], t[1]) == cudaSuccess && cudaEventElapsedTime(&b, t[1], t[2]) == cudaSuccess)
      fold_trial(h, a, b);
    for (cudaEvent_t e : t) h->ev_pool.push_back(e);
  }
  h->ev_pending.erase(h->ev_pending.begin(), h->ev_pending.begin() + (long)k);
  cudaGetLastError();
}

waves_status read_control(waves_handle* h) {
  CK(cudaMemcpyAsync(h->host_c, h->D.c, WAVES_CONTROL_SIZE * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  collect_timing(h);
  return WAVES_OK;
}
waves_status upload_quota(waves_handle* h) {
  *h->host_quota = h->quota.load();
  CK(cudaMemcpyAsync(h->D.c + wg::kQuota, h->host_quota, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  return WAVES_OK;
}

// Host-driven trial: same kernels, control flow decided from the control block, read after every
// `batch` CG iterations (iterations past convergence return at once).
waves_status host_trial(waves_handle* h, int batch = 4) {
  const Dev& D = h->D;
  cudaStream_t s = h->stream;
  // with kernel probes installed, each batch starts behind a fixed delay (~2 ms) so that the
  // host has enqueued the batch before the GPU reaches it
  auto hold = [&] {
    if (wg::g_probe) wg::launch_delay(s, 4000000LL);
  };
  wg::launch_begin(D, s);
  waves_status st;
  if ((st = read_control(h)) != WAVES_OK) return st;
  if (!(h->host_c[4] > .5)) return WAVES_OK;
  hold();
  enqueue_setup(h, s);
  for (int round = 0;; round++) {
    if (round > 0) hold();
    enqueue_cg_begin(h, s);
    if ((st = read_control(h)) != WAVES_OK) return st;
    const double* c = h->host_c;
    while (c[4] > .5 && c[6] < .5 && c[7] < .5) {
      hold();
      for (int k = 0; k < batch; k++) enqueue_cg_iteration(h, s, 0, 0);
      if ((st = read_control(h)) != WAVES_OK) return st;
    }
    hold();
    wg::launch_post(D, s);
    if ((st = read_control(h)) != WAVES_OK) return st;
    if (!(c[57] == 1 && c[7] < .5 && c[4] > .5)) break;
  }
  wg::launch_trial_end(D, s);
  CK(cudaGetLastError());
  return WAVES_OK;
}

bool halted(const double* c) {
  if (!(c[7] > .5)) return false;
  bool recoverable = (c[7] == 20 || (c[7] >= 10 && c[7] <= 12)) && c[29] < 2;
  return !recoverable;
}
bool quota_met(const double* c, double quota) { return quota >= 0 ? c[2] >= quota : c[1] >= -quota; }

}  // namespace

// ====================================================================== C ABI
extern "C" {

waves_status waves_mg_plan(const waves_config* cfg, int32_t* out, int32_t capacity, int32_t* levels) {
  if (!cfg || !levels || capacity < 0 || (capacity > 0 && !out)) return WAVES_INVALID_ARG;
  if (cfg->n[0] < 1 || cfg->n[1] < 1 || cfg->n[2] < 1 || !(cfg->spacing[0] > 0.f) || !(cfg->spacing[1] > 0.f) ||
      !(cfg->spacing[2] > 0.f))
    return WAVES_INVALID_ARG;
  std::vector<HLevel> plan;
  plan_levels_of(*cfg, plan);
  *levels = (int32_t)plan.size();
  for (int l = 0; l < (int)plan.size() && l < capacity; l++) {
    int32_t* o = out + 8 * l;
    for (int a = 0; a < 3; a++) {
      o[a] = plan[l].n[a];
      o[3 + a] = plan[l].f[a];
    }
    o[6] = (int32_t)(plan[l].stencil.size() / 3);
    o[7] = plan[l].aggregate ? 1 : 0;
  }
  return WAVES_OK;
}

waves_status waves_create(const waves_config* cfg, waves_handle** out) {
  if (!out || !cfg) return WAVES_INVALID_ARG;
  *out = nullptr;
  if (cfg->n[0] < 2 || cfg->n[1] < 2 || cfg->n[2] < 1 || !(cfg->spacing[0] > 0) || !(cfg->spacing[1] > 0) ||
      !(cfg->spacing[2] > 0) || !(cfg->dt > 0) || cfg->mg_smoothing < 1 || cfg->mg_smoothing > 8 || cfg->mg_lag < 1 ||
      (cfg->mg_precision != 32 && cfg->mg_precision != 16) || cfg->iterations_per_batch < 1) {
    g_create_error = "invalid configuration";
    return WAVES_INVALID_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device) {
    cudaGetLastError();
    g_create_error = "no CUDA device";
    return WAVES_NO_DEVICE;
  }
  waves_handle* h = new waves_handle;
  h->cfg = *cfg;
  if (const char* e = getenv("WAVES_PDL")) wg::g_pdl = atoi(e) != 0;  // 0 off, 1 on, 2 on with the early trigger
  waves_status st = WAVES_OK;
  auto fail = [&](waves_status s) {
    g_create_error = h->err;
    waves_destroy(h);
    return s;
  };
  if (cudaSetDevice(cfg->device) != cudaSuccess) {
    h->err = "cudaSetDevice failed";
    return fail(WAVES_NO_DEVICE);
  }
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    h->err = "cudaStreamCreate failed";
    return fail(WAVES_CUDA_ERROR);
  }
  if (cudaMallocHost(&h->host_c, WAVES_CONTROL_SIZE * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&h->host_quota, sizeof(double)) != cudaSuccess) {
    h->err = "cudaMallocHost failed";
    return fail(WAVES_CUDA_ERROR);
  }
  wg::mg_kernel_attributes();
  // The MacCormack sampler keeps its trace state on the per-thread stack (about 1.8 KB).
  size_t stack = 0;
  if (cudaDeviceGetLimit(&stack, cudaLimitStackSize) != cudaSuccess || stack < 8192) {
    if (cudaDeviceSetLimit(cudaLimitStackSize, 8192) != cudaSuccess) {
      h->err = "cudaDeviceSetLimit(stack) failed";
      return fail(WAVES_CUDA_ERROR);
    }
  }
  if ((st = setup_device(h)) != WAVES_OK) return fail(st);
  wg::launch_mg_cols(h->D, h->stream);
  wg::launch_ext_masks(h->D, h->stream);
  wg::launch_mac_donor_table(h->D, h->stream);
  wg::launch_initial(h->D, h->stream, h->probes);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    h->err = "initial commands failed";
    return fail(WAVES_CUDA_ERROR);
  }
  count_launches(h);
  const char* mode = getenv("WAVES_SCHEDULE");
  h->graph_mode = !(mode && std::strcmp(mode, "host") == 0);
  if (h->graph_mode && build_graph(h) != WAVES_OK) {
    // keep the message; fall back to host scheduling only if asked to tolerate it
    std::string why = h->err;
    h->err = "graph construction failed: " + why;
    return fail(WAVES_CUDA_ERROR);
  }
  *out = h;
  return WAVES_OK;
}

void waves_destroy(waves_handle* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  if (h->exec_p) cudaGraphExecDestroy(h->exec_p);
  if (h->graph_p) cudaGraphDestroy(h->graph_p);
  for (auto& t : h->ev_pending)
    for (cudaEvent_t e : t) h->ev_pool.push_back(e);
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  for (auto& sub : h->inflight) cudaEventDestroy(sub.done);
  if (h->frame_c) cudaFreeHost(h->frame_c);
  for (auto it = h->allocs.rbegin(); it != h->allocs.rend(); ++it) cudaFree(it->ptr);
  if (h->export_planes) cudaFree(h->export_planes);
  if (h->export_kinds) cudaFree(h->export_kinds);
  if (h->render_buf) cudaFree(h->render_buf);
  if (h->host_c) cudaFreeHost(h->host_c);
  if (h->host_quota) cudaFreeHost(h->host_quota);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

waves_status waves_request_steps(waves_handle* h, int64_t steps) {
  if (!h || steps < 0) return WAVES_INVALID_ARG;
  h->quota.store((double)steps);
  return WAVES_OK;
}
waves_status waves_request_time(waves_handle* h, double seconds) {
  if (!h || !(seconds >= 0) || std::isinf(seconds)) return WAVES_INVALID_ARG;
  h->quota.store(-seconds);
  return WAVES_OK;
}

waves_status waves_advance(waves_handle* h, int32_t max_trials) {
  if (!h || max_trials < 0) return WAVES_INVALID_ARG;
  cudaSetDevice(h->cfg.device);
  waves_status st;
  if ((st = upload_quota(h)) != WAVES_OK) return st;
  for (int t = 0; t < max_trials; t++) {
    if (h->graph_mode) {
      std::array<cudaEvent_t, 3> ev = {take_event(h), take_event(h), take_event(h)};
      CK(cudaEventRecord(ev[0], h->stream));
      CK(cudaGraphLaunch(h->exec, h->stream));
      CK(cudaEventRecord(ev[1], h->stream));
      CK(cudaGraphLaunch(h->exec_p, h->stream));
      CK(cudaEventRecord(ev[2], h->stream));
      h->ev_pending.push_back(ev);
    } else if ((st = host_trial(h)) != WAVES_OK)
      return st;
  }
  return WAVES_OK;
}

waves_status waves_frame(waves_handle* h, const waves_frame_budget* budget, waves_frame_report* report) {
  if (!h || !budget || !report || !(budget->gpu_budget_ms > 0) || budget->max_inflight < 1 ||
      budget->max_inflight > waves_handle::kFrameSlots || budget->max_trials < 1)
    return WAVES_INVALID_ARG;
  cudaSetDevice(h->cfg.device);
  if (!h->frame_c) CK(cudaMallocHost((void**)&h->frame_c, sizeof(double) * WAVES_CONTROL_SIZE * waves_handle::kFrameSlots));
  collect_timing_ready(h);
  // retire finished submissions in order; the latest control block is the telemetry
  while (!h->inflight.empty() && cudaEventQuery(h->inflight.front().done) == cudaSuccess) {
    const auto sub = h->inflight.front();
    std::memcpy(h->last_c, h->frame_c + (size_t)sub.slot * WAVES_CONTROL_SIZE, sizeof(h->last_c));
    h->have_last = true;
    cudaEventDestroy(sub.done);
    h->inflight.erase(h->inflight.begin());
    h->retired++;
  }
  cudaGetLastError();
  std::memset(report, 0, sizeof(*report));
  const double* c = h->last_c;
  const double quota = h->quota.load();
  // work_scheduler.gd:43-48: stop on failure, on a met quota with no trial pending, and at
  // max_inflight unfinished submissions
  const bool halt = h->have_last && halted(c);
  const bool done = h->have_last && quota_met(c, quota) && !(c[4] > .5) && !(c[7] > .5);
  int trials = 0;
  if (!halt && !done && (int)h->inflight.size() < budget->max_inflight) {
    // work_scheduler.gd:55-69: at least one trial, then while the predicted GPU time stays within
    // the budget and the enqueue time within cpu_budget_ms (a trial with no measurement yet is
    // predicted at the whole budget)
    const double cost = h->trial_cost_ms > 0 ? h->trial_cost_ms : budget->gpu_budget_ms;
    const auto t0 = std::chrono::steady_clock::now();
    waves_status st;
    while (trials < budget->max_trials) {
      if (trials > 0 && (trials + 1) * cost > budget->gpu_budget_ms) break;
      if ((st = waves_advance(h, 1)) != WAVES_OK) return st;
      trials++;
      const double cpu_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (budget->cpu_budget_ms > 0 && cpu_ms >= budget->cpu_budget_ms) break;
    }
    const int slot = (int)(h->serial++ % waves_handle::kFrameSlots);
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaMemcpyAsync(h->frame_c + (size_t)slot * WAVES_CONTROL_SIZE, h->D.c, sizeof(double) * WAVES_CONTROL_SIZE,
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaEventRecord(ev, h->stream));
    h->inflight.push_back({ev, slot, trials});
  }
  report->trials_submitted = trials;
  report->queue_depth = (int32_t)h->inflight.size();
  report->idle = done && h->inflight.empty() ? 1 : 0;
  report->halted = halt ? 1 : 0;
  report->trial_cost_ms = h->trial_cost_ms;
  report->predicted_gpu_ms = trials * h->trial_cost_ms;
  report->gpu_ms_total = h->gpu_ms_total;
  report->accepted_time = h->have_last ? c[1] : 0.0;
  report->accepted_steps = h->have_last ? (int64_t)c[2] : 0;
  report->r_fluid = report->accepted_time > 0 ? h->gpu_ms_total / 1e3 / report->accepted_time : -1.0;
  report->submissions_retired = h->retired;
  return WAVES_OK;
}

waves_status waves_synchronize(waves_handle* h) {
  if (!h) return WAVES_INVALID_ARG;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaGetLastError());
  collect_timing(h);
  return WAVES_OK;
}

void* waves_stream(waves_handle* h) { return h ? (void*)h->stream : nullptr; }

waves_status waves_timing(waves_handle* h, double* motion_ms, double* pressure_ms, int64_t* trials, int32_t reset) {
  if (!h) return WAVES_INVALID_ARG;
  CK(cudaStreamSynchronize(h->stream));
  collect_timing(h);
  if (motion_ms) *motion_ms = h->motion_ms;
  if (pressure_ms) *pressure_ms = h->pressure_ms;
  if (trials) *trials = h->timed_trials;
  if (reset) {
    h->motion_ms = h->pressure_ms = 0;
    h->timed_trials = 0;
  }
  return WAVES_OK;
}

waves_status waves_run(waves_handle* h, int32_t trials_per_sync) {
  if (!h || trials_per_sync < 1) return WAVES_INVALID_ARG;
  waves_status st;
  while (true) {
    if ((st = read_control(h)) != WAVES_OK) return st;
    const double* c = h->host_c;
    if (halted(c)) return WAVES_SOLVER_FAILED;
    double quota = h->quota.load();
    if (quota_met(c, quota) && !(c[4] > .5) && !(c[7] > .5)) return WAVES_OK;
    int trials = trials_per_sync;
    if (quota >= 0) {
      double left = quota - c[2];
      if (left >= 1 && left < trials) trials = (int)left;
    }
    if ((st = waves_advance(h, trials)) != WAVES_OK) return st;
  }
}

waves_status waves_control(waves_handle* h, double* c, int32_t count) {
  if (!h || !c || count < 0 || count > WAVES_CONTROL_SIZE) return WAVES_INVALID_ARG;
  waves_status st;
  if ((st = read_control(h)) != WAVES_OK) return st;
  std::memcpy(c, h->host_c, (size_t)count * sizeof(double));
  return WAVES_OK;
}
waves_status waves_set_control(waves_handle* h, const double* c, int32_t count) {
  if (!h || !c || count < 0 || count > WAVES_CONTROL_SIZE) return WAVES_INVALID_ARG;
  CK(cudaStreamSynchronize(h->stream));
  std::memcpy(h->host_c, c, (size_t)count * sizeof(double));
  CK(cudaMemcpyAsync(h->D.c, h->host_c, (size_t)count * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}
waves_status waves_inject_rejection(waves_handle* h) {
  if (!h) return WAVES_INVALID_ARG;
  *h->host_quota = 1.0;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpyAsync(h->D.c + 19, h->host_quota, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}

// Telemetry fields that come from the control block (pressure_gpu.gd:133-137, coupled_gpu.gd:58-65,
// coastal_gpu.gd:34-37): recoverable trial failures read 0 in `failure` (coupled_gpu.gd:61-62).
static void stats_from_control(const double* v, waves_stats_t* o) {
  std::memset(o, 0, sizeof(*o));
  bool recoverable = (v[7] == 20 || (v[7] >= 10 && v[7] <= 12)) && v[29] < 2;
  o->accepted_index = (int32_t)v[0];
  o->accepted_time = v[1];
  o->accepted_steps = (int64_t)v[2];
  o->rejections = (int64_t)v[3];
  o->pending = v[4] > .5;
  o->converged = v[6] > .5;
  o->failure = recoverable ? 0 : (int32_t)v[7];
  o->trial_failure = (int32_t)v[7];
  o->iterations = (int64_t)v[8];
  o->relative_residual = v[13];
  o->max_dt_divergence = v[14];
  o->max_face_speed = v[15];
  o->hydrostatic_error_pa = v[16];
  o->volume_m3 = v[17];
  o->total_iterations = (int64_t)v[18];
  o->dt = v[20];
  o->signed_roundoff_m3 = v[24];
  o->absolute_roundoff_m3 = v[25];
  o->initial_volume_m3 = v[26];
  o->max_CFL = v[27];
  o->mass_defect_m3 = v[28];
  o->retry_count = (int32_t)v[29];
  o->trial_count = (int64_t)v[32];
  o->last_rejection_code = (int32_t)v[33];
  o->last_rejected_dt = v[34];
  o->compression_volume_m3 = v[35];
  o->compression_coverage_errors = (int64_t)v[36];
  o->step_start_volume_m3 = v[37];
  o->raw_compression_volume_m3 = v[38];
  o->tentative_outflow_m3 = v[39];
  o->boundary_outflow_m3 = v[40];
  o->pressure_defect_corrections = (int32_t)v[58];
  o->true_relative_residual = v[60];
  o->rhs_integrated_divergence_l2 = v[62];
  o->residual_integrated_divergence_l2 = v[63];
  o->forcing_volume_m3 = v[72];
  o->ocean_inflow_m3 = v[73];
  o->ocean_outflow_m3 = v[74];
  for (int a = 0; a < 3; a++) o->forcing_momentum[a] = v[75 + a];
  for (int g = 0; g < 8; g++) o->gauges_m[g] = v[80 + g];
  o->forcing_min_F = v[88];
  o->forcing_max_F = v[89];
  o->conservation_residual_m3 = v[wg::kConservation];
  o->staged_forcing_volume_m3 = v[64];
  o->staged_ocean_inflow_m3 = v[65];
  o->staged_ocean_outflow_m3 = v[66];
  o->warm_start_used = (int64_t)v[wg::kWarmUsed];
}

waves_status waves_stats(waves_handle* h, waves_stats_t* o) {
  if (!h || !o) return WAVES_INVALID_ARG;
  waves_status st;
  if ((st = read_control(h)) != WAVES_OK) return st;
  unsigned hs[16];
  CK(cudaMemcpy(hs, h->D.hstate, sizeof(hs), cudaMemcpyDeviceToHost));
  stats_from_control(h->host_c, o);
  o->mg_builds = hs[11];
  o->mg_structure_builds = hs[12];
  o->mg_levels = h->D.L;
  h->last_mg_builds = hs[11];
  h->last_mg_structure_builds = hs[12];
  return WAVES_OK;
}

waves_status waves_frame_stats(const waves_handle* h, waves_stats_t* o) {
  if (!h || !o) return WAVES_INVALID_ARG;
  if (!h->have_last) return WAVES_INVALID_ARG;
  stats_from_control(h->last_c, o);
  o->mg_builds = h->last_mg_builds;
  o->mg_structure_builds = h->last_mg_structure_builds;
  o->mg_levels = h->D.L;
  return WAVES_OK;
}

waves_status waves_export_surface(waves_handle* h, float* planes, float* kinds) {
  if (!h || !planes || !kinds) return WAVES_INVALID_ARG;
  if (!h->export_planes) {
    CK(cudaMalloc(&h->export_planes, (size_t)h->D.N * sizeof(float4)));
    CK(cudaMalloc(&h->export_kinds, (size_t)h->D.N * sizeof(float)));
  }
  wg::launch_export(h->D, h->stream, h->export_planes, h->export_kinds);
  CK(cudaMemcpyAsync(planes, h->export_planes, (size_t)h->D.N * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(kinds, h->export_kinds, (size_t)h->D.N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}

waves_status waves_export_surface_device(waves_handle* h, void* planes, void* kinds, void* clock) {
  if (!h || !planes || !kinds || ((uintptr_t)planes & 15) || ((uintptr_t)kinds & 3) || ((uintptr_t)clock & 15))
    return WAVES_INVALID_ARG;
  cudaSetDevice(h->cfg.device);
  wg::launch_export(h->D, h->stream, (float4*)planes, (float*)kinds, (float4*)clock);
  CK(cudaGetLastError());
  return WAVES_OK;
}

void waves_render_params_default(waves_render_params* p, const waves_config* cfg, int32_t width, int32_t height) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->width = width;
  p->height = height;
  p->mode = 1;
  p->orthographic = 1;
  // camera_preset(1) of presentation.gd:86-93
  const bool wide = cfg && (double)cfg->n[2] * cfg->spacing[2] > 1.0;
  const float tg[3] = {wide ? 2.15f : 3.45f, wide ? -0.12f : -0.08f, 0.f};
  const float off[3] = {wide ? 2.5f : 1.5f, wide ? 4.45f : 2.f, wide ? 5.7f : 3.f};
  for (int k = 0; k < 3; k++) {
    p->target[k] = tg[k];
    p->eye[k] = tg[k] + off[k];
  }
  p->up[1] = 1.f;
  p->size = wide ? 5.25f : 1.5f;
  p->fov_y_deg = 75.f;
  p->water_tint[0] = 0.02745f;
  p->water_tint[1] = 0.56078f;
  p->water_tint[2] = 0.62353f;
  p->attenuation_distance = 0.18f;
  p->ripple_strength = 0.0025f;
  p->surface_roughness = 0.30f;
  p->sun_direction[0] = -0.45f;
  p->sun_direction[1] = 0.65f;
  p->sun_direction[2] = -0.63f;
  p->contact_correction = 1;
  p->clock_ready = 1;
}

namespace {
// Camera basis in FP32 (forward, right = forward x up, up' = right x forward, all normalised
// except up'), with the image half-extents at unit distance (perspective) or in metres
// (orthographic).
bool render_args(waves_handle* h, const waves_render_params* p, wg::RenderArgs& A) {
  if (!p || p->width < 1 || p->height < 1 || p->width > 16384 || p->height > 16384 || (p->mode != 0 && p->mode != 1))
    return false;
  if (p->orthographic ? !(p->size > 0.f) : !(p->fov_y_deg > 0.f && p->fov_y_deg < 179.f)) return false;
  auto nrm = [](float v[3]) {
    const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (!(l > 0.f)) return false;
    for (int k = 0; k < 3; k++) v[k] = v[k] / l;
    return true;
  };
  std::memset(&A, 0, sizeof(A));
  float f[3] = {p->target[0] - p->eye[0], p->target[1] - p->eye[1], p->target[2] - p->eye[2]};
  if (!nrm(f)) return false;
  float r[3] = {f[1] * p->up[2] - f[2] * p->up[1], f[2] * p->up[0] - f[0] * p->up[2], f[0] * p->up[1] - f[1] * p->up[0]};
  if (!nrm(r)) return false;
  const float u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
  for (int k = 0; k < 3; k++) {
    A.eye[k] = p->eye[k];
    A.fwd[k] = f[k];
    A.right[k] = r[k];
    A.up[k] = u[k];
    A.bmin[k] = h->cfg.origin[k];
    A.bmax[k] = h->cfg.origin[k] + (float)h->cfg.n[k] * h->cfg.spacing[k];
    A.tint[k] = p->water_tint[k];
    A.sun[k] = p->sun_direction[k];
  }
  A.half_h = p->orthographic ? p->size * 0.5f : (float)std::tan((double)p->fov_y_deg * M_PI / 360.0);
  A.half_w = A.half_h * ((float)p->width / (float)p->height);
  A.nx = h->cfg.n[0];
  A.ny = h->cfg.n[1];
  A.nz = h->cfg.n[2];
  A.width = p->width;
  A.height = p->height;
  A.mode = p->mode;
  A.ortho = p->orthographic ? 1 : 0;
  A.contact = p->contact_correction ? 1 : 0;
  A.clock_ready = p->clock_ready ? 1 : 0;
  A.slope = h->cfg.slope;
  A.attenuation = p->attenuation_distance;
  A.ripple = p->ripple_strength;
  A.roughness = p->surface_roughness;
  A.c = h->D.c;
  return true;
}
waves_status render_enqueue(waves_handle* h, wg::RenderArgs& A) {
  if (!h->export_planes) {
    CK(cudaMalloc(&h->export_planes, (size_t)h->D.N * sizeof(float4)));
    CK(cudaMalloc(&h->export_kinds, (size_t)h->D.N * sizeof(float)));
  }
  wg::launch_export(h->D, h->stream, h->export_planes, h->export_kinds);
  A.planes = h->export_planes;
  A.kinds = h->export_kinds;
  wg::launch_render(A, h->stream);
  CK(cudaGetLastError());
  return WAVES_OK;
}
}  // namespace

waves_status waves_render_device(waves_handle* h, const waves_render_params* p, void* rgba, void* trace) {
  wg::RenderArgs A;
  if (!h || !rgba || ((uintptr_t)rgba & 15) || ((uintptr_t)trace & 15) || !render_args(h, p, A)) return WAVES_INVALID_ARG;
  cudaSetDevice(h->cfg.device);
  A.rgba = (float4*)rgba;
  A.trace = (float4*)trace;
  return render_enqueue(h, A);
}

waves_status waves_render(waves_handle* h, const waves_render_params* p, float* rgba, float* trace) {
  wg::RenderArgs A;
  if (!h || !rgba || !render_args(h, p, A)) return WAVES_INVALID_ARG;
  cudaSetDevice(h->cfg.device);
  const size_t px = (size_t)p->width * p->height;
  if (h->render_px < px) {
    if (h->render_buf) cudaFree(h->render_buf);
    h->render_buf = nullptr;
    h->render_px = 0;
    CK(cudaMalloc(&h->render_buf, px * 2 * sizeof(float4)));
    h->render_px = px;
  }
  A.rgba = h->render_buf;
  A.trace = trace ? h->render_buf + px : nullptr;
  waves_status st;
  if ((st = render_enqueue(h, A)) != WAVES_OK) return st;
  CK(cudaMemcpyAsync(rgba, A.rgba, px * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
  if (trace) CK(cudaMemcpyAsync(trace, A.trace, px * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}

waves_status waves_get_history(waves_handle* h, float* history, float* coastal, uint32_t* audit) {
  if (!h) return WAVES_INVALID_ARG;
  cudaSetDevice(h->cfg.device);
  const size_t cap = (size_t)std::max(h->cfg.history_capacity, 1);
  if (history) CK(cudaMemcpyAsync(history, h->D.history, 16 * cap * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  if (coastal) CK(cudaMemcpyAsync(coastal, h->D.chistory, 20 * cap * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  if (audit) CK(cudaMemcpyAsync(audit, h->D.hstate, (64 + 32 * cap) * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}

size_t waves_bank_floats(const waves_handle* h) { return h ? (size_t)h->D.S : 0; }

waves_status waves_get_bank(waves_handle* h, int32_t bank, float* out) {
  if (!h || !out || bank < -1 || bank > 1) return WAVES_INVALID_ARG;
  if (bank < 0) {
    waves_status st;
    if ((st = read_control(h)) != WAVES_OK) return st;
    bank = (int)h->host_c[0];
  }
  CK(cudaMemcpyAsync(out, bank == 0 ? h->D.bank0 : h->D.bank1, (size_t)h->D.S * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}
waves_status waves_set_bank(waves_handle* h, int32_t bank, const float* in) {
  if (!h || !in || bank < -1 || bank > 1) return WAVES_INVALID_ARG;
  if (bank < 0) {
    waves_status st;
    if ((st = read_control(h)) != WAVES_OK) return st;
    bank = (int)h->host_c[0];
  }
  CK(cudaMemcpyAsync(bank == 0 ? h->D.bank0 : h->D.bank1, in, (size_t)h->D.S * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}
waves_status waves_get_geometry(waves_handle* h, float* phi, float* kind) {
  if (!h || !phi || !kind) return WAVES_INVALID_ARG;
  std::vector<signed char> k8((size_t)h->D.N);
  CK(cudaMemcpyAsync(phi, h->D.phi, (size_t)h->D.N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(k8.data(), h->D.kind, (size_t)h->D.N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (size_t i = 0; i < k8.size(); i++) kind[i] = (float)k8[i];
  return WAVES_OK;
}
waves_status waves_get_masks(waves_handle* h, float* pmask, float* vband) {
  if (!h || !pmask || !vband) return WAVES_INVALID_ARG;
  const size_t N = (size_t)h->D.N, NF = (size_t)h->D.NF;
  CK(cudaMemcpyAsync(pmask, h->D.pmask0, N * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(pmask + N, h->D.pmask1, N * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(vband, h->D.vband0, NF * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(vband + NF, h->D.vband1, NF * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}
waves_status waves_set_masks(waves_handle* h, const float* pmask, const float* vband) {
  if (!h || !pmask || !vband) return WAVES_INVALID_ARG;
  const size_t N = (size_t)h->D.N, NF = (size_t)h->D.NF;
  CK(cudaMemcpyAsync(h->D.pmask0, pmask, N * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->D.pmask1, pmask + N, N * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->D.vband0, vband, NF * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->D.vband1, vband + NF, NF * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}

// Checkpoint: magic, size, then every persistent allocation in creation order.
waves_status waves_save(waves_handle* h, void* buffer, size_t* bytes) {
  if (!h || !bytes) return WAVES_INVALID_ARG;
  size_t total = 16;
  for (const Alloc& a : h->allocs)
    if (a.persistent) total += a.bytes;
  if (!buffer) {
    *bytes = total;
    return WAVES_OK;
  }
  if (*bytes < total) return WAVES_INVALID_ARG;
  CK(cudaStreamSynchronize(h->stream));
  char* p = (char*)buffer;
  uint64_t magic = 0x3130305345564157ull, sz = total;  // "WAVES001"
  std::memcpy(p, &magic, 8);
  std::memcpy(p + 8, &sz, 8);
  size_t off = 16;
  for (const Alloc& a : h->allocs)
    if (a.persistent) {
      CK(cudaMemcpy(p + off, a.ptr, a.bytes, cudaMemcpyDeviceToHost));
      off += a.bytes;
    }
  *bytes = total;
  return WAVES_OK;
}
waves_status waves_load(waves_handle* h, const void* buffer, size_t bytes) {
  if (!h || !buffer) return WAVES_INVALID_ARG;
  size_t total = 16;
  for (const Alloc& a : h->allocs)
    if (a.persistent) total += a.bytes;
  const char* p = (const char*)buffer;
  uint64_t magic, sz;
  std::memcpy(&magic, p, 8);
  std::memcpy(&sz, p + 8, 8);
  if (bytes < total || magic != 0x3130305345564157ull || sz != total) {
    h->err = "checkpoint does not match this configuration";
    return WAVES_INVALID_ARG;
  }
  CK(cudaStreamSynchronize(h->stream));
  size_t off = 16;
  for (const Alloc& a : h->allocs)
    if (a.persistent) {
      CK(cudaMemcpy(a.ptr, p + off, a.bytes, cudaMemcpyHostToDevice));
      off += a.bytes;
    }
  return WAVES_OK;
}

waves_status waves_set_warm_start(waves_handle* h, const waves_warm_start_model* model) {
  if (!h) return WAVES_INVALID_ARG;
  Dev& D = h->D;
  if (!D.net_on) {
    h->err = "the handle was created without warm_start = 1";
    return WAVES_INVALID_ARG;
  }
  const double off = 0.0, on = 1.0;
  if (!model) {  // back to the previous accepted pressure
    CK(cudaMemcpyAsync(D.c + wg::kNetLoaded, &off, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return WAVES_OK;
  }
  const int ci_of[WAVES_NET_LAYERS] = {3, WAVES_NET_HIDDEN, WAVES_NET_HIDDEN, WAVES_NET_HIDDEN};
  const int co_of[WAVES_NET_LAYERS] = {WAVES_NET_HIDDEN, WAVES_NET_HIDDEN, WAVES_NET_HIDDEN, 1};
  for (int l = 0; l < WAVES_NET_LAYERS; l++)
    if (!model->weights[l] || !model->bias[l]) {
      h->err = "warm-start model with a missing layer";
      return WAVES_INVALID_ARG;
    }
  // weights[co][kz][ky][kx][ci] (BF16 bits) -> mma.m16n8k16 B fragments [tap][n-tile][lane][2]:
  // lane (g = lane / 4, t = lane % 4) holds output channel n = 8 j + g, input channels 2t, 2t + 1
  // (first register) and 2t + 8, 2t + 9 (second), low half first; absent channels are zero.
  std::vector<uint32_t> frag((size_t)WAVES_NET_LAYERS * wg::kNetLayerWords, 0u);
  std::vector<float> bias((size_t)WAVES_NET_LAYERS * 16, 0.f);
  std::vector<uint16_t> wt((size_t)WAVES_NET_LAYERS * 27 * 256, 0);
  for (int l = 0; l < WAVES_NET_LAYERS; l++) {
    const int CI = ci_of[l], CO = co_of[l], tiles = CO > 8 ? 2 : 1;
    auto w = [&](int co, int tap, int ci) -> uint32_t {
      if (co >= CO || ci >= CI) return 0u;
      return model->weights[l][((size_t)co * 27 + tap) * CI + ci];
    };
    for (int tap = 0; tap < 27; tap++)
      for (int j = 0; j < tiles; j++)
        for (int lane = 0; lane < 32; lane++) {
          const int n = 8 * j + lane / 4, t = lane % 4;
          const size_t at = (size_t)l * wg::kNetLayerWords + ((size_t)(tap * tiles + j) * 32 + lane) * 2;
          frag[at] = w(n, tap, 2 * t) | (w(n, tap, 2 * t + 1) << 16);
          frag[at + 1] = w(n, tap, 2 * t + 8) | (w(n, tap, 2 * t + 9) << 16);
        }
    for (int co = 0; co < CO; co++) bias[(size_t)l * 16 + co] = model->bias[l][co];
    // tcgen05 B operand, K-major without swizzle: per tap two planes (input channels 0-7, 8-15),
    // each one 16-byte row of 8 channels per output channel
    for (int tap = 0; tap < 27; tap++)
      for (int half = 0; half < 2; half++)
        for (int n = 0; n < 16; n++)
          for (int k = 0; k < 8; k++)
            wt[(size_t)l * 27 * 256 + (size_t)tap * 256 + half * 128 + n * 8 + k] = (uint16_t)w(n, tap, half * 8 + k);
  }
  const float scale[4] = {model->input_scale[0], model->input_scale[1], model->input_scale[2], model->output_scale};
  CK(cudaMemcpyAsync(D.net_w, frag.data(), frag.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(D.net_wt, wt.data(), wt.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(D.net_b, bias.data(), bias.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(D.net_scale, scale, sizeof(scale), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(D.c + wg::kNetLoaded, &on, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return WAVES_OK;
}

const char* waves_last_error(const waves_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

// ---------------------------------------------------------------- debugging hooks (include/waves_debug.h)
waves_status waves_debug_phase(waves_handle* h, int32_t phase) {
  if (!h) return WAVES_INVALID_ARG;
  const Dev& D = h->D;
  cudaStream_t s = h->stream;
  switch (phase) {
    case 0: upload_quota(h); wg::launch_begin(D, s); break;
    case 1: wg::launch_motion_cfl(D, s); break;
    case 2: wg::launch_sweep(D, s); break;
    case 3: wg::launch_maccormack(D, s); break;
    case 4: if (D.coastal) wg::launch_coastal(D, s); break;
    case 5: wg::launch_geometry(D, s); break;
    case 6: wg::launch_proj_setup(D, s); break;
    case 7: wg::launch_mg_build(D, s); break;
    case 8: enqueue_cg_begin(h, s); break;
    case 9: enqueue_cg_iteration(h, s, 0, 0); break;
    case 10: wg::launch_post(D, s); break;
    case 11: wg::launch_trial_end(D, s); break;
    case 12: wg::launch_warm_start(D, s); break;
    default: return WAVES_INVALID_ARG;
  }
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  return WAVES_OK;
}
waves_status waves_debug_sample(waves_handle* h, const float* x, int32_t axis, int32_t forward, float* out40) {
  if (!h || !x || !out40) return WAVES_INVALID_ARG;
  float* d;
  CK(cudaMalloc(&d, 40 * sizeof(float)));
  wg::launch_debug_sample(h->D, h->stream, x, axis, forward, d);
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(out40, d, 40 * sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(d);
  return WAVES_OK;
}
waves_status waves_debug_probe_trial(waves_handle* h, waves_kernel_probe* out, int32_t capacity, int32_t* trials) {
  if (!h || !out || capacity < 1) return WAVES_INVALID_ARG;
  if (h->cfg.iterations_per_batch < 1) return WAVES_INVALID_ARG;
  for (int k = 0; k < capacity; k++) out[k] = waves_kernel_probe{k, 0, 0.0, 0.0};
  std::vector<wg::ProbeRec> recs;
  wg::g_probe = &recs;
  waves_status st = WAVES_OK;
  int32_t done = 0;
  // one host-scheduled trial with every CG iteration checked: no probed launch is a no-op
  if ((st = upload_quota(h)) == WAVES_OK) st = host_trial(h, 1);
  // calibration: the cost of the two nested event brackets of a probed launch, measured on an
  // empty kernel bracketed the same way (kind kProbeEmpty around kProbeEmptyInner)
  if (st == WAVES_OK)
    for (int k = 0; k < 64; k++)
      wg::probed(wg::kProbeEmpty, h->stream, 0.0, [&] { wg::probed(wg::kProbeEmptyInner, h->stream, 0.0, [&] { wg::launch_empty(h->stream); }); });
  wg::g_probe = nullptr;
  if (st == WAVES_OK) done = 1;
  if (st == WAVES_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) st = WAVES_CUDA_ERROR;
  // the level sweeps visit the active rows only: their bytes, counted over every row, are scaled
  // to the active rows of the trial's hierarchy
  unsigned active[wg::kMaxLevels] = {0};
  if (st == WAVES_OK && cudaMemcpy(active, h->D.mg_rowcount, sizeof(active), cudaMemcpyDeviceToHost) != cudaSuccess)
    st = WAVES_CUDA_ERROR;
  for (wg::ProbeRec& r : recs)
    if (r.level >= 1 && r.level < h->D.L && h->D.lv[r.level].count > 0)
      r.bytes *= (double)active[r.level] / (double)h->D.lv[r.level].count;
  for (const wg::ProbeRec& r : recs) {
    float ms = 0.f;
    if (st == WAVES_OK && r.kind < capacity && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      out[r.kind].launches++;
      out[r.kind].ms += ms;
      out[r.kind].bytes += r.bytes;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  if (trials) *trials = done;
  cudaGetLastError();
  return st;
}

waves_status waves_debug_launch_counts(waves_handle* h, int32_t* out8) {
  if (!h || !out8) return WAVES_INVALID_ARG;
  std::memcpy(out8, h->launches, sizeof(h->launches));
  return WAVES_OK;
}
waves_status waves_debug_read(waves_handle* h, const char* name, void* out, size_t bytes) {
  if (!h || !name || !out) return WAVES_INVALID_ARG;
  for (const Alloc& a : h->allocs)
    if (std::strcmp(a.name, name) == 0) {
      if (bytes > a.bytes) return WAVES_INVALID_ARG;
      CK(cudaStreamSynchronize(h->stream));
      CK(cudaMemcpy(out, a.ptr, bytes, cudaMemcpyDeviceToHost));
      return WAVES_OK;
    }
  h->err = std::string("no device array named ") + name;
  return WAVES_INVALID_ARG;
}

}  // extern "C"
