// TEST INFRASTRUCTURE ONLY — C entry points of the CPU oracle (wo_solver.hpp) for the pytest
// suite (ctypes) and for bench.py's CPU-baseline leg.  Never linked into the product library.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>

#include <omp.h>

#include "wo_solver.hpp"

namespace {
struct Box {
  int precision = 32;
  std::unique_ptr<wo::Solver<float>> f;
  std::unique_ptr<wo::Solver<double>> d;
};
template <class Fn> auto with(void* h, Fn fn) {
  Box* b = static_cast<Box*>(h);
  if (b->precision == 64) return fn(*b->d);
  return fn(*b->f);
}
template <class R> void copy_out(const std::vector<R>& v, float* out) {
  for (size_t i = 0; i < v.size(); i++) out[i] = float(v[i]);
}
template <class R> void copy_in(std::vector<R>& v, const float* in) {
  for (size_t i = 0; i < v.size(); i++) v[i] = R(in[i]);
}
}  // namespace

extern "C" {

// OpenMP threads of the oracle's parallel loops (n <= 0: the number of processors); returns the
// count in effect.  Every parallel loop writes disjoint outputs and every floating-point sum is
// sequential, so results do not depend on it.
int wo_set_threads(int n) {
  omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
  return omp_get_max_threads();
}

// precision 32: FP32 decision-parity oracle; 64: FP64 error oracle.  Runs the initial commands.
void* wo_create(const waves_config* cfg, int precision) {
  Box* b = new Box;
  b->precision = precision;
  if (precision == 64) {
    b->d.reset(new wo::Solver<double>(*cfg));
    b->d->initial_commands();
  } else {
    b->f.reset(new wo::Solver<float>(*cfg));
    b->f->initial_commands();
  }
  return b;
}
void wo_destroy(void* h) { delete static_cast<Box*>(h); }
void wo_set_quota(void* h, double quota) {
  with(h, [&](auto& s) { s.quota = quota; return 0; });
}
int wo_run(void* h, int max_batches) {
  return with(h, [&](auto& s) { return s.run(max_batches); });
}
void wo_batch(void* h) {
  with(h, [&](auto& s) { s.batch(); return 0; });
}
void wo_get_control(void* h, double* out) {
  with(h, [&](auto& s) { std::memcpy(out, s.c, sizeof(s.c)); return 0; });
}
void wo_set_control(void* h, const double* in) {
  with(h, [&](auto& s) { std::memcpy(s.c, in, sizeof(s.c)); return 0; });
}
size_t wo_bank_floats(void* h) {
  return with(h, [&](auto& s) { return s.S; });
}
void wo_get_bank(void* h, int bank, float* out) {
  with(h, [&](auto& s) { copy_out(s.bank[bank], out); return 0; });
}
void wo_get_bank_d(void* h, int bank, double* out) {
  with(h, [&](auto& s) {
    for (size_t i = 0; i < s.S; i++) out[i] = double(s.bank[bank][i]);
    return 0;
  });
}
void wo_set_bank(void* h, int bank, const float* in) {
  with(h, [&](auto& s) { copy_in(s.bank[bank], in); return 0; });
}
void wo_get_geometry(void* h, float* phi, float* kind) {
  with(h, [&](auto& s) { copy_out(s.gphi, phi); copy_out(s.gkind, kind); return 0; });
}
// Signed distance and kind of every cell (the geometry a trial leaves for the next one), e.g. from a
// state the GPU reached.
void wo_set_geometry(void* h, const float* phi, const float* kind) {
  with(h, [&](auto& s) { copy_in(s.gphi, phi); copy_in(s.gkind, kind); return 0; });
}
// Pressure masks and valid bands of both banks: pmask[2N], vband[2 faces].
void wo_get_masks(void* h, float* pmask, float* vband) {
  with(h, [&](auto& s) {
    for (int b = 0; b < 2; b++) {
      copy_out(s.pmask[b], pmask + b * s.N);
      copy_out(s.vband[b], vband + b * s.NF);
    }
    return 0;
  });
}
void wo_set_masks(void* h, const float* pmask, const float* vband) {
  with(h, [&](auto& s) {
    for (int b = 0; b < 2; b++) {
      copy_in(s.pmask[b], pmask + b * s.N);
      copy_in(s.vband[b], vband + b * s.NF);
    }
    return 0;
  });
}
void wo_get_export(void* h, float* planes, float* kinds) {
  with(h, [&](auto& s) {
    for (size_t i = 0; i < s.N; i++) {
      planes[4 * i] = float(s.exp_plane[i].x);
      planes[4 * i + 1] = float(s.exp_plane[i].y);
      planes[4 * i + 2] = float(s.exp_plane[i].z);
      planes[4 * i + 3] = float(s.exp_plane[i].w);
      kinds[i] = float(s.exp_kind[i]);
    }
    return 0;
  });
}
void wo_get_probes(void* h, float* out32) {
  with(h, [&](auto& s) {
    for (int i = 0; i < 8; i++)
      for (int k = 0; k < 4; k++) out32[4 * i + k] = float(s.probe[i][k]);
    return 0;
  });
}
int wo_mg_levels(void* h, int* dims, int* stencils) {
  return with(h, [&](auto& s) {
    int L = s.L();
    for (int l = 0; l < L; l++) {
      for (int a = 0; a < 3; a++) dims[3 * l + a] = s.mg.levels[l].n[a];
      stencils[l] = int(s.mg.levels[l].stencil.size());
    }
    return L;
  });
}
// Stencil offsets of level l (3 ints each).
int wo_mg_stencil(void* h, int l, int* offsets) {
  return with(h, [&](auto& s) {
    const auto& st = s.mg.levels[l].stencil;
    for (size_t k = 0; k < st.size(); k++)
      for (int a = 0; a < 3; a++) offsets[3 * k + a] = st[k][a];
    return int(st.size());
  });
}
// Multigrid audit state header (first 32 words).
void wo_mg_state(void* h, uint32_t* out32) {
  with(h, [&](auto& s) {
    for (int k = 0; k < 32; k++) out32[k] = s.mg.state[k];
    return 0;
  });
}
// The whole audit state: the 64-word header, then 32 words per rebuild.
void wo_mg_audit(void* h, uint32_t* out, size_t words) {
  with(h, [&](auto& s) {
    for (size_t k = 0; k < words && k < s.mg.state.size(); k++) out[k] = s.mg.state[k];
    return 0;
  });
}
// Step history rows (4 per trial) and coastal history rows (5 per step), vec4 each.
void wo_get_history(void* h, float* hist, float* chist) {
  with(h, [&](auto& s) {
    for (size_t i = 0; i < s.history.size(); i++)
      for (int k = 0; k < 4; k++) hist[4 * i + k] = float(s.history[i][k]);
    for (size_t i = 0; i < s.chistory.size(); i++)
      for (int k = 0; k < 4; k++) chist[4 * i + k] = float(s.chistory[i][k]);
    return 0;
  });
}

// Closed-form PLIC functions in FP32 (plic_math.glslinc:3-37).
float wo_cube_volume(float nx, float ny, float nz, float alpha) {
  return wo::Solver<float>::cube_volume(wo::V3<float>(nx, ny, nz), alpha);
}
float wo_inverse_volume(float nx, float ny, float nz, float f) {
  return wo::Solver<float>::inverse_volume(wo::V3<float>(nx, ny, nz), f);
}
double wo_cube_volume_d(double nx, double ny, double nz, double alpha) {
  return wo::Solver<double>::cube_volume(wo::V3<double>(nx, ny, nz), alpha);
}
double wo_inverse_volume_d(double nx, double ny, double nz, double f) {
  return wo::Solver<double>::inverse_volume(wo::V3<double>(nx, ny, nz), f);
}

// Run one phase of a batch, in the phase numbering of include/waves_debug.h.
void wo_phase(void* h, int phase) {
  with(h, [&](auto& s) {
    switch (phase) {
      case 0: s.op43(); s.op1(); break;
      case 1: s.op20_21(); s.op45_46(); s.op22(); break;
      case 2: s.op23(); s.op24(); s.op55_56(); s.op25_26(); break;
      case 3: s.op27_28(27); s.op27_28(28); break;
      case 4: if (s.coastal) { s.op80_81(); s.op82(); s.op83_84(); s.op87_88(); } break;
      case 5: s.op17(); s.op18(); s.op16(); break;
      case 6: s.op2(); s.op47(); break;
      case 7: s.mg_build(); break;
      case 8: s.op63(); s.op64(); s.op3(); s.mg_cycle(0); s.op4(); break;
      case 9: s.op5(); s.op6_7(); s.op8(); s.mg_cycle(1); s.op9(); s.op10(); break;
      case 10: s.op11(); s.op65(); s.op47(); s.op30(); s.op31_33(31); s.op31_33(32); s.op31_33(33); s.op34();
               s.op47(); s.op48_49(false); s.op35_36(); s.op62_66(); s.op12_13(); break;
      case 11: s.op44(); if (s.coastal) { s.op85(); s.op89(); } break;
    }
    return 0;
  });
}
// Scratch arrays by name (float copies): "fwd", "plane" (4N), "coef" (6N), "diag", "r", "z", "d", "q", "b",
// "tcache" (6 faces), "mF", "mci", "src1" (as float).
int wo_read(void* h, const char* name, float* out) {
  return with(h, [&](auto& s) {
    std::string n(name);
    if (n == "fwd") copy_out(s.fwd, out);
    else if (n == "mF") copy_out(s.mF, out);
    else if (n == "mci") copy_out(s.mci, out);
    else if (n == "plane") { for (size_t i = 0; i < s.N; i++) for (int k = 0; k < 4; k++) out[4 * i + k] = float(s.plane[i][k]); }
    else if (n == "coef") { for (size_t i = 0; i < 6 * s.N; i++) out[i] = float(s.work[6 * s.N + i]); }
    else if (n == "diag") { for (size_t i = 0; i < s.N; i++) out[i] = float(s.work[12 * s.N + i]); }
    else if (n == "r") { for (size_t i = 0; i < s.N; i++) out[i] = float(s.work[i]); }
    else if (n == "z") { for (size_t i = 0; i < s.N; i++) out[i] = float(s.work[s.N + i]); }
    else if (n == "d") { for (size_t i = 0; i < s.N; i++) out[i] = float(s.work[2 * s.N + i]); }
    else if (n == "q") { for (size_t i = 0; i < s.N; i++) out[i] = float(s.work[3 * s.N + i]); }
    else if (n == "b") { for (size_t i = 0; i < s.N; i++) out[i] = float(s.work[5 * s.N + i]); }
    else if (n == "pbase") { for (size_t i = 0; i < s.N; i++) out[i] = float(s.work[13 * s.N + i]); }
    else if (n == "tcache") { for (int k = 0; k < 6; k++) copy_out(s.tcache[k], out + k * s.NF); }
    else if (n == "src1") { for (size_t i = 0; i < s.NF; i++) out[i] = float(s.src[1][i]); }
    else return 0;
    return 1;
  });
}

// Seconds of wall time for `batches` batches (CPU-baseline timing).
double wo_time_batches(void* h, int batches) {
  auto t0 = std::chrono::steady_clock::now();
  with(h, [&](auto& s) { return s.run(batches); });
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
