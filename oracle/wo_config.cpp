// TEST INFRASTRUCTURE ONLY — the oracle's own configuration presets, restated from the reference's
// GDScript settings so that the oracle (and bench.py's CPU-baseline leg) builds its inputs without
// the product library.  tests/test_cpu_oracle.py checks that the product's presets
// (waves_gb300/csrc/config.cpp) fill the same struct with the same bits.
#include <cmath>
#include <cstring>

#include "../include/waves.h"

extern "C" {

// lab_runner.gd:19-25: omega^2 = g k tanh(k h) solved for k by 80 bisection steps on [0, 100].
double wo_dispersion_k(double period_s, double depth_m) {
  const double omega = 2.0 * M_PI / period_s;
  double low = 0.0, high = 100.0;
  for (int iteration = 0; iteration < 80; iteration++) {
    const double k = (low + high) * .5;
    if (9.81 * k * std::tanh(k * depth_m) < omega * omega) low = k;
    else high = k;
  }
  return (low + high) * .5;
}

// Defaults of the GDScript chain: pressure_gpu.gd:40-44 (multigrid options: Chebyshev, 3 sweeps,
// lagged maintenance with lag 8, aggregation from level 2), pressure_gpu.gd:67-68 (dt 1/120),
// coupled_gpu.gd:7-22 (transport cache on, interior fast path off, valid-band advection on,
// history 2400, tolerance 1e-4, gravity 1, 8 iterations per batch), coastal_gpu.gd:21-25 (zone
// 2.5 m, rate 12 /s, 4 ramp periods, right absorption 1); geometry: the 64x48x16 wall tank.
void wo_config_default(waves_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->n[0] = 64;
  c->n[1] = 48;
  c->n[2] = 16;
  c->spacing[0] = 0.025f;
  c->spacing[1] = 0.025f;
  c->spacing[2] = 0.05f;
  c->eta = 0.45f;
  c->dt = float(1.0 / 120);
  c->gravity = 1.f;
  c->history_capacity = 2400;
  c->pressure_tolerance = 1e-4f;
  c->active_advection = 1;
  c->transport_cache = 1;
  c->zone_length = 2.5f;
  c->damping_rate = 12.f;
  c->ramp_periods = 4.f;
  c->right_absorption = 1.f;
  c->mg_smoother = 1;
  c->mg_smoothing = 3;
  c->mg_maintenance = 2;
  c->mg_lag = 8;
  c->mg_aggregate_from = 2;
  c->iterations_per_batch = 8;
  c->cfl = 0.45f;  // coupled_motion.glslinc:364
  c->mg_precision = 32;
}

// lab_runner.gd:26: n 310x48x80, spacing (.025, .025, .05), origin (-1.75, -.6, -2), eta 0, shape 7,
// wave (.08, k, 2 pi / 1.4, .45), Stokes-2 on, history 10000, slope 6; through coastal_gpu.gd.
void wo_config_beach(waves_config* c) {
  wo_config_default(c);
  c->n[0] = 310;
  c->n[1] = 48;
  c->n[2] = 80;
  c->origin[0] = -1.75f;
  c->origin[1] = -0.6f;
  c->origin[2] = -2.f;
  c->eta = 0.f;
  c->shape = 7;
  c->wave[0] = 0.08f;
  c->wave[1] = float(wo_dispersion_k(1.4, 0.45));
  c->wave[2] = float(2.0 * M_PI / 1.4);
  c->wave[3] = 0.45f;
  c->stokes_second = 1;
  c->history_capacity = 10000;
  c->slope = 6.f;
  c->coastal = 1;
}

// The sloshing tank of the benchmark's first configuration: 64x48x16, surface
// 0.45 + 0.05 sin(2 pi x / 1.6) (the reference's cosine corrugation shifted by -pi/2), flat floor,
// wall variant, CFL 0.5, CG relative tolerance 1e-6.
void wo_config_tank(waves_config* c) {
  wo_config_default(c);
  c->corrugation = 0.05f;
  c->corrugation_phase = float(-M_PI / 2);
  c->pressure_tolerance = 1e-6f;
  c->cfl = 0.5f;
}

}  // extern "C"
