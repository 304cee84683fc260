// Configuration presets of the C ABI (include/waves.h).
#include <cmath>
#include <cstring>

#include "../../include/waves.h"

extern "C" {

// lab_runner.gd:19-25: solve omega^2 = g k tanh(k h) for k by 80 bisection steps on [0, 100].
double waves_dispersion_k(double period_s, double depth_m) {
  const double omega = 2.0 * M_PI / period_s;
  double low = 0.0, high = 100.0;
  for (int it = 0; it < 80; it++) {
    double k = (low + high) * .5;
    if (9.81 * k * std::tanh(k * depth_m) < omega * omega) low = k;
    else high = k;
  }
  return (low + high) * .5;
}

// Reference defaults: pressure_gpu.gd:40-44,67-68; coupled_gpu.gd:7-22; coastal_gpu.gd:5-25;
// work_scheduler.gd; with the 64x48x16 flat-floor wall tank as geometry.
void waves_config_default(waves_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->n[0] = 64; c->n[1] = 48; c->n[2] = 16;
  c->spacing[0] = 0.025f; c->spacing[1] = 0.025f; c->spacing[2] = 0.05f;
  c->origin[0] = 0.f; c->origin[1] = 0.f; c->origin[2] = 0.f;
  c->eta = 0.45f;
  c->dt = float(1.0 / 120);
  c->periodic_x = 0;
  c->slope = 0.f;
  c->corrugation = 0.f;
  c->corrugation_phase = 0.f;
  c->shape = 0;
  c->gravity = 1.f;
  c->max_face_cfl = 0;
  c->history_capacity = 2400;
  c->pressure_tolerance = 1e-4f;
  c->linear_air = 0;
  c->stokes_second = 0;
  c->height_normals = 0;
  c->active_advection = 1;
  c->transport_cache = 1;
  c->transport_interior = 0;
  c->coastal = 0;
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
  c->cfl = 0.45f;
  c->mg_precision = 32;
  c->warm_start = 0;
  c->device = 0;
}

// lab_runner.gd:26 settings, through coastal_gpu.gd (offshore forcing, Stokes-2 on).
void waves_config_beach(waves_config* c) {
  waves_config_default(c);
  c->n[0] = 310; c->n[1] = 48; c->n[2] = 80;
  c->origin[0] = -1.75f; c->origin[1] = -0.6f; c->origin[2] = -2.f;
  c->eta = 0.f;
  c->shape = 7;
  const double omega = 2.0 * M_PI / 1.4;
  c->wave[0] = 0.08f;
  c->wave[1] = float(waves_dispersion_k(1.4, 0.45));
  c->wave[2] = float(omega);
  c->wave[3] = 0.45f;
  c->stokes_second = 1;
  c->history_capacity = 10000;
  c->slope = 6.f;
  c->coastal = 1;
}

// Sloshing tank: 64x48x16, surface 0.45 + 0.05 sin(2 pi x / 1.6) (cosine corrugation shifted by
// -pi/2), flat floor, wall variant, CFL 0.5, CG tolerance 1e-6.
void waves_config_tank(waves_config* c) {
  waves_config_default(c);
  c->corrugation = 0.05f;
  c->corrugation_phase = float(-M_PI / 2);
  c->pressure_tolerance = 1e-6f;
  c->cfl = 0.5f;
}

}  // extern "C"
