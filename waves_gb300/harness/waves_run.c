/*
 * waves_run: headless driver of the waves solver step through the C ABI only (include/waves.h).
 *
 *   waves_run [--preset beach|large|tank|default] [--seconds S | --steps K] [--tol T] [--mg 32|16]
 *             [--frame DT] [--surface FILE] [--image FILE.ppm] [--view water|clay] [--size WxH]
 *             [--model FILE]
 *
 * It plays the role of the reference's lab runner (water/lab_runner.gd:49-73): it requests
 * accepted time frame by frame (1/60 s by default, request_time), runs the solver until each
 * frame's quota is met, and prints one JSON line per run with the telemetry of waves_stats and
 * the device time of waves_timing.  --surface writes the last accepted surface export (float4
 * planes then float kinds, ops 19/14) to a file; --image renders the last accepted surface
 * (waves_render, the default camera of the configuration) to a binary PPM, sRGB-encoded.  --model
 * loads a learned warm start (waves_set_warm_start, warm_start = 1) from the raw model file that
 * waves_gb300.learned.write_raw_model writes: the 8 bytes "WVNET1\0\0", then per layer
 * (3 -> 16 -> 16 -> 16 -> 1 channels) the BF16 weights [co][27][ci] as little-endian uint16 and
 * the FP32 biases [co], then the three FP32 input scales and the FP32 output scale.  The exit
 * status is 0 on success, 1 on a bad argument (or model file), 2 when the library fails, 3 when
 * the solver halts.
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "waves.h"

/* The learned warm start of a raw model file (format above): 0 on success, -1 on a bad file. */
static const int kCi[WAVES_NET_LAYERS] = {3, 16, 16, 16}, kCo[WAVES_NET_LAYERS] = {16, 16, 16, 1};
static uint16_t* g_weights[WAVES_NET_LAYERS];
static float* g_bias[WAVES_NET_LAYERS];
static int read_model(const char* path, waves_warm_start_model* m) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  char magic[8];
  int ok = fread(magic, 1, 8, f) == 8 && !memcmp(magic, "WVNET1\0\0", 8);
  for (int l = 0; ok && l < WAVES_NET_LAYERS; l++) {
    const size_t nw = (size_t)kCo[l] * 27 * kCi[l];
    g_weights[l] = (uint16_t*)malloc(nw * sizeof(uint16_t));
    g_bias[l] = (float*)malloc((size_t)kCo[l] * sizeof(float));
    ok = g_weights[l] && g_bias[l] && fread(g_weights[l], sizeof(uint16_t), nw, f) == nw &&
         fread(g_bias[l], sizeof(float), (size_t)kCo[l], f) == (size_t)kCo[l];
    m->weights[l] = g_weights[l];
    m->bias[l] = g_bias[l];
  }
  ok = ok && fread(m->input_scale, sizeof(float), 3, f) == 3 && fread(&m->output_scale, sizeof(float), 1, f) == 1;
  ok = ok && fgetc(f) == EOF;
  fclose(f);
  return ok ? 0 : -1;
}

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

int main(int argc, char** argv) {
  const char* preset = "beach";
  const char* surface = NULL;
  const char* image = NULL;
  const char* model_path = NULL;
  int view = 1, width = 1280, height = 720;
  double seconds = 1.0, frame = 1.0 / 60.0, tol = 1e-6;
  long steps = 0;
  int mg = 32;
  for (int i = 1; i < argc; i++) {
    const char* a = argv[i];
    const char* v = i + 1 < argc ? argv[i + 1] : NULL;
    if (!strcmp(a, "--preset") && v) preset = v, i++;
    else if (!strcmp(a, "--seconds") && v) seconds = atof(v), i++;
    else if (!strcmp(a, "--steps") && v) steps = atol(v), i++;
    else if (!strcmp(a, "--tol") && v) tol = atof(v), i++;
    else if (!strcmp(a, "--mg") && v) mg = atoi(v), i++;
    else if (!strcmp(a, "--frame") && v) frame = atof(v), i++;
    else if (!strcmp(a, "--surface") && v) surface = v, i++;
    else if (!strcmp(a, "--image") && v) image = v, i++;
    else if (!strcmp(a, "--model") && v) model_path = v, i++;
    else if (!strcmp(a, "--view") && v && (!strcmp(v, "water") || !strcmp(v, "clay"))) view = !strcmp(v, "water"), i++;
    else if (!strcmp(a, "--size") && v && sscanf(v, "%dx%d", &width, &height) == 2 && width > 0 && height > 0) i++;
    else {
      fprintf(stderr, "usage: %s [--preset beach|large|tank|default] [--seconds S | --steps K] [--tol T] [--mg 32|16] "
                      "[--frame DT] [--surface FILE] [--image FILE.ppm] [--view water|clay] [--size WxH] [--model FILE]\n",
              argv[0]);
      return 1;
    }
  }
  waves_config cfg;
  if (!strcmp(preset, "beach")) waves_config_beach(&cfg);
  else if (!strcmp(preset, "large")) {
    /* the beach at half the spacing: 620 x 96 x 160 cells, 8 multigrid levels */
    waves_config_beach(&cfg);
    cfg.n[0] = 620, cfg.n[1] = 96, cfg.n[2] = 160;
    cfg.spacing[0] = 0.0125f, cfg.spacing[1] = 0.0125f, cfg.spacing[2] = 0.025f;
  } else if (!strcmp(preset, "tank")) waves_config_tank(&cfg);
  else if (!strcmp(preset, "default")) waves_config_default(&cfg);
  else {
    fprintf(stderr, "unknown preset %s\n", preset);
    return 1;
  }
  cfg.pressure_tolerance = (float)tol;
  cfg.mg_precision = mg;
  waves_warm_start_model model;
  memset(&model, 0, sizeof(model));
  if (model_path) {
    if (read_model(model_path, &model) != 0) {
      fprintf(stderr, "bad model file %s\n", model_path);
      return 1;
    }
    cfg.warm_start = 1;
  }
  waves_handle* h = NULL;
  waves_status st = waves_create(&cfg, &h);
  if (st != WAVES_OK) {
    fprintf(stderr, "waves_create: %d %s\n", (int)st, waves_last_error(NULL));
    return 2;
  }
  if (model_path && (st = waves_set_warm_start(h, &model)) != WAVES_OK) {
    fprintf(stderr, "waves_set_warm_start: %d %s\n", (int)st, waves_last_error(h));
    waves_destroy(h);
    return 2;
  }
  int halted = 0;
  const double t0 = now_s();
  if (steps > 0) {
    waves_request_steps(h, steps);
    st = waves_run(h, 4);
    halted = st == WAVES_SOLVER_FAILED;
  } else {
    for (double t = frame; t <= seconds + 1e-9 && !halted; t += frame) {
      waves_request_time(h, t);
      st = waves_run(h, 4);
      halted = st == WAVES_SOLVER_FAILED;
    }
  }
  if (st != WAVES_OK && !halted) {
    fprintf(stderr, "waves_run: %d %s\n", (int)st, waves_last_error(h));
    waves_destroy(h);
    return 2;
  }
  waves_synchronize(h);
  const double wall = now_s() - t0;
  waves_stats_t s;
  waves_stats(h, &s);
  double motion_ms = 0, pressure_ms = 0;
  int64_t trials = 0;
  waves_timing(h, &motion_ms, &pressure_ms, &trials, 0);
  printf("{\"preset\": \"%s\", \"n\": [%d, %d, %d], \"accepted_steps\": %lld, \"accepted_time\": %.9g, "
         "\"trials\": %lld, \"failure\": %d, \"wall_s\": %.6g, \"sim_s_per_wall_s\": %.6g, "
         "\"device_motion_ms\": %.6g, \"device_pressure_ms\": %.6g}\n",
         preset, cfg.n[0], cfg.n[1], cfg.n[2], (long long)s.accepted_steps, s.accepted_time, (long long)trials,
         (int)s.failure, wall, wall > 0 ? s.accepted_time / wall : 0.0, motion_ms, pressure_ms);
  if (surface) {
    const size_t n = (size_t)cfg.n[0] * cfg.n[1] * cfg.n[2];
    float* planes = (float*)malloc(n * 4 * sizeof(float));
    float* kinds = (float*)malloc(n * sizeof(float));
    FILE* f = planes && kinds ? fopen(surface, "wb") : NULL;
    if (f && waves_export_surface(h, planes, kinds) == WAVES_OK) {
      fwrite(planes, sizeof(float), n * 4, f);
      fwrite(kinds, sizeof(float), n, f);
    }
    if (f) fclose(f);
    free(planes);
    free(kinds);
  }
  if (image) {
    waves_render_params p;
    waves_render_params_default(&p, &cfg, width, height);
    p.mode = view;
    const size_t px = (size_t)width * height;
    float* rgba = (float*)malloc(px * 4 * sizeof(float));
    unsigned char* rgb = (unsigned char*)malloc(px * 3);
    FILE* f = rgba && rgb ? fopen(image, "wb") : NULL;
    if (f && waves_render(h, &p, rgba, NULL) == WAVES_OK) {
      for (size_t i = 0; i < px; i++)
        for (int k = 0; k < 3; k++) {
          double c = rgba[4 * i + k];
          c = c <= 0.0 ? 0.0 : (c >= 1.0 ? 1.0 : c);
          rgb[3 * i + k] = (unsigned char)(255.0 * pow(c, 1.0 / 2.2) + 0.5);
        }
      fprintf(f, "P6\n%d %d\n255\n", width, height);
      fwrite(rgb, 1, px * 3, f);
    } else {
      fprintf(stderr, "render failed: %s\n", waves_last_error(h));
    }
    if (f) fclose(f);
    free(rgba);
    free(rgb);
  }
  waves_destroy(h);
  return halted ? 3 : 0;
}
