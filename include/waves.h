/*
 * waves.h — C ABI of the GB300-native waves solver step.
 *
 * One handle owns one simulation on one CUDA device: both physical banks (F, u, v, w, p), the
 * geometry/coefficient work arrays, the multigrid hierarchy, the device control block and its
 * CUDA stream.  No pointer to device memory escapes; every exchange with the caller goes through
 * host buffers that the caller owns.
 *
 * Each entry point names the GDScript interface it replaces in neuron-forest/waves:
 *   water/pressure_gpu.gd   — _init/start (:40-47), request (:48-49), request_time (:52-54),
 *                             close (:55-59), _stats (:133-137), planes/kinds textures (:4-5)
 *   water/coupled_gpu.gd    — step recorder _record_commands (:38-56), _stats (:58-65)
 *   water/coastal_gpu.gd    — coastal forcing layer (:1-38)
 *   water/pressure_multigrid.gd, water/pressure_hierarchy_state.gd — preconditioner (:33-198, :13-41)
 *   water/lab_runner.gd:19-26 — the beach settings dictionary (waves_config_beach)
 *
 * Threading: a handle is used by one thread at a time, except waves_request_steps /
 * waves_request_time, which may be called from any thread (the quota is an atomic).
 * Device: a call on a handle makes the handle's device current on the calling thread (the training
 * calls, the device they are given) and leaves it current.
 * Errors never abort the process: every call returns a waves_status; solver failures are the
 * reference's codes in waves_stats_t.failure.
 */
#ifndef WAVES_H
#define WAVES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WAVES_ABI_VERSION 1

/* Number of doubles in the device control block (reference c[], 96 floats, coastal_gpu.gd:8,
 * widened to FP64 and extended with build-only slots from index 96). */
#define WAVES_CONTROL_SIZE 128

typedef enum waves_status {
  WAVES_OK = 0,
  WAVES_INVALID_ARG = 1,
  WAVES_CUDA_ERROR = 2,
  WAVES_NO_DEVICE = 3,
  WAVES_SOLVER_FAILED = 4, /* stats.failure != 0 (the reference halts, work_scheduler.gd:44) */
  WAVES_NOT_READY = 5,
  WAVES_OUT_OF_MEMORY = 6
} waves_status;

/* Settings dictionary + push-constant fields of the reference (pressure_gpu.gd:67-68,
 * coupled_gpu.gd:16-22, coastal_gpu.gd:21-25) plus the multigrid options set in
 * pressure_gpu.gd:42-43.  Floats are what the reference packs as FP32 push constants. */
typedef struct waves_config {
  int32_t n[3];              /* cells nx, ny, nz                           settings "n" */
  float spacing[3];          /* cell size hx, hy, hz (m)                   settings "spacing" */
  float origin[3];           /* lower corner of cell (0,0,0) (m)           settings "origin" */
  float eta;                 /* still-water level (m)                      settings "eta" */
  float dt;                  /* maximum time step (s), default 1/120       settings "dt" */
  int32_t periodic_x;        /* x periodic                                 settings "periodic_x" */
  float slope;               /* bed slope denominator, 0 = flat floor      settings "slope" */
  float corrugation;         /* cosine surface amplitude (m)               settings "corrugation" */
  float corrugation_phase;   /* phase added to the cosine (rad); 0 in the reference */
  int32_t shape;             /* initial fixture 0..7                       settings "shape" */
  float gravity;             /* gravity multiplier                         settings "gravity" */
  int32_t max_face_cfl;      /* CFL as max over axes (else sum)            settings "max_face_cfl" */
  int32_t history_capacity;  /* rows of per-step history                   settings "history_capacity" */
  float wave[4];             /* amplitude, k, omega, depth                 settings "wave" */
  float pressure_tolerance;  /* CG relative tolerance, default 1e-4        settings "pressure_tolerance" */
  int32_t linear_air;        /* linear air extension                       settings "linear_air" */
  int32_t stokes_second;     /* second-order Stokes target                 settings "stokes_second" */
  int32_t height_normals;    /* height-function normals (flag bit 0)       settings "height_normals" */
  int32_t active_advection;  /* valid-band advection (flag bit 1)          settings "active_advection" */
  int32_t transport_cache;   /* cached MacCormack traces (flag bit 2)      settings "transport_cache" */
  int32_t transport_interior;/* interior sampling fast path (flag bit 3)   settings "transport_interior" */
  int32_t coastal;           /* 1: coastal_gpu.gd (offshore forcing, ocean ghost at x<0);
                                0: coupled_gpu.gd wall variant (the #ifndef COASTAL branches) */
  float zone_length;         /* offshore relaxation zone (m)               settings "zone_length" */
  float damping_rate;        /* maximum relaxation rate (1/s)              settings "damping_rate" */
  float ramp_periods;        /* forcing ramp in wave periods               settings "ramp_periods" */
  float right_absorption;    /* right absorber scale (shape 6)             settings "right_absorption" */
  int32_t mg_smoother;       /* 0 jacobi, 1 chebyshev                      config "mg_smoother" */
  int32_t mg_smoothing;      /* sweeps per smoothing call (1..8)           config "mg_smoothing" */
  int32_t mg_maintenance;    /* 0 rebuild, 1 structure, 2 lagged           config "mg_maintenance" */
  int32_t mg_lag;            /* lag in trials for "lagged"                 config "mg_lag" */
  int32_t mg_aggregate_from; /* first level using aggregation transfers    config "mg_aggregate_from" */
  int32_t iterations_per_batch; /* CG iterations per scheduler batch (8)   coupled_gpu.gd:14 */
  float cfl;                 /* CFL limit; the reference hard-codes 0.45 (coupled_motion.glslinc:364) */
  /* Additions with no reference counterpart. */
  int32_t mg_precision;      /* 32: FP32 multigrid; 16: BF16 storage and smoothing, FP32 accumulation */
  int32_t warm_start;        /* 0: previous accepted pressure (reference); 1: learned network */
  int32_t device;            /* CUDA device ordinal */
} waves_config;

/* Telemetry of pressure_gpu.gd:135, coupled_gpu.gd:64 and coastal_gpu.gd:37.
 * Recoverable trial failures (codes 10-12, 20 with retries left) read 0 in `failure`, as in
 * coupled_gpu.gd:61-62; `trial_failure` keeps the raw code. */
typedef struct waves_stats_t {
  int32_t accepted_index;        /* c0 */
  double accepted_time;          /* c1 */
  int64_t accepted_steps;        /* c2 */
  int64_t rejections;            /* c3 */
  int32_t pending;               /* c4 */
  int32_t converged;             /* c6 */
  int32_t failure;               /* c7 masked */
  int32_t trial_failure;         /* c7 */
  int64_t iterations;            /* c8 */
  double relative_residual;      /* c13 */
  double max_dt_divergence;      /* c14 */
  double max_face_speed;         /* c15 */
  double hydrostatic_error_pa;   /* c16 */
  double volume_m3;              /* c17 */
  int64_t total_iterations;      /* c18 */
  double dt;                     /* c20 */
  double signed_roundoff_m3;     /* c24 */
  double absolute_roundoff_m3;   /* c25 */
  double initial_volume_m3;      /* c26 */
  double max_CFL;                /* c27 */
  double mass_defect_m3;         /* c28 */
  int32_t retry_count;           /* c29 */
  int64_t trial_count;           /* c32 */
  int32_t last_rejection_code;   /* c33 */
  double last_rejected_dt;       /* c34 */
  double compression_volume_m3;  /* c35 */
  int64_t compression_coverage_errors; /* c36 */
  double step_start_volume_m3;   /* c37 */
  double raw_compression_volume_m3; /* c38 */
  double tentative_outflow_m3;   /* c39 */
  double boundary_outflow_m3;    /* c40 */
  int32_t pressure_defect_corrections; /* c58 */
  double true_relative_residual; /* c60 */
  double rhs_integrated_divergence_l2;      /* c62 */
  double residual_integrated_divergence_l2; /* c63 */
  double forcing_volume_m3;      /* c72 */
  double ocean_inflow_m3;        /* c73 */
  double ocean_outflow_m3;       /* c74 */
  double forcing_momentum[3];    /* c75..77 */
  double gauges_m[8];            /* c80..87 */
  double forcing_min_F;          /* c88 */
  double forcing_max_F;          /* c89 */
  double conservation_residual_m3; /* FP64 ledger identity (build addition), c100 */
  int64_t mg_builds;             /* hierarchy numeric rebuilds (pressure_hierarchy_state.glsl state[11]) */
  int64_t mg_structure_builds;   /* structural rebuilds (state[12]) */
  int32_t mg_levels;             /* levels in the hierarchy (pressure_multigrid.gd:40-59) */
  int64_t warm_start_used;       /* trials whose initial pressure came from the learned network */
  double staged_forcing_volume_m3;  /* c64 */
  double staged_ocean_inflow_m3;    /* c65 */
  double staged_ocean_outflow_m3;   /* c66 */
} waves_stats_t;

typedef struct waves_handle waves_handle;

/* Defaults of pressure_gpu.gd:40-44, coupled_gpu.gd:7-15, coastal_gpu.gd:5-8, the 64x48x16
 * flat-floor tank otherwise. */
void waves_config_default(waves_config* cfg);
/* lab_runner.gd:19-26: the 310x48x80 beach (dispersion solved by the same 80-step bisection). */
void waves_config_beach(waves_config* cfg);
/* 64x48x16 wall-variant sloshing tank, surface 0.45 + 0.05 sin(2 pi x / 1.6) m. */
void waves_config_tank(waves_config* cfg);
/* k solving omega^2 = g k tanh(k h) by 80 bisection steps on [0, 100] (lab_runner.gd:19-25). */
double waves_dispersion_k(double period_s, double depth_m);
/* The multigrid level plan that waves_create builds for cfg (pressure_multigrid.gd:37-69, coarse
 * stencils by _basis/_coarse_stencil :181-198), without a device: *levels = the level count, and for
 * each of the first `capacity` levels 8 ints in out: nx, ny, nz, the coarsening factors fx, fy, fz
 * towards the next level, the operator's stencil size, 1 if its transfer is an aggregation. */
waves_status waves_mg_plan(const waves_config* cfg, int32_t* out, int32_t capacity, int32_t* levels);

/* pressure_gpu.gd _init + start + _initialize: allocates everything on cfg->device, builds the
 * multigrid level plan, runs the initial commands (coupled_gpu.gd:34-37, coastal_gpu.gd:26-27).
 * On failure *out is NULL and the reference's host code (97 MG, 98/99 device) is in the status. */
waves_status waves_create(const waves_config* cfg, waves_handle** out);
/* pressure_gpu.gd close()/_free(): releases all device memory in reverse order of creation. */
void waves_destroy(waves_handle* h);

/* Quota, pressure_gpu.gd:48-54: a nonnegative value is an accepted-step count, request_time sets
 * an absolute accepted-time deadline.  Re-issuing is idempotent; only acceptance advances time. */
waves_status waves_request_steps(waves_handle* h, int64_t steps);
waves_status waves_request_time(waves_handle* h, double seconds);

/* Enqueue up to `max_trials` solver trials (one trial = CFL, VOF, MacCormack, forcing, MG build,
 * PCG to convergence incl. defect corrections, acceptance) on the handle's stream.  No host
 * synchronisation inside; a trial that finds the quota met or the solver failed does nothing. */
waves_status waves_advance(waves_handle* h, int32_t max_trials);
/* Advance until the quota is met or the solver fails (synchronises once per `trials_per_sync`). */
waves_status waves_run(waves_handle* h, int32_t trials_per_sync);
/* Wait for the handle's stream. */
waves_status waves_synchronize(waves_handle* h);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their own work after the
 * solver's.  Every enqueue of this library goes to this stream. */
void* waves_stream(waves_handle* h);
/* Device time of the trials submitted so far, from CUDA events recorded on the handle's stream
 * around each trial: the motion part (CFL, VOF, MacCormack, forcing) and the pressure part
 * (geometry through acceptance, i.e. ops 17..13 of the reference).  Synchronises. */
waves_status waves_timing(waves_handle* h, double* motion_ms, double* pressure_ms, int64_t* trials, int32_t reset);

/* Telemetry snapshot (synchronises with the stream). */
waves_status waves_stats(waves_handle* h, waves_stats_t* out);
/* Raw control block, WAVES_CONTROL_SIZE doubles in the reference's index map. */
waves_status waves_control(waves_handle* h, double* c, int32_t count);
/* Overwrite the control block (test and checkpoint use; count <= WAVES_CONTROL_SIZE). */
waves_status waves_set_control(waves_handle* h, const double* c, int32_t count);
/* Host-side fault injection (the reference's op 15, pressure_pass.glslinc:138): sets the
 * inject-rejection flag c19 so that the next acceptance test rejects the trial with code 4. */
waves_status waves_inject_rejection(waves_handle* h);

/* Accepted-surface export (pressure_pass.glslinc:127-130, op 19): planes[4N] = (normal, alpha)
 * per cell and kinds[N] = 0 air, 1 liquid, 2 mixed, x-fastest.  Host buffers. */
waves_status waves_export_surface(waves_handle* h, float* planes, float* kinds);
/* The same export into caller DEVICE buffers (planes 16-byte aligned), enqueued on the handle's
 * stream without waiting: a headless stand-in for the planes/kinds Texture3DRD.  When clock is not
 * NULL (16-byte aligned), the same launch writes the surface clock of surface_clock.glsl:1-7 (run
 * after op 19, coastal_view.gd:19-23): clock[4] = (accepted time, accepted steps, 0, 0) as float,
 * the committed clock of the exported surface, also after a rejected trial. */
waves_status waves_export_surface_device(waves_handle* h, void* planes, void* kinds, void* clock);

/* Headless presentation (water/presentation/water.gdshader:21-176 with daylight.gdshaderinc,
 * water/shaders/render/clay.gdshader:8-66): one ray per pixel through the exported PLIC surface,
 * marched cell by cell, into a float RGBA image (row 0 at the top).  Mode 1 (water) sums the
 * occupied intervals along the ray, shades with the optical normal, ripples driven by the surface
 * clock, Fresnel sky reflection, absorption and a specular sun; what the fragment shader reads from
 * the rendered scene is an analytic scene here (the sky, and the sand bed of presentation.gd:
 * 94-112 when slope > 0).  Mode 0 (clay) shades the first liquid entry.  The optional trace image
 * holds per pixel (first entry distance or -1, occupied length, exit of the first interval (clay:
 * box exit), texture queries). */
typedef struct waves_render_params {
  int32_t width, height;
  int32_t mode;               /* 0 clay, 1 water */
  int32_t orthographic;       /* 1: `size` is the view height (m); 0: perspective, fov_y_deg */
  float eye[3], target[3], up[3];
  float size, fov_y_deg;
  float water_tint[3];        /* water.gdshader:12 */
  float attenuation_distance; /* :14, m */
  float ripple_strength;      /* :15 */
  float surface_roughness;    /* :16 */
  float sun_direction[3];     /* daylight.gdshaderinc:2 */
  int32_t contact_correction; /* :18, with the bed of config slope > 0 */
  int32_t clock_ready;        /* :19, ripple phase from the surface clock (accepted time) */
} waves_render_params;
/* Defaults of water.gdshader and the camera of presentation.gd:83-93 (camera_preset(1),
 * orthographic, "wide" when nz hz > 1 m) at width x height. */
void waves_render_params_default(waves_render_params* p, const waves_config* cfg, int32_t width, int32_t height);
/* Export + render; rgba[4 width height] and trace (NULL or 4 width height) are host buffers. */
waves_status waves_render(waves_handle* h, const waves_render_params* p, float* rgba, float* trace);
/* The same into caller device buffers (16-byte aligned), enqueued on the handle's stream. */
waves_status waves_render_device(waves_handle* h, const waves_render_params* p, void* rgba, void* trace);

/* Telemetry history, each buffer sized by history_capacity (cap); any pointer may be NULL.
 *   history[16 cap]: per trial four float4 rows (coupled_motion.glslinc:338-340): the three VOF
 *     sweeps (min F, max F, summed change, summed |change|), then (accepted time, dt, state:
 *     -failure code or 1 pending / 0 done, accepted steps) (op 44, pressure_pass.glslinc).
 *   coastal[20 cap]: per accepted step five float4 rows of the coastal ledger and the eight gauges
 *     (coastal_pass.glslinc:60-80, op 89).
 *   audit[64 + 32 cap]: the multigrid hierarchy audit words, a 64-word header then one 32-word row
 *     per rebuild (pressure_hierarchy_state.glsl:55-59,67). */
waves_status waves_get_history(waves_handle* h, float* history, float* coastal, uint32_t* audit);

/* Bank access.  bank = 0/1 physical bank, -1 the accepted bank.  A bank is
 * [F: N][u: (nx+1) ny nz][v: nx (ny+1) nz][w: nx ny (nz+1)][p: N] floats, x-fastest. */
size_t waves_bank_floats(const waves_handle* h);
waves_status waves_get_bank(waves_handle* h, int32_t bank, float* out);
waves_status waves_set_bank(waves_handle* h, int32_t bank, const float* in);
/* Signed distance phi and kind (-1 solid, 0 air, 1 wet) of the last geometry pass, N each. */
waves_status waves_get_geometry(waves_handle* h, float* phi, float* kind);
/* Banked pressure masks pmask[2N] and face valid bands vband[2 faces] (coupled_motion.glslinc:
 * 323-337), bank 0 first; values 0/1. */
waves_status waves_get_masks(waves_handle* h, float* pmask, float* vband);
waves_status waves_set_masks(waves_handle* h, const float* pmask, const float* vband);

/* Checkpoint of both banks, the control block, the pressure masks and valid bands and the
 * hierarchy snapshot: waves_save with buffer NULL returns the size in *bytes. */
waves_status waves_save(waves_handle* h, void* buffer, size_t* bytes);
waves_status waves_load(waves_handle* h, const void* buffer, size_t bytes);

/* Frame-budgeted submission (water/work_scheduler.gd:41-87): one call per rendered frame.  It
 * folds the GPU times of finished trials into a running per-trial cost (exponential average,
 * weight 0.25, as the reference averages its chunk costs), retires finished submissions (their
 * control block, copied asynchronously, becomes the reported telemetry), and -- unless the solver
 * halted, the quota is met with no trial pending, or max_inflight submissions are unfinished --
 * enqueues as many trials as gpu_budget_ms admits at that cost (at least one, at most max_trials,
 * stopping early once enqueueing took cpu_budget_ms) followed by the control-block copy.  It
 * never waits for the GPU and never changes a result. */
typedef struct waves_frame_budget {
  double gpu_budget_ms;  /* predicted GPU time per frame (reference default 14) */
  int32_t max_inflight;  /* unfinished submissions allowed (reference 3, at most 8) */
  int32_t max_trials;    /* trials per submission (reference: 96 chunks) */
  double cpu_budget_ms;  /* host enqueue time per frame, <= 0 for none (reference 4) */
} waves_frame_budget;
typedef struct waves_frame_report {
  int32_t trials_submitted;  /* this call */
  int32_t queue_depth;       /* unfinished submissions after this call */
  int32_t idle;              /* 1: quota met and nothing in flight */
  int32_t halted;            /* 1: the solver stopped with a failure (stats.failure) */
  double predicted_gpu_ms;   /* trials_submitted x trial_cost_ms */
  double trial_cost_ms;      /* running GPU cost of one trial (0 before the first measurement) */
  double gpu_ms_total;       /* GPU time of every trial measured so far */
  double r_fluid;            /* GPU seconds per accepted simulated second (R_fluid) */
  double accepted_time;      /* of the latest retired submission */
  int64_t accepted_steps;
  int64_t submissions_retired;
} waves_frame_report;
waves_status waves_frame(waves_handle* h, const waves_frame_budget* budget, waves_frame_report* report);
/* The telemetry of the latest retired waves_frame submission, from its control-block copy: what
 * the reference's asynchronous read-back hands to _stats (work_scheduler.gd:78-82, then
 * pressure_gpu.gd:133-137, coupled_gpu.gd:58-65, coastal_gpu.gd:34-37).  No device access and no
 * wait.  The hierarchy counters (mg_builds, mg_structure_builds) are those of the last
 * waves_stats call.  WAVES_INVALID_ARG while no submission has retired. */
waves_status waves_frame_stats(const waves_handle* h, waves_stats_t* out);

/* Learned warm start (no reference counterpart): 4 layers of 3x3x3 convolutions,
 * channels 3 -> 16 -> 16 -> 16 -> 1, BF16 weights (raw uint16 bit patterns), FP32 biases.
 * Layout per layer: weights[co][kz][ky][kx][ci].  NULL disables it. */
#define WAVES_NET_LAYERS 4
#define WAVES_NET_HIDDEN 16
typedef struct waves_warm_start_model {
  const uint16_t* weights[WAVES_NET_LAYERS];
  const float* bias[WAVES_NET_LAYERS];
  float input_scale[3];  /* F, b, p_prev multipliers applied before the network */
  float output_scale;    /* network output multiplier */
} waves_warm_start_model;
waves_status waves_set_warm_start(waves_handle* h, const waves_warm_start_model* model);

/* Training of the warm-start network on the GPU (own forward, backward and Adam kernels): a batch
 * of crops with zero padding at the crop edge; inputs, weights and activations rounded to BF16 as
 * in the inference kernels.  Weights are the FP32 masters [co][27][ci] (tap (kz * 3 + ky) * 3 + kx),
 * biases [co], per layer; all buffers host.  Two arithmetics:
 *   WAVES_NET_EXACT   FP32 accumulation forward in a fixed order (the CPU oracle's), FP64 sums in
 *                     the weight and input gradients, gradients passed through the roundings in FP32;
 *   WAVES_NET_TENSOR  implicit GEMM on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
 *                     accumulation) for the forward pass, the input gradients and the weight
 *                     gradients; the gradients between layers are BF16 operands, the weight
 *                     gradients' per-block partials are summed in FP64 in a fixed order. */
#define WAVES_NET_EXACT 0
#define WAVES_NET_TENSOR 1
typedef struct waves_net_batch {
  int32_t crops, nz, ny, nx;  /* crop count and size in cells */
  const float* x;             /* [crops][3][nz][ny][nx]: scaled F, b, p_prev */
  const float* target;        /* [crops][nz][ny][nx]: the scaled pressure correction */
  const float* mask;          /* [crops][nz][ny][nx]: 1 where the loss counts */
  int32_t arithmetic;         /* WAVES_NET_EXACT or WAVES_NET_TENSOR */
} waves_net_batch;
/* One forward and backward pass: loss = sum mask (y - target)^2 / max(sum mask, 1), dL/dW and dL/db
 * of every layer, and the output y ([crops][nz][ny][nx], may be NULL). */
waves_status waves_net_gradients(const waves_net_batch* batch, const float* const* weights, const float* const* bias,
                                 double* loss, float* const* grad_w, float* const* grad_b, float* y, int32_t device);
/* `iterations` Adam steps (beta 0.9 / 0.999, eps 1e-8) on the batch; weights and biases updated in
 * place; the loss before each step in loss_history (may be NULL). */
waves_status waves_net_train(const waves_net_batch* batch, float* const* weights, float* const* bias, int32_t iterations,
                             float learning_rate, double* loss_history, int32_t device);

/* Liquid volume sum over cells of F * hx*hy*hz (FP64) of a caller-owned device array F[nx*ny*nz]
 * (x-fastest), written to the caller-owned device double *out, enqueued on `stream` (a
 * cudaStream_t; NULL = default stream).  No counterpart in the reference.  It allocates nothing:
 * for hosts that cannot let the library call cudaMalloc (engine-owned GPU memory, no allocation
 * inside a frame); its scratch is a fixed 64 KiB device array in the library, so it accepts at most
 * 2,097,152 cells (WAVES_INVALID_ARG beyond).  The first call on a device resolves that array's
 * address in the current CUDA context and keeps it, keyed by device and context id (so it is
 * resolved again after cudaDeviceReset or in another context); make that first call before any
 * stream capture.  All calls share the array: calls that overlap on the GPU race.  The additions
 * follow the solver's own volume reduction in the same order, so the result is bit-identical to
 * waves_stats().initial_volume_m3 for the solver's initial F. */
waves_status waves_liquid_volume_noalloc(const float* F, int32_t nx, int32_t ny, int32_t nz, float hx, float hy, float hz,
                                         double* out, void* stream);

/* Last error text of this handle (or of the last failed waves_create when h is NULL). */
const char* waves_last_error(const waves_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* WAVES_H */
