/*
 * waves_debug.h — debugging hooks of the waves library (not part of the solver API).
 *
 * waves_debug_phase enqueues one phase of a trial on the handle's stream and waits for it; the
 * phases are, in trial order: 0 begin (ops 43, 1), 1 CFL and compression pre-check, 2 one VOF
 * sweep, 3 MacCormack, 4 coastal forcing, 5 geometry, 6 projection set-up, 7 multigrid build,
 * 8 CG set-up with the first V-cycle, 9 one CG iteration, 10 projection, extension and
 * acceptance, 11 trial end; 12 is the learned warm start, which a trial runs between phases 6
 * and 7 when it is configured.  waves_debug_read copies a named device array (the names of the
 * allocations in waves_abi.cu) to host memory.
 */
#ifndef WAVES_DEBUG_H
#define WAVES_DEBUG_H
#include "waves.h"
#ifdef __cplusplus
extern "C" {
#endif
waves_status waves_debug_phase(waves_handle* h, int32_t phase);
/* One MacCormack sampled component at local position x (40 floats: value, valid, limits, lattice,
 * then per donor: value, supported, solid, wall). */
waves_status waves_debug_sample(waves_handle* h, const float* x, int32_t axis, int32_t forward, float* out40);
/* Kernel launches per phase: begin, motion, pressure set-up, CG round set-up, CG iteration,
 * projection/extension/acceptance, trial end, condition kernel. */
waves_status waves_debug_launch_counts(waves_handle* h, int32_t* out8);
waves_status waves_debug_read(waves_handle* h, const char* name, void* out, size_t bytes);
/* Kernel probes of one host-scheduled trial (every CG iteration checked, so no probed launch is a
 * no-op): per kind, the launches, their summed CUDA-event time on the handle's stream and their
 * summed algorithmic bytes (distinct inputs read once, outputs written once).  Kinds: 0 MacCormack
 * passes, 1 level-0 Chebyshev sweeps, 2 level >= 1 sweeps (product-parallel rows), 3 level >= 1
 * sweeps of the large levels (four lanes per active row, or one thread per row), 4 VOF flux + update, 5 every kernel of the trial (launches and
 * time only), 6 and 7 the calibration after the trial: 64 launches of an empty kernel bracketed
 * the way a probed launch is (6 the outer, 7 the inner event pair), whose time per launch is the
 * cost the brackets add to each probed launch, 8 the coarse leg of the V-cycle in one cluster
 * launch (bytes of its level sweeps).  The trial advances the simulation like any
 * other; *trials is 0 when no trial was active (quota met). */
typedef struct waves_kernel_probe {
  int32_t kind;
  int32_t launches;
  double ms;
  double bytes;
} waves_kernel_probe;
waves_status waves_debug_probe_trial(waves_handle* h, waves_kernel_probe* out, int32_t capacity, int32_t* trials);
#ifdef __cplusplus
}
#endif
#endif
