/*
 * waves_debug.h — debugging hooks of the waves library (not part of the solver API).
 *
 * waves_debug_phase enqueues one phase of a trial on the handle's stream and waits for it; the
 * phases are, in trial order: 0 begin (ops 43, 1), 1 CFL and compression pre-check, 2 one VOF
 * sweep, 3 MacCormack, 4 coastal forcing, 5 geometry, 6 projection set-up, 7 multigrid build,
 * 8 CG set-up with the first V-cycle, 9 one CG iteration, 10 projection, extension and
 * acceptance, 11 trial end.  waves_debug_read copies a named device array (the names of the
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
#ifdef __cplusplus
}
#endif
#endif
