// Host-side launch functions of the solver kernels (one group per phase of the step).
#pragma once
#include <cuda_runtime.h>

#include "dev.h"

namespace wg {

enum CondKind { kCondActive = 0, kCondSolving = 1, kCondDefect = 2, kCondDefectFirst = 3 };

// k_pcg.cu
void launch_begin(const Dev& D, cudaStream_t s);
void launch_defect_begin(const Dev& D, cudaStream_t s);
void launch_cg_init(const Dev& D, cudaStream_t s);
void launch_cg_matvec(const Dev& D, cudaStream_t s);
void launch_cg_update(const Dev& D, cudaStream_t s);
void launch_cg_direction(const Dev& D, cudaStream_t s, cudaGraphConditionalHandle h, int use_handle);
void launch_set_cond(const Dev& D, cudaStream_t s, cudaGraphConditionalHandle h, int which);
// k_motion.cu
void launch_motion_cfl(const Dev& D, cudaStream_t s);
void launch_sweep(const Dev& D, cudaStream_t s);
void launch_maccormack(const Dev& D, cudaStream_t s);
void launch_debug_sample(const Dev& D, cudaStream_t s, const float* x, int axis, int forward, float* out);
// k_geom.cu
void launch_coastal(const Dev& D, cudaStream_t s);
void launch_geometry(const Dev& D, cudaStream_t s);
void launch_proj_setup(const Dev& D, cudaStream_t s);
void launch_post(const Dev& D, cudaStream_t s);
void launch_trial_end(const Dev& D, cudaStream_t s);
void launch_export(const Dev& D, cudaStream_t s, float4* planes, float* kinds);
// k_mg.cu
void launch_mg_build(const Dev& D, cudaStream_t s);
void launch_mg_vcycle(const Dev& D, cudaStream_t s, int phase);
void mg_kernel_attributes();
void launch_mg_cols(const Dev& D, cudaStream_t s);
// k_init.cu
void launch_initial(const Dev& D, cudaStream_t s, float4* probes);

}  // namespace wg
