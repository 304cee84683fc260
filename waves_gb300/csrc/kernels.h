// Host-side launch functions of the solver kernels (one group per phase of the step).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "dev.h"

namespace wg {

enum CondKind { kCondActive = 0, kCondSolving = 1, kCondDefect = 2, kCondDefectFirst = 3 };

// Kernel probes.  While a probe list is installed on the calling thread (host-scheduled trials
// only, never during graph capture), each probed launch site brackets its launch with two events
// on its stream and records the launch's algorithmic bytes: the distinct input arrays read once
// and the outputs written once, at storage precision.
enum ProbeKind {
  kProbeMac = 0,        // k_mac, MacCormack forward (op 27) and corrected (op 28) passes
  kProbeSmooth0 = 1,    // k_mg0_cheb, level-0 Chebyshev sweeps
  kProbeRows = 2,       // k_mgl_rows, level >= 1 sweeps with the product-parallel apply
  kProbeRowThread = 3,  // k_mgl4 (k_mgl with one lane per row) ops 0-2, level >= 1 sweeps of large levels
  kProbeSweepVof = 4,   // k_sweep_update, VOF flux + update of one direction
  kProbeAll = 5,        // every kernel of the trial (bytes not counted)
  kProbeEmpty = 6,      // calibration: an empty kernel bracketed as a probed launch is (kind + all)
  kProbeEmptyInner = 7, // the inner bracket of that calibration
  kProbeLeg = 8,        // k_mg_leg, the coarse levels and the bottom of a V-cycle in one cluster
  kProbeCount = 9
};
// `level` >= 1 marks a multigrid level sweep whose bytes were counted over all rows of the level;
// the probe scales them to the rows the sweep visits (the active rows) once the trial has run.
struct ProbeRec {
  int kind;
  cudaEvent_t a, b;
  double bytes;
  int level;
};
extern thread_local std::vector<ProbeRec>* g_probe;
template <class F> void probed(int kind, cudaStream_t s, double bytes, F&& launch, int level = -1) {
  std::vector<ProbeRec>* p = g_probe;
  if (!p) {
    launch();
    return;
  }
  ProbeRec r{kind, nullptr, nullptr, bytes, level};
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, s);
  launch();
  cudaEventRecord(r.b, s);
  p->push_back(r);
}

// Programmatic dependent launch: a kernel launched this way may be scheduled while the previous
// kernel on the stream drains; every kernel's first statement is grid_dep_wait()
// (griddepcontrol.wait), which returns once that kernel has completed and its writes are visible,
// so only launch latency overlaps.  WAVES_PDL at handle creation: 0 off, 1 on (default), 2 on with
// the early trigger (kernels release their dependents on entry).
// With a probe list installed, every launch is also bracketed as kind kProbeAll.
extern bool g_pdl;
template <class... KArgs, class... Args>
void pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = g_pdl ? 1 : 0;
  probed(kProbeAll, s, 0.0, [&] { cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...); });
}

// k_pcg.cu
void launch_begin(const Dev& D, cudaStream_t s);
void launch_defect_begin(const Dev& D, cudaStream_t s);
void launch_cg_init(const Dev& D, cudaStream_t s);
void launch_warm_start(const Dev& D, cudaStream_t s);  // learned warm start after op 2 (no-op when not configured)
// k_net.cu
void launch_warm_network(const Dev& D, cudaStream_t s);
void setup_warm_network();  // shared-memory limits of the tcgen05 layers
void launch_cg_matvec(const Dev& D, cudaStream_t s);
void launch_cg_update(const Dev& D, cudaStream_t s);
void launch_cg_direction(const Dev& D, cudaStream_t s, cudaGraphConditionalHandle h, int use_handle);
void launch_set_cond(const Dev& D, cudaStream_t s, cudaGraphConditionalHandle h, int which);
void launch_delay(cudaStream_t s, long long cycles);
void launch_empty(cudaStream_t s);  // one empty one-thread kernel (probe calibration)
// k_motion.cu
void launch_motion_cfl(const Dev& D, cudaStream_t s);
void launch_sweep(const Dev& D, cudaStream_t s);
void launch_mac_donor_table(const Dev& D, cudaStream_t s);  // static, once at set-up
void launch_maccormack(const Dev& D, cudaStream_t s);
int mac_blocks();   // resident blocks of the persistent MacCormack kernel (3 per SM form)
int mac_blocks2();  // the same for the 2-per-SM form
int mac_fast_blocks();  // resident blocks of the interior fast-path MacCormack pass
constexpr int kMacCounters = 8;
void launch_debug_sample(const Dev& D, cudaStream_t s, const float* x, int axis, int forward, float* out);
// k_geom.cu
void launch_coastal(const Dev& D, cudaStream_t s);
void launch_geometry(const Dev& D, cudaStream_t s);
void launch_proj_setup(const Dev& D, cudaStream_t s);
void launch_post(const Dev& D, cudaStream_t s);
void launch_trial_end(const Dev& D, cudaStream_t s);
void launch_ext_masks(const Dev& D, cudaStream_t s);  // static face neighbourhoods (set-up)
void launch_export(const Dev& D, cudaStream_t s, float4* planes, float* kinds, float4* clock = nullptr);
// k_render.cu: headless presentation of the exported surface
struct RenderArgs {
  const float4* planes;
  const float* kinds;
  const double* c;  // control block (surface clock c[1])
  float4* rgba;
  float4* trace;  // optional: first entry, occupied length, first-interval exit (clay: box exit), queries
  int nx, ny, nz, width, height;
  int mode;  // 0 clay, 1 water
  int ortho, contact, clock_ready;
  float bmin[3], bmax[3], slope;
  float eye[3], fwd[3], right[3], up[3], half_w, half_h;
  float tint[3], attenuation, ripple, roughness, sun[3];
};
void launch_render(const RenderArgs& A, cudaStream_t s);
// k_mg.cu
void launch_mg_build(const Dev& D, cudaStream_t s);
void launch_mg_vcycle(const Dev& D, cudaStream_t s, int phase);
void mg_kernel_attributes();
int coarse_blocks(size_t smem);  // blocks of the one-launch coarse V-cycle, 0 when unavailable
// Whether the one-cluster coarse leg can run with `smem` bytes of dynamic shared memory per block
// (a cluster of that shape fits the device, and such a launch can be captured into a graph).
bool leg_available(size_t smem);
constexpr int kLegRowsFrom = 8192;  // the leg starts at the first level with at most this many rows
constexpr size_t kLegSmemMin = 100 * 1024;
void launch_mg_cols(const Dev& D, cudaStream_t s);
// k_init.cu
void launch_initial(const Dev& D, cudaStream_t s, float4* probes);

}  // namespace wg
