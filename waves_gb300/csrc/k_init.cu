// Initial commands (neuron-forest/waves water/coupled_gpu.gd:34-37, water/coastal_gpu.gd:26-27):
// op 0 still water, op 40 fixtures, op 41/42 initial volume, op 49 masks, op 86 target probes.
#include "common.cuh"
#include "kernels.h"

namespace wg {

namespace {
constexpr int NT = 256;

// op 0 (pressure_pass.glslinc:182-198)
__global__ void __launch_bounds__(NT) k_init_still(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  Grid g(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i >= D.S) return;
  float f = 0.f;
  if (i < D.N) {
    I3 q = g.coord(i);
    float ph = g.center(q).y - g.eta(q);
    bool wall = g.solid(q);
    D.phi[i] = ph;
    D.kind[i] = wall ? -1 : (ph < 0.f ? 1 : 0);
    f = wall ? 0.f : clampf_(0.5f - ph / D.hy, 0.f, 1.f);
  }
  D.bank0[i] = f;
  D.bank1[i] = f;
}

DI float streamfunction(const Dev& D, F3 x) {
  const float* w = D.wave;
  float value = w[0] * w[2] / (w[1] * tsinh(w[1] * w[3])) * tsinh(w[1] * (x.y + w[3])) * tcos(w[1] * x.x);
  if (D.stokes2)
    value += .375f * w[0] * w[0] * w[2] / tpow4(tsinh(w[1] * w[3])) * tsinh(2.f * w[1] * (x.y + w[3])) * tcos(2.f * w[1] * x.x);
  return value;
}
DI float block_overlap(const Dev& D, F3 lo, F3 hi, F3 lower, F3 upper) {
  float o[3];
  for (int a = 0; a < 3; a++) {
    float h = a == 0 ? D.hx : (a == 1 ? D.hy : D.hz);
    o[a] = clampf_((mnf(hi[a], upper[a]) - mxf(lo[a], lower[a])) / h, 0.f, 1.f);
  }
  return o[0] * o[1] * o[2];
}
// op 40 (coupled_motion.glslinc:234-270)
__global__ void __launch_bounds__(NT) k_init_fixture(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  Grid g(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  int shape = D.shape;
  if (i < D.N) {
    I3 q = g.coord(i);
    F3 lo = mf((float)q.x * D.hx, (float)q.y * D.hy, (float)q.z * D.hz);
    F3 hi = mf(lo.x + D.hx, lo.y + D.hy, lo.z + D.hz);
    float f = D.bank0[i];
    if (shape > 0 && shape < 3) {
      F3 lower = shape < 2 ? mf(0.f, 0.f, 0.f) : mf(.22f, .28f, .06f);
      F3 upper = shape < 2 ? mf(.28f, .3f, 100.f) : mf(.42f, .48f, .22f);
      f = block_overlap(D, lo, hi, lower, upper);
      if (shape > 1) f += clampf_((.08f - lo.y) / D.hy, 0.f, 1.f);
    }
    if (shape == 4) {
      f = 0.f;
      for (int b = 0; b < 2; b++)
        f += block_overlap(D, lo, hi, mf(b == 0 ? .08f : .36f, .12f, 0.f), mf(b == 0 ? .24f : .52f, .32f, 100.f));
    }
    D.bank0[i] = f;
    D.bank1[i] = f;
  }
  if (i < D.NF) {
    I3 q;
    int axis;
    g.unpack_face(i, q, axis);
    float velocity = (shape == 3 && axis == 0 && !g.wall_face(q, axis) && g.center(q).y < D.eta0 + 3.f * D.hy) ? .25f : 0.f;
    if (shape == 4 && axis == 0 && !g.wall_face(q, axis)) velocity = (float)q.x * D.hx < .3f ? 2.f : -2.f;
    if (shape == 5) {
      F3 x = mf(((float)q.x + .5f) * D.hx + D.ox, ((float)q.y + .5f) * D.hy + D.oy, ((float)q.z + .5f) * D.hz + D.oz);
      x[axis] -= .5f * g.h(axis);
      if (x.y < g.eta(q) + 3.f * D.hy && !g.wall_face(q, axis)) {
        if (axis == 0) {
          float dy = .5f * D.hy;
          velocity = (streamfunction(D, mf(x.x, x.y + dy, x.z)) - streamfunction(D, mf(x.x, x.y - dy, x.z))) / D.hy;
        }
        if (axis == 1) {
          float dx = .5f * D.hx;
          velocity = -(streamfunction(D, mf(x.x + dx, x.y, x.z)) - streamfunction(D, mf(x.x - dx, x.y, x.z))) / D.hx;
        }
      }
    }
    D.bank0[D.N + i] = velocity;
    D.bank1[D.N + i] = velocity;
  }
  if (i == 0) {
    D.c[20] = (double)D.dtcfg;
    D.c[31] = (double)D.grav;
  }
}

// op 41/42
__global__ void __launch_bounds__(NT) k_init_volume(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  double v[1] = {0};
  if (i < D.N) v[0] = (double)bank_ptr(D, acc_bank(D))[i] * D.cell_d;
  const int ops[1] = {0};
  double out[1];
  if (last_block_reduce<NT, 1>(D, kSiteCFL, v, ops, out) && threadIdx.x == 0) D.c[26] = out[0];
}

// op 49 (coupled_motion.glslinc:323-337)
__global__ void __launch_bounds__(NT) k_init_masks(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  Grid g(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i < D.N) {
    float flag = D.kind[i] > 0 ? 1.f : 0.f;
    D.pmask0[i] = flag;
    D.pmask1[i] = flag;
  }
  if (i < D.NF) {
    I3 q;
    int axis;
    g.unpack_face(i, q, axis);
    I3 l = ax(q, axis, -1);
    float v = (!g.wall_face(q, axis) && (g.wet(q) || g.wet(l) || g.center(q).y < g.eta(q) + 3.f * D.hy)) ? 1.f : 0.f;
    D.vband0[i] = v;
    D.vband1[i] = v;
  }
}

// op 86 (coastal_pass.glslinc:78-83)
__global__ void k_probes(const __grid_constant__ Dev D, float4* out) {
  grid_dep_wait(D.pdl_early);
  int i = threadIdx.x;
  if (i >= 8) return;
  Coast cs(D);
  float probe_time = D.forcing[3] * 6.28318530718f / D.wave[2] * (i < 4 ? .37f : 1.f);
  F3 point = mf(D.ox + .17f + (float)i * .23f, -D.wave[3] + (float)i * .07f, 0.f);
  float s0, s1;
  cs.surface(point.x, probe_time, s0, s1);
  F3 vel = cs.velocity(point, probe_time);
  out[i] = make_float4(s0, s1, vel.x, vel.y);
}

unsigned grid_for(long long n) { return (unsigned)((n + NT - 1) / NT); }
}  // namespace

void launch_initial(const Dev& D, cudaStream_t s, float4* probes) {
  pdl_launch(k_init_still, grid_for(D.S), NT, 0, s, D);
  long long n = D.N > D.NF ? D.N : D.NF;
  pdl_launch(k_init_fixture, grid_for(n), NT, 0, s, D);
  launch_geometry(D, s);
  pdl_launch(k_init_volume, grid_for(D.N), NT, 0, s, D);
  pdl_launch(k_init_masks, grid_for(n), NT, 0, s, D);
  if (D.coastal) {
    launch_trial_end(D, s);  // op 85 (ops 44 and 89 are inert before the first trial)
    pdl_launch(k_probes, 1, 32, 0, s, D, probes);
  }
}

}  // namespace wg
