// Multigrid preconditioner: hierarchy audit, Galerkin build and V-cycle
// (neuron-forest/waves water/shaders/compute/pressure_multigrid.glslinc, pressure_mg_coarse.glslinc,
// pressure_hierarchy_state.glsl; command order water/pressure_multigrid.gd:121-176).
//
// Storage type T is float (FP32 multigrid) or __nv_bfloat16 (BF16 storage and smoothing); every
// arithmetic operation is FP32.  The Galerkin product is a deterministic gather.  From level 0:
// for coarse row I, each thread of a group (the children of I in one (y, z) fine row) accumulates
// (a_ij * w_iI) * w_jJ into its own shared-memory row of slots, and the row is the sum of the group
// partials in group order.  From a level >= 1: A P per active fine row, then P^T (A P) per coarse
// row (k_mg_gal_ap, k_mg_gal_pt).  No float atomics touch any result.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace wg {

namespace {
constexpr int NT = 256;
constexpr int GT = 128;  // Galerkin block size

DI bool build_on(const Dev& D) { return !(D.c[7] > .5) && !(D.c[5] < .5); }
DI bool phase_on(const Dev& D, int phase) {
  const double* c = D.c;
  if (c[7] > .5) return false;
  if (phase == 0) return (c[5] > .5 || c[57] == 2) && c[6] < .5;
  return c[4] > .5 && c[6] < .5;
}

DI int pmod(int x, int m) { return pidx(x, m); }

struct MG {
  const Dev& D;
  DI explicit MG(const Dev& d) : D(d) {}
  DI int wrap(int l, I3 q) const {
    const MGLevelDev& v = D.lv[l];
    q.z = pmod(q.z, v.nz);
    if (D.px) q.x = pmod(q.x, v.nx);
    if (q.x < 0 || q.x >= v.nx || q.y < 0 || q.y >= v.ny) return -1;
    return q.x + v.nx * (q.y + v.ny * q.z);
  }
  DI I3 coord(int l, int i) const {
    const MGLevelDev& v = D.lv[l];
    const unsigned u = (unsigned)i, row = u / (unsigned)v.nx;
    return mk(int(u - row * (unsigned)v.nx), int(row % (unsigned)v.ny), int(row / (unsigned)v.ny));
  }
  DI I3 delta(int l, int i, int j) const {
    const MGLevelDev& v = D.lv[l];
    I3 d = subI(coord(l, j), coord(l, i));
    if (D.px) d.x = pmod(d.x + v.nx / 2, v.nx) - v.nx / 2;
    d.z = pmod(d.z + v.nz / 2, v.nz) - v.nz / 2;
    return d;
  }
  DI static int slot(I3 d) { return d.x + 2 + 5 * (d.y + 2 + 5 * (d.z + 2)); }
  // cell coordinates packed 21 bits per axis (the transfer table's coarse coordinates)
  DI static unsigned long long pack(I3 q) {
    return (unsigned long long)q.x | ((unsigned long long)q.y << 21) | ((unsigned long long)q.z << 42);
  }
  DI static I3 unpack(unsigned long long v) {
    return mk(int(v & 0x1fffffull), int((v >> 21) & 0x1fffffull), int(v >> 42));
  }
  // wrap() on coordinates: false where wrap() returns -1, else q wrapped in place
  DI bool wrap_q(int l, I3& q) const {
    const MGLevelDev& v = D.lv[l];
    q.z = pmod(q.z, v.nz);
    if (D.px) q.x = pmod(q.x, v.nx);
    return !(q.x < 0 || q.x >= v.nx || q.y < 0 || q.y >= v.ny);
  }
  // delta() from the coordinates of i (qi) and j (qj)
  DI I3 delta_q(int l, I3 qi, I3 qj) const {
    const MGLevelDev& v = D.lv[l];
    I3 d = subI(qj, qi);
    if (D.px) d.x = pmod(d.x + v.nx / 2, v.nx) - v.nx / 2;
    d.z = pmod(d.z + v.nz / 2, v.nz) - v.nz / 2;
    return d;
  }
  DI I3 offset(int l, int k) const {
    const int* s = D.stencil_tab + 3 * (D.lv[l].soff + k);
    return mk(__ldg(s), __ldg(s + 1), __ldg(s + 2));
  }
  template <class T> DI T* field(int f, int l) const { return (T*)D.mgv + (long long)f * D.mg_nodes + D.lv[l].off; }
  template <class T> DI bool active(int l, int i) const { return i >= 0 && ld_val(field<T>(3, l)[i]) > .5f; }
  DI float fine_coef(int f, int i) const { return D.snapshot[(long long)(f - 6) * D.N + i]; }
  DI const float* coarse_inverse() const { return D.mglinv; }
  // coefficient (pressure_multigrid.glslinc:74-88), build-time values from the FP32 rows
  template <class T> DI float coefficient(int l, int i, int j) const {
    if (j < 0) return 0.f;
    if (!active<T>(l, i) || !active<T>(l, j)) return i == j ? 1.f : 0.f;
    if (l == 0) {
      if (i == j) return fine_coef(12, i);
      I3 q = coord(0, i);
      float value = 0.f;
      for (int axis = 0; axis < 3; axis++)
        for (int side = 0; side < 2; side++)
          if (wrap(0, ax(q, axis, 2 * side - 1)) == j) value -= fine_coef(6 + 2 * axis + side, i);
      return value;
    }
    int a = min(i, j), b = max(i, j);
    I3 d = delta(l, a, b);
    if (abs(d.x) > 2 || abs(d.y) > 2 || abs(d.z) > 2) return 0.f;
    return D.mgmat[D.lv[l].moff + (long long)a * 125 + slot(d)];
  }
  DI bool unique_neighbor(int l, int i, I3 off, int j) const { return j >= 0 && eqI(delta(l, i, j), off); }
  // compute_transfers (pressure_multigrid.glslinc:108-120)
  template <class T> DI int compute_transfers(int l, int i, int* ids, float* ws) const {
    const MGLevelDev& lv = D.lv[l];
    const MGLevelDev& cv = D.lv[l + 1];
    I3 q = coord(l, i);
    int f[3] = {lv.fx, lv.fy, lv.fz};
    if (lv.aggregate) {
      int j = q.x / f[0] + cv.nx * (q.y / f[1] + cv.ny * (q.z / f[2]));
      if (!active<T>(l + 1, j)) return 0;
      ids[0] = j;
      ws[0] = 1.f;
      return 1;
    }
    float t[3];
    int base[3];
    for (int a = 0; a < 3; a++) {
      float pos = ((float)q[a] + .5f) / (float)f[a] - .5f;
      base[a] = (int)floorf(pos);
      t[a] = fract_(pos);
    }
    int size = 0;
    for (int z = 0; z < f[2]; z++)
      for (int y = 0; y < f[1]; y++)
        for (int x = 0; x < f[0]; x++) {
          int bit[3] = {x, y, z};
          I3 nb = mk(base[0] + x, base[1] + y, base[2] + z);
          float w = 1.f;
          for (int a = 0; a < 3; a++)
            if (f[a] > 1) w *= bit[a] == 1 ? t[a] : 1.f - t[a];
          if (nb.y >= cv.ny) continue;
          nb.y = max(nb.y, 0);
          nb.x = D.px ? pmod(nb.x, cv.nx) : min(max(nb.x, 0), cv.nx - 1);
          nb.z = pmod(nb.z, cv.nz);
          int j = nb.x + cv.nx * (nb.y + cv.ny * nb.z);
          if (!active<T>(l + 1, j) || w == 0.f) continue;
          ids[size] = j;
          ws[size] = w;
          size++;
        }
    return size;
  }
  DI int transfers(int l, int i, int* ids, float* ws) const {
    const MGLevelDev& lv = D.lv[l];
    int size = 0;
    for (int k = 0; k < lv.twidth; k++) {
      float w = D.mgtw[lv.toff + (long long)k * lv.count + i];
      if (w > 0.f) {
        ids[size] = D.mgtid[lv.toff + (long long)k * lv.count + i];
        ws[size] = w;
        size++;
      }
    }
    return size;
  }
  // transfers() with every table load issued before the first weight is tested, for the
  // prolongation (the Galerkin build keeps transfers(): there the tests save most loads)
  DI int transfers_prefetched(int l, int i, int* ids, float* ws) const {
    const MGLevelDev& lv = D.lv[l];
    float w[8];
    int id[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < lv.twidth) {
        w[k] = D.mgtw[lv.toff + (long long)k * lv.count + i];
        id[k] = D.mgtid[lv.toff + (long long)k * lv.count + i];
      }
    int size = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < lv.twidth && w[k] > 0.f) {
        ids[size] = id[k];
        ws[size] = w[k];
        size++;
      }
    return size;
  }
  // apply() of a level >= 1 whose stencil has at most SMAX entries, with every load of the row
  // (its activity, the S operator values, the S neighbour values, and for a row near the level's
  // edge the S cached columns first) issued before the first addition; the sum is then formed in
  // stencil order, as apply() forms it, so the value is the same.  A sweep of a large level has
  // few active rows per SM, and this turns the row's three or four dependent memory round trips
  // into one or two.
  template <class T, int SMAX> DI float apply_wide(int l, int f, int i, const int* lin_s) const {
    const T* x = field<T>(f, l);
    const MGLevelDev& lv = D.lv[l];
    const int S = lv.stencil;
    const T* ell = (const T*)D.mgell + lv.eoff;
    const I3 q = coord(l, i);
    const bool inner = q.x >= 2 && q.x < lv.nx - 2 && q.y >= 2 && q.y < lv.ny - 2 && q.z >= 2 && q.z < lv.nz - 2;
    const bool act = active<T>(l, i);
    const float here = ld_val(x[i]);
    const int* col = D.mgcol + lv.eoff;
    float e[SMAX], v[SMAX];
#pragma unroll
    for (int k = 0; k < SMAX; k++)
      if (k < S) {
        const long long at = (long long)k * lv.count + i;
        const int j = inner ? i + lin_s[k] : __ldg(col + at);
        e[k] = ld_val(ell[at]);
        v[k] = ld_val(x[j]);
      }
    if (!act) return here;
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < SMAX; k++)
      if (k < S) sum += e[k] * v[k];
    return sum;
  }
  // apply (pressure_multigrid.glslinc:90-105) with the V-cycle operators; `lin_s` (optional) is a
  // copy of the level's linear stencil offsets in shared memory.
  template <class T> DI float apply(int l, int f, int i, const int* lin_s = nullptr) const {
    const T* x = field<T>(f, l);
    if (!active<T>(l, i)) return ld_val(x[i]);
    float sum = 0.f;
    I3 q = coord(l, i);
    if (l == 0) {
      float here = ld_val(x[i]);
      const T* c0 = (const T*)D.c0;
      for (int axis = 0; axis < 3; axis++)
        for (int side = 0; side < 2; side++) {
          int j = wrap(0, ax(q, axis, 2 * side - 1));
          float other = active<T>(0, j) ? ld_val(x[j]) : 0.f;
          float k = ld_val(c0[(long long)(2 * axis + side) * D.N + i]);
          sum += k * (here - other);
        }
      return sum;
    }
    const MGLevelDev& lv = D.lv[l];
    const T* ell = (const T*)D.mgell + lv.eoff;
    if (q.x >= 2 && q.x < lv.nx - 2 && q.y >= 2 && q.y < lv.ny - 2 && q.z >= 2 && q.z < lv.nz - 2) {
      // every stencil point is inside: the neighbour is i + linear offset, no wrap
      if (lin_s) {
#pragma unroll 13
        for (int k = 0; k < lv.stencil; k++) sum += ld_val(ell[(long long)k * lv.count + i]) * ld_val(x[i + lin_s[k]]);
        return sum;
      }
      const int* lin = D.stencil_lin + lv.soff;
#pragma unroll 8
      for (int k = 0; k < lv.stencil; k++) sum += ld_val(ell[(long long)k * lv.count + i]) * ld_val(x[i + __ldg(lin + k)]);
      return sum;
    }
    // cached columns max(j, 0) (pressure_multigrid.glslinc:180), static geometry
    const int* col = D.mgcol + lv.eoff;
#pragma unroll 8
    for (int k = 0; k < lv.stencil; k++)
      sum += ld_val(ell[(long long)k * lv.count + i]) * ld_val(x[__ldg(col + (long long)k * lv.count + i)]);
    return sum;
  }
};

// ---------------------------------------------------------------- hierarchy audit
DI unsigned signature(const Dev& D, const Grid& g, long long i) {
  if (D.kind[i] < 1) return 0;
  I3 q = g.coord(i);
  unsigned result = 0;
  for (int axis = 0; axis < 3; axis++)
    for (int side = 0; side < 2; side++) {
      I3 nb = ax(q, axis, 2 * side - 1);
      nb.z = pmod(nb.z, D.nz);
      if (D.px) nb.x = pmod(nb.x, D.nx);
      bool inside = nb.x >= 0 && nb.x < D.nx && nb.y >= 0 && nb.y < D.ny;
      bool w = inside && D.kind[g.index3(nb)] > 0;
      unsigned kind = D.coef[(long long)(2 * axis + side) * D.N + i] > 0.f ? (w ? 1u : 2u) : 0u;
      result |= kind << (2 * (2 * axis + side));
    }
  return result;
}
__global__ void k_hs_reset(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D)) return;
  unsigned* s = D.hstate;
  for (int k = 1; k <= 7; k++) s[k] = 0;
  s[14] = s[0];
  s[15] = 0;
  s[16] = 0;
  for (int k = 20; k < 32; k++) s[k] = 0;
}
struct AddU { DI unsigned operator()(unsigned a, unsigned b) const { return a + b; } };
struct MaxU { DI unsigned operator()(unsigned a, unsigned b) const { return a < b ? b : a; } };
__global__ void __launch_bounds__(NT) k_hs_count(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D)) return;
  __shared__ unsigned sh[32];
  Grid g(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  // 1 kind!=snapshot, 2 signature diffs, 3 coefficient bit diffs, 4 kind!=previous,
  // 5 signature diffs vs previous, 6 coefficient diffs vs previous, 7 max ratio bits, 15 invalid, 16 wet
  unsigned a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (i < D.N) {
    const float* cached = D.snapshot;
    const float* prev = D.previous;
    float kind = (float)D.kind[i];
    a[0] = kind != cached[7 * D.N + i];
    a[3] = kind != prev[7 * D.N + i];
    a[8] = kind > .5f;
    unsigned sig = signature(D, g, i), old = (unsigned)cached[8 * D.N + i], pv = (unsigned)prev[8 * D.N + i];
    for (int face = 0; face < 6; face++) {
      a[1] += ((sig >> (2 * face)) & 3u) != ((old >> (2 * face)) & 3u);
      a[4] += ((sig >> (2 * face)) & 3u) != ((pv >> (2 * face)) & 3u);
    }
    float ratio = 0.f;
    bool bad = false;
    for (int k = 0; k < 7; k++) {
      float value = k < 6 ? D.coef[(long long)k * D.N + i] : D.diag[i];
      float was = cached[(long long)k * D.N + i];
      a[2] += __float_as_uint(value) != __float_as_uint(was);
      a[5] += __float_as_uint(value) != __float_as_uint(prev[(long long)k * D.N + i]);
      if (was > 0.f) ratio = mxf(ratio, fabsf(value - was) / was);
      if (isnan(value) || isinf(value) || value < 0.f) bad = true;
    }
    a[6] = __float_as_uint(ratio);
    a[7] = bad ? 1u : 0u;
  }
  unsigned r[9];
  for (int k = 0; k < 9; k++) r[k] = k == 6 ? block_reduce<NT>(a[k], MaxU(), sh) : block_reduce<NT>(a[k], AddU(), sh);
  if (threadIdx.x == 0) {
    unsigned* s = D.hstate;
    const int dst[9] = {1, 2, 3, 4, 5, 6, 7, 15, 16};
    for (int k = 0; k < 9; k++) {
      if (k == 6) atomicMax(&s[7], r[k]);
      else if (r[k]) atomicAdd(&s[dst[k]], r[k]);
    }
  }
}
__global__ void k_hs_decide(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D)) return;
  unsigned* s = D.hstate;
  double* c = D.c;
  if (s[15] > 0) { c[7] = 34; return; }
  bool incompatible = s[0] == 0 || s[1] > 0 || s[2] > 0;
  bool structural = D.mg_mode == 0 || incompatible;
  bool numerical = D.mg_mode == 0 || incompatible || (s[3] > 0 && (D.mg_mode == 1 || s[10] + 1 >= (unsigned)D.mg_lag));
  s[8] = numerical ? 1 : 0;
  s[9] = structural ? 1 : 0;
  s[10] = (numerical || s[3] == 0) ? 0 : s[10] + 1;
  s[11] += s[8];
  s[12] += s[9];
  s[13] += 1;
  s[0] = 1;
  if (s[13] <= (unsigned)D.hist_cap) {
    long long row = 64 + 32 * (long long)(s[13] - 1);
    s[row] = s[13];
    s[row + 1] = __float_as_uint((float)c[1]);
    for (int k = 1; k <= 7; k++) s[row + 1 + k] = s[k];
    s[row + 9] = s[8]; s[row + 10] = s[9]; s[row + 11] = s[10]; s[row + 12] = s[16]; s[row + 13] = s[11];
  }
}
template <class T> __global__ void __launch_bounds__(NT) k_hs_snapshot(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D)) return;
  Grid g(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i >= D.N) return;
  bool num = D.hstate[8] != 0;
  for (int k = 0; k < 7; k++) {
    float value = k < 6 ? D.coef[(long long)k * D.N + i] : D.diag[i];
    D.previous[(long long)k * D.N + i] = value;
    if (num) D.snapshot[(long long)k * D.N + i] = value;
  }
  float kind = (float)D.kind[i], sig = (float)signature(D, g, i);
  D.previous[7 * D.N + i] = kind;
  D.previous[8 * D.N + i] = sig;
  if (num) {
    D.snapshot[7 * D.N + i] = kind;
    D.snapshot[8 * D.N + i] = sig;
    if (D.bf16) {
      T* c0 = (T*)D.c0;
      for (int k = 0; k < 6; k++) c0[(long long)k * D.N + i] = st_val<T>(D.coef[(long long)k * D.N + i]);
    }
  }
}
__global__ void k_hs_record(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D)) return;
  unsigned* s = D.hstate;
  if (s[13] <= (unsigned)D.hist_cap) {
    long long row = 64 + 32 * (long long)(s[13] - 1);
    for (int l = 0; l < 12; l++) s[row + 16 + l] = s[20 + l];
  }
}

// ---------------------------------------------------------------- build ops
template <class T> __global__ void __launch_bounds__(NT) k_mg_mask(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[9] == 0) return;
  __shared__ unsigned sh[32];
  MG m(D);
  int i = blockIdx.x * NT + threadIdx.x;
  const MGLevelDev& lv = D.lv[l];
  unsigned changed = 0;
  if (i < lv.count) {
    float value = 0.f;
    if (l == 0) value = D.kind[i] > 0 ? 1.f : 0.f;
    else {
      const MGLevelDev& pv = D.lv[l - 1];
      I3 base = m.coord(l, i);
      base = mk(base.x * pv.fx, base.y * pv.fy, base.z * pv.fz);
      for (int z = 0; z < pv.fz; z++)
        for (int y = 0; y < pv.fy; y++)
          for (int x = 0; x < pv.fx; x++)
            if (m.active<T>(l - 1, m.wrap(l - 1, addI(base, mk(x, y, z))))) value = 1.f;
    }
    T* f3 = m.field<T>(3, l);
    if (ld_val(f3[i]) != value) changed = 1;
    f3[i] = st_val<T>(value);
  }
  unsigned r = block_reduce<NT>(changed, AddU(), sh);
  if (threadIdx.x == 0 && r) atomicAdd(&D.hstate[20 + l], r);
}
// Active rows of each level >= 1, rebuilt from the current masks at every multigrid build.  The
// sweeps, residuals and prolongations of levels >= 1 visit only these rows: an inactive row's
// entries against active rows are exactly zero, restriction reads active children only and
// prolongation adds at active cells only, so the rows skipped never reach level 0 (their
// iterates stay at the zero the restriction writes).  Warps append contiguously.
__global__ void k_mg_rows_reset(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D)) return;
  if (threadIdx.x < kMaxLevels) D.mg_rowcount[threadIdx.x] = 0u;
}
template <class T> __global__ void __launch_bounds__(NT) k_mg_rowlist(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D)) return;
  MG m(D);
  const MGLevelDev& lv = D.lv[l];
  const int i = blockIdx.x * NT + threadIdx.x;
  const bool act = i < lv.count && m.active<T>(l, i);
  const unsigned ballot = __ballot_sync(0xffffffffu, act);
  const int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (lane == 0 && ballot) base = atomicAdd(&D.mg_rowcount[l], (unsigned)__popc(ballot));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (act) D.mg_rowlist[lv.off + base + __popc(ballot & ((1u << lane) - 1u))] = i;
}
template <class T> __global__ void __launch_bounds__(NT) k_mg_transfer(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || !(D.hstate[14] == 0 || D.hstate[20 + l + 1] != 0)) return;
  MG m(D);
  const MGLevelDev& lv = D.lv[l];
  int i = blockIdx.x * NT + threadIdx.x;
  if (i >= lv.count) return;
  int ids[8];
  float ws[8];
  int size = m.compute_transfers<T>(l, i, ids, ws);
  for (int k = 0; k < lv.twidth; k++) {
    D.mgtid[lv.toff + (long long)k * lv.count + i] = k < size ? ids[k] : 0;
    D.mgtw[lv.toff + (long long)k * lv.count + i] = k < size ? ws[k] : 0.f;
    D.mgtq[lv.toff + (long long)k * lv.count + i] = k < size ? MG::pack(m.coord(l + 1, ids[k])) : 0ull;
  }
}
// l1-Jacobi scale (pressure_multigrid.glslinc:183-189) of level 0; the levels >= 1 take k_mg_scale8,
// whose row sum runs over the level's stencil entries k = 0..S-1, adding |a_ij| for every entry
// whose neighbour j does not repeat an earlier entry's.
template <class T> __global__ void __launch_bounds__(NT) k_mg_scale(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[8] == 0) return;
  MG m(D);
  const int l = 0;
  int i = blockIdx.x * NT + threadIdx.x;
  if (i >= D.lv[0].count) return;
  I3 q = m.coord(l, i);
  float sum = m.fine_coef(12, i);
  for (int axis = 0; axis < 3; axis++)
    for (int side = 0; side < 2; side++)
      if (m.active<T>(0, m.wrap(0, ax(q, axis, 2 * side - 1)))) sum += m.fine_coef(6 + 2 * axis + side, i);
  if (!(sum > 0.f) || isnan(sum) || isinf(sum)) {
    D.c[7] = 32;
    return;
  }
  m.field<T>(4, l)[i] = st_val<T>(1.f / sum);
}
// The l1-Jacobi scale (pressure_multigrid.glslinc:183-189) of a level >= 1 with eight lanes per
// row: lane g forms |a_ij| of the row's entries k = g, g + 8, g + 16, ... (-1 for an entry whose
// neighbour repeats an earlier entry's, or past the stencil), and lane 0 adds the terms from the
// eight lanes by shuffle in stencil order k = 0..S-1: the additions of the sequential loop over the
// stencil, in its order, so the same bits, with the row's loads spread over eight lanes.
constexpr int kScaleLanes = 8;
template <class T> __global__ void __launch_bounds__(NT) k_mg_scale8(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[8] == 0) return;
  const MG m(D);
  const MGLevelDev& lv = D.lv[l];
  const int t = blockIdx.x * NT + threadIdx.x;
  if ((t & ~31) / kScaleLanes >= lv.count) return;  // the warp's first row: uniform over the warp
  const int r = t / kScaleLanes, g = t % kScaleLanes, lane = threadIdx.x & 31;
  const bool ok = r < lv.count;  // no lane of the warp leaves before the shuffles
  const int i = ok ? r : lv.count - 1;
  const I3 q = m.coord(l, i);
  constexpr int E = (kMaxStencil + kScaleLanes - 1) / kScaleLanes;
  float term[E];
#pragma unroll
  for (int e = 0; e < E; e++) {
    const int k = kScaleLanes * e + g;
    term[e] = -1.f;
    if (k < lv.stencil) {
      const I3 off = m.offset(l, k);
      const int j = m.wrap(l, addI(q, off));
      if (m.unique_neighbor(l, i, off, j)) term[e] = fabsf(m.coefficient<T>(l, i, j));
    }
  }
  const int base = lane & ~(kScaleLanes - 1);
  float sum = 0.f;
#pragma unroll
  for (int e = 0; e < E; e++)
#pragma unroll
    for (int h = 0; h < kScaleLanes; h++) {
      const float v = __shfl_sync(0xffffffffu, term[e], base + h);
      if (!(v < 0.f)) sum += v;  // every |a_ij| (a NaN included), never the -1 of no term
    }
  if (!ok || g != 0) return;
  if (!(sum > 0.f) || isnan(sum) || isinf(sum)) {
    D.c[7] = 32;
    return;
  }
  m.field<T>(4, l)[i] = st_val<T>(1.f / sum);
}
// Children box of coarse coordinate qc along one axis of fine level l.
DI void child_range(const Dev& D, int l, int axis, int qc, int& lo, int& ext) {
  const MGLevelDev& lv = D.lv[l];
  int f = axis == 0 ? lv.fx : (axis == 1 ? lv.fy : lv.fz);
  int nf = axis == 0 ? lv.nx : (axis == 1 ? lv.ny : lv.nz);
  if (lv.aggregate || f == 1) { lo = qc * f; ext = f; return; }
  lo = qc * f - 1;
  ext = 4;
  bool periodic = axis == 2 || (axis == 0 && D.px);
  if (periodic && nf <= 4) { lo = 0; ext = nf; }
}
// Deterministic Galerkin product of level l into level l+1 (replaces ops 2 + 3).
template <class T> __global__ void __launch_bounds__(GT) k_mg_galerkin(const __grid_constant__ Dev D, int l, int ex, int ey, int ez) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[8] == 0) return;
  // [slots][GT]: one slot per offset of the 5x5x5 box, or one per stencil entry of the coarse level
  // (gal_slots > 0; the slot map is the same for every row, so each slot's terms are added in the
  // same order either way)
  extern __shared__ float part[];
  MG m(D);
  const int G = ey * ez, rpb = GT / G;
  const MGLevelDev& fl = D.lv[l];
  const MGLevelDev& cl = D.lv[l + 1];
  const int t = threadIdx.x;
  const int nslots = cl.gal_slots > 0 ? cl.gal_slots : 125;
  __shared__ I3 offs[kMaxStencil];
  __shared__ signed char cslot[125];
  for (int k = t; k < fl.stencil; k += GT) offs[k] = m.offset(l, k);
  for (int s = t; s < 125; s += GT) cslot[s] = cl.gal_slots > 0 ? D.gal_cslot[(l + 1) * 125 + s] : (signed char)s;
  for (int s = 0; s < nslots; s++) part[s * GT + t] = 0.f;
  __syncthreads();
  int row_local = t / G, g = t % G;
  int I = blockIdx.x * rpb + row_local;
  // Every lane runs the same loops (bounds made uniform over the warp) and a term is added only
  // where the index form adds it, so the lanes of a warp stay converged.  The terms and their
  // order are those of the index form: for each fine cell i (x fastest in this thread's row of
  // children), each of i's transfers to I, each stencil neighbour j, each of j's transfers.  Cell
  // coordinates are carried along instead of decoded from indices: qi from the loop, qj from
  // qi + offset, the coarse coordinates of j's transfers from the table (mgtq).
  const bool rowok = row_local < rpb && I < cl.count && m.active<T>(l + 1, I);
  const I3 qc = rowok ? m.coord(l + 1, I) : mk(0, 0, 0);
  int lo[3] = {0, 0, 0}, ext[3] = {0, 0, 0};
  if (rowok)
    for (int a = 0; a < 3; a++) child_range(D, l, a, qc[a], lo[a], ext[a]);
  const int gz = g / ey, gy = g % ey;
  const long long tstride = fl.count;
  const int nxi = __reduce_max_sync(0xffffffffu, (unsigned)ext[0]);
  for (int gx = 0; gx < nxi; gx++) {
    I3 qi = mk(lo[0] + gx, lo[1] + gy, lo[2] + gz);
    bool cell = rowok && gx < ext[0] && m.wrap_q(l, qi);
    if (!cell) qi = mk(0, 0, 0);
    const int i = qi.x + fl.nx * (qi.y + fl.ny * qi.z);
    cell = cell && m.active<T>(l, i);
    int li[8];
    float lw[8];
    const int nl = cell ? m.transfers(l, i, li, lw) : 0;
    unsigned match = 0;
    for (int a = 0; a < nl; a++)
      if (li[a] == I) match |= 1u << a;
    const int nmatch = __popc(match);
    const int rounds = __reduce_max_sync(0xffffffffu, (unsigned)nmatch);
    for (int r = 0; r < rounds; r++) {
      const bool has = r < nmatch;
      const int a = has ? __ffs(match) - 1 : 0;
      if (has) match &= match - 1;
      const float lwa = has ? lw[a] : 0.f;
      for (int k = 0; k < fl.stencil; k++) {
        // every load of one neighbour (its activity, the coefficient, its transfers) is issued
        // before the first test; a neighbour outside the grid loads from i instead
        const I3 off = offs[k];
        I3 qj = addI(qi, off);
        const bool in = m.wrap_q(l, qj);
        const int j = in ? qj.x + fl.nx * (qj.y + fl.ny * qj.z) : i;
        if (!in) qj = qi;
        bool uniq = true;
        long long maddr = -1;
        if (l > 0) {
          // unique_neighbor and coefficient() of two active cells
          uniq = eqI(m.delta_q(l, qi, qj), off);
          const bool ilo = i <= j;
          const I3 d = ilo ? m.delta_q(l, qi, qj) : m.delta_q(l, qj, qi);
          if (!(abs(d.x) > 2 || abs(d.y) > 2 || abs(d.z) > 2)) maddr = fl.moff + (long long)(ilo ? i : j) * 125 + MG::slot(d);
        }
        const bool actj = m.active<T>(l, j);
        const float aij = l == 0 ? (k == 0 ? m.fine_coef(12, i) : -m.fine_coef(5 + k, i)) : (maddr >= 0 ? D.mgmat[maddr] : 0.f);
        const long long tj = fl.toff + j;
        float wv[8];
        unsigned long long qv[8];
#pragma unroll
        for (int b = 0; b < 8; b++)
          if (b < fl.twidth) {
            wv[b] = D.mgtw[tj + b * tstride];
            qv[b] = D.mgtq[tj + b * tstride];
          }
        const bool use = has && in && actj && uniq && aij != 0.f;
        const float al = aij * lwa;
#pragma unroll
        for (int b = 0; b < 8; b++) {
          if (b >= fl.twidth) break;
          const bool ub = use && wv[b] > 0.f;
          const I3 d = m.delta_q(l + 1, qc, MG::unpack(qv[b]));
          const bool far = abs(d.x) > 2 || abs(d.y) > 2 || abs(d.z) > 2;
          const int cs = far ? -1 : cslot[MG::slot(d)];
          if (ub && (far || cs < 0)) D.c[7] = 31;
          if (ub && cs >= 0) part[cs * GT + t] += al * wv[b];
        }
      }
    }
  }
  // the rows' activity and coordinates once per row (not once per slot): an inactive row, most of
  // a coarse level, only stores its zeros
  __shared__ bool ract[GT];
  __shared__ I3 rq[GT];
  if (t < rpb) {
    const int row = blockIdx.x * rpb + t;
    ract[t] = row < cl.count && m.active<T>(l + 1, row);
    rq[t] = row < cl.count ? m.coord(l + 1, row) : mk(0, 0, 0);
  }
  __syncthreads();
  for (int u = t; u < rpb * 125; u += GT) {
    int rl = u / 125, s = u % 125;
    int row = blockIdx.x * rpb + rl;
    if (row >= cl.count) continue;
    float out = 0.f;
    if (ract[rl]) {
      float total = 0.f;
      const int cs = cslot[s];
      if (cs >= 0)
        for (int gg = 0; gg < G; gg++) total += part[cs * GT + rl * G + gg];
      const I3 d = mk(s % 5 - 2, (s / 5) % 5 - 2, s / 25 - 2);
      I3 qj = addI(rq[rl], d);
      const bool in = m.wrap_q(l + 1, qj);
      const int J = in ? qj.x + cl.nx * (qj.y + cl.ny * qj.z) : -1;
      const bool canonical = J >= row && eqI(m.delta_q(l + 1, rq[rl], qj), d);
      out = canonical ? total : 0.f;
    }
    D.mgmat[cl.moff + (long long)row * 125 + s] = out;
  }
}
// Galerkin product from a fine level l >= 1 in two stages (the oracle's mg_galerkin_ap and
// mg_galerkin_pt, the same additions in the same order).  Stage 1: one thread per active fine row
// i (the level's active-row list) accumulates A P over the 125 coarse offsets e = delta(home(i), J)
// (home(i) = the coarse cell containing i) in shared memory, in the order stencil neighbour j,
// transfer of j; the block then writes its rows' 125 slots to gal_ap (row-major by fine cell).
constexpr int GA = 64;  // stage-1 threads per block (125 x 64 x 4 B = 32 KB of partials)
template <class T> __global__ void __launch_bounds__(GA) k_mg_gal_ap(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[8] == 0) return;
  extern __shared__ float acc[];  // [125][GA]
  __shared__ I3 offs[kMaxStencil];
  __shared__ int rows[GA];
  const MG m(D);
  const MGLevelDev& fl = D.lv[l];
  const int t = threadIdx.x;
  for (int k = t; k < fl.stencil; k += GA) offs[k] = m.offset(l, k);
  const int nrows = (int)D.mg_rowcount[l];
  const long long tstride = fl.count;
  for (int r0 = blockIdx.x * GA; r0 < nrows; r0 += gridDim.x * GA) {  // uniform over the block
    for (int e = 0; e < 125; e++) acc[e * GA + t] = 0.f;
    const bool ok = r0 + t < nrows;
    const int i = ok ? D.mg_rowlist[fl.off + r0 + t] : 0;
    rows[t] = ok ? i : -1;
    __syncthreads();
    const I3 qi = m.coord(l, i);
    const I3 home = mk(qi.x / fl.fx, qi.y / fl.fy, qi.z / fl.fz);
    for (int k = 0; k < fl.stencil; k++) {
      // every load of one neighbour (its activity, the coefficient, its transfers) is issued
      // before the first test; a neighbour outside the grid loads from i instead
      const I3 off = offs[k];
      I3 qj = addI(qi, off);
      const bool in = m.wrap_q(l, qj);
      const int j = in ? qj.x + fl.nx * (qj.y + fl.ny * qj.z) : i;
      if (!in) qj = qi;
      const bool uniq = eqI(m.delta_q(l, qi, qj), off);
      const bool ilo = i <= j;
      const I3 d = ilo ? m.delta_q(l, qi, qj) : m.delta_q(l, qj, qi);
      const long long maddr =
          (abs(d.x) > 2 || abs(d.y) > 2 || abs(d.z) > 2) ? -1 : fl.moff + (long long)(ilo ? i : j) * 125 + MG::slot(d);
      const bool actj = m.active<T>(l, j);
      const float aij = maddr >= 0 ? D.mgmat[maddr] : 0.f;
      const long long tj = fl.toff + j;
      float wv[8];
      unsigned long long qv[8];
#pragma unroll
      for (int b = 0; b < 8; b++)
        if (b < fl.twidth) {
          wv[b] = D.mgtw[tj + b * tstride];
          qv[b] = D.mgtq[tj + b * tstride];
        }
      const bool use = ok && in && actj && uniq && aij != 0.f;
#pragma unroll
      for (int b = 0; b < 8; b++) {
        if (b >= fl.twidth) break;
        const bool ub = use && wv[b] > 0.f;
        const I3 e = m.delta_q(l + 1, home, MG::unpack(qv[b]));
        const bool far = abs(e.x) > 2 || abs(e.y) > 2 || abs(e.z) > 2;
        if (ub && far) D.c[7] = 31;
        if (ub && !far) acc[MG::slot(e) * GA + t] += aij * wv[b];
      }
    }
    __syncthreads();
    // the block's rows, 125 consecutive floats each
    for (int u = t; u < GA * 125; u += GA) {
      const int r = u / 125, e = u - r * 125;
      if (rows[r] >= 0) D.gal_ap[(long long)rows[r] * 125 + e] = acc[e * GA + r];
    }
    __syncthreads();
  }
}
// Stage 2: one block per coarse row I.  The children of I (the box of child_range, in the order
// gz, gy, gx) with their home cells and their transfer weights to I go to shared memory; thread s
// (a slot, d_s = the 5 x 5 x 5 offset) then adds, for a canonical slot (J = I + d_s, J >= I),
// w_iI * ap_i[delta(home(i), J)] over the children and their transfers to I in order.  Inactive
// rows and non-canonical slots get zeros, as in the one-stage form.
constexpr int GP = 128;
template <class T> __global__ void __launch_bounds__(GP) k_mg_gal_pt(const __grid_constant__ Dev D, int l, int ex, int ey, int ez) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[8] == 0) return;
  __shared__ int ch_i[64];
  __shared__ I3 ch_home[64];
  __shared__ int ch_n[64];
  __shared__ float ch_w[64][8];
  const MG m(D);
  const MGLevelDev& cl = D.lv[l + 1];
  const int t = threadIdx.x, nch = ex * ey * ez;
  for (int I = blockIdx.x; I < cl.count; I += gridDim.x) {  // uniform over the block
    float* row = D.mgmat + cl.moff + (long long)I * 125;
    if (!m.active<T>(l + 1, I)) {
      if (t < 125) row[t] = 0.f;
      continue;
    }
    const I3 qc = m.coord(l + 1, I);
    if (t < nch) {
      int lo[3], ext[3];
      for (int a = 0; a < 3; a++) child_range(D, l, a, qc[a], lo[a], ext[a]);
      const int gx = t % ex, gy = (t / ex) % ey, gz = t / (ex * ey);
      I3 qi = mk(lo[0] + gx, lo[1] + gy, lo[2] + gz);
      const MGLevelDev& fl = D.lv[l];
      bool cell = m.wrap_q(l, qi);
      const int i = cell ? qi.x + fl.nx * (qi.y + fl.ny * qi.z) : 0;
      cell = cell && m.active<T>(l, i);
      int n = 0;
      if (cell) {
        int li[8];
        float lw[8];
        const int nl = m.transfers(l, i, li, lw);
        for (int a = 0; a < nl; a++)
          if (li[a] == I) ch_w[t][n++] = lw[a];
      }
      ch_i[t] = i;
      ch_n[t] = n;
      ch_home[t] = mk(qi.x / fl.fx, qi.y / fl.fy, qi.z / fl.fz);
    }
    __syncthreads();
    if (t < 125) {
      const I3 d = mk(t % 5 - 2, (t / 5) % 5 - 2, t / 25 - 2);
      I3 qj = addI(qc, d);
      const bool in = m.wrap_q(l + 1, qj);
      const int J = in ? qj.x + cl.nx * (qj.y + cl.ny * qj.z) : -1;
      const bool canonical = in && J >= I && eqI(m.delta_q(l + 1, qc, qj), d);
      float total = 0.f;
      if (canonical)
        for (int c = 0; c < nch; c++) {
          const int n = ch_n[c];
          if (n == 0) continue;
          const I3 e = m.delta_q(l + 1, ch_home[c], qj);
          if (abs(e.x) > 2 || abs(e.y) > 2 || abs(e.z) > 2) continue;
          const float v = D.gal_ap[(long long)ch_i[c] * 125 + MG::slot(e)];
          for (int a = 0; a < n; a++) total += ch_w[c][a] * v;
        }
      row[t] = canonical ? total : 0.f;
    }
    __syncthreads();
  }
}

// ELL rows (pressure_multigrid.glslinc:176-182), one thread per entry: entry k of row i (stored at
// k * count + i) is the same function of (i, k) whichever thread forms it, and a row no longer
// waits on its entries' loads one after the other (up to 125 of them on a coarse level).
template <class T> __global__ void __launch_bounds__(NT) k_mg_ell(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[8] == 0) return;
  MG m(D);
  const MGLevelDev& lv = D.lv[l];
  const long long t = (long long)blockIdx.x * NT + threadIdx.x;
  if (t >= (long long)lv.stencil * lv.count) return;
  const int k = (int)(t / lv.count), i = (int)(t - (long long)k * lv.count);
  const I3 q = m.coord(l, i);
  const I3 off = m.offset(l, k);
  const int j = m.wrap(l, addI(q, off));
  const float a = m.unique_neighbor(l, i, off, j) ? m.coefficient<T>(l, i, j) : 0.f;
  ((T*)D.mgell + lv.eoff)[t] = st_val<T>(a);
}
// Dense Cholesky and L^-1 of the last level (pressure_mg_coarse.glslinc:34-48), one block.
template <class T> __global__ void k_mg_chol(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[8] == 0) return;
  __shared__ float dense[64 * 64];
  __shared__ float inv[64 * 64];
  MG m(D);
  const int n = D.lv[l].count;
  const int t = threadIdx.x;
  for (int k = t; k < n * n; k += blockDim.x) dense[k] = m.coefficient<T>(l, k / n, k % n);
  __syncthreads();
  for (int k = 0; k < n; k++) {
    if (t == 0) {
      float d = dense[k * n + k];
      for (int j = 0; j < k; j++) d -= dense[k * n + j] * dense[k * n + j];
      if (!(d > 0.f) || isnan(d) || isinf(d)) {
        D.c[7] = 33;
        d = 1.f;
      }
      dense[k * n + k] = sqrtf(d);
    }
    __syncthreads();
    if (t > k && t < n) {
      float e = dense[t * n + k];
      for (int j = 0; j < k; j++) e -= dense[t * n + j] * dense[k * n + j];
      dense[t * n + k] = e / dense[k * n + k];
    }
    __syncthreads();
  }
  for (int row = 0; row < n; row++) {
    if (t < n) {
      float d = t == row ? 1.f : 0.f;
      for (int j = 0; j < row; j++) d -= dense[row * n + j] * inv[j * n + t];
      inv[row * n + t] = d / dense[row * n + row];
    }
    __syncthreads();
  }
  for (int k = t; k < n * n; k += blockDim.x) D.mglinv[k] = inv[k];
}

// ---------------------------------------------------------------- V-cycle
// Per-cell operations, shared by the grid kernels and by the single-block bottom solver.  `ax`
// is apply(l, source, i) of the cell (unused where the update needs no operator).
template <class T, class M> DI void cheb_update(const M& m, int l, int source, int k, int i, bool src_zero, float ax) {
  float c1 = (float)(2 * k - 3) / (float)(2 * k + 1), c2 = (float)(8 * k - 4) / (float)(2 * k + 1);
  const T* x = m.template field<T>(source, l);
  // A zero iterate makes apply() exactly +0, so r = b exactly; skip the operator.
  float r = src_zero ? ld_val(m.template field<T>(0, l)[i]) : ld_val(m.template field<T>(0, l)[i]) - ax;
  T* v7 = m.template field<T>(7, l);
  float d = (k == 1 ? 0.f : c1 * ld_val(v7[i])) + c2 * ld_val(m.template field<T>(4, l)[i]) * r;
  float xv = (src_zero ? 0.f : ld_val(x[i])) + d;
  v7[i] = st_val<T>(d);
  m.template field<T>(3 - source, l)[i] = st_val<T>(xv);
}
template <class T, class M> DI void jacobi_update(const M& m, int l, int source, int first, int i, float ax) {
  float s = ld_val(m.template field<T>(4, l)[i]), b = ld_val(m.template field<T>(0, l)[i]);
  if (first) m.template field<T>(2, l)[i] = st_val<T>(s * b);
  else m.template field<T>(3 - source, l)[i] = st_val<T>(ld_val(m.template field<T>(source, l)[i]) + s * (b - ax));
}
template <class T, class M> DI void residual_update(const M& m, int l, int i, float ax) {
  m.template field<T>(6, l)[i] = st_val<T>(ld_val(m.template field<T>(0, l)[i]) - ax);
}
template <class T, class M> DI void cheb_cell(const M& m, int l, int source, int k, int i, bool src_zero) {
  cheb_update<T>(m, l, source, k, i, src_zero, src_zero ? 0.f : m.template apply<T>(l, source, i));
}
template <class T, class M> DI void jacobi_cell(const M& m, int l, int source, int first, int i) {
  jacobi_update<T>(m, l, source, first, i, first ? 0.f : m.template apply<T>(l, source, i));
}
template <class T, class M> DI void residual_cell(const M& m, int l, int f, int i) { residual_update<T>(m, l, i, m.template apply<T>(l, f, i)); }

// Product-parallel apply for levels >= 1: the whole block computes the products
// ell[k][i] * x[col(k, i)] of RR consecutive rows into shared memory (every load independent),
// then one thread per row adds its products in stencil order k = 0, 1, ... -- the same roundings
// and the same order as apply(), so the value is bit-identical.
constexpr int RR = 32;
template <class T, int NTB = NT, int RRB = RR>
DI void row_products(const MG& m, int l, int src, const int* rowi, float* prod, bool* inner, int* lin) {
  const Dev& D = m.D;
  const MGLevelDev& lv = D.lv[l];
  const int S = lv.stencil, n = lv.count;
  if (threadIdx.x < RRB) {
    int i = rowi[threadIdx.x];
    I3 q = m.coord(l, i >= 0 ? i : 0);
    inner[threadIdx.x] = q.x >= 2 && q.x < lv.nx - 2 && q.y >= 2 && q.y < lv.ny - 2 && q.z >= 2 && q.z < lv.nz - 2;
  }
  for (int k = threadIdx.x; k < S; k += NTB) lin[k] = __ldg(D.stencil_lin + lv.soff + k);
  __syncthreads();
  const T* x = m.field<T>(src, l);
  const T* ell = (const T*)D.mgell + lv.eoff;
  const int* col = D.mgcol + lv.eoff;
#pragma unroll 4
  for (int p = threadIdx.x; p < S * RRB; p += NTB) {
    const int k = p / RRB, r = p % RRB, i = rowi[r];
    float v = 0.f;
    if (i >= 0) {
      const long long e = (long long)k * n + i;
      const int j = inner[r] ? i + lin[k] : __ldg(col + e);
      v = ld_val(ell[e]) * ld_val(x[j]);
    }
    prod[p] = v;
  }
  __syncthreads();
}
template <class T, int RRB = RR> DI float row_sum(const MG& m, int l, int src, int i, const float* prod) {
  if (!m.active<T>(l, i)) return ld_val(m.field<T>(src, l)[i]);
  const int S = m.D.lv[l].stencil;
  float sum = 0.f;
  // unrolled so that the shared-memory loads run ahead of the additions (which stay in order)
#pragma unroll 8
  for (int k = 0; k < S; k++) sum += prod[k * RRB + threadIdx.x];
  return sum;
}

// op 8: exact P^T restriction into coarse level l (pressure_multigrid.glslinc:200-224); the
// per-axis weights come from the tables built with the same arithmetic at set-up.
template <class T, class M> DI void restrict_cell(const M& m, int l, int i) {
  const Dev& D = m.D;
  const MGLevelDev& cv = D.lv[l];
  const int parent = l - 1;
  const MGLevelDev& pv = D.lv[parent];
  const T* r6 = m.template field<T>(6, parent);
  float sum = 0.f;
  I3 qc = m.coord(l, i);
  if (m.template active<T>(l, i)) {
    if (pv.aggregate) {
      // the (at most 2 x 2 x 2) children's flags and residuals loaded before the additions, which
      // follow in the (z, y, x) order
      bool act[8];
      float rv[8];
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int x = c & 1, y = (c >> 1) & 1, z = c >> 2;
        const bool in = x < pv.fx && y < pv.fy && z < pv.fz;
        const int j = in ? m.wrap(parent, mk(qc.x * pv.fx + x, qc.y * pv.fy + y, qc.z * pv.fz + z)) : -1;
        act[c] = in && m.template active<T>(parent, j);
        rv[c] = j >= 0 ? ld_val(r6[j]) : 0.f;
      }
#pragma unroll
      for (int c = 0; c < 8; c++)
        if (act[c]) sum += rv[c];
    } else {
      const int* ix = D.rt_idx + cv.roff[0] + 4 * qc.x;
      const int* iy = D.rt_idx + cv.roff[1] + 4 * qc.y;
      const int* iz = D.rt_idx + cv.roff[2] + 4 * qc.z;
      const float* wx = D.rt_w + cv.roff[0] + 4 * qc.x;
      const float* wy = D.rt_w + cv.roff[1] + 4 * qc.y;
      const float* wz = D.rt_w + cv.roff[2] + 4 * qc.z;
      // per plane of the children box (at most 4 x 4), every activity flag and residual is loaded
      // before the additions, which follow in the (ty, tx) order with the same weights
      for (int tz = 0; tz < cv.rext[2]; tz++) {
        bool act[4][4];
        float rv[4][4];
#pragma unroll
        for (int ty = 0; ty < 4; ty++)
#pragma unroll
          for (int tx = 0; tx < 4; tx++) {
            const bool ok = ty < cv.rext[1] && tx < cv.rext[0] && iy[ty] >= 0 && ix[tx] >= 0;
            const int j = ok ? ix[tx] + pv.nx * (iy[ty] + pv.ny * iz[tz]) : 0;
            act[ty][tx] = ok && m.template active<T>(parent, j);
            rv[ty][tx] = ld_val(r6[j]);
          }
#pragma unroll
        for (int ty = 0; ty < 4; ty++)
#pragma unroll
          for (int tx = 0; tx < 4; tx++)
            if (act[ty][tx]) {
              float weight = 1.f * wx[tx] * wy[ty] * wz[tz];
              sum += weight * rv[ty][tx];
            }
      }
    }
  }
  m.template field<T>(0, l)[i] = st_val<T>(sum);
  m.template field<T>(1, l)[i] = st_val<T>(0.f);
  m.template field<T>(2, l)[i] = st_val<T>(0.f);
}
template <class T, class M> DI void prolong_cell(const M& m, int l, int ff, int cf, int i) {
  float add = 0.f;
  if (m.template active<T>(l, i)) {
    int ids[8];
    float ws[8];
    // The stored transfers are compute_transfers() on the current coarse mask (rebuilt whenever
    // that mask changes); at level 0 recomputing them is cheaper than reading the table.
    int size = l == 0 ? m.template compute_transfers<T>(l, i, ids, ws) : m.transfers_prefetched(l, i, ids, ws);
    const T* xc = m.template field<T>(cf, l + 1);
    for (int k = 0; k < size; k++) add += ws[k] * ld_val(xc[ids[k]]);
  }
  T* x = m.template field<T>(ff, l);
  x[i] = st_val<T>(ld_val(x[i]) + add);
}
// op 12: x = L^-T (L^-1 b), threads 0..n-1 of one block
template <class T, class M> DI void coarse_block(const M& m, int l, float* small) {
  const Dev& D = m.D;
  const int n = D.lv[l].count, t = threadIdx.x;
  const T* b = m.template field<T>(0, l);
  const float* linv = m.coarse_inverse();
  if (t < n) {
    float d = 0.f;
#pragma unroll 8
    for (int j = 0; j <= t; j++) d += linv[t * n + j] * ld_val(b[j]);
    small[t] = d;
  }
  __syncthreads();
  if (t < n) {
    float d = 0.f;
#pragma unroll 8
    for (int j = t; j < n; j++) d += linv[j * n + t] * small[j];
    m.template field<T>(1, l)[t] = st_val<T>(d);
  }
  __syncthreads();
}

// Level 0: each 256-thread block covers a 32 (x) by 8 (y) tile of one z plane, so a warp reads
// 128 contiguous bytes of every field; mgnb0 holds the neighbour-active bits.  Indices are 32-bit
// (level 0 holds fewer than 2^31 cells).
constexpr int kTileX = 32, kTileY = NT / kTileX;
struct Cell0 {
  int x, y, z, i;
  bool ok;
};
DI Cell0 cell0(const Dev& D) {
  Cell0 c;
  c.x = blockIdx.x * kTileX + (threadIdx.x & (kTileX - 1));
  c.y = blockIdx.y * kTileY + threadIdx.x / kTileX;
  c.z = blockIdx.z;
  c.ok = c.x < D.nx && c.y < D.ny;
  c.i = c.ok ? c.x + D.nx * (c.y + D.ny * c.z) : 0;
  return c;
}
template <class T> DI T* field0(const Dev& D, int f) { return (T*)D.mgv + (size_t)f * (size_t)D.mg_nodes; }
// apply at level 0 (pressure_multigrid.glslinc:93-99) with neighbour activity from one byte.
// Every load is issued before the activity bits are known: neighbour indices are clamped to the
// cell itself where no neighbour exists, and a value whose bit is clear is replaced by zero.
template <class T> DI float apply0(const Dev& D, const T* __restrict__ x, const Cell0& c) {
  const T* __restrict__ c0 = (const T*)D.c0;
  const int nx = D.nx, plane = D.nx * D.ny, N = (int)D.N;
  int nb[6];
  nb[0] = c.x > 0 ? c.i - 1 : c.i + (nx - 1);
  nb[1] = c.x < nx - 1 ? c.i + 1 : c.i - (nx - 1);
  nb[2] = c.y > 0 ? c.i - nx : c.i;
  nb[3] = c.y < D.ny - 1 ? c.i + nx : c.i;
  nb[4] = c.z > 0 ? c.i - plane : c.i + plane * (D.nz - 1);
  nb[5] = c.z < D.nz - 1 ? c.i + plane : c.i - plane * (D.nz - 1);
  const unsigned m = D.mgnb0[c.i];
  const float here = ld_val(x[c.i]);
  float xo[6], kf[6];
#pragma unroll
  for (int f = 0; f < 6; f++) {
    xo[f] = ld_val(x[nb[f]]);
    kf[f] = ld_val(c0[f * N + c.i]);
  }
  if (!(m & 64u)) return here;
  float sum = 0.f;
#pragma unroll
  for (int f = 0; f < 6; f++) {
    float other = (m >> f) & 1u ? xo[f] : 0.f;
    sum += kf[f] * (here - other);
  }
  return sum;
}
// Chebyshev sweep k at level 0 (coefficients c1 = (2k-3)/(2k+1), c2 = (8k-4)/(2k+1), rounded to
// float by the caller); with fin >= 0 it is the last post-smoothing sweep and also does op 10 of
// the cycle (z, partial sums) and the op 4 (phase 0) / op 9 (phase 1) finalisation.
template <class T>
__global__ void __launch_bounds__(NT) k_mg0_cheb(const __grid_constant__ Dev D, int phase, int source, float c1, float c2,
                                                  int first_k, int src_zero, int fin) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  const Cell0 c = cell0(D);
  double v[3] = {0, 0, 0};
  float vmax[1] = {0.f};
  if (c.ok) {
    const T* __restrict__ x = field0<T>(D, source);
    T* v7 = field0<T>(D, 7);
    const float b = ld_val(field0<T>(D, 0)[c.i]);
    const float sc = ld_val(field0<T>(D, 4)[c.i]);
    const float dprev = first_k ? 0.f : ld_val(v7[c.i]);
    const float r = src_zero ? b : b - apply0<T>(D, x, c);
    const float d = (first_k ? 0.f : c1 * dprev) + c2 * sc * r;
    const float xv = (src_zero ? 0.f : ld_val(x[c.i])) + d;
    const T xs = st_val<T>(xv);
    if (fin < 0) {
      v7[c.i] = st_val<T>(d);
      field0<T>(D, 3 - source)[c.i] = xs;
    } else {
      const float rr = D.r[c.i], z = ld_val(xs), bb = D.b[c.i];
      D.z[c.i] = z;
      if (phase == 0) D.d[c.i] = z;
      // FP64 terms only where they can be other than zero
      if (rr != 0.f || !isfinite(z)) {
        v[0] = exact_product(rr, z);
        v[1] = exact_product(rr, rr);
      }
      if (bb != 0.f) v[2] = exact_product(bb, bb);
      vmax[0] = fabsf(rr);
    }
  }
  if (fin < 0) return;
  const int ops[3] = {0, 0, 0};
  double out[4];
  float fout[1];
  if (last_block_reduce_mf<NT, 3, 1>(D, kSiteRZ, v, ops, vmax, out, fout) && threadIdx.x == 0) {
    out[3] = (double)fout[0];
    if (phase == 0) finalize_op4(D, out);
    else finalize_op9(D, out);
  }
}
// The last Chebyshev sweep of a V-cycle (k_mg0_cheb with fin >= 0) over two z planes per block:
// each thread updates the cell of plane 2 bz and of plane 2 bz + 1, the same operations per cell,
// and adds the two cells' FP64 terms before the block reduction, so the launch has half the
// blocks, block trees and partials to combine.
template <class T>
__global__ void __launch_bounds__(NT) k_mg0_cheb_last(const __grid_constant__ Dev D, int phase, int source, float c1, float c2,
                                                       int first_k, int src_zero) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  double v[3] = {0, 0, 0};
  float vmax[1] = {0.f};
  for (int dz = 0; dz < 2; dz++) {
    Cell0 c;
    c.x = blockIdx.x * kTileX + (threadIdx.x & (kTileX - 1));
    c.y = blockIdx.y * kTileY + threadIdx.x / kTileX;
    c.z = 2 * blockIdx.z + dz;
    c.ok = c.x < D.nx && c.y < D.ny && c.z < D.nz;
    c.i = c.ok ? c.x + D.nx * (c.y + D.ny * c.z) : 0;
    if (!c.ok) continue;
    const T* __restrict__ x = field0<T>(D, source);
    const T* v7 = field0<T>(D, 7);
    const float b = ld_val(field0<T>(D, 0)[c.i]);
    const float sc = ld_val(field0<T>(D, 4)[c.i]);
    const float dprev = first_k ? 0.f : ld_val(v7[c.i]);
    const float r = src_zero ? b : b - apply0<T>(D, x, c);
    const float d = (first_k ? 0.f : c1 * dprev) + c2 * sc * r;
    const float xv = (src_zero ? 0.f : ld_val(x[c.i])) + d;
    const T xs = st_val<T>(xv);
    const float rr = D.r[c.i], z = ld_val(xs), bb = D.b[c.i];
    D.z[c.i] = z;
    if (phase == 0) D.d[c.i] = z;
    // FP64 terms only where they can be other than zero
    if (rr != 0.f || !isfinite(z)) {
      v[0] += exact_product(rr, z);
      v[1] += exact_product(rr, rr);
    }
    if (bb != 0.f) v[2] += exact_product(bb, bb);
    vmax[0] = mxf(vmax[0], fabsf(rr));
  }
  const int ops[3] = {0, 0, 0};
  double out[4];
  float fout[1];
  if (last_block_reduce_mf<NT, 3, 1>(D, kSiteRZ, v, ops, vmax, out, fout) && threadIdx.x == 0) {
    out[3] = (double)fout[0];
    if (phase == 0) finalize_op4(D, out);
    else finalize_op9(D, out);
  }
}
template <class T> __global__ void __launch_bounds__(NT) k_mg0_residual(const __grid_constant__ Dev D, int phase, int f) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  const Cell0 c = cell0(D);
  if (!c.ok) return;
  field0<T>(D, 6)[c.i] = st_val<T>(ld_val(field0<T>(D, 0)[c.i]) - apply0<T>(D, field0<T>(D, f), c));
}
// phase 0 load (op 5 of the cycle) fused with the first Chebyshev sweep from zero
template <class T> __global__ void __launch_bounds__(NT) k_mg0_load(const __grid_constant__ Dev D, int phase, int first_sweep) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i >= D.N) return;
  T* v = (T*)D.mgv;
  long long M = D.mg_nodes;
  T b = st_val<T>(D.r[i]);
  v[i] = b;
  v[M + i] = st_val<T>(0.f);
  v[2 * M + i] = st_val<T>(0.f);
  if (first_sweep) {  // k = 1 from x = 0: r = b, d = 0 + c2 s b, x2 = 0 + d
    float c2 = 4.f / 3.f;
    float d = 0.f + c2 * ld_val(v[4 * M + i]) * ld_val(b);
    v[7 * M + i] = st_val<T>(d);
    v[2 * M + i] = st_val<T>(0.f + d);
  }
}

// Restriction into level l (op 3, or op 5 with the level's first pre-smoothing sweep) with four
// lanes per coarse cell, used where the parent level's transfer is not an aggregation and coarsens
// z (a children box of several planes; with one plane the extra lanes cost more than they
// bring: 13.9 -> 38.8 us from level 0 on the beach): the (tz, ty) rows of
// the children box (at most 4 x 4 rows of 4) are shared out, p = tz * ext_y + ty to lane p % 4, each
// lane loading its rows' activity flags and residuals and forming their weighted terms; lane 0 then
// adds every term in the (tz, ty, tx) order of restrict_cell, taking each from its lane with a
// shuffle, and writes the cell as restrict_cell (and op 5's sweep) does.  The sums are the same
// float operations in the same order; the lanes only load in parallel.  An aggregated parent
// level (at most 2 x 2 x 2 children) is left to lane 0 with restrict_cell.
template <class T>
__global__ void __launch_bounds__(NT) k_mg_restrict4(const __grid_constant__ Dev D, int phase, int op, int l) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  const MG m(D);
  const int t = blockIdx.x * NT + threadIdx.x;
  const int i = t >> 2, g = t & 3, lane = threadIdx.x & 31;
  const MGLevelDev& cv = D.lv[l];
  const MGLevelDev& pv = D.lv[l - 1];
  const bool ok = i < cv.count;  // no lane leaves before the shuffles
  const int ic = ok ? i : 0;
  if (pv.aggregate) {  // the same for every thread of the launch
    if (ok && g == 0) {
      restrict_cell<T>(m, l, ic);
      if (op == 5 && m.active<T>(l, ic)) {
        if (D.mg_smoother == 1) cheb_update<T>(m, l, 1, 1, ic, true, 0.f);
        else jacobi_update<T>(m, l, 1, 1, ic, 0.f);
      }
    }
    return;
  }
  const T* r6 = m.field<T>(6, l - 1);
  const I3 qc = m.coord(l, ic);
  const bool act = ok && m.active<T>(l, ic);
  const int* ix = D.rt_idx + cv.roff[0] + 4 * qc.x;
  const int* iy = D.rt_idx + cv.roff[1] + 4 * qc.y;
  const int* iz = D.rt_idx + cv.roff[2] + 4 * qc.z;
  const float* wx = D.rt_w + cv.roff[0] + 4 * qc.x;
  const float* wy = D.rt_w + cv.roff[1] + 4 * qc.y;
  const float* wz = D.rt_w + cv.roff[2] + 4 * qc.z;
  const int ey = cv.rext[1], P = cv.rext[2] * ey;
  float term[4][4];
  unsigned use = 0u;  // bit 4 jp + tx
#pragma unroll
  for (int jp = 0; jp < 4; jp++) {
    const int p = g + 4 * jp, tz = p / ey, ty = p - tz * ey;
#pragma unroll
    for (int tx = 0; tx < 4; tx++) {
      const bool in = act && p < P && tx < cv.rext[0] && iy[ty] >= 0 && ix[tx] >= 0;
      const int j = in ? ix[tx] + pv.nx * (iy[ty] + pv.ny * iz[tz]) : 0;
      const bool a = in && m.active<T>(l - 1, j);
      const float r = ld_val(r6[j]);
      term[jp][tx] = in ? (1.f * wx[tx] * wy[ty] * wz[tz]) * r : 0.f;
      if (a) use |= 1u << (4 * jp + tx);
    }
  }
  const int base = lane & ~3;
  float sum = 0.f;
#pragma unroll
  for (int p = 0; p < 16; p++) {
    const unsigned u = __shfl_sync(0xffffffffu, use, base + (p & 3));
#pragma unroll
    for (int tx = 0; tx < 4; tx++) {
      const float v = __shfl_sync(0xffffffffu, term[p >> 2][tx], base + (p & 3));
      if (p < P && ((u >> (4 * (p >> 2) + tx)) & 1u)) sum += v;
    }
  }
  if (!ok || g != 0) return;
  m.field<T>(0, l)[ic] = st_val<T>(sum);
  m.field<T>(1, l)[ic] = st_val<T>(0.f);
  m.field<T>(2, l)[ic] = st_val<T>(0.f);
  if (op == 5 && act) {
    if (D.mg_smoother == 1) cheb_update<T>(m, l, 1, 1, ic, true, 0.f);
    else jacobi_update<T>(m, l, 1, 1, ic, 0.f);
  }
}

// Generic levels (l >= 1): one thread per cell.
constexpr int kWideStencil = 40;
// RESTRICT: the instance for the restriction ops 3 and 5 where k_mg_restrict4 does not take them
// (its unrolled child loads need more registers than the sweeps and the prolongation, which run
// in the other instance).
template <class T, int NTB = NT, bool RESTRICT = false>
__global__ void __launch_bounds__(NTB) k_mgl(const __grid_constant__ Dev D, int phase, int op, int l, int a, int b, int c) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  __shared__ int lin[kMaxStencil];
  const int* lin_s = nullptr;
  if (op <= 2 && l >= 1) {
    for (int k = threadIdx.x; k < D.lv[l].stencil; k += NTB) lin[k] = __ldg(D.stencil_lin + D.lv[l].soff + k);
    __syncthreads();
    lin_s = lin;
  }
  int i = blockIdx.x * NTB + threadIdx.x;
  if (l >= 1 && op != 3 && op != 5) {  // sweeps, residual, prolongation: active rows only
    if (i >= (int)D.mg_rowcount[l]) return;
    i = D.mg_rowlist[D.lv[l].off + i];
  } else if (i >= D.lv[l].count)
    return;
  MG m(D);
  // the one-thread-per-row FP32 sweeps (128-thread blocks) of a level with a stencil of at most
  // kWideStencil entries issue the row's loads together (apply_wide; the BF16 form would spill)
  auto ax = [&]() {
    if constexpr (NTB == 128 && std::is_same<T, float>::value)
      if (l >= 1 && D.lv[l].stencil <= kWideStencil) return m.apply_wide<T, kWideStencil>(l, a, i, lin_s);
    return m.apply<T>(l, a, i, lin_s);
  };
  if constexpr (!RESTRICT) {
    switch (op) {
      case 0: cheb_update<T>(m, l, a, b, i, c != 0, c != 0 ? 0.f : ax()); break;
      case 1: jacobi_update<T>(m, l, a, b, i, b ? 0.f : ax()); break;
      case 2: residual_update<T>(m, l, i, ax()); break;
      case 4: prolong_cell<T>(m, l, a, b, i); break;
    }
    return;
  }
  switch (op) {
    case 3: restrict_cell<T>(m, l, i); break;
    case 5:
      // restriction into level l fused with the level's first pre-smoothing sweep, which starts
      // from a zero iterate and so needs only the row's own b and scale (Chebyshev k = 1 into
      // field 2, or the Jacobi sweep s b); the skipped inactive rows keep the restriction's zeros
      restrict_cell<T>(m, l, i);
      if (m.active<T>(l, i)) {
        if (D.mg_smoother == 1) cheb_update<T>(m, l, 1, 1, i, true, 0.f);
        else jacobi_update<T>(m, l, 1, 1, i, 0.f);
      }
      break;
  }
}

// Chebyshev (op 0), Jacobi (op 1) and residual (op 2) sweeps of a large level >= 1 whose stencil has
// at most kWideStencil entries, with four lanes per active row: lane g loads the operator values and
// neighbour values of the row's entries k = g, g + 4, g + 8, ... and forms their products; lane 0
// then adds the products in stencil order k = 0..S-1, taking each from its lane with a shuffle, and
// updates the row as k_mgl does.  Every product and every addition is the float operation that
// MG::apply performs (the product rounded, then added, in the same order), so the bits are the
// same; the lanes only load in parallel.  A level-1 sweep of the beach visits about 70,000 active
// rows, which with one thread per row leaves about 14 warps per SM waiting on dependent loads.
constexpr int kLaneEntries = kWideStencil / 4;
template <class T>
__global__ void __launch_bounds__(NT) k_mgl4(const __grid_constant__ Dev D, int phase, int op, int l, int a, int b, int c) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  const MGLevelDev& lv = D.lv[l];
  const int nrows = (int)D.mg_rowcount[l];
  if ((int)((blockIdx.x * NT) >> 2) >= nrows) return;  // uniform over the block
  __shared__ int lin[kWideStencil];
  const int S = min(lv.stencil, kWideStencil);  // Cycle::level_op launches this only for S <= kWideStencil
  for (int k = threadIdx.x; k < S; k += NT) lin[k] = __ldg(D.stencil_lin + lv.soff + k);
  __syncthreads();
  const int t = blockIdx.x * NT + threadIdx.x;
  if (((t & ~31) >> 2) >= nrows) return;  // the warp's first row: uniform over the warp
  const int r = t >> 2, g = t & 3, lane = threadIdx.x & 31;
  const bool ok = r < nrows;  // no lane of the warp leaves before the shuffles
  const int i = D.mg_rowlist[lv.off + (ok ? r : nrows - 1)];
  const MG m(D);
  const bool need = !(op == 0 && c != 0) && !(op == 1 && b != 0);  // uniform over the launch
  float ax = 0.f;
  if (need) {
    const T* x = m.field<T>(a, l);
    const T* ell = (const T*)D.mgell + lv.eoff;
    const int* col = D.mgcol + lv.eoff;
    const I3 q = m.coord(l, i);
    const bool inner = q.x >= 2 && q.x < lv.nx - 2 && q.y >= 2 && q.y < lv.ny - 2 && q.z >= 2 && q.z < lv.nz - 2;
    float e[kLaneEntries], v[kLaneEntries];
#pragma unroll
    for (int j = 0; j < kLaneEntries; j++) {
      const int k = 4 * j + g;
      e[j] = 0.f;
      v[j] = 0.f;
      if (k < S) {
        const long long at = (long long)k * lv.count + i;
        const int n = inner ? i + lin[k] : __ldg(col + at);
        e[j] = ld_val(ell[at]);
        v[j] = ld_val(x[n]);
      }
    }
    const bool act = m.active<T>(l, i);
    const float here = ld_val(x[i]);
    const int base = lane & ~3;
    float sum = 0.f;
#pragma unroll
    for (int j = 0; j < kLaneEntries; j++) {
      const float p = e[j] * v[j];
#pragma unroll
      for (int h = 0; h < 4; h++) {
        const float term = __shfl_sync(0xffffffffu, p, base + h);
        if (4 * j + h < S) sum += term;
      }
    }
    ax = act ? sum : here;
  }
  if (!ok || g != 0) return;
  switch (op) {
    case 0: cheb_update<T>(m, l, a, b, i, c != 0, c != 0 ? 0.f : ax); break;
    case 1: jacobi_update<T>(m, l, a, b, i, b ? 0.f : ax); break;
    case 2: residual_update<T>(m, l, i, ax); break;
  }
}

// Chebyshev (op 0), Jacobi (op 1) and residual (op 2) sweeps of a level >= 1 with the
// product-parallel apply: RR rows per block.
template <class T, int RRB = RR>
__global__ void __launch_bounds__(NT) k_mgl_rows(const __grid_constant__ Dev D, int phase, int op, int l, int a, int b, int c) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  __shared__ float prod[kMaxStencil * RRB];
  __shared__ bool inner[RRB];
  __shared__ int lin[kMaxStencil];
  __shared__ int rowi[RRB];
  const int row0 = blockIdx.x * RRB, nrows = (int)D.mg_rowcount[l];
  if (row0 >= nrows) return;  // uniform over the block
  MG m(D);
  if (threadIdx.x < RRB) rowi[threadIdx.x] = row0 + threadIdx.x < nrows ? D.mg_rowlist[D.lv[l].off + row0 + threadIdx.x] : -1;
  __syncthreads();
  const bool need = !(op == 0 && c != 0) && !(op == 1 && b != 0);
  if (need) row_products<T, NT, RRB>(m, l, a, rowi, prod, inner, lin);
  if (threadIdx.x >= RRB) return;
  const int i = rowi[threadIdx.x];
  if (i < 0) return;
  const float ax = need ? row_sum<T, RRB>(m, l, a, i, prod) : 0.f;
  switch (op) {
    case 0: cheb_update<T>(m, l, a, b, i, c != 0, ax); break;
    case 1: jacobi_update<T>(m, l, a, b, i, ax); break;
    case 2: residual_update<T>(m, l, i, ax); break;
  }
}

// Shared-memory view of the bottom levels lb..L-1: their eight vector fields (one span per field,
// levels in global order), their ELL row values and the cached columns max(wrap(q + offset), 0)
// (as 16-bit indices: a bottom level holds at most 1024 rows) are staged in shared memory, so
// apply() reads the same values in the same order as the global-memory form.
struct MGs : MG {
  void* vec;
  const void* ell;
  const unsigned short* cols;  // the cached columns max(wrap(q + offset), 0) of the staged rows
  const float* linv;           // the staged factor of the dense coarse solve
  int base_off, span;
  long long base_eoff;
  DI MGs(const Dev& d, void* v, const void* e, const unsigned short* c, const float* li, int lb, int sp)
      : MG(d), vec(v), ell(e), cols(c), linv(li), base_off(d.lv[lb].off), span(sp), base_eoff(d.lv[lb].eoff) {}
  DI const float* coarse_inverse() const { return linv; }
  template <class T> DI T* field(int f, int l) const { return (T*)vec + f * span + (D.lv[l].off - base_off); }
  template <class T> DI bool active(int l, int i) const { return i >= 0 && ld_val(field<T>(3, l)[i]) > .5f; }
  template <class T> DI float apply(int l, int f, int i, const int* = nullptr) const {
    const T* x = field<T>(f, l);
    if (!active<T>(l, i)) return ld_val(x[i]);
    const MGLevelDev& lv = D.lv[l];
    const long long at = lv.eoff - base_eoff;
    const T* e = (const T*)ell + at;
    const unsigned short* c = cols + at;
    float sum = 0.f;
    // unrolled so that the shared-memory loads run ahead of the additions (which stay in order)
#pragma unroll 9
    for (int k = 0; k < lv.stencil; k++) sum += ld_val(e[k * lv.count + i]) * ld_val(x[c[k * lv.count + i]]);
    return sum;
  }
};

// Whole sub-cycle from level lb down to the coarsest and back, in one block, over the view `m`
// (global memory, or the shared-memory stage).  The level-lb correction ends in field 1.
template <class T, class M> DI void bottom_cycle(const Dev& D, const M& m, int lb, float* small) {
  const int L = D.L;
  int field[kMaxLevels];
  auto each = [&](int l, auto fn) {
    for (int i = threadIdx.x; i < D.lv[l].count; i += blockDim.x) fn(i);
    __syncthreads();
  };
  auto smooth = [&](int l, int f, bool zero) {
    for (int sweep = 0; sweep < D.mg_smoothing; sweep++) {
      if (D.mg_smoother == 1) each(l, [&](int i) { cheb_cell<T>(m, l, f, sweep + 1, i, zero && sweep == 0); });
      else each(l, [&](int i) { jacobi_cell<T>(m, l, f, zero && sweep == 0 ? 1 : 0, i); });
      f = 3 - f;
    }
    return f;
  };
  for (int l = lb; l < L - 1; l++) {
    int f = smooth(l, 1, true);
    field[l] = f;
    each(l, [&](int i) { residual_cell<T>(m, l, f, i); });
    each(l + 1, [&](int i) { restrict_cell<T>(m, l + 1, i); });
  }
  int cf;
  const int lc = L - 1;
  if (D.lv[lc].count <= 64) {
    coarse_block<T>(m, lc, small);
    cf = 1;
  } else {
    cf = 1;
    for (int sweep = 0; sweep < 32; sweep++) {
      int f = cf;
      each(lc, [&](int i) { jacobi_cell<T>(m, lc, f, sweep == 0 ? 1 : 0, i); });
      cf = 3 - cf;
    }
  }
  for (int l = L - 2; l >= lb; l--) {
    int f = field[l];
    int ccf = cf;
    each(l, [&](int i) { prolong_cell<T>(m, l, f, ccf, i); });
    cf = smooth(l, f, false);
  }
}
template <class T> __global__ void __launch_bounds__(1024) k_mg_bottom(const __grid_constant__ Dev D, int phase, int lb) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  __shared__ float small[64];
  bottom_cycle<T>(D, MG(D), lb, small);
}
// The same with levels lb..L-1 staged in shared memory (D.mg_bottom_smem bytes: 8 fields of
// `span` values, the ELL values and their columns as 16-bit indices, each part 16-byte aligned):
// load, cycle, write the fields back.
// Levels lb..L-1 staged in `stage` by one block, the sub-cycle run there, the fields written back.
// dst[k] = src[at(k)] for k < n over the block, kStageU loads of a thread issued before its stores.
constexpr int kStageU = 8;
template <class D_, class S_, class F> DI void staged_copy(D_* dst, const S_* __restrict__ src, long long n, F at) {
  for (long long k0 = threadIdx.x; k0 < n; k0 += (long long)kStageU * blockDim.x) {
    S_ v[kStageU];
#pragma unroll
    for (int u = 0; u < kStageU; u++) {
      const long long k = k0 + (long long)u * blockDim.x;
      if (k < n) v[u] = src[at((int)k)];
    }
#pragma unroll
    for (int u = 0; u < kStageU; u++) {
      const long long k = k0 + (long long)u * blockDim.x;
      if (k < n) dst[k] = (D_)v[u];
    }
  }
}
template <class T> DI void bottom_staged(const Dev& D, int lb, unsigned char* stage, float* small) {
  const int L = D.L;
  const int span = D.lv[L - 1].off + D.lv[L - 1].count - D.lv[lb].off;
  const long long e0 = D.lv[lb].eoff, e1 = D.lv[L - 1].eoff + (long long)D.lv[L - 1].stencil * D.lv[L - 1].count;
  T* vec = (T*)stage;
  T* ell = (T*)(stage + (((size_t)8 * span * sizeof(T) + 15) & ~(size_t)15));
  unsigned short* cols = (unsigned short*)((unsigned char*)ell + (((size_t)(e1 - e0) * sizeof(T) + 15) & ~(size_t)15));
  // the dense coarse solve's factor (at most 64 x 64) after the columns
  const int nc = D.lv[L - 1].count;
  float* linv = (float*)((unsigned char*)cols + (((size_t)(e1 - e0) * 2 + 15) & ~(size_t)15));
  // every load of a thread's share is issued before its stores (kStageU in flight per array): a
  // single block would otherwise wait out one memory latency per element it stages
  if (nc <= 64) staged_copy(linv, D.mglinv, (long long)nc * nc, [](int k) { return k; });
  const T* gvec = (const T*)D.mgv + D.lv[lb].off;
  const size_t nodes = (size_t)D.mg_nodes;
  staged_copy(vec, gvec, 8LL * span, [span, nodes](int k) { return (size_t)(k / span) * nodes + (size_t)(k % span); });
  const T* gell = (const T*)D.mgell + e0;
  const int* gcol = D.mgcol + e0;
  staged_copy(ell, gell, e1 - e0, [](int k) { return k; });
  staged_copy(cols, gcol, e1 - e0, [](int k) { return k; });
  __syncthreads();
  bottom_cycle<T>(D, MGs(D, vec, ell, cols, nc <= 64 ? linv : D.mglinv, lb, span), lb, small);
  T* out = (T*)D.mgv + D.lv[lb].off;
  for (int f = 0; f < 8; f++)
    for (int k = threadIdx.x; k < span; k += blockDim.x) out[(size_t)f * D.mg_nodes + k] = vec[f * span + k];
}
template <class T> __global__ void __launch_bounds__(1024) k_mg_bottom_smem(const __grid_constant__ Dev D, int phase, int lb) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  extern __shared__ __align__(16) unsigned char stage[];
  __shared__ float small[64];
  bottom_staged<T>(D, lb, stage, small);
}

// ---------------------------------------------------------------- coarse levels in one launch
// Levels mg_coarse_from..L-1 of a V-cycle run in one cooperative launch (one block per SM, all
// blocks resident): every phase of Cycle::level for those levels -- Chebyshev or Jacobi sweeps and
// residuals over the active rows (product-parallel chunks of CRR rows), restrictions, the bottom
// sub-cycle in block 0 and prolongations -- in the same order, with the same per-row functions,
// separated by grid barriers.  The level-from correction ends in field 1, as in Cycle.
constexpr int CNT = 512;  // threads per block of the coarse kernel
constexpr int CRR = 64;   // rows per product-parallel chunk

// Grid barrier: arrive on a counter; the last block resets it and advances the generation the
// others wait on.  The wait is bounded (about a second of __nanosleep): on a timeout the block
// records failure 98 in c[7] and carries on, so no launch can hang.
DI void grid_barrier(const Dev& D) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = D.gbar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(D.gbar, 1u) == gridDim.x - 1) {
      D.gbar[0] = 0u;
      __threadfence();
      atomicAdd(D.gbar + 1, 1u);
    } else {
      unsigned spins = 0;
      while (*gen == g) {
        __nanosleep(128);
        if (++spins > (1u << 23)) {
          D.c[7] = 98;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(CNT) k_mg_coarse(const __grid_constant__ Dev D, int phase, int lt) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;  // the same decision in every block
  extern __shared__ __align__(16) unsigned char dyn[];
  __shared__ bool inner[CRR];
  __shared__ int lin[kMaxStencil];
  __shared__ int rowi[CRR];
  __shared__ float small[64];
  float* prod = (float*)dyn;
  const MG m(D);
  const int lb = D.mg_bottom;
  int field[kMaxLevels];
  auto rows_op = [&](int l, int op, int a, int b, int c) {
    const int nrows = (int)D.mg_rowcount[l];
    const bool need = !(op == 0 && c != 0) && !(op == 1 && b != 0);
    for (int row0 = blockIdx.x * CRR; row0 < nrows; row0 += gridDim.x * CRR) {
      if (threadIdx.x < CRR) rowi[threadIdx.x] = row0 + threadIdx.x < nrows ? D.mg_rowlist[D.lv[l].off + row0 + threadIdx.x] : -1;
      __syncthreads();
      if (need) row_products<T, CNT, CRR>(m, l, a, rowi, prod, inner, lin);
      if (threadIdx.x < CRR && rowi[threadIdx.x] >= 0) {
        const int i = rowi[threadIdx.x];
        const float ax = need ? row_sum<T, CRR>(m, l, a, i, prod) : 0.f;
        if (op == 0) cheb_update<T>(m, l, a, b, i, c != 0, ax);
        else if (op == 1) jacobi_update<T>(m, l, a, b, i, ax);
        else residual_update<T>(m, l, i, ax);
      }
      __syncthreads();
    }
    grid_barrier(D);
  };
  auto smooth = [&](int l, int f, bool zero) {
    for (int sweep = 0; sweep < D.mg_smoothing; sweep++) {
      const bool first = zero && sweep == 0;
      if (D.mg_smoother == 1) rows_op(l, 0, f, sweep + 1, first ? 1 : 0);
      else rows_op(l, 1, f, first ? 1 : 0, 0);
      f = 3 - f;
    }
    return f;
  };
  for (int l = lt; l < lb; l++) {
    const int f = smooth(l, 1, true);
    field[l] = f;
    rows_op(l, 2, f, 0, 0);
    for (int i = blockIdx.x * CNT + threadIdx.x; i < D.lv[l + 1].count; i += gridDim.x * CNT) restrict_cell<T>(m, l + 1, i);
    grid_barrier(D);
  }
  if (blockIdx.x == 0) {
    if (D.mg_bottom_smem > 0) bottom_staged<T>(D, lb, dyn, small);
    else bottom_cycle<T>(D, m, lb, small);
  }
  grid_barrier(D);
  int cf = 1;
  for (int l = lb - 1; l >= lt; l--) {
    const int f = field[l];
    const int nrows = (int)D.mg_rowcount[l];
    for (int t = blockIdx.x * CNT + threadIdx.x; t < nrows; t += gridDim.x * CNT)
      prolong_cell<T>(m, l, f, cf, D.mg_rowlist[D.lv[l].off + t]);
    grid_barrier(D);
    cf = smooth(l, f, false);
  }
}

// ---------------------------------------------------------------- coarse leg in one cluster
// Levels lt..mg_bottom-1 of a V-cycle and the bottom sub-cycle in one launch of one thread-block
// cluster (kLegCtas blocks of kLegThreads, on neighbouring SMs): the phases of Cycle::level for
// those levels in the same order, with the same per-row functions as the per-level kernels
// (product-parallel rows, products summed in stencil order, so the bits are those of
// k_mgl_rows), separated by the cluster's hardware barrier instead of kernel boundaries.  The
// rows of a level are split into kLegCtas contiguous ranges; block 0 runs the bottom sub-cycle
// in its shared memory while the others wait at the barrier.  The barrier's release/acquire
// semantics at cluster scope order every block's global-memory writes of one phase before the
// reads of the next.  No wait is a spin: a cluster barrier completes once every thread of the
// cluster has arrived, and every thread runs the same sequence of phases.
constexpr int kLegCtas = 8;
constexpr int kLegThreads = 1024;
constexpr int kLegRowsMax = 1024;  // rows of one block's chunk (row indices and interior flags)

DI void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <class T>
__global__ void __launch_bounds__(kLegThreads, 1) k_mg_leg(const __grid_constant__ Dev D, int phase, int lt) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;  // the same decision in every block
  extern __shared__ __align__(16) unsigned char dyn[];
  __shared__ int lin[kMaxStencil];
  __shared__ float small[64];
  // dynamic shared memory: the products of a chunk, then its row indices and interior flags (the
  // bottom stage of block 0 reuses all of it)
  const int prod_cap = (D.mg_leg_smem - kLegRowsMax * (int)(sizeof(int) + sizeof(bool))) / (int)sizeof(float);
  float* prod = (float*)dyn;
  int* rowi = (int*)(dyn + (size_t)prod_cap * sizeof(float));
  bool* inner = (bool*)(rowi + kLegRowsMax);
  const MG m(D);
  const int lb = D.mg_bottom;
  const int nb = gridDim.x, b = blockIdx.x, t = threadIdx.x;
  int field[kMaxLevels];
  // sweep op (0 Chebyshev, 1 Jacobi, 2 residual) over this block's range of the active rows
  auto rows_op = [&](int l, int op, int a, int bb, int c) {
    const MGLevelDev& lv = D.lv[l];
    const int nrows = (int)D.mg_rowcount[l], S = lv.stencil, n = lv.count;
    const bool need = !(op == 0 && c != 0) && !(op == 1 && bb != 0);
    const int per = (nrows + nb - 1) / nb, r0 = b * per, r1 = min(nrows, r0 + per);
    const int rc = max(1, min(kLegRowsMax, prod_cap / S));
    for (int k = t; k < S; k += kLegThreads) lin[k] = __ldg(D.stencil_lin + lv.soff + k);
    const T* x = m.field<T>(a, l);
    const T* ell = (const T*)D.mgell + lv.eoff;
    const int* col = D.mgcol + lv.eoff;
    for (int c0 = r0; c0 < r1; c0 += rc) {
      const int cnt = min(rc, r1 - c0);
      for (int r = t; r < cnt; r += kLegThreads) {
        const int i = D.mg_rowlist[lv.off + c0 + r];
        rowi[r] = i;
        const I3 q = m.coord(l, i);
        inner[r] = q.x >= 2 && q.x < lv.nx - 2 && q.y >= 2 && q.y < lv.ny - 2 && q.z >= 2 && q.z < lv.nz - 2;
      }
      __syncthreads();
      if (need) {
#pragma unroll 4
        for (int p = t; p < S * cnt; p += kLegThreads) {
          const int k = p / cnt, r = p - k * cnt, i = rowi[r];
          const long long e = (long long)k * n + i;
          const int j = inner[r] ? i + lin[k] : __ldg(col + e);
          prod[p] = ld_val(ell[e]) * ld_val(x[j]);
        }
        __syncthreads();
      }
      for (int r = t; r < cnt; r += kLegThreads) {
        const int i = rowi[r];
        float ax = 0.f;
        if (need) {
          if (!m.active<T>(l, i)) ax = ld_val(x[i]);
          else {
            float sum = 0.f;
#pragma unroll 8
            for (int k = 0; k < S; k++) sum += prod[k * cnt + r];
            ax = sum;
          }
        }
        if (op == 0) cheb_update<T>(m, l, a, bb, i, c != 0, ax);
        else if (op == 1) jacobi_update<T>(m, l, a, bb, i, ax);
        else residual_update<T>(m, l, i, ax);
      }
      __syncthreads();
    }
    cluster_barrier();
  };
  auto smooth = [&](int l, int f, bool zero) {
    for (int sweep = 0; sweep < D.mg_smoothing; sweep++) {
      const bool first = zero && sweep == 0;
      if (D.mg_smoother == 1) rows_op(l, 0, f, sweep + 1, first ? 1 : 0);
      else rows_op(l, 1, f, first ? 1 : 0, 0);
      f = 3 - f;
    }
    return f;
  };
  for (int l = lt; l < lb; l++) {
    const int f = smooth(l, 1, true);
    field[l] = f;
    rows_op(l, 2, f, 0, 0);
    for (int i = b * kLegThreads + t; i < D.lv[l + 1].count; i += nb * kLegThreads) restrict_cell<T>(m, l + 1, i);
    cluster_barrier();
  }
  if (b == 0) {
    if (D.mg_bottom_smem > 0) bottom_staged<T>(D, lb, dyn, small);
    else bottom_cycle<T>(D, m, lb, small);
  }
  cluster_barrier();
  int cf = 1;
  for (int l = lb - 1; l >= lt; l--) {
    const int f = field[l];
    const int nrows = (int)D.mg_rowcount[l];
    for (int r = b * kLegThreads + t; r < nrows; r += nb * kLegThreads) prolong_cell<T>(m, l, f, cf, D.mg_rowlist[D.lv[l].off + r]);
    cluster_barrier();
    cf = smooth(l, f, false);
  }
}

// op 10 of the cycle + op 4 / op 9 finalisation (Jacobi smoothing path)
template <class T> __global__ void __launch_bounds__(NT) k_mg_finish(const __grid_constant__ Dev D, int phase, int f) {
  grid_dep_wait(D.pdl_early);
  if (!phase_on(D, phase)) return;
  MG m(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  double v[3] = {0, 0, 0};
  float vmax[1] = {0.f};
  if (i < D.N) {
    float r = D.r[i], z = ld_val(m.field<T>(f, 0)[i]), b = D.b[i];
    D.z[i] = z;
    if (phase == 0) D.d[i] = z;
    if (r != 0.f || !isfinite(z)) {
      v[0] = exact_product(r, z);
      v[1] = exact_product(r, r);
    }
    if (b != 0.f) v[2] = exact_product(b, b);
    vmax[0] = fabsf(r);
  }
  const int ops[3] = {0, 0, 0};
  double out[4];
  float fout[1];
  if (last_block_reduce_mf<NT, 3, 1>(D, kSiteRZ, v, ops, vmax, out, fout) && threadIdx.x == 0) {
    out[3] = (double)fout[0];
    if (phase == 0) finalize_op4(D, out);
    else finalize_op9(D, out);
  }
}

unsigned grid_for(long long n) { return (unsigned)((n + NT - 1) / NT); }

// Algorithmic bytes of one level >= 1 sweep (op 0 Chebyshev, 1 Jacobi, 2 residual): with the
// operator, the row values and columns of rows that wrap, the source iterate and the activity
// field; then the op's own vectors.  tb = storage bytes of a multigrid value.
// Chebyshev coefficients of sweep k (pressure_multigrid.glslinc:206-207), correctly rounded
// float quotients exactly as the device computes them in cheb_update.
float cheb_c1(int k) { return (float)(2 * k - 3) / (float)(2 * k + 1); }
float cheb_c2(int k) { return (float)(8 * k - 4) / (float)(2 * k + 1); }

double level_op_bytes(const Dev& D, int l, int op, int b, int c, double tb) {
  const MGLevelDev& v = D.lv[l];
  const double n = v.count;
  const bool need = !(op == 0 && c != 0) && !(op == 1 && b != 0);
  const double inner = (double)std::max(0, v.nx - 4) * std::max(0, v.ny - 4) * std::max(0, v.nz - 4);
  double bytes = need ? n * v.stencil * tb + 2.0 * n * tb + (n - inner) * v.stencil * 4.0 : 0.0;
  if (op == 0) bytes += n * tb * ((b > 1 ? 1.0 : 0.0) + 2.0 + 2.0);  // d_prev, b, scale; d, x
  else if (op == 1) bytes += 3.0 * n * tb;                            // scale, b; x
  else bytes += 2.0 * n * tb;                                         // b; residual
  return bytes;
}
// Level-0 Chebyshev sweep: activity byte, six coefficients, b and scale, the iterate unless it is
// zero, d_prev after the first sweep; writes d and x, or (last sweep) reads r, b and writes z (and d).
double smooth0_bytes(const Dev& D, int phase, int k, int src_zero, int fin, double tb) {
  const double n = (double)D.N;
  double bytes = n * (1.0 + tb * (8.0 + (src_zero ? 0.0 : 1.0) + (k > 1 ? 1.0 : 0.0)));
  bytes += fin < 0 ? 2.0 * n * tb : n * (8.0 + 4.0 + (phase == 0 ? 4.0 : 0.0));
  return bytes;
}

// A cooperative launch of the coarse kernel; the grid must fit the device at once (one block
// per SM), which the launch itself checks.
template <class... KArgs, class... Args>
void coop_launch(void (*kernel)(KArgs...), unsigned blocks, unsigned threads, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  probed(kProbeAll, s, 0.0, [&] { cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...); });
}
// A launch of one thread-block cluster of `ctas` blocks (with programmatic serialization when
// enabled), probed as `kind` with `bytes` tagged with `level`.
template <class... KArgs, class... Args>
void cluster_launch(void (*kernel)(KArgs...), unsigned ctas, unsigned threads, size_t smem, cudaStream_t s, int kind,
                    double bytes, int level, Args&&... args) {
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = g_pdl ? 2 : 1;
  probed(kind, s, bytes, [&] {
    probed(kProbeAll, s, 0.0, [&] { cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...); });
  }, level);
}
__global__ void k_cluster_probe(int* x) {
  cluster_barrier();
  if (threadIdx.x == 0 && blockIdx.x == 0) *x = 1;
}
__global__ void k_coop_probe(int* x) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *x = 1;
}

template <class T> struct Cycle {
  const Dev& D;
  cudaStream_t s;
  int phase;
  int fused_first;  // the level-0 first pre-smoothing sweep was done by the caller
  unsigned rows_grid(int l, int rr) const { return (unsigned)((D.lv[l].count + rr - 1) / rr); }
  // Levels with few rows use the product-parallel kernel (enough independent loads in flight);
  // larger levels keep one thread per row.
  bool few_rows(int l) const { return D.lv[l].count < D.mg_rows_below; }
  void level_op(int l, int op, int a, int b, int c) {
    const double bytes = level_op_bytes(D, l, op, b, c, sizeof(T));
    if (few_rows(l))
      probed(kProbeRows, s, bytes, [&] {
        if (D.mg_rows_rr == 8) pdl_launch((k_mgl_rows<T, 8>), rows_grid(l, 8), NT, 0, s, D, phase, op, l, a, b, c);
        else if (D.mg_rows_rr == 16) pdl_launch((k_mgl_rows<T, 16>), rows_grid(l, 16), NT, 0, s, D, phase, op, l, a, b, c);
        else if (D.mg_rows_rr == 64) pdl_launch((k_mgl_rows<T, 64>), rows_grid(l, 64), NT, 0, s, D, phase, op, l, a, b, c);
        else pdl_launch((k_mgl_rows<T, RR>), rows_grid(l, RR), NT, 0, s, D, phase, op, l, a, b, c);
      }, l);
    else
      probed(kProbeRowThread, s, bytes, [&] {
        if (D.mg_lanes == 4 && D.lv[l].stencil <= kWideStencil && op <= 2)
          pdl_launch((k_mgl4<T>), (unsigned)((4LL * D.lv[l].count + NT - 1) / NT), NT, 0, s, D, phase, op, l, a, b, c);
        else if (D.mg_thread_nt == 128)
          pdl_launch((k_mgl<T, 128>), (unsigned)((D.lv[l].count + 127) / 128), 128, 0, s, D, phase, op, l, a, b, c);
        else
          pdl_launch((k_mgl<T, NT>), grid_for(D.lv[l].count), NT, 0, s, D, phase, op, l, a, b, c);
      }, l);
  }
  dim3 grid0() const { return dim3((unsigned)((D.nx + kTileX - 1) / kTileX), (unsigned)((D.ny + kTileY - 1) / kTileY), (unsigned)D.nz); }
  int smooth(int l, int field, bool zero, bool last0) {
    unsigned gr = grid_for(D.lv[l].count);
    for (int sweep = 0; sweep < D.mg_smoothing; sweep++) {
      bool first = zero && sweep == 0;
      bool fin = last0 && sweep == D.mg_smoothing - 1;
      if (first && (l == 0 ? fused_first != 0 : restrict_fused(l))) {
        field = 3 - field;
        continue;
      }
      if (D.mg_smoother == 1) {
        if (l == 0)
          probed(kProbeSmooth0, s, smooth0_bytes(D, phase, sweep + 1, first ? 1 : 0, fin ? 1 : -1, sizeof(T)), [&] {
            if (fin)
              pdl_launch((k_mg0_cheb_last<T>), dim3(grid0().x, grid0().y, (unsigned)((D.nz + 1) / 2)), NT, 0, s, D, phase, field,
                         cheb_c1(sweep + 1), cheb_c2(sweep + 1), sweep == 0 ? 1 : 0, first ? 1 : 0);
            else
              pdl_launch((k_mg0_cheb<T>), grid0(), NT, 0, s, D, phase, field, cheb_c1(sweep + 1), cheb_c2(sweep + 1),
                         sweep == 0 ? 1 : 0, first ? 1 : 0, -1);
          });
        else level_op(l, 0, field, sweep + 1, first ? 1 : 0);
      } else if (l == 0)
        pdl_launch((k_mgl<T>), gr, NT, 0, s, D, phase, 1, l, field, first ? 1 : 0, 0);
      else
        level_op(l, 1, field, first ? 1 : 0, 0);
      field = 3 - field;
    }
    return field;
  }
  // A level >= 1 reached through the regular per-level path has its first pre-smoothing sweep
  // done by the launch that restricts into it (k_mgl op 5).
  bool restrict_fused(int l) const {
    return l >= 1 && l != D.L - 1 && l != D.mg_bottom && !(D.mg_coarse_from > 0 && l == D.mg_coarse_from && l < D.mg_bottom) &&
           !(D.mg_leg_from > 0 && l == D.mg_leg_from && l < D.mg_bottom);
  }
  // pre- and post-smoothing flip the field mg_smoothing times each: a level ends in field 1
  int bottom_field() const { return 1; }
  int level(int l) {
    unsigned gr = grid_for(D.lv[l].count);
    if (D.mg_coarse_from > 0 && l == D.mg_coarse_from && l < D.mg_bottom) {
      const size_t smem = std::max((size_t)kMaxStencil * CRR * sizeof(float), (size_t)D.mg_bottom_smem);
      coop_launch((k_mg_coarse<T>), D.coarse_blocks, CNT, smem, s, D, phase, l);
      int f = 1;  // the field logic of the kernel: pre- then post-smoothing from field 1
      for (int k = 0; k < 2 * D.mg_smoothing; k++) f = 3 - f;
      return f;
    }
    if (D.mg_leg_from > 0 && l == D.mg_leg_from && l < D.mg_bottom) {
      // algorithmic bytes: the leg's level sweeps and residuals (the bottom's are not counted)
      double bytes = 0.0;
      for (int k = l; k < D.mg_bottom; k++) {
        for (int sweep = 0; sweep < D.mg_smoothing; sweep++) {
          const int op = D.mg_smoother == 1 ? 0 : 1;
          bytes += level_op_bytes(D, k, op, op == 0 ? sweep + 1 : (sweep == 0 ? 1 : 0), op == 0 && sweep == 0 ? 1 : 0, sizeof(T));
          bytes += level_op_bytes(D, k, op, op == 0 ? sweep + 1 : 0, 0, sizeof(T));
        }
        bytes += level_op_bytes(D, k, 2, 0, 0, sizeof(T));
      }
      cluster_launch((k_mg_leg<T>), kLegCtas, kLegThreads, (size_t)D.mg_leg_smem, s, kProbeLeg, bytes, l, D, phase, l);
      int f = 1;  // the field logic of the kernel: pre- then post-smoothing from field 1
      for (int k = 0; k < 2 * D.mg_smoothing; k++) f = 3 - f;
      return f;
    }
    if (l == D.L - 1 || l == D.mg_bottom) {
      if (D.mg_bottom_smem > 0 && l == D.mg_bottom)
        pdl_launch((k_mg_bottom_smem<T>), 1, 1024, D.mg_bottom_smem, s, D, phase, l);
      else
        pdl_launch((k_mg_bottom<T>), 1, 1024, 0, s, D, phase, l);
      // the bottom kernels leave the level's correction in field 1: the dense solve of the
      // coarsest level, its 32 Jacobi sweeps where it has more than 64 rows, and the sub-cycle
      // from mg_bottom down and back alike
      return bottom_field();
    }
    int field = smooth(l, 1, true, false);
    if (l == 0) pdl_launch((k_mg0_residual<T>), grid0(), NT, 0, s, D, phase, field);
    else level_op(l, 2, field, 0, 0);
    {
      // four lanes per coarse cell where the children box has several planes (a transfer that
      // coarsens z: up to 16 rows of children); one thread per coarse cell otherwise
      const int rop = restrict_fused(l + 1) ? 5 : 3;
      if (!D.lv[l].aggregate && D.lv[l + 1].rext[2] > 1)
        pdl_launch((k_mg_restrict4<T>), grid_for(4LL * D.lv[l + 1].count), NT, 0, s, D, phase, rop, l + 1);
      else
        pdl_launch((k_mgl<T, NT, true>), grid_for(D.lv[l + 1].count), NT, 0, s, D, phase, rop, l + 1, 0, 0, 0);
    }
    int cf = level(l + 1);
    pdl_launch((k_mgl<T>), gr, NT, 0, s, D, phase, 4, l, field, cf, 0);
    return smooth(l, field, false, l == 0 && D.mg_smoother == 1);
  }
  void run() {
    if (phase == 0) pdl_launch((k_mg0_load<T>), grid_for(D.N), NT, 0, s, D, phase, D.mg_smoother == 1 ? 1 : 0);
    fused_first = D.mg_smoother == 1;
    int f = level(0);
    // Chebyshev smoothing fuses z and the finalisation into the last level-0 sweep
    if (D.mg_smoother != 1) pdl_launch((k_mg_finish<T>), grid_for(D.N), NT, 0, s, D, phase, f);
  }
};

// Columns of the ELL rows, max(wrap(l, q + offset), 0), computed once (static geometry).
__global__ void __launch_bounds__(NT) k_mg_cols(const __grid_constant__ Dev D, int l) {
  grid_dep_wait(D.pdl_early);
  MG m(D);
  const MGLevelDev& lv = D.lv[l];
  int i = blockIdx.x * NT + threadIdx.x;
  if (i >= lv.count) return;
  I3 q = m.coord(l, i);
  for (int k = 0; k < lv.stencil; k++) {
    int j = m.wrap(l, addI(q, m.offset(l, k)));
    D.mgcol[lv.eoff + (long long)k * lv.count + i] = j > 0 ? j : 0;
  }
}

// Level-0 neighbour-active bits (bit f: neighbour across face f active, bit 6: cell active),
// rebuilt after the masks on structural rebuilds.
template <class T> __global__ void __launch_bounds__(NT) k_mg_nb0(const __grid_constant__ Dev D) {
  grid_dep_wait(D.pdl_early);
  if (!build_on(D) || D.hstate[9] == 0) return;
  MG m(D);
  long long i = (long long)blockIdx.x * NT + threadIdx.x;
  if (i >= D.N) return;
  I3 q = m.coord(0, (int)i);
  unsigned bits = m.active<T>(0, (int)i) ? 64u : 0u;
  for (int axis = 0; axis < 3; axis++)
    for (int side = 0; side < 2; side++)
      if (m.active<T>(0, m.wrap(0, ax(q, axis, 2 * side - 1)))) bits |= 1u << (2 * axis + side);
  D.mgnb0[i] = (unsigned char)bits;
}

template <class T> void build(const Dev& D, cudaStream_t s) {
  pdl_launch(k_hs_reset, 1, 1, 0, s, D);
  pdl_launch(k_hs_count, grid_for(D.N), NT, 0, s, D);
  pdl_launch(k_hs_decide, 1, 1, 0, s, D);
  pdl_launch((k_hs_snapshot<T>), grid_for(D.N), NT, 0, s, D);
  for (int l = 0; l < D.L; l++) pdl_launch((k_mg_mask<T>), grid_for(D.lv[l].count), NT, 0, s, D, l);
  pdl_launch(k_mg_rows_reset, 1, 32, 0, s, D);
  for (int l = 1; l < D.L; l++) pdl_launch((k_mg_rowlist<T>), grid_for(D.lv[l].count), NT, 0, s, D, l);
  pdl_launch((k_mg_nb0<T>), grid_for(D.N), NT, 0, s, D);
  for (int l = 0; l + 1 < D.L; l++) pdl_launch((k_mg_transfer<T>), grid_for(D.lv[l].count), NT, 0, s, D, l);
  pdl_launch((k_mg_scale<T>), grid_for(D.lv[0].count), NT, 0, s, D);
  for (int l = 1; l < D.L; l++) {
    int lo, ext[3];
    // the children box extents of fine level l-1 are the same for every coarse row
    for (int a = 0; a < 3; a++) {
      const MGLevelDev& lv = D.lv[l - 1];
      int f = a == 0 ? lv.fx : (a == 1 ? lv.fy : lv.fz);
      int nf = a == 0 ? lv.nx : (a == 1 ? lv.ny : lv.nz);
      bool periodic = a == 2 || (a == 0 && D.px);
      ext[a] = (lv.aggregate || f == 1) ? f : ((periodic && nf <= 4) ? nf : 4);
    }
    (void)lo;
    if (l - 1 >= 1) {
      // from a fine level >= 1: A P per active fine row, then P^T (A P) per coarse row
      pdl_launch((k_mg_gal_ap<T>), (unsigned)((D.lv[l - 1].count + GA - 1) / GA), GA, (size_t)125 * GA * sizeof(float), s, D, l - 1);
      pdl_launch((k_mg_gal_pt<T>), (unsigned)D.lv[l].count, GP, 0, s, D, l - 1, ext[0], ext[1], ext[2]);
    } else {
      int G = ext[1] * ext[2], rpb = GT / G;
      unsigned gr = (unsigned)((D.lv[l].count + rpb - 1) / rpb);
      const int slots = D.lv[l].gal_slots > 0 ? D.lv[l].gal_slots : 125;
      pdl_launch((k_mg_galerkin<T>), gr, GT, (size_t)slots * GT * sizeof(float), s, D, l - 1, ext[0], ext[1], ext[2]);
    }
    pdl_launch((k_mg_scale8<T>), grid_for((long long)kScaleLanes * D.lv[l].count), NT, 0, s, D, l);
  }
  for (int l = 1; l < D.L; l++) pdl_launch((k_mg_ell<T>), grid_for((long long)D.lv[l].stencil * D.lv[l].count), NT, 0, s, D, l);
  if (D.lv[D.L - 1].count <= 64) pdl_launch((k_mg_chol<T>), 1, 64, 0, s, D, D.L - 1);
  pdl_launch(k_hs_record, 1, 1, 0, s, D);
}

}  // namespace

void launch_mg_cols(const Dev& D, cudaStream_t s) {
  for (int l = 1; l < D.L; l++) pdl_launch(k_mg_cols, grid_for(D.lv[l].count), NT, 0, s, D, l);
}
// Blocks of the coarse launch (one per SM when the kernel fits once per SM, else 0) and whether a
// cooperative launch can be captured into a graph on this device (checked once per call).
int coarse_blocks(size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mg_coarse<float>, CNT, smem) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return 0;
  }
  int per_sm16 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm16, k_mg_coarse<__nv_bfloat16>, CNT, smem) != cudaSuccess || per_sm16 < 1) {
    cudaGetLastError();
    return 0;
  }
  int* x = nullptr;
  cudaStream_t s = nullptr;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
  bool ok = cudaMalloc(&x, sizeof(int)) == cudaSuccess && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)sms);
    cfg.blockDim = dim3(32);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const bool launched = cudaLaunchKernelEx(&cfg, k_coop_probe, x) == cudaSuccess;
    ok = cudaStreamEndCapture(s, &g) == cudaSuccess && launched && g && cudaGraphInstantiate(&e, g, 0) == cudaSuccess &&
         cudaGraphLaunch(e, s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
  }
  if (e) cudaGraphExecDestroy(e);
  if (g) cudaGraphDestroy(g);
  if (s) cudaStreamDestroy(s);
  if (x) cudaFree(x);
  cudaGetLastError();
  return ok ? sms : 0;
}

bool leg_available(size_t smem) {
  if (smem > (size_t)kBottomSmemMax) return false;
  if (cudaFuncSetAttribute(k_mg_leg<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBottomSmemMax) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg_leg<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBottomSmemMax) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchAttribute cl[1];
  cl[0].id = cudaLaunchAttributeClusterDimension;
  cl[0].val.clusterDim.x = kLegCtas;
  cl[0].val.clusterDim.y = 1;
  cl[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t occ = {};
  occ.gridDim = dim3(kLegCtas);
  occ.blockDim = dim3(kLegThreads);
  occ.dynamicSmemBytes = smem;
  occ.attrs = cl;
  occ.numAttrs = 1;
  int n32 = 0, n16 = 0;
  if (cudaOccupancyMaxActiveClusters(&n32, k_mg_leg<float>, &occ) != cudaSuccess ||
      cudaOccupancyMaxActiveClusters(&n16, k_mg_leg<__nv_bfloat16>, &occ) != cudaSuccess || n32 < 1 || n16 < 1) {
    cudaGetLastError();
    return false;
  }
  // the launch form the cycle uses (cluster dimension, programmatic serialization), run once on a
  // stream and once from the body of a conditional graph node, as the CG loop's graphs hold it
  int* x = nullptr;
  cudaStream_t s = nullptr;
  cudaGraph_t g = nullptr, body_out = nullptr;
  cudaGraphExec_t e = nullptr;
  bool ok = cudaMalloc(&x, sizeof(int)) == cudaSuccess && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess;
  cudaLaunchAttribute attr[2];
  attr[0] = cl[0];
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kLegCtas);
  cfg.blockDim = dim3(32);
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = g_pdl ? 2 : 1;
  int got = 0;
  ok = ok && cudaMemsetAsync(x, 0, sizeof(int), s) == cudaSuccess && cudaLaunchKernelEx(&cfg, k_cluster_probe, x) == cudaSuccess &&
       cudaMemcpyAsync(&got, x, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess &&
       got == 1;
  ok = ok && cudaMemsetAsync(x, 0, sizeof(int), s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess &&
       cudaGraphCreate(&g, 0) == cudaSuccess;
  if (ok) {
    cudaGraphConditionalHandle hc;
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    cudaGraphNode_t node;
    ok = cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok) {
      p.conditional.handle = hc;
      p.conditional.type = cudaGraphCondTypeIf;
      p.conditional.size = 1;
      ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p) == cudaSuccess;
    }
    if (ok && cudaStreamBeginCaptureToGraph(s, p.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                  cudaSuccess) {
      const bool launched = cudaLaunchKernelEx(&cfg, k_cluster_probe, x) == cudaSuccess;
      ok = cudaStreamEndCapture(s, &body_out) == cudaSuccess && launched;
    } else
      ok = false;
    got = 0;
    ok = ok && cudaGraphInstantiate(&e, g, 0) == cudaSuccess && cudaGraphLaunch(e, s) == cudaSuccess &&
         cudaMemcpyAsync(&got, x, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess &&
         got == 1;
  }
  if (e) cudaGraphExecDestroy(e);
  if (g) cudaGraphDestroy(g);
  if (s) cudaStreamDestroy(s);
  if (x) cudaFree(x);
  cudaGetLastError();
  return ok;
}

void mg_kernel_attributes() {
  cudaFuncSetAttribute(k_mg_coarse<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBottomSmemMax);
  cudaFuncSetAttribute(k_mg_coarse<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBottomSmemMax);
  cudaFuncSetAttribute(k_mg_bottom_smem<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBottomSmemMax);
  cudaFuncSetAttribute(k_mg_bottom_smem<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBottomSmemMax);
  cudaFuncSetAttribute(k_mg_galerkin<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 125 * GT * (int)sizeof(float));
  cudaFuncSetAttribute(k_mg_galerkin<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 125 * GT * (int)sizeof(float));
}
void launch_mg_build(const Dev& D, cudaStream_t s) {
  if (D.bf16) build<__nv_bfloat16>(D, s);
  else build<float>(D, s);
}
void launch_mg_vcycle(const Dev& D, cudaStream_t s, int phase) {
  if (D.bf16) Cycle<__nv_bfloat16>{D, s, phase, 0}.run();
  else Cycle<float>{D, s, phase, 0}.run();
}

}  // namespace wg
