// Device-side parameter block of one simulation: sizes, push-constant values and raw device
// pointers.  Passed by value to every kernel (a few hundred bytes of kernel parameters).
#pragma once
#include <cstddef>
#include <cstdint>

namespace wg {

constexpr int kMaxLevels = 12;
constexpr int kMaxStencil = 125;
constexpr int kBottomSmemMax = 200 * 1024;  // shared-memory stage of the bottom levels
constexpr int kSolidPad = 16;  // margin of the tabulated solid() lookup
constexpr int kDonorWall = -1;  // donor table: a solid cell on one side of the face only
constexpr int kDonorNone = -2;  // donor table: solid on both sides, no mirror face

// Indices into the double control block beyond the reference's 96 entries.
enum CtrlExtra {
  kSweepRound = 96,     // staged rounding ledger of the three sweeps (FP64)
  kSweepComp = 97,      // staged compression ledger (FP64)
  kRoundCommit = 98,    // committed rounding ledger
  kCompCommit = 99,     // committed compression ledger
  kConservation = 100,  // V_now - V0 - sum of ledgers at the last acceptance
  kQuota = 101,         // request quota (>= 0 steps, < 0 minus a deadline)
  kWarmUsed = 102,      // trials started from the learned warm start
  kDefectRounds = 103,  // defect-correction rounds run since creation
  kNetLoaded = 104,     // 1 once a warm-start network is loaded
  kWarmPick = 105,      // 1 when this trial starts from the network's pressure
};
constexpr int kNetLayerWords = 27 * 2 * 64;  // mma fragments of one layer's weights (uint32)

struct MGLevelDev {
  int nx, ny, nz, count;
  int fx, fy, fz, aggregate;
  int stencil;       // number of stencil offsets
  int twidth;        // transfer-cache width
  int off;           // offset of this level inside the per-field MG vectors
  long long moff;    // offset of this level's canonical 125-slot matrix rows
  long long eoff;    // offset of this level's ELL values
  long long toff;    // offset of this level's transfer cache
  int soff;          // offset of this level's stencil in the stencil table
  int roff[3];       // restriction tables of this (coarse) level, per axis (4 entries per coarse index)
  int rext[3];       // entries used per coarse index, per axis
  int gal_slots;     // > 0: Galerkin partials of this (coarse) level kept per stencil entry (gal_cslot)
};

struct Dev {
  // grid
  int nx, ny, nz;
  long long N, NU, NV, NW, S, NF;
  float hx, hy, hz;
  float dtcfg;
  float ox, oy, oz;
  float eta0;
  int px;
  float slope, corr, corr_phase;
  int shape;
  float grav;
  int max_face_cfl;
  int hist_cap;
  float wave[4];
  float tol;
  int linear_air, stokes2, flags;
  int coastal;
  float forcing[4];
  float right_abs;
  float cfl;
  double cell_d;  // hx*hy*hz in double
  // coastal zone: x columns [0, zone_x_end) hold every cell/face with a nonzero relaxation rate
  int zone_x_end;
  // Wave-target tables, rebuilt every trial for the trial's three times (accepted, CFL look-ahead,
  // new): surface per cell column, u and v target velocities per face column and row, and the
  // relaxation factor per column for the trial's dt.  wstamp holds the three times and that dt;
  // a lookup whose time (or dt) is not stamped, or whose column/row is outside, evaluates directly.
  float2* wsurf;   // [3][wt_w]
  float* wvel;     // [3][2][wt_h][wt_w]
  float* wdecay;   // [2][wt_w]: cell centres, u faces
  float* wstamp;   // [4]
  int wt_x0, wt_w, wt_h;

  // physical banks [F | u | v | w | p]
  float* bank0;
  float* bank1;
  // fine-grid work
  float* r;      // residual
  float* z;      // preconditioned residual
  float* d;      // search direction
  float* q;      // A d
  float* diag;   // operator diagonal (work[12N] of the reference)
  float* b;      // right-hand side
  float* coef;   // 6 N face coefficients (face order -x,+x,-y,+y,-z,+z)
  float* pbase;  // defect-correction base pressure (work[13N])
  float* phi;    // signed distance
  signed char* kind;  // -1 solid, 0 air, 1 wet
  float4* plane;      // PLIC plane per cell
  // motion work
  float* mF;     // scratch F of sweep 1
  float* mci;    // frozen compression indicator c_i
  float* fwd;    // MacCormack forward value per face (also op 82 scratch)
  float* tcache; // 6 faces: lo, hi, valid, start velocity xyz
  int* src0;     // nearest-source banks
  int* src1;
  float* vband0; // valid band per bank
  float* vband1;
  float* pmask0; // pressure mask per bank
  float* pmask1;
  float4* history;   // 4 rows per trial
  float4* chistory;  // 5 rows per step
  // control and reductions
  double* c;            // control block
  double* part;         // per-block partials
  unsigned int* count;  // last-block counters, one per reduction site
  // solid table
  const signed char* solid_tab;
  const signed char* clear_tab;  // 1 when no solid cell lies in the 3x3 (x, y) window
  const unsigned char* mac_class;  // per (axis, y, x) face column: 1 near a solid cell or the domain edge
  unsigned char* ext_nb;         // per face: wall bit and usable extension neighbours (static)
  const signed char* gal_cslot;  // per level, 125 box slots -> stencil entry (-1: not in the stencil)
  int* mac_list;                 // MacCormack work list (faces)
  unsigned* mac_ctr;             // kMacCounters: interior count, boundary count, op 27 / op 28 cursors of
                                 // the general pass, op 27 / op 28 cursors of the fast pass, op 27 / op 28
                                 // counts of faces the fast pass handed over
  int* mac_ovf;                  // faces the fast pass handed over to the general pass
  int* mac_dtab;                 // per face, the donor of its solid neighbourhood (static geometry):
                                 // kDonorWall, kDonorNone, or 2 f (+1 with parity -1) of the face read
  int* geo_queue;                // cells of op 18 that need the neighbourhood search
  unsigned* geo_qcount;          // their count (reset by op 17)
  int geo_seed_grid;             // blocks of the search pass (persistent, grid-stride)
  int mac_grid;                  // persistent MacCormack blocks (3 per SM form)
  int mac_grid2;                 // the same, 2 per SM form
  int mac_fast_grid;             // persistent blocks of the interior fast-path pass
  int mac_minb;                  // which form runs (2 or 3 blocks per SM)
  int mac_split;                 // interior faces on the fast-path pass
  int pdl_early;                 // kernels trigger their dependents' launch on entry
  // learned warm start (allocated when warm_start is configured): weights in mma fragment order,
  // biases [4][16], scales (F, b, p_prev inputs; output), BF16 activations [2][N][16], p_net [N]
  int net_on;
  uint32_t* net_w;
  uint16_t* net_wt;  // the same weights for the tcgen05 layers: [layer][tap][channel half][co][8 ci] BF16
  int net_tc05;      // 1: network layers on tcgen05 (else mma.sync)
  float* net_b;
  float* net_scale;
  unsigned short* net_act;
  float* net_p;
  int tab_w, tab_h;

  // multigrid
  int L;
  MGLevelDev lv[kMaxLevels];
  int mg_smoother, mg_smoothing, mg_mode, mg_lag, mg_aggr;
  int ipb;                   // CG iterations per reference batch (coupled_gpu.gd:14)
  int bf16;                  // storage precision of the MG vectors/operators
  void* mgv;                 // 8 fields x total_nodes (float or bf16): 0 rhs,1/2 x,3 active,4 scale,6 res,7 cheb d
  long long mg_nodes;        // total nodes over all levels
  float* mgmat;              // canonical 125-slot rows of levels >= 1 (FP32, build only)
  float* gal_ap;             // A P of the Galerkin product from a fine level >= 1 (125 per fine cell)
  void* mgell;               // ELL values [k][i] of levels >= 1 (float or bf16)
  int* mgtid;                // transfer cache ids
  float* mgtw;               // transfer cache weights
  unsigned long long* mgtq;  // transfer cache: coarse cell coordinates, 21 bits per axis
  float* mglinv;             // dense L^-1 of the last level
  float* snapshot;           // 9 N hierarchy snapshot
  float* previous;           // 9 N previous-trial audit copy
  void* c0;                  // 6 N level-0 face coefficients for the V-cycle (float or bf16)
  unsigned int* hstate;      // hierarchy audit state
  const int* stencil_tab;    // 3 ints per offset, all levels
  const int* stencil_lin;    // linear offset per stencil entry (interior cells)
  const int* rt_idx;         // restriction tables: fine coordinate (-1 outside)
  const float* rt_w;         // restriction tables: axis weight
  unsigned char* mgnb0;      // level-0 neighbour-active bits
  int* mgcol;                // ELL columns of levels >= 1, same layout as mgell
  int mg_bottom;             // first level solved by the single-block bottom kernel
  int mg_rows_below;         // levels with fewer rows use the product-parallel apply
  int mg_rows_rr;            // rows per block of the product-parallel apply (8, 16, 32 or 64)
  int mg_thread_nt;          // block size of the one-thread-per-row sweeps (128 or 256)
  int mg_lanes;              // lanes per row of the large-level sweeps (4: k_mgl4, 1: k_mgl)
  int* mg_rowlist;           // active rows of each level >= 1 (level l at lv[l].off)
  unsigned* mg_rowcount;     // [kMaxLevels] entries of each list
  int mg_bottom_smem;        // bytes of the shared-memory bottom stage (0: bottom levels too large)
  int mg_coarse_from;        // first level of the one-launch coarse V-cycle (0: not used)
  int coarse_blocks;         // blocks of that cooperative launch (one per SM)
  unsigned* gbar;            // its grid barrier: arrival count, generation
  int mg_leg_from;           // first level of the one-cluster coarse leg (0: not used)
  int mg_leg_smem;           // dynamic shared memory of each block of that launch
};

// Reduction sites (one last-block counter each).
enum Site {
  kSiteCFL = 0,
  kSiteCompress,
  kSiteSweep,
  kSiteCoastF,
  kSiteCoastM,
  kSiteBounds,
  kSiteCGInit,
  kSiteDot,
  kSiteRZ,
  kSiteAccept,
  kSiteHS,
  kSiteWarm,
  kSiteCount
};

}  // namespace wg
