// xg_internal.h — shared host/device declarations of the GB300 hot path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <string>
#include <vector>

#include "../../include/xyce_gb300.h"
#include "xg_bsim4.h"

namespace xg {

constexpr int kRowBlock = 256;       // rows per block of the row kernels (fixed: partial slots)
constexpr int kMaxPwlScan = 1 << 20; // bound on PWL point scans
constexpr int kLongGather = 96;      // gathers longer than this are split into parts, a warp each
constexpr int kLongPart = 256;       // gathered items per part of a long gather
constexpr int kLongSolveRow = 256;   // triangular-solve rows longer than this get a whole block
// Frozen-pivot acceptance on the device: a pivot below this fraction of its
// updated column triggers re-pivoting by the host.
constexpr double kRuntimePivotTol = 1e-2;
// A column whose pivot already failed that test in the analysis' own trial
// factorization (a near-singular matrix: re-pivoting cannot help it) is held
// to this fraction of the pivot ratio it had there instead, so that a frozen
// order that goes bad on later values still re-pivots.
constexpr double kExemptSlack = 1e-4;

// Circuit phases of the device-resident state machine.
enum Phase : int { PH_DC = 0, PH_TRAN = 1, PH_DONE = 2, PH_FAILED = 3, PH_STALL = 4, PH_PAUSED = 5 };

// Per-circuit integrator / Newton state, one struct per circuit in HBM.
// Field names follow StepErrorControl / OneStep / DampedNewton members.
struct CircState {
  // time integration (StepErrorControl, OneStep)
  double t;            // currentTime (last accepted)
  double h;            // currentTimeStep
  double tn;           // time of the step being attempted
  double stopTime;     // next breakpoint or tstop
  double lastTimeStep, tsum, saved, estOverTol;
  double psi[3], beta[3], ck;
  double alpha[3];     // Gear12 coefficients of Q, qH0, qH1 (the residual is F - B + (.)/h)
  double qscale, fscale, hscale;   // residual/Jacobian coefficients of this attempt
  double errwt;        // reltol*max|x_curr| + abstol (NEWLTE = 1)
  double xmax_curr;    // max |x_curr|
  double gshunt;       // operating-point gmin stepping shunt
  // Newton (DampedNewton)
  double normRHS, normRHS_init, normRHS_old, maxNormRHS, wtNormDX, tmpConvRate;
  double wrms_sum;
  int phase, iter, order, numberOfSteps, nef, stepNumber;
  int beginning, lastOk, count, newton_status;
  int need_solve;      // this tick factors/solves/updates
  int step_end;        // 1 = Newton finished this tick (converged or failed)
  int accept;          // 1 accepted / 0 rejected (valid when step_end)
  int start_step;      // 1 = next tick begins a new step attempt (predictor applied)
  int init_jct, init_hist, dc_stage, limited, bp_index, singular, stall_prev;
  // learned predictor (xg_mlp.cu): gate state and per-predictor statistics
  int ml_use, ml_pending, ml_backoff, last_iters, ml_steps, plain_steps;
  double plain_ema;
  long long ml_iters, plain_iters;
  // factor reuse: a circuit without nonlinear devices whose Jacobian
  // coefficients equal those of its last factorization (same analysis) has
  // the same Jacobian bit for bit and skips the refactorization
  int refactor;        // this tick's LU work factors (else only solves)
  int f_gen;           // analysis generation of the last factorization
  double f_qscale, f_fscale, f_gshunt;
  long long factor_skips;
  // counters
  long long accepted, rejected, newton_iters, newton_fail, lte_fail, dcop_iters;
  long long stop_at;   // pause once this many steps are accepted
  int n_out;
};

struct TranParams {
  double tstart, tstop, hmax, hmin, reltol, abstol;
  double nl_reltol, nl_abstol, nl_deltaxtol, nl_rhstol, nl_smallupdatetol;
  int nl_maxstep, max_steps, max_order;
  int gear;  // 1 = Gear12 (BDF1/2), 0 = OneStep
  double bptol;
  // operating-point options (N_NLS_Manager.C:1030-1052)
  double dc_reltol, dc_abstol, dc_deltaxtol, dc_rhstol;
  int dc_maxstep;
  int dc_only;  // stop every circuit once its operating point converges
  int newton_only;  // one Newton solve per circuit, then stop (xg_newton_solve)
  int reuse_factors;  // skip bit-identical refactorizations (xg_lu_set_reuse)
};

constexpr double kGmin = 1.0e-12;  // DeviceOptions gmin default

// MOSFET level-1 model-level (effective model) parameters after temperature
// and geometry processing (N_DEV_MOSFET1.C:383-470, 3487-3730, 3939-4020).
struct Mos1Model {
  double dtype, gamma, tPhi, lambda, vt, DrainSatCur, SourceSatCur, sourceVcrit, drainVcrit;
  double OxideCap, Cgso, Cgdo, Cgbo, Cbd, Cbdsw, Cbs, Cbssw, tDepCap, tBulkPot, MJ, MJSW;
  double f2d, f3d, f4d, f2s, f3s, f4s, M, gammaSqrtPhi;
  double gsatD, gsatS;  // DrainSatCur / vt, SourceSatCur / vt (reverse-bias conductances)
  double gbdR, gbsR;    // gsatD + gmin, gsatS + gmin
  double sqrtPhi;       // sqrt(tPhi)
  double argPhi;        // gamma / (2 sqrt(tPhi)), 0 when sqrt(tPhi) <= 0
  int has_gate_caps, has_junc_caps;
};

// Diode model-level parameters after temperature processing (N_DEV_Diode.C:2040-2237),
// with the instance's AREA and PJ folded in.  Sidewall: sw 0 none, 1 its own
// characteristic (NS given), 2 merged into Isat (JSW given, NS not).
struct DiodeModel {
  double Isat, IsatR, Vte, VteR, VteBRK, Gspr, tVcrit, tIKF, tJctPot, tJctCap, tDepCap;
  double tF1, F2, F3, M, TT, tBrkdwnV;
  double IsatSW, VteSW, CzeroSW, tJctSWPot, tDepSWCap, F2SW, F3SW, MJSW;
  int bvGiven, sw;
};

// Learned predictor MLP 5 -> 64 -> 64 -> 1 (xg_mlp.cu).  Master parameter
// vector (FP32): W1[5][64] | b1[64] | W2[64][64] (in x out) | b2 | w3 | b3.
constexpr int kMlpIn = 5, kMlpInPad = 16, kMlpHid = 64;
constexpr int kMlpOffW1 = 0, kMlpOffB1 = kMlpIn * kMlpHid, kMlpOffW2 = kMlpOffB1 + kMlpHid;
constexpr int kMlpOffB2 = kMlpOffW2 + kMlpHid * kMlpHid, kMlpOffW3 = kMlpOffB2 + kMlpHid;
constexpr int kMlpOffB3 = kMlpOffW3 + kMlpHid, kMlpParams = kMlpOffB3 + 1;
constexpr int kMlpNorm = 2 * kMlpIn + 2;  // in_shift[5], in_scale[5], out_shift, out_scale
constexpr int kMlBackoff = 16;            // polynomial-predictor steps after a worse learned step
constexpr double kMlpScaleFloor = 1e-9;   // V: motion scale floor of the learned correction
constexpr double kMlpActive = 1e-5;       // V: nodes moving less keep the polynomial guess
struct MlpDev {
  float *theta = nullptr, *norm = nullptr;
  unsigned short *w1t = nullptr, *w2t = nullptr, *w2 = nullptr;  // BF16 operand copies
};

// Slot counts per instance.
constexpr int kMosF = 3, kMosQ = 4, kMosL = 4, kMosM = 16;
constexpr int kDioF = 3, kDioQ = 2, kDioL = 2, kDioM = 7;

// Device-resident arrays (all cudaMalloc'd, owned by the context).
struct DevArrays {
  // circuits
  int *circ_of_row = nullptr;
  int *offsets = nullptr;
  CircState *cs = nullptr;
  TranParams *tp = nullptr;
  // linear part (CSR order) and pattern
  int *rp = nullptr, *ci = nullptr, *erow = nullptr, *diag = nullptr;
  double *Glin = nullptr, *Clin = nullptr;
  // contribution lists: per row for vector slots, per CSR entry for matrix slots
  int *vF_ptr = nullptr, *vF_idx = nullptr;
  int *vQ_ptr = nullptr, *vQ_idx = nullptr;
  int *vL_ptr = nullptr, *vL_idx = nullptr;
  int *vB_ptr = nullptr, *vB_idx = nullptr;
  int *m_ptr = nullptr, *m_idx = nullptr;
  char *is_branch = nullptr;                 // per row: voltage-source branch unknown
  // long gathers, reduced by warps in a pre-pass: rows (F, Q, B, L sums) and J entries
  // (a long gather of w items is split into P = ceil(w / kLongPart) parts;
  // part b handles part b - ptr[l] of gather l = *_blk[b]; the parts of
  // gather l are ptr[l] .. ptr[l+1]; part p of P takes the items p*32 + lane
  // + m*32*P of each list)
  int *long_rows = nullptr, *row_long = nullptr, *long_ents = nullptr, *ent_long = nullptr;
  int *lrow_ptr = nullptr, *lrow_blk = nullptr, *lent_ptr = nullptr, *lent_blk = nullptr;
  double *long_rsum = nullptr, *long_esum = nullptr;
  unsigned long long *done_acc = nullptr;  // completion count scratch: [done, Newton iterations, blocks]
  // slot value buffers
  double *sF = nullptr, *sQ = nullptr, *sL = nullptr, *sL2 = nullptr, *sB = nullptr;
  double *sM = nullptr, *sM2 = nullptr;   // combined J slots / (dF, dQ) in separate mode
  // sources
  int *src_kind = nullptr, *src_off = nullptr, *src_circ = nullptr;
  double *src_data = nullptr;
  // MOSFET-1 SoA
  int *m1_node = nullptr;   // 4*n: D,G,S,B planes
  int *m1_model = nullptr, *m1_circ = nullptr;
  double *m1_beta = nullptr, *m1_vbi = nullptr;
  Mos1Model *m1_models = nullptr;
  // BSIM4 SoA
  int *b4_node = nullptr;   // 4*n: D,G,S,B planes
  int *b4_model = nullptr, *b4_circ = nullptr;
  b4::B4Model *b4_models = nullptr;
  // diode SoA
  int *d_node = nullptr;    // 3*n: P,N,R planes
  int *d_model = nullptr, *d_circ = nullptr;
  DiodeModel *d_models = nullptr;
  // state / store (curr = accepted, next = iterate)
  double *sta_curr = nullptr, *sta_next = nullptr, *sto_curr = nullptr, *sto_next = nullptr;
  // vectors (length n)
  double *x = nullptr, *xcurr = nullptr, *xn0 = nullptr, *dx = nullptr, *rhs = nullptr;
  double *Qv = nullptr, *FmB = nullptr, *Fv = nullptr, *Bv = nullptr;
  double *qh0 = nullptr, *qh1 = nullptr, *qh2 = nullptr, *xh1 = nullptr, *xh2 = nullptr;
  double *Qc = nullptr, *FmBc = nullptr, *solwt = nullptr;
  double *J = nullptr;      // Jacobian values (CSR order)
  // learned predictor: network and the differences of the last four accepted solutions
  MlpDev mlp;
  double *mlh1 = nullptr, *mlh2 = nullptr, *mlh3 = nullptr;
  double *out_p = nullptr;  // recorded predictor values (training targets)
  // per-(block,circuit) partial reduction slots
  int *pair_base = nullptr, *blk_cfirst = nullptr, *pair_cstart = nullptr;
  double *pmax = nullptr, *psum = nullptr;
  // recording
  int *probe_idx = nullptr, *probe_ptr = nullptr;
  double *out_t = nullptr, *out_v = nullptr;
  signed char *out_o = nullptr;  // integration order of each recorded point (0: operating point)
  int *status = nullptr;      // mapped host memory: [0] finished circuits, [1] LU breakdown
  int *lu_gen = nullptr;      // generation of the current LU analysis (bumped by every analysis)
  char *circ_linear = nullptr;  // per circuit: no nonlinear devices (its Jacobian is the linear part)
};

// Grouped execution schedule of one triangular sweep (factorization, L solve;
// the U solve runs the factorization schedule backwards).  items[0 .. n_hub)
// are hub items (no dependencies, many dependents) executed first; then
// groups 0 .. n_groups-1, each closed under dependencies and run by one CTA
// with a barrier between its local levels; then the top (group n_groups),
// run by a single CTA.  Group g owns levels [grp_lvl[g], grp_lvl[g+1]); level
// k spans items[lvl_ptr[k] .. lvl_ptr[k+1]).
struct Schedule {
  std::vector<int> items, lvl_ptr, grp_lvl;
  std::vector<char> is_long, is_long_rev;  // whole-block items (forward / backward sweep)
  std::vector<char> is_thread, is_thread_rev;  // single-thread items (forward / backward sweep)
  int n_hub = 0, n_groups = 0, n_top_items = 0;
};

struct SchedDev {
  int *items = nullptr, *lvl_ptr = nullptr, *grp_lvl = nullptr;
  char *is_long = nullptr, *is_long_rev = nullptr;
  char *is_thread = nullptr, *is_thread_rev = nullptr;
  int n_hub = 0, n_groups = 0, n_top_items = 0;
};

// Allocation-free solve (xg_lu_solve_noalloc): largest system it accepts and
// the number of devices whose scratch address is cached.
constexpr int kNoAllocMaxN = XG_NOALLOC_MAX_N;
constexpr int kNoAllocMaxDevices = 64;

constexpr int kLongColumn = 512;   // factor columns longer than this use the whole CTA
constexpr int kHubFanout = 64;     // items with more dependents than this run in the prologue
constexpr int kGroupCap = 512;     // items per dependency-closed group
constexpr int kPackSmall = 4;        // groups of at most this many items are packed together ...
constexpr int kPackCap = 256;        // ... up to this many items ...
constexpr int kPackCapWeight = 1024; // ... and entries per CTA
constexpr int kTopRightLooking = 64;  // tops at least this large factor right-looking
// Ordering choice: estimated time = FMAs / kOrderFmaRate + elimination-tree
// height * kOrderLevelTime (sparse FP64 updates on GB300 run far below the
// FP64 peak; each dependency level costs a few microseconds of latency).
constexpr double kOrderFmaRate = 5e9;
constexpr double kOrderLevelTime = 4e-6;
// Top schedule choice (one CTA vs a launch per level on all SMs): FP64 FMAs
// per second of one SM (GB300: ~0.6 TFMA/s over 152 SMs), the gap between
// back-to-back launches of a graph, a CTA barrier with its dependent loads.
constexpr double kSmFmaRate = 4e9;
constexpr double kNumSms = 152;
constexpr double kLaunchTime = 2.5e-6;
constexpr double kBarrierTime = 1e-6;
constexpr int kGroupSmemBytes = 96 * 1024;  // largest group buffer staged in shared memory
constexpr int kSmemPerSm = 227 * 1024;      // shared memory of an SM available to CTAs
// Short items of the grouped sweeps run on one thread each: a warp-wide FP64
// instruction takes the same FP64-pipe time with one active lane as with 32,
// and GB300's FP64 pipe is narrow, so a warp spent on a 3-entry column wastes
// most of it.
constexpr int kThreadColumn = 32;  // factor columns with at most this many entries ...
constexpr int kThreadWork = 96;    // ... and at most this many update products
constexpr int kThreadRow = 4;      // solve rows with at most this many entries
constexpr int kSolveSmemBytes = 48 * 1024;  // largest solve group staged in shared memory
constexpr int kStageRow = 64;               // staged solve groups: rows of at most this many entries

// LU structures (device) produced by the host analysis.  Plain data: it is
// passed to kernels by value.
struct LUDev {
  int n = 0;
  long long nnz = 0;
  int *row_of_step = nullptr, *col_of_step = nullptr, *circ_of_step = nullptr;
  int *cp = nullptr, *ri = nullptr, *diag = nullptr, *src = nullptr;
  double *lu = nullptr, *y = nullptr;
  int *l_ptr = nullptr, *l_pos = nullptr, *l_col = nullptr;   // L by rows (solves)
  int *u_ptr = nullptr, *u_pos = nullptr, *u_col = nullptr;   // U by rows (solves)
  char *exempt = nullptr;    // per step: threshold test scaled by pscale (kExemptSlack)
  double *pscale = nullptr;  // per exempt step: its threshold as a fraction of pivot_tol
  int *breakdown = nullptr;  // device flag: first failing step + 1
  int *upd_off = nullptr, *upd_pos = nullptr;  // per U entry: target positions of its update
  const int4 *umeta = nullptr;                   // per U entry: see LUHost::umeta
  const int4 *fm_col = nullptr, *fm_ent = nullptr;  // see LUHost::fm_col
  int *fm_eptr = nullptr, *fm_tptr = nullptr, *fm_tgt = nullptr, *fm_gbytes = nullptr;
  int fm_smem[2] = {0, 0};  // launch buffer bytes (double | float factors) when metadata is staged
  int fm_on = 0;            // stage the update metadata of the groups that have it (fm_gbytes > 0)
  SchedDev fs, ls;           // factor (and, backwards, U solve) / L-solve schedules
  int f_levels = 0, l_levels = 0, u_levels = 0;  // plain level counts (statistics)
  // Mixed precision (FP32 factors, FP64 iterative refinement): lu32 holds the
  // factors; each solve is refined n_refine times against the FP64 matrix
  // a_vals (CSR a_rp/a_ci in unknown order, the values last factored).
  int mixed = 0, n_refine = 0;
  // factor schedule's top (n_top_rl steps, ascending, every L row of a top
  // column a top step): a multi-CTA pull of the sub-tree updates, then one
  // right-looking CTA; n_top_rl == 0: the top runs left-looking like a group
  int n_top_rl = 0;
  int *top_items = nullptr;
  char *is_top = nullptr;
  // level-synchronous right-looking top (all SMs; see LUHost::tlv_*): device
  // arrays, and host copies of the level pointers for the per-level launches
  int n_top_lv = 0;
  int *tlv_items = nullptr, *tlv_item_ptr = nullptr, *tlv_grp_ptr = nullptr;
  int *tgrp_col = nullptr, *tgrp_ptr = nullptr, *tgrp_pos = nullptr, *tgrp_k = nullptr;
  const int *h_tlv_item_ptr = nullptr, *h_tlv_grp_ptr = nullptr;
  // the tops of the solves one level per launch on all SMs (when the top is
  // large): host copies of the L- and factor-schedule level pointers and the
  // tops' level ranges [lo, hi)
  const int *h_ls_lvl_ptr = nullptr, *h_fs_lvl_ptr = nullptr;
  // factor groups staged in shared memory (see LUHost::grp_soff); grp_fit[0|1]
  // = entries of the largest group within kGroupSmemBytes as double | float
  int *grp_soff = nullptr, *grp_snz = nullptr;
  int grp_fit[2] = {0, 0};
  int fs_threads = 512, ls_threads = 512, us_threads = 512;  // CTA sizes of the group sweeps
  int ordering = 0;  // XG_ORDER_* of the analysis
  // circuit of every factor / L-solve group (-1: a packed group mixing
  // circuits): an inactive circuit's group returns before staging anything
  int *fs_gcirc = nullptr, *ls_gcirc = nullptr;
  // solve groups staged in shared memory (see LUHost::ls_eptr); *_smem =
  // buffer bytes of the largest staged group (0: none staged)
  int *ls_eptr = nullptr, *ls_epos = nullptr, *ls_esrc = nullptr, *ls_gbytes = nullptr;
  int *us_eptr = nullptr, *us_epos = nullptr, *us_esrc = nullptr, *us_gbytes = nullptr;
  int ls_smem = 0, us_smem = 0;
  int ls_top_lo = 0, ls_top_hi = 0, fs_top_lo = 0, fs_top_hi = 0;
  float *lu32 = nullptr;
  double *ir_r = nullptr;
  const int *a_rp = nullptr, *a_ci = nullptr, *a_circ = nullptr;
  const double *a_vals = nullptr;
};

// Circuit-resident form of the tick (batches of small circuits): one CTA
// runs every stage of a tick for one circuit and loops over ticks until the
// circuit pauses, finishes, fails or parks on a pivot breakdown; CTAs take
// circuits from a queue (largest first).  Per circuit c: its MOSFET-1 and
// diode instances, sources, long rows / long Jacobian entries (CSR lists
// *_ptr[c] .. *_ptr[c+1]), and its LU levels — lv_ptr[c] .. lv_ptr[c+1] are
// level indices into f_lptr (factor; the U solve walks them backwards) and
// l_lptr (L solve), whose items are in f_items / l_items.  Per step: how the
// grouped kernels compute it (f_kind: 0 one thread, 1 a warp, 2 the whole
// CTA; l_meth / u_meth: 0 y = b, 1 one thread in entry order, 2 an 8-lane
// team, 3 the whole CTA in the fixed long-row order), so that both forms
// compute the same bits.
constexpr int kFusedMaxRows = 2048;        // largest circuit the resident form takes
constexpr int kFusedMinCircuits = 64;      // smallest batch the resident form takes
constexpr int kFusedMaxTicks = 4096;       // ticks of one circuit in one launch, at most (then the host relaunches)
// Within a level the items are sorted by how they are computed, and
// f_split / l_split / u_split hold, per level, where the later kinds start
// ({warp, CTA} for the factor, {8-lane team, CTA} for the solves; the L
// solve's first kind covers y = b and one-thread rows, told apart by
// l_meth); u_items holds the factor levels' items in U-solve order.
struct FusedDev {
  int *order = nullptr, *queue = nullptr;
  int *m1_ptr = nullptr, *m1_list = nullptr, *d_ptr = nullptr, *d_list = nullptr;
  int *src_ptr = nullptr, *src_list = nullptr;
  int *lr_ptr = nullptr, *lr_list = nullptr, *le_ptr = nullptr, *le_list = nullptr;
  int *f_cl = nullptr, *f_lptr = nullptr, *f_items = nullptr, *u_items = nullptr;
  int *l_cl = nullptr, *l_lptr = nullptr, *l_items = nullptr;
  int2 *f_split = nullptr, *u_split = nullptr, *l_split = nullptr;
  signed char *f_kind = nullptr, *l_meth = nullptr, *u_meth = nullptr;
  unsigned long long *ticks = nullptr;  // [0] largest tick count of a circuit, [1] circuit-ticks (this launch)
  int max_rows = 0;
  int grid[5] = {0, 0, 0, 0, 0};  // persistent grids of the kResidentThreads CTA sizes
  // the circuit's factor columns staged in shared memory: column j at
  // c_soff[j] of its circuit's buffer (c_fcnt[c] entries); c_umeta as
  // LUDev::umeta with .x the buffer offset of L(k+1.., k); max_fbuf = 0:
  // columns stay in global memory
  int *c_soff = nullptr, *c_fcnt = nullptr;
  const int4 *c_umeta = nullptr;
  int max_fbuf = 0;
};
constexpr int kFusedSmemBytes = 160 * 1024;  // largest resident buffer (row partials + staged columns)
constexpr int kResidentSizes = 5;
constexpr int kResidentThreads[kResidentSizes] = {32, 64, 128, 256, 512};  // CTA sizes the driver tries

// Host-side analysis result.
struct LUHost {
  int n = 0;
  // steps of the factor schedule's top in ascending order when the top can be
  // factored right-looking (every L row of a top column is a top step), else empty
  std::vector<int> top_items;
  // levels of the right-looking top: level l pivots tlv_items[tlv_item_ptr[l] ..
  // tlv_item_ptr[l+1]) (independent columns), then updates the target-column
  // groups tlv_grp_ptr[l] .. tlv_grp_ptr[l+1]; group g is column tgrp_col[g]
  // receiving the U entries (positions) tgrp_pos[tgrp_ptr[g] .. tgrp_ptr[g+1])
  // of pivots tgrp_k[...] of that level
  std::vector<int> tlv_items, tlv_item_ptr, tlv_grp_ptr, tgrp_col, tgrp_ptr, tgrp_pos, tgrp_k;
  // shared-memory staging of the factor groups: column j of a group sits at
  // grp_soff[j] .. grp_soff[j] + nnz(col j) of its group's buffer (-1: not in a
  // group); grp_snz[g] = entries of group g
  std::vector<int> grp_soff, grp_snz;
  // ordering of the core: 0 nested dissection, 1 minimum degree; the
  // estimates it was chosen by (symmetric-factor FMAs, elimination-tree height)
  int ordering = 0;
  bool top_multi = false;        // factor top: a launch pair per level (else one CTA)
  bool solve_top_multi = false;  // solve tops: a launch per level (else one CTA)
  double order_fma[2] = {0, 0};
  int order_height[2] = {0, 0};
  // CTA sizes of the group sweeps (factor, L solve, U solve)
  int fs_threads = 512, ls_threads = 512, us_threads = 512;
  // Solve groups staged in shared memory: the entries of the rows at
  // schedule position t are [xs_eptr[t], xs_eptr[t+1]) of xs_epos (LU
  // position) / xs_esrc (slot of the column's row in its group's buffer, or
  // -(k+1): row k outside the group); xs_gbytes[g] = buffer bytes of group g
  // (0: not staged).  ls = L solve (L schedule), us = U solve (factor schedule).
  std::vector<int> ls_eptr, ls_epos, ls_esrc, ls_gbytes;
  std::vector<int> us_eptr, us_epos, us_esrc, us_gbytes;
  std::vector<int> row_of_step, col_of_step, cp, ri, diag, src;
  std::vector<int> f_lvl_ptr, f_cols, l_lvl_ptr, l_rows, l_ptr, l_pos, l_col;
  std::vector<int> u_lvl_ptr, u_rows, u_ptr, u_pos, u_col;
  std::vector<char> exempt;    // columns held to a scaled pivot threshold (kExemptSlack)
  std::vector<double> pscale;  // that scale: kExemptSlack * analysis pivot ratio / kRuntimePivotTol
  std::vector<int> l_long, u_long;  // per solve level: long rows at the end of the level
  Schedule fsched, lsched;
  std::vector<int> upd_off, upd_pos;  // scatter positions of each U entry's update
  // per U entry p = U(k, j), 4 ints: shared-memory index of L(k+1.., k) in the
  // group buffer (-1: not staged), |L(:, k)| below the diagonal, upd_off[p],
  // global position of L(k+1, k) — one load instead of a chain of three
  std::vector<int> umeta;
  // Factor groups whose update metadata is staged in shared memory too (after
  // the values): per schedule position t, 4 ints {value offset in the group
  // buffer, column entries, diagonal offset, pivot test (0 none: no U row
  // right of the diagonal, 1 the threshold, 2 the exempt column's scaled
  // threshold)}; fm_eptr[t] ..
  // fm_eptr[t+1] its U entries in fm_ent, 4 ints each {L(k+1.., k) source:
  // buffer index, or -(global position)-1; entry count; offset of its targets
  // in the group's fm_tgt segment (from fm_tptr[g]); position of U(k, j) in
  // the column}; fm_gbytes[g] = metadata bytes (0: values only)
  std::vector<int> fm_col, fm_eptr, fm_ent, fm_tptr, fm_tgt, fm_gbytes;
  // the closed-form choice of staging that metadata: on when the launch
  // buffer with it allows as many resident CTAs as the values alone
  bool fm_model_on = false;
};

// weight(j): entries item j touches (caps the packing of tiny groups)
Schedule build_schedule(int n, const std::function<void(int, std::vector<int> &)> &deps_of,
                        const std::function<bool(int)> &is_long,
                        const std::function<bool(int)> &is_long_rev,
                        const std::function<int(int)> &weight);

// Analysis entry (xg_symbolic.cpp): CSR pattern + values -> LUHost.
// keep_rows (optional, length n): columns with keep_rows[j] >= 0 keep that
// pivot row instead of a new match from the values (whole circuits only).
int lu_analyze_host(int n, const std::vector<int> &rp, const std::vector<int> &ci,
                    const std::vector<double> &vals, LUHost &out, std::string &err, int force_ordering = -1,
                    const std::vector<int> *keep_rows = nullptr);

// Kernel launchers (xg_kernels.cu, xg_lu.cu).
void launch_sources_k(cudaStream_t st, const DevArrays &d, int n_v, int n_src, int use_explicit, double t);
void launch_mos1_k(cudaStream_t st, const DevArrays &d, int nm, int sto_base, int combined, int masked,
                   int it, int flags, int sF, int sQ, int sL, int sM);
void launch_bsim4_k(cudaStream_t st, const DevArrays &d, int nb, int sto_base, int sta_base, int combined,
                    int masked, int it, int flags, int sF, int sQ, int sL, int sM);
void launch_diode_k(cudaStream_t st, const DevArrays &d, int nd, int combined, int masked, int it,
                    int flags, int sF, int sQ, int sL, int sM);
void launch_assemble_k(cudaStream_t st, const DevArrays &d, int n, int nnz, int n_long_row_blocks,
                       int n_long_ent_blocks);
void launch_load_vectors_k(cudaStream_t st, const DevArrays &d, int n, const double *x, double *Q,
                           double *F, double *B, double *dFv, double *dQv, int lt);
void launch_load_matrices_k(cudaStream_t st, const DevArrays &d, int nnz, double *dQdx, double *dFdx,
                            int lt);
void launch_newton_ctl_k(cudaStream_t st, const DevArrays &d, int ncirc);
void launch_update_k(cudaStream_t st, const DevArrays &d, int n);
void launch_step_ctl_k(cudaStream_t st, const DevArrays &d, int ncirc, const double *bps,
                       const int *bp_ptr, int cap);
void launch_history_k(cudaStream_t st, const DevArrays &d, int n, int cap, int pmax);
void launch_state_commit_k(cudaStream_t st, const DevArrays &d, int nm, int nd, int sto_base_m, int nb,
                           int sto_base_b, int sta_base_b);
void launch_count_done_k(cudaStream_t st, const DevArrays &d, int ncirc, const int *breakdown,
                         int *status_out);
void launch_unstall_k(cudaStream_t st, const DevArrays &d, int ncirc);
void launch_newton_weights_k(cudaStream_t st, const DevArrays &d, int n);
int resident_prepare_k(int max_rows, int max_fbuf, int device, int *grid);
void launch_resident_k(cudaStream_t st, const DevArrays &d, const LUDev &L, const FusedDev &F, int threads,
                       int ncirc, int nm, int nd, int nv, int sto_base_m, const int *slots, const double *bps,
                       const int *bp_ptr, int cap, int pmax, double pivot_tol,
                       unsigned long long *clk = nullptr);
void launch_set_target_k(cudaStream_t st, const DevArrays &d, int ncirc, int n_steps);
int lu_prepare_k();  // shared-memory opt-in of the staged group factorization
void launch_lu_factor_k(cudaStream_t st, const LUDev &L, const double *vals, CircState *cs, int masked,
                        double pivot_tol);
void launch_lu_solve_k(cudaStream_t st, const LUDev &L, const double *b, double *x, const CircState *cs,
                       int masked);
int noalloc_scratch(int device, double **out, std::string &err);
void launch_ml_predict_k(cudaStream_t st, const DevArrays &d, int n, int ncirc, int enabled);
void launch_mlp_refresh_k(cudaStream_t st, const MlpDev &P);
int launch_mlp_grad_k(cudaStream_t st, const MlpDev &P, const float *X, const float *Y, int N, float *grad,
                      float *loss, int sm_count);
void launch_mlp_adam_k(cudaStream_t st, const MlpDev &P, const float *grad, float *m1, float *m2, float lr,
                       float b1c, float b2c);
void launch_mlp_forward_k(cudaStream_t st, const MlpDev &P, const float *X, int N, float *out);
void launch_lu_solve_noalloc_k(cudaStream_t st, LUDev L, double *scratch, const double *b, double *x,
                               const CircState *cs);

}  // namespace xg
