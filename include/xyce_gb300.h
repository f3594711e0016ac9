/*
 * xyce_gb300.h — C-ABI of the GB300 transient Newton hot path.
 *
 * One library, libxyce_gb300.so, built for sm_103a.  It replaces, behind
 * plain pointers and sizes, the path Xyce runs on every Newton iteration:
 *
 *   Device::DeviceMgr::updateState / loadDAEVectors / loadDAEMatrices
 *     src/DeviceModelPKG/Core/N_DEV_DeviceMgr.C:3857, 4156, 3980
 *     (called by Loader::CktLoader, src/LoaderServicesPKG/N_LOA_CktLoader.C:913, 615, 458,
 *      abstract interface src/LoaderServicesPKG/N_LOA_Loader.h:97-365)
 *   the KLU numeric refactorization and solve
 *     src/LinearAlgebraServicesPKG/N_LAS_AmesosSolver.C:216-440
 *   Nonlinear::DampedNewton::solve / converged_
 *     src/NonlinearSolverPKG/N_NLS_DampedNewton.C:362-520, 1191-1396
 *   TimeIntg::OneStep predictor / residual / Jacobian / step control
 *     src/TimeIntegrationPKG/N_TIA_OneStep.C:135-500, 1584-2240
 *
 * Conventions
 *   - Unknowns are 0-based MNA indices; ground is -1.
 *   - Every vector or matrix-value pointer passed to the loader, solve and
 *     update entry points is a DEVICE pointer (cudaMalloc'd by the caller,
 *     on the context's device).  Setup entry points take HOST arrays.
 *   - Matrix values are in the CSR pattern returned by xg_get_pattern.
 *   - All entry points return an int status: XG_OK (0) or a negative code.
 *   - Calls are ordered on the context's CUDA stream; functions that return
 *     numeric results to the host synchronize that stream.
 *   - No entry point falls back to the CPU: without a usable GB300 (sm_103a)
 *     device, xg_create fails with XG_ERR_CUDA.
 */
#ifndef XYCE_GB300_H
#define XYCE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define XG_OK               0
#define XG_ERR_ARG         -1   /* bad argument or size */
#define XG_ERR_CUDA        -2   /* CUDA runtime failure / no sm_103a device */
#define XG_ERR_STATE       -3   /* call out of order (e.g. load before finalize) */
#define XG_ERR_UNSUPPORTED -4   /* device feature not implemented */
#define XG_ERR_NAN         -6   /* DampedNewton nanFail */
#define XG_ERR_SINGULAR    -9   /* DampedNewton linearSolverFailed: pivot breakdown */
#define XG_ERR_TIMEOUT    -10   /* a bounded device-side wait ran out */

/* ---- loadType (Xyce Loader: ALL / LINEAR / NONLINEAR) ------------------ */
#define XG_LOAD_ALL        0
#define XG_LOAD_LINEAR     1
#define XG_LOAD_NONLINEAR  2

/* ---- solver-state flags for xg_update_state ---------------------------- */
#define XG_FLAG_DCOP       1    /* SolverState::dcopFlag (operating point) */
#define XG_FLAG_INITJCT    2    /* SolverState::initJctFlag_ (first DC iteration) */

/* ---- source waveform kinds (N_DEV_SourceData.C) ------------------------ */
#define XG_WAVE_DC    0   /* data: V                                        */
#define XG_WAVE_SIN   1   /* data: V0 VA FREQ TD THETA PHASE                */
#define XG_WAVE_PULSE 2   /* data: V1 V2 TD TR TF PW PER                    */
#define XG_WAVE_PWL   3   /* data: t0 v0 t1 v1 ...                          */

/* ---- diode parameter row (Diode model/instance params, N_DEV_Diode.C:100-345) */
enum {
  XG_DIODE_IS, XG_DIODE_N, XG_DIODE_RS, XG_DIODE_CJO, XG_DIODE_VJ, XG_DIODE_M,
  XG_DIODE_FC, XG_DIODE_TT, XG_DIODE_BV, XG_DIODE_IBV, XG_DIODE_NBV, XG_DIODE_IKF,
  XG_DIODE_ISR, XG_DIODE_NR, XG_DIODE_EG, XG_DIODE_XTI, XG_DIODE_AREA,
  XG_DIODE_BVGIVEN,
  /* sidewall junction: JSW (0 = none), NS and whether it was given (not
   * given: the sidewall current joins the bottom one), CJSW, VJSW (PHP),
   * MJSW, FCS; the instance perimeter PJ */
  XG_DIODE_JSW, XG_DIODE_NS, XG_DIODE_NSGIVEN, XG_DIODE_CJSW, XG_DIODE_VJSW, XG_DIODE_MJSW,
  XG_DIODE_FCS, XG_DIODE_PJ,
  /* temperature: TNOM (model) and TEMP (the device's own: instance TEMP, else
   * the circuit temperature plus DTEMP), both in kelvin; the coefficients
   * TIKF, TBV1/TBV2, TRS1/TRS2 of IKF, BV and RS (N_DEV_Diode.C:1430-1545) */
  XG_DIODE_TNOM, XG_DIODE_TEMP, XG_DIODE_TIKF, XG_DIODE_TBV1, XG_DIODE_TBV2, XG_DIODE_TRS1,
  XG_DIODE_TRS2,
  XG_DIODE_NPARAM
};

/* ---- MOSFET level-1 parameter row (N_DEV_MOSFET1.C:61-331) --------------
 * RD / RS: series drain / source resistance; RSH sheet resistance with the
 * instance's NRD / NRS squares, used where RD / RS is zero
 * (Instance::processParams, N_DEV_MOSFET1.C:410-450). */
enum {
  XG_MOS1_TYPE, XG_MOS1_VTO, XG_MOS1_KP, XG_MOS1_GAMMA, XG_MOS1_PHI, XG_MOS1_LAMBDA,
  XG_MOS1_RD, XG_MOS1_RS, XG_MOS1_CBD, XG_MOS1_CBS, XG_MOS1_IS, XG_MOS1_PB,
  XG_MOS1_CGSO, XG_MOS1_CGDO, XG_MOS1_CGBO, XG_MOS1_CJ, XG_MOS1_MJ, XG_MOS1_CJSW,
  XG_MOS1_MJSW, XG_MOS1_JS, XG_MOS1_TOX, XG_MOS1_LD, XG_MOS1_FC, XG_MOS1_W, XG_MOS1_L,
  XG_MOS1_AD, XG_MOS1_AS, XG_MOS1_PD, XG_MOS1_PS, XG_MOS1_M, XG_MOS1_RSH, XG_MOS1_NRD,
  XG_MOS1_NRS,
  /* TNOM (model) and TEMP (the device's own: instance TEMP, else the circuit
   * temperature plus DTEMP), kelvin (Instance::updateTemperature,
   * N_DEV_MOSFET1.C:3487-3640) */
  XG_MOS1_TNOM, XG_MOS1_TEMP, XG_MOS1_NPARAM
};

/* ---- BSIM4 (Xyce level 54, BSIM 4.8.2) parameter row --------------------
 * Instance (L W AS AD PS PD M) and model parameters, N_DEV_MOSFET_B4.C:337-4840.
 * A NaN entry means "not given": the library derives it as the reference
 * does (Model::processParams4p82_, N_DEV_MOSFET_B4p82.C:7769-8136).
 * Restated scope: the default model selection (capMod 2, mobMod 0, dioMod 1,
 * every other *MOD 0), no binning, no stress, NF 1, RSH 0 (no internal
 * nodes), device temperature TNOM = 27 C. */
enum {
  XG_B4_TYPE, XG_B4_L, XG_B4_W, XG_B4_AS, XG_B4_AD, XG_B4_PS, XG_B4_PD, XG_B4_M, XG_B4_TOXE,
  XG_B4_TOXP, XG_B4_TOXM, XG_B4_DTOX, XG_B4_EPSROX, XG_B4_VTH0, XG_B4_VFB, XG_B4_K1, XG_B4_K2,
  XG_B4_K3, XG_B4_K3B, XG_B4_W0, XG_B4_LPE0, XG_B4_LPEB, XG_B4_DVT0, XG_B4_DVT1, XG_B4_DVT2,
  XG_B4_DVT0W, XG_B4_DVT1W, XG_B4_DVT2W, XG_B4_DSUB, XG_B4_DROUT, XG_B4_NDEP, XG_B4_NSUB,
  XG_B4_NSD, XG_B4_NGATE, XG_B4_PHIN, XG_B4_XJ, XG_B4_XT, XG_B4_VBM, XG_B4_VBX, XG_B4_GAMMA1,
  XG_B4_GAMMA2, XG_B4_CDSC, XG_B4_CDSCB, XG_B4_CDSCD, XG_B4_CIT, XG_B4_NFACTOR, XG_B4_ETA0,
  XG_B4_ETAB, XG_B4_VOFF, XG_B4_VOFFL, XG_B4_MINV, XG_B4_DVTP0, XG_B4_DVTP1, XG_B4_U0,
  XG_B4_UA, XG_B4_UB, XG_B4_UC, XG_B4_UD, XG_B4_UP, XG_B4_LP, XG_B4_VSAT, XG_B4_A0, XG_B4_AGS,
  XG_B4_A1, XG_B4_A2, XG_B4_B0, XG_B4_B1, XG_B4_KETA, XG_B4_DWG, XG_B4_DWB, XG_B4_RDSW,
  XG_B4_RDSWMIN, XG_B4_PRWG, XG_B4_PRWB, XG_B4_WR, XG_B4_PCLM, XG_B4_PDIBLC1, XG_B4_PDIBLC2,
  XG_B4_PDIBLCB, XG_B4_PVAG, XG_B4_DELTA, XG_B4_FPROUT, XG_B4_PDITS, XG_B4_PDITSD,
  XG_B4_PDITSL, XG_B4_PSCBE1, XG_B4_PSCBE2, XG_B4_ALPHA0, XG_B4_ALPHA1, XG_B4_BETA0,
  XG_B4_AGIDL, XG_B4_BGIDL, XG_B4_CGIDL, XG_B4_EGIDL, XG_B4_AGISL, XG_B4_BGISL, XG_B4_CGISL,
  XG_B4_EGISL, XG_B4_CGSO, XG_B4_CGDO, XG_B4_CGBO, XG_B4_CGSL, XG_B4_CGDL, XG_B4_CKAPPAS,
  XG_B4_CKAPPAD, XG_B4_CF, XG_B4_CLC, XG_B4_CLE, XG_B4_DLC, XG_B4_DWC, XG_B4_DWJ, XG_B4_LINT,
  XG_B4_WINT, XG_B4_XL, XG_B4_XW, XG_B4_NOFF, XG_B4_VOFFCV, XG_B4_ACDE, XG_B4_MOIN, XG_B4_ADOS,
  XG_B4_BDOS, XG_B4_XPART, XG_B4_MINVCV, XG_B4_VOFFCVL, XG_B4_CJS, XG_B4_CJD, XG_B4_CJSWS,
  XG_B4_CJSWD, XG_B4_CJSWGS, XG_B4_CJSWGD, XG_B4_MJS, XG_B4_MJD, XG_B4_MJSWS, XG_B4_MJSWD,
  XG_B4_MJSWGS, XG_B4_MJSWGD, XG_B4_PBS, XG_B4_PBD, XG_B4_PBSWS, XG_B4_PBSWD, XG_B4_PBSWGS,
  XG_B4_PBSWGD, XG_B4_JSS, XG_B4_JSD, XG_B4_JSWS, XG_B4_JSWD, XG_B4_JSWGS, XG_B4_JSWGD,
  XG_B4_NJS, XG_B4_NJD, XG_B4_IJTHSFWD, XG_B4_IJTHDFWD, XG_B4_DMCG, XG_B4_DMCI, XG_B4_DMDG,
  XG_B4_DMCGT, XG_B4_NPARAM
};

typedef struct xg_ctx xg_ctx;

/* ---- context ------------------------------------------------------------ */
/* Replaces Simulator::doAllocations_ for this path (N_CIR_Xyce.C:515-566):
 * binds the calling thread to `device` and creates the context's stream. */
int xg_create(xg_ctx **out, int device);
int xg_destroy(xg_ctx *ctx);
/* Last error message of the context (never NULL). */
const char *xg_error_string(const xg_ctx *ctx);
/* cudaStream_t of the context, as void*. */
void *xg_get_stream(xg_ctx *ctx);
int xg_synchronize(xg_ctx *ctx);

/* ---- topology upload (host arrays) ---------------------------------------
 * Replaces Topology::registerLIDswithDevs + Builder::generateGraphs
 * (N_CIR_Xyce.C:657-696, N_LAS_Builder.C:384-418).  n_circuits independent
 * circuits occupy contiguous unknown ranges [offsets[c], offsets[c+1]).
 * Node index -1 is ground.  Each xg_add_* call checks all n items (node
 * ranges, values, cards) before it appends any: a call that fails leaves the
 * topology as it was. */
int xg_set_unknowns(xg_ctx *ctx, int n_unknowns, int n_circuits, const int *offsets);
/* Resistor::Instance (N_DEV_Resistor.C), value in ohms. */
int xg_add_resistors(xg_ctx *ctx, int n, const int *pos, const int *neg, const double *r);
/* Capacitor::Instance (N_DEV_Capacitor.C), value in farads. */
int xg_add_capacitors(xg_ctx *ctx, int n, const int *pos, const int *neg, const double *c);
/* Vsrc::Instance (N_DEV_Vsrc.C): branch = unknown of the branch current.
 * Waveform k is kind[k] with data[off[k] .. off[k+1]). */
int xg_add_vsources(xg_ctx *ctx, int n, const int *pos, const int *neg, const int *branch,
                    const int *kind, const int *off, const double *data);
/* Inductor::Instance (N_DEV_Inductor.C:540-650), without IC: branch is the
 * unknown carrying its current (as a voltage source's); l in henry.  The
 * stamps are constant and load with the linear part. */
int xg_add_inductors(xg_ctx *ctx, int n, const int *pos, const int *neg, const int *branch,
                     const double *l);
/* ISRC::Instance (N_DEV_ISRC.C). */
int xg_add_isources(xg_ctx *ctx, int n, const int *pos, const int *neg,
                    const int *kind, const int *off, const double *data);
/* Diode::Instance level 1 (N_DEV_Diode.C); pri = internal node (== pos when RS = 0);
 * params is n x XG_DIODE_NPARAM row-major. */
int xg_add_diodes(xg_ctx *ctx, int n, const int *pos, const int *neg, const int *pri,
                  const double *params);
/* MOSFET1::Instance (N_DEV_MOSFET1.C); params n x XG_MOS1_NPARAM row-major.
 * Rows with a series drain/source resistance need the internal nodes:
 * XG_ERR_ARG here, use xg_add_mosfet1_rs. */
int xg_add_mosfet1(xg_ctx *ctx, int n, const int *d, const int *g, const int *s,
                   const int *b, const double *params);
/* The same with the drain' / source' internal nodes (li_DrainPrime /
 * li_SourcePrime, N_DEV_MOSFET1.C:1437-1445): dp[k] must differ from d[k]
 * exactly when the drain conductance (RD, or RSH * NRD) is nonzero, sp[k]
 * likewise.  The device equations act on (dp, g, sp, b); drainConductance *
 * M joins d to dp and sourceConductance * M s to sp.  These constant
 * conductances load with the linear part (loadType XG_LOAD_LINEAR), where
 * the reference loads them with the device: the sum of the two parts is the
 * same. */
int xg_add_mosfet1_rs(xg_ctx *ctx, int n, const int *d, const int *g, const int *s,
                      const int *b, const int *dp, const int *sp, const double *params);
/* MOSFET_B4::Instance (N_DEV_MOSFET_B4.C); params n x XG_B4_NPARAM row-major.
 * A card outside the restated scope is XG_ERR_UNSUPPORTED. */
int xg_add_bsim4(xg_ctx *ctx, int n, const int *d, const int *g, const int *s,
                 const int *b, const double *params);
/* Builds the CSR pattern, the stamp map, device-resident SoA instance
 * arrays and the symbolic structures (DeviceMgr::initializeAll + setupPointers,
 * N_CIR_Xyce.C:698-717, N_DEV_Diode.C:778-800).  XG_ERR_ARG when a device or
 * source connects unknowns of two circuits, or two voltage sources share a
 * branch unknown. */
int xg_finalize(xg_ctx *ctx);

int xg_get_sizes(xg_ctx *ctx, int *n_unknowns, int *nnz, int *n_state, int *n_store);
/* Host copies of the CSR pattern: row_ptr[n+1], col_idx[nnz]. */
int xg_get_pattern(xg_ctx *ctx, int *row_ptr, int *col_idx);

/* ---- loader (DEVICE pointers) --------------------------------------------- */
/* DeviceMgr::updateSources (N_DEV_DeviceMgr.C:4900): source values at `time`. */
int xg_update_sources(xg_ctx *ctx, double time);
/* DeviceMgr::updateState (N_DEV_DeviceMgr.C:3857-3936): evaluates every
 * nonlinear device at next_sol, writes next_sta / next_sto, and keeps the
 * per-instance stamp values for the two load calls that follow.
 * History selection follows the reference: newton_iter == 0 reads curr_sto,
 * later iterations read next_sto as left by the previous call.  flags:
 * XG_FLAG_*.  load_type (XG_LOAD_*) selects the devices as
 * DeviceMaster::updateState does (N_DEV_DeviceMaster.h:688-700): ALL and
 * NONLINEAR evaluate the nonlinear devices; LINEAR has nothing to evaluate
 * (the linear devices are the constant linear part of the matrix). */
int xg_update_state(xg_ctx *ctx, const double *next_sol, const double *curr_sta,
                    const double *curr_sto, double *next_sta, double *next_sto,
                    int newton_iter, int flags, int load_type);
/* DeviceMgr::loadDAEVectors (N_DEV_DeviceMgr.C:4156-4284): ADDS the device
 * contributions into Q, F, B, dFdxdVp, dQdxdVp (length n).  As in the
 * reference, the caller zeroes them first (N_LOA_NonlinearEquationLoader.C:385-390). */
int xg_load_dae_vectors(xg_ctx *ctx, const double *next_sol, double *Q, double *F,
                        double *B, double *dFdxdVp, double *dQdxdVp, int load_type);
/* DeviceMgr::loadDAEMatrices (N_DEV_DeviceMgr.C:3980-4115): ADDS into the
 * dQdx and dFdx CSR value arrays (length nnz); caller zeroes first
 * (N_LOA_NonlinearEquationLoader.C:525-526). */
int xg_load_dae_matrices(xg_ctx *ctx, double *dQdx, double *dFdx, int load_type);

/* ---- sparse direct solve on the frozen pattern ----------------------------
 * AmesosSolver::doSolve with KLU (N_LAS_AmesosSolver.C:216-440): symbolic
 * analysis once (row matching from the values, fill-reducing order,
 * level schedule), numeric refactorization with frozen pivots on every call.
 * xg_lu_factor returns XG_ERR_SINGULAR when a pivot breaks down; calling
 * xg_lu_analyze again with the current values re-pivots. */
int xg_lu_analyze(xg_ctx *ctx, const double *vals);
int xg_lu_factor(xg_ctx *ctx, const double *vals);
int xg_lu_solve(xg_ctx *ctx, const double *rhs, double *x);
/* Allocation-free variant of xg_lu_solve.  No counterpart in the reference:
 * Xyce's solvers allocate their own workspace.  It is for callers that must
 * not call cudaMalloc (device memory fully owned by another allocator, or a
 * loop that must not block on the CUDA allocator): the solve's scratch vector
 * is a static device array of XG_NOALLOC_MAX_N doubles (2 MiB, held by every
 * GPU that loads the library until exit) instead of allocated memory.  Same
 * inputs and outputs as xg_lu_solve (device pointers; the factorization comes
 * from xg_lu_factor on ctx).  Returns XG_ERR_ARG when the system has more than
 * XG_NOALLOC_MAX_N unknowns.  The first call on a device looks the scratch
 * address up and keeps it for the life of the process; make that call
 * before any stream capture, and do not reset the device (cudaDeviceReset)
 * while the library is in use: the kept address belongs to the context it
 * was looked up in.  Every call shares the one scratch array: calls that
 * overlap on the GPU race. */
#define XG_NOALLOC_MAX_N 262144
int xg_lu_solve_noalloc(xg_ctx *ctx, const double *rhs, double *x);

/* Precision of the factors used by xg_lu_factor / xg_lu_solve and by the
 * transient driver.  XG_PREC_FP64 (default): FP64 factors, one solve.
 * XG_PREC_FP32_IR: FP32 factors, then n_refine steps of FP64 iterative
 * refinement per solve (r = b - A x with the FP64 values last passed to
 * xg_lu_factor, x += (LU)^-1 r) — the precedent is Xyce's IRSolver
 * (src/LinearAlgebraServicesPKG/N_LAS_IRSolver.C:428-560), which refines
 * with a stale factorization.  Those values must stay unchanged until the
 * solves that use them are done.  Takes effect at the next xg_lu_analyze (or
 * transient); not allowed while a transient is in progress. */
#define XG_PREC_FP64     0
#define XG_PREC_FP32_IR  1
int xg_lu_set_precision(xg_ctx *ctx, int precision, int n_refine);

/* Statistics of the current analysis: nnz(L+U), factor/solve level counts. */
int xg_lu_info(xg_ctx *ctx, long long *nnz_lu, int *factor_levels, int *lsolve_levels,
               int *usolve_levels);

/* Schedule the current analysis chose: ordering of the core (XG_ORDER_*),
 * how the top of the factorization runs and how the tops of the solves run
 * (XG_TOP_*).  No reference counterpart (KLU's schedule is serial). */
#define XG_ORDER_ND          0   /* nested dissection                        */
#define XG_ORDER_MIN_DEGREE  1   /* approximate minimum degree               */
#define XG_TOP_NONE          0   /* no top: groups cover the matrix          */
#define XG_TOP_ONE_CTA       1   /* one CTA walks the top                    */
#define XG_TOP_LEVELS        2   /* a launch (pair) per level on all SMs     */
int xg_lu_schedule_info(xg_ctx *ctx, int *ordering, int *factor_top, int *solve_top);

/* Override the automatic choices (-1 keeps a choice automatic): the ordering
 * (XG_ORDER_*) and the factor / solve top schedules (XG_TOP_ONE_CTA or
 * XG_TOP_LEVELS; a top below 64 columns always runs in one CTA).  Applies
 * from the next analysis; not allowed while a transient is in progress. */
int xg_lu_set_schedule(xg_ctx *ctx, int ordering, int factor_top, int solve_top);

/* Frozen-pivot acceptance of the refactorization (default 1e-2): a pivot
 * below tol times the largest entry of its updated column is a breakdown
 * (xg_lu_factor returns XG_ERR_SINGULAR; in a transient the circuit parks
 * its Newton iteration, the host re-pivots that circuit alone from the
 * parked Jacobian — every other circuit keeps its pivots, factors and
 * results — and the iteration resumes).  KLU re-pivots on every
 * factorization (N_LAS_AmesosSolver.C:315-318); this is the threshold at
 * which the frozen pivots are given up.  Not allowed while a transient is in
 * progress. */
int xg_lu_set_pivot_tolerance(xg_ctx *ctx, double tol);

/* Factor reuse in the transient.  on = 1 (default): a circuit without
 * nonlinear devices whose Jacobian coefficients (OneStep's qscale / fscale,
 * the operating point's gmin shunt) equal those of its last factorization
 * under the same analysis has the same Jacobian bit for bit; it skips the
 * refactorization and solves with the factors it has — the results are
 * identical.  The reference's IRSolver (N_LAS_IRSolver.C:428-560) reuses
 * stale factors with iterative refinement instead; this reuse is exact.
 * Not allowed while a transient is in progress. */
int xg_lu_set_reuse(xg_ctx *ctx, int on);

/* Launch shapes of the LU sweeps.  XG_TUNE_TIMED (default): after each
 * analysis, candidate shapes — the factorization with and without its
 * update metadata staged in shared memory, at 64..512 threads per CTA; the
 * L and U solves at 64..512 threads — are launched on the matrix the
 * analysis was computed from (L2 flushed before each timed launch) and the
 * fastest are kept; choices are cached per analysis for the life of the
 * process.  XG_TUNE_MODEL: the analysis' closed-form estimates.  Every
 * candidate computes identical results; only the time differs.  Applies
 * from the next analysis; not allowed while a transient is in progress.
 * XG_TUNE_FIXED is set by xg_lu_set_shapes.  No reference counterpart
 * (KLU's factorization is serial). */
#define XG_TUNE_MODEL 0
#define XG_TUNE_TIMED 1
#define XG_TUNE_FIXED 2
int xg_lu_set_tuning(xg_ctx *ctx, int mode);
/* Fixed launch shapes (XG_TUNE_FIXED) from the next analysis: threads per
 * CTA of the factorization, the L solve and the U solve (64, 128, 256 or
 * 512; 0 keeps the analysis' choice) and the factorization's update
 * metadata staged (1), not staged (0) or as the analysis chose (-1;
 * staging needs metadata the analysis laid out, else it stays off). */
int xg_lu_set_shapes(xg_ctx *ctx, int factor_threads, int factor_meta, int lsolve_threads, int usolve_threads);
typedef struct xg_lu_tuning {
  int mode;                 /* XG_TUNE_* of the current analysis */
  int from_cache;           /* 1: timed earlier for the same analysis, in this process */
  int factor_threads, factor_meta, lsolve_threads, usolve_threads;  /* in use */
  int model_factor_threads, model_factor_meta, model_lsolve_threads, model_usolve_threads;
  double factor_us, solve_us;              /* timed: the chosen shapes (one factor, one L+U solve) */
  double model_factor_us, model_solve_us;  /* timed: the closed-form shapes (0 when not timed) */
} xg_lu_tuning;
int xg_lu_tuning_info(xg_ctx *ctx, xg_lu_tuning *out);

/* Host-only analysis of a CSR pattern with values (no context, no device):
 * the numbers xg_lu_info / xg_lu_schedule_info report after xg_lu_analyze —
 * nnz(L+U), the ordering chosen (or forced: ordering = XG_ORDER_*, -1 =
 * automatic), the dependency-closed groups and the top size of the factor
 * schedule.  The counterpart of klu_analyze's statistics. */
int xg_lu_analyze_pattern(int n, const int *row_ptr, const int *col_idx, const double *vals, int ordering,
                          long long *nnz_lu, int *ordering_out, int *n_groups, int *n_top);

/* ---- Newton + time integration driver --------------------------------------
 * Transient::doRun (N_ANP_Transient.C:739-772, 1184-1410, 3262-3325): DC
 * operating point, then OneStep (backward Euler start, trapezoid) with
 * DampedNewton on every step, all device-resident.  Each circuit of a batch
 * runs its own step-size control. */
typedef struct xg_tran_params {
  double tstart, tstop, hmax, hmin;
  double reltol, abstol;                       /* .OPTIONS TIMEINT */
  double nl_reltol, nl_abstol, nl_deltaxtol, nl_rhstol, nl_smallupdatetol;
  int nl_maxstep;                              /* .OPTIONS NONLIN-TRAN */
  int max_steps;                               /* stop after this many accepted steps (0 = none) */
  int max_order;                               /* 1 = backward Euler, 2 = trapezoid / BDF2 */
  int method;                                  /* XG_METHOD_*: .OPTIONS TIMEINT METHOD (0 = ONESTEP) */
} xg_tran_params;

/* Integration methods, numbered as the reference's methodsEnum
 * (src/TimeIntegrationPKG/N_TIA_fwd.h:56-58): OneStep (trapezoid, the
 * default) and Gear12 (BDF1/2, N_TIA_Gear12.C). */
#define XG_METHOD_ONESTEP 7
#define XG_METHOD_GEAR    8

typedef struct xg_tran_stats {
  long long accepted, rejected, newton_iters, newton_fail, lte_fail, dcop_iters;
  long long ticks, device_evals;               /* Newton iterations launched; instance evaluations */
  int status;                                  /* 0 ok, else first failing circuit's code */
  int n_analyze;                               /* symbolic (re)analyses performed */
  double t_final_min, t_final_max;
  double seconds;                              /* wall time of the run */
  int kernels_per_tick;                        /* kernel launches of one tick (its CUDA graph) */
  int form;                                    /* XG_FORM_TICK_GRAPH or XG_FORM_RESIDENT: how it advanced */
  long long kernel_launches;                   /* kernels launched while advancing */
  long long circuit_ticks;                     /* resident form: Newton iterations summed over circuits */
  long long factor_skips;                      /* refactorizations skipped (xg_lu_set_reuse) */
  int resident_threads;                        /* resident form: CTA size of its last launch (0: none) */
  int option;                                  /* advancing option the timed trials chose (-1: not yet):
                                                  0..4 resident with 32/64/128/256/512-thread CTAs,
                                                  5 tick graph */
  double option_us_per_iter[6];                /* device time per circuit Newton iteration of each timed
                                                  option, microseconds (0: not timed) */
  long long tail_launches;                     /* resident launches that finished tick-graph advances
                                                  (xg_tran_set_tail) */
} xg_tran_stats;

/* How a transient advances.  XG_FORM_TICK_GRAPH: a tick (one Newton
 * iteration of every active circuit, 15 kernels) is a captured CUDA graph,
 * replayed in batches between host synchronizations.  XG_FORM_RESIDENT:
 * one kernel runs every stage of every tick for a whole batch — each CTA
 * takes a circuit and iterates its ticks until the circuit pauses,
 * finishes, fails or parks on a pivot breakdown, then takes the next —
 * so a circuit that has finished costs nothing and nothing waits on a
 * grid-wide barrier.  Both compute the same bits.  The resident form needs
 * a batch of at least 64 circuits of at most 2,048 unknowns each, MOSFET-1
 * and diode devices only, FP64 factors, the polynomial predictor and an LU
 * analysis without a top.  XG_FORM_AUTO (default): when the batch admits
 * the resident form, the first advances after the operating point time
 * the options (the tick graph over one advance, then the resident kernel,
 * one launch per CTA size: 128 and 256 threads, then on towards 512 or
 * down to 64 and 32 while the size keeps getting faster) and the rest of
 * the run keeps the one with the shortest device time per circuit Newton
 * iteration; XG_FORM_RESIDENT times the CTA sizes only.  No reference counterpart (Xyce runs one circuit per process).
 * Not allowed while a transient is in progress. */
#define XG_FORM_AUTO        0
#define XG_FORM_TICK_GRAPH  1
#define XG_FORM_RESIDENT    2
int xg_tran_set_form(xg_ctx *ctx, int form);

/* The tail of an advance under XG_FORM_AUTO when the trials kept the tick
 * graph: once at most active_fraction of the batch's circuits are still
 * running (checked between batches of ticks), one resident-kernel launch
 * (256-thread CTAs) finishes them, each circuit at its own pace, instead of
 * more full-batch tick graphs.  The same bits either way.  Applies where
 * the resident form does; 0 turns it off; the default is 0.25.  No
 * reference counterpart. */
int xg_tran_set_tail(xg_ctx *ctx, double active_fraction);

/* Runs the transient.  probes: global unknown indices to record; every
 * circuit records, at each accepted point, its time and the values of the
 * probes inside it (in the order given), up to cap points per circuit.
 * Host outputs: counts[n_circuits], times[n_circuits*cap],
 * values[n_circuits*cap*pmax] where pmax = the largest number of probes in one circuit.
 * Any output pointer may be NULL when cap == 0. */
int xg_transient(xg_ctx *ctx, const xg_tran_params *p, int n_probe, const int *probes,
                 int cap, int *counts, double *times, double *values, xg_tran_stats *stats);
/* The same run in stages, for callers that stream results or time windows:
 * xg_tran_start computes the operating point and the first analysis;
 * xg_tran_advance runs until every circuit has accepted n_steps more steps
 * (n_steps <= 0: to tstop); xg_tran_results copies outputs and statistics so
 * far; xg_tran_end releases the run.  xg_transient = start + advance + results + end. */
int xg_tran_start(xg_ctx *ctx, const xg_tran_params *p, int n_probe, const int *probes, int cap);
int xg_tran_advance(xg_ctx *ctx, int n_steps);
int xg_tran_results(xg_ctx *ctx, int *counts, double *times, double *values, xg_tran_stats *stats);
int xg_tran_end(xg_ctx *ctx);

/* Predictor values of the recorded points (same layout as xg_tran_results'
 * values): at each accepted transient point, the Newton initial guess that
 * step started from — the training target of the learned predictor is the
 * accepted solution minus this guess. */
int xg_tran_predictors(xg_ctx *ctx, double *pred_values);
/* Per-stage device time of ticks of a transient in progress (a tick is one
 * Newton iteration of every active circuit).  n_steps > 0 first opens a
 * window of n_steps more accepted steps per circuit, as xg_tran_advance
 * does.  Runs n_ticks ticks with the tick's kernels launched one stage at a
 * time, CUDA events between stages, and ADDS each stage's milliseconds into
 * stage_ms[XG_STAGE_*]; the run then continues as it would have.  evals
 * (may be NULL) receives, summed over the ticks, the instances the
 * MOSFET-1, BSIM4 and diode stages evaluated (evals[0..2]) and the active
 * circuits (evals[3]).  For
 * profiling: an advance replays the tick as one CUDA graph.  No reference
 * counterpart (Xyce prints its load and solve times per run). */
enum {
  XG_STAGE_SOURCES, XG_STAGE_MOS1, XG_STAGE_BSIM4, XG_STAGE_DIODE, XG_STAGE_ASSEMBLE,
  XG_STAGE_NEWTON, XG_STAGE_LU_FACTOR, XG_STAGE_LU_SOLVE, XG_STAGE_UPDATE, XG_STAGE_STEP,
  XG_STAGE_HISTORY, XG_STAGE_COMMIT, XG_STAGE_COUNT
};
int xg_tran_profile(xg_ctx *ctx, int n_steps, int n_ticks, double *stage_ms, long long *evals);
/* Where the circuit-resident tick (XG_FORM_RESIDENT) spends its time, for a
 * transient in progress whose analysis admits that form.  n_steps > 0 first
 * opens a window as xg_tran_advance does; one launch of the resident kernel
 * with CTAs of `threads` (32, 64 or 128) threads then runs every active
 * circuit with a clock in each CTA, and stage_cycles[XG_RSTAGE_*] receives
 * the SM cycles the CTAs spent in each stage of their ticks (barrier waits
 * included), summed over CTAs and ticks.  circuit_ticks (may be NULL)
 * receives the Newton iterations that launch ran, summed over circuits.
 * The window then finishes as xg_tran_advance would finish it.  No
 * reference counterpart. */
enum {
  XG_RSTAGE_SOURCES, XG_RSTAGE_DEVICES, XG_RSTAGE_LONG_GATHERS, XG_RSTAGE_ASSEMBLE, XG_RSTAGE_NEWTON,
  XG_RSTAGE_FACTOR, XG_RSTAGE_SOLVE, XG_RSTAGE_UPDATE, XG_RSTAGE_STEP, XG_RSTAGE_COMMIT, XG_RSTAGE_COUNT
};
int xg_tran_profile_resident(xg_ctx *ctx, int n_steps, int threads, double *stage_cycles,
                             long long *circuit_ticks);

/* Integration order of the recorded points (layout of xg_tran_results'
 * times, n_circuits x cap): 0 for the operating point, else the order the
 * accepted step was integrated with (1 backward Euler / BDF1, 2 trapezoid /
 * BDF2).  Together with the times it is the accepted step sequence, which
 * another integrator can replay to compare solutions at identical points.
 * No reference counterpart: Xyce keeps the order in
 * WorkingIntegrationMethod and does not output it. */
int xg_tran_orders(xg_ctx *ctx, int *orders);
/* Steps and Newton iterations taken with the learned and with the
 * polynomial predictor in the current run (learned predictor mode). */
int xg_tran_predictor_stats(xg_ctx *ctx, long long *learned_steps, long long *learned_iters,
                            long long *poly_steps, long long *poly_iters);

/* ---- learned predictor ------------------------------------------------------
 * No counterpart in the reference: a per-node MLP (5 -> 64 -> 64 -> 1, tanh,
 * BF16 weights on the tensor cores, FP32 accumulation) corrects the
 * polynomial predictor of WorkingIntegrationMethod::obtainPredictor
 * (src/TimeIntegrationPKG/N_TIA_WorkingIntegrationMethod.C:176) at the start
 * of each step attempt.  With d1 = x_n - x_{n-1}, d2 = x_{n-1} - x_{n-2},
 * d3 = x_{n-2} - x_{n-3} and s = |d1| + |d2| + |d3| + 1e-9 V, the features of
 * node unknown r are d1/s, d2/s, d3/s, x_n, log(h_{n+1} / h_n), standardized
 * as (f - shift) * scale, and Newton starts from the polynomial guess plus
 * s * (out_shift + out_scale * MLP); nodes with s < 1e-5 V keep the
 * polynomial guess.  The polynomial guess stays the
 * predictor of the error estimate and step control.
 * Newton to the unchanged tolerances still decides every step; a circuit
 * whose learned step needs more Newton iterations than its polynomial steps
 * falls back to the polynomial predictor for 16 steps.
 * theta: XG_MLP_NPARAM floats, W1[5][64] | b1[64] | W2[64][64] (in x out) |
 * b2[64] | w3[64] | b3.  norm: in_shift[5], in_scale[5], out_shift, out_scale. */
#define XG_MLP_NPARAM 4609
#define XG_MLP_NNORM  12
#define XG_PRED_POLY     0
#define XG_PRED_LEARNED  1
int xg_set_predictor(xg_ctx *ctx, int mode);
int xg_mlp_set(xg_ctx *ctx, const float *theta, const float *norm);
int xg_mlp_get(xg_ctx *ctx, float *theta, float *norm);
/* Training on the GPU (own forward / backward kernels, Adam): X is n x 5
 * standardized features and Y n standardized targets, DEVICE pointers;
 * loss_hist (host, iters) receives 0.5 mean squared error per iteration. */
int xg_mlp_train(xg_ctx *ctx, const float *X, const float *Y, int n, int iters, float lr,
                 float *loss_hist);
/* Loss and gradient of the current weights on (X, Y) (host outputs). */
int xg_mlp_grad(xg_ctx *ctx, const float *X, const float *Y, int n, float *grad_host,
                float *loss_host);
/* out[r] = MLP(X[r]) in standardized units (DEVICE pointers). */
int xg_mlp_forward(xg_ctx *ctx, const float *X, int n, float *out);

/* ---- Newton solve ---------------------------------------------------------
 * Nonlinear::DampedNewton::solve with full Newton steps
 * (src/NonlinearSolverPKG/N_NLS_DampedNewton.C:362-520; converged_ :1191-1396;
 * updateWeights_ :297-340), every circuit of the context at once, for a
 * caller that keeps its own time integrator: it sets the coefficients of
 * the nonlinear system and calls this once per step attempt.  The residual
 * and Jacobian are those OneStep::obtainResidual / obtainJacobian form
 * (N_TIA_OneStep.C:219-290, 469-500):
 *   RHS = -[qscale (Q(x) - qhist0) + fscale (F(x) - B(time)) + hscale qhist2]
 *         + qscale dQdxdVp + fscale dFdxdVp
 *   J   =  qscale dQdx + fscale dFdx
 * (operating point: qscale = hscale = 0, fscale = 1).  x (DEVICE, length n)
 * is the initial guess on entry and the last iterate on return; x_curr
 * (DEVICE, may be NULL = zeros) is the accepted solution of the weights
 * reltol * max(|x|, |x_curr|) + abstol; qhist0 / qhist2 (DEVICE) may be NULL
 * when their coefficient is 0.  curr_sta / curr_sto are the accepted device
 * state and store, next_sta / next_sto receive the iterate's (as for
 * xg_update_state).  flags: XG_FLAG_DCOP selects the operating-point rules
 * (weights every iteration, device convergence enforced), XG_FLAG_INITJCT
 * the junction initialization of the first iteration.
 * Outputs (HOST, n_circuits each): status[c] = DampedNewton's return code of
 * circuit c — 2 converged, 1 residual norm below machine epsilon, 4 small
 * update, -1 too many steps, -2 diverging, -3 stalled, -6 NaN, -9 linear
 * solve failed; iters[c] (may be NULL) = its Newton iterations.  The return
 * value is XG_OK when every circuit's solve ran to one of those codes, else
 * an XG_ERR_* (arguments, CUDA, repeated pivot breakdown).  Not allowed
 * while a transient is in progress. */
typedef struct xg_newton_params {
  double reltol, abstol, deltaxtol, rhstol, smallupdatetol;  /* .OPTIONS NONLIN(-TRAN) */
  int maxstep;
} xg_newton_params;
int xg_newton_solve(xg_ctx *ctx, const xg_newton_params *p, double time, double qscale,
                    double fscale, double hscale, const double *qhist0, const double *qhist2,
                    double *x, const double *x_curr, const double *curr_sta, const double *curr_sto,
                    double *next_sta, double *next_sto, int flags, int *status, int *iters);

/* Operating point only; x_host receives the n solution values. */
int xg_dcop(xg_ctx *ctx, double *x_host, int *iters);

/* Version of the library (major*10000 + minor*100 + patch). */
int xg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* XYCE_GB300_H */
