/*
 * oracle.h — CPU FP64 restatement of Xyce's transient Newton hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation in xyce_gb300/: only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / reference arm may load it.  The product never
 * links, imports or calls it.
 *
 * What it restates (file:line within the Xyce source tree):
 *   - SourceData SIN/PULSE/PWL       src/DeviceModelPKG/Core/N_DEV_SourceData.C:475,1168,1770
 *   - pnjlim/fetlim/limvds/qmeyer    src/DeviceModelPKG/Core/N_DEV_DeviceSupport.C:161-745
 *   - Resistor/Capacitor/Vsrc/ISRC   src/DeviceModelPKG/OpenModels/N_DEV_{Resistor,Capacitor,Vsrc,ISRC}.C
 *   - Diode level 1                  src/DeviceModelPKG/OpenModels/N_DEV_Diode.C:1072-1950,2040-2237
 *   - MOSFET level 1                 src/DeviceModelPKG/OpenModels/N_DEV_MOSFET1.C:2689-3730,4241-4876
 *   - OneStep (BE/trapezoid)         src/TimeIntegrationPKG/N_TIA_OneStep.C:135-500,1390-1640,1684-2240
 *   - DataStore error weights/WRMS   src/TimeIntegrationPKG/N_TIA_DataStore.C:1304-1550,1737
 *   - StepErrorControl accept test   src/TimeIntegrationPKG/N_TIA_StepErrorControl.C:458-575
 *   - DampedNewton                   src/NonlinearSolverPKG/N_NLS_DampedNewton.C:297-520,1147-1396
 *   - IRSolver factor reuse          src/LinearAlgebraServicesPKG/N_LAS_IRSolver.C:428-560
 *   - Sparse LU: Gilbert-Peierls left-looking LU with threshold partial
 *     pivoting (the algorithm of KLU, which Xyce calls through Amesos in
 *     src/LinearAlgebraServicesPKG/N_LAS_AmesosSolver.C:309-396).  It is
 *     cross-checked against Kundert Sparse 1.3 compiled from the reference's
 *     own sources (src/LinearAlgebraServicesPKG/ksparse) by oracle/Makefile.
 *
 * Parity pinning: the Xyce regression waveforms are not in the reference
 * tree and Xyce cannot be built here (Trilinos absent), so the device
 * models are pinned by finite-difference Jacobian checks (the reference's
 * TESTJAC idea, src/DeviceModelPKG/Core/N_DEV_NumericalJacobian.C:154) and
 * by analytic circuits; the linear solve is pinned by ksparse.
 */
#ifndef XG_ORACLE_H
#define XG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* Waveform kinds shared with the GPU library's C-ABI. */
enum { ORC_WAVE_DC = 0, ORC_WAVE_SIN = 1, ORC_WAVE_PULSE = 2, ORC_WAVE_PWL = 3 };

orc_ctx *orc_create(int n_unknowns, int n_circuits, const int *circuit_offsets);
void orc_destroy(orc_ctx *c);
int orc_add_resistors(orc_ctx *c, int n, const int *pos, const int *neg, const double *r);
int orc_add_capacitors(orc_ctx *c, int n, const int *pos, const int *neg, const double *cap);
int orc_add_vsources(orc_ctx *c, int n, const int *pos, const int *neg, const int *branch,
                     const int *kind, const int *off, const double *data);
/* Inductor (N_DEV_Inductor.C): branch b carries the current; l in henry. */
int orc_add_inductors(orc_ctx *c, int n, const int *p, const int *m, const int *b, const double *l);
int orc_add_isources(orc_ctx *c, int n, const int *pos, const int *neg,
                     const int *kind, const int *off, const double *data);
int orc_add_diodes(orc_ctx *c, int n, const int *pos, const int *neg, const int *pri,
                   const double *params);
/* dp / sp: the drain' / source' nodes (== d / s without series resistance). */
int orc_add_mosfet1(orc_ctx *c, int n, const int *d, const int *g, const int *s, const int *b,
                    const int *dp, const int *sp, const double *params);
/* BSIM 4.8.2 (level 54), restated scope in bsim4.h; params n x b4::P_COUNT
 * (NaN = not given).  Returns -4 for a card outside that scope. */
int orc_add_bsim4(orc_ctx *c, int n, const int *d, const int *g, const int *s, const int *b,
                  const double *params);
int orc_finalize(orc_ctx *c);

int orc_sizes(orc_ctx *c, int *n_unknowns, int *nnz, int *n_state, int *n_store);
int orc_pattern(orc_ctx *c, int *row_ptr, int *col_idx);

/* One device load (updateState + loadDAEVectors + loadDAEMatrices) at
 * x_next, with the reference's zeroed-output precondition done here.
 * flags: bit0 dcop, bit1 initJct, newton_iter selects limiter history. */
int orc_load(orc_ctx *c, double time, const double *x_next, const double *sta_curr,
             const double *sto_curr, const double *sto_next_in, int newton_iter, int flags,
             double *sta_next, double *sto_next, double *F, double *Q, double *B,
             double *dFdxdVp, double *dQdxdVp, double *dFdx, double *dQdx);

/* Sparse LU solve of A x = b on the context's pattern (for solver checks). */
int orc_lu_solve(orc_ctx *c, const double *vals, const double *b, double *x);

typedef struct orc_tran_params {
  double tstart, tstop, hmax, hmin;
  double reltol, abstol;            /* TIMEINT RELTOL/ABSTOL */
  double nl_reltol, nl_abstol, nl_deltaxtol, nl_rhstol, nl_smallupdatetol;
  int nl_maxstep;
  int max_steps;                    /* safety cap on accepted steps, 0 = none */
  int max_order;                    /* 1 = BE only, 2 = trapezoid / BDF2 */
  int method;                       /* 7 = OneStep (trapezoid), 8 = Gear12 (BDF2); 0 = 7 */
} orc_tran_params;

typedef struct orc_tran_stats {
  int accepted, rejected, newton_iters, newton_fail, lte_fail, dcop_iters, status;
  double t_final;
  double time_load, time_solve, time_total;
} orc_tran_stats;

/* Transient run from a DC operating point.  Output: times[] and
 * values[n_probe x cap] at each accepted point (row-major by point). */
int orc_transient(orc_ctx *c, const orc_tran_params *p, int n_probe, const int *probes,
                  int cap, double *times, double *values, int *n_out, orc_tran_stats *st);

/* One DampedNewton solve with caller-given coefficients and histories:
 * RHS = -[qscale (Q - qhist0) + fscale (F - B) + hscale qhist2] + limiter
 * terms, J = qscale dQdx + fscale dFdx (qhist0 / qhist2 may be NULL = zeros);
 * weights reltol * max(|x|, |x_curr|) + abstol (x_curr NULL = zeros).
 * flags: bit0 operating-point rules, bit1 initJct.  x: initial guess in,
 * last iterate out.  Returns DampedNewton's status; *iters its iterations. */
int orc_newton(orc_ctx *c, double time, double qscale, double fscale, double hscale,
               const double *qhist0, const double *qhist2, double *x, const double *x_curr,
               const double *sta_curr, const double *sto_curr, double *sta_next, double *sto_next,
               double reltol, double abstol, double deltaxtol, double rhstol, double smallupdatetol,
               int maxstep, int flags, int *iters);

/* Operating point only (x out, length n_unknowns). */
int orc_dcop(orc_ctx *c, double *x, int *iters);

/* Elimination order of the sparse LU, as KLU's symbolic analysis fixes one
 * (AMD on the pattern of A + A^T) before its numeric factorizations:
 * perm[k] = the unknown eliminated k-th (a permutation of 0..n_unknowns-1),
 * the LU then factors P A P^T with the same threshold pivoting; n = 0
 * restores the natural order.  Returns -1 for anything but a permutation. */
int orc_set_order(orc_ctx *c, const int *perm, int n);

/* Linear solver of the Newton iterations (.OPTIONS LINSOL TYPE): 0 refactors
 * on every iteration (KLU), 1 is IRSolver (reuse of earlier factors with
 * iterative refinement, src/LinearAlgebraServicesPKG/N_LAS_IRSolver.C:428-560)
 * with its IR_SOLVER_TOL (default 1e-9) and IR_MIN_TOL (default 1e-2). */
int orc_set_linear_solver(orc_ctx *c, int type, double ir_tol, double ir_min_tol);
/* out[6]: factorizations, reused solves, refined solves, refinement steps,
 * fallbacks to a refactorization, repeated factorizations (of a matrix equal
 * bit for bit to the one factored before); reset != 0 zeroes them afterwards. */
int orc_lu_counts(orc_ctx *c, long long *out, int reset);

/* Replay of an accepted-step sequence (for comparisons at identical time
 * points): the next orc_transient steps exactly to times[1], times[2], ...
 * with integration orders orders[1], orders[2], ... (times[0] / orders[0]:
 * the operating point), accepts every step whose Newton solve converges
 * (status -51 otherwise) and stops after the last point.  n = 0 returns to
 * free runs.  Returns -1 unless the times increase and the orders are 1 or 2. */
int orc_set_replay(orc_ctx *c, const double *times, const int *orders, int n);

/* Integration order of each point the last orc_transient recorded (0 for
 * the operating point, else 1 or 2); returns how many were written (<= cap). */
int orc_recorded_orders(orc_ctx *c, int *out, int cap);

/* Benchmark support: record wall-clock seconds at each accepted step. */
int orc_set_wall_log(orc_ctx *c, double *buf, int cap);

#ifdef __cplusplus
}
#endif
#endif
