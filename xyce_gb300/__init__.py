"""xyce_gb300 — GB300-native transient Newton hot path of the Xyce circuit simulator.

The compute path is libxyce_gb300.so (hand-written sm_103a CUDA + C++ host,
C-ABI declared in include/xyce_gb300.h).  This module is a thin ctypes
binding to that library; it never computes anything itself and has no CPU
fallback: without the library or without a GB300 device every call raises.

Python mirror of the reference interfaces:
  * :class:`Circuit.update_state` / :meth:`Circuit.load_dae_vectors` /
    :meth:`Circuit.load_dae_matrices` follow Device::DeviceMgr's
    updateState / loadDAEVectors / loadDAEMatrices
    (src/DeviceModelPKG/Core/N_DEV_DeviceMgr.C:3857, 4156, 3980) and take
    torch CUDA tensors as the Linear::Vector / Linear::Matrix storage;
  * :meth:`Circuit.lu_analyze` / :meth:`lu_factor` / :meth:`lu_solve` follow
    AmesosSolver::doSolve (src/LinearAlgebraServicesPKG/N_LAS_AmesosSolver.C:216-440);
  * :meth:`Circuit.transient` runs Transient::doRun (src/AnalysisPKG/N_ANP_Transient.C:739)
    with DampedNewton and OneStep entirely on the device.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import netlist  # noqa: F401  (re-export)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libxyce_gb300.so")

XG_OK = 0
XG_ERR = {-1: "ARG", -2: "CUDA", -3: "STATE", -4: "UNSUPPORTED", -6: "NAN", -9: "SINGULAR",
          -10: "TIMEOUT"}
LOAD_ALL, LOAD_LINEAR, LOAD_NONLINEAR = 0, 1, 2
PREC_FP64, PREC_FP32_IR = 0, 1
ORDER_ND, ORDER_MIN_DEGREE = 0, 1
TOP_ONE_CTA, TOP_LEVELS = 1, 2
PRED_POLY, PRED_LEARNED = 0, 1
TUNE_MODEL, TUNE_TIMED, TUNE_FIXED = 0, 1, 2
FORM_AUTO, FORM_TICK_GRAPH, FORM_RESIDENT = 0, 1, 2
MLP_NPARAM, MLP_NNORM = 4609, 12
FLAG_DCOP, FLAG_INITJCT = 1, 2

# Every symbol declared in include/xyce_gb300.h.
EXPORTED = [
    "xg_create", "xg_destroy", "xg_error_string", "xg_get_stream", "xg_synchronize",
    "xg_set_unknowns", "xg_add_resistors", "xg_add_capacitors", "xg_add_vsources",
    "xg_add_isources", "xg_add_diodes", "xg_add_mosfet1", "xg_add_mosfet1_rs", "xg_add_inductors", "xg_add_bsim4", "xg_finalize", "xg_get_sizes",
    "xg_get_pattern", "xg_update_sources", "xg_update_state", "xg_load_dae_vectors",
    "xg_load_dae_matrices", "xg_lu_analyze", "xg_lu_factor", "xg_lu_solve",
    "xg_lu_solve_noalloc", "xg_lu_set_precision", "xg_lu_info", "xg_lu_schedule_info", "xg_lu_set_schedule", "xg_lu_analyze_pattern",
    "xg_lu_set_tuning", "xg_lu_set_shapes", "xg_lu_tuning_info", "xg_lu_set_reuse", "xg_lu_set_pivot_tolerance",
    "xg_transient", "xg_tran_set_form", "xg_tran_set_tail", "xg_tran_start", "xg_tran_advance", "xg_tran_results", "xg_tran_end",
    "xg_tran_predictors", "xg_tran_orders", "xg_tran_profile", "xg_tran_profile_resident", "xg_tran_predictor_stats", "xg_set_predictor", "xg_mlp_set", "xg_mlp_get",
    "xg_mlp_train", "xg_mlp_grad", "xg_mlp_forward",
    "xg_dcop", "xg_newton_solve", "xg_version",
]


class XgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"xyce_gb300 error {code} ({XG_ERR.get(code, '?')}): {msg}")
        self.code = code


class TranParams(C.Structure):
    _fields_ = [("tstart", C.c_double), ("tstop", C.c_double), ("hmax", C.c_double),
                ("hmin", C.c_double), ("reltol", C.c_double), ("abstol", C.c_double),
                ("nl_reltol", C.c_double), ("nl_abstol", C.c_double),
                ("nl_deltaxtol", C.c_double), ("nl_rhstol", C.c_double),
                ("nl_smallupdatetol", C.c_double), ("nl_maxstep", C.c_int),
                ("max_steps", C.c_int), ("max_order", C.c_int), ("method", C.c_int)]


class NewtonParams(C.Structure):
    _fields_ = [("reltol", C.c_double), ("abstol", C.c_double), ("deltaxtol", C.c_double),
                ("rhstol", C.c_double), ("smallupdatetol", C.c_double), ("maxstep", C.c_int)]


class LuTuning(C.Structure):
    _fields_ = [("mode", C.c_int), ("from_cache", C.c_int), ("factor_threads", C.c_int),
                ("factor_meta", C.c_int), ("lsolve_threads", C.c_int), ("usolve_threads", C.c_int),
                ("model_factor_threads", C.c_int), ("model_factor_meta", C.c_int),
                ("model_lsolve_threads", C.c_int), ("model_usolve_threads", C.c_int),
                ("factor_us", C.c_double), ("solve_us", C.c_double), ("model_factor_us", C.c_double),
                ("model_solve_us", C.c_double)]


class TranStats(C.Structure):
    _fields_ = [("accepted", C.c_longlong), ("rejected", C.c_longlong),
                ("newton_iters", C.c_longlong), ("newton_fail", C.c_longlong),
                ("lte_fail", C.c_longlong), ("dcop_iters", C.c_longlong),
                ("ticks", C.c_longlong), ("device_evals", C.c_longlong), ("status", C.c_int),
                ("n_analyze", C.c_int), ("t_final_min", C.c_double),
                ("t_final_max", C.c_double), ("seconds", C.c_double), ("kernels_per_tick", C.c_int),
                ("form", C.c_int), ("kernel_launches", C.c_longlong), ("circuit_ticks", C.c_longlong),
                ("factor_skips", C.c_longlong), ("resident_threads", C.c_int),
                ("option", C.c_int), ("option_us_per_iter", C.c_double * 6),
                ("tail_launches", C.c_longlong)]

    def as_dict(self):
        out = {}
        for f, _ in self._fields_:
            v = getattr(self, f)
            out[f] = list(v) if isinstance(v, C.Array) else v
        return out


_lib = None


def build(**kw) -> str:
    from .build import build as _b
    return _b(**kw)


def lib() -> C.CDLL:
    """Load libxyce_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    P, I, D = C.c_void_p, C.c_int, C.c_double
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    L.xg_create.argtypes = [C.POINTER(P), I]
    L.xg_destroy.argtypes = [P]
    L.xg_error_string.argtypes = [P]
    L.xg_error_string.restype = C.c_char_p
    L.xg_get_stream.argtypes = [P]
    L.xg_get_stream.restype = P
    L.xg_synchronize.argtypes = [P]
    L.xg_set_unknowns.argtypes = [P, I, I, ip]
    L.xg_add_resistors.argtypes = [P, I, ip, ip, dp]
    L.xg_add_capacitors.argtypes = [P, I, ip, ip, dp]
    L.xg_add_vsources.argtypes = [P, I, ip, ip, ip, ip, ip, dp]
    L.xg_add_isources.argtypes = [P, I, ip, ip, ip, ip, dp]
    L.xg_add_inductors.argtypes = [P, I, ip, ip, ip, dp]
    L.xg_add_diodes.argtypes = [P, I, ip, ip, ip, dp]
    L.xg_add_mosfet1.argtypes = [P, I, ip, ip, ip, ip, dp]
    L.xg_add_mosfet1_rs.argtypes = [P, I, ip, ip, ip, ip, ip, ip, dp]
    L.xg_add_bsim4.argtypes = [P, I, ip, ip, ip, ip, dp]
    L.xg_finalize.argtypes = [P]
    L.xg_get_sizes.argtypes = [P] + [C.POINTER(I)] * 4
    L.xg_get_pattern.argtypes = [P, ip, ip]
    L.xg_update_sources.argtypes = [P, D]
    L.xg_update_state.argtypes = [P, P, P, P, P, P, I, I, I]
    L.xg_load_dae_vectors.argtypes = [P, P, P, P, P, P, P, I]
    L.xg_load_dae_matrices.argtypes = [P, P, P, I]
    L.xg_lu_analyze.argtypes = [P, P]
    L.xg_lu_factor.argtypes = [P, P]
    L.xg_lu_solve.argtypes = [P, P, P]
    L.xg_lu_solve_noalloc.argtypes = [P, P, P]
    L.xg_lu_set_precision.argtypes = [P, I, I]
    L.xg_lu_info.argtypes = [P, C.POINTER(C.c_longlong), C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    L.xg_lu_schedule_info.argtypes = [P, C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    L.xg_lu_set_schedule.argtypes = [P, I, I, I]
    L.xg_lu_set_tuning.argtypes = [P, I]
    L.xg_lu_set_shapes.argtypes = [P, I, I, I, I]
    L.xg_lu_set_reuse.argtypes = [P, I]
    L.xg_lu_set_pivot_tolerance.argtypes = [P, D]
    L.xg_lu_tuning_info.argtypes = [P, C.POINTER(LuTuning)]
    L.xg_lu_analyze_pattern.argtypes = [I, C.POINTER(I), C.POINTER(I), C.POINTER(C.c_double), I,
                                        C.POINTER(C.c_longlong), C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    L.xg_transient.argtypes = [P, C.POINTER(TranParams), I, ip, I, ip, dp, dp, C.POINTER(TranStats)]
    L.xg_tran_start.argtypes = [P, C.POINTER(TranParams), I, ip, I]
    L.xg_tran_advance.argtypes = [P, I]
    L.xg_tran_set_form.argtypes = [P, I]
    L.xg_tran_set_tail.argtypes = [P, C.c_double]
    L.xg_tran_results.argtypes = [P, ip, dp, dp, C.POINTER(TranStats)]
    L.xg_tran_end.argtypes = [P]
    L.xg_dcop.argtypes = [P, dp, C.POINTER(I)]
    L.xg_newton_solve.argtypes = [P, C.POINTER(NewtonParams), D, D, D, D, P, P, P, P, P, P, P, P, I, ip, ip]
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    LL = C.POINTER(C.c_longlong)
    L.xg_tran_predictors.argtypes = [P, dp]
    L.xg_tran_orders.argtypes = [P, ip]
    L.xg_tran_profile.argtypes = [P, I, I, dp, np.ctypeslib.ndpointer(np.int64, flags="C")]
    L.xg_tran_profile_resident.argtypes = [P, I, I, dp, C.POINTER(C.c_longlong)]
    L.xg_tran_predictor_stats.argtypes = [P, LL, LL, LL, LL]
    L.xg_set_predictor.argtypes = [P, I]
    L.xg_mlp_set.argtypes = [P, fp, fp]
    L.xg_mlp_get.argtypes = [P, fp, fp]
    L.xg_mlp_train.argtypes = [P, P, P, I, I, C.c_float, fp]
    L.xg_mlp_grad.argtypes = [P, P, P, I, fp, fp]
    L.xg_mlp_forward.argtypes = [P, P, I, P]
    L.xg_version.argtypes = []
    _lib = L
    return L


def _ptr(t):
    """Device pointer of a torch CUDA tensor (float64, contiguous)."""
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return C.c_void_p(t.data_ptr())


def analyze_pattern(row_ptr, col_idx, vals, ordering=-1):
    """Host-only LU analysis of a CSR matrix (no GPU needed): nnz(L+U), the
    ordering ('nested_dissection' / 'min_degree'), the factor schedule's
    dependency-closed groups and top size."""
    rp = np.ascontiguousarray(row_ptr, np.int32)
    ci = np.ascontiguousarray(col_idx, np.int32)
    v = np.ascontiguousarray(vals, np.float64)
    nnz, o, g, t = C.c_longlong(), C.c_int(), C.c_int(), C.c_int()
    rc = lib().xg_lu_analyze_pattern(len(rp) - 1, rp.ctypes.data_as(C.POINTER(C.c_int)),
                                     ci.ctypes.data_as(C.POINTER(C.c_int)),
                                     v.ctypes.data_as(C.POINTER(C.c_double)), int(ordering),
                                     C.byref(nnz), C.byref(o), C.byref(g), C.byref(t))
    if rc != 0:
        raise XgError(rc, f"xg_lu_analyze_pattern failed ({rc})")
    return dict(nnz_lu=nnz.value, ordering="min_degree" if o.value == 1 else "nested_dissection",
                n_groups=g.value, n_top=t.value)


class Circuit:
    """A netlist (or batch of circuits) resident on one GB300."""

    def __init__(self, nl, device: int = 0, arrays=None):
        """arrays: nl.arrays() when the caller already holds the flat host
        arrays of the C-ABI (they are built from the netlist otherwise)."""
        L = lib()
        self.netlist = nl
        self.h = C.c_void_p()
        rc = L.xg_create(C.byref(self.h), device)
        if rc != XG_OK:
            raise XgError(rc, "xg_create: no usable sm_103a (GB300) device")
        a = arrays if arrays is not None else nl.arrays()
        self._check(L.xg_set_unknowns(self.h, a["n"], len(a["offsets"]) - 1, a["offsets"]))
        p, m, v = a["res"]
        self._check(L.xg_add_resistors(self.h, len(p), p, m, v))
        p, m, v = a["cap"]
        self._check(L.xg_add_capacitors(self.h, len(p), p, m, v))
        p, m, b, k, o, d = a["vsrc"]
        self._check(L.xg_add_vsources(self.h, len(p), p, m, b, k, o, d))
        p, m, k, o, d = a["isrc"]
        self._check(L.xg_add_isources(self.h, len(p), p, m, k, o, d))
        p, m, b, lv = a["ind"]
        if len(p):
            self._check(L.xg_add_inductors(self.h, len(p), p, m, b, lv))
        p, m, r, prm = a["diode"]
        self._check(L.xg_add_diodes(self.h, len(p), p, m, r, prm))
        dd, g, s, b, dpr, spr, prm = a["mos1"]
        self._check(L.xg_add_mosfet1_rs(self.h, len(dd), dd, g, s, b, dpr, spr, prm))
        dd, g, s, b, prm = a["bsim4"]
        if len(dd):
            self._check(L.xg_add_bsim4(self.h, len(dd), dd, g, s, b, np.ascontiguousarray(prm)))
        self._check(L.xg_finalize(self.h))
        n, nnz, nsta, nsto = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._check(L.xg_get_sizes(self.h, C.byref(n), C.byref(nnz), C.byref(nsta), C.byref(nsto)))
        self.n, self.nnz, self.nsta, self.nsto = n.value, nnz.value, nsta.value, nsto.value
        self.row_ptr = np.zeros(self.n + 1, np.int32)
        self.col_idx = np.zeros(self.nnz, np.int32)
        self._check(L.xg_get_pattern(self.h, self.row_ptr, self.col_idx))
        self.n_circuits = len(a["offsets"]) - 1

    def _check(self, rc):
        if rc != XG_OK:
            raise XgError(rc, lib().xg_error_string(self.h).decode())

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().xg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- loader (DeviceMgr mirror) -------------------------------------
    def update_sources(self, time: float):
        self._check(lib().xg_update_sources(self.h, float(time)))

    def update_state(self, next_sol, curr_sta, curr_sto, next_sta, next_sto, newton_iter=0, flags=0,
                     load_type=LOAD_ALL):
        self._check(lib().xg_update_state(self.h, _ptr(next_sol), _ptr(curr_sta), _ptr(curr_sto),
                                          _ptr(next_sta), _ptr(next_sto), int(newton_iter), int(flags),
                                          int(load_type)))

    def load_dae_vectors(self, next_sol, Q, F, B, dFdxdVp, dQdxdVp, load_type=LOAD_ALL):
        self._check(lib().xg_load_dae_vectors(self.h, _ptr(next_sol), _ptr(Q), _ptr(F), _ptr(B),
                                              _ptr(dFdxdVp), _ptr(dQdxdVp), int(load_type)))

    def load_dae_matrices(self, dQdx, dFdx, load_type=LOAD_ALL):
        self._check(lib().xg_load_dae_matrices(self.h, _ptr(dQdx), _ptr(dFdx), int(load_type)))

    def synchronize(self):
        self._check(lib().xg_synchronize(self.h))

    # ---- linear solve (AmesosSolver mirror) ----------------------------
    def lu_analyze(self, vals):
        self._check(lib().xg_lu_analyze(self.h, _ptr(vals)))

    def lu_factor(self, vals):
        self._check(lib().xg_lu_factor(self.h, _ptr(vals)))

    def lu_solve(self, rhs, x):
        self._check(lib().xg_lu_solve(self.h, _ptr(rhs), _ptr(x)))

    def lu_solve_noalloc(self, rhs, x):
        """xg_lu_solve without allocated scratch (see include/xyce_gb300.h)."""
        self._check(lib().xg_lu_solve_noalloc(self.h, _ptr(rhs), _ptr(x)))

    def lu_set_precision(self, precision: int, n_refine: int = 2):
        """PREC_FP64, or PREC_FP32_IR: FP32 factors + n_refine FP64 refinement steps."""
        self._check(lib().xg_lu_set_precision(self.h, int(precision), int(n_refine)))

    def lu_set_schedule(self, ordering=-1, factor_top=-1, solve_top=-1):
        """Override the analysis' choices (-1 = automatic): ORDER_ND /
        ORDER_MIN_DEGREE, and TOP_ONE_CTA / TOP_LEVELS for the factor and
        solve tops; applies from the next analysis."""
        self._check(lib().xg_lu_set_schedule(self.h, int(ordering), int(factor_top), int(solve_top)))

    def lu_set_tuning(self, mode: int):
        """TUNE_TIMED (default): launch shapes of the LU sweeps chosen by
        timed trials after each analysis; TUNE_MODEL: closed-form choice."""
        self._check(lib().xg_lu_set_tuning(self.h, int(mode)))

    def lu_set_shapes(self, factor_threads=0, factor_meta=-1, lsolve_threads=0, usolve_threads=0):
        """Fixed launch shapes of the LU sweeps (TUNE_FIXED; 0 / -1 keep the
        analysis' choice of that part)."""
        self._check(lib().xg_lu_set_shapes(self.h, int(factor_threads), int(factor_meta), int(lsolve_threads),
                                           int(usolve_threads)))

    def lu_set_pivot_tolerance(self, tol: float):
        """Frozen-pivot acceptance threshold (default 1e-2), see xg_lu_set_pivot_tolerance."""
        self._check(lib().xg_lu_set_pivot_tolerance(self.h, float(tol)))

    def lu_set_reuse(self, on: bool):
        """Skip bit-identical refactorizations of linear circuits (default on)."""
        self._check(lib().xg_lu_set_reuse(self.h, int(bool(on))))

    def lu_tuning(self):
        t = LuTuning()
        self._check(lib().xg_lu_tuning_info(self.h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in LuTuning._fields_}

    def lu_info(self):
        nnz = C.c_longlong()
        f, l, u = C.c_int(), C.c_int(), C.c_int()
        self._check(lib().xg_lu_info(self.h, C.byref(nnz), C.byref(f), C.byref(l), C.byref(u)))
        o, ft, stp = C.c_int(), C.c_int(), C.c_int()
        self._check(lib().xg_lu_schedule_info(self.h, C.byref(o), C.byref(ft), C.byref(stp)))
        tops = {0: "none", 1: "one_cta", 2: "levels"}
        return dict(nnz_lu=nnz.value, factor_levels=f.value, lsolve_levels=l.value,
                    usolve_levels=u.value, ordering="min_degree" if o.value == 1 else "nested_dissection",
                    factor_top=tops[ft.value], solve_top=tops[stp.value])

    # ---- analyses -------------------------------------------------------
    def dcop(self):
        x = np.zeros(self.n)
        it = C.c_int()
        self._check(lib().xg_dcop(self.h, x, C.byref(it)))
        return x, it.value

    def newton_solve(self, x, curr_sta, curr_sto, next_sta, next_sto, time=0.0, qscale=0.0, fscale=1.0,
                     hscale=0.0, qhist0=None, qhist2=None, x_curr=None, flags=0, reltol=1e-2,
                     abstol=1e-6, deltaxtol=0.33, rhstol=1e-2, smallupdatetol=1e-6, maxstep=20):
        """DampedNewton on the device for every circuit (xg_newton_solve):
        x (CUDA tensor) holds the initial guess and receives the last iterate;
        returns (status codes, iterations) per circuit.  Defaults are the
        NONLIN-TRAN options (N_NLS_Manager.C:1056-1066)."""
        p = NewtonParams(reltol, abstol, deltaxtol, rhstol, smallupdatetol, maxstep)
        st = np.zeros(self.n_circuits, np.int32)
        it = np.zeros(self.n_circuits, np.int32)
        self._check(lib().xg_newton_solve(self.h, C.byref(p), float(time), float(qscale), float(fscale),
                                          float(hscale), _ptr(qhist0), _ptr(qhist2), _ptr(x), _ptr(x_curr),
                                          _ptr(curr_sta), _ptr(curr_sto), _ptr(next_sta), _ptr(next_sto),
                                          int(flags), st, it))
        return st, it

    def _tran_params(self, tran):
        return TranParams(tran.tstart, tran.tstop, tran.hmax, tran.hmin, tran.reltol, tran.abstol,
                          tran.nl_reltol, tran.nl_abstol, tran.nl_deltaxtol, tran.nl_rhstol,
                          tran.nl_smallupdatetol, tran.nl_maxstep, tran.max_steps, tran.max_order,
                          tran.method)

    def tran_set_form(self, form: int):
        """FORM_AUTO, FORM_TICK_GRAPH or FORM_RESIDENT (see xg_tran_set_form)."""
        self._check(lib().xg_tran_set_form(self.h, int(form)))

    def tran_set_tail(self, active_fraction: float):
        """Finish a tick-graph advance with the resident kernel once at most
        this fraction of the circuits is still running (0: off; see
        xg_tran_set_tail)."""
        self._check(lib().xg_tran_set_tail(self.h, float(active_fraction)))

    def tran_start(self, tran=None, probes=(), cap=0):
        """Operating point + first analysis; keeps the run resident for tran_advance."""
        tran = tran or self.netlist.tran
        probes = np.asarray(probes, np.int32)
        self._check(lib().xg_tran_start(self.h, C.byref(self._tran_params(tran)), len(probes),
                                        probes, int(cap)))
        self._run = (len(probes), cap, probes)  # a rejected start keeps the earlier run's layout

    def tran_advance(self, n_steps: int):
        self._check(lib().xg_tran_advance(self.h, int(n_steps)))

    def tran_results(self):
        """(counts, times, values, stats) of the run so far."""
        n_probe, cap, probes = self._run
        nc = self.n_circuits
        offs = np.asarray(self.netlist.offsets)
        per = np.bincount(np.searchsorted(offs, probes, side="right") - 1, minlength=nc) \
            if n_probe else np.zeros(nc, int)
        pmax = max(1, int(per.max()) if len(per) else 1)
        counts = np.zeros(nc, np.int32)
        times = np.zeros(max(1, nc * cap))
        values = np.zeros(max(1, nc * cap * pmax))
        st = TranStats()
        self._check(lib().xg_tran_results(self.h, counts, times, values, C.byref(st)))
        stats = st.as_dict()
        if cap:
            times = times[: nc * cap].reshape(nc, cap)
            values = values[: nc * cap * pmax].reshape(nc, cap, pmax)
        return counts, times, values, stats

    def tran_end(self):
        self._check(lib().xg_tran_end(self.h))

    def tran_predictors(self):
        """Newton initial guesses of the recorded points, [n_circuits, cap, pmax]."""
        n_probe, cap, probes = self._run
        nc = self.n_circuits
        offs = np.asarray(self.netlist.offsets)
        per = np.bincount(np.searchsorted(offs, probes, side="right") - 1, minlength=nc) \
            if n_probe else np.zeros(nc, int)
        pmax = max(1, int(per.max()) if len(per) else 1)
        out = np.zeros(max(1, nc * cap * pmax))
        self._check(lib().xg_tran_predictors(self.h, out))
        return out[: nc * cap * pmax].reshape(nc, cap, pmax)

    STAGES = ("sources", "mos1", "bsim4", "diode", "assemble", "newton", "lu_factor", "lu_solve", "update",
              "step", "history", "commit")

    def tran_profile(self, n_ticks: int, n_steps: int = 0):
        """Per-stage device milliseconds summed over n_ticks ticks of the
        run in progress (n_steps > 0: in a new window of that many steps),
        and, summed over the ticks, the instances each model stage evaluated
        and the active circuits."""
        ms = np.zeros(len(self.STAGES))
        ev = np.zeros(4, np.int64)
        self._check(lib().xg_tran_profile(self.h, int(n_steps), int(n_ticks), ms, ev))
        return dict(zip(self.STAGES, ms.tolist())), dict(zip(("mos1", "bsim4", "diode", "circuits"), ev.tolist()))

    RSTAGES = ("sources", "devices", "long_gathers", "assemble", "newton", "factor", "solve", "update", "step",
               "commit")

    def tran_profile_resident(self, n_steps: int = 0, threads: int = 64):
        """SM cycles the circuit-resident tick's CTAs spend in each stage
        (summed over CTAs and ticks) over one resident launch of the run in
        progress (n_steps > 0: a new window of that many steps), and the
        circuit Newton iterations that launch ran."""
        cyc = np.zeros(len(self.RSTAGES))
        ticks = C.c_longlong()
        self._check(lib().xg_tran_profile_resident(self.h, int(n_steps), int(threads), cyc, C.byref(ticks)))
        return dict(zip(self.RSTAGES, cyc.tolist())), ticks.value

    def tran_orders(self):
        """Integration order of each recorded point, [n_circuits, cap] (0 at
        the operating point)."""
        n_probe, cap, probes = self._run
        out = np.zeros(max(1, self.n_circuits * cap), np.int32)
        self._check(lib().xg_tran_orders(self.h, out))
        return out[: self.n_circuits * cap].reshape(self.n_circuits, cap)

    def predictor_stats(self):
        v = [C.c_longlong() for _ in range(4)]
        self._check(lib().xg_tran_predictor_stats(self.h, *[C.byref(x) for x in v]))
        return dict(learned_steps=v[0].value, learned_iters=v[1].value, poly_steps=v[2].value,
                    poly_iters=v[3].value)

    # ---- learned predictor ------------------------------------------------
    def set_predictor(self, mode: int):
        self._check(lib().xg_set_predictor(self.h, int(mode)))

    def mlp_set(self, theta, norm):
        self._check(lib().xg_mlp_set(self.h, np.ascontiguousarray(theta, np.float32),
                                     np.ascontiguousarray(norm, np.float32)))

    def mlp_get(self):
        theta, norm = np.zeros(MLP_NPARAM, np.float32), np.zeros(MLP_NNORM, np.float32)
        self._check(lib().xg_mlp_get(self.h, theta, norm))
        return theta, norm

    def mlp_train(self, X, Y, iters: int, lr: float):
        """X (n x 5), Y (n): float32 CUDA tensors; returns the loss history."""
        hist = np.zeros(max(1, iters), np.float32)
        self._check(lib().xg_mlp_train(self.h, _ptr(X), _ptr(Y), int(Y.shape[0]), int(iters),
                                       float(lr), hist))
        return hist[:iters]

    def mlp_grad(self, X, Y):
        g, l = np.zeros(MLP_NPARAM, np.float32), np.zeros(1, np.float32)
        self._check(lib().xg_mlp_grad(self.h, _ptr(X), _ptr(Y), int(Y.shape[0]), g, l))
        return float(l[0]), g

    def mlp_forward(self, X, out):
        self._check(lib().xg_mlp_forward(self.h, _ptr(X), int(X.shape[0]), _ptr(out)))

    def transient(self, tran=None, probes=(), cap=0):
        """Run the transient; returns (counts, times, values, stats) where
        times is [n_circuits, cap] and values [n_circuits, cap, pmax]."""
        tran = tran or self.netlist.tran
        probes = np.asarray(probes, np.int32)
        tp = self._tran_params(tran)
        nc = self.n_circuits
        offs = np.asarray(self.netlist.offsets)
        per = np.bincount(np.searchsorted(offs, probes, side="right") - 1, minlength=nc) \
            if len(probes) else np.zeros(nc, int)
        pmax = max(1, int(per.max()) if len(per) else 1)
        counts = np.zeros(nc, np.int32)
        times = np.zeros(max(1, nc * cap))
        values = np.zeros(max(1, nc * cap * pmax))
        st = TranStats()
        self._check(lib().xg_transient(self.h, C.byref(tp), len(probes), probes, int(cap), counts,
                                       times, values, C.byref(st)))
        stats = st.as_dict()
        if cap:
            times = times[: nc * cap].reshape(nc, cap)
            values = values[: nc * cap * pmax].reshape(nc, cap, pmax)
        return counts, times, values, stats
