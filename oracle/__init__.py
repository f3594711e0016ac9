"""ctypes bridge to the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY.  The oracle is a CPU FP64 restatement of Xyce's
transient Newton hot path (see oracle/oracle.h for the reference functions
it follows).  Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline load it, and only as the checker; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
KSPARSE_PATH = os.path.join(HERE, "_ref", "libksparse.so")
# Root of the reference checkout (read only, and only where it exists): set
# XYCE_REFERENCE_ROOT to point the build recipe and the netlist tests at it.
REFERENCE_ROOT = os.environ.get("XYCE_REFERENCE_ROOT", "/root/reference")
REFERENCE_KSPARSE = os.path.join(REFERENCE_ROOT, "src", "LinearAlgebraServicesPKG", "ksparse")

_lib = None


def build(with_reference: bool | None = None) -> None:
    """Compile the oracle; also compile ksparse from the reference's own
    sources when the reference tree is present."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if with_reference is None:
        with_reference = os.path.isdir(REFERENCE_KSPARSE)
    if with_reference:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_KSPARSE}"])


class TranParams(C.Structure):
    _fields_ = [("tstart", C.c_double), ("tstop", C.c_double), ("hmax", C.c_double),
                ("hmin", C.c_double), ("reltol", C.c_double), ("abstol", C.c_double),
                ("nl_reltol", C.c_double), ("nl_abstol", C.c_double),
                ("nl_deltaxtol", C.c_double), ("nl_rhstol", C.c_double),
                ("nl_smallupdatetol", C.c_double), ("nl_maxstep", C.c_int),
                ("max_steps", C.c_int), ("max_order", C.c_int), ("method", C.c_int)]


class TranStats(C.Structure):
    _fields_ = [("accepted", C.c_int), ("rejected", C.c_int), ("newton_iters", C.c_int),
                ("newton_fail", C.c_int), ("lte_fail", C.c_int), ("dcop_iters", C.c_int),
                ("status", C.c_int), ("t_final", C.c_double), ("time_load", C.c_double),
                ("time_solve", C.c_double), ("time_total", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_reference=False)
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        ip = np.ctypeslib.ndpointer(np.int32, flags="C")
        dp = np.ctypeslib.ndpointer(np.float64, flags="C")
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.c_int, C.c_int, ip]
        L.orc_destroy.argtypes = [P]
        L.orc_add_resistors.argtypes = [P, C.c_int, ip, ip, dp]
        L.orc_add_capacitors.argtypes = [P, C.c_int, ip, ip, dp]
        L.orc_add_vsources.argtypes = [P, C.c_int, ip, ip, ip, ip, ip, dp]
        L.orc_add_isources.argtypes = [P, C.c_int, ip, ip, ip, ip, dp]
        L.orc_add_inductors.argtypes = [P, C.c_int, ip, ip, ip, dp]
        L.orc_add_diodes.argtypes = [P, C.c_int, ip, ip, ip, dp]
        L.orc_add_mosfet1.argtypes = [P, C.c_int, ip, ip, ip, ip, ip, ip, dp]
        L.orc_add_bsim4.argtypes = [P, C.c_int, ip, ip, ip, ip, dp]
        L.orc_finalize.argtypes = [P]
        L.orc_sizes.argtypes = [P] + [C.POINTER(C.c_int)] * 4
        L.orc_pattern.argtypes = [P, ip, ip]
        L.orc_load.argtypes = [P, C.c_double, dp, dp, dp, dp, C.c_int, C.c_int] + [dp] * 9
        L.orc_lu_solve.argtypes = [P, dp, dp, dp]
        L.orc_transient.argtypes = [P, C.POINTER(TranParams), C.c_int, ip, C.c_int, dp, dp,
                                    C.POINTER(C.c_int), C.POINTER(TranStats)]
        L.orc_dcop.argtypes = [P, dp, C.POINTER(C.c_int)]
        L.orc_newton.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_double, P, P, dp, P, dp, dp,
                                 dp, dp] + [C.c_double] * 5 + [C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.orc_set_wall_log.argtypes = [P, C.c_void_p, C.c_int]
        L.orc_set_replay.argtypes = [P, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_recorded_orders.argtypes = [P, ip, C.c_int]
        L.orc_set_linear_solver.argtypes = [P, C.c_int, C.c_double, C.c_double]
        L.orc_set_order.argtypes = [P, C.c_void_p, C.c_int]
        L.orc_lu_counts.argtypes = [P, np.ctypeslib.ndpointer(np.int64, flags="C"), C.c_int]
        _lib = L
    return _lib


class Oracle:
    """One circuit (or batch of circuits) loaded into the CPU oracle."""

    def __init__(self, netlist):
        L = lib()
        a = netlist.arrays()
        self.netlist = netlist
        self.h = L.orc_create(a["n"], len(a["offsets"]) - 1, a["offsets"])
        p, m, v = a["res"]
        L.orc_add_resistors(self.h, len(p), p, m, v)
        p, m, v = a["cap"]
        L.orc_add_capacitors(self.h, len(p), p, m, v)
        p, m, b, k, o, d = a["vsrc"]
        L.orc_add_vsources(self.h, len(p), p, m, b, k, o, d)
        p, m, k, o, d = a["isrc"]
        L.orc_add_isources(self.h, len(p), p, m, k, o, d)
        p, m, b, lv = a["ind"]
        if len(p):
            L.orc_add_inductors(self.h, len(p), p, m, b, lv)
        p, m, r, prm = a["diode"]
        L.orc_add_diodes(self.h, len(p), p, m, r, prm)
        dd, g, s, b, dpr, spr, prm = a["mos1"]
        rc = L.orc_add_mosfet1(self.h, len(dd), dd, g, s, b, dpr, spr, prm)
        if rc != 0:
            raise ValueError("oracle: MOSFET drain'/source' nodes must differ from drain/source "
                             "exactly when the series resistance is nonzero")
        dd, g, s, b, prm = a["bsim4"]
        if len(dd):
            rc = L.orc_add_bsim4(self.h, len(dd), dd, g, s, b, np.ascontiguousarray(prm))
            if rc != 0:
                raise ValueError("oracle: BSIM4 card outside the restated scope")
        L.orc_finalize(self.h)
        n, nnz, nsta, nsto = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.orc_sizes(self.h, C.byref(n), C.byref(nnz), C.byref(nsta), C.byref(nsto))
        self.n, self.nnz, self.nsta, self.nsto = n.value, nnz.value, nsta.value, nsto.value
        self.row_ptr = np.zeros(self.n + 1, np.int32)
        self.col_idx = np.zeros(self.nnz, np.int32)
        L.orc_pattern(self.h, self.row_ptr, self.col_idx)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_destroy(self.h)
            self.h = None

    def load(self, x, time=0.0, sta_curr=None, sto_curr=None, sto_prev=None, newton_iter=0,
             dcop=False, init_jct=False):
        """One device load; returns dict of F, Q, B, dFdxdVp, dQdxdVp, dFdx, dQdx
        (CSR values on self.row_ptr/self.col_idx), sta_next, sto_next."""
        n, nnz = self.n, self.nnz
        z = lambda k: np.zeros(max(1, k))
        sta_curr = z(self.nsta) if sta_curr is None else np.ascontiguousarray(sta_curr, np.float64)
        sto_curr = z(self.nsto) if sto_curr is None else np.ascontiguousarray(sto_curr, np.float64)
        sto_prev = z(self.nsto) if sto_prev is None else np.ascontiguousarray(sto_prev, np.float64)
        out = {k: np.zeros(n) for k in ("F", "Q", "B", "dFdxdVp", "dQdxdVp")}
        out["dFdx"] = np.zeros(nnz)
        out["dQdx"] = np.zeros(nnz)
        out["sta_next"] = z(self.nsta)
        out["sto_next"] = z(self.nsto)
        flags = (1 if dcop else 0) | (2 if init_jct else 0)
        lib().orc_load(self.h, float(time), np.ascontiguousarray(x, np.float64), sta_curr,
                       sto_curr, sto_prev, int(newton_iter), flags, out["sta_next"],
                       out["sto_next"], out["F"], out["Q"], out["B"], out["dFdxdVp"],
                       out["dQdxdVp"], out["dFdx"], out["dQdx"])
        return out

    def lu_solve(self, vals, b):
        x = np.zeros(self.n)
        rc = lib().orc_lu_solve(self.h, np.ascontiguousarray(vals, np.float64),
                                np.ascontiguousarray(b, np.float64), x)
        if rc != 0:
            raise np.linalg.LinAlgError("oracle LU: singular")
        return x

    def set_order(self, perm=None):
        """Elimination order of the LU: perm[k] = the unknown eliminated k-th
        (None: the natural order)."""
        if perm is None:
            rc = lib().orc_set_order(self.h, None, 0)
        else:
            perm = np.ascontiguousarray(perm, np.int32)
            rc = lib().orc_set_order(self.h, perm.ctypes.data, len(perm))
        if rc != 0:
            raise ValueError("oracle: the elimination order must be a permutation of the unknowns")

    def use_minimum_degree(self):
        """Order the LU as KLU does before its numeric factorizations: a
        minimum-degree order of the pattern of A + A^T (min_degree_order)."""
        self.set_order(min_degree_order(self.row_ptr, self.col_idx))

    LU_COUNTS = ("factor", "reuse", "refined", "refine_steps", "fallback", "repeat")

    def set_linear_solver(self, kind="klu", ir_tol=1e-9, ir_min_tol=1e-2):
        """.OPTIONS LINSOL TYPE: "klu" refactors on every Newton iteration,
        "ir" reuses earlier factors with iterative refinement (IRSolver)."""
        rc = lib().orc_set_linear_solver(self.h, {"klu": 0, "ir": 1}[kind], float(ir_tol),
                                         float(ir_min_tol))
        if rc != 0:
            raise ValueError("oracle: bad linear solver options")

    def lu_counts(self, reset=True):
        """What the linear solves did since the last reset (LU_COUNTS order)."""
        out = np.zeros(len(self.LU_COUNTS), np.int64)
        lib().orc_lu_counts(self.h, out, int(reset))
        return dict(zip(self.LU_COUNTS, out.tolist()))

    def newton(self, x, time=0.0, qscale=0.0, fscale=1.0, hscale=0.0, qhist0=None, qhist2=None,
               x_curr=None, sta_curr=None, sto_curr=None, flags=0, reltol=1e-2, abstol=1e-6,
               deltaxtol=0.33, rhstol=1e-2, smallupdatetol=1e-6, maxstep=20):
        """One DampedNewton solve (orc_newton); returns (status, iterations,
        x, sta_next, sto_next)."""
        f64 = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        xv = np.array(x, np.float64)
        z = lambda k: np.zeros(max(1, k))
        sta_c = z(self.nsta) if sta_curr is None else f64(sta_curr)
        sto_c = z(self.nsto) if sto_curr is None else f64(sto_curr)
        sta_n, sto_n = z(self.nsta), z(self.nsto)
        q0, q2, xc = f64(qhist0), f64(qhist2), f64(x_curr)
        ptr = lambda a: None if a is None else a.ctypes.data
        it = C.c_int()
        st = lib().orc_newton(self.h, float(time), float(qscale), float(fscale), float(hscale), ptr(q0),
                              ptr(q2), xv, ptr(xc), sta_c, sto_c, sta_n, sto_n, float(reltol), float(abstol),
                              float(deltaxtol), float(rhstol), float(smallupdatetol), int(maxstep),
                              int(flags), C.byref(it))
        return st, it.value, xv, sta_n, sto_n

    def dcop(self):
        x = np.zeros(self.n)
        it = C.c_int()
        st = lib().orc_dcop(self.h, x, C.byref(it))
        return st, x, it.value

    def replay(self, times, orders, tran=None, probes=None):
        """Transient run through a given accepted-step sequence: times[k] and
        orders[k] of point k (point 0 = the operating point), as recorded by
        the GPU path (xg_tran_results / xg_tran_orders).  Every step goes to
        the recorded time with the recorded order; returns what transient()
        returns, at exactly those points."""
        t = np.ascontiguousarray(times, np.float64)
        o = np.ascontiguousarray(orders, np.int32)
        if len(t) != len(o) or len(t) < 2:
            raise ValueError("replay needs matching times and orders, at least two points")
        if lib().orc_set_replay(self.h, t.ctypes.data, o.ctypes.data, len(t)) != 0:
            raise ValueError("replay: times must increase and orders be 1 or 2")
        try:
            return self.transient(tran, probes, cap=len(t) + 1)
        finally:
            lib().orc_set_replay(self.h, None, None, 0)

    def recorded_orders(self, count):
        """Integration order of the points the last transient recorded (0 at
        the operating point)."""
        out = np.zeros(max(1, count), np.int32)
        k = lib().orc_recorded_orders(self.h, out, len(out))
        return out[:k]

    def transient(self, tran=None, probes=None, cap=2_000_000, wall_log=None):
        """Transient run; wall_log (float64 array) receives the wall-clock
        seconds at each accepted step when given."""
        tran = tran or self.netlist.tran
        if wall_log is not None:
            lib().orc_set_wall_log(self.h, wall_log.ctypes.data, len(wall_log))
        else:
            lib().orc_set_wall_log(self.h, None, 0)
        probes = np.asarray(probes if probes is not None else [], np.int32)
        tp = TranParams(tran.tstart, tran.tstop, tran.hmax, tran.hmin, tran.reltol,
                        tran.abstol, tran.nl_reltol, tran.nl_abstol, tran.nl_deltaxtol,
                        tran.nl_rhstol, tran.nl_smallupdatetol, tran.nl_maxstep,
                        tran.max_steps, tran.max_order, tran.method)
        times = np.zeros(cap)
        vals = np.zeros(cap * max(1, len(probes)))
        nout = C.c_int()
        st = TranStats()
        lib().orc_transient(self.h, C.byref(tp), len(probes), probes, cap, times, vals,
                            C.byref(nout), C.byref(st))
        k = nout.value
        return (times[:k].copy(), vals[: k * len(probes)].reshape(k, len(probes)).copy(),
                {f: getattr(st, f) for f, _ in TranStats._fields_})


def min_degree_order(row_ptr, col_idx):
    """A minimum-degree elimination order of the pattern of A + A^T.

    KLU (the reference's default solver, SuiteSparse, through Amesos) orders
    each diagonal block with AMD on A + A^T once, in its symbolic analysis.
    AMD is not in this image; SuperLU's multiple minimum degree on A + A^T
    (scipy's splu, permc_spec "MMD_AT_PLUS_A") is the same family of
    ordering.  Only the pattern matters: it is factored with unit entries and
    a dominant diagonal so that the factorization that returns the order
    cannot break down.  Returns perm with perm[k] = the unknown eliminated
    k-th."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    row_ptr = np.asarray(row_ptr, np.int64)
    col_idx = np.asarray(col_idx, np.int64)
    n = len(row_ptr) - 1
    if n == 0:
        return np.zeros(0, np.int32)
    A = sp.csr_matrix((np.ones(len(col_idx)), col_idx, row_ptr), shape=(n, n))
    A = (A + A.T).tocsc()
    A.data[:] = 1.0
    deg = np.diff(A.indptr).astype(np.float64)
    A = (A + sp.diags(deg + 1.0)).tocsc()
    lu = spl.splu(A, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0,
                  options=dict(SymmetricMode=True))
    # Pr A Pc = L U with column j of A Pc = column i of A where perm_c[i] = j
    return np.argsort(lu.perm_c).astype(np.int32)


def ksparse_solve(row_ptr, col_idx, vals, b):
    """Solve with Kundert Sparse compiled from the reference sources
    (oracle/_ref/libksparse.so); raises FileNotFoundError when not built."""
    if not os.path.exists(KSPARSE_PATH):
        raise FileNotFoundError(KSPARSE_PATH)
    L = C.CDLL(KSPARSE_PATH)
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    L.ks_solve.argtypes = [C.c_int, ip, ip, dp, dp, dp]
    n = len(row_ptr) - 1
    x = np.zeros(n)
    rc = L.ks_solve(n, np.ascontiguousarray(row_ptr, np.int32), np.ascontiguousarray(col_idx, np.int32),
                    np.ascontiguousarray(vals, np.float64), np.ascontiguousarray(b, np.float64), x)
    if rc != 0:
        raise np.linalg.LinAlgError(f"ksparse status {rc}")
    return x


def _replay_worker(task):
    """One oracle run in a worker process: task = (netlist, probes, times,
    orders, variant); times None = a free run.  The variant is None (the
    natural elimination order), "md" (minimum-degree order), "reverse" (the
    natural order backwards) or "ulp" (natural order, every replayed time
    after the operating point moved up by one unit in the last place — the
    same steps perturbed at round-off level).  Returns (times, values,
    stats)."""
    nl, probes, times, orders, order = task
    o = Oracle(nl)
    if order is True or order == "md":
        o.use_minimum_degree()
    elif order == "reverse":
        o.set_order(np.arange(o.n - 1, -1, -1, dtype=np.int32))
    elif order == "ulp":
        if times is not None:
            times = np.array(times, np.float64)
            times[1:] = np.nextafter(times[1:], np.inf)
    elif order not in (None, False):
        raise ValueError(f"unknown variant {order!r}")
    if times is None:
        t, v, st = o.transient(probes=probes)
        return t, v, st
    t, v, st = o.replay(times, orders, probes=probes)
    return t, v, st


def run_many(tasks, processes=None):
    """Oracle runs of several circuits in parallel worker processes (spawned,
    so that a caller holding a CUDA context may use it).  Each task is
    (netlist, probes, times, orders, elimination order — see _replay_worker):
    with times and orders given, a replay of that accepted-step sequence,
    else a free run.
    Returns [(times, values, stats)] in task order."""
    import multiprocessing as mp
    if not os.path.exists(LIB_PATH):
        build(with_reference=False)
    procs = max(1, min(len(tasks), processes or os.cpu_count() or 1))
    if procs == 1:
        return [_replay_worker(t) for t in tasks]
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.map(_replay_worker, tasks, chunksize=1)
