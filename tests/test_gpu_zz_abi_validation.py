"""Topology validation of the C-ABI on a GPU: an xg_add_* call that rejects
one item appends none of them, and a two-terminal device or source whose
nodes lie in two circuits of a batch is refused at finalize."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda(xg):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return xg.lib()


def _ctx(xg, L, n, offsets):
    h = C.c_void_p()
    assert L.xg_create(C.byref(h), 0) == xg.XG_OK
    assert L.xg_set_unknowns(h, n, len(offsets) - 1, np.array(offsets, np.int32)) == xg.XG_OK
    return h


def test_rejected_add_appends_nothing(xg, cuda):
    L = cuda
    i32 = lambda *v: np.array(v, np.int32)
    h = _ctx(xg, L, 4, [0, 4])
    assert L.xg_add_resistors(h, 1, i32(0), i32(1), np.array([1.0])) == xg.XG_OK
    # the second item is out of range: the first, valid one is not kept either
    assert L.xg_add_resistors(h, 2, i32(2, 0), i32(3, 9), np.array([1.0, 1.0])) == -1  # XG_ERR_ARG
    assert L.xg_finalize(h) == xg.XG_OK
    n, nnz, nsta, nsto = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    assert L.xg_get_sizes(h, C.byref(n), C.byref(nnz), C.byref(nsta), C.byref(nsto)) == xg.XG_OK
    # the 2x2 block of the kept resistor and the diagonals of nodes 2 and 3
    assert (n.value, nnz.value) == (4, 6)
    assert L.xg_destroy(h) == xg.XG_OK


def test_device_across_circuits_refused(xg, cuda):
    L = cuda
    h = _ctx(xg, L, 4, [0, 2, 4])
    assert L.xg_add_resistors(h, 1, np.array([1], np.int32), np.array([2], np.int32),
                              np.array([1.0])) == xg.XG_OK
    assert L.xg_finalize(h) == -1  # XG_ERR_ARG
    assert b"spans two circuits" in L.xg_error_string(h)
    assert L.xg_destroy(h) == xg.XG_OK


def test_transient_parameters_checked(xg, cuda):
    """Tolerances the error weights divide by, the Newton step limit and the
    order are checked before anything is allocated; the context stays usable."""
    import dataclasses
    from xyce_gb300 import netlist as N
    nl = N.rc_step()
    c = xg.Circuit(nl)
    for bad in (dict(reltol=0.0), dict(abstol=-1e-9), dict(nl_rhstol=float("nan")), dict(nl_maxstep=0),
                dict(max_order=3), dict(hmin=-1.0)):
        with pytest.raises(xg.XgError) as e:
            c.tran_start(dataclasses.replace(nl.tran, **bad), probes=[nl.names["out"]], cap=16)
        assert e.value.code == -1
    counts, t, v, st = c.transient(probes=[nl.names["out"]], cap=20000)
    assert st["status"] == 0 and counts[0] > 10
    c.close()


def test_rejected_tran_start_leaves_no_half_built_run(xg, cuda):
    """A start rejected for a probe out of range or listed twice allocates
    nothing and builds no run: advancing afterwards is XG_ERR_STATE.  A
    rejected start after a good one keeps that run and its results."""
    from xyce_gb300 import netlist as N
    nl = N.rc_step()
    c = xg.Circuit(nl)
    out = nl.names["out"]
    for probes in ([nl.n + 5], [out, out]):
        with pytest.raises(xg.XgError) as e:
            c.tran_start(probes=probes, cap=16)
        assert e.value.code == -1
        with pytest.raises(xg.XgError) as e:
            c.tran_advance(4)
        assert e.value.code == -3  # XG_ERR_STATE: no run
    c.tran_start(probes=[out], cap=64)
    c.tran_advance(5)
    with pytest.raises(xg.XgError):
        c.tran_start(probes=[out, out], cap=64)
    c.tran_advance(5)  # the earlier run is still there
    counts, t, v, st = c.tran_results()
    assert st["accepted"] >= 10 and counts[0] >= 11
    c.tran_end()
    c.close()


def test_tuning_form_and_tail_setters_checked(xg, cuda):
    """The launch-shape, form and tail setters reject values outside their
    ranges, and refuse to change while a transient is in progress."""
    from xyce_gb300 import netlist as N
    L = cuda
    nl = N.monte_carlo_rings(64, 11, 21, seed=3)
    nl.tran.tstop = 0.05e-9
    c = xg.Circuit(nl)
    h = c.h
    assert L.xg_lu_set_shapes(h, 96, 0, 0, 0) == -1          # not a CTA size
    assert L.xg_lu_set_shapes(h, 128, 2, 0, 0) == -1         # meta must be -1, 0 or 1
    assert L.xg_lu_set_shapes(h, 0, -1, 64, 1024) == -1      # too large
    assert L.xg_tran_set_tail(h, C.c_double(-0.1)) == -1
    assert L.xg_tran_set_tail(h, C.c_double(1.5)) == -1
    assert L.xg_tran_set_form(h, 7) == -1
    assert L.xg_lu_set_shapes(h, 128, 1, 64, 64) == xg.XG_OK
    c.tran_start(probes=[0], cap=16)
    assert c.lu_tuning()["mode"] == xg.TUNE_FIXED and c.lu_tuning()["factor_threads"] == 128
    assert L.xg_lu_set_shapes(h, 256, 0, 0, 0) == -3         # XG_ERR_STATE during a transient
    assert L.xg_tran_set_form(h, xg.FORM_TICK_GRAPH) == -3
    c.tran_advance(0)
    c.tran_end()
    assert L.xg_tran_set_tail(h, C.c_double(0.5)) == xg.XG_OK
    c.close()
