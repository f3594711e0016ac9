"""Error behaviour of the C-ABI on a GPU: bad sizes and nodes, calls out of
order, cards outside the restated scope, and systems that cannot be
factored — each returns its status code and leaves the context usable."""
import ctypes as C

import numpy as np
import pytest

from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _ctx(xg, n=3):
    L = xg.lib()
    h = C.c_void_p()
    assert L.xg_create(C.byref(h), 0) == xg.XG_OK
    offs = np.array([0, n], np.int32)
    assert L.xg_set_unknowns(h, n, 1, offs) == xg.XG_OK
    return L, h


def test_bad_arguments_and_order(xg, torch_cuda):
    L, h = _ctx(xg)
    i32 = lambda *v: np.array(v, np.int32)
    # node out of range
    assert L.xg_add_resistors(h, 1, i32(0), i32(7), np.array([1.0])) == -1
    # load before finalize
    x = torch_cuda.zeros(3, dtype=torch_cuda.float64, device="cuda:0")
    assert L.xg_load_dae_matrices(h, C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), 0) == -3
    # LU before analysis
    assert L.xg_lu_factor(h, C.c_void_p(x.data_ptr())) == -3
    # unknown precision mode
    assert L.xg_lu_set_precision(h, 7, 2) == -1
    assert b"precision" in L.xg_error_string(h)
    # unknown predictor mode
    assert L.xg_set_predictor(h, 5) == -1
    assert L.xg_add_resistors(h, 1, i32(0), i32(1), np.array([1.0])) == xg.XG_OK
    assert L.xg_finalize(h) == xg.XG_OK
    assert L.xg_finalize(h) == -3  # twice
    assert L.xg_destroy(h) == xg.XG_OK


def test_mosfet1_series_resistance_nodes_checked(xg, torch_cuda):
    """A row with RD (or RSH) needs the drain' node: xg_add_mosfet1 refuses
    it, and xg_add_mosfet1_rs wants d' != d exactly when the conductance is
    nonzero."""
    L, h = _ctx(xg, n=4)
    i32 = lambda *v: np.array(v, np.int32)
    row = N.mos1_row(TYPE=1.0, VTO=0.5, KP=1e-4, RD=10.0)
    assert L.xg_add_mosfet1(h, 1, i32(0), i32(1), i32(-1), i32(-1), row) == -1
    assert b"xg_add_mosfet1_rs" in L.xg_error_string(h)
    assert L.xg_add_mosfet1_rs(h, 1, i32(0), i32(1), i32(-1), i32(-1), i32(0), i32(-1), row) == -1
    assert L.xg_add_mosfet1_rs(h, 1, i32(0), i32(1), i32(-1), i32(-1), i32(2), i32(3), row) == -1
    ok = N.mos1_row(TYPE=1.0, VTO=0.5, KP=1e-4, RSH=5.0, NRD=2.0)  # RS = 0, RSH * NRS = 5 ohm
    assert L.xg_add_mosfet1_rs(h, 1, i32(0), i32(1), i32(-1), i32(-1), i32(2), i32(3), ok) == xg.XG_OK
    bad = N.mos1_row(TYPE=1.0, VTO=0.5, KP=1e-4, RSH=5.0, NRD=0.0)  # 1/(RSH * 0)
    assert L.xg_add_mosfet1_rs(h, 1, i32(0), i32(1), i32(-1), i32(-1), i32(2), i32(3), bad) == -1
    assert L.xg_destroy(h) == xg.XG_OK


def test_unsupported_device_cards(xg, torch_cuda):
    nl = N.Netlist(label="b4_bad_type")
    a, b = nl.node("a"), nl.node("b")
    nl.M4(a, b, -1, -1, TYPE=0.5, L=45e-9, W=90e-9)  # TYPE must be +-1
    with pytest.raises(xg.XgError) as e:
        xg.Circuit(nl)
    assert e.value.code == -4


def test_singular_system_reports_and_recovers(xg, torch_cuda):
    """An all-zero matrix fails with XG_ERR_SINGULAR (in the analysis, or in
    the factorization when the analysis keeps the structural diagonal); the
    same context then factors a regular matrix of the same pattern."""
    nl = N.Netlist(label="float")
    a, b = nl.node("a"), nl.node("b")
    nl.R(a, -1, 1.0)
    nl.C(b, -1, 1e-12)
    c = xg.Circuit(nl)
    vals = np.zeros(c.nnz)
    torch = torch_cuda
    v = torch.as_tensor(vals, device="cuda:0")
    try:
        c.lu_analyze(v)
    except xg.XgError as e:
        assert e.code == -9
    else:
        with pytest.raises(xg.XgError) as e:
            c.lu_factor(v)
        assert e.value.code == -9
    vals[:] = 1.0  # diagonal entries only: identity
    v = torch.as_tensor(vals, device="cuda:0")
    c.lu_analyze(v)
    c.lu_factor(v)
    rhs = torch.tensor([2.0, 3.0], dtype=torch.float64, device="cuda:0")
    x = torch.zeros_like(rhs)
    c.lu_solve(rhs, x)
    torch.cuda.synchronize()
    np.testing.assert_allclose(x.cpu().numpy(), [2.0, 3.0])
    c.close()


def test_circuits_without_nonlinear_devices(xg, torch_cuda):
    """Empty device classes: an RC-only circuit runs the transient with no
    MOSFET, BSIM4 or diode kernels to launch."""
    nl = N.rc_step()
    counts, t, v, st = xg.Circuit(nl).transient(probes=[nl.names["out"]], cap=20000)
    assert st["status"] == 0 and counts[0] > 10
