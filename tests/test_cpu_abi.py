"""The C-ABI library loads and exports every symbol include/xyce_gb300.h declares
(no compute calls: this container has no GPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xyce_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("xg_create", "xg_update_state", "xg_load_dae_vectors", "xg_load_dae_matrices",
              "xg_lu_factor", "xg_lu_solve", "xg_transient"):
        assert s in syms


def test_library_exports_every_declared_symbol(xg):
    lib = C.CDLL(xg.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(xg.EXPORTED) == declared_symbols()


def test_version_without_device(xg):
    assert xg.lib().xg_version() == 100


def test_create_fails_loudly_without_gpu(xg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert xg.lib().xg_create(C.byref(h), 0) == -2  # XG_ERR_CUDA: no CPU fallback
    with pytest.raises(xg.XgError):
        xg.Circuit(__import__("xyce_gb300.netlist", fromlist=["x"]).test_netlist1())


def test_bsim4_row_layout_matches_header_and_oracle():
    """XG_B4_* (C header), the oracle's row and netlist.B4_FIELDS agree."""
    from xyce_gb300 import netlist as N
    hdr = open(HEADER).read()
    body = hdr[hdr.index("XG_B4_TYPE"):hdr.index("XG_B4_NPARAM")]
    names = re.findall(r"XG_B4_(\w+)", body)
    assert names == N.B4_FIELDS
    orc = open(os.path.join(os.path.dirname(HEADER), "..", "oracle", "bsim4.h")).read()
    body = orc[orc.index("#define ORC_B4_PARAMS"):orc.index("#define ORC_B4_ENUM")]
    assert re.findall(r"X\((\w+)\)", body) == N.B4_FIELDS
