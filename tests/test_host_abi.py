"""The C-ABI library on the CPU: it loads, exports every entry point declared
in include/lss.h, and rejects bad input with status codes (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def test_library_exports_every_declared_symbol(built):
    import lss
    L = lss.load()
    header = open(os.path.join(ROOT, "include", "lss.h")).read()
    declared = sorted(set(re.findall(r"\b(lss_[a-z0-9_A]+)\s*\(", header)))
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(lss.solver.EXPORTS)


def test_status_strings(built):
    import lss
    L = lss.load()
    assert L.lss_status_string(0) == b"ok"
    assert L.lss_status_string(3) == b"out of memory"


def test_invalid_parameters_are_rejected_before_device_use(built):
    import lss
    L = lss.load()
    h = C.c_void_p()
    st = L.lss_create(b'{"GPUHybrid": {"block_size": 7}}', C.byref(h))
    assert st == 1 and b"block_size" in L.lss_last_error(None)
    st = L.lss_create(b'{"GPUHybrid": {', C.byref(h))
    assert st == 1 and b"JSON" in L.lss_last_error(None)
    st = L.lss_create(b'{"solver": "Pardiso"}', C.byref(h))
    assert st == 10
    st = L.lss_create(b'{"gb300": {"precision": "fp16"}}', C.byref(h))
    assert st == 1
    st = L.lss_create(b'{"gb300": {"spmv_lanes": 3}}', C.byref(h))
    assert st == 1 and b"spmv_lanes" in L.lss_last_error(None)
    st = L.lss_create(b'{"gb300": {"outer_spmv": "fp32"}}', C.byref(h))
    assert st == 1 and b"outer_spmv" in L.lss_last_error(None)


def test_no_device_is_an_error_not_a_fallback(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import lss
    with pytest.raises(lss.LssError) as e:
        lss.Solver.create({"solver": "GPUHybrid"})
    assert e.value.status == "LSS_ERR_NO_DEVICE"
    with pytest.raises(lss.LssError):
        lss.row_l1_norms(__import__("scipy.sparse", fromlist=["eye"]).eye(4, format="csc"))


def test_null_arguments(built):
    import lss
    L = lss.load()
    assert L.lss_create(None, None) == 1
    assert L.lss_destroy(None) == 0
    assert L.lss_solve(None, None, None, 1, 1) == 1
    cnt = C.c_int32(0)
    assert L.lss_selected_dofs(None, None, 0, C.byref(cnt)) == 1
