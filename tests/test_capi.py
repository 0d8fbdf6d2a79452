"""The C-ABI library loads and exports every entry point include/mtgpu.h
declares; argument errors are reported without touching a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    with open(os.path.join(ROOT, "include", "mtgpu.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mtgpu_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from mtcalc_with_dfp_cocr_gb300 import build, _lib
    build.build()
    return _lib.lib()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from mtcalc_with_dfp_cocr_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_argument_errors_without_gpu(lib):
    from mtcalc_with_dfp_cocr_gb300 import _lib
    z = np.zeros(4, np.int32)
    d = np.zeros(4)
    # odd n
    rc = lib.mtgpu_pcocr_2x2_folded_ex(3, z, z, z, z, d, d, d, d, 1e-8, 10, 0, 1, 1, d, z, z, d,
                                       z, z, z, d, z, None, None)
    assert rc == _lib.MTGPU_ERR_ARG
    assert "even" in _lib.last_error()
    # a column index in the upper triangle
    ig = np.array([0, 0, 1], np.int32)
    jg = np.array([1], np.int32)
    idi = np.array([0, 2, 4], np.int32)
    ijg = np.array([0, 1], np.int32)
    rc = lib.mtgpu_mult_mv_block_2x2(2, ig, jg, idi, ijg, d, d, d, d)
    assert rc == _lib.MTGPU_ERR_ARG
    assert "lower" in _lib.last_error()


def test_receiver_argument_errors_without_gpu(lib):
    from mtcalc_with_dfp_cocr_gb300 import _lib
    pts = np.zeros(3)
    out = C.c_void_p()
    assert lib.mtgpu_receivers_create(None, 1, pts, C.byref(out)) == _lib.MTGPU_ERR_ARG
    assert "null" in _lib.last_error()
    assert lib.mtgpu_receivers_info(None, None, None, None) == _lib.MTGPU_ERR_ARG
    i1 = np.zeros(1, np.int32)
    d1 = np.ones(1)
    assert lib.mtgpu_mt_response(None, 1, d1, i1, i1, 1, None, None, None) == _lib.MTGPU_ERR_ARG


def test_adjoint_argument_errors_without_gpu(lib):
    from mtcalc_with_dfp_cocr_gb300 import _lib
    i1 = np.zeros(1, np.int32)
    d1 = np.ones(1)
    J = C.c_double()
    rc = lib.mtgpu_adjoint_source(None, 1, d1, i1, i1, 2, None, None, None, None, C.byref(J))
    assert rc == _lib.MTGPU_ERR_ARG
    rc = lib.mtgpu_adjoint_gradient(None, 1, d1, i1, 2, d1, d1, d1, None, None, None)
    assert rc == _lib.MTGPU_ERR_ARG
