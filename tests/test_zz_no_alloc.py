"""The allocation-free SpMV entry point, mtgpu_mult_mv_block_2x2_noalloc.

It exists for callers that own every GPU buffer (their own pool or caching
allocator) and must not have the library call cudaMalloc.  The test keeps the
matrix and vectors in caller-owned device memory (torch tensors here), calls
the entry point twice in a row through the C ABI -- the second call must not
see the first call's leftovers in the shared static scratch -- and compares
each result with the oracle's port of the reference's Mult_MV_block_2x2
(Code/COCR_FP/block_2x2_solver.cpp:73-173) on the CPU, within the tolerance
of the other SpMV tests.  It is collected last so that a run stopping at the
first failure has run every other test already.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from mtcalc_with_dfp_cocr_gb300 import _lib, normal1d, workloads
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _device_slae(torch, s, base=0):
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    return dict(ig=t(s.ig + base, torch.int32), jg=t(s.jg + base, torch.int32),
                idi=t(s.idi + base, torch.int32), ijg=t(s.ijg + base, torch.int32),
                di=t(s.di, torch.float64), gg=t(s.gg, torch.float64))


def _noalloc_spmv(torch, d, nb, x):
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    dy = torch.full_like(dx, float("nan"))          # the call must write every entry
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    torch.cuda.synchronize()
    rc = _lib.lib().mtgpu_mult_mv_block_2x2_noalloc(
        nb, p(d["ig"]), p(d["jg"]), p(d["idi"]), p(d["ijg"]), p(d["di"]), p(d["gg"]), p(dx), p(dy),
        p(status), None)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    return dy.cpu().numpy(), int(status.item())


def _c1_slae():
    w = workloads.make("c1")
    z, us, uc = normal1d.solve_1d(1.0, [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers])
    return O.assemble(w.mesh, 1.0, 1, z, us, uc)


@pytest.mark.parametrize("case", ["small", "c1"])
def test_noalloc_matches_oracle_twice(gpu, case):
    torch = gpu
    s = load_golden(case)[1] if case == "small" else _c1_slae()
    d = _device_slae(torch, s)
    rng = np.random.default_rng(11)
    for call in range(2):
        x = rng.standard_normal(s.n) * (10.0 if call else 1.0)
        y, status = _noalloc_spmv(torch, d, s.nb, x)
        y_ref = O.spmv(s, x)
        assert status == 0
        assert np.all(np.isfinite(y))
        assert np.max(np.abs(y - y_ref)) <= 1e-14 * np.max(np.abs(y_ref)), call


def test_noalloc_flags_one_based_arrays(gpu):
    # the reference's files are 1-based; passed unchanged, the kernels read
    # only the first element of each index array and report it
    torch = gpu
    s = load_golden("small")[1]
    d = _device_slae(torch, s, base=1)
    _, status = _noalloc_spmv(torch, d, s.nb, np.ones(s.n))
    assert status == _lib.MTGPU_NOALLOC_NOT_ZERO_BASED


def test_noalloc_rejects_too_many_edges(gpu):
    rc = _lib.lib().mtgpu_mult_mv_block_2x2_noalloc(
        (1 << 20) + 1, *([C.c_void_p(16)] * 9), None)
    assert rc == _lib.MTGPU_ERR_ARG
    assert "1048576" in _lib.last_error()
