"""The smoothing receiver output (the reference's default OutputNu path) on
the GPU against the restatement oracle/smoothing.py, which is pinned to the
reference's own smoothing classes (tests/test_oracle_smoothing.py)."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from mtcalc_with_dfp_cocr_gb300 import assembly, normal1d, receivers, workloads
from oracle import pyoracle as O
from oracle import smoothing

sys.path.insert(0, GOLDEN)
from make_golden_smoothing import c1_values  # noqa: E402

pytestmark = pytest.mark.gpu

TWO_PI = 2.0 * 3.1415926535897932384626433832795


def _oracle_totals(m, rec, v3, nu, alfa, z1d, us, uc):
    a, curl = smoothing.smoothed_fields(m, rec, v3)
    e1, b1 = O.normal_field(rec, z1d, us, uc, alfa, TWO_PI * nu)
    return O.receiver_fields(a, curl, TWO_PI * nu, e1, b1)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "smoothing.npz"))


def test_small_reference_solutions(gpu, golden):
    torch = gpu
    r = np.load(os.path.join(GOLDEN, "receivers_small.npz"))
    m = workloads.make("small").mesh
    A = assembly.Assembly(m)
    rec = golden["rec_small"]
    R = receivers.Receivers(A, rec, output="smooth")
    nu = float(r["nu"])
    x = torch.tensor(np.stack([r["v3_x"], r["v3_y"]]), dtype=torch.float64, device="cuda")
    us = np.stack([r["usin_x"], r["usin_y"]])
    uc = np.stack([r["ucos_x"], r["ucos_y"]])
    E, H, S = R.fields(x, [nu, nu], [1, 0], r["z1d_x"], us, uc)
    E, H, S = E.cpu().numpy(), H.cpu().numpy(), S.cpu().numpy()
    info = R.smoothing_info()
    np.testing.assert_array_equal(np.stack([info["nodes"], info["cells"]], 1), golden["sub_small"])
    assert 0 < info["iterations"] <= 200
    for k, (p, alfa) in enumerate((("x", 1), ("y", 0))):
        e, h, s = _oracle_totals(m, rec, r[f"v3_{p}"], nu, alfa, r[f"z1d_{p}"], r[f"usin_{p}"],
                                 r[f"ucos_{p}"])
        assert _rel(E[k], e) < 1e-11
        assert _rel(H[k], h) < 1e-10
        assert _rel(S[k], s) < 1e-10
    # the smoothed output differs from the direct one by the smoothing itself
    Rd = receivers.Receivers(A, rec)
    Ed, Hd, _ = Rd.fields(x, [nu, nu], [1, 0], r["z1d_x"], us, uc)
    assert 1e-6 < _rel(Ed.cpu().numpy(), E) < 0.5


def test_c1_batched_random_values(gpu, golden):
    """Four systems at once (random edge values, two frequencies and both
    polarisations): every system as the oracle smooths it alone."""
    torch = gpu
    w = workloads.make("c1")
    m = w.mesh
    A = assembly.Assembly(m)
    rec = golden["rec_c1"]
    R = receivers.Receivers(A, rec, output="smooth")
    info = R.smoothing_info()
    np.testing.assert_array_equal(np.stack([info["nodes"], info["cells"]], 1), golden["sub_c1"])
    vals = [c1_values(m.nb, golden["seed_c1"] + k).ravel() for k in range(4)]
    nus = [0.1, 0.1, 10.0, 10.0]
    alfas = [1, 0, 1, 0]
    tops = [l.top for l in m.layers]
    sig = [l.sigma for l in m.layers]
    tabs = [normal1d.solve_1d(nu, tops, sig) for nu in nus]
    z1d = tabs[0][0]
    us = np.stack([t[1] for t in tabs])
    uc = np.stack([t[2] for t in tabs])
    x = torch.tensor(np.stack(vals), dtype=torch.float64, device="cuda")
    E, H, S = R.fields(x, nus, alfas, z1d, us, uc)
    E, H = E.cpu().numpy(), H.cpu().numpy()
    for k in range(4):
        e, h, _ = _oracle_totals(m, rec, vals[k], nus[k], alfas[k], z1d, us[k], uc[k])
        assert _rel(E[k], e) < 1e-11, k
        assert _rel(H[k], h) < 1e-10, k


def test_adjoint_refuses_smoothed_receivers(gpu):
    torch = gpu
    m = workloads.make("tiny").mesh
    A = assembly.Assembly(m)
    R = receivers.Receivers(A, [[0.0, 0.0, 0.0]], output="smooth")
    from mtcalc_with_dfp_cocr_gb300 import _lib
    import ctypes as C
    e = torch.zeros(2 * 6, dtype=torch.float64, device="cuda")
    z = torch.zeros(8, dtype=torch.float64, device="cuda")
    src = torch.zeros(2 * 2 * m.nb, dtype=torch.float64, device="cuda")
    rc = _lib.lib().mtgpu_adjoint_source(
        R._h, 1, np.array([1.0]), np.array([0], np.int32), np.array([1], np.int32), 2,
        C.c_void_p(e.data_ptr()), C.c_void_p(e.data_ptr()), C.c_void_p(z.data_ptr()),
        C.c_void_p(src.data_ptr()), None)
    assert rc == -101
