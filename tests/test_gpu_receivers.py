"""Receiver fields and MT responses on the GPU against the oracle (whose
receiver evaluation is pinned to the reference's own OutputNu code and whose
normal field is pinned to the reference Harm1D's e2d / b2d)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mtcalc_with_dfp_cocr_gb300 import assembly, normal1d, receivers, slae_io, survey, workloads
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

TWO_PI = 2.0 * 3.1415926535897932384626433832795


def _oracle_fields(m, rec, v3, nu, alfa, z1d, us, uc):
    a, curl = O.receiver_eval(m, rec, v3)
    e1, b1 = O.normal_field(rec, z1d, us, uc, alfa, TWO_PI * nu)
    return O.receiver_fields(a, curl, TWO_PI * nu, e1, b1)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def small_fixture(gpu):
    torch = gpu
    g = np.load(os.path.join(GOLDEN, "receivers_small.npz"))
    m = workloads.make("small").mesh
    A = assembly.Assembly(m)
    R = receivers.Receivers(A, g["rec"])
    nu = float(g["nu"])
    x = torch.tensor(np.stack([g["v3_x"], g["v3_y"]]), dtype=torch.float64, device="cuda")
    us = np.stack([g["usin_x"], g["usin_y"]])
    uc = np.stack([g["ucos_x"], g["ucos_y"]])
    E, H, S = R.fields(x, [nu, nu], [1, 0], g["z1d_x"], us, uc)
    return g, m, A, R, E.cpu().numpy(), H.cpu().numpy(), S.cpu().numpy(), E, H


def test_location_matches_oracle(small_fixture):
    g, m, A, R, *_ = small_fixture
    miss, elem = R.info()
    assert miss == 0
    np.testing.assert_array_equal(elem, O.locate_receivers(m, g["rec"]))


def test_fields_match_oracle_on_reference_solutions(small_fixture):
    g, m, A, R, E, H, S, *_ = small_fixture
    nu = float(g["nu"])
    for k, (p, alfa) in enumerate((("x", 1), ("y", 0))):
        e, h, s = _oracle_fields(m, g["rec"], g[f"v3_{p}"], nu, alfa, g[f"z1d_{p}"],
                                 g[f"usin_{p}"], g[f"ucos_{p}"])
        assert _rel(E[k], e) < 1e-13
        # H: the anomalous part is curl A, which cancels ~4 digits in the air
        assert _rel(H[k], h) < 1e-11
        assert _rel(S[k], s) < 1e-11


def test_mt_response_matches_oracle(small_fixture):
    g, m, A, R, E, H, S, Et, Ht = small_fixture
    nu = float(g["nu"])
    out = R.mt_response([nu], [0], [1], Et, Ht).cpu().numpy()[0]
    for r in range(R.nrec):
        ref = O.mt_response(E[0, r], H[0, r], E[1, r], H[1, r], TWO_PI * nu)
        zs = np.abs(ref[:8]).max()
        np.testing.assert_allclose(out[r, :8], ref[:8], rtol=0, atol=1e-12 * zs)
        np.testing.assert_allclose(out[r, 8:12], ref[8:12], rtol=0, atol=1e-11)
        np.testing.assert_allclose(out[r, 12:16], ref[12:16], rtol=1e-11, atol=1e-12 * zs)
        np.testing.assert_allclose(out[r, 20:24], ref[20:24], rtol=1e-11,
                                   atol=1e-11 * ref[20:24].max())
        np.testing.assert_allclose(out[r, 28], ref[28], rtol=1e-11)
        np.testing.assert_allclose(out[r, 30:32], ref[30:32], rtol=1e-10, atol=1e-12)
        # phases: degrees, near +-180 a sign flip is the same angle
        for i in list(range(16, 20)) + list(range(24, 28)) + [29, 32, 33]:
            d = abs(out[r, i] - ref[i]) % 360.0
            assert min(d, 360.0 - d) < 1e-7, (r, i, out[r, i], ref[i])


def test_unlocated_receiver_gets_normal_field(gpu):
    torch = gpu
    m = workloads.make("tiny").mesh
    A = assembly.Assembly(m)
    rec = np.array([[0.0, 0.0, 0.0], [1e7, 0.0, 0.0]])
    R = receivers.Receivers(A, rec)
    miss, elem = R.info()
    assert miss == 1 and elem[1] == -1 and elem[0] >= 0
    tops, sig = [l.top for l in m.layers], [l.sigma for l in m.layers]
    z1d, us, uc = normal1d.solve_1d(1.0, tops, sig)
    x = torch.zeros(1, 2 * m.nb, dtype=torch.float64, device="cuda")
    E, H, _ = R.fields(x, [1.0], [1], z1d, us[None], uc[None])
    e1, b1 = O.normal_field(rec, z1d, us, uc, 1, TWO_PI)
    z = np.zeros((2, 3), complex)
    e, h, _ = O.receiver_fields(z, z, TWO_PI, e1, b1)
    np.testing.assert_allclose(E[0].cpu().numpy(), e, rtol=1e-14, atol=0)
    np.testing.assert_allclose(H[0].cpu().numpy(), h, rtol=1e-14, atol=0)


def test_survey_to_impedance_pipeline(gpu):
    """Assembly -> batched survey solve -> receivers -> MT responses, all on
    the GPU, against the oracle's FP64 pipeline on the same systems."""
    torch = gpu
    w = workloads.make("small")
    freqs = [0.1, 10.0]
    systems = [(f, a) for f in freqs for a in (1, 0)]
    nus = [f for f, _ in systems]
    alfas = [a for _, a in systems]
    tops, sig = [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers]
    tabs = [normal1d.solve_1d(nu, tops, sig) for nu in nus]
    A = assembly.Assembly(w.mesh)
    S = len(systems)
    b = torch.empty(S, 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    us, uc = np.stack([t[1] for t in tabs]), np.stack([t[2] for t in tabs])
    A.rhs(nus, alfas, tabs[0][0], us, uc, b)
    x = torch.zeros_like(b)
    code, st = survey.Survey(A, nus).solve(b, x, eps=1e-8, verify=True)
    assert code == 0
    R = receivers.Receivers(A, w.receivers)
    E, H, _ = R.fields(x, nus, alfas, tabs[0][0], us, uc)
    out = R.mt_response(freqs, [0, 2], [1, 3], E, H).cpu().numpy()

    mesh = slae_io.mesh_to_solve_mesh(w.mesh)
    fields = []
    for k, (nu, alfa) in enumerate(systems):
        s = O.assemble(w.mesh, nu, alfa, *tabs[k])
        c, x64, _ = O.pcocr(s, mesh, nthreads=4)
        assert c == 0
        fields.append(_oracle_fields(w.mesh, w.receivers, x64, nu, alfa, *tabs[k]))
    for f, nu in enumerate(freqs):
        (e0, h0, _), (e1, h1, _) = fields[2 * f], fields[2 * f + 1]
        for r in range(R.nrec):
            ref = O.mt_response(e0[r], h0[r], e1[r], h1[r], TWO_PI * nu)
            zs = np.abs(ref[:8]).max()
            # two independent solves to 1e-8 relative residual
            np.testing.assert_allclose(out[f, r, :8], ref[:8], rtol=0, atol=1e-6 * zs)
            np.testing.assert_allclose(out[f, r, 21:23], ref[21:23], rtol=1e-6)
            np.testing.assert_allclose(out[f, r, 17:19], ref[17:19], rtol=0, atol=1e-4)
