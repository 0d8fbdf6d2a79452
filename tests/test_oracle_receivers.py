"""The receiver / MT-response restatement in the oracle, pinned against the
reference: the receiver evaluation against the reference's own
OutputVect3d::OutputFieldAtReceivers (fixture from
tests/golden/make_golden_receivers.py), the normal field against the
reference Harm1D's e2d / b2d, and the impedance solve (calcimpedance.for,
for which no Fortran compiler exists here) against exact algebraic and
physical identities."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import pyoracle as P
from mtcalc_with_dfp_cocr_gb300 import normal1d, workloads

MU0_OUT = 1.25663706143591729e-6          # Code/OutputNu/stdafx.h:31
TWO_PI = 2.0 * 3.1415926535897932384626433832795


@pytest.fixture(scope="module")
def rcv():
    return np.load(os.path.join(GOLDEN, "receivers_small.npz")), workloads.make("small").mesh


def brute_force_elements(m, rec):
    nodes = m.cell_nodes()
    xyz = m.xyz()
    lo, hi = xyz[nodes[:, 0]], xyz[nodes[:, 7]]
    out = []
    for p in rec:
        inside = np.all((p >= lo) & (p <= hi), axis=1)
        out.append(int(np.argmax(inside)) if inside.any() else -1)
    return np.array(out)


def test_locate_first_containing_element(rcv):
    g, m = rcv
    elem = P.locate_receivers(m, g["rec"])
    assert (elem >= 0).all()
    np.testing.assert_array_equal(elem, brute_force_elements(m, g["rec"]))
    # a surface receiver on cell corners lies in 8 cells; the lowest index
    # (below the surface, lowest x and y) wins
    z0 = m.xyz()[m.cell_nodes()[elem, 7], 2]
    assert (z0[:9] == 0.0).all()


def test_locate_outside_mesh():
    m = workloads.make("tiny").mesh
    rec = np.array([[1e7, 0.0, 0.0], [0.0, 0.0, 0.0]])
    elem = P.locate_receivers(m, rec)
    assert elem[0] == -1 and elem[1] >= 0


@pytest.mark.parametrize("pol", ["x", "y"])
def test_receiver_eval_matches_reference(rcv, pol):
    g, m = rcv
    a, curl = P.receiver_eval(m, g["rec"], g[f"v3_{pol}"])
    ra, rc = g[f"ref_a_{pol}"], g[f"ref_curl_{pol}"]
    # A: the same products in the same order up to grouping
    assert np.abs(a - ra).max() <= 1e-14 * np.abs(ra).max()
    # curl A cancels ~4 digits of the gauge-dominated air potential; the
    # grouping of the 8 terms differs from the reference's, so compare
    # against the largest component at 1e-11
    assert np.abs(curl - rc).max() <= 1e-11 * np.abs(rc).max()


@pytest.mark.parametrize("pol", ["x", "y"])
def test_normal_field_matches_harm1d(rcv, pol):
    g, m = rcv
    alfa = 1 if pol == "x" else 0
    e, b = P.normal_field(g["rec"], g[f"z1d_{pol}"], g[f"usin_{pol}"], g[f"ucos_{pol}"], alfa,
                          TWO_PI * float(g["nu"]))
    # e2d / b2d are printed with 15 significant digits; the tables with 14
    np.testing.assert_allclose(e, g[f"e2d_{pol}"], rtol=0, atol=1e-12 * np.abs(e).max())
    np.testing.assert_allclose(b, g[f"b2d_{pol}"], rtol=0, atol=1e-12 * np.abs(b).max())


def test_dspline_cases():
    z = np.array([-3.0, -2.0, -1.0, 0.0])
    v = z ** 2
    assert P.dspline(-1.0, z, v) == pytest.approx(-2.0)        # interior node
    assert P.dspline(-3.5, z, v) == pytest.approx(-5.0)        # below: end slope
    assert P.dspline(0.5, z, v) == pytest.approx(-1.0)         # above: end slope
    assert P.dspline(-2.0, z, v) == pytest.approx(-5.0)        # first node: interval slope


def test_receiver_fields_conventions(rcv):
    g, m = rcv
    w = TWO_PI * float(g["nu"])
    a, curl = P.receiver_eval(m, g["rec"], g["v3_x"])
    zero = np.zeros((len(a), 6))
    e, h, s = P.receiver_fields(a, curl, w, zero, zero)
    np.testing.assert_allclose(e, -1j * w * a, rtol=1e-15, atol=0)
    np.testing.assert_allclose(h, curl / MU0_OUT, rtol=1e-15, atol=0)
    # the normal field goes to x and y only
    e1 = np.tile(np.arange(1.0, 7.0), (len(a), 1))
    e2, h2, _ = P.receiver_fields(a, curl, w, e1, 2 * e1)
    np.testing.assert_allclose(e2[:, :2] - e[:, :2], [[1 + 4j, 2 + 5j]] * len(a), rtol=1e-12)
    np.testing.assert_allclose(h2[:, :2] - h[:, :2], [[2 + 8j, 4 + 10j]] / np.float64(MU0_OUT)
                               * np.ones((len(a), 1)), rtol=1e-12)
    assert (e2[:, 2] == e[:, 2]).all() and (h2[:, 2] == h[:, 2]).all()
    ere, eim = np.linalg.norm(e2.real, axis=1), np.linalg.norm(e2.imag, axis=1)
    hre, him = np.linalg.norm(h2.real, axis=1), np.linalg.norm(h2.imag, axis=1)
    ratio = np.hypot(ere, eim) / np.hypot(hre, him)
    _, _, s2 = P.receiver_fields(a, curl, w, e1, 2 * e1)
    np.testing.assert_allclose(s2[:, 1], ratio, rtol=1e-14)
    np.testing.assert_allclose(s2[:, 0], ratio ** 2 / (w * MU0_OUT), rtol=1e-14)


def test_mt_response_recovers_impedance_and_tipper():
    rng = np.random.default_rng(7)
    for _ in range(20):
        Z = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
        W = rng.standard_normal(2) + 1j * rng.standard_normal(2)
        H = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))  # [pol][x, y]
        E = H @ Z.T                                   # E_pol = Z H_pol
        hz = H @ W
        h0 = np.array([H[0, 0], H[0, 1], hz[0]])
        h1 = np.array([H[1, 0], H[1, 1], hz[1]])
        e0 = np.array([E[0, 0], E[0, 1], 0])
        e1 = np.array([E[1, 0], E[1, 1], 0])
        w = 3.0
        out = P.mt_response(e0, h0, e1, h1, w)
        z = out[0:8].view(np.complex128)
        np.testing.assert_allclose(z, Z.ravel(), rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(out[8:12].view(np.complex128), W, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(out[12:16], np.abs(Z.ravel()), rtol=1e-12)
        np.testing.assert_allclose(out[16:20], -np.degrees(np.angle(Z.ravel())), atol=1e-9)
        mu0 = 4e-7 * np.pi
        np.testing.assert_allclose(out[20:24], np.abs(Z.ravel()) ** 2 / (mu0 * w), rtol=1e-12)
        np.testing.assert_allclose(out[24:28], 2 * out[16:20], rtol=1e-12)
        det = np.linalg.det(Z)
        np.testing.assert_allclose(out[28], abs(det) / (mu0 * w), rtol=1e-12)
        np.testing.assert_allclose(out[29], -np.degrees(np.angle(det)), atol=1e-9)
        np.testing.assert_allclose(out[30:32], np.abs(W), rtol=1e-12)
        np.testing.assert_allclose(out[32:34], -np.degrees(np.angle(W)), atol=1e-9)


def test_mt_phase_axis_rules():
    # calcimpedance.for:163-171: near-axis overrides; exact zero -> 0 here
    h0 = np.array([1.0, 0.0, 0.0], complex)
    h1 = np.array([0.0, 1.0, 0.0], complex)
    for zxx, phase in ((1.0, 0.0), (1j, 90.0), (-1.0, 180.0), (-1j, -90.0), (0.0, 0.0),
                       (-1.0 - 1e-16j, 180.0)):
        out = P.mt_response(np.array([zxx, 0, 0]), h0, np.array([0, 0, 0]), h1, 1.0)
        assert out[16] == pytest.approx(-phase)


@pytest.mark.parametrize("sigma", [0.01, 0.1])
def test_half_space_apparent_resistivity(sigma):
    """A homogeneous half-space has no anomalous field: rho_a = 1/sigma and a
    45-degree impedance phase from the normal field alone."""
    nu = 1.0
    w = TWO_PI * nu
    z1d, us, uc = normal1d.solve_1d(nu, [0.0], [sigma])
    rec = np.zeros((1, 3))
    fields = []
    for alfa in (1, 0):
        e, b = P.normal_field(rec, z1d, us, uc, alfa, w)
        a0 = np.zeros((1, 3), complex)
        E, H, _ = P.receiver_fields(a0, a0, w, e, b)
        fields.append((E[0], H[0]))
    out = P.mt_response(fields[0][0], fields[0][1], fields[1][0], fields[1][1], w)
    assert out[21] == pytest.approx(1.0 / sigma, rel=1e-4)       # rho_xy
    assert out[22] == pytest.approx(1.0 / sigma, rel=1e-4)       # rho_yx
    assert abs(out[17]) == pytest.approx(135.0, abs=1e-4)        # phase of Zxy
    assert out[18] == pytest.approx(-45.0, abs=1e-4)             # phase of Zyx
    assert out[12] == 0.0 and out[15] == 0.0                     # Zxx = Zyy = 0


def test_dtm_fixture_mesh():
    """The fixture of the published DTM case rebuilds the reference
    RegularMeshBuilder's mesh: air above z = 0, the 0.01 S/m half-space as
    background everywhere below, the three objects' conductivities."""
    from mtcalc_with_dfp_cocr_gb300 import mesh as M
    g = np.load(os.path.join(GOLDEN, "dtm_625_500.npz"))
    cm = g["cell_mat"].astype(np.int64)
    layers = [M.Layer(float(t), float(s)) for t, s in zip(g["layer_tops"], g["layer_sigma"])]
    m = M.RegularMesh(g["x"], g["y"], g["z"], layers, g["mat_sigma"][cm], g["mat_sigma0"][cm])
    assert (m.nx, m.ny, m.nz) == (104, 144, 28) and m.nb == 1236064
    zc = 0.5 * (g["z"][:-1] + g["z"][1:])
    cz = np.repeat(zc, (m.nx - 1) * (m.ny - 1))
    assert np.all(m.cell_sigma[cz > 0] == 1e-8)
    assert np.all(m.cell_sigma0[cz < 0] == 0.01)
    assert set(np.unique(m.cell_sigma[cz < 0])) == {1e-4, 1e-2, 1e-1, 1.0}
    assert g["published"].shape == (53, 21, 8) and len(g["periods"]) == 21


@pytest.mark.parametrize("prefix,steps", [("", (625.0, 500.0)), ("ex_", None)])
def test_meshbuilder_matches_reference_builder(prefix, steps):
    """meshbuilder.build_mesh on the reference's example inputs reproduces
    the reference RegularMeshBuilder's mesh lines bit for bit and its cell
    conductivities, at the published run's 625/500 m steps and at the
    example's own settings."""
    from mtcalc_with_dfp_cocr_gb300 import meshbuilder as MB
    g = np.load(os.path.join(GOLDEN, "dtm_625_500.npz"))
    case = MB.Case(
        freqs=1.0 / g["periods"], receivers=g["receivers"],
        layers=[MB.Layer(float(t), float(s)) for t, s in zip(g["layer_tops"], g["layer_sigma"])],
        objects=g["objects"], steps=steps or tuple(g["settings"][0]),
        sparse=tuple(g["settings"][1]), gap=tuple(g["settings"][2]),
        far=tuple(g["settings"][3]), eps=1e-4, maxiter=10000)
    m = MB.build_mesh(case)
    for a, b in ((m.x, g[prefix + "x"]), (m.y, g[prefix + "y"]), (m.z, g[prefix + "z"])):
        np.testing.assert_array_equal(a, b)
    cm = g[prefix + "cell_mat"].astype(np.int64)
    np.testing.assert_array_equal(m.cell_sigma, g[prefix + "mat_sigma"][cm])
    np.testing.assert_array_equal(m.cell_sigma0, g[prefix + "mat_sigma0"][cm])


def test_driver_table_layout(tmp_path):
    """The survey driver's results table has the published table's layout:
    per receiver and ascending period, northing = x, easting = -y, |Z| and
    rho_a of the four components."""
    from mtcalc_with_dfp_cocr_gb300 import calc, meshbuilder as MB
    case = MB.Case(freqs=np.array([0.1, 10.0]), receivers=np.array([[1.0, 2.0, 0.0]]),
                   layers=[MB.Layer(0.0, 0.01)], objects=np.zeros((0, 7)),
                   steps=(100.0, 100.0), sparse=(1.5, 1.5), gap=(100.0, 100.0),
                   far=(1000.0, 1000.0), eps=1e-8, maxiter=10)
    resp = np.zeros((2, 1, 34))
    resp[:, 0, 12:16] = [[1, 2, 3, 4], [5, 6, 7, 8]]
    resp[:, 0, 20:24] = [[9, 10, 11, 12], [13, 14, 15, 16]]
    out = str(tmp_path / "t.txt")
    calc.write_table(out, case, resp)
    tab = np.loadtxt(out, skiprows=1)
    np.testing.assert_allclose(tab[0], [1, -2, 0.1, 5, 6, 7, 8, 13, 14, 15, 16])
    np.testing.assert_allclose(tab[1], [1, -2, 10.0, 1, 2, 3, 4, 9, 10, 11, 12])


def test_impedance_result_files(tmp_path):
    """calcimpedance's result files and ImpedanceZToEdsAll's edsall0_0_imp
    from MT records: 4-byte records receiver-major with the frequencies in
    list order (calcimpedance.for:240-301, 430-465); edsall blocks per type
    (|Z|, phase, rho_a, rho_a phase), component and receiver with the
    frequencies reversed and the phases folded (main.cpp:318-347, 578-606).
    The records come from the oracle's impedance solve on synthetic fields."""
    from mtcalc_with_dfp_cocr_gb300 import edsall
    rng = np.random.default_rng(3)
    freqs = np.array([0.1, 1.0, 10.0])
    rec = np.array([[100.0, -250.5, 0.0], [1.0e4, 2.0e3, -5.0]])
    resp = np.zeros((3, 2, 34))
    for f, nu in enumerate(freqs):
        for r in range(2):
            e0, h0, e1, h1 = (rng.standard_normal(3) + 1j * rng.standard_normal(3) for _ in range(4))
            resp[f, r] = P.mt_response(e0, h0, e1, h1, 2 * np.pi * nu)
    out = str(tmp_path)
    names = edsall.write_results(out, freqs, rec, resp)
    assert {"Zxy", "Fyx", "Rxx", "Fiyy", "Reff", "Fieff", "Wzx", "WFzy", "ZxyRe", "WzyIm"} <= set(names)
    zxy = edsall.read_result(out, "Zxy", 2, 3)
    np.testing.assert_allclose(zxy, resp[:, :, 13].T.astype(np.float32))
    np.testing.assert_allclose(edsall.read_result(out, "Reff", 2, 3), resp[:, :, 28].T.astype(np.float32))
    lines = open(os.path.join(out, "edsall0_0_imp")).read().splitlines()
    block = 6 + len(freqs)
    assert len(lines) == 4 * 4 * 2 * block
    assert open(os.path.join(out, "ft0_0")).read().split() == [str(t) for t in (1, 2, 3, 4)
                                                               for _ in range(4 * 2)]
    # type 1 (|Z|), component xy (the second group of 2 receivers), receiver 1
    b = lines[(1 * 2 + 1) * block:(1 * 2 + 2) * block]
    assert b[0] == "10000 2000" and b[1] == "10000 2000 -5"
    assert b[2:5] == ["1", "1 1 1 1", "1"] and b[5] == "\tnu\tUn\tUa\tUs"
    rows = [list(map(float, l.split())) for l in b[6:]]
    np.testing.assert_allclose([r_[0] for r_ in rows], freqs[::-1])
    np.testing.assert_allclose([r_[2] for r_ in rows], zxy[1, ::-1], rtol=1e-5)
    assert all(r_[1] == 0.0 and r_[2] == r_[3] for r_ in rows)
    # type 2 (phase), component yx, receiver 0: -arg Zyx folded as the reference folds it
    b = lines[(4 * 2 + 2 * 2) * block:(4 * 2 + 2 * 2 + 1) * block]
    f = edsall.read_result(out, "Fyx", 2, 3)[0, ::-1].astype(np.float64)
    f[f > 180.0] -= 180.0
    f[f < -180.0] += 180.0
    np.testing.assert_allclose([float(l.split()[2]) for l in b[6:]], f, rtol=1e-5, atol=1e-4)
