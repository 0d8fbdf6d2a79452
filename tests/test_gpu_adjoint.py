"""Adjoint gradient of the impedance misfit with respect to per-cell
log-conductivity: batched (double-float) against the FP64 GPU gradient,
both against central finite differences of the FP64 forward solve, and the
torch.autograd.Function."""
import numpy as np
import pytest

from mtcalc_with_dfp_cocr_gb300 import adjoint, workloads

pytestmark = pytest.mark.gpu

FREQS = [0.1, 10.0]


def _setup(name="small", seed=11):
    w = workloads.make(name)
    m = w.mesh
    m0 = np.log(np.asarray(m.cell_sigma, np.float64))
    rng = np.random.default_rng(seed)
    # "observed" impedances from the model with the earth cells under the
    # receivers perturbed by +-0.3 in log10(sigma)
    xyz = m.xyz()
    nodes = m.cell_nodes()
    c = 0.5 * (xyz[nodes[:, 0]] + xyz[nodes[:, 7]])
    earth_core = (c[:, 2] < 0) & (np.abs(c[:, 0]) < 200) & (np.abs(c[:, 1]) < 200)
    m_true = m0.copy()
    m_true[earth_core] += 0.3 * np.log(10.0) * rng.choice([-1.0, 1.0], earth_core.sum())
    return w, m0, m_true, earth_core, rng


@pytest.fixture(scope="module")
def case(gpu):
    w, m0, m_true, earth_core, rng = _setup()
    p64 = adjoint.ImpedanceProblem(w.mesh, FREQS, w.receivers, solver="fp64", eps=1e-11)
    resp, _ = p64.forward(m_true)
    z_obs = adjoint.impedances(resp).cpu().numpy()
    p64.set_observed(z_obs)
    pb = adjoint.ImpedanceProblem(w.mesh, FREQS, w.receivers, z_obs=z_obs, solver="batched",
                                  eps=1e-10)
    return w, m0, earth_core, rng, p64, pb


def test_batched_gradient_matches_fp64_gradient(case):
    w, m0, earth_core, rng, p64, pb = case
    J64, st64 = p64.misfit(m0)
    g64 = p64.gradient(st64).cpu().numpy()
    Jb, stb = pb.misfit(m0)
    gb = pb.gradient(stb).cpu().numpy()
    assert J64 > 0
    assert abs(Jb - J64) <= 1e-8 * J64
    earth = np.asarray(w.mesh.cell_sigma0) > 1e-6
    err = np.linalg.norm((gb - g64)[earth]) / np.linalg.norm(g64[earth])
    assert err < 1e-6, err


def test_fp64_gradient_matches_central_differences(case):
    w, m0, earth_core, rng, p64, pb = case
    J0, st = p64.misfit(m0)
    g = p64.gradient(st).cpu().numpy()
    cand = np.nonzero(earth_core)[0]
    cells = rng.choice(cand, 6, replace=False)
    h = 1e-4
    for c in cells:
        mp, mm = m0.copy(), m0.copy()
        mp[c] += h
        mm[c] -= h
        fd = (p64.misfit(mp)[0] - p64.misfit(mm)[0]) / (2 * h)
        assert abs(fd - g[c]) <= 1e-4 * abs(g[c]) + 1e-6 * np.abs(g).max(), (c, fd, g[c])


def test_autograd_function(case):
    import torch
    w, m0, earth_core, rng, p64, pb = case
    t = torch.tensor(m0, dtype=torch.float64, requires_grad=True)
    J = adjoint.ImpedanceMisfit.apply(t, pb)
    J.backward()
    J2, st = pb.misfit(m0)
    g = pb.gradient(st).cpu().numpy()
    assert float(J.detach()) == pytest.approx(J2, rel=1e-12)
    np.testing.assert_allclose(t.grad.numpy(), g, rtol=1e-9, atol=1e-12 * np.abs(g).max())


def test_batched_problem_with_more_than_16_frequencies(gpu):
    """More than 16 frequencies (over 32 systems: two solver batches in one
    survey) in the batched problem: the misfit equals the FP64 problem's."""
    w, m0, m_true, earth_core, rng = _setup()
    freqs = list(np.logspace(-1, 2, 17))
    p64 = adjoint.ImpedanceProblem(w.mesh, freqs, w.receivers, solver="fp64", eps=1e-11)
    resp, _ = p64.forward(m_true)
    z_obs = adjoint.impedances(resp).cpu().numpy()
    p64.set_observed(z_obs)
    pb = adjoint.ImpedanceProblem(w.mesh, freqs, w.receivers, z_obs=z_obs, solver="batched",
                                  eps=1e-10)
    J64, _ = p64.misfit(m0)
    Jb, _ = pb.misfit(m0)
    assert J64 > 0.0
    assert abs(Jb - J64) <= 1e-6 * abs(J64)
