"""GPU parity: libmtgpu through its C ABI against the CPU oracle and the
reference's golden outputs."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, load_golden
from mtcalc_with_dfp_cocr_gb300 import normal1d, slae_io, solver, workloads
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _c1_system(alfa=1):
    w = workloads.make("c1")
    z, us, uc = normal1d.solve_1d(1.0, [l.top for l in w.mesh.layers],
                                  [l.sigma for l in w.mesh.layers])
    return w, O.assemble(w.mesh, 1.0, alfa, z, us, uc), slae_io.mesh_to_solve_mesh(w.mesh)


def _true_rel_res(slae, x):
    r = slae.pr - O.spmv(slae, x)
    return np.linalg.norm(r) / np.linalg.norm(slae.pr)


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_spmv_parity(gpu, name):
    w, s, *_ = load_golden(name)
    x = np.random.default_rng(3).standard_normal(s.n)
    y = solver.mult_mv_block_2x2(s, x)
    yo = O.spmv(s, x)
    assert np.max(np.abs(y - yo)) <= 1e-14 * np.max(np.abs(yo))


def test_spmv_parity_c1(gpu):
    w, s, mesh = _c1_system()
    x = np.random.default_rng(4).standard_normal(s.n)
    y = solver.mult_mv_block_2x2(s, x)
    yo = O.spmv(s, x)
    assert np.max(np.abs(y - yo)) <= 1e-14 * np.max(np.abs(yo))


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_folded_preconditioner_parity(gpu, name):
    w, s, mesh, *_ = load_golden(name)
    x = np.random.default_rng(5).standard_normal(s.n)
    y, da, ds = solver.folded_apply(s, mesh, x)
    yo, dao, dso = O.folded_apply(s, mesh, x)
    assert len(ds) == len(dso)
    assert np.max(np.abs(da - dao)) <= 1e-14 * np.max(np.abs(dao))
    # Re diag(G A G^T) is a cancellation (the curl-curl part annihilates
    # gradients), so D_S in the air depends on the summation order; the GPU
    # set-up adds in the reference's order, which keeps D_S to ~1e-15.
    dsc, dsoc = ds[0::2] + 1j * ds[1::2], dso[0::2] + 1j * dso[1::2]
    assert np.max(np.abs(dsc - dsoc) / np.abs(dsoc)) <= 1e-13
    assert np.max(np.abs(y - yo)) <= 1e-12 * np.max(np.abs(yo))


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_solve_parity_golden(gpu, name):
    """Same stop rule as the reference; the GPU sums in a different order, so
    the iterate drifts at roundoff level (the reference itself moves ~1e-7
    between 1 and 7 OpenMP threads)."""
    w, s, mesh, z1d, us, uc, v3, kit_iter, kit_r, nu, alfa = load_golden(name)
    code, x, st = solver.pcocr_2x2_folded(s, mesh)
    assert code == 0
    assert abs(st.iterations - kit_iter) <= 2
    assert st.residual_rel < s.eps
    assert np.linalg.norm(x - v3) <= 1e-6 * np.linalg.norm(v3)
    assert abs(st.true_residual_rel - _true_rel_res(s, x)) <= 1e-3 * st.true_residual_rel


def test_solve_parity_c1(gpu):
    with open(os.path.join(GOLDEN, "c1_summary.json")) as f:
        summ = json.load(f)["systems"]
    for sysd in summ:
        w, s, mesh = _c1_system(sysd["alfa"])
        code, x, st = solver.pcocr_2x2_folded(s, mesh)
        code_o, xo, st_o = O.pcocr(s, mesh, nthreads=4)
        assert code == 0 and code_o == 0
        assert abs(st.iterations - sysd["iterations"]) <= 3
        assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)
        xc = x[0::2] + 1j * x[1::2]
        idx = np.array(sysd["sample_index"])
        ref = np.array(sysd["sample_re"]) + 1j * np.array(sysd["sample_im"])
        assert np.max(np.abs(xc[idx] - ref)) <= 1e-5 * np.max(np.abs(ref))
        assert _true_rel_res(s, x) < 2e-8


def test_stop_on_true_residual(gpu):
    w, s, mesh = _c1_system()
    code, x, st = solver.pcocr_2x2_folded(s, mesh, stop_on_true_residual=True)
    assert code == 0
    assert st.true_residual_rel < s.eps
    assert _true_rel_res(s, x) < s.eps


def test_maxiter_and_x0_codes(gpu):
    w, s, mesh, *_ = load_golden("small")
    code, x, st = solver.pcocr_2x2_folded(s, mesh, maxiter=5)
    code_o, xo, st_o = O.pcocr(s, mesh, maxiter=5)
    assert code == code_o == -3
    assert st.iterations == st_o.iterations == 6
    # The early iterates of this system amplify summation-order differences:
    # the oracle itself moves ~1e-6 between 1 and 4 OpenMP threads here.
    _, x4, _ = O.pcocr(s, mesh, maxiter=5, nthreads=4)
    spread = np.linalg.norm(x4 - xo)
    assert np.linalg.norm(x - xo) <= 10 * spread + 1e-12 * np.linalg.norm(xo)
    # x0 already the solution: b = 0, x = 0
    s0 = slae_io.BlockSLAE(s.nb, s.ig, s.jg, s.idi, s.ijg, s.di, s.gg, np.zeros(s.n), s.eps, s.maxiter)
    code, x, st = solver.pcocr_2x2_folded(s0, mesh)
    assert code == -1 and st.iterations == 0


def test_nan_rhs_matches_oracle(gpu):
    w, s, mesh, *_ = load_golden("tiny")
    pr = s.pr.copy()
    pr[5] = np.nan
    sn = slae_io.BlockSLAE(s.nb, s.ig, s.jg, s.idi, s.ijg, s.di, s.gg, pr, s.eps, 20)
    code, x, st = solver.pcocr_2x2_folded(sn, mesh)
    code_o, xo, st_o = O.pcocr(sn, mesh)
    assert code == code_o and st.iterations == st_o.iterations


def test_breakdown_code(gpu):
    """(a, w) underflows below 1e-40 -> REQ_DIV_BY_ZERO, as in the oracle."""
    one = np.array([0, 0], np.int32)
    s = slae_io.BlockSLAE(1, np.array([0, 0], np.int32), np.zeros(0, np.int32),
                          np.array([0, 2], np.int32), np.array([0], np.int32),
                          np.array([1e200, 0.0]), np.zeros(0), np.array([1.0, 0.0]), 1e-8, 100)
    mesh = slae_io.SolveMesh(0, 1, 2, np.zeros((2, 3)), np.zeros(1, np.int32),
                             np.zeros((1, 14), np.int32), np.ones(1), np.array([[0, 1]], np.int32),
                             np.zeros(3, np.int32), np.zeros(1, np.int32), np.zeros(1),
                             np.ones(2, np.int32))
    code, x, st = solver.pcocr_2x2_folded(s, mesh)
    code_o, xo, st_o = O.pcocr(s, mesh)
    assert code == code_o == -2
    assert st.iterations == st_o.iterations == 1


def test_device_context_matches_host_entry(gpu):
    torch = gpu
    w, s, mesh, *_ = load_golden("small")
    ctx = solver.CocrContext(s, mesh)
    nc, nr, m = ctx.info()
    assert nc == s.nb + 2 * int(np.sum(np.diff(s.ijg) == 2))
    b = torch.tensor(s.pr, device="cuda")
    x = torch.zeros_like(b)
    code, st = ctx.solve(b, x, eps=s.eps, maxiter=s.maxiter)
    code2, x2, st2 = solver.pcocr_2x2_folded(s, mesh)
    assert code == code2 == 0 and st.iterations == st2.iterations
    assert np.array_equal(x.cpu().numpy(), x2)     # deterministic reductions
    y = torch.empty_like(b)
    ctx.spmv(x, y)
    assert np.allclose(y.cpu().numpy(), O.spmv(s, x2), rtol=0, atol=1e-12 * np.abs(s.pr).max())
    ctx.close()


def test_dropin_executable(gpu, tmp_path):
    from mtcalc_with_dfp_cocr_gb300 import build
    w, s, mesh, z1d, us, uc, v3, kit_iter, kit_r, nu, alfa = load_golden("small")
    d = str(tmp_path)
    w.mesh.write(d, nu=nu, alfa=alfa, eps=s.eps, maxiter=s.maxiter, receivers=w.receivers)
    slae_io.write_slae(d, s)
    r = subprocess.run([build.EXE], cwd=d, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    x = slae_io.read_v3(os.path.join(d, "v3.dat"), s.n)
    assert np.linalg.norm(x - v3) <= 1e-6 * np.linalg.norm(v3)
    kr, keps, kit, ktime = slae_io.read_kit(os.path.join(d, "kit"))
    assert abs(kit - kit_iter) <= 2 and kr < s.eps


def test_dropin_double_float(gpu):
    """The reference entry point in double-float arithmetic: same iteration
    count as FP64 and the true relative residual 1e-8 (checked in FP64 on
    the CPU)."""
    w, s, mesh = _c1_system(0)
    code, x, st = solver.pcocr_2x2_folded(s, mesh, double_float=True, stop_on_true_residual=True)
    code64, x64, st64 = solver.pcocr_2x2_folded(s, mesh, stop_on_true_residual=True)
    assert code == code64 == 0
    assert abs(st.iterations - st64.iterations) <= 3
    assert st.true_residual_rel < 1e-8
    assert _true_rel_res(s, x) < 1e-8
    # earth and surface edges agree to ~1e-8; air gradient components are
    # free at ~1e-5 under a 1e-8 residual (see test_gpu_survey)
    xyz = w.mesh.xyz()
    e = w.mesh.edges()
    earth = 0.5 * (xyz[e[:, 0], 2] + xyz[e[:, 1], 2]) <= 0.0
    c, c64 = x[0::2] + 1j * x[1::2], x64[0::2] + 1j * x64[1::2]
    assert np.linalg.norm((c - c64)[earth]) <= 1e-7 * np.linalg.norm(c64[earth])


def test_dropin_double_float_rejects_bad_input(gpu):
    """The double-float entry point checks every row of the uploaded SLAE and
    every entry of the uploaded mesh tables on the device, with the codes and
    messages of the host validation of the FP64 path: a column outside the
    lower triangle, an off-diagonal block size of 3, a negative edge node and
    a negative cell node are each MTGPU_ERR_ARG, and a good input still
    solves afterwards."""
    import copy
    w, s, mesh = _c1_system(1)
    row = s.nb // 2
    q = int(s.ig[row])
    cases = []
    b = copy.deepcopy(s)
    b.jg = s.jg.copy()
    b.jg[q] = row                                 # not below the diagonal
    cases.append((b, mesh, "lower-triangle"))
    b = copy.deepcopy(s)
    b.ijg = s.ijg.copy()
    b.ijg[q + 1:] += 2                            # block q spans 3 values
    b.gg = np.concatenate([s.gg, np.zeros(2)])
    cases.append((b, mesh, "block size"))
    m = copy.deepcopy(mesh)
    m.edges = mesh.edges.copy()
    m.edges[3, 1] = -1
    cases.append((s, m, "negative node"))
    m = copy.deepcopy(mesh)
    m.nver = mesh.nver.copy()
    m.nver[3, 2] = -5
    cases.append((s, m, "nver"))
    for slae, msh, words in cases:
        with pytest.raises(RuntimeError, match=words):
            solver.pcocr_2x2_folded(slae, msh, double_float=True, stop_on_true_residual=True)
    code, x, st = solver.pcocr_2x2_folded(s, mesh, double_float=True, stop_on_true_residual=True)
    assert code == 0 and st.true_residual_rel < 1e-8


def test_kit_unwritable_keeps_solution(gpu, tmp_path):
    """The reference entry point writes its `kit` line after the solve; a kit
    file that cannot be created is reported and the solver's code returned,
    with x solved (the reference writes the solution regardless,
    HarmVect3d.cpp:322-328)."""
    w, s, mesh = _c1_system(1)
    (tmp_path / "kit").mkdir()          # fopen("kit", "w") fails on a directory
    code, x, _ = solver.pcocr_2x2_folded(s, mesh, write_kit_in=str(tmp_path))
    assert code == 0
    assert _true_rel_res(s, x) < 1e-7
