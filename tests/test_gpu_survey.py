"""Batched double-float survey solver: the reference's COCR iteration for
every system at once, in double-float arithmetic on the FP32 pipes.  It must
follow the FP64 solver's iteration counts and reach the true FP64 relative
residual 1e-8."""
import numpy as np
import pytest

from mtcalc_with_dfp_cocr_gb300 import assembly, normal1d, slae_io, solver, survey, workloads
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _tables(w, nus):
    tops, sig = [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers]
    return [normal1d.solve_1d(nu, tops, sig) for nu in nus]


def _run(torch, name, systems, eps=1e-8, verify=True, maxiter=20000):
    w = workloads.make(name)
    nus = [f for f, _ in systems]
    alfas = [a for _, a in systems]
    tabs = _tables(w, nus)
    A = assembly.Assembly(w.mesh)
    S = len(systems)
    b = torch.empty(S, 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    A.rhs(nus, alfas, tabs[0][0], np.stack([t[1] for t in tabs]), np.stack([t[2] for t in tabs]), b)
    x = torch.zeros_like(b)
    sv = survey.Survey(A, nus)
    code, st = sv.solve(b, x, eps=eps, maxiter=maxiter, verify=verify)
    return w, A, tabs, b, x, code, st


def _assert_close_in_earth(w, x, x64):
    """Both solutions meet ||b - A x|| < 1e-8 ||b||.  On edges in the earth
    and at the surface (receivers) they agree to ~1e-8; in the air the
    gradient (null-space) components of the potential are regularised only by
    sigma = 1e-8 S/m, so a 1e-8 residual leaves them free at the ~1e-5 level
    for any solver."""
    xyz = w.mesh.xyz()
    e = w.mesh.edges()
    air = 0.5 * (xyz[e[:, 0], 2] + xyz[e[:, 1], 2]) > 0.0
    c, c64 = x[0::2] + 1j * x[1::2], x64[0::2] + 1j * x64[1::2]
    n = np.linalg.norm
    assert n((c - c64)[~air]) <= 1e-7 * n(c64[~air])
    assert n(c - c64) <= 1e-4 * n(c64)


@pytest.mark.parametrize("name,systems", [
    ("small", [(0.1, 1), (0.1, 0), (10.0, 1)]),
    ("c1", [(1.0, 1), (1.0, 0)]),
])
def test_survey_follows_fp64_and_reaches_true_residual(gpu, name, systems):
    torch = gpu
    w, A, tabs, b, x, code, st = _run(torch, name, systems)
    assert code == 0, st
    mesh = slae_io.mesh_to_solve_mesh(w.mesh)
    for k, (nu, alfa) in enumerate(systems):
        assert st["status"][k] == 0
        assert st["true_residual_rel"][k] < 1e-8
        s = A.block2x2(nu, alfa, *tabs[k])
        xk = x[k].cpu().numpy()
        r = s.pr - O.spmv(s, xk)
        assert np.linalg.norm(r) / np.linalg.norm(s.pr) < 1e-8        # checked in FP64 on the CPU
        code64, x64, st64 = solver.pcocr_2x2_folded(s, mesh, stop_on_true_residual=True)
        assert code64 == 0
        assert abs(st["iterations"][k] - st64.iterations) <= 3
        _assert_close_in_earth(w, xk, x64)


def test_survey_reference_stop_rule_matches_oracle(gpu):
    """Without verification the stop rule is the reference's alone; the
    iteration counts match the oracle's."""
    torch = gpu
    w, A, tabs, b, x, code, st = _run(torch, "c1", [(1.0, 1), (1.0, 0)], verify=False)
    assert code == 0
    mesh = slae_io.mesh_to_solve_mesh(w.mesh)
    for k, alfa in enumerate((1, 0)):
        s = A.block2x2(1.0, alfa, *tabs[k])
        c, xo, sto = O.pcocr(s, mesh, nthreads=4)
        assert abs(st["iterations"][k] - sto.iterations) <= 2


def test_survey_single_system_and_padding(gpu):
    torch = gpu
    w, A, tabs, b, x, code, st = _run(torch, "tiny", [(1.0, 1)])
    assert code == 0 and st["true_residual_rel"][0] < 1e-8
    # five systems pad to eight lanes; all must finish
    w, A, tabs, b, x, code, st = _run(torch, "tiny", [(0.01, 1), (0.1, 0), (1.0, 1), (10.0, 0), (100.0, 1)])
    assert code == 0 and max(st["true_residual_rel"]) < 1e-8


def test_survey_iteration_limit(gpu):
    torch = gpu
    w, A, tabs, b, x, code, st = _run(torch, "small", [(0.1, 1)], maxiter=5)
    assert code == -3 and st["status"][0] == -3 and st["iterations"][0] == 6


@pytest.mark.parametrize("name,S", [("c1", 2), ("c1", 4), ("small", 32)])
def test_spmv_variants_agree(gpu, name, S):
    """Every SpMV variant (x staged in shared memory per tile, gathered with
    2, 4, 8 slots in flight, or, for two systems, one thread per row for
    both) sums the same products in the same order; only the block grouping
    of the dot products differs with the launch grid, so the solves agree to
    rounding.  The matrix-free variant (32, available on these tensor
    meshes) computes the same operator in another order: its solves agree
    to the same bounds."""
    torch = gpu
    w = workloads.make(name)
    freqs = np.logspace(-2, 2, S // 2)
    systems = [(f, a) for f in freqs for a in (1, 0)]
    nus = [f for f, _ in systems]
    tabs = _tables(w, nus)
    A = assembly.Assembly(w.mesh)
    b = torch.empty(S, 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    A.rhs(nus, [a for _, a in systems], tabs[0][0], np.stack([t[1] for t in tabs]),
          np.stack([t[2] for t in tabs]), b)
    sv = survey.Survey(A, nus)
    ref = None
    for v in (0, 1, 2, 4, 8, 32, 33, 34, 35) + ((18, 20) if S == 2 else ()):
        sv.set_spmv_variant(v)
        x = torch.zeros_like(b)
        code, st = sv.solve(b, x, eps=1e-8, maxiter=20000, verify=True)
        assert code == 0
        assert max(st["true_residual_rel"]) < 1e-8
        if ref is None:
            ref = (x.clone(), st["iterations"], st["verifications"])
            continue
        # rounding moves the stop by a few iterations; where a run's first
        # stop leaves the true residual just above eps, the continuation
        # rounds (a tighter recurrence threshold, the FP64 residual checked
        # again) add a rounding-dependent number of iterations, so the counts
        # are compared where neither run needed one.  The earth and surface
        # edges agree either way (the air's gradient components are free at
        # 1e-8)
        for i, j, nv, nr in zip(st["iterations"], ref[1], st["verifications"], ref[2]):
            if nv <= 1 and nr <= 1:
                assert abs(i - j) <= 3 + 0.03 * j, (v, st["iterations"], ref[1])
        xyz = w.mesh.xyz()
        e = w.mesh.edges()
        earth = 0.5 * (xyz[e[:, 0], 2] + xyz[e[:, 1], 2]) <= 0.0
        # every variant rounds its products or dot products in its own order
        # (the matrix-free operator its own summation, the stored ones their
        # launch grids' block partials), so the trajectories part at rounding
        # level and only the 1e-8 FP64 residual ties the solutions together:
        # that leaves the earth edges free at ~cond x 1e-8, measured up to
        # ~4e-7
        tol = 1e-6
        for k in range(S):
            a = x[k].cpu().numpy().view(np.complex128)[earth]
            r = ref[0][k].cpu().numpy().view(np.complex128)[earth]
            assert np.linalg.norm(a - r) <= tol * np.linalg.norm(r), (v, k)


def test_survey_iteration_guard_times_out(gpu, monkeypatch):
    """The host loop around the graph launches gives up with MTGPU_ERR_TIMEOUT
    once it has run more iterations than its guard allows (the device stops
    every system at maxiter, so the test lowers the guard through
    MTGPU_SURVEY_GUARD_ITERS); the survey object stays usable."""
    torch = gpu
    from mtcalc_with_dfp_cocr_gb300 import _lib
    w = workloads.make("small")
    tabs = _tables(w, [0.1])
    A = assembly.Assembly(w.mesh)
    b = torch.empty(1, 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    A.rhs([0.1], [1], tabs[0][0], np.stack([tabs[0][1]]), np.stack([tabs[0][2]]), b)
    sv = survey.Survey(A, [0.1])
    x = torch.zeros_like(b)
    monkeypatch.setenv("MTGPU_SURVEY_GUARD_ITERS", "8")
    with pytest.raises(_lib.MtgpuError) as e:
        sv.solve(b, x, eps=1e-8, maxiter=20000, verify=True)
    assert "guard" in str(e.value)
    monkeypatch.delenv("MTGPU_SURVEY_GUARD_ITERS")
    x.zero_()
    code, st = sv.solve(b, x, eps=1e-8, maxiter=20000, verify=True)
    assert code == 0 and st["true_residual_rel"][0] < 1e-8
    sv.close()
    A.close()


@pytest.mark.parametrize("variant", [32, 33, 34, 35])
def test_matfree_operator_on_gradients(gpu, variant):
    """The matrix-free SpMV on discrete gradients x = grad(phi): the curl-curl
    part vanishes (curl grad = 0), so y = i omega M x checks the mass part
    alone, which the set-up check (a random vector, dominated by the
    curl-curl part) cannot resolve below ~1e-9.  Compared per system with
    the oracle's port of Mult_MV_block_2x2 on the assembled SLAE."""
    torch = gpu
    w = workloads.make("c1")
    nus = [1.0, 10.0, 0.01, 100.0]
    tabs = _tables(w, nus)
    A = assembly.Assembly(w.mesh)
    sv = survey.Survey(A, nus)
    sv.set_spmv_variant(variant)
    e = w.mesh.edges()
    bound = np.zeros(len(w.mesh.xyz()), bool)
    bound[w.mesh.boundary_nodes()] = True
    rng = np.random.default_rng(5)
    X = np.zeros((len(nus), 2 * w.mesh.nb))
    for k in range(len(nus)):
        phi = rng.standard_normal(len(bound)) + 1j * rng.standard_normal(len(bound))
        phi[bound] = 0.0
        g = phi[e[:, 1]] - phi[e[:, 0]]
        X[k, 0::2], X[k, 1::2] = g.real, g.imag
    x = torch.tensor(X, device="cuda")
    y = torch.empty_like(x)
    sv.spmv(x, y)
    Y = y.cpu().numpy()
    for k, nu in enumerate(nus):
        s = O.assemble(w.mesh, nu, 1, *tabs[k])
        y_ref = O.spmv(s, X[k])
        assert np.max(np.abs(Y[k] - y_ref)) <= 1e-9 * np.max(np.abs(y_ref)), (variant, nu)
    sv.close()
    A.close()


@pytest.mark.parametrize("name,S", [("tiny", 1), ("small", 3), ("c1", 2), ("c1", 5), ("small", 32)])
def test_tiled_matfree_equals_two_kernel_form(gpu, name, S):
    """Variant 34 (one tiled kernel, edge values and face circulations in
    shared memory) sums in the order of variant 32 (faces through global
    memory): the products agree to the last bit, for every layout width
    (1 to 32 systems) and for tiles that overhang the mesh."""
    torch = gpu
    w = workloads.make(name)
    nus = list(np.logspace(-2, 2, S))
    A = assembly.Assembly(w.mesh)
    sv = survey.Survey(A, nus)
    rng = np.random.default_rng(S)
    x = torch.tensor(rng.standard_normal((S, 2 * w.mesh.nb)), device="cuda")
    y32, y34 = torch.empty_like(x), torch.empty_like(x)
    sv.set_spmv_variant(32)
    sv.spmv(x, y32)
    sv.set_spmv_variant(34)
    sv.spmv(x, y34)
    assert torch.equal(y32, y34)
    sv.close()
    A.close()


def _oracle_check(w, nu, alfa, tab, x, x_ref=None):
    """FP64 true residual of x on the oracle's SLAE, and the oracle's own
    FP64 solution for the comparison on earth edges."""
    s = O.assemble(w.mesh, nu, alfa, *tab)
    rel = np.linalg.norm(s.pr - O.spmv(s, x)) / np.linalg.norm(s.pr)
    code, x64, _ = O.pcocr(s, slae_io.mesh_to_solve_mesh(w.mesh), nthreads=4)
    assert code == 0
    return rel, x64


def test_survey_42_systems_in_one_survey(gpu):
    """The published survey's size (21 frequencies x 2 polarisations, CalcStarter
    runs them one by one, Code/CalcStarter/main.cpp:311-325) in one survey
    object: two batches (32 + 10 systems) side by side; every system against
    the oracle's FP64 solve."""
    torch = gpu
    w = workloads.make("small")
    freqs = np.logspace(-2, 3, 21)
    systems = [(f, a) for f in freqs for a in (1, 0)]
    nus = [f for f, _ in systems]
    tabs = {f: normal1d.solve_1d(f, [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers])
            for f in freqs}
    A = assembly.Assembly(w.mesh)
    b = torch.empty(len(systems), 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    A.rhs(nus, [a for _, a in systems], tabs[freqs[0]][0], np.stack([tabs[f][1] for f in nus]),
          np.stack([tabs[f][2] for f in nus]), b)
    x = torch.zeros_like(b)
    sv = survey.Survey(A, nus)
    assert sv.batches == 2
    code, st = sv.solve(b, x, eps=1e-8, maxiter=20000, verify=True)
    assert code == 0, st
    X = x.cpu().numpy()
    xyz = w.mesh.xyz()
    e = w.mesh.edges()
    earth = 0.5 * (xyz[e[:, 0], 2] + xyz[e[:, 1], 2]) <= 0.0
    for k, (f, a) in enumerate(systems):
        assert st["status"][k] == 0 and st["true_residual_rel"][k] < 1e-8
        rel, x64 = _oracle_check(w, f, a, tabs[f], X[k])
        assert rel < 1e-8, (f, a, rel)
        # earth and surface edges only: down to 0.01 Hz the air's gradient
        # components are left free (~1e-4 here) by any solver at a 1e-8
        # residual
        c, c64 = X[k][0::2] + 1j * X[k][1::2], x64[0::2] + 1j * x64[1::2]
        assert np.linalg.norm((c - c64)[earth]) <= 1e-7 * np.linalg.norm(c64[earth]), (f, a)
    sv.close()
    A.close()


def test_survey_two_meshes_packed(gpu):
    """Systems of two meshes of different sizes in one survey, their vectors
    packed one after the other (offsets from the library); every system
    against the oracle's FP64 solve on its own mesh."""
    torch = gpu
    parts = [("tiny", [1.0, 10.0]), ("small", [0.1, 0.1, 10.0])]
    alfa_of = {("tiny", 0): 1, ("tiny", 1): 0, ("small", 0): 1, ("small", 1): 0, ("small", 2): 1}
    ws, As, rhs, tabs = [], [], [], []
    for name, nus in parts:
        w = workloads.make(name)
        t = [normal1d.solve_1d(f, [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers])
             for f in nus]
        A = assembly.Assembly(w.mesh)
        b = torch.empty(len(nus), 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
        al = [alfa_of[(name, k)] for k in range(len(nus))]
        A.rhs(nus, al, t[0][0], np.stack([q[1] for q in t]), np.stack([q[2] for q in t]), b)
        ws.append(w)
        As.append(A)
        rhs.append(b.reshape(-1))
        tabs.append(t)
    sv = survey.Survey.multi([(A, nus) for A, (_, nus) in zip(As, parts)])
    off = sv.offsets
    assert off[-1] == sum(r.numel() for r in rhs)
    b = torch.cat(rhs)
    x = torch.zeros_like(b)
    code, st = sv.solve(b, x, eps=1e-8, maxiter=20000, verify=True)
    assert code == 0, st
    X = x.cpu().numpy()
    k = 0
    for m, (name, nus) in enumerate(parts):
        for j, nu in enumerate(nus):
            xk = X[off[k]:off[k + 1]]
            assert len(xk) == 2 * ws[m].mesh.nb
            rel, x64 = _oracle_check(ws[m], nu, alfa_of[(name, j)], tabs[m][j], xk)
            assert rel < 1e-8, (name, nu, rel)
            _assert_close_in_earth(ws[m], xk, x64)
            k += 1
    sv.close()
    for A in As:
        A.close()


@pytest.mark.parametrize("name,S", [("tiny", 1), ("small", 3), ("c1", 2), ("small", 32)])
def test_face_mass_form_matches_two_kernel_form(gpu, name, S):
    """Variant 35 applies the face mass matrix once per face (D^T (F f));
    it sums the same terms in another grouping, so its product agrees with
    variant 32's to the double-float rounding of the curl-curl sums, and
    with the oracle's assembled matrix like variant 32."""
    torch = gpu
    w = workloads.make(name)
    nus = list(np.logspace(-2, 2, S))
    A = assembly.Assembly(w.mesh)
    sv = survey.Survey(A, nus)
    rng = np.random.default_rng(7 + S)
    x = torch.tensor(rng.standard_normal((S, 2 * w.mesh.nb)), device="cuda")
    y32, y35 = torch.empty_like(x), torch.empty_like(x)
    sv.set_spmv_variant(32)
    sv.spmv(x, y32)
    sv.set_spmv_variant(35)
    sv.spmv(x, y35)
    d = (y35 - y32).abs().max().item()
    assert d <= 1e-12 * y32.abs().max().item(), d
    sv.close()
    A.close()


@pytest.mark.parametrize("name,systems", [("small", [(0.1, 1), (0.1, 0), (10.0, 1)]),
                                          ("c1", [(1.0, 1), (1.0, 0)])])
def test_fused_preconditioner(gpu, monkeypatch, name, systems):
    """The folded preconditioner in one kernel (h of a tile's nodes in shared
    memory), requested with MTGPU_PREC_TILE=1, is enabled on these tensor
    meshes only after a set-up step of it equals the node and edge kernels'
    bit for bit; with and without it the solves reach the FP64 true residual
    with the same iteration counts up to rounding (the (a, w) sums are
    grouped differently)."""
    torch = gpu
    res = {}
    for force in ("1", "0"):
        monkeypatch.setenv("MTGPU_PREC_TILE", force)
        w = workloads.make(name)
        nus = [f for f, _ in systems]
        tabs = _tables(w, nus)
        A = assembly.Assembly(w.mesh)
        b = torch.empty(len(systems), 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
        A.rhs(nus, [a for _, a in systems], tabs[0][0], np.stack([t[1] for t in tabs]),
              np.stack([t[2] for t in tabs]), b)
        x = torch.zeros_like(b)
        sv = survey.Survey(A, nus)
        fused, _ = sv.preconditioner()
        assert fused == (force == "1")
        code, st = sv.solve(b, x, eps=1e-8, maxiter=20000, verify=True)
        assert code == 0 and max(st["true_residual_rel"]) < 1e-8
        res[force] = (st["iterations"], x.cpu().numpy())
        sv.close()
        A.close()
    for i, j in zip(res["1"][0], res["0"][0]):
        assert abs(i - j) <= 3 + 0.03 * j
    w = workloads.make(name)
    xyz = w.mesh.xyz()
    e = w.mesh.edges()
    earth = 0.5 * (xyz[e[:, 0], 2] + xyz[e[:, 1], 2]) <= 0.0
    for k in range(len(systems)):
        a = res["1"][1][k].view(np.complex128)[earth]
        r = res["0"][1][k].view(np.complex128)[earth]
        assert np.linalg.norm(a - r) <= 1e-7 * np.linalg.norm(r)


@pytest.mark.parametrize("name,systems", [("small", [(0.1, 1), (0.1, 0), (10.0, 1)]),
                                          ("c1", [(1.0, 1), (1.0, 0)])])
def test_preconditioner_diagonal_passes_agree(gpu, monkeypatch, name, systems):
    """diag(G K G^T) and diag(G M G^T) from the per-edge passes (meshes with
    the compact G^T: row k of A read once for both nodes of edge k) have the
    terms and the summation order of the per-entry passes
    (MTGPU_GDIAG_ENTRIES=1): with one SpMV variant pinned, the two set-ups
    give the same solves bit for bit."""
    torch = gpu
    monkeypatch.setenv("MTGPU_SPMV_VARIANT", "4")
    monkeypatch.setenv("MTGPU_PREC_TILE", "0")
    out = {}
    for entries in ("0", "1"):
        monkeypatch.setenv("MTGPU_GDIAG_ENTRIES", entries)
        w, A, tabs, b, x, code, st = _run(torch, name, systems)
        assert code == 0 and max(st["true_residual_rel"]) < 1e-8
        out[entries] = (st["iterations"], x.clone())
        A.close()
    assert out["0"][0] == out["1"][0]
    assert torch.equal(out["0"][1], out["1"][1])
