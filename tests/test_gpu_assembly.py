"""GPU assembly (replacing BuildMatrix) against the reference's own SLAE
files (golden) and the CPU oracle."""
import numpy as np
import pytest

from conftest import load_golden
from mtcalc_with_dfp_cocr_gb300 import assembly, normal1d, slae_io, solver, workloads
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _same_slae(a, b, tol=1e-13):
    for k in ("ig", "jg", "idi", "ijg"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    for k in ("di", "gg", "pr"):
        x, y = getattr(a, k), getattr(b, k)
        assert np.max(np.abs(x - y)) <= tol * np.max(np.abs(y)), k


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_assembly_matches_reference_files(gpu, name):
    w, ref, mesh, z1d, us, uc, v3, kit_iter, kit_r, nu, alfa = load_golden(name)
    A = assembly.Assembly(w.mesh)
    s = A.block2x2(nu, alfa, z1d, us, uc)
    _same_slae(s, ref)
    A.close()


def test_assembly_matches_oracle_c1_both_polarisations(gpu):
    w = workloads.make("c1")
    z, us, uc = normal1d.solve_1d(1.0, [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers])
    A = assembly.Assembly(w.mesh)
    for alfa in (1, 0):
        _same_slae(A.block2x2(1.0, alfa, z, us, uc), O.assemble(w.mesh, 1.0, alfa, z, us, uc))
    A.close()


def test_device_rhs_and_solve_from_assembly(gpu):
    torch = gpu
    w = workloads.make("c1")
    tops, sig = [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers]
    z, us, uc = normal1d.solve_1d(1.0, tops, sig)
    A = assembly.Assembly(w.mesh)
    rhs = torch.empty(2, 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    A.rhs([1.0, 1.0], [1, 0], z, np.stack([us, us]), np.stack([uc, uc]), rhs)
    host = [A.block2x2(1.0, a, z, us, uc) for a in (1, 0)]
    for k in range(2):
        assert np.array_equal(rhs[k].cpu().numpy(), host[k].pr)
    ctx = A.cocr(1.0)
    x = torch.zeros_like(rhs)
    for k in range(2):
        code, st = ctx.solve(rhs[k], x[k], eps=1e-8, maxiter=10000, stop_on_true_residual=True)
        assert code == 0 and st.true_residual_rel < 1e-8
        code2, x2, st2 = solver.pcocr_2x2_folded(host[k], slae_io.mesh_to_solve_mesh(w.mesh))
        xs = x[k].cpu().numpy()
        assert np.linalg.norm(xs - x2) <= 1e-6 * np.linalg.norm(x2)
    ctx.close()
    A.close()


def test_assembly_rejects_bad_mesh(gpu):
    from mtcalc_with_dfp_cocr_gb300 import _lib
    w = workloads.make("tiny")
    w.mesh.nvkat = w.mesh.nvkat.copy()
    w.mesh.nvkat[3] = 99
    with pytest.raises(_lib.MtgpuError, match="nvkat"):
        assembly.Assembly(w.mesh, tables="host")
    with pytest.raises(_lib.MtgpuError, match="cell material out of range"):
        assembly.Assembly(w.mesh, tables="device")


@pytest.mark.parametrize("name", ["small", "c1"])
def test_device_mesh_tables_equal_host_tables(gpu, name):
    """The mesh tables generated on the device from the node lines
    (RegularMeshBuilder's numbering) give the same assembly, bit for bit, as
    the tables built on the host and uploaded: the SLAE in the reference's
    block format and the right-hand sides of both polarisations."""
    torch = gpu
    w = workloads.make(name)
    nu = 1.0
    z, us, uc = normal1d.solve_1d(nu, [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers])
    Ad = assembly.Assembly(w.mesh, tables="device")
    Ah = assembly.Assembly(w.mesh, tables="host")
    for alfa in (1, 0):
        sd = Ad.block2x2(nu, alfa, z, us, uc)
        sh = Ah.block2x2(nu, alfa, z, us, uc)
        for f in ("ig", "jg", "idi", "ijg", "di", "gg", "pr"):
            assert np.array_equal(getattr(sd, f), getattr(sh, f)), f
    bd = torch.empty(2, 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    bh = torch.empty_like(bd)
    Ad.rhs([nu, nu], [1, 0], z, np.stack([us, us]), np.stack([uc, uc]), bd)
    Ah.rhs([nu, nu], [1, 0], z, np.stack([us, us]), np.stack([uc, uc]), bh)
    assert torch.equal(bd, bh)
    Ad.close()
    Ah.close()


@pytest.mark.parametrize("name,tables", [("tiny", "host"), ("small", "device"), ("c1", "device"),
                                         ("c1", "host")])
def test_device_preconditioner_g_equals_host(gpu, name, tables):
    """The folded preconditioner's G (rows of the interior nodes of
    conductive cells, -1/2 and +1/2 per edge, FoldedPreconditioner.cpp:68-259)
    and G^T, built on the device by every solver set-up, equal the host
    construction entry for entry, including the order of every row (the
    D_S sums and the node gathers run in that order)."""
    w = workloads.make(name)
    A = assembly.Assembly(w.mesh, tables=tables)
    assert A.check_preconditioner()
    A.close()
