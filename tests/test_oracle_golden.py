"""The CPU oracle against the reference's own outputs (tests/golden, made by
running the reference programs built from source)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from mtcalc_with_dfp_cocr_gb300 import normal1d, slae_io, workloads
from oracle import pyoracle as O


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_assembly_matches_reference(name):
    w, ref, mesh, z1d, us, uc, v3, kit_iter, kit_r, nu, alfa = load_golden(name)
    mine = O.assemble(w.mesh, nu, alfa, z1d, us, uc)
    for k in ("ig", "jg", "idi", "ijg"):
        assert np.array_equal(getattr(ref, k), getattr(mine, k)), k
    for k in ("di", "gg", "pr"):
        a, b = getattr(ref, k), getattr(mine, k)
        assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(a)), k


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_solve_matches_reference_bitwise(name):
    """Single-threaded, the oracle repeats the reference's arithmetic."""
    w, ref, mesh, z1d, us, uc, v3, kit_iter, kit_r, nu, alfa = load_golden(name)
    code, x, st = O.pcocr(ref, mesh, nthreads=1)
    assert code == 0
    assert st.iterations == kit_iter
    assert abs(st.residual_rel - kit_r) <= 1e-6 * kit_r   # kit prints %e
    assert np.max(np.abs(x - v3)) <= 1e-13 * np.max(np.abs(v3))


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_spmv_matches_dense(name):
    w, ref, *_ = load_golden(name)
    x = np.random.default_rng(7).standard_normal(ref.n)
    y = O.spmv(ref, x)
    A = ref.to_dense()
    yd = A @ (x[0::2] + 1j * x[1::2])
    assert np.max(np.abs(y[0::2] + 1j * y[1::2] - yd)) <= 1e-13 * np.max(np.abs(yd))
    y4 = O.spmv(ref, x, nthreads=4)
    assert np.max(np.abs(y4 - y)) <= 1e-13 * np.max(np.abs(y))


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_normal_field_matches_harm1d(name):
    """The 1-D normal-field restatement against the reference Harm1D.  The
    1-D system spans 0.01 m to 1e4 km element sizes; its conditioning limits
    agreement between two direct solvers to ~1e-9 relative."""
    w, ref, mesh, z1d, us, uc, *_rest = load_golden(name)
    nu = _rest[-2]
    z, s, c = normal1d.solve_1d(nu, [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers])
    assert np.array_equal(z, z1d)
    scale = max(np.abs(us).max(), np.abs(uc).max())
    assert np.max(np.abs(s - us)) <= 1e-8 * scale
    assert np.max(np.abs(c - uc)) <= 1e-8 * scale


def test_c1_oracle_matches_reference_summary():
    """24x24x24 benchmark mesh: assembly checksums and the solve."""
    with open(os.path.join(GOLDEN, "c1_summary.json")) as f:
        summ = json.load(f)
    w = workloads.make("c1")
    mesh = slae_io.mesh_to_solve_mesh(w.mesh)
    sysd = summ["systems"][0]
    z, us, uc = normal1d.solve_1d(sysd["nu"], [l.top for l in w.mesh.layers],
                                  [l.sigma for l in w.mesh.layers])
    s = O.assemble(w.mesh, sysd["nu"], sysd["alfa"], z, us, uc)
    assert s.nb == sysd["nb"] and s.ig[-1] == sysd["nnz_lower"]
    assert s.idi[-1] == sysd["di_len"] and s.ijg[-1] == sysd["gg_len"]
    assert abs(s.di.sum() - sysd["sum_di"]) <= 1e-12 * abs(sysd["sum_di"])
    assert abs(np.abs(s.gg).sum() - sysd["sum_abs_gg"]) <= 1e-12 * sysd["sum_abs_gg"]
    # the RHS carries the 1-D field, which agrees with Harm1D to ~1e-9
    assert abs(np.linalg.norm(s.pr) - sysd["norm_pr"]) <= 1e-7 * sysd["norm_pr"]
    code, x, st = O.pcocr(s, mesh, nthreads=1)
    assert code == 0
    assert abs(st.iterations - sysd["iterations"]) <= 2
    xc = x[0::2] + 1j * x[1::2]
    idx = np.array(sysd["sample_index"])
    ref = np.array(sysd["sample_re"]) + 1j * np.array(sysd["sample_im"])
    assert np.max(np.abs(xc[idx] - ref)) <= 1e-5 * np.max(np.abs(ref))
    assert abs(np.linalg.norm(x) - sysd["norm_v3"]) <= 1e-6 * sysd["norm_v3"]


def test_brick_matrices_properties():
    """Local curl-curl and mass matrices: symmetric, the curl-curl annihilates
    gradients of nodal functions (its null space), mass is positive definite."""
    b, c = O.brick_bc(100.0, 70.0, 40.0)
    assert np.allclose(b, b.T) and np.allclose(c, c.T)
    assert np.all(np.linalg.eigvalsh(c) > 0)
    # gradient of the nodal function of node 0 (x-,y-,z-) in edge dofs:
    # dof = (h/2) * tangential derivative averaged -> +-1/2 along its edges
    from mtcalc_with_dfp_cocr_gb300 import mesh as M
    m = M.layered_model([0, 100.0], [0, 70.0], [0, 40.0], [M.Layer(0.0, 0.01)])
    ed = m.cell_edges()[0]
    edges = m.edges()
    for node in range(8):
        g = np.zeros(12)
        for j in range(12):
            n1, n2 = edges[ed[j]]
            g[j] = -0.5 if n1 == node else (0.5 if n2 == node else 0.0)
        assert np.max(np.abs(b @ g)) <= 1e-12 * np.max(np.abs(b))
