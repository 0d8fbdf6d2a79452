"""The matrix-free SpMV's operator (survey.cu, k_mf_faces / k_mf_edges),
restated in numpy with the same weights and multipliers, against the matrix
assembled from the brick matrices (oracle/mtcalc_oracle.c orc_brick_bc, the
restatement of T_Brick.cpp:1361-1395 pinned to BuildMatrix):

    K = D^T F D    D: edge -> face circulations (+-1), F per direction
                   (2 h_d / (h_t1 h_t2) / mu) m, m = [[2, 1], [1, 2]] / 3
    M              per direction (sigma h_t1 h_t2 / h_d) (m (x) m)

with the kernel's scaled weights wF / 3 and wM / 9 and integer multipliers,
Dirichlet edges read as 0 and mapped to themselves."""
import numpy as np
import pytest
import scipy.sparse as sp

from mtcalc_with_dfp_cocr_gb300 import workloads
from oracle import pyoracle as O

MU0 = 1.25663706143591729e-6


def assembled(m, omega):
    xyz, cn, ce = m.xyz(), m.cell_nodes(), m.cell_edges()
    sig = m.mat_sigma[m.nvkat]
    rows, cols, vals = [], [], []
    b, c = np.zeros(144), np.zeros(144)
    for cell in range(m.kpar):
        h = xyz[cn[cell, 7]] - xyz[cn[cell, 0]]
        O.lib().orc_brick_bc(h[0], h[1], h[2], b, c)
        e = ce[cell]
        rows += list(np.repeat(e, 12))
        cols += list(np.tile(e, 12))
        vals += list(b / MU0 + 1j * omega * sig[cell] * c)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(m.nb, m.nb))
    nx, ny, nz = m.nx, m.ny, m.nz
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    bnode = ((ix == 0) | (ix == nx - 1) | (iy == 0) | (iy == ny - 1) | (iz == 0) |
             (iz == nz - 1)).ravel()
    E = m.edges()
    bedge = bnode[E[:, 0]] & bnode[E[:, 1]]
    D = sp.diags((~bedge).astype(float))
    return D @ A @ D + sp.diags(bedge.astype(float)), bedge


def matrix_free(m, omega, x, bedge):
    nx, ny, nz = m.nx, m.ny, m.nz
    h = [np.diff(m.x), np.diff(m.y), np.diff(m.z)]
    sigc = m.mat_sigma[m.nvkat].reshape(nz - 1, ny - 1, nx - 1)
    ex, ey, ez = (a.reshape(nz, ny, nx) for a in m._edge_ids())
    eid = [ex, ey, ez]
    xm = np.where(bedge, 0, x)

    def xe(d, p):
        return xm[eid[d][p[2], p[1], p[0]]]

    # face circulations, counterclockwise seen from +n
    F = [np.zeros((nx, ny - 1, nz - 1), complex), np.zeros((nx - 1, ny, nz - 1), complex),
         np.zeros((nx - 1, ny - 1, nz), complex)]
    for n in range(3):
        a, b_ = (n + 1) % 3, (n + 2) % 3
        for idx in np.ndindex(F[n].shape):
            p = list(idx)
            pa = list(p); pa[b_] += 1   # the a-edge on the far b side
            pb = list(p); pb[a] += 1    # the b-edge on the far a side
            F[n][idx] = xe(a, p) + xe(b_, pb) - xe(a, pa) - xe(b_, p)

    def cellw(p):
        hh = [h[0][p[0]], h[1][p[1]], h[2][p[2]]]
        wf = [2 * hh[d] / (hh[(d + 1) % 3] * hh[(d + 2) % 3]) / MU0 / 3 for d in range(3)]
        wm = [sigc[p[2], p[1], p[0]] * hh[(d + 1) % 3] * hh[(d + 2) % 3] / hh[d] / 9
              for d in range(3)]
        return wf, wm

    y = np.where(bedge, x, 0).astype(complex)
    for d in range(3):
        t1, t2 = (d + 1) % 3, (d + 2) % 3
        for idx in np.ndindex(eid[d].shape[::-1]):
            p = list(idx)
            if p[d] >= (nx, ny, nz)[d] - 1:
                continue
            e = eid[d][p[2], p[1], p[0]]
            if bedge[e]:
                continue
            w = {}
            for a in (0, 1):
                for b_ in (0, 1):
                    c = list(p); c[t1] += a - 1; c[t2] += b_ - 1
                    w[a, b_] = cellw(c)
            k = 0
            for nn, (n, o) in enumerate(((t1, t2), (t2, t1))):
                for b_ in (0, 1):
                    q = list(p); q[o] += b_ - 1
                    sg = (1 if b_ == 0 else -1) if nn == 0 else (-1 if b_ == 0 else 1)
                    wa = w[0, b_][0][n] if nn == 0 else w[b_, 0][0][n]
                    wb = w[1, b_][0][n] if nn == 0 else w[b_, 1][0][n]
                    qm = list(q); qm[n] -= 1
                    qp = list(q); qp[n] += 1
                    k += sg * (wa * F[n][tuple(qm)] + 2 * (wa + wb) * F[n][tuple(q)] +
                               wb * F[n][tuple(qp)])
            wm = {key: v[1][d] for key, v in w.items()}
            s0, s1 = wm[0, 0] + wm[0, 1], wm[1, 0] + wm[1, 1]
            r0, r1 = wm[0, 0] + wm[1, 0], wm[0, 1] + wm[1, 1]
            cm = [[wm[0, 0], 2 * s0, wm[0, 1]], [2 * r0, 4 * (s0 + s1), 2 * r1],
                  [wm[1, 0], 2 * s1, wm[1, 1]]]
            mm = 0
            for a in range(3):
                for b_ in range(3):
                    q = list(p); q[t1] += a - 1; q[t2] += b_ - 1
                    mm += cm[a][b_] * xe(d, q)
            y[e] = k + 1j * omega * mm
    return y


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_matrix_free_operator_equals_assembled(name):
    m = workloads.make(name).mesh
    omega = 2 * np.pi * 0.1
    A, bedge = assembled(m, omega)
    rng = np.random.default_rng(7)
    x = rng.standard_normal(m.nb) + 1j * rng.standard_normal(m.nb)
    ref = A @ x
    got = matrix_free(m, omega, x, bedge)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
