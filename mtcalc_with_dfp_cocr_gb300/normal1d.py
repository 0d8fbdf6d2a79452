"""1-D normal (background) field of the layered half-space.

Restates the reference's Harm1D program (Code/Harm1D), whose output tables
`usin.dat` / `ucos.dat` give the plane-wave vector potential A0(z) that the
3-D right-hand side is built from:

* 1-D mesh from z = 0 down to z = -1e7 with a first step of 0.01 m growing by
  1.02, each layer interface inserted as a node
  (Code/Harm1D/mesh_1d_mtz.cpp:96-187; constants mesh_1d_mtz.h:21-24);
* linear elements for  -(1/mu) u'' + i*omega*sigma*u = 0  in the real 2x2
  block form (local_matrix_1d.cpp:36-111,
  global_slae_1d_harm_prof.cpp:69-127);
* u = 0 at the bottom node and a unit real flux at z = 0
  (global_slae_1d_harm_prof.cpp:129-140);
* the tables are printed with "%25.13e" (divgrad_1d.cpp:203-217), so the
  values returned here are rounded the same way.

The reference factorises the system with a profile LU; here the same
tridiagonal complex system is solved by the Thomas algorithm.
"""
from __future__ import annotations

import numpy as np

MU0_1D = 4.0 * 3.1415926535897932 * 1e-7   # Code/Harm1D/mesh_1d_mtz.cpp:71
PI_1D = 3.1415926535897932                 # Code/Harm1D/stdafx.h:10
X0_1D = -10000000.0
X1_1D = 0.0
COEF_RAZR = 1.02
STEP0 = 1e-2


def _q13(v):
    return np.array([float(f"{t:.13e}") for t in np.asarray(v, np.float64)])


def mesh_1d(layer_tops):
    """Node coordinates (ascending) and element layer index (0-based, bottom
    layer = 0) for layer tops given bottom-up, the last top being 0."""
    n_layers = len(layer_tops)
    layers = [X0_1D] + [float(t) for t in layer_tops]
    x = X1_1D
    step = STEP0
    coords = []
    for i in range(n_layers):
        coords.append(layers[n_layers - i])
        while True:
            x -= step
            if x <= layers[n_layers - i - 1]:
                break
            step *= COEF_RAZR
            coords.append(x)
    coords.append(X0_1D)
    coords = np.array(coords[::-1])
    centers = 0.5 * (coords[:-1] + coords[1:])
    elem_layer = np.empty(len(centers), np.int64)
    for e, c in enumerate(centers):
        for j in range(n_layers):
            if layers[j] < c < layers[j + 1]:
                elem_layer[e] = j
                break
    return coords, elem_layer


def solve_1d(nu: float, layer_tops, layer_sigma):
    """Returns (coords, usin, ucos) as Harm1D writes them."""
    coords, elem_layer = mesh_1d(layer_tops)
    omega = float(nu) * 2.0 * PI_1D
    sig = np.asarray(layer_sigma, np.float64)[elem_layer]
    h = coords[1:] - coords[:-1]
    b = 1.0 / (MU0_1D * h)
    c = sig * omega * h / 6.0
    n = len(coords)
    # complex tridiagonal: diag d, off-diagonal o (symmetric)
    d = np.zeros(n, np.complex128)
    o = b * -1.0 + 1j * c                    # (b01 + i c01) with b01 = -b, c01 = c
    np.add.at(d, np.arange(n - 1), b + 2j * c)
    np.add.at(d, np.arange(1, n), b + 2j * c)
    f = np.zeros(n, np.complex128)
    f[-1] = 1.0
    # Dirichlet u[0] = 0: solve for nodes 1..n-1
    dd = d[1:].copy()
    oo = o[1:].copy()          # coupling between node k and k+1 for k >= 1
    ff = f[1:].copy()
    m = len(dd)
    for k in range(1, m):
        w = oo[k - 1] / dd[k - 1]
        dd[k] -= w * oo[k - 1]
        ff[k] -= w * ff[k - 1]
    u = np.zeros(m, np.complex128)
    u[-1] = ff[-1] / dd[-1]
    for k in range(m - 2, -1, -1):
        u[k] = (ff[k] - oo[k] * u[k + 1]) / dd[k]
    sol = np.concatenate([[0.0], u])
    return _q13(coords), _q13(sol.real), _q13(sol.imag)


def write_tables(path: str, coords, usin, ucos) -> None:
    import os
    with open(os.path.join(path, "usin.dat"), "w") as f:
        for z, v in zip(coords, usin):
            f.write(f"{z:25.13e} {v:25.13e}\n")
    with open(os.path.join(path, "ucos.dat"), "w") as f:
        for z, v in zip(coords, ucos):
            f.write(f"{z:25.13e} {v:25.13e}\n")
    with open(os.path.join(path, "setka1DEy"), "w") as f:
        f.write(f"{len(coords)}")


def read_tables(path: str):
    import os
    a = np.loadtxt(os.path.join(path, "usin.dat"))
    b = np.loadtxt(os.path.join(path, "ucos.dat"))
    return a[:, 0].copy(), a[:, 1].copy(), b[:, 1].copy()
