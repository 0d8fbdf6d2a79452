"""Receiver output by subdomain L2-projection smoothing — CPU restatement,
TEST INFRASTRUCTURE ONLY (imported by tests/ as the checker; the product
never imports it).

Restates the reference's default E/H output (Code/OutputNu, taken when
direct output is off, give_out_vec_mt.cpp:200-237):

* receiver location (OutputResultant3d::FindPointsForElems,
  OutputResultant3d.cpp:293-450): the first cell in index order whose box,
  grown by 1e-6 on every side, holds the receiver; for A (E) cells of
  material 0, the air, are skipped;
* subdomains (OutputResultant3d::InitSubdomains, :83-147; Subdomain::Init,
  Subdomain.cpp:132-478): for curl A one subdomain over all materials, for A
  one per material that holds a receiver; each starts from its receivers'
  cells and grows `levels` (5) times by every cell of its material that
  shares a node with it (the node set is that of the cells before the
  level);
* nodal trilinear mass matrix over the subdomain's cells
  (Subdomain::AsmGlobalMatrix, :483-622; Hex_Local_Matrix.cpp:120-198:
  V/27, V/54, V/108, V/216 by the number of differing local axes) and the
  right-hand side sum over cells of (row sum of the cell matrix) x (value at
  the cell centre) (Subdomain::AsmGlobalVector, :626-661;
  Give_out_vec_mt::GetValueInElementCenter, give_out_vec_mt.cpp:645-688);
* the projection solve (PARDISO there, scipy's sparse direct solver here);
* the receiver value: the trilinear interpolant of the nodal values in the
  receiver's cell (OutputResultant3d::Output, :152-199;
  T_Brick::ScalarFieldOnParCff, T_Brick.cpp:2060-2073).

Conforming (tensor) meshes only: they have no terminal nodes, so the
T-matrix part of Subdomain (BuildSigmaStruct, Correct_T_Node, BuildTMatrix)
is empty.  Checked against the reference's own classes
(oracle/_ref/ref_smoothing, tests/golden/smoothing.npz).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import pyoracle

AIR = 0          # material 0: the air (RegularMeshBuilder main.cpp:1184-1188)
LEVELS = 5       # OutputResultant3d.cpp:45 (no C:\GI\n_neib file)
BOX_EPS = 1e-6   # OutputResultant3d.cpp:337-344


def locate(m, rec, skip_air):
    """Cell of every receiver (-1: none), OutputResultant3d.cpp:293-450."""
    nodes = m.cell_nodes()
    xyz = m.xyz()
    lo = xyz[nodes[:, 0]] - BOX_EPS
    hi = xyz[nodes[:, 7]] + BOX_EPS
    ok = (m.nvkat != AIR) if skip_air else np.ones(m.kpar, bool)
    out = np.full(len(rec), -1, np.int64)
    for r, p in enumerate(np.asarray(rec, np.float64)):
        hit = np.flatnonzero(ok & np.all(lo <= p, axis=1) & np.all(p <= hi, axis=1))
        if len(hit):
            out[r] = hit[0]
    return out


def subdomain(m, seed_cells, material, levels=LEVELS):
    """Cells and nodes (ascending global indices) of one subdomain,
    Subdomain.cpp:132-246."""
    nodes = m.cell_nodes()
    allowed = np.ones(m.kpar, bool) if material < 0 else (m.nvkat == material)
    in_cell = np.zeros(m.kpar, bool)
    seed = np.asarray([c for c in seed_cells if c >= 0 and allowed[c]], np.int64)
    in_cell[seed] = True
    in_node = np.zeros(m.kuzlov, bool)
    in_node[nodes[seed].ravel()] = True
    for _ in range(levels):
        new = ~in_cell & allowed & in_node[nodes].any(axis=1)
        in_cell |= new
        in_node[nodes[new].ravel()] = True
    return np.flatnonzero(in_cell), np.flatnonzero(in_node)


def cell_mass(hx, hy, hz):
    """(n, 8, 8) trilinear mass matrices of bricks, Hex_Local_Matrix.cpp:120-198."""
    t2 = hx * hy * hz
    t = np.stack([t2 / 27.0, t2 / 54.0, t2 / 108.0, t2 / 216.0], axis=-1)
    j = np.arange(8)
    diff = np.array([[bin(a ^ b).count("1") for b in j] for a in j])
    return t[:, diff]


def centre_values(m, cells, v3):
    """(n, 6) complex: A and curl A at the cell centres (local point 0)."""
    xyz = m.xyz()
    nodes = m.cell_nodes()[cells]
    ctr = 0.5 * (xyz[nodes[:, 0]] + xyz[nodes[:, 7]])
    a, curl = pyoracle.receiver_eval(m, ctr, v3, elem=np.asarray(cells, np.int32))
    return np.concatenate([a, curl], axis=1)


def project(m, cells, nodes, values):
    """Nodal values (len(nodes), k) of the L2 projection of the cellwise
    constants values (len(cells), k), Subdomain.cpp:483-661."""
    cn = m.cell_nodes()[cells]
    xyz = m.xyz()
    h = xyz[cn[:, 7]] - xyz[cn[:, 0]]
    b = cell_mass(h[:, 0], h[:, 1], h[:, 2])
    loc = np.searchsorted(nodes, cn)
    rows = np.repeat(loc, 8, axis=1).ravel()
    cols = np.tile(loc, (1, 8)).ravel()
    M = sp.csc_matrix((b.ravel(), (rows, cols)), shape=(len(nodes), len(nodes)))
    g = b.sum(axis=2)                                  # (n, 8) row sums
    rhs = np.zeros((len(nodes), values.shape[1]), values.dtype)
    np.add.at(rhs, loc.ravel(), (g[:, :, None] * values[:, None, :]).reshape(-1, values.shape[1]))
    lu = spla.splu(M)
    if np.iscomplexobj(rhs):
        return lu.solve(rhs.real) + 1j * lu.solve(rhs.imag)
    return lu.solve(rhs)


def trilinear(m, cell, p):
    """The 8 nodal basis values at point p of a brick, T_Brick.cpp:866-887, 2010-2023."""
    xyz = m.xyz()
    n = m.cell_nodes()[cell]
    a, b = xyz[n[0]], xyz[n[7]]
    loc = (2.0 * np.asarray(p) - a - b) / (b - a)
    l0, l1 = 0.5 * (1.0 - loc), 0.5 * (1.0 + loc)
    return np.array([l0[0] * l0[1] * l0[2], l1[0] * l0[1] * l0[2], l0[0] * l1[1] * l0[2],
                     l1[0] * l1[1] * l0[2], l0[0] * l0[1] * l1[2], l1[0] * l0[1] * l1[2],
                     l0[0] * l1[1] * l1[2], l1[0] * l1[1] * l1[2]])


def smoothed_fields(m, rec, v3, levels=LEVELS):
    """Smoothed A and curl A at the receivers: two (R, 3) complex arrays
    (zero where a receiver has no cell), for one solution v3 (nb complex, or
    real (re, im) pairs as (nb, 2) or interleaved)."""
    v3 = np.asarray(v3)
    if not np.iscomplexobj(v3):
        v3 = np.ascontiguousarray(v3, np.float64).reshape(-1, 2)
        v3 = v3[:, 0] + 1j * v3[:, 1]
    v3 = np.ascontiguousarray(v3, np.complex128)
    rec = np.asarray(rec, np.float64)
    R = len(rec)
    a_out = np.zeros((R, 3), np.complex128)
    c_out = np.zeros((R, 3), np.complex128)
    cn = m.cell_nodes()
    # curl A: one subdomain over all materials
    eb = locate(m, rec, skip_air=False)
    groups = [(eb, -1, c_out, slice(3, 6))]
    # A: one subdomain per material holding a receiver
    ea = locate(m, rec, skip_air=True)
    for mat in sorted({int(m.nvkat[c]) for c in ea if c >= 0}):
        groups.append((ea, mat, a_out, slice(0, 3)))
    for elem, mat, dst, cols in groups:
        seed = [c for c in elem if c >= 0 and (mat < 0 or m.nvkat[c] == mat)]
        cells, nodes = subdomain(m, seed, mat, levels)
        vals = centre_values(m, cells, v3)[:, cols]
        u = project(m, cells, nodes, vals)
        for r in range(R):
            c = elem[r]
            if c < 0 or (mat >= 0 and m.nvkat[c] != mat):
                continue
            w = trilinear(m, c, rec[r])
            dst[r] = w @ u[np.searchsorted(nodes, cn[c])]
    return a_out, c_out
