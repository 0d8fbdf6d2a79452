"""Reading and writing the solve stage's file interface.

The block SLAE files are the contract between BuildMatrix and COCR_FP
(Code/BuildMatrix/t_global_slae.cpp:174-202 writes them,
Code/COCR_FP/HarmVect3d.cpp:118-336 reads them): raw little-endian arrays,
int32 indices 1-based, float64 values, no headers.

    kuslau   text "n eps maxiter" (n = 2 * number of edges)
    pr       f64[n]            right-hand side, re/im interleaved
    ig       i32[nb+1]         lower-triangle row pointers
    jg       i32[ig[nb]-1]     column indices
    idi      i32[nb+1]         offsets of the diagonal blocks in di
    ijg      i32[ig[nb]]       offsets of the off-diagonal blocks in gg
    di, gg   f64               block values: 1 double (real) or 2 (re, im)
    v3.dat   f64[n]            the solution, re/im interleaved

Everything returned here is 0-based.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np


@dataclass
class BlockSLAE:
    nb: int
    ig: np.ndarray
    jg: np.ndarray
    idi: np.ndarray
    ijg: np.ndarray
    di: np.ndarray
    gg: np.ndarray
    pr: np.ndarray
    eps: float = 1e-8
    maxiter: int = 10000

    @property
    def n(self) -> int:
        return 2 * self.nb

    def to_dense(self) -> np.ndarray:
        """Complex dense matrix (small cases only)."""
        A = np.zeros((self.nb, self.nb), np.complex128)
        for i in range(self.nb):
            s = self.idi[i + 1] - self.idi[i]
            A[i, i] = self.di[self.idi[i]] + (1j * self.di[self.idi[i] + 1] if s == 2 else 0)
            for q in range(self.ig[i], self.ig[i + 1]):
                j = self.jg[q]
                s = self.ijg[q + 1] - self.ijg[q]
                v = self.gg[self.ijg[q]] + (1j * self.gg[self.ijg[q] + 1] if s == 2 else 0)
                A[i, j] = v
                A[j, i] = v
        return A


def _rd(path, dtype, count=-1):
    a = np.fromfile(path, dtype=dtype, count=count)
    if count >= 0 and a.size != count:
        raise IOError(f"cannot read {count} values from {path} (got {a.size})")
    return a


def read_slae(path: str) -> BlockSLAE:
    P = lambda f: os.path.join(path, f)
    with open(P("kuslau")) as f:
        tok = f.read().split()
    n, eps, maxiter = int(tok[0]), float(tok[1]), int(tok[2])
    nb = n // 2
    pr = _rd(P("pr"), "<f8", n)
    ig = _rd(P("ig"), "<i4", nb + 1).astype(np.int32) - 1
    idi = _rd(P("idi"), "<i4", nb + 1).astype(np.int32) - 1
    nnz = int(ig[nb])
    jg = _rd(P("jg"), "<i4", nnz).astype(np.int32) - 1
    ijg = _rd(P("ijg"), "<i4", nnz + 1).astype(np.int32) - 1
    di = _rd(P("di"), "<f8", int(idi[nb]))
    gg = _rd(P("gg"), "<f8", int(ijg[nnz]))
    return BlockSLAE(nb, ig, jg, idi, ijg, di, gg, pr, eps, maxiter)


def write_slae(path: str, s: BlockSLAE) -> None:
    os.makedirs(path, exist_ok=True)
    P = lambda f: os.path.join(path, f)
    with open(P("kuslau"), "w") as f:
        f.write(f"{s.n}\n{s.eps:e}\n{s.maxiter}\n")
    s.pr.astype("<f8").tofile(P("pr"))
    s.di.astype("<f8").tofile(P("di"))
    s.gg.astype("<f8").tofile(P("gg"))
    (s.ig + 1).astype("<i4").tofile(P("ig"))
    (s.jg + 1).astype("<i4").tofile(P("jg"))
    (s.idi + 1).astype("<i4").tofile(P("idi"))
    (s.ijg + 1).astype("<i4").tofile(P("ijg"))


@dataclass
class SolveMesh:
    """The mesh arrays PCOCR_2x2_Folded takes for the folded preconditioner
    (Code/COCR_FP/pcocr.h:27-31), 0-based."""
    kpar: int
    n_edges_c: int
    n_nodes_c: int
    xyz: np.ndarray          # (kuzlov, 3) f64
    nvkat: np.ndarray        # (kpar,) i32
    nver: np.ndarray         # (kpar, 14) i32
    sigma: np.ndarray        # (n_materials,) f64: 1 where sigma3d != 0 else 0
    edges: np.ndarray        # (nb, 2) i32
    ig_t: np.ndarray         # (kuzlov+1,) i32
    jg_t: np.ndarray         # i32
    gg_t: np.ndarray         # f64
    is_node_bound: np.ndarray  # (kuzlov,) i32


def read_inftry(path: str):
    with open(path) as f:
        tok = f.read().split()
    out = {}
    for i, t in enumerate(tok):
        if t in ("KUZLOV=", "KPAR=", "KT1="):
            out[t[:-1]] = int(tok[i + 1])
    return out["KUZLOV"], out["KPAR"], out["KT1"]


def read_solve_mesh(path: str) -> SolveMesh:
    """Read the mesh files COCR_FP reads (HarmVect3d.cpp:36-112, 247-316,
    vec_prep_data.cpp:55-187) for a conforming mesh (tsize3d = 0)."""
    P = lambda f: os.path.join(path, f)
    kuzlov, kpar, kt1 = read_inftry(P("inftry.dat"))
    xyz = _rd(P("xyz.dat"), "<f8", kuzlov * 3).reshape(kuzlov, 3)
    nver = (_rd(P("nver.dat"), "<i4", kpar * 14).reshape(kpar, 14) - 1).astype(np.int32)
    nvkat = (_rd(P("nvkat.dat"), "<i4", kpar) - 1).astype(np.int32)
    l13d = (_rd(P("l13d.dat"), "<i4", kt1) - 1).astype(np.int32)
    with open(P("tsize3d_.dat")) as f:
        tok = f.read().split()
    nb = int(tok[1])
    edges = (_rd(P("nodesforedges.dat"), "<i4", nb * 2).reshape(nb, 2) - 1).astype(np.int32)
    sig = np.loadtxt(P("sig3d"), ndmin=2)
    nmat = int(sig[:, 0].max())
    sigma3d = np.zeros(nmat)
    sigma3d[sig[:, 0].astype(int) - 1] = sig[:, 1]
    bound = np.zeros(kuzlov, np.int32)
    bound[l13d] = 1
    tsize = 0
    if os.path.exists(P("tsize3d.dat")):
        with open(P("tsize3d.dat")) as f:
            tsize = int(f.read().split()[0])
    if tsize != 0:
        raise NotImplementedError("non-conforming meshes (tsize3d.dat > 0)")
    return SolveMesh(kpar, nb, kuzlov - tsize, xyz, nvkat, nver,
                     (sigma3d != 0).astype(np.float64), edges,
                     np.zeros(kuzlov + 1, np.int32), np.zeros(1, np.int32),
                     np.zeros(1, np.float64), bound)


def mesh_to_solve_mesh(m) -> SolveMesh:
    """SolveMesh from an in-memory RegularMesh."""
    nver = np.zeros((m.kpar, 14), np.int32)
    nver[:, :8] = m.cell_nodes()
    return SolveMesh(m.kpar, m.nb, m.kuzlov, m.xyz(), m.nvkat, nver,
                     np.asarray(m.mat_sigma, np.float64), m.edges(),
                     np.zeros(m.kuzlov + 1, np.int32), np.zeros(1, np.int32),
                     np.zeros(1, np.float64), m.is_node_bound())


def read_v3(path: str, n: int) -> np.ndarray:
    return _rd(path, "<f8", n)


def write_v3(path: str, x: np.ndarray) -> None:
    np.asarray(x, "<f8").tofile(path)


def read_kit(path: str):
    """Parse the `kit` line "r=%e\teps=%e\tkit=%d\ttime=%lf sec"
    (Code/COCR_FP/base_solver.cpp:181-200)."""
    with open(path) as f:
        s = f.read()
    out = {}
    for tok in s.replace("\t", " ").split():
        if "=" in tok:
            k, v = tok.split("=", 1)
            out[k] = v
    return float(out["r"]), float(out["eps"]), int(out["kit"]), float(out["time"])
