"""ctypes access to the CPU oracle (oracle/mtcalc_oracle.c) — TEST
INFRASTRUCTURE ONLY.  Imported by tests/, smoke() and bench.py's CPU-baseline
arm as the checker; the product never imports it."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_i = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    src = os.path.join(HERE, "mtcalc_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11",
                               "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


class OrcStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("residual_rel", C.c_double), ("seconds", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_spmv_block2x2.argtypes = [C.c_int, _i, _i, _i, _i, _d, _d, _d, _d, C.c_int]
        L.orc_pcocr_2x2_folded.argtypes = [
            C.c_int, _i, _i, _i, _i, _d, _d, _d, _d, C.c_double, C.c_int,
            C.c_int, C.c_int, C.c_int, _i, _i, _d, _i, _i, _i, _d, _i,
            C.c_int, C.c_int, C.POINTER(OrcStats)]
        L.orc_portrait.argtypes = [C.c_int, C.c_int, _i, C.c_int, _i, C.POINTER(C.POINTER(C.c_int))]
        L.orc_block_types.argtypes = [C.c_int, C.c_int, _i, C.c_int, _i, _i, _i, _i]
        L.orc_assemble.argtypes = [
            C.c_int, C.c_int, _d, _i, _i, C.c_int, _i, _i, _d, _d, _d, _d, _d, _d,
            C.c_double, C.c_int, C.c_int, _d, _d, _d, C.c_int, C.c_int, _i,
            _i, _i, _i, _i, _d, _d, _d]
        L.orc_folded_apply_once.argtypes = [
            C.c_int, _i, _i, _i, _i, _d, _d, C.c_int, C.c_int, _i, _i, _d, _i, _i, _i, _d, _i,
            _d, _d, _d, _d]
        L.orc_brick_bc.argtypes = [C.c_double, C.c_double, C.c_double, _d, _d]
        L.orc_locate_receivers.argtypes = [C.c_int, _i, _d, C.c_int, _d, _i]
        L.orc_receiver_eval.argtypes = [_i, _i, _d, C.c_int, _d, _i, _d, _d, _d]
        L.orc_dspline.restype = C.c_double
        L.orc_dspline.argtypes = [C.c_double, C.c_int, _d, _d]
        L.orc_normal_field.argtypes = [C.c_double, C.c_int, _d, _d, _d, C.c_int, C.c_double,
                                       _d, _d]
        L.orc_receiver_fields.argtypes = [C.c_int, _d, _d, C.c_double, _d, _d, _d, _d, _d]
        L.orc_mt_response.argtypes = [_d, _d, _d, _d, C.c_double, _d]
        _lib = L
    return _lib


def c32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def spmv(slae, x, nthreads=1):
    y = np.zeros(2 * slae.nb)
    lib().orc_spmv_block2x2(slae.nb, c32(slae.ig), c32(slae.jg), c32(slae.idi), c32(slae.ijg),
                            c64(slae.di), c64(slae.gg), c64(x), y, nthreads)
    return y


def pcocr(slae, mesh, x0=None, eps=None, maxiter=None, nthreads=1, iter_limit=0):
    """Returns (code, x, stats) of the oracle's PCOCR_2x2_Folded."""
    x = np.zeros(slae.n) if x0 is None else np.array(x0, np.float64)
    st = OrcStats()
    code = lib().orc_pcocr_2x2_folded(
        slae.n, c32(slae.ig), c32(slae.jg), c32(slae.idi), c32(slae.ijg),
        c64(slae.di), c64(slae.gg), c64(slae.pr), x,
        slae.eps if eps is None else eps, slae.maxiter if maxiter is None else maxiter,
        mesh.kpar, mesh.n_edges_c, mesh.n_nodes_c, c32(mesh.nvkat), c32(mesh.nver),
        c64(mesh.sigma), c32(mesh.edges), c32(mesh.ig_t), c32(mesh.jg_t), c64(mesh.gg_t),
        c32(mesh.is_node_bound), nthreads, iter_limit, C.byref(st))
    return code, x, st


def folded_apply(slae, mesh, x):
    """Returns (y, diag_a, diag_gagt) of the oracle's folded preconditioner."""
    y = np.zeros(slae.n)
    da = np.zeros(slae.n)
    ds = np.zeros(2 * mesh.n_nodes_c + 2)
    m = lib().orc_folded_apply_once(
        slae.nb, c32(slae.ig), c32(slae.jg), c32(slae.idi), c32(slae.ijg), c64(slae.di),
        c64(slae.gg), mesh.kpar, mesh.n_nodes_c, c32(mesh.nvkat), c32(mesh.nver).ravel(),
        c64(mesh.sigma), c32(mesh.edges).ravel(), c32(mesh.ig_t), c32(mesh.jg_t),
        c64(mesh.gg_t), c32(mesh.is_node_bound), c64(x), y, da, ds)
    return y, da, ds[: 2 * m]


def brick_bc(hx, hy, hz):
    b = np.zeros(144)
    c = np.zeros(144)
    lib().orc_brick_bc(hx, hy, hz, b, c)
    return b.reshape(12, 12), c.reshape(12, 12)


def assemble(m, nu, alfa, z1d, usin, ucos, eps=1e-8, maxiter=10000):
    """Assemble the block SLAE of a RegularMesh; returns a BlockSLAE."""
    from mtcalc_with_dfp_cocr_gb300.slae_io import BlockSLAE
    L = lib()
    nb, kpar = m.nb, m.kpar
    ed = c32(m.cell_edges())
    ig = np.zeros(nb + 1, np.int32)
    pj = C.POINTER(C.c_int)()
    nnz = L.orc_portrait(nb, kpar, ed, 12, ig, C.byref(pj))
    jg = np.ctypeslib.as_array(pj, shape=(max(nnz, 1),))[:nnz].copy()
    C.CDLL(None).free(pj)
    idi = np.zeros(nb + 1, np.int32)
    ijg = np.zeros(nnz + 1, np.int32)
    L.orc_block_types(nb, kpar, ed, 12, ig, jg, idi, ijg)
    di = np.zeros(int(idi[nb]))
    gg = np.zeros(int(ijg[nnz]))
    pr = np.zeros(2 * nb)
    nver = np.zeros((kpar, 14), np.int32)
    nver[:, :8] = m.cell_nodes()
    nmat = len(m.mat_sigma)
    MU_0 = 1.25663706143591729e-6
    mu = np.full(nmat, MU_0)
    zero = np.zeros(nmat)
    bnd = c32(m.boundary_nodes())
    L.orc_assemble(nb, kpar, c64(m.xyz()), nver, ed, 12, c32(m.edges()), c32(m.nvkat),
                   mu, mu.copy(), c64(m.mat_sigma), c64(m.mat_sigma0), zero, zero.copy(),
                   float(nu), int(alfa), len(z1d), c64(z1d), c64(usin), c64(ucos),
                   m.kuzlov, len(bnd), bnd, ig, jg, idi, ijg, di, gg, pr)
    return BlockSLAE(nb, ig, jg, idi, ijg, di, gg, pr, eps, maxiter)


# ---- receivers and MT responses ---------------------------------------------

MT_RECORD = 34


def locate_receivers(m, rec):
    """First element (index order) whose closed box holds each receiver."""
    nver = np.zeros((m.kpar, 14), np.int32)
    nver[:, :8] = m.cell_nodes()
    rec = c64(rec)
    elem = np.empty(len(rec), np.int32)
    lib().orc_locate_receivers(m.kpar, nver, c64(m.xyz()), len(rec), rec, elem)
    return elem


def receiver_eval(m, rec, v3, elem=None):
    """A and curl A at the receivers: two (R, 3) complex arrays."""
    rec = c64(rec)
    if elem is None:
        elem = locate_receivers(m, rec)
    nver = np.zeros((m.kpar, 14), np.int32)
    nver[:, :8] = m.cell_nodes()
    ed = np.zeros((m.kpar, 25), np.int32)
    ed[:, :12] = m.cell_edges()
    v = c64(np.asarray(v3).view(np.float64) if np.iscomplexobj(v3) else v3)
    a = np.zeros(6 * len(rec))
    curl = np.zeros(6 * len(rec))
    lib().orc_receiver_eval(nver, ed, c64(m.xyz()), len(rec), rec, c32(elem), v, a, curl)
    return a.view(np.complex128).reshape(-1, 3), curl.view(np.complex128).reshape(-1, 3)


def dspline(x, z, v):
    return lib().orc_dspline(float(x), len(z), c64(z), c64(v))


def normal_field(rec, z1d, usin, ucos, alfa, omega):
    """e2d / b2d rows (R, 6) of the 1-D field at the receivers."""
    rec = np.asarray(rec, np.float64)
    e = np.zeros((len(rec), 6))
    b = np.zeros((len(rec), 6))
    for r in range(len(rec)):
        er, br = np.zeros(6), np.zeros(6)
        lib().orc_normal_field(float(rec[r, 2]), len(z1d), c64(z1d), c64(usin), c64(ucos),
                               int(alfa), float(omega), er, br)
        e[r], b[r] = er, br
    return e, b


def receiver_fields(a, curl, omega, e1d, b1d):
    """Total E, H (R, 3) complex and the (rho, |Z|) scalars (R, 2)."""
    R = len(a)
    e = np.zeros(6 * R)
    h = np.zeros(6 * R)
    s = np.zeros(2 * R)
    lib().orc_receiver_fields(R, c64(np.asarray(a, np.complex128).view(np.float64)),
                              c64(np.asarray(curl, np.complex128).view(np.float64)),
                              float(omega), c64(e1d), c64(b1d), e, h, s)
    return e.view(np.complex128).reshape(R, 3), h.view(np.complex128).reshape(R, 3), \
        s.reshape(R, 2)


def mt_response(e0, h0, e1, h1, omega):
    """MT_RECORD doubles from the X- and Y-polarisation fields (3 complex each)."""
    out = np.zeros(MT_RECORD)
    f = lambda v: c64(np.asarray(v, np.complex128).view(np.float64))
    lib().orc_mt_response(f(e0), f(h0), f(e1), f(h1), float(omega), out)
    return out
