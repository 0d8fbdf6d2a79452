"""Device assembly (replaces the reference's BuildMatrix) over libmtgpu.

    Assembly(mesh)              K, M and the Dirichlet conditions on the GPU
    .block2x2(nu, alfa, ...)    the SLAE of one system in the reference's
                                lower-triangle block format (host arrays), as
                                BuildMatrix writes it
    .rhs(...)                   right-hand sides of S systems, on the device
    .cocr(nu)                   a CocrContext for A(2 pi nu), built on the GPU
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .slae_io import BlockSLAE
from .solver import CocrContext

MU_0 = 1.25663706143591729e-6   # Code/BuildMatrix/stdafx.h:31


class Assembly:
    def __init__(self, mesh, cell_sigma=None, tables="device"):
        """mesh: a RegularMesh (mesh.py).  cell_sigma: optional conductivity
        of every cell (unrounded); then every cell is its own material, with
        the mesh's background conductivity as its sigma0.  tables: "device"
        generates the mesh tables on the GPU from the node lines
        (mtgpu_assembly_create_regular); "host" builds them here and uploads
        them (mtgpu_assembly_create), as for a mesh read from files."""
        L = _lib.lib()
        if cell_sigma is None:
            nvkat, sig, sig0 = mesh.nvkat, mesh.mat_sigma, mesh.mat_sigma0
        else:
            sig = np.asarray(cell_sigma, np.float64).reshape(mesh.kpar)
            nvkat = np.arange(mesh.kpar, dtype=np.int32)
            sig0 = mesh.cell_sigma0
        self.nb = mesh.nb
        if tables == "device":
            f = lambda v: np.ascontiguousarray(v, np.float64)
            self._arrays = dict(nvkat=np.ascontiguousarray(nvkat, np.int32), sigma=f(sig),
                                sigma0=f(sig0), mu=np.full(len(sig), MU_0))
            a = self._arrays
            h = C.c_void_p()
            _lib.check(L.mtgpu_assembly_create_regular(
                mesh.nx, mesh.ny, mesh.nz, f(mesh.x), f(mesh.y), f(mesh.z), a["nvkat"],
                len(a["sigma"]), a["mu"], a["sigma"], a["sigma0"], C.byref(h)),
                "mtgpu_assembly_create_regular")
            self._h = h
            return
        if tables != "host":
            raise ValueError(f"tables must be 'device' or 'host', not {tables!r}")
        nver = np.ascontiguousarray(mesh.cell_nodes(), np.int32)
        ed = np.ascontiguousarray(mesh.cell_edges(), np.int32)
        self._arrays = dict(
            xyz=np.ascontiguousarray(mesh.xyz(), np.float64), nver=nver, ed=ed,
            edges=np.ascontiguousarray(mesh.edges(), np.int32),
            nvkat=np.ascontiguousarray(nvkat, np.int32),
            mu=np.full(len(sig), MU_0),
            sigma=np.ascontiguousarray(sig, np.float64),
            sigma0=np.ascontiguousarray(sig0, np.float64),
            bound=np.ascontiguousarray(mesh.boundary_nodes(), np.int32))
        a = self._arrays
        p = lambda k: a[k].ctypes.data_as(C.c_void_p)
        fm = _lib.FemMesh(mesh.kuzlov, mesh.kpar, mesh.nb, len(a["sigma"]), p("xyz"), p("nver"),
                          8, p("ed"), 12, p("edges"), p("nvkat"), p("mu"), None, p("sigma"),
                          p("sigma0"), None, None, len(a["bound"]), p("bound"))
        h = C.c_void_p()
        _lib.check(L.mtgpu_assembly_create(C.byref(fm), C.byref(h)), "mtgpu_assembly_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().mtgpu_assembly_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        a, b, c, d = C.c_longlong(), C.c_longlong(), C.c_int(), C.c_longlong()
        _lib.check(_lib.lib().mtgpu_assembly_info(self._h, C.byref(a), C.byref(b), C.byref(c),
                                                  C.byref(d)), "mtgpu_assembly_info")
        return dict(nnz_complex=a.value, nnz_real=b.value, nnz_lower=c.value, gg_len=d.value)

    def check_preconditioner(self):
        """True if the folded preconditioner's G and G^T built on the device
        (every solver set-up) equal the host construction entry for entry."""
        eq = C.c_int()
        _lib.check(_lib.lib().mtgpu_assembly_check_preconditioner(self._h, C.byref(eq)),
                   "mtgpu_assembly_check_preconditioner")
        return bool(eq.value)

    def block2x2(self, nu, alfa, z1d, usin, ucos, eps=1e-8, maxiter=10000) -> BlockSLAE:
        inf = self.info()
        nb, nnz = self.nb, inf["nnz_lower"]
        ig = np.zeros(nb + 1, np.int32)
        jg = np.zeros(max(nnz, 1), np.int32)
        idi = np.zeros(nb + 1, np.int32)
        ijg = np.zeros(nnz + 1, np.int32)
        di = np.zeros(2 * nb)
        gg = np.zeros(max(inf["gg_len"], 1))
        pr = np.zeros(2 * nb)
        f = lambda v: np.ascontiguousarray(v, np.float64)
        rc = _lib.lib().mtgpu_assembly_block2x2(self._h, float(nu), int(alfa), len(z1d), f(z1d),
                                                f(usin), f(ucos), ig, jg, idi, ijg, di, gg, pr)
        _lib.check(rc, "mtgpu_assembly_block2x2")
        return BlockSLAE(nb, ig, jg[:nnz], idi, ijg, di, gg[: inf["gg_len"]], pr, eps, maxiter)

    def rhs(self, nus, alfas, z1d, usins, ucoss, out):
        """out: torch CUDA float64 tensor of S * 2 nb (system-major)."""
        nus = np.ascontiguousarray(nus, np.float64)
        S = len(nus)
        rc = _lib.lib().mtgpu_assembly_rhs(
            self._h, S, nus, np.ascontiguousarray(alfas, np.int32), len(z1d),
            np.ascontiguousarray(z1d, np.float64),
            np.ascontiguousarray(np.reshape(usins, (S, -1)), np.float64),
            np.ascontiguousarray(np.reshape(ucoss, (S, -1)), np.float64),
            C.c_void_p(out.data_ptr()))
        _lib.check(rc, "mtgpu_assembly_rhs")

    def cocr(self, nu, stream=None) -> CocrContext:
        """stream: a torch.cuda.Stream (or None for a private stream)."""
        h = C.c_void_p()
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        rc = _lib.lib().mtgpu_cocr_create_from_assembly(self._h, float(nu), sp, C.byref(h))
        _lib.check(rc, "mtgpu_cocr_create_from_assembly")
        return CocrContext(handle=h, nb=self.nb)
