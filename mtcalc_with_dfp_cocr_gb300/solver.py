"""Host-side mirror of the reference solver interface, over libmtgpu.

    pcocr_2x2_folded   PCOCR::PCOCR_2x2_Folded  (Code/COCR_FP/pcocr.cpp:40-126)
    mult_mv_block_2x2  Block_2x2_solver::Mult_MV_block_2x2
                       (Code/COCR_FP/block_2x2_solver.cpp:73-173)
    folded_apply       FoldedPreconditioner::BuildGMatrix + BuildDiagComplex +
                       ApplyPreconditionerComplex
                       (Code/COCR_FP/FoldedPreconditioner.cpp)
    CocrContext        the device-resident form: matrix, preconditioner and
                       vectors stay in GPU memory (torch tensors as buffers)

Return codes are the reference's (0, -1 x0 is the solution, -2 breakdown,
-3 maxiter); library failures raise MtgpuError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from .slae_io import BlockSLAE, SolveMesh

i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)


def _mesh_args(m: SolveMesh):
    return (m.kpar, m.n_edges_c, m.n_nodes_c, f64(m.xyz).ravel(), i32(m.nvkat),
            i32(m.nver).ravel(), f64(m.sigma), i32(m.edges).ravel(), i32(m.ig_t),
            i32(m.jg_t), f64(m.gg_t), i32(m.is_node_bound))


def pcocr_2x2_folded(slae: BlockSLAE, mesh: SolveMesh, x0=None, eps=None, maxiter=None,
                     stop_on_true_residual=False, iterations_per_launch=0, write_kit_in=None,
                     double_float=False, x=None):
    """Solve A x = pr on the GPU.  Returns (code, x, stats).

    x0: initial guess (copied); x: a contiguous float64 array used in place
    instead, initial guess in and solution out (as the reference's x), e.g.
    in pinned host memory.  write_kit_in: a directory; when given, the
    reference entry point (mtgpu_pcocr_2x2_folded) runs there and writes its
    `kit` file."""
    L = _lib.lib()
    if x is not None:
        assert x.dtype == np.float64 and x.flags.c_contiguous and x.size == slae.n
    else:
        x = np.zeros(slae.n) if x0 is None else np.array(x0, np.float64)
    eps = slae.eps if eps is None else eps
    maxiter = slae.maxiter if maxiter is None else maxiter
    slae_args = (slae.n, i32(slae.ig), i32(slae.jg), i32(slae.idi), i32(slae.ijg),
                 f64(slae.di), f64(slae.gg), f64(slae.pr), x, float(eps), int(maxiter))
    if write_kit_in is not None:
        cwd = os.getcwd()
        os.chdir(write_kit_in)
        try:
            rc = L.mtgpu_pcocr_2x2_folded(*slae_args, None, *_mesh_args(mesh))
        finally:
            os.chdir(cwd)
        _lib.check(rc, "mtgpu_pcocr_2x2_folded")
        return rc, x, None
    st = _lib.SolveStats()
    opts = _lib.SolveOpts(int(stop_on_true_residual), int(iterations_per_launch),
                          int(double_float))
    rc = L.mtgpu_pcocr_2x2_folded_ex(*slae_args, *_mesh_args(mesh), C.byref(opts), C.byref(st))
    _lib.check(rc, "mtgpu_pcocr_2x2_folded_ex")
    return rc, x, st


def mult_mv_block_2x2(slae: BlockSLAE, x) -> np.ndarray:
    y = np.zeros(slae.n)
    rc = _lib.lib().mtgpu_mult_mv_block_2x2(slae.nb, i32(slae.ig), i32(slae.jg), i32(slae.idi),
                                            i32(slae.ijg), f64(slae.di), f64(slae.gg), f64(x), y)
    _lib.check(rc, "mtgpu_mult_mv_block_2x2")
    return y


def folded_apply(slae: BlockSLAE, mesh: SolveMesh, x):
    """Returns (y, diag_a, diag_gagt) with y = D_A x + G^T D_S G x."""
    y = np.zeros(slae.n)
    da = np.zeros(slae.n)
    ds = np.zeros(2 * mesh.n_nodes_c + 2)
    m = C.c_int(0)
    rc = _lib.lib().mtgpu_folded_apply(
        slae.nb, i32(slae.ig), i32(slae.jg), i32(slae.idi), i32(slae.ijg), f64(slae.di),
        f64(slae.gg), mesh.kpar, mesh.n_nodes_c, i32(mesh.nvkat), i32(mesh.nver).ravel(),
        f64(mesh.sigma), i32(mesh.edges).ravel(), i32(mesh.ig_t), i32(mesh.jg_t),
        f64(mesh.gg_t), i32(mesh.is_node_bound), f64(x), y, C.byref(m),
        da.ctypes.data_as(C.c_void_p), ds.ctypes.data_as(C.c_void_p))
    _lib.check(rc, "mtgpu_folded_apply")
    return y, da, ds[: 2 * m.value]


class CocrContext:
    """Matrix + folded preconditioner resident on the GPU.

    slae: a BlockSLAE (host arrays) or a dict of torch CUDA tensors with keys
    ig, jg, idi, ijg (int32) and di, gg (float64) holding the same 0-based
    lower storage (device-resident input)."""

    def __init__(self, slae=None, mesh: SolveMesh | None = None, nb: int | None = None,
                 handle=None):
        L = _lib.lib()
        self._keep = []
        if handle is not None:          # built elsewhere (e.g. from a device assembly)
            self._h, self.nb = handle, int(nb)
            return
        h = C.c_void_p()
        if isinstance(slae, BlockSLAE):
            self.nb = slae.nb
            arrs = [i32(slae.ig), i32(slae.jg), i32(slae.idi), i32(slae.ijg), f64(slae.di),
                    f64(slae.gg)]
            self._keep += arrs
            ptrs = [a.ctypes.data_as(C.c_void_p) for a in arrs]
            on_dev, nnz = 0, int(slae.ig[slae.nb])
        else:
            self.nb = int(nb)
            ptrs = [C.c_void_p(slae[k].data_ptr()) for k in ("ig", "jg", "idi", "ijg", "di", "gg")]
            self._keep.append(slae)
            on_dev, nnz = 1, int(slae["jg"].numel())
        margs = [i32(mesh.nvkat), i32(mesh.nver).ravel(), f64(mesh.sigma),
                 i32(mesh.edges).ravel(), i32(mesh.ig_t), i32(mesh.jg_t), f64(mesh.gg_t),
                 i32(mesh.is_node_bound)]
        rc = L.mtgpu_cocr_create(self.nb, nnz, *ptrs, on_dev, mesh.kpar, mesh.n_nodes_c,
                                 *margs, None, C.byref(h))
        _lib.check(rc, "mtgpu_cocr_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().mtgpu_cocr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        a, b, m = C.c_longlong(), C.c_longlong(), C.c_int()
        _lib.check(_lib.lib().mtgpu_cocr_info(self._h, C.byref(a), C.byref(b), C.byref(m)),
                   "mtgpu_cocr_info")
        return a.value, b.value, m.value

    def solve(self, b, x, eps=1e-8, maxiter=10000, stop_on_true_residual=False,
              iterations_per_launch=0):
        """b, x: torch CUDA float64 tensors of 2*nb; x is updated in place."""
        st = _lib.SolveStats()
        opts = _lib.SolveOpts(int(stop_on_true_residual), int(iterations_per_launch), 0)
        rc = _lib.lib().mtgpu_cocr_solve(self._h, C.c_void_p(b.data_ptr()),
                                         C.c_void_p(x.data_ptr()), float(eps), int(maxiter),
                                         C.byref(opts), C.byref(st))
        _lib.check(rc, "mtgpu_cocr_solve")
        return rc, st

    def spmv(self, x, y):
        _lib.check(_lib.lib().mtgpu_cocr_spmv(self._h, C.c_void_p(x.data_ptr()),
                                              C.c_void_p(y.data_ptr())), "mtgpu_cocr_spmv")

    def spmv_timed(self, x, y, reps):
        """Device milliseconds of `reps` back-to-back SpMV launches."""
        ms = C.c_float()
        _lib.check(_lib.lib().mtgpu_cocr_spmv_timed(self._h, C.c_void_p(x.data_ptr()),
                                                    C.c_void_p(y.data_ptr()), int(reps),
                                                    C.byref(ms)), "mtgpu_cocr_spmv_timed")
        return ms.value

    def precond(self, x, y):
        _lib.check(_lib.lib().mtgpu_cocr_precond(self._h, C.c_void_p(x.data_ptr()),
                                                 C.c_void_p(y.data_ptr())), "mtgpu_cocr_precond")
