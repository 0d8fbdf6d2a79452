"""Batched survey solver over libmtgpu.

All frequencies x polarisations of a survey share the mesh, hence the
sparsity pattern and the matrices K and M of A(omega) = K + i omega M.
Survey solves such systems together with the reference's COCR, folded
preconditioner and MRS stop test, one lane per system in batches of up to
32 (the batches run side by side on streams of their own), in double-float
arithmetic (FP32 pairs, 48-bit significand) on the FP32 pipes; with
verify=True every system also reaches a true relative residual
||b - A x|| / ||b|| below eps.  Survey.multi puts systems of several meshes
(uneven sizes) in one survey, their vectors packed one after the other.

The reference solves the systems one by one in FP64 (CalcStarter runs
COCR_FP per frequency and polarisation, Code/CalcStarter/main.cpp:311-325).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


SPMV_VARIANTS = (0, 1, 2, 4, 8, 18, 20, 32, 33, 34, 35)   # include/mtgpu.h, mtgpu_survey_tuning


class Survey:
    def __init__(self, assembly, nus, stream=None, _parts=None):
        """assembly: an Assembly; nus: frequency [Hz] of every system."""
        parts = _parts if _parts is not None else [(assembly, nus)]
        self._assemblies = [a for a, _ in parts]
        counts = np.array([len(n) for _, n in parts], np.int32)
        nus = np.ascontiguousarray(np.concatenate([np.asarray(n, np.float64) for _, n in parts]))
        self.S = len(nus)
        self.nb = parts[0][0].nb
        self._assembly = parts[0][0]
        h = C.c_void_p()
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        arr = (C.c_void_p * len(parts))(*[a._h.value for a, _ in parts])
        rc = _lib.lib().mtgpu_survey_create_multi(len(parts), arr, counts, nus, sp, C.byref(h))
        _lib.check(rc, "mtgpu_survey_create_multi")
        self._h = h
        off = (C.c_longlong * (self.S + 1))()
        ng = C.c_int()
        _lib.check(_lib.lib().mtgpu_survey_info(h, None, C.byref(ng), off), "mtgpu_survey_info")
        self.offsets = np.array(off[:], np.int64)
        self.batches = ng.value

    @classmethod
    def multi(cls, parts, stream=None):
        """Systems on several meshes: parts = [(assembly, nus), ...].  The
        right-hand sides and solutions are flat float64 tensors, system k
        at [offsets[k], offsets[k + 1])."""
        return cls(None, None, stream, _parts=list(parts))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().mtgpu_survey_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spmv_timed(self, reps):
        """Device milliseconds of `reps` batched double-float SpMV launches."""
        ms = C.c_float()
        _lib.check(_lib.lib().mtgpu_survey_spmv_timed(self._h, int(reps), C.byref(ms)),
                   "mtgpu_survey_spmv_timed")
        return ms.value

    def spmv(self, x, y):
        """y[k] = A_k x[k] for every system with the SpMV variant in use;
        x, y: torch CUDA float64 tensors shaped (S, 2 nb)."""
        _lib.check(_lib.lib().mtgpu_survey_spmv(self._h, C.c_void_p(x.data_ptr()),
                                                C.c_void_p(y.data_ptr())), "mtgpu_survey_spmv")

    def tuning(self):
        """(chosen SpMV variant, {variant: ms per launch}) of the set-up
        autotuning; variants 0 and 1 stage x in shared memory per tile,
        18 and 20 (two systems) run one thread per row for both systems, 32
        is the matrix-free SpMV of tensor meshes, 33 the same with two
        systems per thread, 34 the same in one tiled kernel with the edge
        values and face circulations in shared memory, 35 the curl-curl part
        as D^T (F f) with the face mass matrix applied once per face."""
        v = C.c_int()
        ms = (C.c_float * len(SPMV_VARIANTS))()
        _lib.check(_lib.lib().mtgpu_survey_tuning(self._h, C.byref(v), ms),
                   "mtgpu_survey_tuning")
        return v.value, {c: ms[i] for i, c in enumerate(SPMV_VARIANTS) if ms[i] > 0}

    def preconditioner(self):
        """(fused, (ms per iteration unfused, fused)): whether the iteration's
        folded preconditioner runs as one fused kernel (tensor meshes)."""
        f = C.c_int()
        ms = (C.c_float * 2)()
        _lib.check(_lib.lib().mtgpu_survey_preconditioner(self._h, C.byref(f), ms),
                   "mtgpu_survey_preconditioner")
        return bool(f.value), (ms[0], ms[1])

    def set_spmv_variant(self, variant):
        """Pin the SpMV variant (0 x and matrix staged, 1 x staged, 2, 4, 8
        slots in flight, 18, 20 row per thread for two systems, 32-35
        matrix-free) instead of the autotuned one."""
        _lib.check(_lib.lib().mtgpu_survey_set_spmv_variant(self._h, int(variant)),
                   "mtgpu_survey_set_spmv_variant")

    def solve(self, b, x, eps=1e-8, maxiter=20000, verify=True):
        """b, x: torch CUDA float64 tensors, (S, 2 nb) on one mesh or flat
        with the packing `offsets`; x: initial guesses in, solutions out.
        Returns (code, stats dict)."""
        assert b.is_contiguous() and x.is_contiguous()
        assert b.numel() == x.numel() == int(self.offsets[-1])
        st = _lib.SurveyStats()
        rc = _lib.lib().mtgpu_survey_solve(self._h, C.c_void_p(b.data_ptr()),
                                           C.c_void_p(x.data_ptr()), float(eps), int(maxiter),
                                           int(verify), C.byref(st))
        _lib.check(rc, "mtgpu_survey_solve")
        S = self.S
        return rc, {"status": list(st.status[:S]), "iterations": list(st.iterations[:S]),
                    "verifications": list(st.verifications[:S]),
                    "fp64_iterations": list(st.fp64_iterations[:S]),
                    "true_residual_rel": list(st.true_residual_rel[:S]),
                    "residual_rel": list(st.residual_rel[:S]), "seconds": st.seconds}
