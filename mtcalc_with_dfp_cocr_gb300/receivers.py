"""Receiver fields and MT responses on the GPU (over libmtgpu).

    Receivers(assembly, points, output="direct" | "smooth", levels=5)
                                    locate the receivers in the mesh
    .fields(x, nus, alfas, ...)     E, H at the receivers for S solutions, as
                                    the reference's OutputNu gives them (its
                                    direct evaluation, or its default
                                    subdomain smoothing) plus Harm1D's
                                    normal field
    .mt_response(nus, sys_x, sys_y, E, H)
                                    impedance tensor, tipper, apparent
                                    resistivities and phases per frequency
                                    (calcimpedance), one record of
                                    MT_RECORD doubles per receiver

Device arrays are torch CUDA tensors (float64).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

MT_RECORD = 34
# offsets in one record (include/mtgpu.h MTGPU_MT_*)
MT_Z, MT_W, MT_ZABS, MT_ZPHASE, MT_RHO, MT_RHOPHASE, MT_RHOEFF, MT_WABS = (
    0, 8, 12, 16, 20, 24, 28, 30)


OUTPUTS = {"direct": 0, "smooth": 1}   # MTGPU_OUTPUT_DIRECT / MTGPU_OUTPUT_SMOOTH


class Receivers:
    """output="direct": the edge basis evaluated at the receiver (the
    reference's direct output); output="smooth": the reference's default
    output, subdomain L2-projection smoothing over `levels` neighbour levels
    (include/mtgpu.h, mtgpu_receivers_set_output).  The assembly must outlive
    a smoothed Receivers."""

    def __init__(self, assembly, points, output="direct", levels=5):
        pts = np.ascontiguousarray(np.reshape(points, (-1, 3)), np.float64)
        if output not in OUTPUTS:
            raise ValueError(f"output must be one of {sorted(OUTPUTS)}")
        h = C.c_void_p()
        rc = _lib.lib().mtgpu_receivers_create(assembly._h, len(pts), pts, C.byref(h))
        _lib.check(rc, "mtgpu_receivers_create")
        self._h = h
        self.nrec = len(pts)
        self.points = pts
        self.output = output
        self._assembly = assembly   # kept alive for the smoothing output
        if output != "direct":
            rc = _lib.lib().mtgpu_receivers_set_output(h, assembly._h, OUTPUTS[output], levels)
            _lib.check(rc, "mtgpu_receivers_set_output")

    def smoothing_info(self):
        """Per smoothing subdomain (0: curl A, all materials; then A per
        material): material, bricks, nodes; and the conjugate-gradient
        iterations of the last fields() call."""
        n, it = C.c_int(), C.c_int()
        mx = 64
        mat, cells, nodes = (np.zeros(mx, np.int32) for _ in range(3))
        rc = _lib.lib().mtgpu_receivers_smoothing_info(
            self._h, mx, C.byref(n), mat.ctypes.data_as(C.c_void_p),
            cells.ctypes.data_as(C.c_void_p), nodes.ctypes.data_as(C.c_void_p), C.byref(it))
        _lib.check(rc, "mtgpu_receivers_smoothing_info")
        k = min(n.value, mx)
        return {"material": mat[:k].tolist(), "cells": cells[:k].tolist(),
                "nodes": nodes[:k].tolist(), "iterations": it.value}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().mtgpu_receivers_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        """(n_unlocated, elem[nrec]) of the receiver location."""
        n, miss = C.c_int(), C.c_int()
        elem = np.empty(self.nrec, np.int32)
        rc = _lib.lib().mtgpu_receivers_info(self._h, C.byref(n), C.byref(miss),
                                             elem.ctypes.data_as(C.c_void_p))
        _lib.check(rc, "mtgpu_receivers_info")
        return miss.value, elem

    def fields(self, x, nus, alfas, z1d, usins, ucoss):
        """x: CUDA float64 tensor of S * 2 nb (system-major solutions).
        Returns E, H as complex128 CUDA tensors (S, nrec, 3) and the
        reference's (rho, |Z|) scalars (S, nrec, 2)."""
        nus = np.ascontiguousarray(nus, np.float64)
        S = len(nus)
        dev = x.device
        e = torch.empty(S * self.nrec * 6, dtype=torch.float64, device=dev)
        h = torch.empty_like(e)
        s = torch.empty(S * self.nrec * 2, dtype=torch.float64, device=dev)
        rc = _lib.lib().mtgpu_receivers_fields(
            self._h, S, nus, np.ascontiguousarray(alfas, np.int32), len(z1d),
            np.ascontiguousarray(z1d, np.float64),
            np.ascontiguousarray(np.reshape(usins, (S, -1)), np.float64),
            np.ascontiguousarray(np.reshape(ucoss, (S, -1)), np.float64),
            C.c_void_p(x.data_ptr()), C.c_void_p(e.data_ptr()), C.c_void_p(h.data_ptr()),
            C.c_void_p(s.data_ptr()))
        _lib.check(rc, "mtgpu_receivers_fields")
        cplx = lambda t: torch.view_as_complex(t.view(S, self.nrec, 3, 2))
        return cplx(e), cplx(h), s.view(S, self.nrec, 2)

    def mt_response(self, nus, sys_x, sys_y, E, H):
        """E, H: (S, nrec, 3) complex128 CUDA tensors from fields().
        Returns a float64 CUDA tensor (nf, nrec, MT_RECORD)."""
        nus = np.ascontiguousarray(nus, np.float64)
        nf = len(nus)
        S = E.shape[0]
        Er = torch.view_as_real(E.contiguous())
        Hr = torch.view_as_real(H.contiguous())
        out = torch.empty(nf * self.nrec * MT_RECORD, dtype=torch.float64, device=E.device)
        rc = _lib.lib().mtgpu_mt_response(
            self._h, nf, nus, np.ascontiguousarray(sys_x, np.int32),
            np.ascontiguousarray(sys_y, np.int32), S, C.c_void_p(Er.data_ptr()),
            C.c_void_p(Hr.data_ptr()), C.c_void_p(out.data_ptr()))
        _lib.check(rc, "mtgpu_mt_response")
        return out.view(nf, self.nrec, MT_RECORD)
