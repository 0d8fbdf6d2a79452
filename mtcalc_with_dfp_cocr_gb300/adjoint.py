"""Impedance misfit and its adjoint gradient with respect to per-cell
log-conductivity, on the GPU (over libmtgpu).

    problem = ImpedanceProblem(mesh, freqs, receivers, z_obs)
    J, state = problem.misfit(log_sigma)           # forward: assembly, solve,
                                                   # receivers, impedances
    grad = problem.gradient(state)                 # adjoint solve + fused
                                                   # per-cell reduction
    ImpedanceMisfit.apply(log_sigma_tensor, problem)   # the same behind
                                                       # torch.autograd

J = sum over frequencies f and receivers r of sum_{i,j in x,y}
|Z_ij - Zobs_ij|^2; log_sigma = ln(sigma) of every cell (air cells
included).  Every frequency is solved for both polarisations; the adjoint
systems reuse the forward matrices (A is complex symmetric).

solver="batched" runs every solve through the batched double-float survey
solver; solver="fp64" solves each system with the FP64 COCR (the FP64 GPU
reference gradient).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, normal1d
from .assembly import Assembly
from .receivers import Receivers
from .survey import Survey


@dataclass
class State:
    assembly: Assembly
    receivers: Receivers
    u: torch.Tensor          # (S, 2 nb) forward solutions
    E: torch.Tensor
    H: torch.Tensor
    src: torch.Tensor        # (S, 2 nb) adjoint right-hand sides
    J: float
    response: torch.Tensor   # (nf, nrec, MT_RECORD)


class ImpedanceProblem:
    def __init__(self, mesh, freqs, receivers, z_obs=None, solver="batched", eps=1e-8,
                 maxiter=20000, device="cuda"):
        self.mesh = mesh
        self.freqs = np.asarray(freqs, np.float64)
        self.points = np.asarray(receivers, np.float64).reshape(-1, 3)
        self.solver = solver
        self.eps = eps
        self.maxiter = maxiter
        self.device = device
        nf = len(self.freqs)
        self.nus = np.repeat(self.freqs, 2)                       # system 2f: X, 2f+1: Y
        self.alfas = np.tile(np.array([1, 0], np.int32), nf)
        self.sys_x = np.arange(0, 2 * nf, 2, dtype=np.int32)
        self.sys_y = self.sys_x + 1
        tops = [l.top for l in mesh.layers]
        sig = [l.sigma for l in mesh.layers]
        tabs = [normal1d.solve_1d(f, tops, sig) for f in self.freqs]
        self.z1d = tabs[0][0]
        for t in tabs:
            if len(t[0]) != len(self.z1d) or not np.array_equal(t[0], self.z1d):
                raise ValueError("the 1-D tables of all frequencies must share z")
        self.usin = np.repeat(np.stack([t[1] for t in tabs]), 2, axis=0)
        self.ucos = np.repeat(np.stack([t[2] for t in tabs]), 2, axis=0)
        self.z_obs = None
        if z_obs is not None:
            self.set_observed(z_obs)

    @property
    def S(self):
        return len(self.nus)

    def set_observed(self, z_obs):
        """z_obs: (nf, nrec, 4) complex (Zxx, Zxy, Zyx, Zyy)."""
        z = torch.as_tensor(np.asarray(z_obs, np.complex128)).reshape(len(self.freqs), -1, 4)
        self.z_obs = torch.view_as_real(z).contiguous().to(self.device)

    # ------------------------------------------------------------ solves
    def _solve(self, A, b):
        x = torch.zeros_like(b)
        if self.solver == "batched":
            code, st = Survey(A, self.nus).solve(b, x, eps=self.eps, maxiter=self.maxiter,
                                                 verify=True)
            if code != 0:
                raise RuntimeError(f"batched solve failed: code {code}, {st}")
        elif self.solver == "fp64":
            for k, nu in enumerate(self.nus):
                ctx = A.cocr(nu)
                rc, st = ctx.solve(b[k], x[k], eps=self.eps, maxiter=self.maxiter,
                                   stop_on_true_residual=True)
                ctx.close()
                # pushed below its stagnation level the COCR recurrence can
                # break down ((a, w) = 0); the iterate is then as good as
                # its true residual says
                if rc != 0 and not (rc == -2 and st.true_residual_rel < 10 * self.eps):
                    raise RuntimeError(f"FP64 solve of system {k} failed: code {rc}, "
                                       f"true residual {st.true_residual_rel:.3e}")
        else:
            raise ValueError(f"unknown solver {self.solver!r}")
        return x

    def forward(self, log_sigma):
        """Impedance responses (nf, nrec, MT_RECORD) and the state."""
        sigma = np.exp(np.asarray(log_sigma, np.float64).reshape(self.mesh.kpar))
        A = Assembly(self.mesh, cell_sigma=sigma)
        b = torch.empty(self.S, 2 * self.mesh.nb, dtype=torch.float64, device=self.device)
        A.rhs(self.nus, self.alfas, self.z1d, self.usin, self.ucos, b)
        u = self._solve(A, b)
        R = Receivers(A, self.points)
        E, H, _ = R.fields(u, self.nus, self.alfas, self.z1d, self.usin, self.ucos)
        resp = R.mt_response(self.freqs, self.sys_x, self.sys_y, E, H)
        return resp, State(A, R, u, E, H, None, float("nan"), resp)

    def misfit(self, log_sigma):
        """J and the state that gradient() needs."""
        if self.z_obs is None:
            raise ValueError("no observed impedances")
        resp, st = self.forward(log_sigma)
        src = torch.empty_like(st.u)
        Er, Hr = torch.view_as_real(st.E.contiguous()), torch.view_as_real(st.H.contiguous())
        J = C.c_double()
        rc = _lib.lib().mtgpu_adjoint_source(
            st.receivers._h, len(self.freqs), self.freqs, self.sys_x, self.sys_y, self.S,
            C.c_void_p(Er.data_ptr()), C.c_void_p(Hr.data_ptr()),
            C.c_void_p(self.z_obs.data_ptr()), C.c_void_p(src.data_ptr()), C.byref(J))
        _lib.check(rc, "mtgpu_adjoint_source")
        st.src = src
        st.J = J.value
        return J.value, st

    def gradient(self, st: State):
        """dJ/d ln(sigma) of every cell: (kpar,) float64 CUDA tensor."""
        lam = self._solve(st.assembly, st.src)
        grad = torch.empty(self.mesh.kpar, dtype=torch.float64, device=self.device)
        rc = _lib.lib().mtgpu_adjoint_gradient(
            st.assembly._h, self.S, self.nus, self.alfas, len(self.z1d), self.z1d,
            np.ascontiguousarray(self.usin), np.ascontiguousarray(self.ucos),
            C.c_void_p(st.u.data_ptr()), C.c_void_p(lam.data_ptr()),
            C.c_void_p(grad.data_ptr()))
        _lib.check(rc, "mtgpu_adjoint_gradient")
        return grad


def impedances(response):
    """Complex (nf, nrec, 4) impedances from a response tensor."""
    z = response[..., :8].contiguous().view(*response.shape[:-1], 4, 2)
    return torch.view_as_complex(z)


class ImpedanceMisfit(torch.autograd.Function):
    """J(log_sigma) with the adjoint gradient as its backward."""

    @staticmethod
    def forward(ctx, log_sigma, problem):
        J, st = problem.misfit(log_sigma.detach().cpu().numpy())
        ctx.problem = problem
        ctx.state = st
        return torch.tensor(J, dtype=torch.float64, device=log_sigma.device)

    @staticmethod
    def backward(ctx, gJ):
        grad = ctx.problem.gradient(ctx.state).to(gJ.device)
        ctx.state = None
        return gJ * grad.to(gJ.dtype), None

