"""Gradients of driven Lindblad propagations: the hand-written discrete adjoint.

The forward map is the reference's driven propagation (``_lindblad_driven``,
``pyqed/oqs.py:1699-1806``): H(t) = H0 - sum_d E_d(t) mu_d frozen at t_{k+1}
for the four RK4 stages (``pyqed/phys.py:1051-1064``), collapse operators
L_k = sqrt(gamma_k) L^_k, observables o_k = Tr[O rho_k] after every step.
``DrivenBatch.forward`` runs it on the GPU (FP32 CTA kernel) keeping rho every
``checkpoint_every`` steps; ``DrivenBatch.backward`` calls the C ABI's
``lgb_plan_adjoint``, which recomputes each checkpoint segment and propagates
the costate backwards with the adjoint generator.  ``DrivenObservables`` wraps
both as a ``torch.autograd.Function`` with gradients for E(t) and gamma.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi as C
from .engine import Propagator, pack, to_dense

__all__ = ["DrivenBatch", "DrivenObservables"]


class DrivenBatch:
    """Instances b with H0[b], drive operators mu[b] = [mu_1..mu_D], collapse
    operator shapes Lhat[b] = [L^_1..L^_K], initial states and observables.
    The drive samples E (shape [D, nt]) are shared by all instances."""

    def __init__(self, H0, mu, Lhat, rho0, O, dt, nt, checkpoint_every=0, device=None):
        self.n_inst = len(H0)
        self.dims = np.array([to_dense(h).shape[0] for h in H0], dtype=np.int32)
        self.D = len(mu[0])
        self.K = len(Lhat[0])
        self.E_ops = len(O[0])
        self.nt, self.dt = int(nt), float(dt)
        self.H0 = pack([to_dense(h) for h in H0])
        self.mu = pack([to_dense(m) for ml in mu for m in ml])
        self.Lhat = [[to_dense(l) for l in ll] for ll in Lhat]
        self.O = pack([to_dense(o) for ol in O for o in ol])
        self.rho0_host = pack([to_dense(r) for r in rho0])
        self.prop = Propagator(self.dims, nt=nt, dt=dt, n_cops=self.K,
                               cops_kind="dense" if self.K else "none", n_eops=self.E_ops,
                               n_drive=self.D, obs_t0=False, precision="fp32",
                               schedule="cta", drive_shared=True, device=device,
                               flags=C.FLAG_ADJOINT, checkpoint_every=checkpoint_every)
        self.device = self.prop.device
        self.rho0 = self.prop.to_device(self.rho0_host)
        self._gamma = None
        self._drive = None

    def set_gamma(self, gamma):
        gamma = np.asarray(gamma, dtype=np.float64).reshape(self.n_inst, self.K)
        if self._gamma is not None and np.array_equal(gamma, self._gamma):
            return
        cops = pack([np.sqrt(gamma[b, k]) * self.Lhat[b][k]
                     for b in range(self.n_inst) for k in range(self.K)]) if self.K else None
        self.prop.set_operators(self.H0, cops, self.O, self.mu)
        self._gamma = gamma.copy()

    def forward(self, E, gamma):
        """Observables, shape (n_inst, nt, n_eops), complex128 (device tensor)."""
        self.set_gamma(gamma)
        E = torch.as_tensor(E, dtype=torch.float64).reshape(self.D, self.nt)
        self._drive = E.to(self.device).contiguous()
        out = self.prop.alloc_outputs(want_obs=True, want_rho=False)
        obs, _, _ = self.prop.propagate_device(self.rho0, self._drive, out)
        self.prop.check_errors()
        return obs.reshape(self.n_inst, self.nt, self.E_ops)

    def backward(self, obs_grad, want_h=False, want_rho0=False):
        """obs_grad: dJ/dRe(o) + i dJ/dIm(o), shape (n_inst, nt, n_eops).
        Returns dict(dE [D, nt] summed over instances, dE_inst, dgamma
        [n_inst, K], optionally dH0 / drho0 (lists of N x N))."""
        g = torch.as_tensor(obs_grad).to(self.device, torch.complex128).contiguous()
        z = lambda n: torch.zeros(int(n), dtype=torch.float64, device=self.device)  # noqa: E731
        dE = z(self.n_inst * self.D * self.nt)
        dscale = z(self.n_inst * self.K)
        off = self.prop.off
        dH = torch.zeros(int(off[-1]), dtype=torch.complex128, device=self.device) if want_h else None
        dr = torch.zeros(int(off[-1]), dtype=torch.complex128, device=self.device) if want_rho0 else None
        ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else None  # noqa: E731
        with torch.cuda.device(self.device):
            C.check(self.prop._lib.lgb_plan_adjoint(
                self.prop._plan, ptr(self.rho0), ptr(self._drive), ptr(g), ptr(dE), ptr(dscale),
                ptr(dH), ptr(dr), ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)),
                "lgb_plan_adjoint")
        self.prop.check_errors()
        dE_inst = dE.reshape(self.n_inst, self.D, self.nt)
        res = dict(dE=dE_inst.sum(0), dE_inst=dE_inst,
                   dgamma=(dscale.reshape(self.n_inst, self.K).cpu().numpy() / self._gamma)
                   if self.K else np.zeros((self.n_inst, 0)))
        if want_h:
            res["dH0"] = self.prop.unpack_rho(dH)
        if want_rho0:
            res["drho0"] = self.prop.unpack_rho(dr)
        return res


class DrivenObservables(torch.autograd.Function):
    """obs = DrivenObservables.apply(E, gamma, batch): E [D, nt] float64,
    gamma [n_inst, K] float64 -> observables [n_inst, nt, n_eops] complex128."""

    @staticmethod
    def forward(ctx, E, gamma, batch):
        ctx.batch = batch
        obs = batch.forward(E.detach(), gamma.detach().cpu().numpy())
        return obs.to(E.device)

    @staticmethod
    def backward(ctx, grad_obs):
        r = ctx.batch.backward(grad_obs)
        dE = r["dE"].to(grad_obs.device)
        dgam = torch.as_tensor(r["dgamma"], dtype=torch.float64, device=grad_obs.device)
        return dE, dgam, None
