"""Drop-in mirror of the reference's eigen-decomposition Lindblad solver.

``Lindblad_solver`` follows ``pyqed.superoperator.Lindblad_solver``
(``pyqed/superoperator.py:455-770``): the Liouvillian L (row-major vec) is
diagonalised once, ``L r_n = lambda_n r_n``, ``l_n^dag L = lambda_n l_n^dag``,
and every result is a sum over the modes n.

* ``eigenstates()`` runs the same dense LAPACK eigensolver as the reference
  (``scipy.linalg.eig`` with left and right vectors) on the host and keeps
  the reference's normalisation ``norm_n = Re(l_n^dag r_n)``.  That real part
  drops the imaginary part of ``l_n^dag r_n``, which is not zero in general,
  so the reference's correlations carry an error that depends on the
  eigenvector phases (about 2e-2 on the 6-level Jaynes-Cummings system).
  ``eigenstates(complex_norm=True)`` uses ``l_n^dag r_n`` itself, and the
  sums are then exact.
* The mode sums run on the GPU (``lgb_spectral_sum``: exp(lambda t) at
  every time point, -1/(lambda + i w) at every frequency) and the two-time
  correlation is two complex128 GEMMs (``lgb_spectral_2t``).  Mode weights
  are formed from the eigenvectors on the device (torch complex128 algebra).

Deviations, documented: ``evolve`` returns the intended ``Result`` (the
reference's ``Result(times=tlist)`` raises a TypeError); ``eigenstates(k)``
with a truncated mode count raises NotImplementedError (the reference's
raises a NameError); the correlation methods diagonalise L on first use
instead of requiring an explicit ``eigenstates()`` call.
``correlation_3op_2t`` returns the reference's (len(taulist), len(tlist))
matrix.
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.linalg
import torch

from . import _capi as C
from .engine import to_dense
from .mol import Result
from .oqs import liouvillian

__all__ = ["Lindblad_solver"]


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Lindblad_solver:
    """``pyqed.superoperator.Lindblad_solver`` with the mode sums on the GPU."""

    def __init__(self, H, c_ops=None, *, device=None):
        self.H = H
        self.c_ops = c_ops
        self.L = None
        self.dim = H.shape[-1] ** 2
        self.idv = np.identity(H.shape[-1]).flatten()
        self.left_eigvecs = None
        self.right_eigvecs = None
        self.eigvals = None
        self.norm = None
        self.device = torch.device(device if device is not None else "cuda")
        self._dev = None  # device copies of (eigvals, right, left^dag / norm)

    def liouvillian(self):
        self.L = liouvillian(self.H, self.c_ops)
        return self.L

    def eigenstates(self, k=None, *, complex_norm=False):
        """(eigvals, right eigenvectors, left eigenvectors) of L, all modes."""
        if k is not None:
            raise NotImplementedError("a truncated mode set (k) is not supported; the reference raises here too")
        L = self.L if self.L is not None else self.liouvillian()
        w, vl, vr = scipy.linalg.eig(L.toarray(), left=True, right=True)
        nrm = np.diagonal(vl.conj().T @ vr)
        self.eigvals, self.left_eigvecs, self.right_eigvecs = w, vl, vr
        self.norm = nrm if complex_norm else nrm.real
        self._dev = None
        return w, vr, vl

    # ---- device side -----------------------------------------------------
    def _modes(self):
        if self.eigvals is None:
            self.eigenstates()
        if self._dev is None:
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).to(self.device)  # noqa: E731
            # rows of P = l_n^dag / norm_n: the expansion coefficient of v is (P v)_n
            P = t(self.left_eigvecs.conj().T) / t(self.norm)[:, None]
            self._dev = (t(self.eigvals), t(self.right_eigvecs), P)
        return self._dev

    def _trace_left(self, a, U1):
        """Tr[a U_n] for every mode (the reference's vdot(idv, left(a) U1[:, n]))."""
        N = int(round(np.sqrt(U1.shape[0])))
        A = torch.from_numpy(np.ascontiguousarray(to_dense(a), dtype=np.complex128)).to(self.device)
        return torch.einsum("ij,jin->n", A, U1.reshape(N, N, -1))

    def _vec(self, m):
        return torch.from_numpy(np.ascontiguousarray(to_dense(m), dtype=np.complex128).ravel()).to(self.device)

    def _sum(self, W, x, kind):
        """out[p][o] = sum_n W[o][n] f(lambda_n, x_p) on the GPU."""
        lam = self._modes()[0]
        xs = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=self.device)
        L = C.lib()
        parts = []
        for o0 in range(0, W.shape[0], 16):  # at most 16 sums per call
            Wc = W[o0:o0 + 16].contiguous()
            n_out, k = Wc.shape
            out = torch.empty((xs.numel(), n_out), dtype=torch.complex128, device=self.device)
            with torch.cuda.device(self.device):
                st = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
                C.check(L.lgb_spectral_sum(k, n_out, xs.numel(), kind, _dptr(lam), _dptr(Wc), _dptr(xs),
                                           _dptr(out), st), "lgb_spectral_sum")
            parts.append(out)
        return torch.cat(parts, dim=1).cpu().numpy()

    # ---- the reference's methods -------------------------------------------
    def evolve(self, rho0, tlist, e_ops):
        """Observables Tr[e rho(t)] at every t of ``tlist``: Result with
        ``times = tlist`` and ``observables`` (len(tlist), len(e_ops))."""
        lam, U1, P = self._modes()
        tlist = np.asarray(tlist, dtype=np.float64)
        coeff = P @ self._vec(rho0)
        W = torch.stack([self._trace_left(e, U1) * coeff for e in e_ops]) if e_ops else None
        result = Result(dt=(tlist[1] - tlist[0]) if tlist.size > 1 else 0.0, Nt=max(tlist.size - 1, 0))
        result.times = tlist
        result.observables = self._sum(W, tlist, 0) if W is not None else np.zeros((tlist.size, 0), complex)
        return result

    def _coeff_2op(self, rho0, a, b):
        lam, U1, P = self._modes()
        return self._trace_left(a, U1) * (P @ self._vec(to_dense(b) @ to_dense(rho0)))

    def _coeff_3op(self, rho0, a, b, c):
        lam, U1, P = self._modes()
        return self._trace_left(b, U1) * (P @ self._vec(to_dense(c) @ to_dense(rho0) @ to_dense(a)))

    def correlation_2op_1t(self, rho0, ops, tlist):
        """<A(t) B> = sum_n exp(lambda_n t) Tr[A r_n] (l_n^dag vec(B rho0)) / norm_n."""
        a, b = ops
        return self._sum(self._coeff_2op(rho0, a, b)[None, :], tlist, 0)[:, 0]

    def correlation_2op_1w(self, rho0, ops, w):
        """S(w) = sum_n -coeff_n / (lambda_n + i w)."""
        a, b = ops
        return self._sum(self._coeff_2op(rho0, a, b)[None, :], w, 1)[:, 0]

    def correlation_3op_1t(self, rho0, ops, t):
        """<A B(t) C> = sum_n exp(lambda_n t) Tr[B r_n] (l_n^dag vec(C rho0 A)) / norm_n."""
        a, b, c = ops
        return self._sum(self._coeff_3op(rho0, a, b, c)[None, :], t, 0)[:, 0]

    def correlation_3op_1w(self, rho0, ops, w):
        a, b, c = ops
        return self._sum(self._coeff_3op(rho0, a, b, c)[None, :], w, 1)[:, 0]

    def correlation_3op_2t(self, rho0, ops, tlist, taulist, k=None):
        """<A(t) B(t+tau) C(t)>, the (len(taulist), len(tlist)) matrix
        E(tau) coeff E(t) of the reference."""
        if k is not None and k != self.dim:
            raise NotImplementedError("a truncated mode set (k) is not supported")
        a, b, c = (torch.from_numpy(np.ascontiguousarray(to_dense(o), dtype=np.complex128)).to(self.device)
                   for o in ops)
        lam, U1, P = self._modes()
        N = a.shape[0]
        U = U1.T.reshape(-1, N, N)                            # U[n] = r_n as a matrix
        M = (c @ U @ a).reshape(U.shape[0], -1).T             # columns vec(C r_n A)
        coeff = self._trace_left(ops[1], U1)[:, None] * (P @ M) * (P @ self._vec(rho0))[None, :]
        coeff = coeff.contiguous()
        tl = torch.as_tensor(np.ascontiguousarray(tlist, dtype=np.float64), device=self.device)
        ta = torch.as_tensor(np.ascontiguousarray(taulist, dtype=np.float64), device=self.device)
        cor = torch.empty((ta.numel(), tl.numel()), dtype=torch.complex128, device=self.device)
        L = C.lib()
        with torch.cuda.device(self.device):
            st = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            C.check(L.lgb_spectral_2t(lam.numel(), ta.numel(), tl.numel(), _dptr(lam), _dptr(coeff), _dptr(ta),
                                      _dptr(tl), _dptr(cor), st), "lgb_spectral_2t")
        return cor.cpu().numpy()

    def correlation_4op_2t(self, rho0, ops, tlist, taulist, k=None):
        """<A(t) B(t+tau) C(t+tau) D(t)> as 3op_2t with [A, B C, D]."""
        if len(ops) != 4:
            raise ValueError('Number of operators is not 4.')
        a, b, c, d = ops
        return self.correlation_3op_2t(rho0, [a, to_dense(b) @ to_dense(c), d], tlist, taulist, k=k)
