"""Drop-in mirror of the reference's HEOM solver on the GPU.

``HEOMSolver`` follows ``pyqed.oqs.HEOMSolver`` (``pyqed/oqs.py:1332-1431``):
the constructor ``(H, c_ops, e_ops)`` with ``c_ops[0]`` the system-bath
operator, the setters, ``run(rho0, dt, nt, temperature, cutoff,
reorganization, nado)`` returning the observables Tr[e rho] after every step
as an (n_e, nt) complex array (``_heom``, ``pyqed/oqs.py:1808-1875``), and
``propagator(dt, nt, temperature, cutoff, reorganization, nado)`` returning
the (nado, N^2, N^2) Liouville-space propagators (``_heom_propagator``,
``pyqed/oqs.py:1877-1935``).  Both print the bath parameters as the reference
does.  ``correlation_2op_1t`` is the Lindblad correlation of the same
operators, as in the reference (``pyqed/oqs.py:1372-1401``);
``correlation_3op_2t`` returns the intended (Nt, Ntau) matrix where the
reference raises on a shape mismatch (``pyqed/oqs.py:1404-1431``).

The hierarchy is swept on the GPU (``lgb_heom_*``, one thread group per
system, the levels resident in shared memory).  ``heom_batch`` runs many
systems, each with its own bath, in one launch.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi as C
from .engine import _device, to_dense

__all__ = ["HEOMSolver", "heom_batch", "bath_run", "bath_propagator"]

AU2K = 315775.13  # pyqed/units.py:6
_PREC = {"fp64": C.PREC["fp64"], "fp32": C.PREC["fp32"]}


def bath_run(temperature, cutoff, reorganization):
    """(gamma, D0) of ``_heom``: gamma = cutoff, T = temperature,
    D0 = lambda gamma (coth(gamma / 2T) - i) (``pyqed/oqs.py:1829-1841``)."""
    gamma = float(cutoff)
    D0 = reorganization * gamma * (1.0 / np.tanh(gamma / (2.0 * temperature)) - 1j)
    return gamma, complex(D0)


def bath_propagator(temperature, cutoff, reorganization):
    """(gamma, D0) of ``_heom_propagator``: T = temperature / au2k,
    D0 = pi lambda T (``pyqed/oqs.py:1891-1905``)."""
    T = temperature / AU2K
    return float(cutoff), complex(np.pi * reorganization * T, 0.0)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else None


class _Plan:
    def __init__(self, dims, nt, dt, nado, n_eops, precision, flags, device):
        self.dev = _device(device)
        self.dims = np.asarray(dims, dtype=np.int32)
        self.L = C.lib()
        if precision not in _PREC:
            raise ValueError("precision must be 'fp64' or 'fp32' for HEOM")
        prob = C.HeomProblem(n_inst=len(dims), n_eops=n_eops, nt=nt, nado=nado, precision=_PREC[precision],
                             flags=flags, dt=dt)
        self.plan = ctypes.c_void_p()
        with torch.cuda.device(self.dev):
            C.check(self.L.lgb_heom_create(ctypes.byref(self.plan), ctypes.byref(prob),
                                           (ctypes.c_int32 * len(dims))(*self.dims.tolist())), "lgb_heom_create")
        self.nt, self.nado, self.n_eops = nt, nado, n_eops
        self.voff = np.concatenate([[0], np.cumsum(self.dims.astype(np.int64) ** 2)])

    def stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def layout(self):
        info = (ctypes.c_int32 * 4)()
        C.check(self.L.lgb_heom_layout(self.plan, info), "lgb_heom_layout")
        return dict(threads_per_system=info[0], systems_per_cta=info[1], on_chip=bool(info[2]),
                    smem_bytes=info[3])

    def close(self):
        if self.plan.value:
            self.L.lgb_heom_destroy(self.plan)
            self.plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, H, sz, bath, Ot):
        with torch.cuda.device(self.dev):
            C.check(self.L.lgb_heom_set(self.plan, _ptr(H), _ptr(sz), _ptr(bath), _ptr(Ot), self.stream()),
                    "lgb_heom_set")

    def propagate(self, r0, want_ado=False, out=None):
        n = len(self.dims)
        z = lambda k: torch.empty(int(k), dtype=torch.complex128, device=self.dev)  # noqa: E731
        if out is None:
            out = dict(obs=z(n * self.n_eops * self.nt) if self.n_eops and self.nt else None,
                       rho=z(self.voff[-1]), ado=z(self.nado * self.voff[-1]) if want_ado else None)
        with torch.cuda.device(self.dev):
            C.check(self.L.lgb_heom_propagate(self.plan, _ptr(r0), _ptr(out["obs"]), _ptr(out["rho"]),
                                              _ptr(out["ado"]), self.stream()), "lgb_heom_propagate")
        return out

    def check_errors(self):
        n = len(self.dims)
        flags = (ctypes.c_int32 * n)()
        C.check(self.L.lgb_heom_errors(self.plan, flags), "lgb_heom_errors")
        bad = [i for i in range(n) if flags[i]]
        if bad:
            raise C.LindbladError(int(flags[bad[0]]), "system %d" % bad[0])


def _pack(mats):
    return np.concatenate([np.ascontiguousarray(m, dtype=np.complex128).ravel() for m in mats]) if mats \
        else np.zeros(0, complex)


def heom_batch(H, sz, rho0, e_ops=None, *, nado, dt, nt, temperature=None, cutoff=None, reorganization=None,
               bath=None, precision="fp32", return_ado=False, flags=0, sz_kind="auto", device=None,
               _plan_out=None):
    """Many HEOM systems in one launch.

    H, sz, rho0: per-system lists of N x N matrices (N may differ); e_ops:
    per-system lists of observables (the same count for every system).  The
    bath of system b is ``bath[b] = (gamma, D0)``, or is formed from
    ``temperature``/``cutoff``/``reorganization`` (scalars or per-system
    arrays) by ``bath_run``.  ``sz_kind``: 'auto' takes the O(N^2) path when
    every sz is diagonal, 'dense' or 'diag' force one.  Returns
    dict(observables (n, n_e, nt) complex128, rho list of the final X_0, ado
    list of (nado, N, N) or None, layout)."""
    n = len(H)
    Hs = [to_dense(h) for h in H]
    Ss = [to_dense(s) for s in sz]
    dims = [h.shape[0] for h in Hs]
    e_ops = [[] for _ in range(n)] if e_ops is None else e_ops
    E = len(e_ops[0]) if n else 0
    if any(len(e) != E for e in e_ops):
        raise ValueError("every system needs the same number of e_ops")
    if bath is None:
        T, cu, lam = (np.broadcast_to(np.asarray(v, dtype=float), (n,)) for v in
                      (temperature, cutoff, reorganization))
        bath = [bath_run(T[b], cu[b], lam[b]) for b in range(n)]
    coef = np.array([[g, d.real, d.imag] for g, d in bath], dtype=np.float64).ravel()
    if sz_kind not in ("auto", "dense", "diag"):
        raise ValueError("sz_kind must be 'auto', 'dense' or 'diag'")
    diag = all(not np.any(s - np.diag(np.diag(s))) for s in Ss) if sz_kind == "auto" else sz_kind == "diag"
    if diag:
        flags |= C.HEOM_DIAG_SZ
    plan = _Plan(dims, nt, dt, nado, E, precision, flags, device)
    try:
        dev = plan.dev
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        Ot = _pack([to_dense(e).T for es in e_ops for e in es])
        plan.set(t(_pack(Hs)), t(_pack(Ss)), t(coef), t(Ot))
        out = plan.propagate(t(_pack([to_dense(r).astype(complex) for r in rho0])), want_ado=return_ado)
        layout = plan.layout()
        if _plan_out is not None:
            _plan_out.append(plan)
        else:
            plan.check_errors()
    finally:
        if _plan_out is None:
            plan.close()
    layout["sz"] = "diag" if diag else "dense"
    res = dict(observables=None, rho=[], ado=None, layout=layout)
    res["observables"] = out["obs"].cpu().numpy().reshape(n, E, nt) if out["obs"] is not None \
        else np.zeros((n, E, nt), complex)
    rh = out["rho"].cpu().numpy()
    res["rho"] = [rh[plan.voff[b]:plan.voff[b + 1]].reshape(dims[b], dims[b]) for b in range(n)]
    if return_ado:
        ah = out["ado"].cpu().numpy()
        res["ado"] = [ah[nado * plan.voff[b]:nado * plan.voff[b + 1]].reshape(nado, dims[b], dims[b])
                      for b in range(n)]
    return res


class HEOMSolver:
    """``pyqed.oqs.HEOMSolver`` on the GPU (``pyqed/oqs.py:1332-1431``)."""

    def __init__(self, H=None, c_ops=None, e_ops=None):
        self.c_ops = c_ops
        self.e_ops = e_ops
        self.H = H

    def set_c_ops(self, c_ops):
        self.c_ops = c_ops

    def set_e_ops(self, e_ops):
        """set observable operators"""
        self.e_ops = e_ops

    def setH(self, H):
        self.H = H

    def configure(self, c_ops, e_ops):
        self.c_ops = c_ops
        self.e_ops = e_ops

    def run(self, rho0, dt, nt, temperature, cutoff, reorganization, nado, *, precision="fp64", verbose=True):
        """``_heom``: the observables Tr[e rho(t_k)], k = 1..nt, as (n_e, nt)."""
        gamma, D0 = bath_run(temperature, cutoff, reorganization)
        if verbose:
            T = temperature
            print('Temperature of the environment = {}'.format(T))
            print('Cutoff gamma/(kT) = {}'.format(gamma / T))
            if gamma / T > 0.8:
                print('WARNING: High-Temperature Approximation may fail.')
            print('Reorganization energy = {}'.format(reorganization))
            print('Amplitude of the fluctuations = {}'.format(D0))
        e_ops = list(self.e_ops) if self.e_ops is not None else []
        res = heom_batch([self.H], [self.c_ops[0]], [rho0], [e_ops], nado=nado, dt=dt, nt=nt,
                         bath=[(gamma, D0)], precision=precision)
        return res["observables"][0]

    def propagator(self, dt, nt, temperature, cutoff, reorganization, nado, *, precision="fp64", verbose=True):
        """``_heom_propagator``: u (nado, N^2, N^2) with u[0](0) = 1, i.e.
        the sweep applied to every basis matrix (row-major vec), level 0
        advanced twice per step as in the reference."""
        gamma, D0 = bath_propagator(temperature, cutoff, reorganization)
        if verbose:
            T = temperature / AU2K
            print('Temperature of the environment = {}'.format(T))
            print('High-Temperature check gamma/(kT) = {}'.format(gamma / T))
            if gamma / T > 0.8:
                print('WARNING: High-Temperature Approximation may fail.')
            print('Reorganization energy = {}'.format(reorganization))
            print('Amplitude of the fluctuations = {}'.format(D0.real))
        H = to_dense(self.H)
        sz = to_dense(self.c_ops[0])
        N = H.shape[0]
        basis = []
        for c in range(N * N):
            e = np.zeros((N, N), complex)
            e.flat[c] = 1.0
            basis.append(e)
        res = heom_batch([H] * (N * N), [sz] * (N * N), basis, None, nado=nado, dt=dt, nt=nt,
                         bath=[(gamma, D0)] * (N * N), precision=precision, return_ado=True,
                         flags=C.HEOM_DOUBLE_FIRST)
        ado = np.stack(res["ado"])  # (N^2 columns, nado, N, N)
        return np.ascontiguousarray(ado.reshape(N * N, nado, N * N).transpose(1, 2, 0))

    def correlation_2op_1t(self, rho0, a_op, b_op, dt, Nt, output='cor.dat'):
        """The Lindblad two-point correlation <A(t)B> with these c_ops, as the
        reference (``_correlation_2p_1t``)."""
        from .oqs import LindbladSolver
        return LindbladSolver(self.H, self.c_ops).correlation_2op_1t(rho0, a_op, b_op, dt, Nt, output=output)

    def correlation_3op_2t(self, rho0, ops, dt, Nt, Ntau):
        """<A(t) B(t+tau) C(t)> from the Lindblad path, the (Nt, Ntau+1) matrix
        of ``LindbladSolver.correlation_3op_2t``; the reference raises here."""
        from .oqs import LindbladSolver
        return LindbladSolver(self.H, self.c_ops).correlation_3op_2t(rho0, ops, dt, Nt, Ntau)
