"""Drop-in ``LindbladSolver`` for ``pyqed.oqs.LindbladSolver``
(``pyqed/oqs.py:1114-1330``), propagated by the CUDA library.

Same constructor, setters, ``run``/``evolve``, ``evolve_fast`` and
correlation entry points, the same ``Result`` fields and row conventions:

* static ``run`` (``_lindblad``, ``pyqed/oqs.py:1596-1696``): observables have
  Nt+1 rows, row 0 at t0; ``rholist`` holds the Nt states after each step.
* driven ``run`` with ``H = [H0, [H1, f1], ...]`` (``_lindblad_driven``,
  ``pyqed/oqs.py:1699-1806``): H(t) = H0 - sum_i f_i(t) H_i evaluated once
  per step at t_{k+1} = t0 + (k+1) dt and held for the four RK4 stages;
  Nt observable rows (no t0 row).
* ``run`` reads only its ``e_ops`` argument, not ``self.e_ops``
  (``pyqed/oqs.py:1186``), and the static path starts its clock at 0.

Extensions are keyword-only: ``precision`` ('fp64' default = the
reference's complex128; 'fp32', '3xtf32', '3xbf16'), ``schedule``,
``store_states``, ``rholist_format``, ``nout`` (keep every nout-th step),
``check`` (per-step FP64 trace/hermiticity check) and ``device``.  Inputs may be numpy,
scipy.sparse or torch (the reference's ``run`` accepts only scipy.sparse).
Collapse operators that are all diagonal are passed to the kernels as
diagonals (an exact rewrite of the same RHS).
"""
from __future__ import annotations

import numpy as np
from scipy.sparse import csr_matrix, identity, kron

from .engine import Propagator, diagonal_of, pack, to_dense
from .mol import Result

__all__ = ["LindbladSolver", "liouvillian"]


def liouvillian(H, c_ops):
    """Sparse row-major Liouvillian superoperator, as the reference's
    ``pyqed.superoperator.liouvillian`` (``pyqed/superoperator.py:29-57``):
    -i (H x I - I x H^T) + sum_c [c x c* - 1/2 (c^dag c x I + I x (c^dag c)^T)].
    """
    # the same operations in the same order as the reference (dense c^dag c,
    # each dissipator formed before it is added), so that L is bit-identical:
    # the eigenvector phases of the spectral solver depend on its last bits
    H = to_dense(H)
    N = H.shape[0]
    idm = identity(N)
    L = -1j * (kron(H, idm) - kron(idm, H.T))
    for c in (c_ops or []):
        c = to_dense(c)
        cdc = c.conjugate().transpose().dot(c)
        L = L + (kron(c, c.conj()) - 0.5 * (kron(cdc, idm) + kron(idm, cdc.T)))
    return csr_matrix(L)


def _cops_for_engine(c_ops):
    """-> (kind, n_cops, packed host array)"""
    c_ops = list(c_ops or [])
    if not c_ops:
        return "none", 0, None
    diags = [diagonal_of(c) for c in c_ops]
    if all(d is not None for d in diags):
        return "diag", len(c_ops), pack(diags)
    return "dense", len(c_ops), pack([to_dense(c) for c in c_ops])


def _eval_drive(terms, Nt, dt, t0):
    """Samples f_i(t_{k+1}); t accumulates as in ``pyqed/oqs.py:1790-1794``."""
    out = np.zeros((len(terms), Nt), dtype=np.float64)
    for i, (_, f) in enumerate(terms):
        if callable(f):
            t = t0
            for k in range(Nt):
                t += dt
                v = complex(f(t))
                if v.imag != 0.0:
                    raise ValueError("drive amplitude f(t) must be real")
                out[i, k] = v.real
        else:
            a = np.asarray(f, dtype=np.float64).ravel()
            if a.size != Nt:
                raise ValueError("drive samples must have length Nt")
            out[i] = a
    return out


class LindbladSolver:
    """Lindblad master-equation solver (``pyqed/oqs.py:1114-1330``)."""

    def __init__(self, H=None, c_ops=None, e_ops=None, *, precision="fp64", schedule="auto",
                 device=None):
        self.c_ops = c_ops
        self.e_ops = e_ops
        self.H = H
        self.precision = precision
        self.schedule = schedule
        self.device = device

    # -- setters (pyqed/oqs.py:1121-1139) ---------------------------------------
    def set_c_ops(self, c_ops):
        self.c_ops = c_ops

    def set_e_ops(self, e_ops):
        self.e_ops = e_ops

    def setH(self, H):
        self.H = H

    def configure(self, c_ops, e_ops):
        self.c_ops = c_ops
        self.e_ops = e_ops

    def liouvillian(self):
        return liouvillian(self.H, self.c_ops)

    def steady_state(self):
        """Not implemented in the reference either (``pyqed/oqs.py:1146-1147``)."""
        return None

    # -- core --------------------------------------------------------------------
    def _propagate(self, rho0, dt, Nt, e_ops, *, t0=0.0, obs_t0=True, store_states=False,
                   precision=None, H=None, store_every=1, check=None):
        H = self.H if H is None else H
        if isinstance(H, list):
            H0 = to_dense(H[0])
            terms = [(to_dense(h), f) for h, f in H[1:]]
        else:
            H0, terms = to_dense(H), []
        N = H0.shape[0]
        rho0 = to_dense(rho0)
        if rho0.shape != (N, N):
            raise ValueError("rho0 has shape %s, expected %s" % (rho0.shape, (N, N)))
        e_list = [to_dense(e) for e in (e_ops or [])]
        kind, K, cops = _cops_for_engine(self.c_ops)
        prop = Propagator([N], nt=Nt, dt=dt, n_cops=K, cops_kind=kind, n_eops=len(e_list),
                          n_drive=len(terms), obs_t0=obs_t0,
                          store_every=store_every if store_states else 0,
                          precision=precision or self.precision, schedule=self.schedule,
                          drive_shared=True, device=self.device)
        self.last_check = None
        try:
            if check:
                prop.set_check(check)
            prop.set_operators(H0, cops, pack(e_list) if e_list else None,
                               pack([h for h, _ in terms]) if terms else None)
            drive = None
            if terms:
                import torch
                drive = torch.from_numpy(_eval_drive(terms, Nt, dt, t0).ravel()).to(prop.device)
            out = prop.alloc_outputs(want_obs=True, want_rho=True, want_states=store_states)
            obs, rho, st = prop.propagate_device(prop.to_device(rho0), drive, out)
            flags = prop.check_errors()
            if check:
                tr, he = prop.check_stats()[0]
                self.last_check = dict(tolerance=float(check), trace_drift=float(tr),
                                       hermiticity=None if he < 0 else float(he),
                                       ok=bool(flags[0] == 0))
            nrows = Nt + int(obs_t0)
            obs_h = prop.unpack_obs(obs)[0] if obs is not None else np.zeros((nrows, 0), complex)
            rho_h = prop.unpack_rho(rho)[0]
            st_h = prop.unpack_states(st)[0] if st is not None else None
        finally:
            prop.close()
        return obs_h, rho_h, st_h

    @staticmethod
    def _as_list(states, fmt):
        if states is None:
            return []
        if fmt == "csr":
            return [csr_matrix(s) for s in states]
        return [s.copy() for s in states]

    def run(self, rho0, dt, Nt, t0=0., e_ops=None, return_result=True, *, precision=None,
            store_states=True, rholist_format="csr", nout=1, check=None):
        """Propagate Nt RK4 steps (``pyqed/oqs.py:1149-1187``).

        ``nout`` (keyword extension; the reference's ``Result`` carries it,
        ``pyqed/mol.py:98-114``): keep every nout-th step only.  The states
        after steps nout, 2 nout, ... go to ``rholist`` and the observables of
        those steps (plus t0 on the static path) to ``observables``, so that
        the rows match ``Result.times`` = t0 + arange(Nt // nout + 1) dt nout.

        ``check=tol`` (keyword extension) checks after every step, in FP64 on
        the GPU, that the trace and (for a Hermitian rho0) the hermiticity of
        rho stay within ``tol``; the result's ``check`` attribute holds the
        largest deviations.  The state is not renormalised.
        """
        nout = int(nout)
        if nout < 1:
            raise ValueError("nout must be >= 1")
        if isinstance(self.H, list):
            obs, rho, st = self._propagate(rho0, dt, Nt, e_ops, t0=t0, obs_t0=False,
                                           store_states=store_states and return_result,
                                           precision=precision, store_every=nout, check=check)
            if not return_result:
                # pyqed/oqs.py:1745-1780: observables to obs.dat, den_mat.dat
                # opened (and left empty), the final state returned
                fmt = "{} " * (obs.shape[1] + 1) + "\n"
                with open("obs.dat", "w") as f:
                    t = t0
                    for k in range(Nt):
                        t += dt
                        f.write(fmt.format(t, *obs[k]))
                open("den_mat.dat", "w").close()
                return csr_matrix(rho) if rholist_format == "csr" else rho
            result = Result(dt=dt, Nt=Nt, rho0=rho0, nout=nout)
            result.observables = obs[nout - 1::nout] if nout > 1 else obs
            result.rholist = self._as_list(st, rholist_format)
            if check:
                result.check = self.last_check
            return result
        obs, rho, st = self._propagate(rho0, dt, Nt, e_ops, obs_t0=True,
                                       store_states=store_states, precision=precision,
                                       store_every=nout, check=check)
        result = Result(dt=dt, Nt=Nt, rho0=rho0, nout=nout)
        result.observables = obs[::nout] if nout > 1 else obs
        result.rholist = self._as_list(st, rholist_format)
        if check:
            result.check = self.last_check
        return result

    evolve = run

    def evolve_fast(self, rho0, dt, Nt, t0=0., e_ops=None, return_result=True, fast=True, *,
                    precision=None, check=None):
        """Final state after Nt steps (``_fast_lindblad``, ``pyqed/oqs.py:1492-1594``).

        Like the reference, a writable complex ndarray ``rho0`` is overwritten
        with the final state.  Unlike it, ``e_ops=None`` is accepted.
        """
        _, rho, _ = self._propagate(rho0, dt, Nt, None, obs_t0=False, store_states=False,
                                    precision=precision, check=check)
        if isinstance(rho0, np.ndarray) and np.iscomplexobj(rho0) and rho0.flags.writeable:
            rho0[...] = rho
            return rho0
        return rho

    # -- correlation functions (pyqed/oqs.py:1193-1330) ---------------------------
    def correlation_2op_1t(self, rho0, a_op, b_op, dt, Nt, output="cor.dat", *, precision=None):
        """<A(t)B> = Tr[A e^{Lt}(B rho0)], t = dt..Nt dt (``pyqed/oqs.py:717-791``).

        Writes ``output`` with one "t C(t)" line per step, as the reference."""
        H = self.H[0] if isinstance(self.H, list) else self.H
        rho = to_dense(b_op) @ to_dense(rho0)
        obs, _, _ = self._propagate(rho, dt, Nt, [a_op], obs_t0=False, precision=precision,
                                    H=H)
        cor = obs[:, 0].copy()
        if output is not None:
            with open(output, "w") as f:
                t = 0.0
                for k in range(Nt):
                    t += dt
                    f.write("{} {} \n".format(t, cor[k]))
        return cor

    def correlation_3op_1t(self, rho0, oplist, dt=0.005, Nt=1, *, precision=None):
        """<A B(t) C>, Nt+1 values including t = 0 (``pyqed/oqs.py:1224-1243``)."""
        a_op, b_op, c_op = [to_dense(o) for o in oplist]
        obs, _, _ = self._propagate(c_op @ to_dense(rho0) @ a_op, dt, Nt, [b_op], obs_t0=True,
                                    precision=precision)
        return obs[:, 0].copy()

    def correlation_4op_1t(self, rho0, ops, dt, nt, *, precision=None):
        """<A B(t) C(t) D> (``pyqed/oqs.py:1298-1312``, the definition that wins)."""
        if len(ops) != 4:
            raise ValueError('Number of operators is not 4.')
        a, b, c, d = [to_dense(o) for o in ops]
        return self.correlation_3op_1t(rho0, [a, b @ c, d], dt, nt, precision=precision)

    def correlation_3op_2t(self, rho0, ops, dt, Nt, Ntau, *, precision=None):
        """<A(t) B(t+tau) C(t)>, shape (Nt, Ntau+1).

        The reference (``pyqed/oqs.py:1265-1296``) propagates each stored
        rho(t_k), k = 1..Nt, for Ntau steps from C rho(t_k) A with e_ops [B],
        then fails to fit the Ntau+1 values into an Ntau-wide row.  Here the
        intended matrix is returned with its tau = 0 column, and the Nt
        tau-propagations run as one batch on the GPU.
        """
        from .batch import propagate_batch
        a_op, b_op, c_op = [to_dense(o) for o in ops]
        _, _, states = self._propagate(rho0, dt, Nt, None, obs_t0=False, store_states=True,
                                       precision=precision)
        H = self.H[0] if isinstance(self.H, list) else self.H
        seeds = [c_op @ s @ a_op for s in states]
        res = propagate_batch([H] * Nt, [self.c_ops] * Nt, seeds, dt, Ntau, e_ops=[[b_op]] * Nt,
                              obs_t0=True, precision=precision or self.precision,
                              device=self.device)
        return res["observables"][:, :, 0]

    def correlation_4op_2t(self, rho0, ops, dt, nt, ntau, *, precision=None):
        """<A(t) B(t+tau) C(t+tau) D(t)> (``pyqed/oqs.py:1314-1330``)."""
        if len(ops) != 4:
            raise ValueError('Number of operators is not 4.')
        a, b, c, d = [to_dense(o) for o in ops]
        return self.correlation_3op_2t(rho0, [a, b @ c, d], dt, nt, ntau, precision=precision)
