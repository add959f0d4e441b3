"""CPU oracle for the Lindblad RK4 propagator -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain numpy complex128, the algorithm of the
reference's Lindblad master-equation path (binggu56/pyqed 0.1.3).  It is the
checker: only the test suite, the smoke check and the CPU-baseline leg of the
benchmark may import it.  The product path (``pyqed_gb300``) never calls it and
fails loudly when its CUDA library is missing.

Pinned against the reference: ``tests/golden/make_golden.py`` runs the
reference's own ``LindbladSolver.run``, ``_lindblad_driven``,
``_fast_lindblad`` and ``_correlation_2p_1t`` on seeded inputs and commits the
outputs as ``tests/golden/*.npz``; ``tests/test_oracle.py`` checks every
function below against those fixtures at 1e-12.

Reference anchors (paths inside the pyqed project):
* RHS   ``pyqed/oqs.py:697-715`` (``liouvillian``, ``lindbladian``):
  -i[H, rho] + sum_k (L rho L^dag - 1/2 {L^dag L, rho}).
* RK4   ``pyqed/phys.py:1051-1064`` (``rk4``): classic four-stage RK4,
  stage inputs rho + k1 dt/2, rho + k2 dt/2, rho + k3 dt.
* obs   ``pyqed/phys.py:1257-1264`` (``obs_dm``): Tr[O rho].
* static propagation ``pyqed/oqs.py:1596-1696`` (``_lindblad``): Nt+1
  observable rows (row 0 = rho0), Nt stored states excluding rho0.
* driven propagation ``pyqed/oqs.py:1699-1806`` (``_lindblad_driven``):
  H(t) = H0 - sum_i f_i(t) H_i evaluated once per step at t_{k+1} and held
  for all four stages; Nt observable rows, no t0 row.
* dense propagation ``pyqed/oqs.py:1492-1594`` (``_fast_lindblad``): final
  state only (the reference mutates its input; this restatement does not).
* two-point correlation ``pyqed/oqs.py:717-791`` (``_correlation_2p_1t``):
  rho <- B rho0, C_k = Tr[A rho(t_k)] for k = 1..Nt.
* three/four-operator correlations ``pyqed/oqs.py:1224-1243, 1298-1312``.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "rhs", "rk4_step", "obs_dm", "lindblad", "lindblad_driven", "fast_lindblad",
    "correlation_2op_1t", "correlation_3op_1t", "correlation_4op_1t",
    "rhs_diag", "propagate_diag_correlation", "liouvillian_superop",
]


def _dense(a):
    return a.toarray() if hasattr(a, "toarray") else np.asarray(a)


def rhs(rho, H, c_ops):
    """Lindblad right-hand side, ``pyqed/oqs.py:697-715``.

    -1j*(H rho - rho H) + sum_k [L rho L^dag - 0.5 (L^dag L rho + rho L^dag L)].
    """
    out = -1j * (H @ rho - rho @ H)
    for L in c_ops:
        Ld = L.conj().T
        LdL = Ld @ L
        out = out + (L @ (rho @ Ld) - 0.5 * (LdL @ rho + rho @ LdL))
    return out


def rk4_step(rho, dt, H, c_ops, f=rhs):
    """One classic RK4 step, ``pyqed/phys.py:1051-1064``."""
    dt2 = dt / 2.0
    k1 = f(rho, H, c_ops)
    k2 = f(rho + k1 * dt2, H, c_ops)
    k3 = f(rho + k2 * dt2, H, c_ops)
    k4 = f(rho + k3 * dt, H, c_ops)
    return rho + (k1 + 2 * k2 + 2 * k3 + k4) / 6.0 * dt


def obs_dm(rho, O):
    """Tr[O rho], ``pyqed/phys.py:1257-1264``."""
    return np.einsum("ij,ji->", O, rho)


def lindblad(H, rho0, c_ops, e_ops=None, Nt=1, dt=0.005, store_states=True):
    """Static propagation, ``pyqed/oqs.py:1596-1696``.

    Returns (observables (Nt+1, n_e) with row 0 at t0, list of Nt states).
    """
    H = _dense(H)
    c_ops = [_dense(c) for c in (c_ops or [])]
    e_ops = [_dense(e) for e in (e_ops or [])]
    rho = _dense(rho0).astype(complex).copy()
    obs = np.zeros((Nt + 1, len(e_ops)), dtype=complex)
    obs[0, :] = [obs_dm(rho, e) for e in e_ops]
    states = []
    for k in range(Nt):
        rho = rk4_step(rho, dt, H, c_ops)
        if store_states:
            states.append(rho.copy())
        obs[k + 1, :] = [obs_dm(rho, e) for e in e_ops]
    return obs, states


def lindblad_driven(H, rho0, c_ops=None, e_ops=None, Nt=1, dt=0.005, t0=0.0,
                    store_states=True):
    """Driven propagation, ``pyqed/oqs.py:1699-1806``.

    ``H = [H0, [H1, f1], [H2, f2], ...]`` with H(t) = H0 - sum_i f_i(t) H_i,
    evaluated at t_{k+1} = t0 + (k+1) dt and frozen for the four stages.
    Each f_i is a callable of t or an array of length Nt holding f_i(t_{k+1}).
    Returns (observables (Nt, n_e), list of Nt states).
    """
    H0 = _dense(H[0])
    terms = [(_dense(h), f) for h, f in H[1:]]
    c_ops = [_dense(c) for c in (c_ops or [])]
    e_ops = [_dense(e) for e in (e_ops or [])]
    rho = _dense(rho0).astype(complex).copy()
    obs = np.zeros((Nt, len(e_ops)), dtype=complex)
    states = []
    t = t0
    for k in range(Nt):
        t += dt
        Ht = H0.copy()
        for h, f in terms:
            ft = f(t) if callable(f) else f[k]
            Ht = Ht - ft * h
        rho = rk4_step(rho, dt, Ht, c_ops)
        if store_states:
            states.append(rho.copy())
        obs[k, :] = [obs_dm(rho, e) for e in e_ops]
    return obs, states


def fast_lindblad(H, rho0, c_ops, Nt=1, dt=0.005):
    """Dense propagation to the final state, ``pyqed/oqs.py:1492-1594``."""
    H = _dense(H)
    c_ops = [_dense(c) for c in (c_ops or [])]
    rho = _dense(rho0).astype(complex).copy()
    for _ in range(Nt):
        rho = rk4_step(rho, dt, H, c_ops)
    return rho


def correlation_2op_1t(H, rho0, a_op, b_op, c_ops, dt, Nt):
    """<A(t) B> by the quantum regression theorem, ``pyqed/oqs.py:717-791``.

    rho(0) = B rho0; returns C_k = Tr[A rho(t_k)], t_k = k dt, k = 1..Nt.
    """
    H = _dense(H)
    c_ops = [_dense(c) for c in (c_ops or [])]
    A = _dense(a_op)
    rho = _dense(b_op) @ _dense(rho0)
    cor = np.zeros(Nt, dtype=complex)
    for k in range(Nt):
        rho = rk4_step(rho, dt, H, c_ops)
        cor[k] = obs_dm(rho, A)
    return cor


def correlation_3op_1t(H, rho0, oplist, c_ops, dt, Nt):
    """<A B(t) C>, ``pyqed/oqs.py:1224-1243``: Nt+1 values including t = 0."""
    a, b, c = [_dense(o) for o in oplist]
    obs, _ = lindblad(H, c @ _dense(rho0) @ a, c_ops, [b], Nt=Nt, dt=dt,
                      store_states=False)
    return obs[:, 0]


def correlation_4op_1t(H, rho0, oplist, c_ops, dt, Nt):
    """<A B(t) C(t) D>, ``pyqed/oqs.py:1298-1312`` (the second definition)."""
    a, b, c, d = [_dense(o) for o in oplist]
    return correlation_3op_1t(H, rho0, [a, b @ c, d], c_ops, dt, Nt)


# --- diagonal collapse operators -------------------------------------------
# For L_k = diag(l_k) the reference's RHS (``pyqed/oqs.py:697-715``) is
# algebraically -i(H_eff rho - rho H_eff^dag) + D o rho with
# H_eff = H - (i/2) sum_k diag(|l_k|^2) and D_ij = sum_k l_k[i] conj(l_k[j]).
# ``rhs_diag`` evaluates it in that form; the tests check it against ``rhs``
# with the same operators given densely.

def rhs_diag(rho, H, c_diag):
    """RHS for collapse operators given by their diagonals (K x N array)."""
    c_diag = np.asarray(c_diag)
    if c_diag.size == 0:
        return -1j * (H @ rho - rho @ H)
    g = np.sum(np.abs(c_diag) ** 2, axis=0)
    Heff = H - 0.5j * np.diag(g)
    D = np.einsum("ki,kj->ij", c_diag, c_diag.conj())
    return -1j * (Heff @ rho - rho @ Heff.conj().T) + D * rho


def propagate_diag_correlation(H, mu, rho_g, c_diag, dt, Nt, return_rho=False):
    """C_k = Tr[mu rho(t_k)], rho(0) = mu rho_g, diagonal collapse operators.

    Same recurrence as ``correlation_2op_1t`` with A = B = mu.  With
    ``return_rho`` the final rho(t_Nt) is returned as well.
    """
    rho = mu @ rho_g
    cor = np.zeros(Nt, dtype=complex)
    for k in range(Nt):
        rho = rk4_step(rho, dt, H, c_diag, f=rhs_diag)
        cor[k] = obs_dm(rho, mu)
    return (cor, rho) if return_rho else cor


def liouvillian_superop(H, c_ops):
    """Row-major vectorised Liouvillian, ``pyqed/superoperator.py:29-57,200-251``.

    vec(rho)[i*N + j] = rho[i, j]; d vec(rho)/dt = L vec(rho).
    """
    H = _dense(H)
    N = H.shape[0]
    I = np.eye(N)
    L = -1j * (np.kron(H, I) - np.kron(I, H.T))
    for c in (c_ops or []):
        c = _dense(c)
        cdc = c.conj().T @ c
        L = L + np.kron(c, c.conj()) - 0.5 * (np.kron(cdc, I) + np.kron(I, cdc.T))
    return L
