"""Test infrastructure: numpy complex128 restatement of the reference's HEOM
solver, the checker for ``pyqed_gb300.heom``.  Only ``tests/`` may use it.

Follows binggu56/pyqed 0.1.3:
  * ``_heom``            ``pyqed/oqs.py:1808-1875``: one exponential bath mode
    (leading Matsubara term, D0 = lambda gamma (coth(gamma / 2T) - i)), a chain
    of ``nado`` auxiliary density operators (ADOs) with the last one the zero
    terminator, explicit Euler steps swept level by level in place (level n
    sees the already-updated level n-1 and the old level n+1), observables
    Tr[e rho] after every step, returned as (n_e, nt);
  * ``_heom_propagator`` ``pyqed/oqs.py:1877-1935``: the same sweep on the
    Liouville-space propagator u[n] (N^2 x N^2, row-major vec,
    ``operator_to_superoperator`` ``pyqed/superoperator.py:200-246``), with
    T = temperature / au2k, D0 = pi lambda T (real) and level 0 advanced twice
    per step (once before the level loop and again as its n = 0 entry);
  * ``HEOMSolver``       ``pyqed/oqs.py:1332-1371`` (``run`` and ``propagator``).
Pinned by ``tests/golden/heom_*.npz`` (outputs of the reference itself).
"""
import numpy as np

AU2K = 315775.13  # pyqed/units.py:6


def coefficients_run(temperature, cutoff, reorganization):
    """(gamma, D0) of ``_heom`` (``pyqed/oqs.py:1829-1841``)."""
    gamma = cutoff
    T = temperature
    D0 = reorganization * gamma * (1.0 / np.tanh(gamma / (2.0 * T)) - 1j)
    return gamma, D0


def coefficients_propagator(temperature, cutoff, reorganization):
    """(gamma, D0) of ``_heom_propagator`` (``pyqed/oqs.py:1891-1905``)."""
    T = temperature / AU2K
    return cutoff, complex(np.pi * reorganization * T, 0.0)


def _comm(a, b):
    return a @ b - b @ a


def _acomm(a, b):
    return a @ b + b @ a


def sweep(ado, H, sz, gamma, D0, dt, double_first=False):
    """One Euler step of the hierarchy in matrix form, in place.  ``ado`` is
    (nado, N, N); level nado-1 is never written (the terminator)."""
    nado = ado.shape[0]
    if double_first:  # _heom_propagator's extra level-0 update
        ado[0] = ado[0] - 1j * _comm(H, ado[0]) * dt - _comm(sz, ado[1]) * dt
    ado[0] = ado[0] - 1j * _comm(H, ado[0]) * dt - _comm(sz, ado[1]) * dt
    for n in range(1, nado - 1):
        ado[n] = ado[n] + (-1j * _comm(H, ado[n]) - _comm(sz, ado[n + 1]) - n * gamma * ado[n]
                           + n * (D0.real * _comm(sz, ado[n - 1]) + 1j * D0.imag * _acomm(sz, ado[n - 1]))) * dt
    return ado


def heom_run(H, rho0, sz, e_ops, temperature, cutoff, reorganization, nado, dt, nt, return_ado=False):
    """``_heom``: observables (n_e, nt); with ``return_ado`` also the final
    ADOs (nado, N, N)."""
    H = np.asarray(H, dtype=complex)
    sz = np.asarray(sz, dtype=complex)
    N = H.shape[0]
    gamma, D0 = coefficients_run(temperature, cutoff, reorganization)
    ado = np.zeros((nado, N, N), dtype=complex)
    ado[0] = rho0
    obs = np.zeros((len(e_ops), nt), dtype=complex)
    es = [np.asarray(e, dtype=complex) for e in e_ops]
    for k in range(nt):
        sweep(ado, H, sz, gamma, D0, dt)
        obs[:, k] = [np.trace(e @ ado[0]) for e in es]
    return (obs, ado) if return_ado else obs


def heom_propagator(H, sz, temperature, cutoff, reorganization, nado, dt, nt):
    """``_heom_propagator`` restated on the Liouville space itself: u
    (nado, N^2, N^2), u[0] starting at the identity."""
    H = np.asarray(H, dtype=complex)
    sz = np.asarray(sz, dtype=complex)
    N = H.shape[0]
    I = np.eye(N)
    L0 = np.kron(H, I) - np.kron(I, H.T)
    Sm = np.kron(sz, I) - np.kron(I, sz.T)
    Sp = np.kron(sz, I) + np.kron(I, sz.T)
    gamma, D0 = coefficients_propagator(temperature, cutoff, reorganization)
    a, b = D0.real, D0.imag
    u = np.zeros((nado, N * N, N * N), dtype=complex)
    u[0] = np.eye(N * N)
    for k in range(nt):
        u[0] = u[0] - 1j * L0 @ u[0] * dt - Sm @ u[1] * dt
        for n in range(nado - 1):
            # n = 0 advances level 0 a second time; its u[n-1] term carries a factor 0
            low = (a * Sm + 1j * b * Sp) @ u[n - 1] if n > 0 else 0.0
            u[n] = u[n] + (-1j * L0 @ u[n] + (-Sm @ u[n + 1]) - n * gamma * u[n] + n * low) * dt
    return u
