"""Test infrastructure: numpy complex128 restatement of the reference's Redfield
solver, the checker for ``pyqed_gb300.redfield``.  Only ``tests/`` may use it.

Follows binggu56/pyqed 0.1.3:
  * ``redfield_tensor``   ``pyqed/oqs.py:519-563`` (with ``op2sop``/``left``/
    ``right`` of ``pyqed/superoperator.py:172-270``: row-major vec,
    left(a) = a (x) 1, right(a) = 1 (x) a^T)
  * ``_redfield``         ``pyqed/oqs.py:364-459`` (the ``return_result`` branch)
  * ``rk4``               ``pyqed/phys.py:1051-1064``; ``transform`` ``:1121-1140``;
    ``obs_dm`` ``:1257-1264``
  * ``RedfieldSolver.propagator`` / ``expect`` / ``correlation_4op_3t``
                          ``pyqed/oqs.py:161-330`` (with ``expm``
    ``pyqed/phys.py:2049-2097`` for the 'EOM' propagator)
Pinned by ``tests/golden/redfield*.npz`` (outputs of the reference itself).
"""
import numpy as np


def _dag(a):
    return a.conj().T


def _op2sop(a):
    n = a.shape[-1]
    i = np.eye(n)
    return np.kron(a, i) - np.kron(i, a.T)


def _left(a):
    return np.kron(a, np.eye(a.shape[-1]))


def _right(a):
    return np.kron(np.eye(a.shape[-1]), a.T)


def redfield_tensor(H, a_ops, spectra):
    """R (dense, N^2 x N^2) with d vec(rho)/dt = R vec(rho) in the eigenbasis of
    H, and the eigenvectors (columns).  ``pyqed/oqs.py:519-563``."""
    H = np.asarray(H.toarray() if hasattr(H, "toarray") else H, dtype=complex)
    a_ops = [np.asarray(a.toarray() if hasattr(a, "toarray") else a, dtype=complex) for a in a_ops]
    for a in a_ops:
        if not np.allclose(a, _dag(a)):
            raise TypeError("Operators in a_ops must be Hermitian.")
    import scipy.linalg
    evals, evecs = scipy.linalg.eigh(H)  # the reference's eigensolver: eigenbasis quantities depend on its signs
    W = np.real(evals[:, None] - evals[None, :])
    N = len(evals)
    R = -1j * _op2sop(np.diag(evals))
    for k, a in enumerate(a_ops):
        C = np.array([[spectra[k](-W[n, m]) for m in range(N)] for n in range(N)])
        A = _dag(evecs) @ a @ evecs
        L = C * A
        R = R - _op2sop(A) @ (_left(L) - _right(_dag(L)))
    return R, evecs


def redfield_elementwise(evals, A_list, C_list):
    """The same tensor from its element formula (the GPU builds it this way):
    R[(a,b),(x,y)] = -i (e_a - e_b) d_ax d_by
                     - sum_k [ (A L)_ax d_by - A_ax (L^dag)_yb - L_ax A_yb + d_ax (L^dag A)_yb ]
    with L = C o A."""
    N = len(evals)
    I = np.eye(N)
    R = -1j * np.einsum("ax,by->abxy", np.diag(evals), I) + 1j * np.einsum("ax,by->abxy", I, np.diag(evals))
    for A, C in zip(A_list, C_list):
        L = C * A
        Ld = _dag(L)
        R = R - np.einsum("ax,by->abxy", A @ L, I) + np.einsum("ax,yb->abxy", A, Ld) \
            + np.einsum("ax,yb->abxy", L, A) - np.einsum("ax,yb->abxy", I, Ld @ A)
    return R.reshape(N * N, N * N)


def rk4_vec(y, R, dt):
    """``pyqed/phys.py:1051-1064`` with rhs(psi, R) = R psi (``pyqed/oqs.py:462``)."""
    k1 = R @ y
    k2 = R @ (y + 0.5 * dt * k1)
    k3 = R @ (y + 0.5 * dt * k2)
    k4 = R @ (y + dt * k3)
    return y + dt / 6.0 * (k1 + 2.0 * k2 + 2.0 * k3 + k4)


def redfield_propagate(R, rho0, evecs, Nt, dt, e_ops=()):
    """``_redfield`` (``pyqed/oqs.py:364-459``): rho0 and e_ops taken to the
    eigenbasis, Nt RK4 steps of vec(rho); observables Tr[e rho] after every
    step and the states transformed back (rholist).  Returns (obs (Nt, E),
    rholist, rho0 in the eigenbasis)."""
    N = rho0.shape[0]
    r0 = _dag(evecs) @ rho0 @ evecs
    es = [_dag(evecs) @ np.asarray(e, dtype=complex) @ evecs for e in e_ops]
    y = r0.flatten().astype(complex)
    obs = np.zeros((Nt, len(es)), dtype=complex)
    rholist = []
    for k in range(Nt):
        y = rk4_vec(y, R, dt)
        tmp = y.reshape(N, N)
        rholist.append(evecs @ tmp @ _dag(evecs))
        obs[k, :] = [np.trace(e @ tmp) for e in es]
    return obs, rholist, r0


def propagator_sos(R, t):
    """U(t_k) = U1 exp(lambda t_k) U1^-1, (M, M, len(t)) (``propagator`` 'SOS')."""
    import scipy.linalg
    evals, U1 = scipy.linalg.eig(R)
    U2 = scipy.linalg.inv(U1)
    E = np.exp(evals[:, None] * np.asarray(t)[None, :])
    return np.einsum('aj,jk,jb->abk', U1, E, U2)


def propagator_eom(R, t):
    """RK4 steps of dU/dt = R U from the identity with dt = t[1] - t[0]
    (``expm`` 'EOM', ``pyqed/phys.py:2081-2097``)."""
    M = R.shape[0]
    U = np.eye(M, dtype=complex)
    out = []
    dt = t[1] - t[0] if len(t) > 1 else 0.0
    for _ in range(len(t)):
        out.append(U.copy())
        U = rk4_vec(U, R, dt)
    return np.dstack(out)


def expect(U, rho0, evecs, e_ops):
    """``RedfieldSolver.expect`` with an ndarray propagator: sum_ab e_ab rho_ab(t)
    in the eigenbasis (``pyqed/oqs.py:319-344``)."""
    r0 = (_dag(evecs) @ rho0 @ evecs).flatten()
    rho = np.tensordot(U, r0, axes=([1], [0]))
    return np.stack([(_dag(evecs) @ e @ evecs).flatten() @ rho for e in e_ops], axis=1)


def superop(a, kind):
    n = a.shape[-1]
    i = np.eye(n)
    return {"l": np.kron(a, i), "r": np.kron(i, a.T), "c": np.kron(a, i) - np.kron(i, a.T),
            "a": np.kron(a, i) + np.kron(i, a.T)}[kind]


def correlation_4op_3t(G, rho0, oplist, signature):
    """``RedfieldSolver.correlation_4op_3t`` (``pyqed/oqs.py:239-330``) with the
    Green's function G (M, M, T): (tau3, tau2, tau1)."""
    a, b, c, d = (superop(o, s) for o, s in zip(oplist, signature))
    n = rho0.shape[0]
    rho = d @ rho0.flatten()
    tmp = np.tensordot(G, rho, axes=(1, 0))
    tmp = c @ tmp
    tmp = np.tensordot(G, tmp, axes=([1], [0]))
    tmp = np.tensordot(b, tmp, axes=([1], [0]))
    tmp = np.tensordot(G, tmp, axes=([1], [0]))
    return np.einsum('a,ab,bijk->ijk', np.eye(n).flatten(), a, tmp)
