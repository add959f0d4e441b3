"""Test infrastructure: numpy restatement of the reference's eigen-decomposition
(spectral) Lindblad solver, the checker for ``pyqed_gb300.spectral``.  Only
``tests/`` may use it.

Follows binggu56/pyqed 0.1.3 ``pyqed/superoperator.py``:
  * ``liouvillian``         ``:29-57`` (-i [H, .] + sum_k D[L_k], row-major vec,
                            ``lindblad_dissipator`` ``:249-252``)
  * ``Lindblad_solver``     ``:455-770``: ``eigenstates`` (dense left/right
    eigenvectors of L, norm_n = Re(vl_n^dag vr_n)), ``evolve``,
    ``correlation_2op_1t``/``_1w``, ``correlation_3op_1t``/``_1w``,
    ``correlation_3op_2t`` (returned as (n_tau, n_t)), ``correlation_4op_2t``.
The reference normalises with the REAL part of vl_n^dag vr_n; ``complex_norm``
selects the exact (complex) normalisation instead.  Pinned by
``tests/golden/spectral_jc.npz`` (outputs of the reference itself).
"""
import numpy as np
import scipy.linalg


def liouvillian(H, c_ops):
    """Dense L with d vec(rho)/dt = L vec(rho), row-major vec."""
    H = np.asarray(H, dtype=complex)
    N = H.shape[0]
    I = np.eye(N)
    L = -1j * (np.kron(H, I) - np.kron(I, H.T))
    for c in c_ops or []:
        c = np.asarray(c, dtype=complex)
        cdc = c.conjugate().transpose().dot(c)
        # each dissipator is formed before it is added, as in the reference
        L = L + (np.kron(c, c.conj()) - 0.5 * (np.kron(cdc, I) + np.kron(I, cdc.T)))
    return L


def eigenstates(L, complex_norm=False):
    """(eigvals, right, left, norm) as ``Lindblad_solver.eigenstates``."""
    w, vl, vr = scipy.linalg.eig(L, left=True, right=True)
    nrm = np.diagonal(vl.conj().T @ vr)
    return w, vr, vl, (nrm if complex_norm else nrm.real)


def _trace_left(a, U):
    """Tr[a U_n] for every column n of U (vdot(idv, left(a) U_n))."""
    N = a.shape[0]
    Um = U.T.reshape(-1, N, N)
    return np.einsum("ij,nji->n", a, Um)


def evolve(eig, rho0, tlist, e_ops):
    w, U1, U2, nrm = eig
    coeff = (U2.conj().T @ np.asarray(rho0, dtype=complex).flatten()) / nrm
    out = np.zeros((len(tlist), len(e_ops)), dtype=complex)
    for i, t in enumerate(tlist):
        rho = U1 @ (coeff * np.exp(w * t))
        N = int(round(np.sqrt(rho.size)))
        out[i] = [np.trace(np.asarray(e) @ rho.reshape(N, N)) for e in e_ops]
    return out


def coeff_2op(eig, rho0, a, b):
    w, U1, U2, nrm = eig
    return _trace_left(a, U1) * (U2.conj().T @ (b @ rho0).flatten()) / nrm


def coeff_3op(eig, rho0, a, b, c):
    w, U1, U2, nrm = eig
    return _trace_left(b, U1) * (U2.conj().T @ (c @ rho0 @ a).flatten()) / nrm


def sum_t(w, coeff, tlist):
    return np.array([np.sum(np.exp(w * t) * coeff) for t in tlist])


def sum_w(w, coeff, omegas):
    return np.array([np.sum(-1.0 / (w + 1j * om) * coeff) for om in omegas])


def correlation_3op_2t(eig, rho0, a, b, c, tlist, taulist):
    w, U1, U2, nrm = eig
    N = a.shape[0]
    # right(a) left(c) U1_n = vec(c U_n a)
    M = np.stack([(c @ U1[:, n].reshape(N, N) @ a).flatten() for n in range(U1.shape[1])], axis=1)
    coeff = (_trace_left(b, U1) / nrm)[:, None] * (U2.conj().T @ M) * \
        ((U2.conj().T @ np.asarray(rho0, dtype=complex).flatten()) / nrm)[None, :]
    tmp1 = np.exp(np.outer(w, taulist))
    tmp2 = np.exp(np.outer(w, tlist))
    return tmp1.T @ coeff @ tmp2
