"""Drop-in mirror of the reference's Redfield solver on the GPU.

``RedfieldSolver`` follows ``pyqed.oqs.RedfieldSolver`` (``pyqed/oqs.py:30-100``):
same constructor (H, c_ops = the Hermitian system-bath operators, spectra =
one callable S_k(w) per operator, e_ops), ``redfield_tensor()`` returning the
generator as a CSR matrix and the eigenvectors (``pyqed/oqs.py:519-563``) and
``evolve()`` returning a ``Result`` with the observables after every step and
the states transformed back to the original basis (``_redfield``,
``pyqed/oqs.py:364-459``).  The N^2 x N^2 generator is built on the GPU
(``lgb_redfield_tensor``, O(N^4 K)) and propagated there by the batched RK4
kernel (``lgb_redfield_propagate``).  The eigendecomposition of H and the
bath spectra (Python callables) are evaluated on the host, as in the
reference.  ``redfield_batch`` propagates many systems in one launch.
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.linalg
import torch

from . import _capi as C
from .engine import _device, to_dense
from .mol import Result

__all__ = ["RedfieldSolver", "redfield_batch", "build_tensor", "build_tensors"]

_PREC = {"fp64": C.PREC["fp64"], "fp32": C.PREC["fp32"]}


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else None


def _herm_check(a_ops):
    for a in a_ops:
        if not np.allclose(a, a.conj().T):
            raise TypeError("Operators in a_ops must be Hermitian.")


def _eigen_parts(H, a_ops, spectra):
    """Host part of ``redfield_tensor``: eigenbasis, A_k = V^dag a_k V and the
    spectra C_k[m][l] = S_k(-(e_m - e_l))."""
    H = to_dense(H)
    a_ops = [to_dense(a) for a in a_ops]
    _herm_check(a_ops)
    # the reference's eigensolver (scipy.linalg.eigh): R, the propagator and
    # every other eigenbasis quantity depend on the signs it picks
    evals, evecs = scipy.linalg.eigh(H)
    W = np.real(evals[:, None] - evals[None, :])
    N = len(evals)
    A = np.stack([evecs.conj().T @ a @ evecs for a in a_ops]) if a_ops else np.zeros((0, N, N), complex)
    Cs = np.stack([np.array([[float(s(-W[n, m])) for m in range(N)] for n in range(N)]) for s in spectra[:len(a_ops)]]) \
        if a_ops else np.zeros((0, N, N))
    return evals, evecs, A, Cs


def build_tensor(evals, A, Cs, device=None):
    """The generator R (device complex128, N^2 x N^2) from the eigenvalues,
    the operators in the eigenbasis and the spectra (``lgb_redfield_tensor``)."""
    dev = _device(device)
    N = len(evals)
    L = C.lib()
    ev = torch.from_numpy(np.ascontiguousarray(evals, dtype=np.float64)).to(dev)
    At = torch.from_numpy(np.ascontiguousarray(A, dtype=np.complex128)).to(dev)
    Ct = torch.from_numpy(np.ascontiguousarray(Cs, dtype=np.float64)).to(dev)
    R = torch.empty(N ** 4, dtype=torch.complex128, device=dev)
    with torch.cuda.device(dev):
        C.check(L.lgb_redfield_tensor(N, len(A), _ptr(ev), _ptr(At), _ptr(Ct), _ptr(R),
                                      ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)),
                "lgb_redfield_tensor")
    return R


def build_tensors(parts, device=None):
    """Generators of many systems (``_eigen_parts`` results with the same
    operator count) in one launch (``lgb_redfield_tensor_batch``): packed
    complex128 on the device, system b at sum_{c<b} N_c^4."""
    dev = _device(device)
    dims = [len(p[0]) for p in parts]
    K = parts[0][2].shape[0]
    if any(p[2].shape[0] != K for p in parts):
        return torch.cat([build_tensor(p[0], p[2], p[3], dev) for p in parts])
    L = C.lib()
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)  # noqa: E731
    ev = t(np.concatenate([p[0] for p in parts]), np.float64)
    At = t(np.concatenate([p[2].ravel() for p in parts]) if K else np.zeros(0), np.complex128)
    Ct = t(np.concatenate([p[3].ravel() for p in parts]) if K else np.zeros(0), np.float64)
    R = torch.empty(int(sum(n ** 4 for n in dims)), dtype=torch.complex128, device=dev)
    with torch.cuda.device(dev):
        C.check(L.lgb_redfield_tensor_batch(len(dims), (ctypes.c_int32 * len(dims))(*dims), K, _ptr(ev), _ptr(At),
                                            _ptr(Ct), _ptr(R),
                                            ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)),
                "lgb_redfield_tensor_batch")
    return R


class _Plan:
    def __init__(self, dims, nt, dt, n_eops, precision, store_every, device):
        self.dev = _device(device)
        self.dims = np.asarray(dims, dtype=np.int32)
        self.L = C.lib()
        prob = C.RedfieldProblem(n_inst=len(dims), n_eops=n_eops, nt=nt, precision=_PREC[precision],
                                 store_every=store_every, reserved=0, dt=dt)
        self.plan = ctypes.c_void_p()
        with torch.cuda.device(self.dev):
            C.check(self.L.lgb_redfield_create(ctypes.byref(self.plan), ctypes.byref(prob),
                                               (ctypes.c_int32 * len(dims))(*self.dims.tolist())),
                    "lgb_redfield_create")
        self.nt, self.n_eops, self.store_every = nt, n_eops, store_every
        self.voff = np.concatenate([[0], np.cumsum(self.dims.astype(np.int64) ** 2)])

    def stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def close(self):
        if self.plan.value:
            self.L.lgb_redfield_destroy(self.plan)
            self.plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, R, Ot):
        with torch.cuda.device(self.dev):
            C.check(self.L.lgb_redfield_set(self.plan, _ptr(R), _ptr(Ot), self.stream()), "lgb_redfield_set")

    def propagate(self, r0, want_states=False):
        n = len(self.dims)
        z = lambda k: torch.empty(int(k), dtype=torch.complex128, device=self.dev)  # noqa: E731
        obs = z(n * self.nt * self.n_eops) if self.n_eops else None
        rho = z(self.voff[-1])
        ns = self.nt // self.store_every if self.store_every else 0
        st = z(ns * self.voff[-1]) if (want_states and ns) else None
        with torch.cuda.device(self.dev):
            C.check(self.L.lgb_redfield_propagate(self.plan, _ptr(r0), _ptr(obs), _ptr(rho), _ptr(st),
                                                  self.stream()), "lgb_redfield_propagate")
        flags = (ctypes.c_int32 * n)()
        self.L.lgb_redfield_errors(self.plan, flags)
        bad = [i for i in range(n) if flags[i]]
        if bad:
            raise C.LindbladError(int(flags[bad[0]]), "system %d" % bad[0])
        return obs, rho, st


class RedfieldSolver:
    """``pyqed.oqs.RedfieldSolver`` on the GPU (``pyqed/oqs.py:30-360``).

    Beside ``evolve``: ``propagator`` (the Liouville-space propagator U(t) in
    the eigenbasis; 'SOS' by the eigendecomposition of R, 'EOM' by RK4 with
    dt = t[1] - t[0] on the batched RK4 kernel, one system per basis vector),
    ``gf`` (G(t) = -i U(t)), ``expect``, ``correlation_2op_1t`` and
    ``correlation_4op_3t`` (``pyqed/oqs.py:136-330``).  Deviations, where the
    reference's method cannot run: ``gf(method='EOM')`` returns -i U(t) (the
    reference multiplies a list by -1j), ``correlation_2op_1t`` returns
    <<1| a G(tau) b |rho0>> (the reference's vector shapes do not match),
    ``steady_state`` returns the normalised null vector of R in the original
    basis (the reference's takes no ``self``)."""

    def __init__(self, H, c_ops=None, spectra=None, e_ops=None):
        self.H = H
        self.c_ops = c_ops
        self.R = None
        self.spectra = spectra
        self.evecs = None
        self.dim = H.shape[0]
        self.U = None
        self.G = None
        self.e_ops = e_ops
        self._Rdev = None
        self.U = None
        self.G = None

    def idm(self, sp=True):
        """vec of the identity in Liouville space (row-major)."""
        from scipy.sparse import csr_matrix
        v = np.eye(self.dim).flatten()
        return csr_matrix(v.reshape(-1, 1)) if sp else v

    def configure(self, H, c_ops, e_ops):
        self.c_ops = c_ops
        self.e_ops = e_ops
        self.H = H
        self.R = None
        self._Rdev = None

    def redfield_tensor(self, secular=False):
        """(R as CSR, eigenvectors), ``pyqed/oqs.py:519-563``; R is built on the GPU."""
        from scipy.sparse import csr_matrix
        if self.spectra is None:
            raise TypeError('Specify the bath spectral function.')
        evals, evecs, A, Cs = _eigen_parts(self.H, self.c_ops or [], self.spectra)
        self._Rdev = build_tensor(evals, A, Cs)
        N = len(evals)
        self.R = csr_matrix(self._Rdev.cpu().numpy().reshape(N * N, N * N))
        self.evecs = evecs
        return self.R, evecs

    # ---- Liouville-space propagator and correlations (pyqed/oqs.py:133-330) -------
    def _dense_R(self):
        return self._Rdev.reshape(self.dim ** 2, self.dim ** 2)

    def propagator(self, t, method='SOS'):
        """U(t_k) (M x M x len(t), eigenbasis, M = N^2); also sets ``U`` and
        ``G = -1j U``."""
        if self.R is None:
            raise TypeError('Redfield tensor is not computed. Please call redfield_tensor()')
        t = np.asarray(t, dtype=float)
        M = self.dim ** 2
        dev = self._Rdev.device
        if method == 'EOM':
            # RK4 with dt = t[1] - t[0] from the identity: the M basis vectors
            # as a batch of systems sharing R, every state kept
            nt = len(t) - 1
            U = np.zeros((M, M, len(t)), dtype=complex)
            U[:, :, 0] = np.eye(M)
            if nt > 0:
                plan = _Plan([self.dim] * M, nt, float(t[1] - t[0]), 0, "fp64", 1, dev)
                try:
                    plan.set(self._Rdev.repeat(M), torch.zeros(0, dtype=torch.complex128, device=dev))
                    r0 = torch.eye(M, dtype=torch.complex128, device=dev).reshape(-1)
                    _, _, st = plan.propagate(r0, want_states=True)
                finally:
                    plan.close()
                # system c holds nt consecutive states: U[:, c, k + 1]
                U[:, :, 1:] = st.reshape(M, nt, M).permute(2, 0, 1).cpu().numpy()
        elif method in ['eseries', 'SOS']:
            evals, U1 = scipy.linalg.eig(self.R.toarray())
            U2 = scipy.linalg.inv(U1)
            td = torch.from_numpy(t).to(dev)
            lam = torch.from_numpy(evals).to(dev)
            A = torch.from_numpy(U1).to(dev)
            B = torch.from_numpy(U2).to(dev)
            E = torch.exp(lam[None, :] * td[:, None])              # (T, M)
            U = ((A[None, :, :] * E[:, None, :]) @ B[None]).permute(1, 2, 0).cpu().numpy()
        else:
            raise ValueError('method must be EOM, SOS or eseries')
        self.U = U
        self.G = -1j * self.U
        return self.U

    def gf(self, t, w=None, secular=False, k=1, domain='time', method='EOM'):
        """Liouville-space Green's function G(t) = -i U(t), M x M x len(t)."""
        if self.R is None:
            self.redfield_tensor(secular=secular)
        if method == 'EOM':
            return -1j * self.propagator(t, method='EOM')
        if method in ['eseries', 'diag', 'diagonalization']:
            return -1j * self.propagator(np.asarray(t, dtype=float), method='SOS')
        raise ValueError('method must be EOM, eseries, diag or diagonalization')

    def expect(self, rho0, e_ops):
        """sum_ab e_ab rho_ab(t) in the eigenbasis for every t of the last
        ``propagator`` (the reference's contraction, ``pyqed/oqs.py:319-344``)."""
        V = self.evecs
        r0 = (V.conj().T @ to_dense(rho0) @ V).flatten()
        es = [(V.conj().T @ to_dense(e) @ V).flatten() for e in e_ops]
        dev = self._Rdev.device
        Ud = torch.from_numpy(np.ascontiguousarray(self.U)).to(dev)                  # (M, M, T)
        rho = torch.einsum('abk,b->ak', Ud, torch.from_numpy(r0).to(dev))          # (M, T)
        E = torch.from_numpy(np.stack(es) if es else np.zeros((0, r0.size), complex)).to(dev)
        return (E @ rho).T.cpu().numpy()

    def correlation_2op_1t(self, rho0, a, b, tau):
        """<<1| a G(tau) b |rho0>> for Liouville-space operators a, b (M x M)."""
        if self.G is None:
            self.propagator(tau)
        dev = self._Rdev.device
        den = lambda x: torch.from_numpy(np.ascontiguousarray(to_dense(x), dtype=complex)).to(dev)  # noqa: E731
        r0 = to_dense(rho0)
        r0 = r0.flatten() if r0.ndim == 2 else r0
        G = torch.from_numpy(np.ascontiguousarray(self.G)).to(dev)
        v = den(b) @ torch.from_numpy(np.asarray(r0, dtype=complex)).to(dev)
        tmp = den(a) @ torch.einsum('abk,b->ak', G, v)                               # (M, T)
        idm = torch.from_numpy(np.eye(self.dim).flatten().astype(complex)).to(dev)
        return (idm @ tmp).cpu().numpy()

    def correlation_4op_3t(self, rho0, oplist, signature, tau):
        """<<1| A G(tau3) B G(tau2) C G(tau1) D |rho0>> as (tau3, tau2, tau1)
        (``pyqed/oqs.py:239-330``); the operators act as the superoperators
        ``signature`` names ('l', 'r', 'c', 'a'), all in the eigenbasis.  Uses
        the stored G when there is one, as the reference."""
        if len(oplist) != 4:
            raise ValueError('Number of operators is not 4.')
        sup = [_superop(to_dense(o), sgn) for o, sgn in zip(oplist, signature)]
        if self.G is None:
            self.propagator(tau)
        dev = self._Rdev.device
        tt = lambda x: torch.from_numpy(np.ascontiguousarray(x, dtype=complex)).to(dev)  # noqa: E731
        G = tt(self.G)
        a, b, c, d = (tt(x) for x in sup)
        rho = d @ tt(to_dense(rho0).flatten())
        tmp = torch.einsum('abk,b->ak', G, rho)
        tmp = c @ tmp
        tmp = torch.einsum('abj,bk->ajk', G, tmp)
        tmp = torch.einsum('ab,bjk->ajk', b, tmp)
        tmp = torch.einsum('abi,bjk->aijk', G, tmp)
        idm = tt(np.eye(self.dim).flatten())
        return torch.einsum('a,ab,bijk->ijk', idm, a, tmp).cpu().numpy()

    def steady_state(self):
        """The null vector of R (eigenvalue of smallest modulus), normalised
        to unit trace, as a density matrix in the original basis."""
        if self.R is None:
            self.redfield_tensor()
        evals, vecs = scipy.linalg.eig(self.R.toarray())
        v = vecs[:, np.argmin(np.abs(evals))].reshape(self.dim, self.dim)
        v = v / np.trace(v)
        return self.evecs @ v @ self.evecs.conj().T

    def evolve(self, rho0, dt, Nt, evecs=None, e_ops=[], store_states=False, t0=0, nout=1, *,
               precision="fp64"):
        """``_redfield`` (``pyqed/oqs.py:364-459``): Result with the
        observables Tr[O rho] after every step (Nt rows) and rholist, the Nt
        states in the original basis."""
        if self.R is None or self._Rdev is None:
            self.redfield_tensor()
        V = self.evecs
        N = V.shape[0]
        e_ops = [] if e_ops is None else list(e_ops)
        r0 = V.conj().T @ to_dense(rho0) @ V
        es = [V.conj().T @ to_dense(e) @ V for e in e_ops]
        plan = _Plan([N], Nt, dt, len(es), precision, 1 if Nt > 0 else 0, None)
        try:
            Ot = torch.from_numpy(np.concatenate([e.T.flatten() for e in es]) if es
                                  else np.zeros(0, complex)).to(plan.dev)
            plan.set(self._Rdev.to(plan.dev), Ot)
            r0d = torch.from_numpy(np.ascontiguousarray(r0.flatten())).to(plan.dev)
            obs, rho, st = plan.propagate(r0d, want_states=Nt > 0)
        finally:
            plan.close()
        result = Result(dt=dt, Nt=Nt, rho0=r0, t0=t0)
        result.observables = obs.cpu().numpy().reshape(Nt, len(es)) if obs is not None \
            else np.zeros((Nt, 0), complex)
        if st is not None:
            Vt = torch.from_numpy(V).to(st.device)
            S = st.reshape(Nt, N, N)
            result.rholist = list((Vt @ S @ Vt.conj().T).cpu().numpy())
        else:
            result.rholist = []
        return result


def _superop(a, kind):
    """Row-major superoperator of ``a`` (``operator_to_superoperator``,
    ``pyqed/superoperator.py:200-246``)."""
    n = a.shape[-1]
    i = np.eye(n)
    if kind in ['commutator', 'c', '-']:
        return np.kron(a, i) - np.kron(i, a.T)
    if kind in ['left', 'l']:
        return np.kron(a, i)
    if kind in ['right', 'r']:
        return np.kron(i, a.T)
    if kind in ['anticommutator', 'a', '+']:
        return np.kron(a, i) + np.kron(i, a.T)
    raise ValueError('Error: superoperator {} does not exist.'.format(kind))


def redfield_batch(H, a_ops, spectra, rho0, dt, Nt, e_ops=None, *, precision="fp32", store_every=0,
                   device=None):
    """Many Redfield systems in one launch.  H, a_ops, spectra, rho0, e_ops:
    per-system lists.  Returns dict(observables list of (Nt, E), rho list
    (original basis), states list of (Nt / store_every, N, N) or None)."""
    n = len(H)
    e_ops = e_ops if e_ops is not None else [[] for _ in range(n)]
    E = len(e_ops[0]) if n else 0
    parts = [_eigen_parts(H[b], a_ops[b], spectra[b]) for b in range(n)]
    dims = [len(p[0]) for p in parts]
    plan = _Plan(dims, Nt, dt, E, precision, store_every, device)
    try:
        R = build_tensors(parts, plan.dev)
        Ot = np.concatenate([np.concatenate([(p[1].conj().T @ to_dense(e) @ p[1]).T.flatten()
                                             for e in e_ops[b]]) if E else np.zeros(0, complex)
                             for b, p in enumerate(parts)])
        plan.set(R, torch.from_numpy(Ot).to(plan.dev))
        r0 = np.concatenate([(p[1].conj().T @ to_dense(rho0[b]) @ p[1]).flatten() for b, p in enumerate(parts)])
        obs, rho, st = plan.propagate(torch.from_numpy(r0).to(plan.dev), want_states=store_every > 0)
    finally:
        plan.close()
    res = dict(observables=[], rho=[], states=None)
    oh = obs.cpu().numpy().reshape(n, Nt, E) if obs is not None else np.zeros((n, Nt, 0), complex)
    rh = rho.cpu().numpy()
    for b, p in enumerate(parts):
        N, V = dims[b], p[1]
        res["observables"].append(oh[b])
        res["rho"].append(V @ rh[plan.voff[b]:plan.voff[b + 1]].reshape(N, N) @ V.conj().T)
    if st is not None:
        sh = st.cpu().numpy()
        ns = Nt // store_every
        res["states"] = []
        for b, p in enumerate(parts):
            N, V = dims[b], p[1]
            blk = sh[ns * plan.voff[b]: ns * plan.voff[b + 1]].reshape(ns, N, N)
            res["states"].append(V @ blk @ V.conj().T)
    return res
