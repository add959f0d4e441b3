"""Seeded synthetic inputs for the five Lindblad workloads.

Every generator is deterministic in its seed and returns complex128 numpy
arrays.  All workloads use natural units (hbar = 1).  The reference publishes
no benchmark data for its Lindblad solver, so these generators are the
workloads; they follow the shapes and value distributions of the reference's
use of ``pyqed.oqs.LindbladSolver`` (``pyqed/oqs.py:1114-1330``):

* ``jaynes_cummings``: cavity (Fock cutoff 8) x two-level molecule, N = 16,
  two collapse operators, e_ops a^dag a and sigma+ sigma-.
* ``gue_instance``: one dense instance with a GUE Hamiltonian and K dense
  complex-Gaussian collapse operators (N = 256, K = 4 and N = 1024, K = 8).
* ``exciton_instance`` / ``exciton_batch``: Frenkel-exciton aggregates in the
  ground + single-excitation space (N = n + 1, n ~ U{8..64}) with pure
  dephasing, for the two-point dipole correlation C(t) = Tr[mu rho(t)],
  rho(0) = mu |g><g|.
* ``driven_batch``: N = 64 instances driven by -mu E(t) with a smooth
  Gaussian-process pulse E(t).
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "jaynes_cummings", "gue_matrix", "gue_instance", "exciton_dims",
    "exciton_instance", "exciton_batch", "gp_pulse", "driven_batch",
    "ohmic_spectrum", "redfield_chain", "WORKLOADS",
]


def _cnormal(rng, shape):
    """Complex standard normal: E|z|^2 = 1."""
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0)


def jaynes_cummings(nfock=8, wc=1.0, wm=1.0, g=0.05, kappa=0.01, gamma=0.005,
                    dt=0.02, nt=2000):
    """Jaynes-Cummings cavity + two-level molecule.

    Basis index 2n + s with Fock number n in 0..nfock-1 and s in {g=0, e=1}.
    H = wc a^dag a + wm sigma+ sigma- + g (a^dag sigma- + a sigma+);
    c_ops = sqrt(kappa) a, sqrt(gamma) sigma-; rho0 = |n=1, g><n=1, g|.
    """
    a1 = np.diag(np.sqrt(np.arange(1, nfock)), 1).astype(complex)
    sm1 = np.array([[0, 1], [0, 0]], dtype=complex)  # |g><e|
    a = np.kron(a1, np.eye(2))
    sm = np.kron(np.eye(nfock), sm1)
    ad, sp = a.conj().T, sm.conj().T
    H = wc * ad @ a + wm * sp @ sm + g * (ad @ sm + a @ sp)
    c_ops = [np.sqrt(kappa) * a, np.sqrt(gamma) * sm]
    N = 2 * nfock
    psi = np.zeros(N, complex)
    psi[2 * 1 + 0] = 1.0
    rho0 = np.outer(psi, psi.conj())
    e_ops = [ad @ a, sp @ sm]
    return dict(H=H, c_ops=c_ops, rho0=rho0, e_ops=e_ops, dt=dt, nt=nt)


def gue_matrix(rng, N):
    """H = (G + G^dag)/2 with G_ij complex N(0,1)/sqrt(N)."""
    G = _cnormal(rng, (N, N)) / np.sqrt(N)
    return 0.5 * (G + G.conj().T)


def gue_instance(N=256, K=4, scale=0.05, rank=1, seed=2, dt=0.01, nt=10000):
    """One dense instance: GUE H, K complex-Gaussian collapse operators
    (entries x scale/sqrt(N)) and a random rank-``rank`` initial state.

    rank 1: rho0 = |psi><psi|, psi a normalised complex Gaussian vector.
    rank r > 1: rho0 = sum_i p_i |psi_i><psi_i|, psi_i orthonormalised by QR
    of a complex Gaussian N x r matrix and p ~ Dirichlet(1).
    """
    rng = np.random.default_rng(seed)
    H = gue_matrix(rng, N)
    c_ops = [_cnormal(rng, (N, N)) * (scale / np.sqrt(N)) for _ in range(K)]
    if rank == 1:
        psi = _cnormal(rng, N)
        psi /= np.linalg.norm(psi)
        rho0 = np.outer(psi, psi.conj())
    else:
        Q, _ = np.linalg.qr(_cnormal(rng, (N, rank)))
        p = rng.dirichlet(np.ones(rank))
        rho0 = (Q * p) @ Q.conj().T
    return dict(H=H, c_ops=c_ops, rho0=rho0, e_ops=[], dt=dt, nt=nt)


def exciton_dims(n_inst=4096, seed=3, nmin=8, nmax=64):
    """Site counts n ~ U{nmin..nmax}; the instance dimension is N = n + 1."""
    rng = np.random.default_rng(seed)
    return rng.integers(nmin, nmax + 1, size=n_inst) + 1


def exciton_instance(n, index=0, seed=3, e0=1.0, sigma=0.05, J=-0.02, gamma=0.01):
    """One Frenkel-exciton aggregate of n sites in the {|g>, |1..n>} basis.

    H_gg = 0, H_kk = e0 + sigma xi_k, H_{k,k+1} = J; mu_gk = mu_kg = c_k with
    c_k ~ U[-1, 1] (orientation cosine of a unit dipole); collapse operators
    sqrt(gamma)|k><k| for k = 1..n, returned as their diagonals;
    rho_g = |g><g|.
    """
    rng = np.random.default_rng((seed, index))
    N = n + 1
    H = np.zeros((N, N), complex)
    xi = rng.standard_normal(n)
    H[np.arange(1, N), np.arange(1, N)] = e0 + sigma * xi
    k = np.arange(1, N - 1)
    H[k, k + 1] = J
    H[k + 1, k] = J
    c = rng.uniform(-1.0, 1.0, size=n)
    mu = np.zeros((N, N), complex)
    mu[0, 1:] = c
    mu[1:, 0] = c
    cdiag = np.zeros((n, N), complex)
    cdiag[np.arange(n), np.arange(1, N)] = np.sqrt(gamma)
    rho_g = np.zeros((N, N), complex)
    rho_g[0, 0] = 1.0
    return dict(H=H, mu=mu, c_diag=cdiag, rho_g=rho_g)


def exciton_batch(n_inst=4096, seed=3, indices=None, dt=0.05, nt=4000):
    """Batch of exciton instances (see ``exciton_instance``).

    ``indices`` selects a subset of the full batch (same per-instance draws).
    Returns a dict of lists plus dt, nt.
    """
    dims = exciton_dims(n_inst, seed)
    if indices is None:
        indices = range(n_inst)
    insts = [exciton_instance(int(dims[i]) - 1, index=int(i), seed=seed) for i in indices]
    return dict(
        H=[d["H"] for d in insts], mu=[d["mu"] for d in insts],
        c_diag=[d["c_diag"] for d in insts], rho_g=[d["rho_g"] for d in insts],
        dims=np.array([d["H"].shape[0] for d in insts]), dt=dt, nt=nt)


def gp_pulse(nt, dt, seed, length=2.0, amp=0.05, nfeat=256):
    """Smooth Gaussian-process pulse E(t_k), t_k = (k+1) dt, k = 0..nt-1.

    A squared-exponential-kernel GP (length scale ``length``, amplitude
    ``amp``) sampled by random Fourier features: E(t) = amp sqrt(2/M)
    sum_m w_m cos(omega_m t + phi_m), omega_m ~ N(0, 1/length^2),
    w_m ~ N(0,1), phi_m ~ U[0, 2 pi).
    """
    rng = np.random.default_rng(seed)
    om = rng.standard_normal(nfeat) / length
    ph = rng.uniform(0.0, 2 * np.pi, nfeat)
    w = rng.standard_normal(nfeat)
    t = (np.arange(nt) + 1) * dt
    return amp * np.sqrt(2.0 / nfeat) * (np.cos(np.outer(t, om) + ph) @ w)


def driven_batch(n_inst=256, N=64, K=2, seed=5, dt=0.01, nt=2000,
                 length=2.0, amp=0.05, damp=0.01):
    """Driven instances: H(t) = H0 - E(t) mu, K collapse operators
    sqrt(gamma_k) L_k (L_k complex Gaussian / sqrt(N), gamma_k ~ U[0.005,
    0.02]), a random pure initial state and a GUE observable O per instance.
    E is shared by all instances; ``E_target`` = E + dE (dE a GP sample of
    amplitude ``damp``) defines the target trajectory of the adjoint loss.
    """
    H0, mu, Lhat, gam, rho0, O = [], [], [], [], [], []
    for b in range(n_inst):
        rng = np.random.default_rng((seed, b))
        H0.append(gue_matrix(rng, N))
        mu.append(gue_matrix(rng, N))
        Lhat.append([_cnormal(rng, (N, N)) / np.sqrt(N) for _ in range(K)])
        gam.append(rng.uniform(0.005, 0.02, size=K))
        psi = _cnormal(rng, N)
        psi /= np.linalg.norm(psi)
        rho0.append(np.outer(psi, psi.conj()))
        O.append(gue_matrix(rng, N))
    E = gp_pulse(nt, dt, seed=(seed * 1000 + 1), length=length, amp=amp)
    dE = gp_pulse(nt, dt, seed=(seed * 1000 + 2), length=length, amp=damp)
    return dict(H0=H0, mu=mu, L=Lhat, gamma=np.array(gam), rho0=rho0, O=O,
                E=E, E_target=E + dE, dt=dt, nt=nt)


WORKLOADS = {
    "jc16": "Jaynes-Cummings N=16, K=2, dt=0.02, 2000 steps",
    "gue256": "GUE N=256, K=4 dense collapse ops, dt=0.01, 10000 steps",
    "exciton4096": "4096 Frenkel-exciton instances, N=n+1, n~U{8..64}, diagonal dephasing, "
                   "dt=0.05, 4000 steps, C(t)=Tr[mu rho(t)]",
    "gue1024": "GUE N=1024, K=8 dense collapse ops, rank-4 rho0, dt=0.005, 1000 steps",
    "driven256": "256 driven instances N=64, K=2, H(t)=H0-E(t)mu, dt=0.01, 2000 steps",
}


class ohmic_spectrum:
    """Bath spectral function for the Redfield tensor: Ohmic density with an
    exponential cutoff at inverse temperature beta,
        S(w) = 2 eta w exp(-|w| / wc) / (1 - exp(-beta w)),   S(0) = 2 eta / beta,
    so that S(w) / S(-w) = exp(beta w) (detailed balance).  A picklable
    callable of one float, as ``RedfieldSolver(spectra=[...])`` expects."""

    def __init__(self, eta=0.05, wc=0.5, beta=5.0):
        self.eta, self.wc, self.beta = float(eta), float(wc), float(beta)

    def __call__(self, w):
        w = float(w)
        if abs(w) < 1e-12:
            return 2.0 * self.eta / self.beta
        return 2.0 * self.eta * w * np.exp(-abs(w) / self.wc) / (1.0 - np.exp(-self.beta * w))


def redfield_chain(n=6, seed=7, e0=0.0, sigma=0.05, J=0.02, eta=0.05, wc=0.5, beta=5.0):
    """Disordered exciton chain (single-excitation manifold, N = n sites) with
    one independent Ohmic bath per site: a_ops = |k><k|, the Redfield setting
    of ``pyqed/oqs.py:30-100``.  rho0 = |n-1><n-1|; e_ops = the site populations
    of the first and last site."""
    rng = np.random.default_rng(seed)
    H = np.diag(e0 + sigma * rng.standard_normal(n) + 0.08 * np.arange(n)).astype(complex)
    k = np.arange(n - 1)
    H[k, k + 1] = J
    H[k + 1, k] = J
    a_ops = [np.diag((np.arange(n) == s).astype(complex)) for s in range(n)]
    rho0 = np.zeros((n, n), complex)
    rho0[n - 1, n - 1] = 1.0
    e_ops = [a_ops[0], a_ops[n - 1]]
    return dict(H=H, a_ops=a_ops, spectra=[ohmic_spectrum(eta, wc, beta)] * n, rho0=rho0, e_ops=e_ops,
                eta=eta, wc=wc, beta=beta)



def heom_spin_boson(delta=1.0, eps0=1.0):
    """Spin-boson setting of the reference's HEOM example: H = -delta/2 sx -
    eps0/2 sz, bath coupling sz, rho0 = |1><1|, e_ops = [sz]."""
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    sz = np.array([[1, 0], [0, -1]], dtype=complex)
    H = -0.5 * delta * sx - 0.5 * eps0 * sz
    rho0 = np.zeros((2, 2), complex)
    rho0[1, 1] = 1.0
    return dict(H=H, sz=sz, rho0=rho0, e_ops=[sz])


def heom_chain(n=6, seed=11, sigma=0.05, J=0.1):
    """Disordered n-site chain coupled to one bath through the collective
    coordinate sz = diag(linspace(1, -1, n)) (the reference's HEOM takes one
    system-bath operator); rho0 = |0><0|, e_ops = populations of the first and
    last site."""
    rng = np.random.default_rng(seed)
    H = np.diag(sigma * rng.standard_normal(n) + 0.05 * np.arange(n)).astype(complex)
    k = np.arange(n - 1)
    H[k, k + 1] = J
    H[k + 1, k] = J
    sz = np.diag(np.linspace(1.0, -1.0, n)).astype(complex)
    rho0 = np.zeros((n, n), complex)
    rho0[0, 0] = 1.0
    e_ops = [np.diag((np.arange(n) == 0).astype(complex)), np.diag((np.arange(n) == n - 1).astype(complex))]
    return dict(H=H, sz=sz, rho0=rho0, e_ops=e_ops)


def heom_ensemble(n_inst=4096, n=8, seed=13):
    """Parameter sweep for the batched HEOM: n_inst disordered n-site chains
    (``heom_chain`` with per-instance seeds), each with its own bath:
    temperature ~ U[0.5, 2], cutoff ~ U[0.2, 1], reorganization ~ U[0.01, 0.05]."""
    rng = np.random.default_rng(seed)
    T = rng.uniform(0.5, 2.0, n_inst)
    cut = rng.uniform(0.2, 1.0, n_inst)
    lam = rng.uniform(0.01, 0.05, n_inst)
    seeds = rng.integers(0, 2 ** 31, n_inst)
    chains = [heom_chain(n, int(s)) for s in seeds]
    return dict(H=[c["H"] for c in chains], sz=[c["sz"] for c in chains], rho0=[c["rho0"] for c in chains],
                e_ops=[c["e_ops"] for c in chains], temperature=T, cutoff=cut, reorganization=lam)
