"""Generate the golden fixtures from the reference implementation itself.

Run in a container where the reference (binggu56/pyqed 0.1.3) is mounted,
with ``PYQED_REFERENCE`` set to its directory:

    PYQED_REFERENCE=/root/reference python tests/golden/make_golden.py
    PYQED_REFERENCE=/root/reference python tests/golden/make_golden.py long

(the second form writes the full-length fixtures listed last below; its N=1024
run takes over an hour on 8 cores).

Every fixture holds the inputs (or, for N >= 256, a checksum of the seeded
inputs) and the outputs of the reference's own entry points:

* ``jc16.npz``       ``LindbladSolver.run`` (CSR path, ``pyqed/oqs.py:1149-1187``
                     -> ``_lindblad`` ``pyqed/oqs.py:1596-1696``), full 2000 steps.
* ``gue64.npz``      ``_fast_lindblad`` (``pyqed/oqs.py:1492-1594``), N=64, K=4.
* ``gue256.npz``     ``_fast_lindblad``, the N=256, K=4 workload, 4 steps.
* ``gue1024.npz``    ``_fast_lindblad``, the N=1024, K=8 workload, 2 steps
                     (rows 0..7, the diagonal and the trace of the final state).
* ``exciton.npz``    ``_correlation_2p_1t`` (``pyqed/oqs.py:717-791``) on 8
                     instances of the exciton batch, 40 steps.
* ``driven64.npz``   ``LindbladSolver.run`` with ``H = [H0, [mu, f]]``
                     (``_lindblad_driven``, ``pyqed/oqs.py:1699-1806``), 2
                     instances of the driven batch, 30 steps.
* ``corr_jc.npz``    ``correlation_2op_1t``, ``correlation_3op_1t`` and
                     ``correlation_4op_1t`` (``pyqed/oqs.py:1193-1312``) on the
                     Jaynes-Cummings system, 50 steps.
* ``redfield_*.npz`` ``RedfieldSolver.redfield_tensor`` / ``evolve``.
* ``spectral_jc.npz`` the eigen-decomposition ``Lindblad_solver``
                     (``pyqed/superoperator.py:455-770``) correlations on
                     the Jaynes-Cummings system with 3 Fock states.
* ``api_signatures.json`` the public methods and parameter names of the
                     reference classes the mirrors replace.
* ``heom_*.npz``     ``HEOMSolver.run`` (``_heom``) on the reference's
                     spin-boson example and a 6-site chain, and
                     ``HEOMSolver.propagator`` (``_heom_propagator``) on a
                     3-site chain.
* ``gue256_long.npz``, ``gue1024_long.npz``, ``driven64_long.npz``: the dense
                     and driven workloads at their full configured lengths
                     (10000, 1000 and 2000 steps), see ``long_fixtures``.
"""
from __future__ import annotations

import hashlib
import os
import sys
import tempfile

import numpy as np
from scipy.sparse import csr_matrix

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from pyqed_gb300 import workloads as W  # noqa: E402
from ref_loader import load  # noqa: E402


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.complex128).tobytes())
    return h.hexdigest()


def redfield_fixtures(oqs):
    out = {}
    # 8. Redfield solver (pyqed/oqs.py:30-100, 364-459, 519-563): a disordered
    # chain with one Ohmic bath per site, and a complex GUE Hamiltonian with
    # two general Hermitian system-bath operators
    ch = W.redfield_chain(n=6, seed=7)
    sol = oqs.RedfieldSolver(ch["H"], c_ops=ch["a_ops"], spectra=ch["spectra"])
    r = sol.evolve(ch["rho0"], dt=0.1, Nt=200, e_ops=ch["e_ops"])
    keep = [0, 99, 199]
    out["redfield_chain"] = dict(
        H=ch["H"], a_ops=np.stack(ch["a_ops"]), rho0=ch["rho0"], e_ops=np.stack(ch["e_ops"]),
        eta=ch["eta"], wc=ch["wc"], beta=ch["beta"], dt=0.1, nt=200, R=sol.R.toarray(),
        evecs=sol.evecs, observables=r.observables, state_index=np.array(keep),
        states=np.stack([r.rholist[k] for k in keep]))
    rng = np.random.default_rng(8)
    N = 8
    H = W.gue_matrix(rng, N)
    a_ops = []
    for _ in range(2):
        m = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.3
        a_ops.append(0.5 * (m + m.conj().T))
    spectra = [W.ohmic_spectrum(0.04, 1.0, 2.0), W.ohmic_spectrum(0.02, 0.5, 8.0)]
    psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    psi /= np.linalg.norm(psi)
    rho0 = np.outer(psi, psi.conj())
    sol = oqs.RedfieldSolver(H, c_ops=a_ops, spectra=spectra)
    r = sol.evolve(rho0, dt=0.05, Nt=120, e_ops=[H, a_ops[0]])
    out["redfield_gue"] = dict(
        H=H, a_ops=np.stack(a_ops), spectra=np.array([[0.04, 1.0, 2.0], [0.02, 0.5, 8.0]]),
        rho0=rho0, e_ops=np.stack([H, a_ops[0]]), dt=0.05, nt=120, R=sol.R.toarray(), evecs=sol.evecs,
        observables=r.observables, rho_last=r.rholist[-1])

    # the Liouville-space propagator, expectation values, Green's function and
    # 4-point correlation of a 3-site chain (pyqed/oqs.py:136-330)
    import contextlib
    import io
    ch = W.redfield_chain(n=3, seed=5)
    t = np.linspace(0.0, 2.0, 6)
    ops = [ch["e_ops"][0], ch["a_ops"][1], ch["a_ops"][0], ch["e_ops"][1]]
    with contextlib.redirect_stdout(io.StringIO()):
        sol = oqs.RedfieldSolver(ch["H"], c_ops=ch["a_ops"], spectra=ch["spectra"])
        R, V = sol.redfield_tensor()
        sol.evecs = V
        U_sos = sol.propagator(t)
        ex = sol.expect(ch["rho0"], ch["e_ops"])
        c4 = sol.correlation_4op_3t(ch["rho0"], ops, "llrr", t[:4])
        G = sol.gf(t, method="diag")
        sol2 = oqs.RedfieldSolver(ch["H"], c_ops=ch["a_ops"], spectra=ch["spectra"])
        sol2.redfield_tensor()
        U_eom = sol2.propagator(t, method="EOM")
    out["redfield_aux"] = dict(t=t, R=R.toarray(), evecs=V, U_sos=U_sos, U_eom=U_eom, expect=ex, c4=c4, gf=G,
                               ops=np.stack(ops), rho0=ch["rho0"])
    return out


def heom_fixtures(oqs):
    import contextlib
    import io
    out = {}
    # 9. HEOM (pyqed/oqs.py:1332-1371, 1808-1935); the reference prints its
    # bath parameters, which are discarded here
    quiet = contextlib.redirect_stdout(io.StringIO())
    sb = W.heom_spin_boson()
    runs = [dict(temperature=600.0, cutoff=5.0, reorganization=0.2, nado=5, dt=0.02, nt=100),
            dict(temperature=1.0, cutoff=0.5, reorganization=0.2, nado=8, dt=0.02, nt=400)]
    obs = []
    with quiet:
        for r in runs:
            sol = oqs.HEOMSolver(sb["H"], c_ops=[sb["sz"]], e_ops=sb["e_ops"])
            obs.append(sol.run(rho0=sb["rho0"].real.copy(), **r))
    out["heom_spinboson"] = dict(
        H=sb["H"], sz=sb["sz"], rho0=sb["rho0"], e_ops=np.stack(sb["e_ops"]),
        params=np.array([[r["temperature"], r["cutoff"], r["reorganization"], r["nado"], r["dt"], r["nt"]]
                         for r in runs]), obs0=obs[0], obs1=obs[1])
    ch = W.heom_chain(n=6, seed=11)
    par = dict(temperature=1.0, cutoff=0.5, reorganization=0.03, nado=8, dt=0.01, nt=500)
    with quiet:
        sol = oqs.HEOMSolver(ch["H"], c_ops=[ch["sz"]], e_ops=ch["e_ops"])
        o = sol.run(rho0=ch["rho0"], **par)
    out["heom_chain"] = dict(H=ch["H"], sz=ch["sz"], rho0=ch["rho0"], e_ops=np.stack(ch["e_ops"]),
                             params=np.array([par[k] for k in ("temperature", "cutoff", "reorganization",
                                                               "nado", "dt", "nt")]), observables=o)
    ch = W.heom_chain(n=3, seed=12)
    par = dict(dt=0.005, nt=60, temperature=300.0, cutoff=5.0, reorganization=0.2, nado=5)
    with quiet:
        sol = oqs.HEOMSolver(ch["H"], c_ops=[ch["sz"]], e_ops=ch["e_ops"])
        u = sol.propagator(**par)
    out["heom_propagator"] = dict(H=ch["H"], sz=ch["sz"],
                                  params=np.array([par[k] for k in ("temperature", "cutoff", "reorganization",
                                                                    "nado", "dt", "nt")]), u=u)
    return out


def spectral_fixtures():
    import importlib
    load()
    so = importlib.import_module("pyqed.superoperator")
    # 10. eigen-decomposition Lindblad solver (pyqed/superoperator.py:455-770)
    # on the Jaynes-Cummings system with 3 Fock states (N = 6, 36 modes)
    jc = W.jaynes_cummings(nfock=3)
    H, c_ops, rho0 = jc["H"], jc["c_ops"], jc["rho0"]
    a, b, c, d = jc["e_ops"][0], jc["c_ops"][0], jc["e_ops"][1], jc["c_ops"][1]
    sol = so.Lindblad_solver(H, c_ops)
    w, vr, vl = sol.eigenstates()
    tl = np.linspace(0.0, 6.0, 13)
    tau = np.linspace(0.0, 3.0, 5)
    om = np.linspace(-2.1, 2.1, 8)
    return {"spectral_jc": dict(
        H=H, c_ops=np.stack(c_ops), rho0=rho0, ops=np.stack([a, b, c, d]), tlist=tl, taulist=tau, omegas=om,
        eigvals=w, L=sol.L.toarray(),
        c2_1t=sol.correlation_2op_1t(rho0, [a, b], tl), c2_1w=sol.correlation_2op_1w(rho0, [a, b], om),
        c3_1t=sol.correlation_3op_1t(rho0, [a, b, c], tl), c3_1w=sol.correlation_3op_1w(rho0, [a, b, c], om),
        c3_2t=sol.correlation_3op_2t(rho0, [a, b, c], tl, tau),
        c4_2t=sol.correlation_4op_2t(rho0, [a, b, c, d], tl, tau))}


def api_fixture():
    """Public method names and parameter names of the reference classes the
    mirrors replace (a drop-in must accept the same calls)."""
    import importlib
    import inspect
    import json
    oqs = load()
    so = importlib.import_module("pyqed.superoperator")
    api = {}
    for key, cls in (("LindbladSolver", oqs.LindbladSolver), ("RedfieldSolver", oqs.RedfieldSolver),
                     ("HEOMSolver", oqs.HEOMSolver), ("Lindblad_solver", so.Lindblad_solver)):
        api[key] = {name: [p.name for p in inspect.signature(f).parameters.values()]
                    for name, f in inspect.getmembers(cls, inspect.isfunction)
                    if not name.startswith("_") or name == "__init__"}
    path = os.path.join(HERE, "api_signatures.json")
    with open(path, "w") as f:
        json.dump(api, f, indent=1, sort_keys=True)
    print("api_signatures", os.path.getsize(path), "bytes")


def main():
    oqs = load()
    out = {}

    # 1. Jaynes-Cummings via the public run() (CSR operators, as it requires)
    jc = W.jaynes_cummings()
    sol = oqs.LindbladSolver(csr_matrix(jc["H"]), [csr_matrix(c) for c in jc["c_ops"]])
    r = sol.run(jc["rho0"], dt=jc["dt"], Nt=jc["nt"], e_ops=[csr_matrix(e) for e in jc["e_ops"]])
    keep = [0, 499, 1999]
    out["jc16"] = dict(
        H=jc["H"], c_ops=np.stack(jc["c_ops"]), rho0=jc["rho0"], e_ops=np.stack(jc["e_ops"]),
        dt=jc["dt"], nt=jc["nt"], observables=r.observables, times=r.times,
        state_index=np.array(keep), states=np.stack([r.rholist[k].toarray() for k in keep]))

    # 2. GUE N=64, K=4, dense path
    g = W.gue_instance(N=64, K=4, seed=12, nt=50)
    rho = oqs._fast_lindblad(g["H"], g["rho0"].copy(), g["c_ops"], e_ops=[], Nt=g["nt"], dt=g["dt"])
    out["gue64"] = dict(H=g["H"], c_ops=np.stack(g["c_ops"]), rho0=g["rho0"], dt=g["dt"],
                        nt=g["nt"], rho=rho)

    # 3. GUE N=256, K=4 (the workload's own seed), 4 steps
    g = W.gue_instance(N=256, K=4, seed=2)
    nt = 4
    rho = oqs._fast_lindblad(g["H"], g["rho0"].copy(), g["c_ops"], e_ops=[], Nt=nt, dt=g["dt"])
    out["gue256"] = dict(digest=digest(g["H"], *g["c_ops"], g["rho0"]), dt=g["dt"], nt=nt, rho=rho)

    # 4. GUE N=1024, K=8, rank-4 rho0, 2 steps (slices only)
    g = W.gue_instance(N=1024, K=8, scale=0.02, rank=4, seed=4, dt=0.005, nt=1000)
    nt = 2
    rho = oqs._fast_lindblad(g["H"], g["rho0"].copy(), g["c_ops"], e_ops=[], Nt=nt, dt=g["dt"])
    # rho0 comes from a QR factorisation whose last bits depend on the BLAS
    # build, so the operators are pinned by digest and rho0 by its diagonal
    out["gue1024"] = dict(digest_ops=digest(g["H"], *g["c_ops"]), rho0_diag=np.diag(g["rho0"]).copy(),
                          dt=g["dt"], nt=nt, rows=rho[:8, :], diag=np.diag(rho).copy(),
                          trace=np.trace(rho), fro=np.linalg.norm(rho))

    # 5. exciton correlation functions, 8 instances spanning n = 8..64
    dims = W.exciton_dims()
    want = [9, 17, 24, 33, 40, 49, 57, 65]
    idx = [int(np.nonzero(dims == n)[0][0]) for n in want]
    ex = W.exciton_batch(indices=idx, nt=40)
    cors = []
    with tempfile.TemporaryDirectory() as td:
        for i in range(len(idx)):
            cops = [np.diag(c) for c in ex["c_diag"][i]]
            cors.append(oqs._correlation_2p_1t(ex["H"][i], ex["rho_g"][i], [ex["mu"][i], ex["mu"][i]],
                                               cops, ex["dt"], ex["nt"],
                                               output=os.path.join(td, "cor.dat")))
    Nmax = max(want)
    Hp = np.zeros((len(idx), Nmax, Nmax), complex)
    Mp = np.zeros_like(Hp)
    for i, n in enumerate(want):
        Hp[i, :n, :n] = ex["H"][i]
        Mp[i, :n, :n] = ex["mu"][i]
    out["exciton"] = dict(indices=np.array(idx), dims=np.array(want), H=Hp, mu=Mp,
                          dt=ex["dt"], nt=ex["nt"], cor=np.stack(cors))

    # 6. driven instances through run() with a list Hamiltonian
    d = W.driven_batch(n_inst=2, nt=30)
    obs_all, rho_all = [], []
    for b in range(2):
        E = d["E"]

        def f(t, E=E, dt=d["dt"]):
            return E[int(round(t / dt)) - 1]
        Lk = [np.sqrt(d["gamma"][b][k]) * d["L"][b][k] for k in range(2)]
        sol = oqs.LindbladSolver([csr_matrix(d["H0"][b]), [csr_matrix(d["mu"][b]), f]],
                                 [csr_matrix(L) for L in Lk])
        r = sol.run(d["rho0"][b], dt=d["dt"], Nt=d["nt"], e_ops=[csr_matrix(d["O"][b])])
        obs_all.append(r.observables[:, 0])
        rho_all.append(r.rholist[-1].toarray())
    out["driven64"] = dict(
        H0=np.stack(d["H0"][:2]), mu=np.stack(d["mu"][:2]),
        L=np.stack([np.stack([np.sqrt(d["gamma"][b][k]) * d["L"][b][k] for k in range(2)])
                    for b in range(2)]),
        rho0=np.stack(d["rho0"][:2]), O=np.stack(d["O"][:2]), E=d["E"], dt=d["dt"], nt=d["nt"],
        observables=np.stack(obs_all), rho=np.stack(rho_all))

    # 7. correlation entry points on the JC system
    jc = W.jaynes_cummings()
    Hs, cs = csr_matrix(jc["H"]), [csr_matrix(c) for c in jc["c_ops"]]
    a = np.kron(np.diag(np.sqrt(np.arange(1, 8)), 1), np.eye(2)).astype(complex)
    sm = np.kron(np.eye(8), np.array([[0, 1], [0, 0]], complex))
    ad, sp = a.conj().T, sm.conj().T
    sol = oqs.LindbladSolver(Hs, cs)
    with tempfile.TemporaryDirectory() as td:
        fn = os.path.join(td, "cor.dat")
        c2 = sol.correlation_2op_1t(jc["rho0"], ad, a, dt=0.02, Nt=50, output=fn)
        cor_dat = open(fn).read()
    c3 = sol.correlation_3op_1t(jc["rho0"], [csr_matrix(ad), csr_matrix(a @ ad), csr_matrix(a)],
                                dt=0.02, Nt=50)
    c4 = sol.correlation_4op_1t(jc["rho0"], [csr_matrix(ad), csr_matrix(sp), csr_matrix(sm),
                                             csr_matrix(a)], dt=0.02, nt=50)
    out["corr_jc"] = dict(a=a, sm=sm, c2=c2, c3=c3, c4=c4, cor_dat=np.array(cor_dat))

    out.update(redfield_fixtures(oqs))
    out.update(heom_fixtures(oqs))
    out.update(spectral_fixtures())
    save(out)
    api_fixture()


def long_fixtures(oqs, which=("driven", "gue256", "gue1024")):
    """The dense and driven workloads at their full configured lengths.

    * ``gue256_long.npz``  ``_fast_lindblad``, GUE N=256, K=4, 10000 steps:
                           the final state in full.
    * ``gue1024_long.npz`` ``_fast_lindblad``, GUE N=1024, K=8, rank-4 rho0,
                           1000 steps: rows 0..15, the diagonal, the trace and
                           the Frobenius norm of the final state.
    * ``driven64_long.npz`` ``LindbladSolver.run`` with ``H = [H0, [mu, f]]``,
                           2 instances of the driven batch, 2000 steps: the
                           observable at every step and the final states.
    Each is written as soon as it is done (the N=1024 run takes over an hour).
    """
    if "driven" in which:
        d = W.driven_batch(n_inst=2, nt=2000)
        obs_all, rho_all = [], []
        for b in range(2):
            E = d["E"]

            def f(t, E=E, dt=d["dt"]):
                return E[int(round(t / dt)) - 1]
            Lk = [np.sqrt(d["gamma"][b][k]) * d["L"][b][k] for k in range(2)]
            sol = oqs.LindbladSolver([csr_matrix(d["H0"][b]), [csr_matrix(d["mu"][b]), f]],
                                     [csr_matrix(L) for L in Lk])
            r = sol.run(d["rho0"][b], dt=d["dt"], Nt=d["nt"], e_ops=[csr_matrix(d["O"][b])])
            obs_all.append(r.observables[:, 0])
            rho_all.append(r.rholist[-1].toarray())
        # rho0 is stored itself (its normalisation goes through a BLAS norm,
        # whose last bits differ between BLAS builds); the other inputs are
        # pinned by a digest
        save({"driven64_long": dict(digest_ops=digest(*d["H0"][:2], *d["mu"][:2], *d["O"][:2],
                                                      *[L for b in range(2) for L in d["L"][b]]),
                                    rho0=np.stack(d["rho0"][:2]), gamma=d["gamma"][:2],
                                    E=d["E"], dt=d["dt"], nt=d["nt"], observables=np.stack(obs_all),
                                    rho=np.stack(rho_all))})
    if "gue256" in which:
        g = W.gue_instance(N=256, K=4, seed=2)
        rho = oqs._fast_lindblad(g["H"], g["rho0"].copy(), g["c_ops"], e_ops=[], Nt=g["nt"], dt=g["dt"])
        save({"gue256_long": dict(digest=digest(g["H"], *g["c_ops"], g["rho0"]), dt=g["dt"], nt=g["nt"],
                                  rho=rho)})
    if "gue1024" in which:
        g = W.gue_instance(N=1024, K=8, scale=0.02, rank=4, seed=4, dt=0.005, nt=1000)
        rho = oqs._fast_lindblad(g["H"], g["rho0"].copy(), g["c_ops"], e_ops=[], Nt=g["nt"], dt=g["dt"])
        save({"gue1024_long": dict(digest_ops=digest(g["H"], *g["c_ops"]),
                                   rho0_diag=np.diag(g["rho0"]).copy(), dt=g["dt"], nt=g["nt"],
                                   rows=rho[:16, :], diag=np.diag(rho).copy(), trace=np.trace(rho),
                                   fro=np.linalg.norm(rho))})


def save(out):
    for name, arrs in out.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **arrs)
        print(name, os.path.getsize(path), "bytes", flush=True)


if __name__ == "__main__":
    if sys.argv[1:] == ["redfield"]:
        save(redfield_fixtures(load()))
    elif sys.argv[1:] == ["heom"]:
        save(heom_fixtures(load()))
    elif sys.argv[1:] == ["spectral"]:
        save(spectral_fixtures())
    elif sys.argv[1:] == ["api"]:
        api_fixture()
    elif sys.argv[1:2] == ["long"]:
        long_fixtures(load(), tuple(sys.argv[2:]) or ("driven", "gue256", "gue1024"))
    else:
        main()
