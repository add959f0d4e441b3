"""GPU parity: the CUDA propagator against the reference's own outputs
(tests/golden, produced by running binggu56/pyqed) and against the oracle on
seeded inputs.

Tolerances: 1e-12 max-abs for the FP64 path; 1e-5 max-abs on rho(t) (and on
C(t) relative to max|C|) for the FP32 and split-precision paths.
"""
import os

import numpy as np
import pytest
from scipy.sparse import csr_matrix

from oracle import lindblad_oracle as O
from pyqed_gb300 import LindbladSolver, correlation_batch, propagate_batch
from pyqed_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5
# 3xBF16 holds operands to ~2^-17 relative; with the diagonal of A applied in
# FP32 on the tensor-core kernel it meets the same bar (measured on the dense
# GEMM-schedule cases: 1e-8 .. 1e-7)
TOLBF = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300.build import build
    build()


# ---- golden fixtures (reference outputs) ----------------------------------------

@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32)])
def test_jc16_run_golden(golden, prec, tol):
    g = golden("jc16")
    sol = LindbladSolver(csr_matrix(g["H"]), [csr_matrix(c) for c in g["c_ops"]])
    r = sol.run(g["rho0"], dt=float(g["dt"]), Nt=int(g["nt"]),
                e_ops=[csr_matrix(e) for e in g["e_ops"]], precision=prec)
    assert r.observables.shape == (2001, 2)
    assert len(r.rholist) == 2000 and r.times.shape == (2001,)
    assert np.abs(r.observables - g["observables"]).max() < tol
    for k, s in zip(g["state_index"], g["states"]):
        assert np.abs(r.rholist[k].toarray() - s).max() < tol


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32)])
def test_gue64_evolve_fast_golden(golden, prec, tol):
    g = golden("gue64")
    sol = LindbladSolver(g["H"], list(g["c_ops"]))
    rho0 = g["rho0"].copy()
    rho = sol.evolve_fast(rho0, dt=float(g["dt"]), Nt=int(g["nt"]), e_ops=[], precision=prec)
    assert np.abs(rho - g["rho"]).max() < tol
    assert np.abs(rho0 - g["rho"]).max() < tol  # the reference overwrites rho0 too


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32)])
def test_exciton_correlation_golden(golden, prec, tol):
    g = golden("exciton")
    ex = W.exciton_batch(indices=[int(i) for i in g["indices"]], nt=int(g["nt"]))
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    C = correlation_batch(ex["H"], cops, ex["rho_g"], ex["mu"], ex["mu"], ex["dt"], ex["nt"],
                          precision=prec)
    ref = g["cor"]
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err < tol, err


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32)])
def test_driven_run_golden(golden, prec, tol):
    g = golden("driven64")
    dt, nt = float(g["dt"]), int(g["nt"])
    for b in range(2):
        E = g["E"]
        sol = LindbladSolver([csr_matrix(g["H0"][b]), [csr_matrix(g["mu"][b]),
                              lambda t, E=E: E[int(round(t / dt)) - 1]]],
                             [csr_matrix(L) for L in g["L"][b]])
        r = sol.run(g["rho0"][b], dt=dt, Nt=nt, e_ops=[csr_matrix(g["O"][b])], precision=prec)
        assert r.observables.shape == (nt, 1)
        assert np.abs(r.observables[:, 0] - g["observables"][b]).max() < tol
        assert np.abs(r.rholist[-1].toarray() - g["rho"][b]).max() < tol


def test_run_nout_keeps_every_nth_step(golden):
    # the reference's Result.times for nout (pyqed/mol.py:113); rows and states
    # are those of the full run at the kept steps
    g = golden("jc16")
    sol = LindbladSolver(csr_matrix(g["H"]), [csr_matrix(c) for c in g["c_ops"]])
    e_ops = [csr_matrix(e) for e in g["e_ops"]]
    r = sol.run(g["rho0"], dt=float(g["dt"]), Nt=int(g["nt"]), e_ops=e_ops, nout=5)
    assert r.times.shape == (int(g["nt"]) // 5 + 1,) and r.nout == 5
    assert r.observables.shape == r.times.shape + (2,)
    assert np.abs(r.observables - g["observables"][::5]).max() < TOL64
    assert len(r.rholist) == int(g["nt"]) // 5
    for k, st in zip(g["state_index"], g["states"]):
        if (k + 1) % 5 == 0:
            assert np.abs(r.rholist[(k + 1) // 5 - 1].toarray() - st).max() < TOL64
    d = golden("driven64")
    dt, nt = float(d["dt"]), int(d["nt"])
    E = d["E"]
    sol = LindbladSolver([csr_matrix(d["H0"][0]), [csr_matrix(d["mu"][0]),
                          lambda t, E=E: E[int(round(t / dt)) - 1]]],
                         [csr_matrix(L) for L in d["L"][0]])
    r = sol.run(d["rho0"][0], dt=dt, Nt=nt, e_ops=[csr_matrix(d["O"][0])], nout=3)
    assert r.observables.shape == (nt // 3, 1)
    assert np.abs(r.observables[:, 0] - d["observables"][0][2::3]).max() < TOL64
    assert len(r.rholist) == nt // 3
    assert np.abs(r.rholist[-1].toarray() - d["rho"][0]).max() < TOL64  # 30 = 10 x 3


def test_correlation_entry_points_golden(golden, tmp_path):
    g = golden("corr_jc")
    jc = W.jaynes_cummings()
    a, sm = g["a"], g["sm"]
    ad, sp = a.conj().T, sm.conj().T
    sol = LindbladSolver(jc["H"], jc["c_ops"])
    fn = str(tmp_path / "cor.dat")
    c2 = sol.correlation_2op_1t(jc["rho0"], ad, a, dt=0.02, Nt=50, output=fn)
    assert np.abs(c2 - g["c2"]).max() < TOL64
    # same file layout as the reference: "t C(t) " per line
    ours = [l.split() for l in open(fn).read().splitlines()]
    theirs = [l.split() for l in str(g["cor_dat"]).splitlines()]
    assert len(ours) == len(theirs) == 50
    assert all(o[0] == t[0] for o, t in zip(ours, theirs))
    assert np.allclose([complex(o[1]) for o in ours], [complex(t[1]) for t in theirs],
                       atol=1e-12, rtol=0)
    c3 = sol.correlation_3op_1t(jc["rho0"], [ad, a @ ad, a], dt=0.02, Nt=50)
    assert c3.shape == (51,) and np.abs(c3 - g["c3"]).max() < TOL64
    c4 = sol.correlation_4op_1t(jc["rho0"], [ad, sp, sm, a], 0.02, 50)
    assert np.abs(c4 - g["c4"]).max() < TOL64


# ---- seeded cases against the oracle ----------------------------------------------

def _random_instance(rng, N, K):
    H = W.gue_matrix(rng, N)
    cops = [(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.05 / np.sqrt(N)
            for _ in range(K)]
    psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    psi /= np.linalg.norm(psi)
    O_ = W.gue_matrix(rng, N)
    return H, cops, np.outer(psi, psi.conj()), O_


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32)])
def test_uneven_batch_dense_cops_vs_oracle(prec, tol):
    rng = np.random.default_rng(11)
    dims = [1, 3, 5, 17, 33, 64, 65, 2] + ([88] if prec != "fp64" else [68])
    insts = [_random_instance(rng, N, 2) for N in dims]
    nt, dt = 12, 0.05
    res = propagate_batch([i[0] for i in insts], [i[1] for i in insts], [i[2] for i in insts],
                          dt, nt, e_ops=[[i[3]] for i in insts], obs_t0=True, precision=prec)
    for b, (H, cops, rho0, O_) in enumerate(insts):
        obs, states = O.lindblad(H, rho0, cops, [O_], Nt=nt, dt=dt)
        assert np.abs(res["rho"][b] - states[-1]).max() < tol, (b, dims[b])
        assert np.abs(res["observables"][b, :, 0] - obs[:, 0]).max() < tol * max(1, dims[b] ** 0.5)


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32)])
def test_uneven_batch_diag_cops_nonhermitian_vs_oracle(prec, tol):
    ex = W.exciton_batch(indices=list(range(24)), nt=30)
    C = correlation_batch(ex["H"], [[np.diag(c) for c in cd] for cd in ex["c_diag"]],
                          ex["rho_g"], ex["mu"], ex["mu"], ex["dt"], ex["nt"], precision=prec)
    for i in range(24):
        ref = O.propagate_diag_correlation(ex["H"][i], ex["mu"][i], ex["rho_g"][i],
                                           ex["c_diag"][i], ex["dt"], ex["nt"])
        assert np.abs(C[i] - ref).max() / np.abs(ref).max() < tol


def test_no_cops_no_eops_and_zero_steps():
    rng = np.random.default_rng(3)
    H, _, rho0, _ = _random_instance(rng, 6, 0)
    sol = LindbladSolver(H, None)
    r = sol.run(rho0, dt=0.1, Nt=0, precision="fp64")
    assert r.observables.shape == (1, 0) and r.rholist == []
    r = sol.run(rho0, dt=0.1, Nt=5, precision="fp64", rholist_format="dense")
    _, states = O.lindblad(H, rho0, [], [], Nt=5, dt=0.1)
    assert np.abs(r.rholist[-1] - states[-1]).max() < TOL64


def test_nonfinite_state_is_reported():
    from pyqed_gb300._capi import LindbladError
    rng = np.random.default_rng(4)
    H, cops, rho0, _ = _random_instance(rng, 8, 1)
    rho0 = rho0.copy()
    rho0[2, 3] = np.nan
    sol = LindbladSolver(H, cops)
    with pytest.raises(LindbladError, match="non-finite"):
        sol.run(rho0, dt=0.1, Nt=3, precision="fp32")


def test_correlation_two_time_intended_semantics():
    jc = W.jaynes_cummings()
    a = np.kron(np.diag(np.sqrt(np.arange(1, 8)), 1), np.eye(2)).astype(complex)
    ad = a.conj().T
    sol = LindbladSolver(jc["H"], jc["c_ops"])
    M = sol.correlation_3op_2t(jc["rho0"], [ad, a @ ad, a], 0.02, 4, 6)
    assert M.shape == (4, 7)
    _, states = O.lindblad(jc["H"], jc["rho0"], jc["c_ops"], [], Nt=4, dt=0.02)
    for k in range(4):
        ref = O.correlation_3op_1t(jc["H"], states[k], [ad, a @ ad, a], jc["c_ops"], 0.02, 6)
        assert np.abs(M[k] - ref).max() < TOL64


# ---- split-precision tensor-core path --------------------------------------------

# 3xBF16 keeps the diagonal of A out of the split products (applied in FP32),
# so on the exciton family (couplings small beside the energy spread) it meets
# the FP32 bar.
@pytest.mark.parametrize("prec,tol", [("3xtf32", TOL32), ("3xbf16", TOL32)])
def test_split_exciton_golden(golden, prec, tol):
    g = golden("exciton")
    ex = W.exciton_batch(indices=[int(i) for i in g["indices"]], nt=int(g["nt"]))
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    C = correlation_batch(ex["H"], cops, ex["rho_g"], ex["mu"], ex["mu"], ex["dt"], ex["nt"],
                          precision=prec)
    ref = g["cor"]
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err < tol, err


@pytest.mark.parametrize("prec,tol", [("3xtf32", TOL32), ("3xbf16", TOL32)])
def test_split_uneven_batch_vs_oracle(prec, tol):
    # every padded size class of the tensor-core kernel (16/32/48/64) plus N=65
    idx = list(range(40))
    ex = W.exciton_batch(indices=idx, nt=25)
    C = correlation_batch(ex["H"], [[np.diag(c) for c in cd] for cd in ex["c_diag"]],
                          ex["rho_g"], ex["mu"], ex["mu"], ex["dt"], ex["nt"], precision=prec)
    for i in range(len(idx)):
        ref = O.propagate_diag_correlation(ex["H"][i], ex["mu"][i], ex["rho_g"][i],
                                           ex["c_diag"][i], ex["dt"], ex["nt"])
        assert np.abs(C[i] - ref).max() / np.abs(ref).max() < tol, (i, ex["dims"][i])


def test_split_complex_dissipator_and_states():
    """Complex diagonal collapse operators (D complex), no observables' t0 row,
    states stored every 2 steps, Hermitian and non-Hermitian initial states."""
    rng = np.random.default_rng(21)
    dims = [5, 16, 17, 40, 64, 70]
    H, cops, rho0 = [], [], []
    for N in dims:
        H.append(W.gue_matrix(rng, N))
        cops.append([np.diag((rng.standard_normal(N) + 1j * rng.standard_normal(N)) * 0.1)
                     for _ in range(3)])
        r = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        rho0.append(r / np.linalg.norm(r))
    res = propagate_batch(H, cops, rho0, 0.02, 10, e_ops=[[h] for h in H], obs_t0=True,
                          store_every=2, precision="3xtf32")
    for b, N in enumerate(dims):
        obs, states = O.lindblad(H[b], rho0[b], cops[b], [H[b]], Nt=10, dt=0.02)
        assert np.abs(res["rho"][b] - states[-1]).max() < TOL32
        assert np.abs(res["observables"][b, :, 0] - obs[:, 0]).max() < TOL32 * N
        for k in range(5):
            assert np.abs(res["states"][b][k] - states[2 * k + 1]).max() < TOL32


@pytest.mark.parametrize("prec,tol", [("3xtf32", TOL32), ("3xbf16", TOLBF)])
@pytest.mark.parametrize("kind", ["dephasing", "complex"])
def test_split_border_n65_vs_oracle(prec, tol, kind):
    """N = 65 runs on the tensor cores as a 64 x 64 block plus a SIMT border
    row and column: dense GUE H (every border coupling non-zero), diagonal
    collapse operators (pure dephasing, or complex with off-diagonal D),
    observables with a t0 row and stored states, beside N = 64 and N = 16."""
    rng = np.random.default_rng(31)
    dims = [65, 64, 65, 16]
    H, cops, rho0, eops = [], [], [], []
    for N in dims:
        H.append(W.gue_matrix(rng, N))
        if kind == "dephasing":
            cops.append([np.diag(np.sqrt(0.05) * (np.arange(N) == k)).astype(complex) for k in range(0, N, 7)])
        else:
            cops.append([np.diag((rng.standard_normal(N) + 1j * rng.standard_normal(N)) * 0.1) for _ in range(2)])
        r = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        rho0.append(r / np.linalg.norm(r))
        eops.append([H[-1], W.gue_matrix(rng, N)])
    nt, dt = 16, 0.02
    res = propagate_batch(H, cops, rho0, dt, nt, e_ops=eops, obs_t0=True, store_every=4, precision=prec)
    for b, N in enumerate(dims):
        obs, states = O.lindblad(H[b], rho0[b], cops[b], eops[b], Nt=nt, dt=dt)
        assert np.abs(res["rho"][b] - states[-1]).max() < tol, (b, N)
        assert np.abs(res["observables"][b] - obs).max() < tol * N, (b, N)
        for k in range(nt // 4):
            assert np.abs(res["states"][b][k] - states[4 * k + 3]).max() < tol, (b, N, k)


def test_split_border_driven_n65_takes_the_fp32_kernel():
    """A driven N = 65 instance keeps the FP32 wide kernel beside tensor-core ones."""
    rng = np.random.default_rng(32)
    dims = [65, 40]
    E = W.gp_pulse(12, 0.02, seed=3, amp=0.3)
    H0 = [W.gue_matrix(rng, N) for N in dims]
    mu = [W.gue_matrix(rng, N) for N in dims]
    cops = [[np.diag(np.sqrt(0.02) * (np.arange(N) == k)) for k in range(3)] for N in dims]
    rho0 = []
    for N in dims:
        psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        psi /= np.linalg.norm(psi)
        rho0.append(np.outer(psi, psi.conj()))
    res = propagate_batch(H0, cops, rho0, 0.02, 12, e_ops=[[m] for m in mu], obs_t0=False,
                          precision="3xtf32", drive_ops=[[m] for m in mu], drive=E[None, :])
    for b in range(len(dims)):
        obs, states = O.lindblad_driven([H0[b], [mu[b], E]], rho0[b], cops[b], [mu[b]], Nt=12, dt=0.02)
        assert np.abs(res["rho"][b] - states[-1]).max() < TOL32
        assert np.abs(res["observables"][b, :, 0] - obs[:, 0]).max() < TOL32 * 10


@pytest.mark.parametrize("prec,tol", [("3xtf32", TOL32), ("3xbf16", TOLBF)])
def test_split_driven_diag_vs_oracle(prec, tol):
    """Driven H(t): the A operand (and, for BF16, its diagonal kept in FP32)
    is rebuilt every step."""
    rng = np.random.default_rng(22)
    dims = [8, 33, 64]
    E = W.gp_pulse(15, 0.02, seed=9, amp=0.3)
    H0 = [W.gue_matrix(rng, N) for N in dims]
    mu = [W.gue_matrix(rng, N) for N in dims]
    cops = [[np.diag(np.sqrt(0.02) * (np.arange(N) == k)) for k in range(2)] for N in dims]
    rho0 = []
    for N in dims:
        psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        psi /= np.linalg.norm(psi)
        rho0.append(np.outer(psi, psi.conj()))
    res = propagate_batch(H0, cops, rho0, 0.02, 15, e_ops=[[m] for m in mu], obs_t0=False,
                          precision=prec, drive_ops=[[m] for m in mu], drive=E[None, :])
    for b in range(len(dims)):
        obs, states = O.lindblad_driven([H0[b], [mu[b], E]], rho0[b], cops[b], [mu[b]],
                                        Nt=15, dt=0.02)
        assert np.abs(res["rho"][b] - states[-1]).max() < tol
        assert np.abs(res["observables"][b, :, 0] - obs[:, 0]).max() < tol * 10


def test_split_solver_run_matches_fp64():
    jc = W.jaynes_cummings(nt=200)
    sol = LindbladSolver(jc["H"], jc["c_ops"])
    r64 = sol.run(jc["rho0"], dt=jc["dt"], Nt=200, e_ops=jc["e_ops"], precision="fp64")
    r32 = sol.run(jc["rho0"], dt=jc["dt"], Nt=200, e_ops=jc["e_ops"], precision="3xtf32")
    assert np.abs(r32.observables - r64.observables).max() < TOL32


# ---- grid-wide GEMM schedule (large N) ----------------------------------------------

def _digest(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.complex128).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32), ("3xtf32", TOL32),
                                      ("3xbf16", TOLBF)])
def test_gue256_golden(golden, prec, tol):
    g = golden("gue256")
    w = W.gue_instance(N=256, K=4, seed=2)
    if _digest(w["H"], *w["c_ops"], w["rho0"]) != str(g["digest"]):
        pytest.skip("numpy's generator stream differs from the fixture's")
    sol = LindbladSolver(w["H"], w["c_ops"])
    rho = sol.evolve_fast(w["rho0"].copy(), dt=float(g["dt"]), Nt=int(g["nt"]), precision=prec)
    assert np.abs(rho - g["rho"]).max() < tol


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32), ("3xtf32", TOL32),
                                      ("3xbf16", TOLBF)])
def test_gue1024_golden(golden, prec, tol):
    g = golden("gue1024")
    w = W.gue_instance(N=1024, K=8, scale=0.02, rank=4, seed=4, dt=0.005, nt=1000)
    if _digest(w["H"], *w["c_ops"]) != str(g["digest_ops"]):
        pytest.skip("numpy's generator stream differs from the fixture's")
    assert np.abs(np.diag(w["rho0"]) - g["rho0_diag"]).max() < 1e-14
    sol = LindbladSolver(w["H"], w["c_ops"])
    rho = sol.evolve_fast(w["rho0"].copy(), dt=float(g["dt"]), Nt=int(g["nt"]), precision=prec)
    assert np.abs(rho[:8, :] - g["rows"]).max() < tol
    assert np.abs(np.diag(rho) - g["diag"]).max() < tol
    assert abs(np.trace(rho) - g["trace"]) < tol * 10


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32), ("3xtf32", TOL32),
                                      ("3xbf16", TOLBF)])
@pytest.mark.parametrize("kind", ["dense", "diag"])
def test_gemm_schedule_vs_oracle(prec, tol, kind):
    rng = np.random.default_rng(31)
    dims = [3, 20, 33]
    H, cops, rho0, eops = [], [], [], []
    for N in dims:
        h, c, r, o = _random_instance(rng, N, 3)
        if kind == "diag":
            c = [np.diag((rng.standard_normal(N) + 1j * rng.standard_normal(N)) * 0.1) for _ in range(3)]
        H.append(h), cops.append(c), rho0.append(r), eops.append([o, h])
    res = propagate_batch(H, cops, rho0, 0.03, 9, e_ops=eops, obs_t0=True, store_every=3,
                          precision=prec, schedule="gemm")
    assert res["info"]["schedule"] == "gemm"
    for b, N in enumerate(dims):
        obs, states = O.lindblad(H[b], rho0[b], cops[b], eops[b], Nt=9, dt=0.03)
        assert np.abs(res["rho"][b] - states[-1]).max() < tol
        assert np.abs(res["observables"][b] - obs).max() < tol * N
        for k in range(3):
            assert np.abs(res["states"][b][k] - states[3 * k + 2]).max() < tol


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32), ("3xtf32", TOL32),
                                      ("3xbf16", TOLBF)])
def test_gemm_schedule_driven_vs_oracle(prec, tol):
    rng = np.random.default_rng(32)
    dims = [12, 100]
    E = W.gp_pulse(8, 0.02, seed=3, amp=0.4)
    H0 = [W.gue_matrix(rng, N) for N in dims]
    mu = [W.gue_matrix(rng, N) for N in dims]
    cops = [[(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.02 for _ in range(2)]
            for N in dims]
    rho0 = [np.eye(N, dtype=complex) / N for N in dims]
    res = propagate_batch(H0, cops, rho0, 0.02, 8, e_ops=[[m] for m in mu], obs_t0=False,
                          precision=prec, drive_ops=[[m] for m in mu], drive=E[None, :])
    assert res["info"]["schedule"] == "gemm"  # N = 100 exceeds the CTA kernels
    for b in range(2):
        obs, states = O.lindblad_driven([H0[b], [mu[b], E]], rho0[b], cops[b], [mu[b]], Nt=8, dt=0.02)
        assert np.abs(res["rho"][b] - states[-1]).max() < tol
        assert np.abs(res["observables"][b, :, 0] - obs[:, 0]).max() < tol * 10


def test_gemm_tuning_options_change_only_the_schedule():
    """The GEMM schedule's tuning options (steps per captured CUDA graph, the
    split-K cap and waves) reschedule the same arithmetic: the results agree
    with the default schedule within the precision's tolerance and with the
    oracle."""
    from pyqed_gb300.batch import prepare_batch
    from pyqed_gb300.engine import Propagator
    rng = np.random.default_rng(35)
    N, nt, dt = 130, 40, 0.01
    H, cops, rho0, O_ = _random_instance(rng, N, 3)
    bi = prepare_batch([H], [cops], [rho0], [[O_]])
    _, states = O.lindblad(H, rho0, cops, [O_], Nt=nt, dt=dt)
    for prec, tol in (("fp32", TOL32), ("3xtf32", TOL32)):
        out = {}
        for opts in ({}, {"graph_steps": 8}, {"gemm_ksplit": 4}, {"gemm_ksplit": 1, "gemm_waves": 2},
                     {"graph_steps": 32, "gemm_ksplit": 8}):
            if prec == "fp32" and set(opts) - {"graph_steps"}:
                continue
            prop = Propagator(bi.dims, nt=nt, dt=dt, n_cops=bi.n_cops, cops_kind=bi.cops_kind, n_eops=1,
                              precision=prec, schedule="gemm")
            try:
                for k, v in opts.items():
                    prop.set_option(k, v)
                prop.set_operators(bi.H, bi.cops, bi.eops, bi.dops)
                o = prop.alloc_outputs(want_obs=True, want_rho=True)
                prop.propagate_device(prop.to_device(bi.rho0), None, o)
                prop.check_errors()
                out[tuple(sorted(opts.items()))] = prop.unpack_rho(o[1])[0]
            finally:
                prop.close()
        for k, r in out.items():
            assert np.abs(r - states[-1]).max() < tol, (prec, k)
            assert np.abs(r - out[()]).max() < tol, (prec, k)


@pytest.mark.parametrize("prec", ["3xtf32", "3xbf16"])
@pytest.mark.parametrize("N,K,kind", [(100, 3, "dense"), (128, 0, "none"), (129, 1, "dense"),
                                      (160, 2, "dense"), (200, 2, "diag"), (256, 4, "dense"),
                                      (250, 5, "dense")])
def test_gemm_persistent_kernel_vs_oracle(prec, N, K, kind):
    """The persistent split-precision kernel (one launch, clusters of 4 CTAs,
    split-K partials summed through distributed shared memory) at both padded
    sizes (NP = 128, 256) and every G1 split (K = 1: 4-way, 2: 2-way, 3 and 4:
    one product per CTA, 5: two rounds), no collapse operators, diagonal ones;
    observables with a t0 row, states stored every 3 steps: against the
    complex128 oracle, and against the graph-replayed kernels of the same
    precision (option gemm_persist = 0)."""
    from pyqed_gb300.batch import prepare_batch
    from pyqed_gb300.engine import Propagator
    rng = np.random.default_rng(100 + N + K)
    H, cops, rho0, O_ = _random_instance(rng, N, K)
    if kind == "diag":
        cops = [np.diag((rng.standard_normal(N) + 1j * rng.standard_normal(N)) * 0.1) for _ in range(K)]
    nt, dt = 9, 0.02
    obs, states = O.lindblad(H, rho0, cops, [O_, H], Nt=nt, dt=dt)
    bi = prepare_batch([H], [cops], [rho0], [[O_, H]])
    tol = TOL32 if prec == "3xtf32" else TOLBF
    out = {}
    for persist in (1, 0):
        prop = Propagator(bi.dims, nt=nt, dt=dt, n_cops=bi.n_cops, cops_kind=bi.cops_kind, n_eops=2,
                          precision=prec, schedule="gemm", store_every=3, obs_t0=True)
        try:
            prop.set_option("gemm_persist", persist)
            prop.set_operators(bi.H, bi.cops, bi.eops, bi.dops)
            assert prop.info()["persistent_instances"] == persist
            o = prop.alloc_outputs(want_obs=True, want_rho=True, want_states=True)
            prop.propagate_device(prop.to_device(bi.rho0), None, o)
            prop.check_errors()
            out[persist] = (prop.unpack_rho(o[1])[0], prop.unpack_obs(o[0])[0],
                            prop.unpack_states(o[2])[0])
        finally:
            prop.close()
    for persist, (rho, ob, st) in out.items():
        assert np.abs(rho - states[-1]).max() < tol, persist
        assert np.abs(ob - obs).max() < tol * N, persist
        for k in range(nt // 3):
            assert np.abs(st[k] - states[3 * k + 2]).max() < tol, (persist, k)
    assert np.abs(out[1][0] - out[0][0]).max() < tol


def test_gemm_persistent_kernel_sixteen_observables_three_g1_rounds():
    """The persistent kernel at its limits: 16 observables (every partial
    slot), K = 9 dense collapse operators (three rounds of G1 products through
    the one receive buffer), every step stored, against the oracle."""
    from pyqed_gb300.batch import prepare_batch
    from pyqed_gb300.engine import Propagator
    rng = np.random.default_rng(77)
    N, K, nt, dt = 192, 9, 5, 0.02
    H, cops, rho0, _ = _random_instance(rng, N, K)
    eops = [W.gue_matrix(rng, N) for _ in range(16)]
    obs, states = O.lindblad(H, rho0, cops, eops, Nt=nt, dt=dt)
    bi = prepare_batch([H], [cops], [rho0], [eops])
    prop = Propagator(bi.dims, nt=nt, dt=dt, n_cops=bi.n_cops, cops_kind=bi.cops_kind, n_eops=16,
                      precision="3xtf32", schedule="gemm", store_every=1, obs_t0=True)
    try:
        prop.set_operators(bi.H, bi.cops, bi.eops, bi.dops)
        assert prop.info()["persistent_instances"] == 1
        o = prop.alloc_outputs(want_obs=True, want_rho=True, want_states=True)
        prop.propagate_device(prop.to_device(bi.rho0), None, o)
        prop.check_errors()
        rho, ob, st = prop.unpack_rho(o[1])[0], prop.unpack_obs(o[0])[0], prop.unpack_states(o[2])[0]
    finally:
        prop.close()
    assert np.abs(rho - states[-1]).max() < TOL32
    assert np.abs(ob - obs).max() < TOL32 * N
    for k in range(nt):
        assert np.abs(st[k] - states[k]).max() < TOL32  # (states[k]: after step k + 1)


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32), ("3xtf32", TOL32)])
def test_gemm_schedule_graph_replay_vs_oracle(prec, tol):
    """45 steps: two replays of a captured 16-step CUDA graph and one of a
    13-step one, with a drive term, stored states and the t0 observable row
    (all step-dependent outputs resolved from the device step counter)."""
    rng = np.random.default_rng(33)
    N, nt, dt = 100, 45, 0.01
    E = W.gp_pulse(nt, dt, seed=5, amp=0.3)
    H0, mu = W.gue_matrix(rng, N), W.gue_matrix(rng, N)
    cops = [(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.02 for _ in range(2)]
    rho0 = np.eye(N, dtype=complex) / N
    res = propagate_batch([H0], [cops], [rho0], dt, nt, e_ops=[[mu]], obs_t0=True, store_every=7,
                          precision=prec, schedule="gemm", drive_ops=[[mu]], drive=E[None, :])
    assert res["info"]["schedule"] == "gemm"
    obs, states = O.lindblad_driven([H0, [mu, E]], rho0, cops, [mu], Nt=nt, dt=dt)
    assert np.abs(res["rho"][0] - states[-1]).max() < tol
    for k in range(nt // 7):
        assert np.abs(res["states"][0][k] - states[7 * k + 6]).max() < tol
    ref_rows = np.concatenate([[[np.trace(mu @ rho0)]], obs], axis=0)
    assert np.abs(res["observables"][0] - ref_rows).max() < tol * 10


def test_bounded_wait_timeout_is_reported_and_context_survives():
    """Error path of the tensor-core kernel's bounded waits: with the test hook
    the first MMA commit is never issued, the wait gives up after 4096 polls,
    every instance reports LGB_ERR_TIMEOUT (5), and the context keeps working."""
    from pyqed_gb300.engine import Propagator
    from pyqed_gb300.batch import prepare_batch
    import torch
    ex = W.exciton_batch(n_inst=40, nt=20)
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    seeds = [m @ r for m, r in zip(ex["mu"], ex["rho_g"])]
    bi = prepare_batch(ex["H"], cops, seeds, [[m] for m in ex["mu"]])
    dims = bi.dims
    tc = dims <= 64

    def run(stall):
        prop = Propagator(bi.dims, nt=20, dt=ex["dt"], n_cops=bi.n_cops, cops_kind=bi.cops_kind,
                          n_eops=1, precision="3xtf32")
        try:
            prop.set_option("test_stall", stall)
            prop.set_operators(bi.H, bi.cops, bi.eops)
            out = prop.alloc_outputs(want_obs=True, want_rho=True)
            prop.propagate_device(prop.to_device(bi.rho0), None, out)
            torch.cuda.synchronize()
            return prop.errors(), prop.unpack_obs(out[0])
        finally:
            prop.close()
    err, _ = run(1)
    assert np.all(err[tc] == 5) and np.all(err[~tc] == 0)
    err, obs = run(0)
    assert np.all(err == 0)
    b = int(np.argmax(tc))
    ref = O.propagate_diag_correlation(ex["H"][b], ex["mu"][b], ex["rho_g"][b], ex["c_diag"][b],
                                       ex["dt"], 20)
    assert np.abs(obs[b, :, 0] - ref).max() < 1e-5 * np.abs(ref).max()
