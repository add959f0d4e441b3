"""Parity at the workloads' full configured lengths.

* GUE N = 256, K = 4, 10 000 steps, and GUE N = 1024, K = 8, rank-4 rho0,
  1000 steps: every path against the reference's own ``_fast_lindblad`` run
  to the end (``tests/golden/gue256_long.npz``, ``gue1024_long.npz``).
* Driven N = 64, K = 2, 2000 steps: the reference's ``LindbladSolver.run``
  with a list Hamiltonian on two instances (``driven64_long.npz``), and the
  256-instance batch on the FP32 path against the FP64 path (pinned by that
  fixture) at full rho.
* The exciton batch, 4000 steps: instances of every padding class (and the
  N = 65 one) on every path against the complex128 oracle, which the
  reference's ``_correlation_2p_1t`` fixture pins.

Bars: 1e-12 for FP64 (1e-10 after 10 000 steps at N = 256), 1e-5 max-abs
on rho (and on C(t) relative to max |C|) for FP32, 3xTF32 and 3xBF16 (each
test prints the measured error).
"""
import hashlib
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
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300.build import build
    build()


def _fixture(name):
    path = os.path.join(GOLD, name + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated" % name)
    return np.load(path)


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.complex128).tobytes())
    return h.hexdigest()


def _report(name, err):
    print("%s max-abs error %.3e" % (name, err))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", TOL32), ("3xtf32", TOL32),
                                      ("3xbf16", TOL32)])
def test_gue256_full_length(prec, tol):
    g = _fixture("gue256_long")
    w = W.gue_instance(N=256, K=4, seed=2)
    if _digest(w["H"], *w["c_ops"], w["rho0"]) != str(g["digest"]):
        pytest.skip("numpy's generator stream differs from the fixture's")
    assert int(g["nt"]) == 10000
    sol = LindbladSolver(w["H"], w["c_ops"])
    rho = sol.evolve_fast(w["rho0"].copy(), dt=float(g["dt"]), Nt=int(g["nt"]), precision=prec)
    err = np.abs(rho - g["rho"]).max()
    _report("gue256 10000 steps " + prec, err)
    assert err < tol


@pytest.mark.parametrize("prec,tol", [("fp32", TOL32), ("3xtf32", TOL32), ("3xbf16", TOL32)])
def test_gue1024_full_length(prec, tol):
    g = _fixture("gue1024_long")
    w = W.gue_instance(N=1024, K=8, scale=0.02, rank=4, seed=4, dt=0.005, nt=1000)
    if _digest(w["H"], *w["c_ops"]) != str(g["digest_ops"]):
        pytest.skip("numpy's generator stream differs from the fixture's")
    assert np.abs(np.diag(w["rho0"]) - g["rho0_diag"]).max() < 1e-14
    assert int(g["nt"]) == 1000
    sol = LindbladSolver(w["H"], w["c_ops"])
    rho = sol.evolve_fast(w["rho0"].copy(), dt=float(g["dt"]), Nt=int(g["nt"]), precision=prec)
    err = max(np.abs(rho[:16, :] - g["rows"]).max(), np.abs(np.diag(rho) - g["diag"]).max())
    _report("gue1024 1000 steps " + prec, err)
    assert err < tol
    assert abs(np.trace(rho) - g["trace"]) < tol * 10


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32", TOL32)])
def test_driven_full_length_golden(prec, tol):
    g = _fixture("driven64_long")
    d = W.driven_batch(n_inst=2, nt=2000)
    if _digest(*d["H0"][:2], *d["mu"][:2], *d["O"][:2],
               *[L for b in range(2) for L in d["L"][b]]) != str(g["digest_ops"]):
        pytest.skip("numpy's generator stream differs from the fixture's")
    # rho0 as the reference run had it (its normalisation's last bits depend on the BLAS build)
    assert np.abs(g["rho0"] - np.stack(d["rho0"][:2])).max() < 1e-14
    assert np.array_equal(g["gamma"], d["gamma"][:2])
    dt, nt = float(g["dt"]), int(g["nt"])
    assert nt == 2000
    for b in range(2):
        E = g["E"]
        Lk = [np.sqrt(d["gamma"][b][k]) * d["L"][b][k] for k in range(2)]
        sol = LindbladSolver([csr_matrix(d["H0"][b]), [csr_matrix(d["mu"][b]),
                              lambda t, E=E: E[int(round(t / dt)) - 1]]], [csr_matrix(L) for L in Lk])
        r = sol.run(g["rho0"][b], dt=dt, Nt=nt, e_ops=[csr_matrix(d["O"][b])], precision=prec,
                    rholist_format="dense", nout=nt)
        err_obs = np.abs(r.observables[:, 0] - g["observables"][b][nt - 1::nt]).max()
        err_rho = np.abs(r.rholist[-1] - g["rho"][b]).max()
        full = sol.run(g["rho0"][b], dt=dt, Nt=nt, e_ops=[csr_matrix(d["O"][b])], precision=prec,
                       store_states=False)
        err_all = np.abs(full.observables[:, 0] - g["observables"][b]).max()
        _report("driven64 2000 steps %s instance %d <O>" % (prec, b), err_all)
        _report("driven64 2000 steps %s instance %d rho" % (prec, b), err_rho)
        assert err_rho < tol
        assert max(err_obs, err_all) < tol * 10  # <O> of a GUE observable sums N terms of rho


def test_driven_batch_256_full_length_fp32_vs_fp64():
    d = W.driven_batch(n_inst=256, nt=2000)
    cops = [[np.sqrt(d["gamma"][b][k]) * d["L"][b][k] for k in range(2)] for b in range(256)]
    args = (d["H0"], cops, d["rho0"], d["dt"], d["nt"])
    kw = dict(e_ops=[[o] for o in d["O"]], obs_t0=False, drive_ops=[[m] for m in d["mu"]],
              drive=d["E"][None, :])
    r64 = propagate_batch(*args, precision="fp64", **kw)
    r32 = propagate_batch(*args, precision="fp32", **kw)
    err_rho = max(np.abs(a - b).max() for a, b in zip(r32["rho"], r64["rho"]))
    err_obs = np.abs(r32["observables"] - r64["observables"]).max()
    _report("driven256 2000 steps fp32 rho", err_rho)
    _report("driven256 2000 steps fp32 <O>", err_obs)
    assert err_rho < TOL32
    assert err_obs < TOL32 * 10  # <O> of a GUE observable sums N terms of rho


@pytest.mark.parametrize("prec", ["fp32", "3xtf32", "3xbf16"])
def test_exciton_full_length_vs_oracle(prec):
    dims = W.exciton_dims()
    want = [9, 16, 17, 32, 33, 48, 49, 64, 65]  # both ends of every padding class, and the border
    idx = [int(np.nonzero(dims == n)[0][0]) for n in want]
    ex = W.exciton_batch(indices=idx)
    assert ex["nt"] == 4000
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    seeds = [m @ r for m, r in zip(ex["mu"], ex["rho_g"])]
    res = propagate_batch(ex["H"], cops, seeds, ex["dt"], ex["nt"], e_ops=[[m] for m in ex["mu"]],
                          obs_t0=False, precision=prec)
    worst_c = worst_r = 0.0
    for k in range(len(idx)):
        ref, rho = O.propagate_diag_correlation(ex["H"][k], ex["mu"][k], ex["rho_g"][k], ex["c_diag"][k],
                                                ex["dt"], ex["nt"], return_rho=True)
        worst_c = max(worst_c, np.abs(res["observables"][k, :, 0] - ref).max() / np.abs(ref).max())
        worst_r = max(worst_r, np.abs(res["rho"][k] - rho).max())
    _report("exciton 4000 steps %s C(t) relative" % prec, worst_c)
    _report("exciton 4000 steps %s rho" % prec, worst_r)
    assert worst_c < TOL32
    assert worst_r < TOL32


def test_exciton_correlation_batch_full_length_fp64_vs_oracle():
    dims = W.exciton_dims()
    idx = [int(np.nonzero(dims == n)[0][0]) for n in (9, 40, 65)]
    ex = W.exciton_batch(indices=idx)
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    C = correlation_batch(ex["H"], cops, ex["rho_g"], ex["mu"], ex["mu"], ex["dt"], ex["nt"],
                          precision="fp64")
    for k in range(len(idx)):
        ref = O.propagate_diag_correlation(ex["H"][k], ex["mu"][k], ex["rho_g"][k], ex["c_diag"][k],
                                           ex["dt"], ex["nt"])
        assert np.abs(C[k] - ref).max() < 1e-11
