"""The per-step FP64 state check (``LGB_OPT_CHECK``; ``check=`` on the
Python entry points) on every schedule: the trace drift and hermiticity
deviation it reports stay tiny on correct propagations, trace-zero
correlation seeds are checked for their trace only, results are unchanged
by the check, and a tolerance below the propagation's own rounding flags
the instances (``LGB_ERR_CHECK``) without stopping them."""
import warnings

import numpy as np
import pytest
from scipy.sparse import csr_matrix

from oracle import lindblad_oracle as O
from pyqed_gb300 import LindbladSolver, propagate_batch
from pyqed_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300.build import build
    build()


def _hermitian_batch(dims, K, kind, seed=3):
    rng = np.random.default_rng(seed)
    H, cops, rho0 = [], [], []
    for N in dims:
        H.append(W.gue_matrix(rng, N))
        if kind == "diag":
            cops.append([np.diag((rng.standard_normal(N) + 1j * rng.standard_normal(N)) * 0.1)
                         for _ in range(K)])
        else:
            cops.append([(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.05 / np.sqrt(N)
                         for _ in range(K)])
        psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        psi /= np.linalg.norm(psi)
        rho0.append(np.outer(psi, psi.conj()))
    return H, cops, rho0


@pytest.mark.parametrize("prec,schedule,kind,dims,bound", [
    ("fp64", "auto", "dense", [5, 24, 60], 1e-12),
    ("fp32", "auto", "dense", [5, 24, 60, 80], 1e-5),
    ("3xtf32", "auto", "diag", [9, 30, 64, 65], 1e-5),
    ("3xbf16", "auto", "diag", [9, 30, 48, 64, 65], 1e-4),
    ("fp64", "gemm", "dense", [40], 1e-12),
    ("fp32", "gemm", "dense", [40], 1e-5),
    ("3xtf32", "gemm", "dense", [130], 1e-5),
])
def test_check_reports_small_deviations_and_leaves_results_unchanged(prec, schedule, kind, dims, bound):
    H, cops, rho0 = _hermitian_batch(dims, 2, kind)
    args = (H, cops, rho0, 0.02, 60)
    kw = dict(e_ops=[[h] for h in H], precision=prec, schedule=schedule)
    plain = propagate_batch(*args, **kw)
    res = propagate_batch(*args, check=1e-3, **kw)
    assert res["check"].shape == (len(dims), 2)
    assert res["check_flags"].all()
    assert np.all(res["check"][:, 0] < bound * 10)     # trace drift
    assert np.all(res["check"][:, 1] >= 0.0)           # rho0 Hermitian: checked
    assert np.all(res["check"][:, 1] < bound * 10)     # hermiticity
    for a, b in zip(res["rho"], plain["rho"]):
        assert np.array_equal(a, b)
    assert np.array_equal(res["observables"], plain["observables"])


def test_check_trace_zero_seed_checks_trace_only():
    # exciton correlation seeds mu rho_g: trace zero, not Hermitian
    ex = W.exciton_batch(indices=[0, 1, 313], nt=50)
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    seeds = [m @ r for m, r in zip(ex["mu"], ex["rho_g"])]
    for prec in ("fp64", "fp32", "3xbf16"):
        res = propagate_batch(ex["H"], cops, seeds, ex["dt"], ex["nt"], e_ops=[[m] for m in ex["mu"]],
                              obs_t0=False, precision=prec, check=1e-4)
        assert res["check_flags"].all(), prec
        assert np.all(res["check"][:, 1] == -1.0), prec  # hermiticity not checked
        assert np.all(res["check"][:, 0] < 1e-5), (prec, res["check"])


def test_check_below_rounding_flags_without_stopping():
    H, cops, rho0 = _hermitian_batch([12, 40], 2, "dense", seed=5)
    plain = propagate_batch(H, cops, rho0, 0.05, 200, precision="fp32")
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        res = propagate_batch(H, cops, rho0, 0.05, 200, precision="fp32", check=1e-15)
    assert any(issubclass(x.category, RuntimeWarning) for x in w)
    assert not res["check_flags"].all()
    for a, b in zip(res["rho"], plain["rho"]):
        assert np.array_equal(a, b)  # flagged instances still completed


def test_solver_run_check_attribute(golden):
    g = golden("jc16")
    sol = LindbladSolver(csr_matrix(g["H"]), [csr_matrix(c) for c in g["c_ops"]])
    r = sol.run(g["rho0"], dt=float(g["dt"]), Nt=int(g["nt"]),
                e_ops=[csr_matrix(e) for e in g["e_ops"]], check=1e-10)
    assert r.check["ok"] and r.check["hermiticity"] is not None
    assert r.check["trace_drift"] < 1e-12 and r.check["hermiticity"] < 1e-12
    assert np.abs(r.observables - g["observables"]).max() < 1e-12
    # the oracle's own trace stays at 1 as well
    obs, states = O.lindblad(g["H"], g["rho0"], list(g["c_ops"]), list(g["e_ops"]), Nt=20, dt=float(g["dt"]))
    assert abs(np.trace(states[-1]) - 1.0) < 1e-12


@pytest.mark.parametrize("prec,nt", [("3xtf32", 40), ("3xbf16", 40), ("3xbf16", 1)])
def test_check_on_the_persistent_kernel(prec, nt):
    """The persistent split-precision kernel (64 < N <= 256, static) runs the
    per-step check itself: its results are bitwise those of an unchecked
    run, its maxima agree with the graph-replayed kernels' check to
    rounding, and a tolerance below rounding flags the instance (also for a
    single step, where only the final step's check runs)."""
    from pyqed_gb300.batch import prepare_batch
    from pyqed_gb300.engine import Propagator
    H, cops, rho0 = _hermitian_batch([200], 2, "dense", seed=7)
    bi = prepare_batch(H, cops, rho0, [[h] for h in H])
    out = {}
    for persist, tol in ((1, None), (1, 1e-3), (0, 1e-3), (1, 1e-15)):
        prop = Propagator(bi.dims, nt=nt, dt=0.02, n_cops=bi.n_cops, cops_kind=bi.cops_kind, n_eops=1,
                          precision=prec, schedule="gemm")
        try:
            prop.set_option("gemm_persist", persist)
            prop.set_check(tol)
            prop.set_operators(bi.H, bi.cops, bi.eops, bi.dops)
            assert prop.info()["persistent_instances"] == persist
            o = prop.alloc_outputs(want_obs=True, want_rho=True)
            prop.propagate_device(prop.to_device(bi.rho0), None, o)
            with warnings.catch_warnings(record=True):
                warnings.simplefilter("always")
                flags = prop.check_errors()
            out[(persist, tol)] = (prop.unpack_rho(o[1])[0], prop.unpack_obs(o[0])[0], flags.copy(),
                                   prop.check_stats()[0] if tol else None)
        finally:
            prop.close()
    rho, obs, flags, _ = out[(1, None)]
    for key in ((1, 1e-3), (1, 1e-15)):
        assert np.array_equal(out[key][0], rho) and np.array_equal(out[key][1], obs)
    assert (out[(1, 1e-3)][2] == 0).all() and (out[(0, 1e-3)][2] == 0).all()
    assert (out[(1, 1e-15)][2] != 0).all()
    st_p, st_g = out[(1, 1e-3)][3], out[(0, 1e-3)][3]
    assert 0.0 <= st_p[0] < 1e-4 and 0.0 <= st_p[1] < 1e-4
    assert np.all(np.abs(st_p - st_g) < 1e-5)
