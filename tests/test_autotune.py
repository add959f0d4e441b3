"""Autotuner: candidate enumeration, selection and cache (CPU, injected
timings) and one tuned propagation on the GPU against the untuned one."""
import numpy as np
import pytest

from pyqed_gb300 import autotune
from pyqed_gb300.batch import prepare_batch


def _batch(dims, kind="diag"):
    rng = np.random.default_rng(0)
    H, cops, rho0 = [], [], []
    for N in dims:
        h = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        H.append(h + h.conj().T)
        if kind == "diag":
            cops.append([np.diag(rng.uniform(0, 0.1, N)).astype(complex)])
        else:
            cops.append([rng.standard_normal((N, N)) * 0.01 + 0j])
        psi = rng.standard_normal(N) + 0j
        psi /= np.linalg.norm(psi)
        rho0.append(np.outer(psi, psi.conj()))
    return prepare_batch(H, cops, rho0, [[h] for h in H])


def test_candidates():
    c = autotune.candidates([20, 40, 60], "3xtf32", "diag", 1)
    assert dict(schedule="auto", options={}) in c
    assert dict(schedule="auto", options={"tc_pairs": 0}) in c
    assert dict(schedule="gemm", options={"gemm_waves": 2}) in c
    # large batches never time the per-instance GEMM schedule
    c = autotune.candidates(np.full(4096, 40), "fp32", "diag", 1)
    assert all(x["schedule"] != "gemm" for x in c)
    # dense collapse operators: no tensor-core pairing option
    c = autotune.candidates([20, 40], "3xtf32", "dense", 2)
    assert all("tc_pairs" not in x["options"] for x in c)


def test_gemm_candidates_cover_graph_length_and_split_k():
    c = autotune.candidates([1024], "3xtf32", "dense", 4)
    gemm = [x["options"] for x in c if x["schedule"] == "gemm"]
    assert {} in gemm and {"graph_steps": 32} in gemm
    assert {"gemm_waves": 2} in gemm and {"gemm_ksplit": 4} in gemm
    assert {"graph_steps": 32, "gemm_ksplit": 8} in gemm
    assert all("gemm_persist" not in x for x in gemm)
    # 64 < N <= 256, static: the persistent kernel (default) against the
    # graph-replayed kernels, whose shapes are timed with it switched off
    c = autotune.candidates([256], "3xbf16", "dense", 4)
    gemm = [x["options"] for x in c if x["schedule"] == "gemm"]
    assert gemm[0] == {} and {"gemm_persist": 0} in gemm
    assert {"gemm_persist": 0, "graph_steps": 32, "gemm_ksplit": 8} in gemm
    assert all(x.get("gemm_persist") == 0 for x in gemm[1:])
    # driven instances never take the persistent kernel
    c = autotune.candidates([256], "3xtf32", "dense", 4, n_drive=1)
    assert all("gemm_persist" not in x["options"] for x in c)
    # the plain precisions have no split-K shape to tune
    c = autotune.candidates([256], "fp32", "dense", 4)
    assert all(set(x["options"]) <= {"graph_steps"} for x in c)


def test_bf16_candidates_keep_the_fp32_diagonal():
    # 3xBF16 on instances that fit the tensor-core kernel: only that kernel
    # (its diagonal of A is applied in FP32), never the GEMM schedule
    c = autotune.candidates([20, 40, 60, 65], "3xbf16", "diag", 1)
    assert c == [dict(schedule="auto", options={}), dict(schedule="auto", options={"tc_pairs": 0})]
    c = autotune.candidates([40, 64], "3xbf16", "none", 0, n_drive=1)
    assert c == [dict(schedule="auto", options={})]
    # a driven N = 65 instance, dense collapse operators or N > 65 leave the
    # tensor-core kernel, and the GEMM schedule is timed again
    for args in (([65], "diag", 1, 1), ([40], "dense", 2, 0), ([40, 100], "diag", 1, 0)):
        dims, kind, k, nd = args
        c = autotune.candidates(dims, "3xbf16", kind, k, n_drive=nd)
        assert any(x["schedule"] == "gemm" for x in c), args


def test_tune_selects_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("PYQED_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    bi = _batch([20, 40, 60])
    fake = {("auto", ()): 3.0, ("auto", (("tc_pairs", 0),)): 2.0, ("gemm", ()): None,
            ("gemm", (("gemm_waves", 2),)): 5.0}
    calls = []

    def timer(c):
        calls.append(c)
        return fake.get((c["schedule"], tuple(sorted(c["options"].items()))), 7.0)
    r = autotune.tune(bi, dt=0.01, precision="3xtf32", timer=timer)
    assert (r["schedule"], r["options"], r["cached"]) == ("auto", {"tc_pairs": 0}, False)
    n_cand = len(autotune.candidates(bi.dims, "3xtf32", bi.cops_kind, bi.n_cops))
    assert len(r["timings_ms"]) == n_cand - 1  # the invalid candidate (None) is dropped
    n = len(calls)
    r2 = autotune.tune(bi, dt=0.01, precision="3xtf32", timer=timer)
    assert r2["cached"] and r2["options"] == {"tc_pairs": 0} and len(calls) == n
    # another precision is another problem
    autotune.tune(bi, dt=0.01, precision="fp32", timer=lambda c: 1.0)
    assert len(calls) == n


def test_signature_is_order_independent():
    a = autotune.signature([3, 1, 2], 1, "diag", 1, 0, "fp32", "x")
    b = autotune.signature([1, 2, 3], 1, "diag", 1, 0, "fp32", "x")
    assert a == b and a != autotune.signature([1, 2, 4], 1, "diag", 1, 0, "fp32", "x")


@pytest.mark.gpu
def test_tuned_propagation_matches_default(tmp_path, monkeypatch):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300 import propagate_batch
    from pyqed_gb300 import workloads as W
    from pyqed_gb300.build import build
    build()
    monkeypatch.setenv("PYQED_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    ex = W.exciton_batch(n_inst=24, nt=30)
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    seeds = [m @ r for m, r in zip(ex["mu"], ex["rho_g"])]
    eops = [[m] for m in ex["mu"]]
    a = propagate_batch(ex["H"], cops, seeds, ex["dt"], 30, e_ops=eops, obs_t0=False,
                        precision="3xtf32", schedule="auto")
    b = propagate_batch(ex["H"], cops, seeds, ex["dt"], 30, e_ops=eops, obs_t0=False,
                        precision="3xtf32", schedule="tune")
    assert not b["tuned"]["cached"] and len(b["tuned"]["timings_ms"]) >= 2
    assert np.abs(a["observables"] - b["observables"]).max() < 1e-5
    c = propagate_batch(ex["H"], cops, seeds, ex["dt"], 30, e_ops=eops, obs_t0=False,
                        precision="3xtf32", schedule="tune")
    assert c["tuned"]["cached"]
