"""CPU checks of the C-ABI library and the host logic (no compute calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from pyqed_gb300 import _capi as C
from pyqed_gb300 import engine, oqs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lindblad_gb300.h")


def _declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(lgb_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(C.LIBPATH):
        from pyqed_gb300.build import build
        build()
    return C.lib()


def test_header_declares_exports():
    assert _declared() == sorted(C.EXPORTS)


def test_library_exports_every_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_version_and_status_strings(lib):
    assert lib.lgb_get_version() == 10000
    assert lib.lgb_status_string(C.LGB_OK) == b"ok"
    assert lib.lgb_status_string(C.LGB_ERR_NONFINITE) == b"state became non-finite"
    assert lib.lgb_status_string(12345) == b"unknown status"


def test_plan_create_rejects_bad_arguments(lib):
    plan = ctypes.c_void_p()
    dims = (ctypes.c_int32 * 1)(4)
    bad = C.Problem(n_inst=0, nt=1, dt=0.1)
    assert lib.lgb_plan_create(ctypes.byref(plan), ctypes.byref(bad), dims) == C.LGB_ERR_INVALID_ARG
    bad = C.Problem(n_inst=1, nt=1, dt=0.1, n_eops=17)
    assert lib.lgb_plan_create(ctypes.byref(plan), ctypes.byref(bad), dims) == C.LGB_ERR_INVALID_ARG
    bad = C.Problem(n_inst=1, nt=1, dt=0.1, cops_kind=C.COPS_DENSE, n_cops=0)
    assert lib.lgb_plan_create(ctypes.byref(plan), ctypes.byref(bad), dims) == C.LGB_ERR_INVALID_ARG
    assert lib.lgb_plan_create(None, ctypes.byref(bad), dims) == C.LGB_ERR_INVALID_ARG
    assert lib.lgb_plan_destroy(None) == C.LGB_ERR_INVALID_ARG


def test_plan_create_without_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    plan = ctypes.c_void_p()
    dims = (ctypes.c_int32 * 1)(4)
    ok = C.Problem(n_inst=1, nt=1, dt=0.1)
    assert lib.lgb_plan_create(ctypes.byref(plan), ctypes.byref(ok), dims) == C.LGB_ERR_NO_DEVICE


def test_product_path_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    s = oqs.LindbladSolver(np.eye(2), [])
    with pytest.raises(RuntimeError, match="CUDA"):
        s.run(np.eye(2) / 2, dt=0.1, Nt=1)


def test_pack_and_diagonal_detection():
    from scipy.sparse import csr_matrix
    a = np.arange(4).reshape(2, 2).astype(complex)
    assert np.array_equal(engine.pack([a, np.eye(1)]), np.array([0, 1, 2, 3, 1], complex))
    assert engine.diagonal_of(np.diag([1, 2j])) is not None
    assert engine.diagonal_of(a) is None
    assert np.array_equal(engine.diagonal_of(csr_matrix(np.diag([3, 4]))), [3, 4])
    assert engine.diagonal_of(csr_matrix(a)) is None


def test_drive_sampling_matches_reference_clock():
    # pyqed/oqs.py:1790-1794: t accumulates by += dt and f is evaluated at t_{k+1}
    seen = []
    out = oqs._eval_drive([(None, lambda t: seen.append(t) or 2 * t)], 3, 0.1, 0.5)
    t, exp = 0.5, []
    for _ in range(3):
        t += 0.1
        exp.append(t)
    assert seen == exp
    assert np.allclose(out[0], 2 * np.array(exp))
    with pytest.raises(ValueError):
        oqs._eval_drive([(None, np.zeros(2))], 3, 0.1, 0.0)


def test_liouvillian_superoperator_matches_oracle():
    from oracle.lindblad_oracle import liouvillian_superop
    from pyqed_gb300 import workloads as W
    jc = W.jaynes_cummings()
    L = oqs.liouvillian(jc["H"], jc["c_ops"]).toarray()
    assert np.abs(L - liouvillian_superop(jc["H"], jc["c_ops"])).max() < 1e-14


def test_result_conventions(tmp_path):
    from pyqed_gb300.mol import Result, load_result
    r = Result(dt=0.1, Nt=10, rho0=np.eye(2))
    assert r.times.shape == (11,) and r.times[-1] == pytest.approx(1.0)
    r.observables = np.zeros((11, 1))
    r.dump(str(tmp_path / "r.pkl"))
    assert load_result(str(tmp_path / "r.pkl")).nt == 10


def test_heom_create_validates_before_any_device_call():
    import ctypes
    L = C.lib()
    plan = ctypes.c_void_p()
    dims = (ctypes.c_int32 * 1)(4)
    for bad in (dict(nado=1), dict(n_eops=17), dict(flags=8), dict(nt=-1)):
        kw = dict(n_inst=1, n_eops=0, nt=10, nado=4, precision=C.PREC["fp32"], flags=0, dt=0.01)
        kw.update(bad)
        prob = C.HeomProblem(**kw)
        assert L.lgb_heom_create(ctypes.byref(plan), ctypes.byref(prob), dims) == C.LGB_ERR_INVALID_ARG
    prob = C.HeomProblem(n_inst=1, n_eops=0, nt=10, nado=4, precision=C.PREC["3xtf32"], flags=0, dt=0.01)
    assert L.lgb_heom_create(ctypes.byref(plan), ctypes.byref(prob), dims) == C.LGB_ERR_UNSUPPORTED
    assert L.lgb_heom_max_dim(C.PREC["fp32"]) == 64
    # N = 16: 200 KB of shared memory less the two operators, 4 KB per level
    assert L.lgb_heom_max_levels_on_chip(16, C.PREC["fp64"]) == (200 * 1024 - 2 * 256 * 16) // 4096
