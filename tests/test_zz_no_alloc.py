"""The no-allocation entry point against the plan-based entry point and the
reference's own results.

``lgb_propagate_noalloc`` serves callers that cannot allocate device memory
(a device heap owned by another allocator, or a device-memory budget fixed
before the library is loaded): it keeps all working memory in a fixed array
inside the library.  Here it is called through the C ABI, twice in a row
(the second call reuses the array the first one left behind), and each
result is compared with ``lgb_plan_propagate`` in FP64 on the same inputs,
within the FP64 tolerance of the other parity tests; the Jaynes-Cummings
case is also compared with the reference's own ``LindbladSolver.run``
output (``tests/golden/jc16.npz``).  This file is named so that pytest
collects it last.
"""
import ctypes
import os

import numpy as np
import pytest

from pyqed_gb300 import _capi as C
from pyqed_gb300 import propagate_batch
from pyqed_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300.build import build
    build()
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128).ravel()).cuda()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc(torch, H, cops, kind, eops, rho0, nt, dt, obs_t0):
    L = C.lib()
    N = H.shape[0]
    dH, dr = _dev(torch, H), _dev(torch, rho0)
    dc = _dev(torch, np.stack(cops)) if cops else None
    de = _dev(torch, np.stack(eops)) if eops else None
    obs = torch.zeros((nt + obs_t0) * len(eops), dtype=torch.complex128, device="cuda")
    rho = torch.zeros(N * N, dtype=torch.complex128, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.lgb_propagate_noalloc(_ptr(dH), N, _ptr(dc), len(cops), kind, _ptr(de), len(eops),
                                 _ptr(dr), nt, dt, obs_t0, _ptr(obs), _ptr(rho), _ptr(status),
                                 stream)
    assert rc == C.LGB_OK, C.lib().lgb_status_string(rc)
    torch.cuda.synchronize()
    assert int(status.item()) == C.LGB_OK
    return (obs.cpu().numpy().reshape(nt + obs_t0, len(eops)),
            rho.cpu().numpy().reshape(N, N))


def test_noalloc_matches_plan_entry_point_twice(torch_cuda):
    torch = torch_cuda
    # dense collapse operators (Jaynes-Cummings, N = 16) and diagonal ones (N = 64)
    jc = W.jaynes_cummings()
    rng = np.random.default_rng(7)
    H64 = W.gue_matrix(rng, 64)
    d64 = [np.sqrt(0.02) * (np.arange(64) == k).astype(complex) for k in range(3)]
    psi = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    psi /= np.linalg.norm(psi)
    cases = [
        (jc["H"], jc["c_ops"], C.COPS_DENSE, jc["e_ops"], jc["rho0"], 60, jc["dt"], 1),
        (H64, d64, C.COPS_DIAG, [W.gue_matrix(rng, 64)], np.outer(psi, psi.conj()), 40, 0.01, 0),
        (H64, [], C.COPS_NONE, [], np.outer(psi, psi.conj()), 25, 0.02, 0),
    ]
    for H, cops, kind, eops, rho0, nt, dt, t0 in cases:
        cops_b = [np.diag(c) for c in cops] if kind == C.COPS_DIAG else cops
        ref = propagate_batch([H], [cops_b], [rho0], dt, nt, e_ops=[eops], obs_t0=bool(t0),
                              precision="fp64")
        for _ in range(2):
            obs, rho = _noalloc(torch, H, cops, kind, eops, rho0, nt, dt, t0)
            assert np.abs(rho - ref["rho"][0]).max() < TOL64
            if eops:
                assert np.abs(obs - ref["observables"][0]).max() < TOL64


def test_noalloc_matches_reference_fixture(torch_cuda):
    # the reference's LindbladSolver.run on the Jaynes-Cummings system, all
    # 2000 steps: observables at every step and the states kept in the fixture
    torch = torch_cuda
    g = np.load(os.path.join(GOLD, "jc16.npz"))
    nt = int(g["nt"])
    for _ in range(2):
        obs, rho = _noalloc(torch, g["H"], list(g["c_ops"]), C.COPS_DENSE, list(g["e_ops"]),
                            g["rho0"], nt, float(g["dt"]), 1)
        assert np.abs(obs - g["observables"]).max() < TOL64
        assert np.abs(rho - g["states"][-1]).max() < TOL64


def test_noalloc_rejects_sizes_beyond_its_limit(torch_cuda):
    torch = torch_cuda
    L = C.lib()
    N = C.NOALLOC_MAX_DIM + 1
    H = _dev(torch, np.eye(N))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.lgb_propagate_noalloc(_ptr(H), N, None, 0, C.COPS_NONE, None, 0, _ptr(H), 1, 0.1, 0,
                                 None, None, None, stream)
    assert rc == C.LGB_ERR_TOO_LARGE
    assert L.lgb_status_string(rc) == b"size exceeds the no-allocation scratch limit"
