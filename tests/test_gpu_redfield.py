"""GPU parity of the Redfield solver against the reference's outputs
(tests/golden/redfield_*.npz, produced by running binggu56/pyqed) and the
oracle.  Tolerances: 1e-12 max-abs for FP64, 1e-5 for FP32."""
import numpy as np
import pytest

from oracle import redfield_oracle as RO
from pyqed_gb300 import RedfieldSolver, redfield_batch
from pyqed_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300.build import build
    build()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_redfield_chain_golden(golden, prec, tol):
    g = golden("redfield_chain")
    ch = W.redfield_chain(n=6, seed=7)
    sol = RedfieldSolver(ch["H"], c_ops=ch["a_ops"], spectra=ch["spectra"])
    r = sol.evolve(ch["rho0"], dt=float(g["dt"]), Nt=int(g["nt"]), e_ops=ch["e_ops"], precision=prec)
    assert r.observables.shape == g["observables"].shape and len(r.rholist) == int(g["nt"])
    assert np.abs(r.observables - g["observables"]).max() < tol
    for k, s in zip(g["state_index"], g["states"]):
        assert np.abs(r.rholist[k] - s).max() < tol


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_redfield_gue_golden(golden, prec, tol):
    g = golden("redfield_gue")
    spectra = [W.ohmic_spectrum(*p) for p in g["spectra"]]
    sol = RedfieldSolver(g["H"], c_ops=list(g["a_ops"]), spectra=spectra)
    R, V = sol.redfield_tensor()
    Ro, Vo = RO.redfield_tensor(g["H"], list(g["a_ops"]), spectra)
    assert np.abs(R.toarray() - Ro).max() < 1e-12  # same eigensolver, same basis
    r = sol.evolve(g["rho0"], dt=float(g["dt"]), Nt=int(g["nt"]), e_ops=list(g["e_ops"]), precision=prec)
    assert np.abs(r.observables - g["observables"]).max() < tol * 10
    assert np.abs(r.rholist[-1] - g["rho_last"]).max() < tol


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
@pytest.mark.parametrize("dims", [[3, 6, 11, 16], [1, 2, 5, 8, 7, 8]])
def test_redfield_batch_uneven_vs_oracle(prec, tol, dims):
    # N = 16 keeps the generator in L2 (streamed) in both precisions, N <= 6 in
    # shared memory; a batch with every N <= 8 runs FP32 with R in registers
    rng = np.random.default_rng(4 + len(dims))
    H, A, S, R0, E = [], [], [], [], []
    for N in dims:
        h = W.gue_matrix(rng, N) * 0.5
        a = [np.diag(rng.uniform(-1, 1, N)).astype(complex)]
        m = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.2
        a.append(0.5 * (m + m.conj().T))
        psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        psi /= np.linalg.norm(psi)
        H.append(h), A.append(a), S.append([W.ohmic_spectrum(0.05, 0.8, 3.0), W.ohmic_spectrum(0.02, 1.5, 1.0)])
        R0.append(np.outer(psi, psi.conj())), E.append([h, a[1]])
    nt, dt = 60, 0.05
    res = redfield_batch(H, A, S, R0, dt, nt, e_ops=E, precision=prec, store_every=20)
    for b in range(len(dims)):
        R, V = RO.redfield_tensor(H[b], A[b], S[b])
        obs, rholist, _ = RO.redfield_propagate(R, R0[b], V, nt, dt, E[b])
        assert np.abs(res["observables"][b] - obs).max() < tol * 10
        assert np.abs(res["rho"][b] - rholist[-1]).max() < tol
        for k in range(3):
            assert np.abs(res["states"][b][k] - rholist[20 * k + 19]).max() < tol


def test_redfield_fp32_register_kernel_nonfinite():
    """A non-finite state stops its own system only (register-resident kernel)."""
    rng = np.random.default_rng(9)
    dims = [4, 8, 6]
    H, A, S, R0, E = [], [], [], [], []
    for N in dims:
        h = W.gue_matrix(rng, N) * 0.5
        H.append(h), A.append([np.diag(rng.uniform(-1, 1, N)).astype(complex)])
        S.append([W.ohmic_spectrum(0.05, 0.8, 3.0)])
        psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        R0.append(np.outer(psi, psi.conj()) / np.vdot(psi, psi).real), E.append([h])
    R0[1] = R0[1].copy()
    R0[1][0, 0] = np.nan
    from pyqed_gb300 import _capi as C
    with pytest.raises(C.LindbladError) as ei:
        redfield_batch(H, A, S, R0, 0.05, 10, e_ops=E, precision="fp32")
    assert ei.value.status == C.LGB_ERR_NONFINITE and "system 1" in str(ei.value)


def test_redfield_batched_tensor_build_matches_single():
    from pyqed_gb300.redfield import _eigen_parts, build_tensor, build_tensors
    parts = [_eigen_parts(c["H"], c["a_ops"], c["spectra"])
             for c in (W.redfield_chain(n=n, seed=s) for n, s in ((3, 1), (6, 2), (8, 3), (5, 4)))]
    Rb = build_tensors(parts).cpu().numpy()
    off = 0
    for p in parts:
        n = len(p[0])
        R1 = build_tensor(p[0], p[2], p[3]).cpu().numpy()
        assert np.array_equal(Rb[off:off + n ** 4], R1)
        off += n ** 4


def test_redfield_solver_propagator_expect_gf_c4_golden(golden):
    g = golden("redfield_aux")
    ch = W.redfield_chain(n=3, seed=5)
    sol = RedfieldSolver(ch["H"], c_ops=ch["a_ops"], spectra=ch["spectra"])
    R, V = sol.redfield_tensor()
    t = g["t"]
    U = sol.propagator(t)
    assert U.shape == g["U_sos"].shape and np.abs(U - g["U_sos"]).max() < 1e-10
    assert np.abs(sol.expect(ch["rho0"], ch["e_ops"]) - g["expect"]).max() < 1e-10
    # the stored G is used, whatever tau is given (as the reference)
    c4 = sol.correlation_4op_3t(ch["rho0"], list(g["ops"]), "llrr", t[:4])
    assert c4.shape == g["c4"].shape and np.abs(c4 - g["c4"]).max() < 1e-10
    assert np.abs(sol.gf(t, method="diag") - g["gf"]).max() < 1e-10
    sol2 = RedfieldSolver(ch["H"], c_ops=ch["a_ops"], spectra=ch["spectra"])
    sol2.redfield_tensor()
    U2 = sol2.propagator(t, method="EOM")
    assert np.abs(U2 - g["U_eom"]).max() < 1e-12
    assert np.abs(sol2.gf(t) + 1j * g["U_eom"]).max() < 1e-12


def test_redfield_solver_correlation_2op_and_steady_state():
    from oracle import redfield_oracle as RO
    ch = W.redfield_chain(n=4, seed=6)
    sol = RedfieldSolver(ch["H"], c_ops=ch["a_ops"], spectra=ch["spectra"])
    R, V = sol.redfield_tensor()
    M = 16
    tau = np.linspace(0.0, 3.0, 7)
    a = RO.superop(ch["e_ops"][0], "l")
    b = RO.superop(ch["a_ops"][1], "l")
    r0 = V.conj().T @ ch["rho0"] @ V
    c = sol.correlation_2op_1t(r0, a, b, tau)
    G = -1j * RO.propagator_sos(R.toarray(), tau)
    ref = np.eye(4).flatten() @ (a @ np.tensordot(G, b @ r0.flatten(), axes=([1], [0])))
    assert c.shape == (7,) and np.abs(c - ref).max() < 1e-10
    rss = sol.steady_state()
    assert abs(np.trace(rss) - 1) < 1e-10
    v = (V.conj().T @ rss @ V).flatten()
    assert np.abs(R.toarray() @ v).max() < 1e-10
    del M
