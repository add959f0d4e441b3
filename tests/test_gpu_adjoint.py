"""The hand-written discrete adjoint against float64 autograd through a plain
PyTorch RK4 of the same discrete map (the reference's frozen-H RK4,
pyqed/oqs.py:1699-1806 with pyqed/phys.py:1051-1064) and against central
finite differences.  Gradient tolerance: 2e-3 relative to the gradient's
largest entry (the adjoint runs in FP32; the checks run in FP64)."""
import numpy as np
import pytest
import torch

from pyqed_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL = 2e-3


def _problem(n_inst=3, N=8, K=2, nt=30, dt=0.05, seed=41):
    d = W.driven_batch(n_inst=n_inst, N=N, K=K, seed=seed, dt=dt, nt=nt, amp=0.3, damp=0.05)
    return d


def _torch_loss(d, E, gamma, target):
    """float64 autograd through a plain PyTorch RK4 (test reference)."""
    tot = 0.0
    nt, dt = d["nt"], d["dt"]
    for b in range(len(d["H0"])):
        H0 = torch.tensor(d["H0"][b])
        mu = torch.tensor(d["mu"][b])
        Ls = [torch.sqrt(gamma[b, k]) * torch.tensor(d["L"][b][k]) for k in range(gamma.shape[1])]
        O = torch.tensor(d["O"][b])
        rho = torch.tensor(d["rho0"][b])

        def rhs(r, H):
            out = -1j * (H @ r - r @ H)
            for L in Ls:
                Ld = L.conj().T
                out = out + L @ r @ Ld - 0.5 * (Ld @ L @ r + r @ Ld @ L)
            return out
        for k in range(nt):
            H = H0 - E[k] * mu
            k1 = rhs(rho, H)
            k2 = rhs(rho + 0.5 * dt * k1, H)
            k3 = rhs(rho + 0.5 * dt * k2, H)
            k4 = rhs(rho + dt * k3, H)
            rho = rho + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
            o = torch.trace(O @ rho)
            tot = tot + torch.abs(o - target[b, k]) ** 2
    return tot


@pytest.fixture(scope="module")
def built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyqed_gb300.build import build
    build()


@pytest.mark.parametrize("ckpt", [7, 0])
def test_adjoint_matches_float64_autograd(built, ckpt):
    from pyqed_gb300.adjoint import DrivenBatch, DrivenObservables
    d = _problem()
    n, K, nt = len(d["H0"]), 2, d["nt"]
    target = np.stack([np.full(nt, 0.05 + 0.01j * b) for b in range(n)])
    batch = DrivenBatch(d["H0"], [[m] for m in d["mu"]], d["L"], d["rho0"], [[o] for o in d["O"]],
                        d["dt"], nt, checkpoint_every=ckpt, device="cuda")
    E = torch.tensor(d["E"][None, :], dtype=torch.float64, device="cuda", requires_grad=True)
    gam = torch.tensor(d["gamma"], dtype=torch.float64, device="cuda", requires_grad=True)
    obs = DrivenObservables.apply(E, gam, batch)
    loss = (torch.abs(obs[:, :, 0] - torch.tensor(target, device="cuda")) ** 2).sum()
    loss.backward()
    # reference
    Er = torch.tensor(d["E"], dtype=torch.float64, requires_grad=True)
    gr = torch.tensor(d["gamma"], dtype=torch.float64, requires_grad=True)
    lr = _torch_loss(d, Er, gr, torch.tensor(target))
    lr.backward()
    assert abs(loss.item() - lr.item()) < 1e-5 * max(1.0, abs(lr.item()))
    gE, gEr = E.grad[0].cpu().numpy(), Er.grad.numpy()
    assert np.abs(gE - gEr).max() < RTOL * np.abs(gEr).max()
    gg, ggr = gam.grad.cpu().numpy(), gr.grad.numpy()
    assert np.abs(gg - ggr).max() < RTOL * np.abs(ggr).max()


def test_adjoint_h0_and_rho0_gradients(built):
    from pyqed_gb300.adjoint import DrivenBatch
    d = _problem(n_inst=2, N=6, nt=12, seed=43)
    nt = d["nt"]
    batch = DrivenBatch(d["H0"], [[m] for m in d["mu"]], d["L"], d["rho0"], [[o] for o in d["O"]],
                        d["dt"], nt, checkpoint_every=5, device="cuda")
    obs = batch.forward(d["E"][None, :], d["gamma"])
    # J = sum_k Re(o_k): dJ/dRe o = 1, dJ/dIm o = 0
    g = torch.ones_like(obs)
    r = batch.backward(g, want_h=True, want_rho0=True)
    for b in range(2):
        H0 = torch.tensor(d["H0"][b], requires_grad=True)
        rho0 = torch.tensor(d["rho0"][b], requires_grad=True)
        mu, O = torch.tensor(d["mu"][b]), torch.tensor(d["O"][b])
        Ls = [np.sqrt(d["gamma"][b][k]) * torch.tensor(d["L"][b][k]) for k in range(2)]

        def rhs(x, H):
            out = -1j * (H @ x - x @ H)
            for L in Ls:
                Ld = L.conj().T
                out = out + L @ x @ Ld - 0.5 * (Ld @ L @ x + x @ Ld @ L)
            return out
        rho, J = rho0, 0.0
        for k in range(nt):
            H = H0 - float(d["E"][k]) * mu
            k1 = rhs(rho, H)
            k2 = rhs(rho + 0.5 * d["dt"] * k1, H)
            k3 = rhs(rho + 0.5 * d["dt"] * k2, H)
            k4 = rhs(rho + d["dt"] * k3, H)
            rho = rho + d["dt"] / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
            J = J + torch.trace(O @ rho).real
        J.backward()
        # torch's gradient of a real J w.r.t. complex z is dJ/dRe z + i dJ/dIm z,
        # the same convention as Gamma (dJ = Re Tr[Gamma^dag dZ])
        gH, gR = H0.grad.numpy(), rho0.grad.numpy()
        assert np.abs(r["dH0"][b] - gH).max() < RTOL * np.abs(gH).max()
        assert np.abs(r["drho0"][b] - gR).max() < RTOL * np.abs(gR).max()


def test_adjoint_finite_differences_in_E(built):
    """Central differences of the FP64 oracle at a few drive samples."""
    from oracle import lindblad_oracle as Orc
    from pyqed_gb300.adjoint import DrivenBatch
    d = _problem(n_inst=1, N=8, nt=20, seed=47)
    nt, dt = d["nt"], d["dt"]
    Ls = [np.sqrt(d["gamma"][0][k]) * d["L"][0][k] for k in range(2)]

    def J(E):
        obs, _ = Orc.lindblad_driven([d["H0"][0], [d["mu"][0], E]], d["rho0"][0], Ls, [d["O"][0]],
                                     Nt=nt, dt=dt, store_states=False)
        return float(np.sum(obs[:, 0].real))
    batch = DrivenBatch(d["H0"], [[m] for m in d["mu"]], d["L"], d["rho0"], [[o] for o in d["O"]],
                        dt, nt, checkpoint_every=6, device="cuda")
    obs = batch.forward(d["E"][None, :], d["gamma"])
    r = batch.backward(torch.ones_like(obs))
    gE = r["dE"][0].cpu().numpy()
    eps = 1e-5
    for k in (0, 7, nt - 1):
        Ep, Em = d["E"].copy(), d["E"].copy()
        Ep[k] += eps
        Em[k] -= eps
        fd = (J(Ep) - J(Em)) / (2 * eps)
        assert abs(gE[k] - fd) < RTOL * max(np.abs(gE).max(), 1e-8)


def test_adjoint_driven_workload_n64_k2_checkpoints_45(built):
    """The driven workload's own shape: N = 64, K = 2 collapse operators with
    rates gamma_k in [0.005, 0.02], the smooth Gaussian-process pulse, dt =
    0.01, checkpoints every 45 steps, and the loss against the trajectory of a
    perturbed pulse E + dE.  200 of the 2000 steps (four full checkpoint
    segments and a partial one) keep the float64 reference affordable;
    gradients in E(t) and gamma_k against float64 autograd on two instances
    and central differences of the FP64 oracle at a few samples."""
    from oracle import lindblad_oracle as Orc
    from pyqed_gb300.adjoint import DrivenBatch, DrivenObservables
    nt = 200
    d = W.driven_batch(n_inst=2, N=64, K=2, nt=nt)
    n, dt = len(d["H0"]), d["dt"]
    batch = DrivenBatch(d["H0"], [[m] for m in d["mu"]], d["L"], d["rho0"], [[o] for o in d["O"]],
                        dt, nt, checkpoint_every=45, device="cuda")
    # target: the observables of the perturbed pulse
    target = batch.forward(d["E_target"][None, :], d["gamma"])[:, :, 0].detach().clone()
    E = torch.tensor(d["E"][None, :], dtype=torch.float64, device="cuda", requires_grad=True)
    gam = torch.tensor(d["gamma"], dtype=torch.float64, device="cuda", requires_grad=True)
    obs = DrivenObservables.apply(E, gam, batch)
    loss = (torch.abs(obs[:, :, 0] - target) ** 2).sum()
    loss.backward()
    Er = torch.tensor(d["E"], dtype=torch.float64, requires_grad=True)
    gr = torch.tensor(d["gamma"], dtype=torch.float64, requires_grad=True)
    lr = _torch_loss(d, Er, gr, target.cpu())
    lr.backward()
    assert abs(loss.item() - lr.item()) < 1e-4 * max(1e-12, abs(lr.item()))
    gE, gEr = E.grad[0].cpu().numpy(), Er.grad.numpy()
    assert np.abs(gE - gEr).max() < RTOL * np.abs(gEr).max()
    gg, ggr = gam.grad.cpu().numpy(), gr.grad.numpy()
    assert np.abs(gg - ggr).max() < RTOL * np.abs(ggr).max()
    # central differences of the FP64 oracle (instance 0, the same loss)
    tg = target[0].cpu().numpy()

    def J(Ev, g0):
        Ls = [np.sqrt(g0[k]) * d["L"][0][k] for k in range(2)]
        o, _ = Orc.lindblad_driven([d["H0"][0], [d["mu"][0], Ev]], d["rho0"][0], Ls, [d["O"][0]],
                                   Nt=nt, dt=dt, store_states=False)
        return float(np.sum(np.abs(o[:, 0] - tg) ** 2))
    gE0 = torch.autograd.grad((torch.abs(DrivenObservables.apply(E, gam, batch)[0, :, 0] - target[0]) ** 2).sum(),
                              E)[0][0].cpu().numpy()
    eps = 1e-4
    for k in (3, 97, nt - 1):
        Ep, Em = d["E"].copy(), d["E"].copy()
        Ep[k] += eps
        Em[k] -= eps
        fd = (J(Ep, d["gamma"][0]) - J(Em, d["gamma"][0])) / (2 * eps)
        assert abs(gE0[k] - fd) < 5 * RTOL * np.abs(gE0).max(), (k, gE0[k], fd)
