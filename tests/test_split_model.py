"""CPU model of the tensor-core kernel's split-precision arithmetic
(pyqed_gb300/csrc/lgb_tc.cu): the interleaved real embedding of the two
complex products, the exact splitting-off of the diagonal of A, and why the
3xBF16 path needs that splitting-off (rounding emulated in NumPy)."""
import numpy as np

from pyqed_gb300 import workloads as W


def mrow(c, i):
    return ((i >> 4) << 5) + (c << 4) + (i & 15)


def ncol(p, j):
    return ((j >> 4) << 5) + ((1 - p) << 4) + (j & 15)


def test_interleaved_embedding_gives_both_products():
    """D[(c,i)][(p,j)] = (P_c Q_p)[i][j] with the kernel's operand choices:
    A X (P = A, Q = X) plus X A^dag (P = -i X, Q = i A^dag read from the A
    buffer as the N side) combine to A X + X A^dag."""
    rng = np.random.default_rng(0)
    NP = 48
    A = rng.standard_normal((NP, NP)) + 1j * rng.standard_normal((NP, NP))
    X = rng.standard_normal((NP, NP)) + 1j * rng.standard_normal((NP, NP))
    M = 2 * NP
    Abuf = np.zeros((M, NP))          # rows (0, r) = Ar[r], (1, r) = Ai[r]
    XM = np.zeros((M, NP))            # rows (0, i) = Xi[i], (1, i) = -Xr[i]
    XT = np.zeros((M, NP))            # N side of A X: row ncol(p, j), K index k: part p of X[k][j]
    for r in range(NP):
        Abuf[mrow(0, r)], Abuf[mrow(1, r)] = A[r].real, A[r].imag
        XM[mrow(0, r)], XM[mrow(1, r)] = X[r].imag, -X[r].real
    for j in range(NP):
        XT[ncol(0, j)], XT[ncol(1, j)] = X[:, j].real, X[:, j].imag
    # the A buffer read as the N side: row ncol(p, j) must hold part p of
    # i conj(A[j][k]) = Ai + i Ar, i.e. part 0 = Ai[j], part 1 = Ar[j]
    for j in range(NP):
        assert np.array_equal(Abuf[ncol(0, j)], A[j].imag)
        assert np.array_equal(Abuf[ncol(1, j)], A[j].real)
    D = Abuf @ XT.T + XM @ Abuf.T
    R = np.empty((NP, NP), complex)
    for i in range(NP):
        for j in range(NP):
            re = D[mrow(0, i), ncol(0, j)] - D[mrow(1, i), ncol(1, j)]
            im = D[mrow(1, i), ncol(0, j)] + D[mrow(0, i), ncol(1, j)]
            R[i, j] = re + 1j * im
    ref = A @ X + X @ A.conj().T
    assert np.abs(R - ref).max() < 1e-10 * np.abs(ref).max()


def test_diagonal_of_a_splits_off_exactly():
    """A X + X A^dag = A_off X + X A_off^dag + (a_i + conj(a_j)) X_ij."""
    rng = np.random.default_rng(1)
    N = 17
    A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    X = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    a = np.diag(A).copy()
    Ao = A - np.diag(a)
    lhs = A @ X + X @ A.conj().T
    rhs = Ao @ X + X @ Ao.conj().T + (a[:, None] + a.conj()[None, :]) * X
    assert np.abs(lhs - rhs).max() < 1e-12


def _round_bf16(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _split_product(P, Q):
    """P @ Q with every real operand split into BF16 hi + lo and the three
    leading terms kept (hi hi + hi lo + lo hi), accumulated exactly."""
    def parts(x):
        x = np.asarray(x, np.float32)
        h = _round_bf16(x)
        lo = _round_bf16(np.float32(x - h))
        return h.astype(np.float64), lo.astype(np.float64)

    def mul(a, b):
        return a[0] @ b[0] + a[0] @ b[1] + a[1] @ b[0]

    pr, pi, qr, qi = parts(P.real), parts(P.imag), parts(Q.real), parts(Q.imag)
    return (mul(pr, qr) - mul(pi, qi)) + 1j * (mul(pr, qi) + mul(pi, qr))


def _propagate(A, Dm, X0, dt, nt, diag_exact):
    if diag_exact:
        a = np.diag(A).copy()
        Ao = A - np.diag(a)
        Dx = a[:, None] + a.conj()[None, :] + Dm
    else:
        Ao, Dx = A, Dm

    def f(X):
        return _split_product(Ao, X) + _split_product(X, Ao.conj().T) + Dx * X

    X = X0.copy()
    for _ in range(nt):
        k1 = f(X)
        k2 = f(X + 0.5 * dt * k1)
        k3 = f(X + 0.5 * dt * k2)
        k4 = f(X + dt * k3)
        X = X + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    return X


def test_bf16_split_needs_the_diagonal_in_fp32():
    """On an exciton aggregate the diagonal of A (the energies, of order one
    after the trace shift) dominates the BF16 split error; applied exactly it
    leaves an error far below the 1e-5 bar."""
    inst = W.exciton_instance(16, index=7, seed=3)
    H = inst["H"]
    N = H.shape[0]
    g = np.zeros(N)
    for cd in inst["c_diag"]:
        g += np.abs(cd) ** 2
    A = -1j * (H - np.real(np.trace(H)) / N * np.eye(N)) - 0.5 * np.diag(g)
    Dm = np.diag(g)
    X0 = inst["mu"] @ inst["rho_g"]
    dt, nt = 0.05, 300
    exact = X0.astype(complex)
    for _ in range(nt):
        f = lambda X: A @ X + X @ A.conj().T + Dm * X  # noqa: E731
        k1 = f(exact)
        k2 = f(exact + 0.5 * dt * k1)
        k3 = f(exact + 0.5 * dt * k2)
        k4 = f(exact + dt * k3)
        exact = exact + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    err_full = np.abs(_propagate(A, Dm, X0, dt, nt, False) - exact).max()
    err_diag = np.abs(_propagate(A, Dm, X0, dt, nt, True) - exact).max()
    assert err_diag < 1e-6, err_diag
    assert err_full > 10 * err_diag, (err_full, err_diag)
