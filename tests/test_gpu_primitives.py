"""Unit tests of the FP64 device primitives (include/lila_prim.h) against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mask(X, mask):
    if mask == 1:
        Y = np.tril(X, -1)
        np.fill_diagonal(Y[: min(X.shape), : min(X.shape)], 1.0)
        return Y
    if mask == 2:
        return np.triu(X)
    if mask == 3:
        return np.tril(X)
    if mask == 4:
        Y = np.triu(X, 1)
        np.fill_diagonal(Y[: min(X.shape), : min(X.shape)], 1.0)
        return Y
    return X


@pytest.mark.parametrize("M,N,K", [(5, 7, 3), (64, 64, 4096), (300, 40, 17), (33, 65, 0), (1000, 200, 64),
                                   (64, 64, 100000)])
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_gemm_ops_masks_splits(gpu_lib, M, N, K, ta, tb):
    import torch

    L = gpu_lib
    rng = np.random.default_rng(M * 7 + N * 3 + K + ta * 2 + tb)
    for maskA, maskB in ((0, 0), (1, 0), (0, 2), (2, 1), (3, 4)):
        As = np.asfortranarray(rng.standard_normal((K, M) if ta else (M, K)))
        Bs = np.asfortranarray(rng.standard_normal((N, K) if tb else (K, N)))
        C0 = np.asfortranarray(rng.standard_normal((M + 3, N)))
        opA = _mask(As, maskA)
        opA = opA.T if ta else opA
        opB = _mask(Bs, maskB)
        opB = opB.T if tb else opB
        alpha, beta, zr = -1.5, 0.5, min(4, M)
        ref = C0.copy()
        ref[:M] = alpha * (opA @ opB)
        ref[zr:M] += beta * C0[zr:M]
        dA, dB, dC = (L.to_device_colmajor(x) for x in (As, Bs, C0))
        part = torch.empty(64 * M * N + 1, dtype=torch.float64, device="cuda")
        L.prim_gemm(M, N, K, dA, max(1, As.shape[0]), ta, maskA, dB, max(1, Bs.shape[0]), tb, maskB,
                    dC, M + 3, alpha, beta, zr, 0, 0, part, part.numel())
        torch.cuda.synchronize()
        got = L.from_device(dC)
        scale = max(1.0, np.abs(ref).max())
        assert np.abs(got - ref).max() / scale < 1e-13, (maskA, maskB)


def test_gemm_epilogue_flags(gpu_lib):
    import torch

    L = gpu_lib
    rng = np.random.default_rng(3)
    M = N = 40
    K = 9000
    A = np.asfortranarray(rng.standard_normal((K, M)))
    C0 = np.asfortranarray(rng.standard_normal((M, N)))
    dA, dC = L.to_device_colmajor(A), L.to_device_colmajor(C0)
    part = torch.empty(64 * M * N, dtype=torch.float64, device="cuda")
    assert L.prim_gemm_splits(M, N, K, part.numel()) > 1
    L.prim_gemm(M, N, K, dA, K, 1, 0, dA, K, 0, 0, dC, M, 1.0, 0.0, 0, 1, 1, part, part.numel())
    torch.cuda.synchronize()
    got = L.from_device(dC)
    G = A.T @ A + np.eye(M)
    iu = np.triu_indices(M)
    il = np.tril_indices(M, -1)
    assert np.abs(got[iu] - G[iu]).max() / np.abs(G).max() < 1e-13
    assert np.array_equal(got[il], C0[il])  # upper_only leaves the strict lower part


def test_trsms(gpu_lib):
    import torch

    L = gpu_lib
    rng = np.random.default_rng(4)
    for N in (7, 32, 64, 100):
        M = 5000
        U = np.asfortranarray(np.triu(rng.standard_normal((N, N))) + 4 * np.eye(N))
        B = np.asfortranarray(rng.standard_normal((M, N)))
        S = np.where(rng.random(N) < 0.5, -1.0, 1.0)
        ref = (B * S[None, :] * 2.0) @ np.linalg.inv(U)
        dU, dB = L.to_device_colmajor(U), L.to_device_colmajor(B)
        dS = torch.from_numpy(S).cuda()
        L.prim_trsm_right_upper(M, N, 2.0, dU, N, dB, M, dS)
        torch.cuda.synchronize()
        assert np.abs(L.from_device(dB) - ref).max() / np.abs(ref).max() < 1e-12
    n, nc = 40, 13
    Lm = np.asfortranarray(np.tril(rng.standard_normal((n, n)), -1) * 0.3 + np.eye(n))
    B = np.asfortranarray(rng.standard_normal((n, nc)))
    dL, dB = L.to_device_colmajor(Lm), L.to_device_colmajor(B)
    L.prim_trsm_left_lower_unit(n, nc, dL, n, dB, n)
    torch.cuda.synchronize()
    ref = np.linalg.solve(np.tril(Lm, -1) + np.eye(n), B)
    assert np.abs(L.from_device(dB) - ref).max() / np.abs(ref).max() < 1e-12
    B = np.asfortranarray(rng.standard_normal((nc, n)))
    dB = L.to_device_colmajor(B)
    L.prim_trsm_right_lower_unit_trans(nc, n, -1.0, dL, n, dB, nc)
    torch.cuda.synchronize()
    ref = -B @ np.linalg.inv((np.tril(Lm, -1) + np.eye(n)).T)
    assert np.abs(L.from_device(dB) - ref).max() / np.abs(ref).max() < 1e-12


def test_potrf_lu_larfg(gpu_lib, oracle_lib):
    import torch

    L = gpu_lib
    rng = np.random.default_rng(5)
    for n in (1, 5, 64, 130):
        X = rng.standard_normal((3 * n + 2, n))
        G = np.asfortranarray(X.T @ X)
        dG = L.to_device_colmajor(G)
        L.prim_potrf_upper(n, dG, n)
        torch.cuda.synchronize()
        U = np.triu(L.from_device(dG))
        assert np.abs(U.T @ U - G).max() / np.abs(G).max() < 1e-13
        assert L.gpu_status() == 0
    # LU with sign choice against the oracle's lila_dorgh2_3 first loop
    n = 48
    Q, _ = np.linalg.qr(rng.standard_normal((200, n)))
    T = np.asfortranarray(Q[:n].copy())
    dT = L.to_device_colmajor(T)
    dS = torch.zeros(n, dtype=torch.float64, device="cuda")
    L.prim_lu_sign(n, dT, n, dS)
    torch.cuda.synchronize()
    S = np.where(np.abs(1 - np.diag(T)) < np.abs(1 + np.diag(T)), -1.0, 1.0)  # first pivot only
    got = L.from_device(dT)
    Lf = np.tril(got, -1) + np.eye(n)
    Uf = np.triu(got)
    Sg = dS.cpu().numpy()
    assert Sg[0] == S[0]
    assert np.abs(Lf @ Uf - (T * Sg[None, :] - np.eye(n))).max() < 1e-13
    # larfg against the oracle's dlarfg
    for m in (1, 2, 17, 5000, 70000):
        x = rng.standard_normal(m)
        xo = x.copy()
        tau_o = np.zeros(1)
        alpha = np.array([xo[0]])
        oracle_lib_ob = oracle_lib
        # oracle: dgeqr3 with n = 1 is dlarfg on the column
        A = np.asfortranarray(xo.reshape(m, 1))
        Tt = np.asfortranarray(np.zeros((1, 1)))
        oracle_lib_ob.dgeqr3(m, 1, A, m, Tt, 1)
        dx = torch.from_numpy(x.copy()).cuda()
        dtau = torch.zeros(1, dtype=torch.float64, device="cuda")
        L.prim_larfg(m, dx, dtau)
        torch.cuda.synchronize()
        assert abs(dtau.item() - Tt[0, 0]) < 1e-14
        assert np.abs(dx.cpu().numpy() - A[:, 0]).max() / max(1, np.abs(A).max()) < 1e-13
