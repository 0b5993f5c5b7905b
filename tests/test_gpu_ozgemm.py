"""General FP64-grade split-precision GEMM on the BF16 tensor cores
(lila_prim_ozgemm) against double-double products of the oracle, and the
factorizations run with LILA_PRECISION_SPLIT against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U = 2.0 ** -53


def masked(X, mask):
    X = X.copy()
    if mask == 1:  # unit lower trapezoid
        X = np.tril(X, -1)
        np.fill_diagonal(X, 1.0)
    elif mask == 2:
        X = np.triu(X)
    elif mask == 3:
        X = np.tril(X)
    elif mask == 4:
        X = np.triu(X, 1)
        np.fill_diagonal(X, 1.0)
    return X


def run_case(L, oracle_lib, M, N, K, ta, tb, ma, mb, alpha, beta, zero_rows=0, add_diag=0, upper_only=0,
             split=False, seed=0, scale_rows=False):
    import torch

    rng = np.random.default_rng(seed)
    As = rng.standard_normal((M, K) if ta == 0 else (K, M))
    Bs = rng.standard_normal((K, N) if tb == 0 else (N, K))
    if scale_rows:  # rows of op(A) over 12 orders of magnitude
        sc = 10.0 ** rng.uniform(-6, 6, size=M)
        As = As * (sc[:, None] if ta == 0 else sc[None, :])
    C0 = rng.standard_normal((M, N))
    opA = masked(As, ma) if ta == 0 else masked(As, ma).T
    opB = masked(Bs, mb) if tb == 0 else masked(Bs, mb).T
    opA, opB = np.asfortranarray(opA), np.asfortranarray(opB)
    P = np.asfortranarray(np.zeros((M, N)))
    oracle_lib.gemm_dd(0, M, N, K, opA, M, opB, K, P, M)
    exp = alpha * P
    if add_diag:
        exp[np.arange(min(M, N)), np.arange(min(M, N))] += 1.0
    bmask = np.ones((M, 1))
    bmask[:zero_rows] = 0.0
    exp = exp + beta * C0 * bmask
    dA = L.to_device_colmajor(np.asfortranarray(As))
    dB = L.to_device_colmajor(np.asfortranarray(Bs))
    dC = L.to_device_colmajor(np.asfortranarray(C0))
    part, plen = None, 0
    if split:
        plen = 64 * M * N
        part = torch.empty(plen, dtype=torch.float64, device="cuda")
        assert L.prim_ozgemm_splits(M, N, K, plen) > 1
    assert L.prim_ozgemm(M, N, K, dA, As.shape[0], ta, ma, dB, Bs.shape[0], tb, mb, dC, M, alpha, beta,
                         zero_rows, add_diag, upper_only, part, plen) == 0
    torch.cuda.synchronize()
    got = L.from_device(dC)
    aA, aB = np.abs(opA), np.abs(opB)
    bound = abs(alpha) * 2.0 ** -50 * (np.outer(aA.max(axis=1), aB.sum(axis=0)) + np.outer(aA.sum(axis=1), aB.max(axis=0)))
    bound += 4 * U * (np.abs(alpha * P) + np.abs(beta * C0)) + (aA @ aB) * abs(alpha) * (64 * U if split else 0.0)
    if upper_only:
        keep = np.triu(np.ones((M, N), dtype=bool))
        assert np.array_equal(got[~keep], C0[~keep])
        got, exp, bound = got[keep], exp[keep], bound[keep]
    err = np.abs(got - exp)
    assert np.all(err <= bound + 1e-300), (err / (bound + 1e-300)).max()
    assert L.gpu_status() == 0


@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_ozgemm_transposes(gpu_lib, oracle_lib, ta, tb):
    run_case(gpu_lib, oracle_lib, 200, 100, 300, ta, tb, 0, 0, 1.0, 0.0, seed=ta * 2 + tb)


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (128, 64, 32), (129, 65, 33), (300, 70, 7), (64, 500, 1000)])
def test_ozgemm_shapes(gpu_lib, oracle_lib, M, N, K):
    run_case(gpu_lib, oracle_lib, M, N, K, 1, 0, 0, 0, -1.0, 1.0, seed=M + N + K)


def test_ozgemm_masks_and_epilogue(gpu_lib, oracle_lib):
    # the block-reflector shapes: W = V^T C (V unit lower, transposed) and C -= V W
    run_case(gpu_lib, oracle_lib, 96, 200, 700, 1, 0, 1, 0, 1.0, 0.0, seed=3)
    run_case(gpu_lib, oracle_lib, 700, 200, 96, 0, 0, 1, 0, -1.0, 1.0, seed=4)
    run_case(gpu_lib, oracle_lib, 150, 150, 150, 0, 1, 2, 3, 0.5, -2.0, zero_rows=7, add_diag=1, seed=5)
    run_case(gpu_lib, oracle_lib, 150, 150, 150, 1, 0, 4, 0, 1.0, 1.0, upper_only=1, seed=6)


def test_ozgemm_split_k_and_scaled_rows(gpu_lib, oracle_lib):
    run_case(gpu_lib, oracle_lib, 128, 64, 20000, 1, 0, 0, 0, 1.0, 0.0, split=True, seed=7)
    run_case(gpu_lib, oracle_lib, 256, 128, 3000, 0, 0, 0, 0, 1.0, 1.0, seed=8, scale_rows=True)


def test_split_precision_recursive_qr(gpu_lib, oracle_lib):
    """The recursive Householder QR with its large products on the tensor
    cores: accuracy gates and agreement with the oracle."""
    import torch

    import lila_cases as C

    L = gpu_lib
    m, n, mt, nx = 3000, 1200, 128, 128
    A = np.asfortranarray(np.random.default_rng(11).standard_normal((m, n)))
    lp = [0, 1, 1, nx]
    dA = L.to_device_colmajor(A)
    dT, dQ = L.colmajor(mt, n, fill=0.0), L.colmajor(m, n, fill=0.0)
    lw = L.query_dgeqrf_w03_recursive(lp, m, n, 0, mt, None, m, None, mt, None, m, None, -1)
    W = torch.empty(lw, dtype=torch.float64, device="cuda")
    prev = L.gpu_set_precision(1)
    try:
        l0 = L.launch_count()
        L.trace(True)
        assert L.dgeqrf_w03_recursive(lp, m, n, 0, mt, dA, m, dT, mt, dQ, m, W, lw) == 0
        torch.cuda.synchronize()
        tr = L.trace_summary()
        L.trace(False)
    finally:
        L.gpu_set_precision(prev)
    assert "ozgemm" in tr and tr["ozgemm"][0] > 0
    Ag, Qg = L.from_device(dA), L.from_device(dQ)
    R = np.triu(Ag[:n])
    tol = 50 * n * U
    assert np.linalg.norm(Qg @ R - A) / np.linalg.norm(A) < tol
    assert np.linalg.norm(np.eye(n) - Qg.T @ Qg) < tol
    lib = __import__("oracle").load("oracle_ob") or __import__("oracle").load("oracle")
    Ao = A.copy(order="F")
    To = np.asfortranarray(np.zeros((mt, n)))
    Qo = np.asfortranarray(np.zeros((m, n)))
    work = np.zeros(8 * m * mt + 4 * n * n)
    lib.dgeqrf_w03_recursive(C.lparam(1, 1, nx), m, n, 0, mt, Ao, m, To, mt, Qo, m, work, work.size)
    assert C.max_rel(Ag, Ao) < C.TOL
    assert C.max_rel(Qg, Qo) < C.TOL
    assert L.gpu_status() == 0
