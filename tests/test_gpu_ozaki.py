"""Split-precision (Ozaki) tensor-core products against double-double references.

The kernels represent each scaling group (a column of A for the Gram, a row
of A and a column of X for the row map) in 56-bit fixed point relative to the
group's largest entry, so the error of an entry of a product is bounded by
2^-50 (max_k |a_ik| sum_k |b_kj| + sum_k |a_ik| max_k |b_kj|): FP64 grade for
entries of comparable size, like a FP64 GEMM's gamma_K |A||B| bound."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tcgen05_tile_exact(gpu_lib):
    import torch

    L = gpu_lib
    rng = np.random.default_rng(0)
    for N in (64, 128, 256):
        A = rng.integers(-8, 9, (128, 64)).astype(np.float32)
        B = rng.integers(-8, 9, (N, 64)).astype(np.float32)
        dA = torch.from_numpy(A).to(torch.bfloat16).cuda()
        dB = torch.from_numpy(B).to(torch.bfloat16).cuda()
        dD = torch.full((128, N), -1.0, dtype=torch.float32, device="cuda")
        assert L.prim_tc_selftest(dA, dB, dD, N, 0) == 0
        torch.cuda.synchronize()
        assert np.array_equal(dD.cpu().numpy(), A @ B.T)
    assert L.gpu_status() == 0


def _graded(rng, m, n, decades=6.0):
    A = rng.standard_normal((m, n)) * (10.0 ** (-decades * np.arange(n) / max(1, n - 1)))[None, :]
    return np.asfortranarray(A)


@pytest.mark.parametrize("m,n", [(100003, 64), (7777, 37), (64, 64), (1, 5), (300000, 64)])
def test_ozaki_gram(gpu_lib, oracle_lib, m, n):
    import torch

    L = gpu_lib
    rng = np.random.default_rng(m + n)
    A = _graded(rng, m, n)
    if n > 3:
        A[:, 2] = 0.0  # an all-zero column
    G = np.asfortranarray(np.zeros((n, n)))
    oracle_lib.gemm_dd(1, n, n, m, A, m, A, m, G, n)
    dA = L.to_device_colmajor(A)
    dG = L.colmajor(n, n, fill=0.0)
    lw = L.lib().lila_prim_ozaki_gram_work()
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.prim_ozaki_gram(m, n, dA, m, dG, n, dW, lw) == 0
    torch.cuda.synchronize()
    Gg = L.from_device(dG)
    absA = np.abs(A)
    cmax = absA.max(axis=0)
    csum = absA.sum(axis=0)
    bound = np.outer(cmax, csum) + np.outer(csum, cmax)
    err = np.abs(Gg - G)
    assert np.all(err <= 2.0 ** -50 * bound + 1e-300), err.max()
    assert L.gpu_status() == 0


@pytest.mark.parametrize("m,n,nout", [(50000, 64, 64), (1000, 30, 17), (129, 64, 64), (300000, 64, 64)])
def test_ozaki_map(gpu_lib, oracle_lib, m, n, nout):
    L = gpu_lib
    rng = np.random.default_rng(m + 3 * n + nout)
    A = _graded(rng, m, n, 4.0)
    A[7 % m, :] = 0.0  # an all-zero row
    X = np.asfortranarray(np.triu(rng.standard_normal((n, nout))) * 10.0 ** rng.uniform(-3, 3, (1, nout)))
    ref = np.asfortranarray(np.zeros((m, nout)))
    oracle_lib.gemm_dd(0, m, nout, n, A, m, X, n, ref, m)
    dA, dX = L.to_device_colmajor(A), L.to_device_colmajor(X)
    dO = L.colmajor(m, nout, fill=0.0)
    assert L.prim_ozaki_map(m, n, dA, m, dX, n, nout, dO, m) == 0
    got = L.from_device(dO)
    rmax = np.abs(A).max(axis=1)
    bound = np.outer(rmax, np.abs(X).sum(axis=0)) + np.outer(np.abs(A).sum(axis=1), np.abs(X).max(axis=0))
    err = np.abs(got - ref)
    assert np.all(err <= 2.0 ** -50 * bound + 1e-300), err.max()
    # in place: out = A (first nout columns)
    if nout == n:
        assert L.prim_ozaki_map(m, n, dA, m, dX, n, nout, dA, m) == 0
        got2 = L.from_device(dA)
        assert np.array_equal(got2, got)
    assert L.gpu_status() == 0
