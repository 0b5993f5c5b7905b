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


@pytest.mark.parametrize("path", [0, 1], ids=["tma", "regs"])
@pytest.mark.parametrize("m,n", [(100003, 64), (100004, 64), (7777, 37), (7778, 37), (64, 64), (1, 5),
                                 (300000, 64)])
def test_ozaki_gram(gpu_lib, oracle_lib, m, n, path):
    L = gpu_lib
    prev = L.prim_ozaki_map_path(path)
    try:
        _check_gram(L, oracle_lib, m, n)
    finally:
        L.prim_ozaki_map_path(prev)


def _check_gram(L, oracle_lib, m, n):
    import torch

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


@pytest.mark.parametrize("path", [0, 1, 2, 3], ids=["default", "regs", "tma_fp64asm", "tma_intasm"])
@pytest.mark.parametrize("m,n,nout", [(50000, 64, 64), (1000, 30, 17), (129, 64, 64), (300000, 64, 64)])
def test_ozaki_map(gpu_lib, oracle_lib, m, n, nout, path):
    L = gpu_lib
    prev = L.prim_ozaki_map_path(path)
    try:
        _check_map(L, oracle_lib, m, n, nout)
    finally:
        L.prim_ozaki_map_path(prev)


def _check_map(L, oracle_lib, m, n, nout):
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


@pytest.mark.parametrize("m,n,nout,lda,off", [
    (50000, 64, 64, 50000, 0),     # full tiles of both halves
    (4097, 20, 33, 4100, 0),       # n <= 32: the second half tile lies beyond A
    (77, 64, 64, 80, 0),           # one partial tile
    (33, 64, 64, 34, 0),           # a 32-row tile and one row
    (152 * 32 * 3 + 5, 64, 64, 152 * 32 * 3 + 6, 0),  # every CTA with three tiles, one more row
    (131072 + 55, 48, 64, 131200, 0),
    (9000, 64, 64, 9001, 0),       # odd lda: the register-fed kernel
    (9000, 64, 64, 9002, 1),       # A at an odd offset: not 16-byte aligned
    (9000, 64, 64, 9002, 2),       # A at an even offset: TMA
])
def test_ozaki_map_kernels_agree_bitwise(gpu_lib, m, n, nout, lda, off):
    """The TMA-fed warp-specialised kernel on transposed 32-row tiles (path 3:
    integer assembly of the outputs; path 2: FP64-pipe conversion) and the
    register-fed one (paths 0 and 1) compute the same exact digit products
    (integer sums in FP32 TMEM; the transposed kernel adds its two halves'
    integer partials) and round the same integer to FP64, so their outputs
    are identical bit for bit, in place too."""
    import torch

    L = gpu_lib
    rng = np.random.default_rng(m + n + lda + off)
    buf = np.asfortranarray(rng.standard_normal((lda, n + 1)) * 10.0 ** rng.uniform(-5, 5, (lda, 1)))
    X = np.asfortranarray(rng.standard_normal((n, nout)) * 10.0 ** rng.uniform(-3, 3, (1, nout)))
    dbuf, dX = L.to_device_colmajor(buf), L.to_device_colmajor(X)
    outs = []
    for path in (1, 2, 3):
        prev = L.prim_ozaki_map_path(path)
        try:
            dO = L.colmajor(m, nout, fill=0.0)
            assert L.prim_ozaki_map(m, n, (dbuf, off), lda, dX, n, nout, dO, m) == 0
            outs.append(L.from_device(dO))
            if nout == n:
                dIn = L.to_device_colmajor(buf)
                assert L.prim_ozaki_map(m, n, (dIn, off), lda, dX, n, nout, (dIn, off), lda) == 0
                got = L.from_device(dIn)
                flat = got.reshape(-1, order="F")[off:off + lda * n].reshape((lda, n), order="F")
                assert np.array_equal(flat[:m, :nout], outs[-1])
        finally:
            L.prim_ozaki_map_path(prev)
    torch.cuda.synchronize()
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[0], outs[2])
    assert np.isfinite(outs[0]).all()
    assert L.gpu_status() == 0


@pytest.mark.parametrize("m,n,lda,rows_per", [
    (1048576, 64, 1048576, 0),
    (100004, 64, 100010, 0),
    (7778, 37, 7778, 0),
    (5000, 20, 5002, 0),
    (200000, 64, 200000, 1344),   # every CTA busy, the last one partly
    (200000, 64, 200000, 6400),   # 32 CTAs with rows, the others with none
])
def test_ozaki_gram_kernels_agree_bitwise(gpu_lib, m, n, lda, rows_per):
    """The TMA-fed Gram and the register-fed one sum the same exact integer
    digit products over the same row ranges, so G is identical bit for bit."""
    import torch

    L = gpu_lib
    rng = np.random.default_rng(m + n + lda)
    A = np.asfortranarray(rng.standard_normal((lda, n)) * 10.0 ** rng.uniform(-4, 4, (1, n)))
    A[3::17, :] *= 1e3
    dA = L.to_device_colmajor(A)
    lw = L.lib().lila_prim_ozaki_gram_work()
    outs = []
    for path in (0, 1):
        prev = L.prim_ozaki_map_path(path)
        try:
            dG = L.colmajor(n, n, fill=0.0)
            dW = torch.empty(lw, dtype=torch.float64, device="cuda")
            if rows_per:
                assert L.prim_ozaki_gram_rows(m, n, dA, lda, dG, n, dW, lw, rows_per) == 0
            else:
                assert L.prim_ozaki_gram(m, n, dA, lda, dG, n, dW, lw) == 0
            outs.append(L.from_device(dG))
        finally:
            L.prim_ozaki_map_path(prev)
    assert np.array_equal(outs[0], outs[1])
    assert np.isfinite(outs[0]).all()
    assert L.gpu_status() == 0
