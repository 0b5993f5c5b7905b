"""lila_dormqrf_w03_noalloc: the block-reflector update for callers that cannot
allocate device memory (its scratch is a fixed device array).  Checked
through the C ABI against lila_dormqrf_w03 with a caller workspace and against
the oracle, on two calls in a row (the shared scratch keeps the first call's
contents); repeated calls leave the device's free memory and torch's
allocator unchanged; the split-precision products (large enough to run on the
tensor cores, with the rest of the array as their split-K space) agree with
the workspace entry point too."""
import numpy as np
import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu


def _factored(oracle_lib, m, n, ii, mt, seed):
    return C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, 1, 1, 7, seed=seed)


def _case(L, oracle_lib, m, n, ii, mt, nc, seed, precision=0):
    import torch

    A, T, Q = _factored(oracle_lib, m, n, ii, mt, seed)
    rng = np.random.default_rng(100 + seed)
    Aw = np.asfortranarray(np.hstack([A, rng.standard_normal((m, nc))]))
    j = n + ii
    d_ref, d_new = L.to_device_colmajor(Aw), L.to_device_colmajor(Aw)
    dT = L.to_device_colmajor(T)
    lw = L.query_dormqrf_w03(m, nc, n, ii, j, mt, None, m, None, mt, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    prev = L.gpu_set_precision(precision)
    try:
        assert L.dormqrf_w03(m, nc, n, ii, j, mt, d_ref, m, dT, mt, dW, lw) == 0
        assert L.dormqrf_w03_noalloc(m, nc, n, ii, j, mt, d_new, m, dT, mt) == 0
        torch.cuda.synchronize()
    finally:
        L.gpu_set_precision(prev)
    Ao = Aw.copy(order="F")
    work = np.zeros(8 * m * (nc + mt))
    oracle_lib.dormqrf_w03(m, nc, n, ii, j, mt, Ao, m, T, mt, work, work.size)
    return L.from_device(d_ref), L.from_device(d_new), Ao


def test_noalloc_matches_workspace_entry_point(gpu_lib, oracle_lib):
    L = gpu_lib
    for call, (m, n, ii, mt, nc, seed) in enumerate([(300, 70, 5, 16, 40, 21), (2000, 96, 0, 32, 64, 22)]):
        ref, got, orc = _case(L, oracle_lib, m, n, ii, mt, nc, seed)
        assert C.max_rel(got, ref) < C.TOL, call
        assert C.max_rel(got, orc) < C.TOL, call
    assert L.gpu_status() == 0


def test_noalloc_allocates_nothing(gpu_lib, oracle_lib):
    """The second and third calls (the first may make the driver load the
    library's kernels) change neither the device's free memory nor torch's
    allocator."""
    import torch

    L = gpu_lib
    m, n, ii, mt, nc = 1500, 64, 0, 32, 48
    A, T, Q = _factored(oracle_lib, m, n, ii, mt, 23)
    Aw = np.asfortranarray(np.hstack([A, np.random.default_rng(5).standard_normal((m, nc))]))
    dA, dT = L.to_device_colmajor(Aw), L.to_device_colmajor(T)
    assert L.dormqrf_w03_noalloc(m, nc, n, ii, n, mt, dA, m, dT, mt) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for _ in range(2):
        assert L.dormqrf_w03_noalloc(m, nc, n, ii, n, mt, dA, m, dT, mt) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0
    assert L.gpu_status() == 0


def test_noalloc_split_precision(gpu_lib, oracle_lib):
    """Products of 128 x 256 x 16384 (above the 2^27 threshold of the
    split-precision GEMM) with the leftover array as split-K space; two calls
    in a row."""
    L = gpu_lib
    for seed in (24, 25):
        ref, got, orc = _case(L, oracle_lib, 16384, 128, 0, 128, 256, seed, precision=1)
        assert C.max_rel(got, ref) < 1e-12
        assert C.max_rel(got, orc) < 1e-11
    assert L.gpu_status() == 0


def test_noalloc_rejects_oversized_problems(gpu_lib):
    import torch

    L = gpu_lib
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    # 2 * min(mt, k) * n = 2 * 512 * 1024 doubles > 524288
    assert L.dormqrf_w03_noalloc(4096, 1024, 512, 0, 512, 512, d, 4096, d, 512) == -101
