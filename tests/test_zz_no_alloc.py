"""lila_dormqrf_w03_noalloc: the block-reflector update for callers that cannot
allocate device memory (its scratch is a fixed device array).  Checked
through the C ABI against lila_dormqrf_w03 with a caller workspace, on two
calls in a row (the shared scratch keeps the first call's contents)."""
import numpy as np
import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu


def _factored(oracle_lib, m, n, ii, mt, seed):
    return C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, 1, 1, 7, seed=seed)


def test_noalloc_matches_workspace_entry_point(gpu_lib, oracle_lib):
    import torch

    L = gpu_lib
    for call, (m, n, ii, mt, nc, seed) in enumerate([(300, 70, 5, 16, 40, 21), (2000, 96, 0, 32, 64, 22)]):
        A, T, Q = _factored(oracle_lib, m, n, ii, mt, seed)
        rng = np.random.default_rng(100 + call)
        Aw = np.asfortranarray(np.hstack([A, rng.standard_normal((m, nc))]))
        j = n + ii
        d_ref, d_new = L.to_device_colmajor(Aw), L.to_device_colmajor(Aw)
        dT = L.to_device_colmajor(T)
        lw = L.query_dormqrf_w03(m, nc, n, ii, j, mt, None, m, None, mt, None, -1)
        dW = torch.empty(lw, dtype=torch.float64, device="cuda")
        assert L.dormqrf_w03(m, nc, n, ii, j, mt, d_ref, m, dT, mt, dW, lw) == 0
        assert L.dormqrf_w03_noalloc(m, nc, n, ii, j, mt, d_new, m, dT, mt) == 0
        torch.cuda.synchronize()
        ref, got = L.from_device(d_ref), L.from_device(d_new)
        assert C.max_rel(got, ref) < C.TOL, call
    assert L.gpu_status() == 0


def test_noalloc_rejects_oversized_problems(gpu_lib):
    import torch

    L = gpu_lib
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    # 2 * min(mt, k) * n = 2 * 512 * 1024 doubles > 524288
    assert L.dormqrf_w03_noalloc(4096, 1024, 512, 0, 512, 512, d, 4096, d, 512) == -101
