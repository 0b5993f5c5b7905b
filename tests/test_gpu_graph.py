"""Graph mode: repeated calls with identical arguments replay a captured CUDA
graph and give the same results as direct execution."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _recursive_once(L, torch, A, m, n, mt, lp, bufs):
    dA, dT, dQ, W, lw = bufs
    dA.copy_(torch.as_tensor(A.T.copy(), device="cuda").t())
    dT.zero_()
    dQ.zero_()
    assert L.dgeqrf_w03_recursive(lp, m, n, 0, mt, dA, m, dT, mt, dQ, m, W, lw) == 0
    torch.cuda.synchronize()
    return L.from_device(dA), L.from_device(dT), L.from_device(dQ)


def test_graph_replay_matches_direct(gpu_lib):
    import torch

    L = gpu_lib
    m, n, mt = 1500, 300, 32
    lp = [0, 1, 1, 32]
    A = np.asfortranarray(np.random.default_rng(3).standard_normal((m, n)))
    lw = L.query_dgeqrf_w03_recursive(lp, m, n, 0, mt, None, m, None, mt, None, m, None, -1)
    bufs = (L.colmajor(m, n), L.colmajor(mt, n), L.colmajor(m, n),
            torch.empty(lw, dtype=torch.float64, device="cuda"), lw)
    prev = L.gpu_graph_mode(0)
    try:
        ref = _recursive_once(L, torch, A, m, n, mt, lp, bufs)
        L.gpu_graph_mode(1)
        r0 = L.lib().lila_gpu_graph_replays()
        first = _recursive_once(L, torch, A, m, n, mt, lp, bufs)   # captured, then launched
        c0 = L.launch_count()
        second = _recursive_once(L, torch, A, m, n, mt, lp, bufs)  # replayed
        assert L.lib().lila_gpu_graph_replays() == r0 + 1
        assert L.launch_count() - c0 > 100  # a replay counts the graph's kernels
        for a, b, c in zip(ref, first, second):
            assert np.array_equal(a, b) and np.array_equal(a, c)
        # a different lila_param is a different key: captured anew, still correct
        lp2 = [0, 1, 1, 64]
        other = _recursive_once(L, torch, A, m, n, mt, lp2, bufs)
        assert L.lib().lila_gpu_graph_replays() == r0 + 1
        R = np.triu(other[0][:n])
        assert np.linalg.norm(other[2] @ R - A) / np.linalg.norm(A) < 1e-14
        assert L.gpu_status() == 0
    finally:
        L.gpu_graph_mode(prev)
        L.gpu_graph_cache_clear()


def test_uncapturable_call_runs_directly(gpu_lib):
    """The adaptive split-precision leaf synchronises the host; in graph mode
    it still runs (directly) and stays correct."""
    import torch

    from test_gpu_mixed import run_mixed, usv

    L = gpu_lib
    prev = L.gpu_graph_mode(1)
    try:
        m, n = 20000, 48
        A = usv(m, n, 1e10, 5, 6)
        for _ in range(2):
            dA, dT, dQ = run_mixed(L, A, 32)
            Qg = L.from_device(dQ)
            R = np.triu(L.from_device(dA)[:n, :n])
            assert np.linalg.norm(np.eye(n) - Qg.T @ Qg) < 50 * n * 2.0 ** -53
            assert np.linalg.norm(Qg @ R - A) / np.linalg.norm(A) < 50 * n * 2.0 ** -53
        assert L.gpu_status() == 0
    finally:
        L.gpu_graph_mode(prev)
        L.gpu_graph_cache_clear()
