"""Batched least squares (one persistent launch over uneven instances) against
the oracle's least-squares restatement (least-squares/main_ls_qr3.c:94-119)
and the instances' known solutions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch(count, seed, mmax=600, nmax=48, kmax=1e8, nrhs=4):
    rng = np.random.default_rng(seed)
    probs = []
    for t in range(count):
        while True:
            m = int(rng.integers(16, mmax + 1))
            n = int(rng.integers(2, nmax + 1))
            if m >= 2 * n:
                break
        kappa = 10 ** rng.uniform(1, np.log10(kmax))
        U, _ = np.linalg.qr(rng.standard_normal((m, n)))
        V, _ = np.linalg.qr(rng.standard_normal((n, n)))
        sig = kappa ** (-np.arange(n) / max(1, n - 1))
        A = np.asfortranarray((U * sig) @ V.T)
        xs = rng.standard_normal((n, nrhs))
        b = np.asfortranarray(A @ xs + 1e-10 * rng.standard_normal((m, nrhs)))
        probs.append((A, b, xs, kappa))
    return probs


def test_batched_ls_against_oracle_and_truth(gpu_lib, oracle_lib):
    import torch

    L = gpu_lib
    nrhs = 4
    probs = make_batch(300, 7)
    dA = [L.to_device_colmajor(A) for A, _, _, _ in probs]
    dB = [L.to_device_colmajor(b) for _, b, _, _ in probs]
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    work_bytes = L.lib().lila_query_dgels_batched(len(probs))
    work = torch.empty(work_bytes, dtype=torch.uint8, device="cuda")
    info = torch.full((len(probs),), -1, dtype=torch.int32, device="cuda")
    assert L.dgels_batched_prepare(len(probs), ms, ns, nrhs, dA, ms, dB, ms, work, work_bytes) == 0
    assert L.dgels_batched_run(len(probs), nrhs, work, info) == 0
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    worst_fwd = 0.0
    for t, (A, b, xs, kappa) in enumerate(probs):
        m, n = A.shape
        x = L.from_device(dB[t])[:n]
        # the oracle's restatement of the reference driver on the same data
        Ao, bo = A.copy(order="F"), b.copy(order="F")
        T = np.asfortranarray(np.zeros((n, n)))
        oracle_lib.ls_solve(m, n, nrhs, Ao, m, T, n, bo, m, np.zeros(n * nrhs))
        xo = bo[:n]
        # same algorithm: agreement within a few kappa u
        assert np.abs(x - xo).max() / np.abs(xo).max() <= 64 * kappa * 2.0 ** -53 + 1e-13, t
        # and R matches the oracle's R up to rounding
        Rg = np.triu(L.from_device(dA[t])[:n])
        assert np.abs(np.abs(np.diag(Rg)) - np.abs(np.diag(Ao[:n, :n]))).max() <= 1e-12 * np.abs(np.diag(Ao)).max()
        # least-squares forward error: kappa u + kappa^2 ||r|| / (||A|| ||x||) (noise 1e-10)
        r = np.linalg.norm(b - A @ xs)
        bound = kappa * 2.0 ** -53 + kappa ** 2 * r / (np.linalg.norm(A, 2) * np.linalg.norm(xs)) + 1e-12
        worst_fwd = max(worst_fwd, np.abs(x - xs).max() / np.abs(xs).max() / bound)
    assert worst_fwd < 1e3


def test_batched_ls_graph_replay_and_rank_deficiency(gpu_lib):
    import torch

    L = gpu_lib
    nrhs = 2
    probs = make_batch(40, 8, mmax=300, nmax=20, nrhs=nrhs)
    # an exactly rank-deficient instance: a zero column
    A0 = probs[5][0].copy(order="F")
    A0[:, 3] = 0.0
    probs[5] = (A0, probs[5][1], probs[5][2], probs[5][3])
    saved = [(A.copy(order="F"), b.copy(order="F")) for A, b, _, _ in probs]
    dA = [L.to_device_colmajor(A) for A, _, _, _ in probs]
    dB = [L.to_device_colmajor(b) for _, b, _, _ in probs]
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    nb = L.lib().lila_query_dgels_batched(len(probs))
    work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    info = torch.zeros(len(probs), dtype=torch.int32, device="cuda")
    assert L.dgels_batched_prepare(len(probs), ms, ns, nrhs, dA, ms, dB, ms, work, nb) == 0
    L._use_torch_stream()
    g = L.lib().lila_dgels_batched_graph(len(probs), nrhs, L.dptr(work), L.dptr(info))
    assert g
    results = []
    for rep in range(2):
        for t, (A, b) in enumerate(saved):
            dA[t].copy_(L.to_device_colmajor(A))
            dB[t].copy_(L.to_device_colmajor(b))
        assert L.gpu_graph_launch(g) == 0
        torch.cuda.synchronize()
        results.append([L.from_device(x).copy() for x in dB])
    L.gpu_graph_destroy(g)
    for t in range(len(probs)):
        assert np.array_equal(results[0][t], results[1][t], equal_nan=True)
    inf = info.cpu().numpy()
    assert inf[5] != 0 and np.all(np.delete(inf, 5) == 0)
