"""TSQR reduction-tree leaf: accuracy at any condition number, reflector
consistency, and parity with the oracle (Householder QR after sign
normalisation; Cholesky QR + reconstruction on a well-conditioned block)."""
import numpy as np
import pytest

import lila_cases as C
from test_gpu_mixed import reflectors_reproduce_q, usv

pytestmark = pytest.mark.gpu


def run_tsqr(L, A, mt, mb=0, arity=0, i=0):
    import torch

    m = A.shape[0]
    n = A.shape[1] - i
    dA = L.to_device_colmajor(A)
    dT = L.colmajor(mt, n + i, fill=0.0)
    dQ = L.colmajor(m, n + i, fill=0.0)
    lw = L.query_dgeqrf_w03_tsqr(mb if mb else 256, arity if arity else 4, m, n, i, mt)
    lw = max(lw, L.query_dgeqrf_w03_tsqr(128, 2, m, n, i, mt))
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    rc = L.dgeqrf_w03_tsqr(mb, arity, m, n, i, mt, dA, m, dT, mt, dQ, m, dW, lw)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return dA, dT, dQ


@pytest.mark.parametrize("kappa", [1e2, 1e10, 1e15])
@pytest.mark.parametrize("mb,arity", [(256, 4), (128, 2), (64, 3)])
def test_tsqr_accuracy(gpu_lib, kappa, mb, arity):
    L = gpu_lib
    L.gpu_clear_status()
    m, n, mt = 100003, 64, 32
    A = usv(m, n, kappa, 31, 32)
    dA, dT, dQ = run_tsqr(L, A, mt, mb, arity)
    Ag, Qg = L.from_device(dA), L.from_device(dQ)
    R = np.triu(Ag[:n, :n])
    tol = 50 * n * 2.0 ** -53
    assert np.linalg.norm(Qg @ R - A) / np.linalg.norm(A) <= tol
    assert np.linalg.norm(np.eye(n) - Qg.T @ Qg) <= tol
    assert reflectors_reproduce_q(L, dA, dT, dQ, m, n, mt) < 1e-12
    assert L.gpu_status() == 0


def test_tsqr_matches_oracle(gpu_lib, oracle_lib):
    L = gpu_lib
    m, n, i, mt = 9000, 40, 5, 16
    rng = np.random.default_rng(17)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, n + i)))
    dA, dT, dQ = run_tsqr(L, A, mt, 128, 2, i=i)
    Ao, To, Qo = A.copy(order="F"), np.asfortranarray(np.zeros((mt, n + i))), np.asfortranarray(np.zeros((m, n + i)))
    work = np.zeros(oracle_lib.query_dgeqrf_w03_mt_hr(m, n, i, mt) + 16)
    oracle_lib.dgeqrf_w03_mt_hr(m, n, i, mt, Ao, m, To, mt, Qo, m, work, work.size)
    err = C.compare_factor((L.from_device(dA), L.from_device(dT), L.from_device(dQ)), (Ao, To, Qo), m, n, i, mt)
    assert max(err.values()) < 1e-12, err
    # R and Q against Householder QR after sign normalisation
    Ag, Qg = L.from_device(dA), L.from_device(dQ)
    Rg = np.triu(Ag[i:i + n, i:i + n])
    Ah = A[i:, i:].copy(order="F")
    Th = np.asfortranarray(np.zeros((mt, n)))
    Qh = np.asfortranarray(np.zeros((m - i, n)))
    w2 = np.zeros(8 * m * mt + 4 * n * n)
    oracle_lib.dgeqrf_w03_recursive(C.lparam(1, 1, 16), m - i, n, 0, mt, Ah, m - i, Th, mt, Qh, m - i, w2, w2.size)
    Rh = np.triu(Ah[:n, :n])
    sg, sh = np.sign(np.diag(Rg)), np.sign(np.diag(Rh))
    assert C.max_rel(Rg * sg[:, None], Rh * sh[:, None]) < 1e-12
    assert C.max_rel(Qg[i:, i:] * sg[None, :], Qh * sh[None, :]) < 1e-12


def test_tsqr_autotune(gpu_lib):
    import torch

    L = gpu_lib
    m, n, mt = 50000, 64, 32
    A = usv(m, n, 1e4, 41, 42)
    dA, dQ = L.to_device_colmajor(A), L.colmajor(m, n, fill=0.0)
    dT = L.colmajor(mt, n, fill=0.0)
    lw = max(L.query_dgeqrf_w03_tsqr(128, 2, m, n, 0, mt), L.query_dgeqrf_w03_tsqr(256, 4, m, n, 0, mt))
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    code = L.gpu_tsqr_autotune(m, n, dA, m, dT, mt, dQ, m, dW, lw)
    assert code // 100 in (128, 256) and code % 100 in (2, 4)
    dA2, dT2, dQ2 = run_tsqr(L, A, mt)  # uses the tuned (mb, arity)
    Qg = L.from_device(dQ2)
    assert np.linalg.norm(np.eye(n) - Qg.T @ Qg) <= 50 * n * 2.0 ** -53
