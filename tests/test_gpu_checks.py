"""On-device accuracy checks (lila_test_qq_orth_1, lila_test_qr_repres_1)
against the oracle's restatement of the packaged library's metrics."""
import numpy as np
import pytest

from test_gpu_mixed import run_mixed, usv

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,i", [(50000, 64, 0), (3000, 90, 7)])
def test_checks_match_oracle(gpu_lib, oracle_lib, m, n, i):
    L = gpu_lib
    rng = np.random.default_rng(m + n)
    A0 = np.asfortranarray(rng.standard_normal((m, n + i)))
    # a slightly non-orthonormal Q and an R so that both metrics are far from 0
    Q = np.asfortranarray(np.linalg.qr(A0)[0] + 1e-9 * rng.standard_normal((m, n + i)))
    R = np.asfortranarray(np.triu(rng.standard_normal((n + i, n + i))))
    dQ, dA, dR = L.to_device_colmajor(Q), L.to_device_colmajor(A0), L.to_device_colmajor(R)
    o = L.test_qq_orth_1(m, n, i, dQ, m)
    oo = oracle_lib.test_qq_orth_1(m, n, i, Q, m)
    assert abs(o - oo) <= 1e-12 * max(1.0, oo), (o, oo)
    r = L.test_qr_repres_1(m, n, i, dA, m, dQ, m, dR, n + i)
    ro = oracle_lib.test_qr_repres_1(m, n, i, A0, m, Q, m, R, n + i)
    assert abs(r - ro) <= 1e-12 * max(1.0, ro), (r, ro)


def test_checks_on_a_factorization(gpu_lib, oracle_lib):
    L = gpu_lib
    m, n, mt = 100000, 64, 32
    A = usv(m, n, 1e6, 3, 4)
    dA, dT, dQ = run_mixed(L, A, mt)
    dA0 = L.to_device_colmajor(A)
    orth = L.test_qq_orth_1(m, n, 0, dQ, m)
    res = L.test_qr_repres_1(m, n, 0, dA0, m, dQ, m, dA, m)
    Qg = L.from_device(dQ)
    R = np.asfortranarray(np.triu(L.from_device(dA)[:n, :n]))
    # references from double-double products (an FP64 GEMM over 1e5 rows has
    # summation errors of the size of the metrics themselves); forming Q^T Q
    # or Q R in FP64 quantises the metrics by about sqrt(n) 2^-53 either way
    G = np.asfortranarray(np.zeros((n, n)))
    oracle_lib.gemm_dd(1, n, n, m, Qg, m, Qg, m, G, n)
    C = np.asfortranarray(np.zeros((m, n)))
    oracle_lib.gemm_dd(0, m, n, n, Qg, m, R, n, C, m)
    orth_dd = np.linalg.norm(np.eye(n) - G)
    res_dd = np.linalg.norm(C - A) / np.linalg.norm(A)
    assert abs(orth - orth_dd) <= 2 * np.sqrt(n) * 2.0 ** -53, (orth, orth_dd)
    assert abs(res - res_dd) <= 4 * 2.0 ** -53, (res, res_dd)
    assert orth < 50 * n * 2.0 ** -53 and res < 50 * n * 2.0 ** -53
