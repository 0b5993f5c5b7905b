"""On-device accuracy check and FP64 fallback of the split-precision tall-skinny
leaf (lila_dgeqrf_w03_mt_hr_mixed), and non-finite input.

The check measures ||I - Q^T Q||_F and ||A - Q R||_F / ||A||_F of the leaf's
result (the measures of lila_test_qq_orth_1 / lila_test_qr_repres_1,
lila-c-lila_param/lila/src/lila_test_qq_orth_1.c:3-19,
lila_test_qr_repres_1.c:3-27) against 50 n 2^-53; a failure re-solves the
leaf in FP64 through the TSQR leaf.  Exactly rank-deficient input and a
condition number beyond 1/u exercise the fallback; NaN / Inf input must be
reported (status bit, positive return) without a trap.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M, N, MT = 200000, 64, 32
TOL = 50 * N * 2.0 ** -53


def usv(m, n, sig, seed_u=201, seed_v=202):
    rng = np.random.default_rng(seed_u)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    rv = np.random.default_rng(seed_v)
    V, Rv = np.linalg.qr(rv.standard_normal((n, n)))
    V = V * np.sign(np.diag(Rv))[None, :]
    return np.asfortranarray((U * sig[None, :]) @ V.T)


def logspaced(kappa, n=N):
    return kappa ** (-np.arange(n) / (n - 1))


def run(L, A, lwork=None):
    import torch

    m, n = A.shape
    dA = L.to_device_colmajor(A)
    dT = L.colmajor(MT, n, fill=0.0)
    dQ = L.colmajor(m, n, fill=0.0)
    lw = L.query_dgeqrf_w03_mt_hr_mixed(m, n, 0, MT, None, m, None, MT, None, m, None, -1)
    if lwork is not None:
        lw = lwork
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    rc = L.dgeqrf_w03_mt_hr_mixed(m, n, 0, MT, dA, m, dT, MT, dQ, m, dW, lw)
    torch.cuda.synchronize()
    return rc, L.from_device(dA), L.from_device(dT), L.from_device(dQ)


def gates(A, Af, Q):
    n = A.shape[1]
    R = np.triu(Af[:n, :n])
    return np.linalg.norm(Q @ R - A) / np.linalg.norm(A), np.linalg.norm(np.eye(n) - Q.T @ Q)


def test_check_values_track_the_true_measures(gpu_lib):
    L = gpu_lib
    L.gpu_clear_status()
    A = usv(M, N, logspaced(1e6))
    for level in (1, 2):
        prev = L.gpu_set_check(level)
        try:
            rc, Af, _, Q = run(L, A)
        finally:
            L.gpu_set_check(prev)
        assert rc == 0
        res, orth = gates(A, Af, Q)
        cres, corth = L.gpu_last_check()
        print("level %d res %.3g (check %.3g) orth %.3g (check %.3g)" % (level, res, cres, orth, corth))
        assert res <= TOL and orth <= TOL
        assert 0.0 <= cres <= TOL and 0.0 <= corth <= TOL
        # the orthogonality measure agrees with the host's to the rounding of
        # the final map (level 1) or of the Gram (level 2)
        assert abs(corth - orth) < 2e-14
        # the sampled residual is an estimate of the same order
        assert cres < 20 * res + 1e-15
        assert L.gpu_last_fallback() == 0
    prev = L.gpu_set_check(0)
    try:
        assert run(L, A)[0] == 0
        assert L.gpu_last_check() == (-1.0, -1.0)
    finally:
        L.gpu_set_check(prev)
    assert L.gpu_status() == 0


def zero_column_input():
    """Exactly rank deficient with no rounding noise in the null direction:
    sigma_n = 0 and V = I, so the last column is exactly zero.  Every shifted
    pass keeps that column of the candidate exactly zero, so the passes never
    reach two unshifted ones and the leaf must fall back."""
    rng = np.random.default_rng(7)
    U, _ = np.linalg.qr(rng.standard_normal((M, N)))
    sig = logspaced(1e6)
    sig[-1] = 0.0
    return np.asfortranarray(U * sig[None, :])


@pytest.mark.parametrize("case", ["zero_column", "sigma_n_zero", "kappa_1e17"])
def test_fallback_meets_the_gates(gpu_lib, case):
    L = gpu_lib
    L.gpu_clear_status()
    if case == "zero_column":
        A = zero_column_input()
    elif case == "sigma_n_zero":
        sig = logspaced(1e12)
        sig[-1] = 0.0  # sigma_n = 0 with a Haar V (rank deficient up to the rounding of A)
        A = usv(M, N, sig, seed_u=7, seed_v=8)
    else:
        A = usv(M, N, logspaced(1e17), seed_u=7, seed_v=8)
    rc, Af, T, Q = run(L, A)
    res, orth = gates(A, Af, Q)
    cres, corth = L.gpu_last_check()
    fb = L.gpu_last_fallback()
    print("%s: rc %d fallback %d passes %d res %.3g orth %.3g (check %.3g %.3g)" % (
        case, rc, fb, L.gpu_last_passes(), res, orth, cres, corth))
    assert rc == 0
    assert res <= TOL and orth <= TOL, (res, orth)
    assert 0.0 <= cres <= TOL and 0.0 <= corth <= TOL
    if case == "zero_column":
        assert fb == 1
    assert L.gpu_status() == 0
    # the reflectors reproduce the returned Q: H^T (Q S) = [I; 0]
    import torch

    dA, dT, dB = L.to_device_colmajor(Af), L.to_device_colmajor(T), L.to_device_colmajor(Q)
    lw = L.query_dormqrf_w03(M, N, N, 0, 0, MT, None, M, None, MT, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dormqrf_z03(M, N, N, 0, 0, MT, dA, M, dT, MT, dB, M, dW, lw) == 0
    B = L.from_device(dB)
    B[:N] -= np.eye(N)
    assert np.abs(B).max() < 1e-12


def test_failure_without_fallback_workspace_is_reported(gpu_lib):
    """With only the leaf's own workspace the failed check is not re-solved:
    LILA_ST_CHECK_FAILED and a positive return."""
    L = gpu_lib
    L.gpu_clear_status()
    A = zero_column_input()
    full = L.query_dgeqrf_w03_mt_hr_mixed(M, N, 0, MT, None, M, None, MT, None, M, None, -1)
    small = L.query_dgeqrf_w03_mt_hr_mixed(1000, N, 0, MT, None, 1000, None, MT, None, 1000, None, -1)
    assert small < full
    rc, _, _, _ = run(L, A, lwork=small)
    assert rc == 1
    assert L.gpu_status() & 8  # LILA_ST_CHECK_FAILED
    assert L.gpu_last_fallback() == 0
    L.gpu_clear_status()


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_input_is_reported(gpu_lib, bad):
    L = gpu_lib
    L.gpu_clear_status()
    A = usv(20000, N, logspaced(1e2))
    A[1234, 17] = bad
    rc, _, _, _ = run(L, A)
    st = L.gpu_status()
    assert rc == 1
    assert st & 4  # LILA_ST_NONFINITE
    assert st & 8  # LILA_ST_CHECK_FAILED
    assert not st & 16  # no wait gave up
    # the context stays usable: a clean call afterwards succeeds
    L.gpu_clear_status()
    A2 = usv(20000, N, logspaced(1e2))
    rc, Af, _, Q = run(L, A2)
    assert rc == 0
    res, orth = gates(A2, Af, Q)
    assert res <= TOL and orth <= TOL
    assert L.gpu_status() == 0
