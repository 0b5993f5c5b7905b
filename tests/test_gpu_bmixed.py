"""Batched least squares with per-instance variants (lila_gels_mixed_*):
Cholesky QR 2 / shifted Cholesky QR 3 on FP64-grade tensor-core products with
the on-device orthogonality check, and the FP64 Householder fallback, against
the oracle's restatement of the reference least-squares driver
(least-squares/main_ls_qr3.c:94-119) and the instances' known solutions; the
selector inputs against the CPU restatement in oracle/selector.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U53 = 2.0 ** -53


def make_batch(count, seed, mmax=700, nmax=56, kmax=1e15, nrhs=4, p_rankdef=0.05):
    rng = np.random.default_rng(seed)
    probs = []
    for t in range(count):
        while True:
            m = int(rng.integers(64, mmax + 1))
            n = int(rng.integers(4, nmax + 1))
            if m >= 2 * n:
                break
        kappa = 10 ** rng.uniform(1, np.log10(kmax))
        U, _ = np.linalg.qr(rng.standard_normal((m, n)))
        V, _ = np.linalg.qr(rng.standard_normal((n, n)))
        sig = kappa ** (-np.arange(n) / max(1, n - 1))
        rankdef = rng.random() < p_rankdef
        if rankdef:
            sig[-1] = 0.0
            kappa = np.inf
        A = np.asfortranarray((U * sig) @ V.T)
        xs = rng.standard_normal((n, nrhs))
        b = np.asfortranarray(A @ xs + 1e-10 * rng.standard_normal((m, nrhs)))
        probs.append((A, b, xs, kappa))
    return probs


def upload(L, probs):
    dA = [L.to_device_colmajor(A) for A, _, _, _ in probs]
    dB = [L.to_device_colmajor(b) for _, b, _, _ in probs]
    return dA, dB


def ls_bound(A, x, b, kappa, c=2000.0):
    """Forward-error scale of a backward-stable least-squares solve."""
    r = b - A @ x
    nA = np.linalg.norm(A, 2)
    return c * A.shape[1] * U53 * (kappa + kappa ** 2 * np.linalg.norm(r) / (nA * np.linalg.norm(x)))


def check_residual(A, b, x, xo):
    n = A.shape[1]
    for j in range(b.shape[1]):
        r = np.linalg.norm(b[:, j] - A @ x[:, j])
        ro = np.linalg.norm(b[:, j] - A @ xo[:, j])
        slack = 100 * n * U53 * np.linalg.norm(A, 2) * max(np.linalg.norm(x[:, j]), np.linalg.norm(xo[:, j]))
        assert r <= ro + slack + 1e-14 * np.linalg.norm(b[:, j]), (r, ro, slack)


def oracle_x(oracle_lib, A, b):
    m, n = A.shape
    Ao, bo = A.copy(order="F"), b.copy(order="F")
    T = np.asfortranarray(np.zeros((n, n)))
    oracle_lib.ls_solve(m, n, b.shape[1], Ao, m, T, n, bo, m, np.zeros(n * b.shape[1]))
    return bo[:n]


@pytest.mark.parametrize("variant,nmax,trial", [(0, 56, True), (1, 56, True), (0, 128, True), (1, 128, True),
                                               (0, 128, False)])
def test_mixed_variant_checked_solutions(gpu_lib, oracle_lib, variant, nmax, trial):
    import torch

    L = gpu_lib
    probs = make_batch(160, 11 + variant + nmax, mmax=900, nmax=nmax)
    dA, dB = upload(L, probs)
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    h = L.GelsMixed(ms, ns, 4, dA, ms, dB, ms)
    flags = L.GELS_NO_FALLBACK | (0 if trial else L.GELS_NO_TRIAL)
    fails, info, orth = h.run([variant] * len(probs), flags=flags)
    torch.cuda.synchronize()
    assert fails == sum(1 for v in info if v == 1)
    passed = 0
    for t, (A, b, xs, kappa) in enumerate(probs):
        m, n = A.shape
        if info[t] == 0:
            passed += 1
            assert 0.0 <= orth[t] <= 50 * n * U53, (t, orth[t])
            x = L.from_device(dB[t])[:n]
            xo = oracle_x(oracle_lib, A, b)
            if not np.isfinite(kappa):
                # exactly rank deficient: x is not unique, but a backward
                # stable solve leaves a residual within n u ||A|| ||x|| of the
                # least one
                check_residual(A, b, x, xo)
                continue
            err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
            assert err <= ls_bound(A, xo, b, kappa), (t, kappa, err)
        else:
            assert info[t] == 1
            # B is untouched when the check fails without fallback
            assert np.array_equal(L.from_device(dB[t]), b)
        # A is never written by the mixed variants
        assert np.array_equal(L.from_device(dA[t]), A)
        lim = 1e6 if variant == 0 else 1e12
        if kappa <= lim:
            assert info[t] == 0, (t, kappa, orth[t])
    assert passed >= len(probs) // 3
    h.close()


def test_routed_solve_with_fallback(gpu_lib, oracle_lib):
    import torch

    L = gpu_lib
    probs = make_batch(150, 21, mmax=900, nmax=128)
    dA, dB = upload(L, probs)
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    h = L.GelsMixed(ms, ns, 4, dA, ms, dB, ms)
    route = [t % 3 for t in range(len(probs))]
    fails, info, orth = h.run(route)
    torch.cuda.synchronize()
    for t, (A, b, xs, kappa) in enumerate(probs):
        m, n = A.shape
        x = L.from_device(dB[t])[:n]
        if not np.isfinite(kappa):
            assert info[t] in (0, 1) or info[t] < 0
            if info[t] >= 0:
                check_residual(A, b, x, oracle_x(oracle_lib, A, b))
            continue
        assert info[t] in (0, 1), (t, info[t])
        xo = oracle_x(oracle_lib, A, b)
        err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
        assert err <= ls_bound(A, xo, b, kappa), (t, route[t], kappa, err, info[t])
        if route[t] == 2:
            assert orth[t] == -2.0
        else:
            assert orth[t] != -2.0
    h.close()


def test_cholqr2_failures_retried_by_shifted_cholqr3(gpu_lib, oracle_lib):
    """Instances routed to Cholesky QR 2 whose check fails (kappa 1e9..1e11)
    are solved by shifted Cholesky QR 3 before any FP64 fallback: info 1, the
    orthogonality of the retry within 50 n 2^-53, A untouched (the FP64
    Householder solver would overwrite it)."""
    import torch

    L = gpu_lib
    rng = np.random.default_rng(77)
    probs = []
    for t in range(24):
        m, n = int(rng.integers(300, 900)), int(rng.integers(8, 100))
        kappa = 10 ** rng.uniform(9, 11)
        U, _ = np.linalg.qr(rng.standard_normal((m, n)))
        V, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = np.asfortranarray((U * kappa ** (-np.arange(n) / (n - 1))) @ V.T)
        xs = rng.standard_normal((n, 4))
        probs.append((A, np.asfortranarray(A @ xs + 1e-10 * rng.standard_normal((m, 4))), xs, kappa))
    dA, dB = upload(L, probs)
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    h = L.GelsMixed(ms, ns, 4, dA, ms, dB, ms)
    fails, info, orth = h.run([0] * len(probs), flags=L.GELS_NO_TRIAL)
    torch.cuda.synchronize()
    assert fails >= len(probs) // 2, fails
    assert sum(h.shifted()) == 0
    for t, (A, b, xs, kappa) in enumerate(probs):
        n = A.shape[1]
        assert np.array_equal(L.from_device(dA[t]), A), t
        if info[t] == 1:
            assert 0.0 <= orth[t] <= 50 * n * U53, (t, kappa, orth[t])
        x = L.from_device(dB[t])[:n]
        xo = oracle_x(oracle_lib, A, b)
        err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
        assert err <= ls_bound(A, xo, b, kappa), (t, kappa, err, info[t])
    h.close()


def test_trial_factor_chooses_the_shift(gpu_lib, oracle_lib):
    """Variant 0's trial Cholesky of the FP64-grade Gram: well-conditioned
    instances (kappa 1e2..1e4) keep Cholesky QR 2; most ill-conditioned ones
    (kappa 1e9..1e11, where Cholesky QR 2 fails its check) continue as
    shifted Cholesky QR 3, and those pass the check and solve to the
    backward-stable bound without any retry or fallback."""
    import torch

    L = gpu_lib
    rng = np.random.default_rng(78)
    probs = []
    for t in range(32):
        m, n = int(rng.integers(300, 900)), int(rng.integers(8, 128))
        lk = rng.uniform(2, 4) if t % 2 == 0 else rng.uniform(9, 11)
        kappa = 10 ** lk
        U, _ = np.linalg.qr(rng.standard_normal((m, n)))
        V, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = np.asfortranarray((U * kappa ** (-np.arange(n) / (n - 1))) @ V.T)
        xs = rng.standard_normal((n, 4))
        probs.append((A, np.asfortranarray(A @ xs + 1e-10 * rng.standard_normal((m, 4))), xs, kappa))
    dA, dB = upload(L, probs)
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    h = L.GelsMixed(ms, ns, 4, dA, ms, dB, ms)
    with pytest.raises(ValueError):
        h.set_trial_limit(0.0)
    fails, info, orth = h.run([0] * len(probs), flags=L.GELS_NO_FALLBACK)
    torch.cuda.synchronize()
    sh = h.shifted()
    assert sum(sh) == L.lib().lila_gels_mixed_shifted(h.h, None)
    high = [t for t in range(len(probs)) if probs[t][3] > 1e8]
    assert sum(sh[t] for t in high) >= 3 * len(high) // 4, [(probs[t][3], sh[t], info[t]) for t in high]
    for t, (A, b, xs, kappa) in enumerate(probs):
        n = A.shape[1]
        assert np.array_equal(L.from_device(dA[t]), A), t
        if kappa < 1e5:
            assert sh[t] == 0 and info[t] == 0, (t, kappa, sh[t], info[t])
        if info[t] == 0:
            assert 0.0 <= orth[t] <= 50 * n * U53, (t, kappa, orth[t])
            x = L.from_device(dB[t])[:n]
            xo = oracle_x(oracle_lib, A, b)
            err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
            assert err <= ls_bound(A, xo, b, kappa), (t, kappa, err)
        if sh[t]:
            assert info[t] == 0, (t, kappa, orth[t])
    h.close()


def test_edge_shapes_route_and_solve(gpu_lib, oracle_lib):
    """n = 1..3, m = n (square), m just below 2n, n = 128 with 8 right-hand
    sides: instances the mixed variants cannot take (m < 2n) are solved by
    variant 2 whatever their route, the others by their variant; every
    solution against the oracle's restatement of the reference driver."""
    import torch

    L = gpu_lib
    rng = np.random.default_rng(91)
    shapes = [(64, 1), (64, 2), (70, 3), (5, 5), (39, 20), (40, 20), (300, 128), (256, 128), (255, 128)]
    probs = []
    for m, n in shapes:
        A = np.asfortranarray(rng.standard_normal((m, n)))
        xs = rng.standard_normal((n, 8))
        probs.append((A, np.asfortranarray(A @ xs + 1e-10 * rng.standard_normal((m, 8))), xs, np.linalg.cond(A)))
    dA, dB = upload(L, probs)
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    h = L.GelsMixed(ms, ns, 8, dA, ms, dB, ms)
    F = torch.ones((len(probs), 5), dtype=torch.float32, device="cuda")
    assert h.features(F) == 0
    torch.cuda.synchronize()
    Fh = F.cpu().numpy()
    for variant in (0, 1):
        for t in range(len(probs)):
            dA[t].copy_(L.to_device_colmajor(probs[t][0]))
            dB[t].copy_(L.to_device_colmajor(probs[t][1]))
        fails, info, orth = h.run([variant] * len(probs))
        torch.cuda.synchronize()
        for t, (A, b, xs, kappa) in enumerate(probs):
            m, n = A.shape
            mixed_ok = m >= 2 * n
            assert (orth[t] == -2.0) == (not mixed_ok), (t, m, n, orth[t])
            if not mixed_ok:
                assert np.all(Fh[t] == 0.0), (t, Fh[t])
            x = L.from_device(dB[t])[:n]
            xo = oracle_x(oracle_lib, A, b)
            err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
            assert err <= ls_bound(A, xo, b, kappa), (variant, t, m, n, err)
    h.close()


def test_features_match_oracle(gpu_lib):
    import torch
    import selector as S

    L = gpu_lib
    probs = make_batch(60, 5, mmax=900, nmax=128, kmax=1e14)
    dA, dB = upload(L, probs)
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    h = L.GelsMixed(ms, ns, 4, dA, ms, dB, ms)
    F = torch.zeros((len(probs), 5), dtype=torch.float32, device="cuda")
    assert h.features(F) == 0
    torch.cuda.synchronize()
    Fg = F.cpu().numpy().astype(np.float64)
    for t, (A, b, xs, kappa) in enumerate(probs):
        fo = S.features(A)
        assert abs(Fg[t, 0] - fo[0]) < 1e-6 and abs(Fg[t, 1] - fo[1]) < 1e-6
        assert abs(Fg[t, 2] - fo[2]) < 1e-3, (t, Fg[t], fo)
        if np.isfinite(kappa) and kappa < 1e12:
            # FP64 sketch: the same condition estimate up to rounding
            assert abs(Fg[t, 3] - fo[3]) < 0.02, (t, kappa, Fg[t], fo)
            # and within a modest factor of the true 1-norm condition number
            R = np.linalg.qr(A, mode="r")
            k1 = np.abs(R).sum(0).max() * np.abs(np.linalg.inv(R)).sum(0).max()
            assert abs(Fg[t, 3] * 10 - np.log10(k1)) < 1.5, (t, kappa, Fg[t, 3], k1)
        else:
            assert Fg[t, 3] >= 1.2, (t, kappa, Fg[t])
        if kappa < 30 and fo[4] < 2.0:
            assert abs(Fg[t, 4] - fo[4]) < 0.02, (t, Fg[t], fo)
    h.close()


def test_trained_selector_gains_over_routing_without_it(gpu_lib):
    """What the trained network (lila_gb300/data/selector_params.f32) gains
    over the method without it, on instances drawn like its workload (kappa
    log-uniform to 1e15, 5 % rank deficient): its routes agree with the
    labels the method itself gives (cheapest variant whose check passes) on
    at least 90 % of the instances, and far fewer of its mixed attempts fail
    their check (each failure is a wasted mixed solve before the FP64
    solver) than when every instance starts with Cholesky QR 2, with or
    without the trial factor.  Its time cost, the FP64 sketch QR of its
    inputs, is measured by the bench."""
    import torch

    from lila_gb300 import selector_train as ST
    from lila_gb300 import workload as W

    L = gpu_lib
    params = ST.load_params()
    b = W.make_ls_batch(800, 777000, nhi=128, klo=1.0, khi=15.0, p_rankdef=0.05)
    _, y = ST.label_batch(L, b)
    h = L.GelsMixed(b.m, b.n, 4, b.A_ptr, b.lda, b.B_ptr, b.lda)
    fails_l, info_l, _, route = h.solve(params)
    torch.cuda.synchronize()
    b.restore()
    fails_t, _, _ = h.run([0] * b.count)
    torch.cuda.synchronize()
    b.restore()
    fails_0, _, _ = h.run([0] * b.count, flags=L.GELS_NO_TRIAL)
    torch.cuda.synchronize()
    b.restore()
    h.close()
    route = np.asarray(route)
    agree = float(np.mean(route == y))
    print("agreement %.3f, failed checks: learned %d, trial %d, Cholesky QR 2 first %d, labels %s" % (
        agree, fails_l, fails_t, fails_0, np.bincount(y, minlength=3).tolist()))
    assert agree >= 0.9, agree
    assert 4 * fails_l < fails_t, (fails_l, fails_t)
    assert 10 * fails_l < fails_0, (fails_l, fails_0)
    assert all(v in (0, 1) or v < 0 for v in info_l)
