"""The split leaf's per-pass FP64 factor (one CTA): the pivot step's
reciprocal square root against long-double references, and the trial /
shifted Cholesky factor, its inverse and the shift decision against LAPACK
(numpy / scipy) on the same Gram."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_rsqrt_within_two_ulp(gpu_lib):
    import torch

    L = gpu_lib
    rng = np.random.default_rng(7)
    d = np.concatenate([10.0 ** rng.uniform(-307, 308, 200000),
                        rng.uniform(1.0, 4.0, 20000),
                        np.array([5e-324, 1e-320, 2.2250738585072009e-308, 2.2250738585072014e-308,
                                  1.0, 2.0, 4.0, np.nextafter(4.0, 0.0), np.nextafter(1.0, 2.0),
                                  1.7976931348623157e308])])
    dd = torch.from_numpy(d).cuda()
    out = torch.empty_like(dd)
    assert L.prim_rsqrt(d.size, dd, out) == 0
    y = out.cpu().numpy()
    ref = 1.0 / np.sqrt(d.astype(np.longdouble))
    ulp = np.spacing(ref.astype(np.float64)).astype(np.longdouble)
    err = np.abs(y.astype(np.longdouble) - ref) / ulp
    assert float(err.max()) <= 2.0, float(err.max())
    bad = torch.tensor([0.0, -1.0, float("inf"), float("nan")], dtype=torch.float64, device="cuda")
    ob = torch.full_like(bad, 7.0)
    assert L.prim_rsqrt(4, bad, ob) == 0
    assert np.array_equal(ob.cpu().numpy(), np.zeros(4))


def _norm1_upper(B):
    return np.abs(np.triu(B)).sum(axis=0).max()


def _run(L, G, variant, shift_factor=1e-10, cond_limit=1e7):
    import torch

    n = G.shape[0]
    dG = L.to_device_colmajor(np.asfortranarray(G))
    dR = L.colmajor(n, n, fill=np.nan)
    dX = L.colmajor(n, n, fill=np.nan)
    rc = L.prim_factor_pass(n, dG, n, dR, n, dX, n, variant, shift_factor, cond_limit)
    torch.cuda.synchronize()
    return rc, L.from_device(dR), L.from_device(dX)


def _check_factor(G, R, X, sigma=0.0):
    """Backward error of R (|R^T R - G - sigma I| <= (n + 1) u |R|^T |R|
    elementwise, Cholesky's bound) and X against LAPACK's inverse of the
    same R (|X R - I| within 64 kappa_1(R) u)."""
    import scipy.linalg as sl

    n = G.shape[0]
    u = 2.0 ** -53
    assert np.array_equal(np.tril(R, -1), np.zeros((n, n)))
    assert np.array_equal(np.tril(X, -1), np.zeros((n, n)))
    Gs = G + sigma * np.eye(n)
    assert np.all(np.abs(R.T @ R - Gs) <= 2 * (n + 1) * u * (np.abs(R).T @ np.abs(R)) + 1e-300)
    Xref = sl.solve_triangular(R, np.eye(n))
    kap = _norm1_upper(R) * _norm1_upper(Xref)
    assert np.abs(X @ R - np.eye(n)).max() <= 64 * kap * u
    assert np.abs(X - Xref).max() <= 64 * kap * u * np.abs(Xref).max()


@pytest.mark.parametrize("n", [64, 63, 37, 8, 5, 1])
def test_trial_factor_accepted(gpu_lib, n):
    L = gpu_lib
    rng = np.random.default_rng(100 + n)
    A = rng.standard_normal((4 * n + 8, n)) * 10.0 ** rng.uniform(-1, 1, n)
    G = A.T @ A
    Rref = np.linalg.cholesky(G).T
    for variant in (0, 1):
        rc, R, X = _run(L, G, variant)
        assert rc == 0
        _check_factor(G, R, X)
        assert np.abs(R - Rref).max() <= 1e-11 * np.abs(Rref).max()
    assert L.gpu_status() == 0


def test_ill_conditioned_gram_selects_the_shift(gpu_lib):
    L = gpu_lib
    rng = np.random.default_rng(5)
    n = 64
    Q, _ = np.linalg.qr(rng.standard_normal((200, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (Q * 10.0 ** -np.linspace(0, 10, n)) @ V.T
    G = A.T @ A
    sf = 1e-10
    rc, R, X = _run(L, G, 0, sf)
    assert rc == 1
    _check_factor(G, R, X, sf * np.trace(G))
    # variant 2 takes the shift on its first pass whatever the Gram
    rng2 = np.random.default_rng(6)
    B = rng2.standard_normal((300, 40))
    G2 = B.T @ B
    rc, R, X = _run(L, G2, 2, sf)
    assert rc == 1
    _check_factor(G2, R, X, sf * np.trace(G2))
    assert L.gpu_status() == 0


def test_condition_estimate_selects_the_shift(gpu_lib):
    """Unit diagonal (ratio 1) but ||R^-1||_1 growing as 1.5^(n-1): only
    the 1-norm estimate sees it.  Below the limit (n = 8) and above it
    (n = 20) the decision follows ||R||_1 ||R^-1||_1 from LAPACK."""
    import scipy.linalg as sl

    L = gpu_lib
    for n, expect in ((20, 1), (8, 0)):
        Rt = np.eye(n) - np.triu(np.ones((n, n)), 1) * 0.5
        G = Rt.T @ Rt
        Rr = np.linalg.cholesky(G).T
        kap = _norm1_upper(Rr) * _norm1_upper(sl.solve_triangular(Rr, np.eye(n)))
        assert (kap > 1e3) == bool(expect)
        rc, R, X = _run(L, G, 0, 1e-12, 1e3)
        assert rc == expect, (n, kap)
        _check_factor(G, R, X, 1e-12 * np.trace(G) if expect else 0.0)
    assert L.gpu_status() == 0


def test_breakdown_reported_only_for_the_kept_factor(gpu_lib):
    L = gpu_lib
    rng = np.random.default_rng(9)
    n = 30
    A = rng.standard_normal((100, n))
    G = A.T @ A
    Gi = G.copy()
    Gi[11, 11] = -1.0  # indefinite: the trial and the shifted factor break down
    L.gpu_clear_status()
    rc, R, X = _run(L, Gi, 0, 1e-10)
    assert rc == 1
    assert L.gpu_status() & 1
    L.gpu_clear_status()
    # rank deficient (a repeated column): the trial fails, the shifted factor exists
    A2 = A.copy()
    A2[:, 7] = A2[:, 3]
    G2 = A2.T @ A2
    rc, R, X = _run(L, G2, 0, 1e-8)
    assert rc == 1
    assert L.gpu_status() == 0
    _check_factor(G2, R, X, 1e-8 * np.trace(G2))
    # variant 1 keeps its (broken-down) factor and reports it
    rc, R, X = _run(L, Gi, 1)
    assert rc == 0
    assert L.gpu_status() & 1
    L.gpu_clear_status()
    assert L.prim_factor_pass(65, None, 65, None, 65, None, 65, 0, 0.0, 1e7) == -1
