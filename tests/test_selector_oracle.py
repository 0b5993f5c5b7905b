"""CPU checks of the selector oracle (oracle/selector.py): its gradient is the
derivative of its loss, and its features behave as documented."""
import numpy as np

def test_gradient_is_the_loss_derivative():
    """The oracle's gradient against central differences of its loss."""
    import selector as S

    rng = np.random.default_rng(3)
    p = rng.normal(0, 0.3, S.NPAR)
    X = rng.uniform(0, 2, size=(40, 5))
    y = rng.integers(0, 3, size=40)
    cw = np.array([1.0, 2.0, 0.5])
    _, g = S.loss_and_grad(p, X, y, cw)
    for k in rng.choice(S.NPAR, 40, replace=False):
        e = np.zeros(S.NPAR)
        e[k] = 1e-6
        fd = (S.loss_and_grad(p + e, X, y, cw)[0] - S.loss_and_grad(p - e, X, y, cw)[0]) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), k



def test_feature_condition_estimate_tracks_kappa():
    import selector as S

    rng = np.random.default_rng(4)
    m, n = 400, 24
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    prev = -1.0
    for kappa in (1e2, 1e5, 1e8, 1e11, 1e14):
        A = (U * kappa ** (-np.arange(n) / (n - 1))) @ V.T
        f = S.features(A)
        assert abs(f[0] - np.log2(m) / 12) < 1e-12 and abs(f[1] - np.log2(n) / 7) < 1e-12
        assert abs(10 * f[3] - np.log10(kappa)) < 1.5, (kappa, f)
        assert f[3] > prev
        prev = f[3]
    A[:, -1] = A[:, 0]  # exactly rank deficient
    assert S.features(A)[3] >= 1.4
