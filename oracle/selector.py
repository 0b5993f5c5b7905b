"""CPU oracle (test infrastructure only) for the learned variant selector and
its input features.  Nothing in the product imports this module; tests use it
to check the GPU kernels of lila_gb300/csrc/lg_select.cu and lg_bmixed.cu.

The selector has no counterpart in the reference: the reference's routines
(lila-c/lila_dgeqrf_w03_mt_hr.c, least-squares/main_ls_qr3.c) run one fixed
method per call.  This module restates, in float64 numpy:

* the 5 -> 64 -> 64 -> 64 -> 3 perceptron (ReLU hidden layers, softmax
  output) with the flat parameter layout W1 | b1 | W2 | b2 | W3 | b3 | W4 | b4
  (W row-major, W[j, i] maps input i to output j), its class-weighted mean
  cross-entropy loss and the loss's gradient;
* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected);
* the five instance features (m, n, column-norm spread, condition estimate
  from a min(2n, 176) x n sparse-sign sketch, FP32 Cholesky pivot ratio) with
  the same hashed sketch.
"""
import numpy as np

NIN, H, NOUT = 5, 64, 3
SHAPES = [("W1", (H, NIN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
          ("W4", (NOUT, H)), ("b4", (NOUT,))]
NPAR = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, o = {}, 0
    for name, shp in SHAPES:
        k = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + k], dtype=np.float64).reshape(shp)
        o += k
    return out


def pack(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SHAPES])


def forward(p, X):
    w = unpack(p)
    h1 = np.maximum(X @ w["W1"].T + w["b1"], 0.0)
    h2 = np.maximum(h1 @ w["W2"].T + w["b2"], 0.0)
    h3 = np.maximum(h2 @ w["W3"].T + w["b3"], 0.0)
    z = h3 @ w["W4"].T + w["b4"]
    return z, (X, h1, h2, h3)


def loss_and_grad(p, X, y, cw):
    """Class-weighted mean cross entropy and its gradient (flat, float64)."""
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.int64)
    cw = np.asarray(cw, dtype=np.float64)
    N = X.shape[0]
    w = unpack(p)
    z, (x0, h1, h2, h3) = forward(p, X)
    zm = z - z.max(axis=1, keepdims=True)
    e = np.exp(zm)
    sm = e / e.sum(axis=1, keepdims=True)
    wy = cw[y]
    loss = float(np.sum(wy * (np.log(e.sum(axis=1)) - zm[np.arange(N), y])) / N)
    dz = sm.copy()
    dz[np.arange(N), y] -= 1.0
    dz *= (wy / N)[:, None]
    g = {"W4": dz.T @ h3, "b4": dz.sum(0)}
    d3 = (dz @ w["W4"]) * (h3 > 0)
    g["W3"], g["b3"] = d3.T @ h2, d3.sum(0)
    d2 = (d3 @ w["W3"]) * (h2 > 0)
    g["W2"], g["b2"] = d2.T @ h1, d2.sum(0)
    d1 = (d2 @ w["W2"]) * (h1 > 0)
    g["W1"], g["b1"] = d1.T @ x0, d1.sum(0)
    return loss, pack(g)


def adam_step(p, g, m1, m2, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m1 = b1 * m1 + (1 - b1) * g
    m2 = b2 * m2 + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return p - lr * (m1 / c1) / (np.sqrt(m2 / c2) + eps), m1, m2


def _mix32(x):
    x = np.asarray(x, dtype=np.uint64) & 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def sketch_rows(m, n):
    """Bucket (in [0, min(2n, 176))) and sign (+1/-1) of each row of the
    sparse sketch."""
    r = np.arange(m, dtype=np.uint64)
    h = _mix32((r * 0x9E3779B9 + 0x3C6EF372) & 0xFFFFFFFF)
    return ((h >> 1) % min(2 * n, 176)).astype(np.int64), np.where(h & 1, 1.0, -1.0)


def features(A):
    """The five selector inputs of one instance (float64; the GPU computes
    f2 and f4 in FP32 and f3 in FP64 with another summation order)."""
    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    A32 = A.astype(np.float32)
    G = (A32.T.astype(np.float64) @ A32.astype(np.float64))
    norms = np.sqrt(np.maximum(np.diag(G), 0))
    f2 = min(np.log10(norms.max() / norms.min()) / 4.0, 4.0) if norms.min() > 0 else 4.0
    try:
        R32 = np.linalg.cholesky(G.astype(np.float32)).T
        d = np.abs(np.diag(R32)).astype(np.float64)
        f4 = min(np.log10(d.max() / d.min()) / 3.0, 2.0) if np.all(np.isfinite(d)) and d.min() > 0 else 2.0
    except np.linalg.LinAlgError:
        f4 = 2.0
    if True:
        b, s = sketch_rows(m, n)
        SA = np.zeros((min(2 * n, 176), n))
        np.add.at(SA, b, s[:, None] * A)
        R = np.linalg.qr(SA, mode="r")
        with np.errstate(divide="ignore", invalid="ignore"):
            try:
                Ri = np.linalg.inv(np.triu(R))
                k1 = np.abs(R).sum(0).max() * np.abs(Ri).sum(0).max()
            except np.linalg.LinAlgError:
                k1 = np.inf
        f3 = (min(np.log10(max(k1, 1.0)), 20.0) if np.isfinite(k1) else 20.0) / 10.0
    return np.array([np.log2(m) / 12.0, np.log2(n) / 7.0, f2, f3, f4])
