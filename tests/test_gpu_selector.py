"""Learned variant selector kernels (lila_sel_*): inference, gradient and Adam
against the float64 CPU restatement in oracle/selector.py, and training on the
GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(x, dtype):
    import torch

    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def test_param_count(gpu_lib):
    import selector as S

    assert gpu_lib.sel_params() == S.NPAR == 8899


@pytest.mark.parametrize("count", [1, 64, 200])
def test_grad_matches_oracle(gpu_lib, count):
    import torch
    import selector as S

    L = gpu_lib
    rng = np.random.default_rng(count)
    p = torch.empty(S.NPAR, dtype=torch.float32, device="cuda")
    assert L.sel_init(p, 17) == 0
    X = rng.uniform(0, 2, size=(count, 5))
    y = rng.integers(0, 3, size=count)
    cw = np.array([1.0, 1.5, 3.0])
    dX, dy, dcw = _dev(X, torch.float32), _dev(y, torch.int32), _dev(cw, torch.float32)
    grad = torch.zeros(S.NPAR, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    lw = L.sel_grad_work(count)
    work = torch.empty(lw, dtype=torch.float32, device="cuda")
    assert L.sel_grad(count, p, dX, dy, None, dcw, grad, loss, work, lw) == 0
    torch.cuda.synchronize()
    p64 = p.cpu().numpy().astype(np.float64)
    X32 = X.astype(np.float32).astype(np.float64)
    lo, go = S.loss_and_grad(p64, X32, y, cw)
    g = grad.cpu().numpy().astype(np.float64)
    assert abs(float(loss.item()) - lo) <= 1e-5 * max(1.0, abs(lo))
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)
    # each parameter block separately (no block hidden by a larger one)
    o = 0
    for name, shp in S.SHAPES:
        k = int(np.prod(shp))
        gb, ob = g[o:o + k], go[o:o + k]
        assert np.linalg.norm(gb - ob) <= 1e-4 * np.linalg.norm(go) + 1e-4 * np.linalg.norm(ob), name
        o += k
    # inference logits and argmax
    logits = torch.zeros((count, 3), dtype=torch.float32, device="cuda")
    choice = torch.zeros(count, dtype=torch.int32, device="cuda")
    assert L.sel_infer(count, p, dX, logits, choice) == 0
    torch.cuda.synchronize()
    zo, _ = S.forward(p64, X32)
    assert np.abs(logits.cpu().numpy() - zo).max() <= 1e-4 * max(1.0, np.abs(zo).max())
    zg = logits.cpu().numpy()
    assert np.array_equal(choice.cpu().numpy(), zg.argmax(1))


def test_adam_matches_oracle(gpu_lib):
    import torch
    import selector as S

    L = gpu_lib
    rng = np.random.default_rng(9)
    p = rng.normal(0, 0.2, S.NPAR).astype(np.float32)
    m1 = rng.normal(0, 0.01, S.NPAR).astype(np.float32)
    m2 = rng.uniform(0, 0.01, S.NPAR).astype(np.float32)
    g = rng.normal(0, 0.1, S.NPAR).astype(np.float32)
    dp, dm1, dm2, dg = (_dev(v, torch.float32) for v in (p, m1, m2, g))
    assert L.sel_adam(dg, dp, dm1, dm2, 7, 1e-3) == 0
    torch.cuda.synchronize()
    po, m1o, m2o = S.adam_step(p.astype(np.float64), g.astype(np.float64), m1.astype(np.float64),
                              m2.astype(np.float64), 7, 1e-3)
    assert np.abs(dp.cpu().numpy() - po).max() <= 1e-6
    assert np.abs(dm1.cpu().numpy() - m1o).max() <= 1e-7
    assert np.abs(dm2.cpu().numpy() - m2o).max() <= 1e-7


def test_training_learns_a_rule(gpu_lib):
    """GPU training drives the loss down and fits a separable labelling."""
    import torch
    import selector as S

    L = gpu_lib
    rng = np.random.default_rng(1)
    n = 6000
    X = rng.uniform(0, 2, size=(n, 5)).astype(np.float32)
    y = np.where(X[:, 3] < 0.7, 0, np.where(X[:, 3] < 1.45, 1, 2)).astype(np.int32)
    dX, dy = _dev(X, torch.float32), _dev(y, torch.int32)
    cw = _dev(np.ones(3), torch.float32)
    p = torch.empty(S.NPAR, dtype=torch.float32, device="cuda")
    L.sel_init(p, 5)
    lw = L.sel_train_work(n, 256)
    work = torch.empty(lw, dtype=torch.float32, device="cuda")
    import ctypes

    losses = (ctypes.c_float * 40)()
    assert L.sel_train(n, dX, dy, cw, p, 40, 256, 3e-3, 1, work, lw, ctypes.addressof(losses)) == 0
    torch.cuda.synchronize()
    choice = torch.zeros(n, dtype=torch.int32, device="cuda")
    L.sel_infer(n, p, dX, None, choice)
    torch.cuda.synchronize()
    acc = float((choice.cpu().numpy() == y).mean())
    assert losses[-1] < 0.5 * losses[0]
    assert acc >= 0.97, acc
