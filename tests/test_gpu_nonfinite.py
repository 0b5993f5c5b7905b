"""Non-finite input on the recursive Householder driver and the batched
least-squares solver, injected on the host.  The call returns (no device
wait gives up, nothing traps); in split precision the FP64-grade tensor-core
products see the non-finite scale and report LILA_ST_NONFINITE; the FP64
path propagates the NaN into its outputs as the reference's FP64 code does;
the other instances of a batch are solved as usual, and the context stays
usable for the next call."""
import numpy as np
import pytest

import lila_cases as C
from test_gpu_bmixed import ls_bound, make_batch, oracle_x, upload

pytestmark = pytest.mark.gpu

ST_NONFINITE, ST_WAIT_TIMEOUT = 4, 16


def _recursive(L, A, m, n, mt, nx):
    import torch

    dA = L.to_device_colmajor(A)
    dT, dQ = L.colmajor(mt, n, fill=0.0), L.colmajor(m, n, fill=0.0)
    lp = [0, 1, 1, nx]
    lw = L.query_dgeqrf_w03_recursive(lp, m, n, 0, mt, None, m, None, mt, None, m, None, -1)
    W = torch.empty(lw, dtype=torch.float64, device="cuda")
    rc = L.dgeqrf_w03_recursive(lp, m, n, 0, mt, dA, m, dT, mt, dQ, m, W, lw)
    torch.cuda.synchronize()
    return rc, L.from_device(dA), L.from_device(dQ)


@pytest.mark.parametrize("bad", [np.nan, np.inf])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "split"])
def test_recursive_driver_nonfinite_input(gpu_lib, oracle_lib, bad, precision):
    L = gpu_lib
    m, n, mt, nx = 2048, 1024, 128, 128  # trailing updates large enough for the tensor-core products
    A, _, _ = C.inputs(m, n, 0, mt, seed=5)
    A = np.asfortranarray(A)
    A[700, 3] = bad
    L.gpu_clear_status()
    prev = L.gpu_set_precision(precision)
    try:
        rc, Af, Q = _recursive(L, A, m, n, mt, nx)
        st = L.gpu_status()
    finally:
        L.gpu_set_precision(prev)
    assert rc == 0
    assert not st & ST_WAIT_TIMEOUT, st
    assert not np.isfinite(Af).all() or not np.isfinite(Q).all()
    if precision == 1:
        assert st & ST_NONFINITE, st
    # the context is usable: a clean matrix gives the oracle's factors
    L.gpu_clear_status()
    out = C.run_gpu(L, "recursive", 300, 200, 0, 32, 1, 1, 64, seed=2)
    ref = C.run_cpu(oracle_lib, "recursive", 300, 200, 0, 32, 1, 1, 64, seed=2)
    err = C.compare_factor(out, ref, 300, 200, 0, 32)
    assert max(err.values()) < C.TOL, err
    assert L.gpu_status() == 0


@pytest.mark.parametrize("route", [0, 1, 2], ids=["cholqr2", "shifted_cholqr3", "fp64"])
def test_batched_solver_nonfinite_instances(gpu_lib, oracle_lib, route):
    import torch

    L = gpu_lib
    probs = make_batch(40, 31 + route, mmax=600, nmax=48, kmax=1e6, p_rankdef=0.0)
    bad = {5: np.nan, 17: np.inf}
    for t, v in bad.items():
        probs[t][0][3, 1] = v
    dA, dB = upload(L, probs)
    ms = [A.shape[0] for A, _, _, _ in probs]
    ns = [A.shape[1] for A, _, _, _ in probs]
    L.gpu_clear_status()
    h = L.GelsMixed(ms, ns, 4, dA, ms, dB, ms)
    fails, info, orth = h.run([route] * len(probs))
    torch.cuda.synchronize()
    st = L.gpu_status()
    h.close()
    assert not st & ST_WAIT_TIMEOUT, st
    if route < 2:
        assert st & ST_NONFINITE, st
    for t, (A, b, xs, kappa) in enumerate(probs):
        if t in bad:
            continue
        n = A.shape[1]
        assert info[t] in (0, 1), (t, info[t])
        x = L.from_device(dB[t])[:n]
        xo = oracle_x(oracle_lib, A, b)
        err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
        assert err <= ls_bound(A, xo, b, kappa), (t, kappa, err)
    L.gpu_clear_status()
