"""The one-launch cooperative Householder panel behind dgeqr3 (n <= 64,
m >= 256) against the oracle's dgeqr3 restatement (lila-c/dgeqr3.c:3-114),
including ragged row blocks, zero columns (tau = 0) and the recursive
driver on the 4000 x 1000 shape."""
import numpy as np
import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n", [(256, 2), (300, 37), (3000, 64), (4001, 63), (16384, 64), (2431, 17)])
def test_dgeqr3_cooperative_panel(gpu_lib, oracle_lib, m, n):
    L = gpu_lib
    rng = np.random.default_rng(m + n)
    A = np.asfortranarray(rng.standard_normal((m, n)))
    if n > 5:
        A[:, 3] = 0.0  # a zero column below the pivot as well: tau = 0 there
    T = np.asfortranarray(np.zeros((n, n)))
    Ao, To = A.copy(order="F"), T.copy(order="F")
    oracle_lib.dgeqr3(m, n, Ao, m, To, n)
    dA, dT = L.to_device_colmajor(A), L.to_device_colmajor(T)
    L.trace(True)
    assert L.dgeqr3(m, n, dA, m, dT, n) == 0
    tr = L.trace_summary()
    L.trace(False)
    assert "panel_coop" in tr, tr
    assert C.max_rel(L.from_device(dA), Ao) < C.TOL
    assert C.max_rel(np.triu(L.from_device(dT)), np.triu(To)) < C.TOL
    assert L.gpu_status() == 0


def test_panel_falls_back_below_threshold(gpu_lib, oracle_lib):
    """Panels under 256 rows keep the recursive dgeqr3 kernels."""
    L = gpu_lib
    m, n = 200, 37
    A = np.asfortranarray(np.random.default_rng(2).standard_normal((m, n)))
    Ao, To = A.copy(order="F"), np.asfortranarray(np.zeros((n, n)))
    oracle_lib.dgeqr3(m, n, Ao, m, To, n)
    dA, dT = L.to_device_colmajor(A), L.colmajor(n, n, fill=0.0)
    L.trace(True)
    assert L.dgeqr3(m, n, dA, m, dT, n) == 0
    tr = L.trace_summary()
    L.trace(False)
    assert "panel_coop" not in tr
    assert C.max_rel(L.from_device(dA), Ao) < C.TOL
