"""Failure path of a bounded device-side wait, run without faulting the GPU.

The cooperative Householder panel (dgeqr3's one-launch panel) synchronises
its CTAs through grid barriers whose waits give up after a caller-set number
of clock cycles (lila_gpu_set_wait_limit).  lila_prim_panel_phantom launches
the same kernel with every barrier waiting for one arrival that never comes
-- a flag nothing sets -- so each CTA's wait runs out, the kernel records
LILA_ST_WAIT_TIMEOUT and returns; the context stays usable and the next
panel computes the reference's reflectors again."""
import time

import numpy as np
import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu

ST_WAIT_TIMEOUT = 16


def test_panel_barrier_wait_runs_out_and_returns(gpu_lib, oracle_lib):
    import torch

    L = gpu_lib
    so = L.lib()
    m, nb = 4000, 32
    rng = np.random.default_rng(11)
    A = np.asfortranarray(rng.standard_normal((m, nb)))
    dA, dT = L.to_device_colmajor(A), L.colmajor(nb, nb, fill=0.0)
    dW = torch.empty(so.lila_prim_panel_work(nb), dtype=torch.float64, device="cuda")
    L.gpu_clear_status()
    prev = so.lila_gpu_set_wait_limit(2000000)  # about 1 ms at 2 GHz
    try:
        t0 = time.time()
        assert L.prim_panel_phantom(m, nb, dA, m, dT, nb, dW, 1) == 1
        torch.cuda.synchronize()
        elapsed = time.time() - t0
        st = L.gpu_status()
    finally:
        assert so.lila_gpu_set_wait_limit(prev) == 2000000
    assert st & ST_WAIT_TIMEOUT, st
    assert elapsed < 30.0, elapsed
    # the context is usable and the panel is right again with the default limit
    L.gpu_clear_status()
    assert L.gpu_status() == 0
    dA, dT = L.to_device_colmajor(A), L.colmajor(nb, nb, fill=0.0)
    Ao, To = A.copy(order="F"), np.asfortranarray(np.zeros((nb, nb)))
    oracle_lib.dgeqr3(m, nb, Ao, m, To, nb)
    L.trace(True)
    assert L.dgeqr3(m, nb, dA, m, dT, nb) == 0
    tr = L.trace_summary()
    L.trace(False)
    assert "panel_coop" in tr, tr
    assert C.max_rel(L.from_device(dA), Ao) < C.TOL
    assert L.gpu_status() == 0


def test_wait_limit_setting_keeps_positive_values(gpu_lib):
    so = gpu_lib.lib()
    prev = so.lila_gpu_set_wait_limit(0)  # <= 0 keeps the setting
    assert prev > 0
    assert so.lila_gpu_set_wait_limit(-5) == prev
    assert so.lila_gpu_set_wait_limit(prev) == prev
