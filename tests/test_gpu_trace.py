"""Per-launch event trace: counts, and traced durations that add up to no
more than the elapsed time of the traced work (the end event of one launch
starts the next one while the device is still behind)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trace_counts_and_bounds(gpu_lib):
    import torch

    L = gpu_lib
    m, n = 400000, 64
    rng = np.random.default_rng(3)
    dA = L.to_device_colmajor(rng.standard_normal((m, n)))
    dX = L.to_device_colmajor(np.triu(rng.standard_normal((n, n))))
    dO = L.colmajor(m, n, fill=0.0)
    lw = L.lib().lila_prim_ozaki_gram_work()
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    dG = L.colmajor(n, n, fill=0.0)
    assert L.prim_ozaki_map(m, n, dA, m, dX, n, n, dO, m) == 0
    torch.cuda.synchronize()
    L.trace(True)
    t0 = time.perf_counter()
    for _ in range(6):
        assert L.prim_ozaki_map(m, n, dA, m, dX, n, n, dO, m) == 0
        assert L.prim_ozaki_gram(m, n, dO, m, dG, n, dW, lw) == 0
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t0) * 1e3
    tr = L.trace_summary()
    L.trace(False)
    assert tr["ozaki_map"][0] == 6 and tr["ozaki_gram"][0] == 6, tr
    total = sum(ms for _, ms in tr.values())
    assert all(ms > 0.0 for _, ms in tr.values()), tr
    assert total <= wall_ms, (total, wall_ms)
    # an idle host gap between calls is not counted in the next launch
    L.trace(True)
    assert L.prim_ozaki_map(m, n, dA, m, dX, n, n, dO, m) == 0
    torch.cuda.synchronize()
    time.sleep(0.2)
    assert L.prim_ozaki_map(m, n, dA, m, dX, n, n, dO, m) == 0
    torch.cuda.synchronize()
    tr2 = L.trace_summary()
    L.trace(False)
    per_map = tr["ozaki_map"][1] / 6
    assert tr2["ozaki_map"][0] == 2
    assert tr2["ozaki_map"][1] < 4 * per_map + 1.0, (tr2, per_map)
    assert L.gpu_status() == 0
