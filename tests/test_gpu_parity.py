"""GPU parity: the sm_103a library against the CPU oracle and the golden fixtures.

Every call goes through the C ABI (include/lila.h) with device buffers.  The
bar is elementwise agreement to 1e-12 relative (lila_cases.TOL) over the
defined outputs (A's V and R, the upper triangles of the T tiles, Q).
"""
import glob
import os

import numpy as np
import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("case", C.UGLY, ids=lambda c: "x".join(map(str, c)))
def test_recursive_vs_oracle(gpu_lib, oracle_lib, torch_cuda, case):
    m, n, ii, mt, lda, ldq, leaf, panel, nx = case
    out = C.run_gpu(gpu_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=1)
    ref = C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=1)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err
    # padding rows of A beyond m and columns before ii stay untouched
    A0, _, _ = C.inputs(m, n, ii, mt, lda, ldq, seed=1)
    assert np.array_equal(out[0][m:], A0[m:])
    assert np.array_equal(out[0][:, :ii], A0[:, :ii])


@pytest.mark.parametrize("leaf,panel", [(1, 1), (1, 0), (0, 0), (1, 2), (2, 0)])
@pytest.mark.parametrize("nb", [[10], [20, 5], [16, 8, 4]])
def test_levelx_vs_oracle(gpu_lib, oracle_lib, torch_cuda, nb, leaf, panel):
    m, n, ii, mt = 87, 53, 6, 4
    if leaf == 2:
        mt = 16  # CholQR leaves need tiles wider than the smallest levelx block
    out = C.run_gpu(gpu_lib, "levelx", m, n, ii, mt, leaf, panel, None, seed=2, nb=nb)
    ref = C.run_cpu(oracle_lib, "levelx", m, n, ii, mt, leaf, panel, None, seed=2, nb=nb)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


def _golden_driver_files():
    return sorted(f for f in glob.glob(os.path.join(GOLD, "*.npz"))
                  if os.path.basename(f).startswith(("rec_", "lvx_")))


@pytest.mark.parametrize("path", _golden_driver_files(), ids=os.path.basename)
def test_gpu_matches_golden(gpu_lib, torch_cuda, path):
    g = np.load(path)
    m, n, ii, mt, lda, ldq, leaf, panel = [int(v) for v in g["shape"]]
    nb = [int(v) for v in g["nb"]]
    mode = "levelx" if os.path.basename(path).startswith("lvx_") else "recursive"
    out = C.run_gpu(gpu_lib, mode, m, n, ii, mt, leaf, panel, nb[0] if mode == "recursive" else None,
                    lda, ldq, seed=0, nb=nb if mode == "levelx" else None)
    err = C.compare_factor(out, (g["A"], g["T"], g["Q"]), m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


def _factored(oracle_lib, m, n, ii, mt, seed=5):
    return C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, 1, 1, 7, seed=seed)


def test_dormqrf_z03_and_w03(gpu_lib, oracle_lib, torch_cuda):
    L, torch = gpu_lib, torch_cuda
    m, n, ii, mt, nrhs = 150, 61, 7, 6, 9
    A, T, Q = _factored(oracle_lib, m, n, ii, mt)
    rng = np.random.default_rng(11)
    B = np.asfortranarray(rng.standard_normal((m, nrhs + 3)))
    # separate block, columns 3..3+nrhs
    Bo = B.copy(order="F")
    work = np.zeros(8 * m * (nrhs + mt))
    oracle_lib.dormqrf_z03(m, nrhs, n, ii, 3, mt, A, m, T, mt, Bo, m, work, work.size)
    dA, dT, dB = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(B)
    lw = L.query_dormqrf_w03(m, nrhs, n, ii, 3, mt, None, m, None, mt, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dormqrf_z03(m, nrhs, n, ii, 3, mt, dA, m, dT, mt, dB, m, dW, lw) == 0
    assert C.max_rel(L.from_device(dB), Bo) < C.TOL
    # in place on trailing columns of A: A' = [A | B]
    Aw = np.asfortranarray(np.hstack([A, B]))
    Awo = Aw.copy(order="F")
    oracle_lib.dormqrf_w03(m, nrhs, n, ii, n + ii + 3, mt, Awo, m, T, mt, work, work.size)
    dAw = L.to_device_colmajor(Aw)
    assert L.dormqrf_w03(m, nrhs, n, ii, n + ii + 3, mt, dAw, m, dT, mt, dW, lw) == 0
    assert C.max_rel(L.from_device(dAw), Awo) < C.TOL


def test_dormqrbz_connect_dlarft(gpu_lib, oracle_lib, torch_cuda):
    L, torch = gpu_lib, torch_cuda
    m, n, ii, mt = 120, 50, 5, 8
    A, T, Q = _factored(oracle_lib, m, n, ii, mt)
    rng = np.random.default_rng(12)
    # dormqrbz: Q(i:m, j:j+nc) = H [0; X]
    k, i, nc = 30, ii, 7
    j = i + k
    Qx = np.asfortranarray(np.hstack([Q, rng.standard_normal((m, nc + j))]))
    Qo = Qx.copy(order="F")
    work = np.zeros(8 * m * (n + mt + nc))
    oracle_lib.dormqrbz_w03(m, nc, k, i, j, mt, A, m, Qo, m, T, mt, work, work.size)
    dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Qx)
    lw = L.query_dormqrbz_w03(m, nc, k, i, j, mt, None, m, None, m, None, mt, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dormqrbz_w03(m, nc, k, i, j, mt, dA, m, dQ, m, dT, mt, dW, lw) == 0
    got = L.from_device(dQ)
    assert C.max_rel(got[i:, j:j + nc], Qo[i:, j:j + nc]) < C.TOL
    # dlarft_connect on a T whose connection block was zeroed
    for (ci, cj) in [(ii + 13, ii), (ii + 16, ii + 3), (ii + 27, ii + 21)]:
        Tz = T.copy(order="F")
        vb = min(mt - ci % mt, 9)
        wb = ci - cj if cj // mt == ci // mt else ci % mt
        Tz[ci % mt - wb:ci % mt, ci:ci + vb] = 0.0
        To = Tz.copy(order="F")
        oracle_lib.dlarft_connect_w03(m, 9, ci, cj, mt, A, m, To, mt)
        dTz = L.to_device_colmajor(Tz)
        assert L.dlarft_connect_w03(m, 9, ci, cj, mt, dA, m, dTz, mt) == 0
        assert C.max_rel(L.from_device(dTz), To) < C.TOL
    # dlarft_w03 from V and tau; dT2tau / dV2tau
    tau = np.zeros(n)
    oracle_lib.dT2tau_w03(m, n, ii, mt, T, mt, tau)
    dtau = torch.empty(n, dtype=torch.float64, device="cuda")
    assert L.dT2tau_w03(m, n, ii, mt, dT, mt, dtau) == 0
    assert np.max(np.abs(dtau.cpu().numpy() - tau)) < 1e-15
    tau2 = np.zeros(n)
    oracle_lib.dV2tau_w03(m, n, ii, mt, A, m, tau2)
    assert L.dV2tau_w03(m, n, ii, mt, dA, m, dtau) == 0
    assert np.max(np.abs(dtau.cpu().numpy() - tau2)) < 1e-13
    Tn = np.asfortranarray(np.zeros_like(T))
    oracle_lib.dlarft_w03(m, n, ii, mt, A, m, Tn, mt, tau)
    dTn = L.to_device_colmajor(np.zeros_like(T))
    dtau = torch.from_numpy(tau).cuda()
    assert L.dlarft_w03(m, n, ii, mt, dA, m, dTn, mt, dtau) == 0
    M = C.tile_mask(n, ii, mt)
    assert C.max_rel(L.from_device(dTn)[M], Tn[M]) < C.TOL


def test_dgeqr3_and_panels(gpu_lib, oracle_lib, torch_cuda):
    L, torch = gpu_lib, torch_cuda
    rng = np.random.default_rng(13)
    m, n = 200, 37
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, n)))
    T = np.asfortranarray(np.zeros((n, n)))
    Ao, To = A.copy(order="F"), T.copy(order="F")
    oracle_lib.dgeqr3(m, n, Ao, m, To, n)
    dA, dT = L.to_device_colmajor(A), L.to_device_colmajor(T)
    assert L.dgeqr3(m, n, dA, m, dT, n) == 0
    assert C.max_rel(L.from_device(dA), Ao) < C.TOL
    assert C.max_rel(np.triu(L.from_device(dT)), np.triu(To)) < C.TOL
    # the three panels inside one tile
    m, n, i, mt = 90, 12, 20, 16
    for name in ("dgeqr2_w03_l", "dgeqr2_w03_3", "dgeqr2_w03_hr"):
        A = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, i + n)))
        Q = np.asfortranarray(np.zeros((m, i + n)))
        T = np.asfortranarray(np.zeros((mt, i + n)))
        Ao, To, Qo = A.copy(order="F"), T.copy(order="F"), Q.copy(order="F")
        work = np.zeros(4 * m * mt + 4 * n * n)
        getattr(oracle_lib, name)(m, n, i, mt, Ao, m, To, mt, Qo, m, work, work.size)
        dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
        lw = getattr(L, "query_" + name)(m, n, i, mt, None, m, None, mt, None, m, None, -1)
        dW = torch.empty(lw, dtype=torch.float64, device="cuda")
        assert getattr(L, name)(m, n, i, mt, dA, m, dT, mt, dQ, m, dW, lw) == 0
        Mk = C.tile_mask(n, i, mt)
        assert C.max_rel(L.from_device(dA), Ao) < C.TOL, name
        assert C.max_rel(L.from_device(dT)[Mk], To[Mk]) < C.TOL, name
        assert C.max_rel(L.from_device(dQ)[i:, i:], Qo[i:, i:]) < C.TOL, name


def test_mt_hr_many_tiles_and_dorgh2(gpu_lib, oracle_lib, torch_cuda):
    """CholQR leaf spanning 4 tiles (where the reference's S alias breaks) and lila_dorgh2."""
    L, torch = gpu_lib, torch_cuda
    m, n, ii, mt = 300, 53, 6, 16
    A, T, Q = C.inputs(m, n, ii, mt, seed=4)
    Ao, To, Qo = A.copy(order="F"), T.copy(order="F"), Q.copy(order="F")
    work = np.zeros(oracle_lib.query_dgeqrf_w03_mt_hr(m, n, ii, mt) + 10)
    oracle_lib.dgeqrf_w03_mt_hr(m, n, ii, mt, Ao, m, To, mt, Qo, m, work, work.size)
    dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
    lw = L.query_dgeqrf_w03_mt_hr(m, n, ii, mt, None, m, None, mt, None, m, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dgeqrf_w03_mt_hr(m, n, ii, mt, dA, m, dT, mt, dQ, m, dW, lw) == 0
    err = C.compare_factor((L.from_device(dA), L.from_device(dT), L.from_device(dQ)), (Ao, To, Qo), m, n, ii, mt)
    assert max(err.values()) < C.TOL, err
    res, orth = C.residuals(A, (L.from_device(dA), None, L.from_device(dQ)), m, n, ii)
    assert res < 1e-14 and orth < 1e-13


def test_appendcols(gpu_lib, oracle_lib, torch_cuda):
    L, torch = gpu_lib, torch_cuda
    m, k, n, mt = 130, 40, 30, 8
    lp = C.lparam(1, 1, 9)
    A, T, Q = C.inputs(m, k + n, 0, mt, seed=6)
    Ao, To, Qo = A.copy(order="F"), T.copy(order="F"), Q.copy(order="F")
    work = np.zeros(8 * m * (k + n + mt))
    oracle_lib.dgeqrf_w03_recursive(lp, m, k, 0, mt, Ao, m, To, mt, Qo, m, work, work.size)
    A1, T1, Q1 = Ao.copy(order="F"), To.copy(order="F"), Qo.copy(order="F")
    oracle_lib.dgeqrf_w03_appendcols(lp, m, k, n, mt, Ao, m, Qo, m, To, mt, work, work.size)
    dA, dT, dQ = L.to_device_colmajor(A1), L.to_device_colmajor(T1), L.to_device_colmajor(Q1)
    lw = L.query_dgeqrf_w03_recursive(list(lp), m, k + n, 0, mt, None, m, None, mt, None, m, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dgeqrf_w03_appendcols(list(lp), m, k, n, mt, dA, m, dQ, m, dT, mt, dW, lw) == 0
    err = C.compare_factor((L.from_device(dA), L.from_device(dT), L.from_device(dQ)), (Ao, To, Qo), m, k + n, 0, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("case", C.VQ_CASES, ids=lambda c: "x".join(map(str, c)))
def test_v03_q03_vs_oracle(gpu_lib, oracle_lib, torch_cuda, case):
    """V, R, T by lila_dgeqrf_v03_recursive, then Q by lila_dgeqrf_q03_recursive."""
    m, n, ii, mt, lda, ldq, leaf, panel, nx = case
    out = C.run_gpu_vq(gpu_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=3)
    ref = C.run_cpu_vq(oracle_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=3)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err
    A0, _, Q0 = C.inputs(m, n, ii, mt, lda, ldq, seed=3)
    assert np.array_equal(out[0][:, :ii], A0[:, :ii])
    assert np.array_equal(out[2][:, :ii], Q0[:, :ii])


@pytest.mark.parametrize("nb", [[10], [20, 5], [16, 8, 4]])
def test_v03_q03_levelx_vs_oracle(gpu_lib, oracle_lib, torch_cuda, nb):
    m, n, ii, mt = 87, 53, 6, 4
    out = C.run_gpu_vq(gpu_lib, "levelx", m, n, ii, mt, 1, 1, None, seed=4, nb=nb)
    ref = C.run_cpu_vq(oracle_lib, "levelx", m, n, ii, mt, 1, 1, None, seed=4, nb=nb)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "vq_*.npz"))), ids=os.path.basename)
def test_v03_q03_match_golden(gpu_lib, torch_cuda, path):
    """Against the reference's own v03 / q03 outputs (tests/golden/make_golden.py)."""
    g = np.load(path)
    m, n, ii, mt, lda, ldq, leaf, panel = [int(v) for v in g["shape"]]
    nb = [int(v) for v in g["nb"]]
    mode = "levelx" if "_lvx_" in os.path.basename(path) else "recursive"
    out = C.run_gpu_vq(gpu_lib, mode, m, n, ii, mt, leaf, panel, nb[0] if mode == "recursive" else None,
                       lda, ldq, seed=0, nb=nb if mode == "levelx" else None)
    err = C.compare_factor(out, (g["A"], g["T"], g["Q"]), m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


def test_v03_q03_leaves_panels_and_errors(gpu_lib, oracle_lib, torch_cuda):
    """The leaf, panel and dispatcher entry points of v03 / q03 one by one,
    leaf 2 / panel 2 as no-ops (as in the reference) and argument checks."""
    L, torch = gpu_lib, torch_cuda
    m, n, ii, mt = 120, 24, 8, 8
    lw = 8 * (m + n + ii) * (n + ii + mt) + 4096
    for leaf, panel in ((0, 0), (1, 0), (1, 1)):
        lp = np.array([0, leaf, panel, 64], dtype=np.int32)
        A, T, Q = C.inputs(m, n, ii, mt, seed=6)
        dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
        dW = torch.empty(lw, dtype=torch.float64, device="cuda")
        w = np.zeros(lw)
        assert L.dgeqrf_v03_mt(list(lp), m, n, ii, mt, dA, m, dT, mt, dW, lw) == 0
        oracle_lib.dgeqrf_v03_mt(lp, m, n, ii, mt, A, m, T, mt, w, lw)
        assert L.dgeqrf_q03_mt(list(lp), m, n, ii, mt, dA, m, dT, mt, dQ, m, dW, lw) == 0
        oracle_lib.dgeqrf_q03_mt(lp, m, n, ii, mt, A, m, T, mt, Q, m, w, lw)
        torch.cuda.synchronize()
        err = C.compare_factor((L.from_device(dA), L.from_device(dT), L.from_device(dQ)), (A, T, Q), m, n, ii, mt)
        assert max(err.values()) < C.TOL, (leaf, panel, err)
    # one tile's panel (ii % mt + n <= mt): v03_3 / q03_l / q03_3 and the dispatchers
    pn, pi = 6, 9
    for vfn, qfn, lp in (("dgeqr2_v03_3", "dgeqr2_q03_3", None), ("dgeqr2_v03_l", "dgeqr2_q03_l", None),
                         ("dgeqr2_v03", "dgeqr2_q03", [0, 1, 1, 4])):
        A, T, Q = C.inputs(m, pn + pi, 0, mt, seed=7)
        dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
        dW = torch.empty(lw, dtype=torch.float64, device="cuda")
        w = np.zeros(lw)
        head = [lp] if lp else []
        headc = [np.array(lp, dtype=np.int32)] if lp else []
        assert getattr(L, vfn)(*head, m, pn, pi, mt, dA, m, dT, mt, dW, lw) == 0
        getattr(oracle_lib, vfn)(*headc, m, pn, pi, mt, A, m, T, mt, w, lw)
        assert getattr(L, qfn)(*head, m, pn, pi, mt, dA, m, dT, mt, dQ, m, dW, lw) == 0
        getattr(oracle_lib, qfn)(*headc, m, pn, pi, mt, A, m, T, mt, Q, m, w, lw)
        torch.cuda.synchronize()
        err = C.compare_factor((L.from_device(dA), L.from_device(dT), L.from_device(dQ)), (A, T, Q), m, pn, pi, mt)
        assert max(err.values()) < C.TOL, (vfn, err)
    # leaf 2: nothing happens (the tile updates around a panel-2 no-op do run, as in the reference)
    A, T, Q = C.inputs(m, n, ii, mt, seed=8)
    dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dgeqrf_v03_recursive([0, 2, 0, 64], m, n, ii, mt, dA, m, dT, mt, dW, lw) == 0
    assert L.dgeqrf_q03_recursive([0, 2, 1, 64], m, n, ii, mt, dA, m, dT, mt, dQ, m, dW, lw) == 0
    torch.cuda.synchronize()
    assert np.array_equal(L.from_device(dA), A) and np.array_equal(L.from_device(dT), T)
    assert np.array_equal(L.from_device(dQ), Q)
    # argument checks
    d = torch.zeros(64, dtype=torch.float64, device="cuda")
    assert L.dgeqrf_v03_recursive([0, 3, 1, 8], 10, 5, 0, 4, d, 10, d, 4, d, 64) == -1  # no split leaf
    assert L.dgeqrf_v03_recursive([0, 1, 1, 8], 10, 20, 0, 4, d, 10, d, 4, d, 64) == -3  # n > m
    assert L.dgeqrf_v03_recursive([0, 1, 1, 8], 10, 5, 0, 4, d, 5, d, 4, d, 64) == -7   # lda < m
    assert L.dgeqrf_v03_recursive([0, 1, 1, 2], 100, 50, 0, 8, d, 100, d, 8, d, 1) == -11  # lwork
    assert L.dgeqrf_q03_recursive([0, 1, 1, 8], 10, 5, 0, 4, d, 10, d, 4, d, 5, d, 64) == -11  # ldq < m
    assert L.dgeqrf_q03_recursive([0, 1, 1, 2], 100, 50, 0, 8, d, 100, d, 8, d, 100, d, 1) == -13  # lwork
    assert L.dgeqr2_v03_3(10, 5, 2, 4, d, 10, d, 4, d, 64) == -2  # panel crosses a tile
    torch.cuda.synchronize()
    assert L.gpu_status() == 0


def test_recursive_autotune(gpu_lib, oracle_lib, torch_cuda):
    """lila_gpu_recursive_autotune picks (mt, nx) from its candidates without
    touching A, and the recursive driver with the picked values stays in
    parity with the oracle."""
    L, torch = gpu_lib, torch_cuda
    m, n = 600, 300
    A0, _, _ = C.inputs(m, n, 0, 128, seed=9)
    dA0 = L.to_device_colmajor(A0)
    dS, dT, dQ = L.colmajor(m, n), L.colmajor(128, n, fill=0.0), L.colmajor(m, n, fill=0.0)
    lw = max(L.query_dgeqrf_w03_recursive([0, 1, 1, x], m, n, 0, t, None, m, None, t, None, m, None, -1)
             for t in (32, 64, 128) for x in (32, 64, 128, 256))
    W = torch.empty(lw, dtype=torch.float64, device="cuda")
    rc, mt, nx = L.recursive_autotune([0, 1, 1, 64], m, n, dA0, m, dS, dT, 128, dQ, m, W, lw)
    assert rc > 0 and mt in (32, 64, 128) and nx in (32, 64, 128, 256, 512), (rc, mt, nx)
    assert np.array_equal(L.from_device(dA0), A0)
    out = C.run_gpu(L, "recursive", m, n, 0, mt, 1, 1, nx, seed=10)
    ref = C.run_cpu(oracle_lib, "recursive", m, n, 0, mt, 1, 1, nx, seed=10)
    err = C.compare_factor(out, ref, m, n, 0, mt)
    assert max(err.values()) < C.TOL, (mt, nx, err)
    # the split-precision leaf keeps nx <= 64; no candidate fits a tiny workspace
    lw3 = max(L.query_dgeqrf_w03_recursive([0, 3, 1, x], m, 64, 0, t, None, m, None, t, None, m, None, -1)
              for t in (32, 64, 128) for x in (32, 64))
    W3 = torch.empty(lw3, dtype=torch.float64, device="cuda")
    rc, mt3, nx3 = L.recursive_autotune([0, 3, 1, 64], m, 64, dA0, m, dS, dT, 128, dQ, m, W3, lw3)
    assert rc > 0 and nx3 <= 64, (rc, mt3, nx3)
    assert L.recursive_autotune([0, 1, 1, 64], m, n, dA0, m, dS, dT, 128, dQ, m, W, 1)[0] == -12
    torch.cuda.synchronize()
    assert L.gpu_status() == 0


def test_invalid_arguments_are_rejected(gpu_lib, torch_cuda):
    L, torch = gpu_lib, torch_cuda
    d = torch.zeros(64, dtype=torch.float64, device="cuda")
    lp = [0, 1, 1, 8]
    assert L.dgeqrf_w03_recursive(lp, 10, 20, 0, 4, d, 10, d, 4, d, 10, d, 64) == -3  # n > m
    assert L.dgeqrf_w03_recursive(lp, 10, 5, 0, 4, d, 5, d, 4, d, 10, d, 64) == -7   # lda < m
    assert L.dgeqrf_w03_recursive(lp, 10, 5, 0, 0, d, 10, d, 4, d, 10, d, 64) == -5  # mt = 0
    assert L.dgeqrf_w03_recursive(lp, 100, 50, 0, 8, d, 100, d, 8, d, 100, d, 1) == -13  # lwork
    assert L.dgeqrf_w03_recursive([0, 5, 1, 8], 10, 5, 0, 4, d, 10, d, 4, d, 10, d, 64) == -1
    assert L.dormqrf_w03(10, 3, 2, 0, 1, 4, d, 10, d, 4, d, 64) == -5  # j inside the reflectors
    # empty problems are no-ops
    assert L.dgeqrf_w03_recursive(lp, 10, 0, 0, 4, d, 10, d, 4, d, 10, d, 64) == 0
    assert L.dormqrf_w03(10, 0, 2, 0, 2, 4, d, 10, d, 4, d, 64) == 0
    torch.cuda.synchronize()
    assert L.gpu_status() == 0


def test_recursive_4000x1000_accuracy(gpu_lib, torch_cuda):
    """4000 x 1000 recursive QR + explicit Q (the recursive workload's shape): accuracy gates."""
    import oracle as O

    L, torch = gpu_lib, torch_cuda
    m, n, mt, nx = 4000, 1000, 64, 64
    rng = np.random.default_rng(101)
    A = np.asfortranarray(rng.standard_normal((m, n)))
    dA = L.to_device_colmajor(A)
    dT = L.colmajor(mt, n, fill=0.0)
    dQ = L.colmajor(m, n, fill=0.0)
    lp = [0, 1, 1, nx]
    lw = L.query_dgeqrf_w03_recursive(lp, m, n, 0, mt, None, m, None, mt, None, m, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dgeqrf_w03_recursive(lp, m, n, 0, mt, dA, m, dT, mt, dQ, m, dW, lw) == 0
    torch.cuda.synchronize()
    Ag = L.from_device(dA)
    Qg = L.from_device(dQ)
    R = np.triu(Ag[:n, :n])
    tol = 50 * n * 2.0 ** -53
    assert np.linalg.norm(Qg @ R - A) / np.linalg.norm(A) < tol
    assert np.linalg.norm(np.eye(n) - Qg.T @ Qg) < tol
    # elementwise against the oracle restatement (on OpenBLAS when present, for speed)
    lib = O.load("oracle_ob") or O.load("oracle")
    Ao = A.copy(order="F")
    To = np.asfortranarray(np.zeros((mt, n)))
    Qo = np.asfortranarray(np.zeros((m, n)))
    work = np.zeros(8 * m * mt + 4 * n * n)
    lib.dgeqrf_w03_recursive(C.lparam(1, 1, nx), m, n, 0, mt, Ao, m, To, mt, Qo, m, work, work.size)
    assert C.max_rel(Ag, Ao) < C.TOL
    assert C.max_rel(Qg, Qo) < C.TOL
