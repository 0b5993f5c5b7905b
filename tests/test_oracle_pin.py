"""Pin the CPU oracle (oracle/lila_oracle.c) to the reference.

Two sources of truth:
  * the committed fixtures in tests/golden/ (made by the reference's own C
    code, see tests/golden/make_golden.py) -- always checked;
  * the reference compiled into oracle/_ref/ -- checked on the reference's
    sweep shapes wherever that checkout exists.
"""
import glob
import os

import numpy as np
import pytest

import lila_cases as C

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden_driver_files():
    return sorted(f for f in glob.glob(os.path.join(GOLD, "*.npz"))
                  if os.path.basename(f).startswith(("rec_", "lvx_")))


@pytest.mark.parametrize("path", _golden_driver_files(), ids=os.path.basename)
def test_oracle_matches_golden(oracle_lib, path):
    g = np.load(path)
    m, n, ii, mt, lda, ldq, leaf, panel = [int(v) for v in g["shape"]]
    nb = [int(v) for v in g["nb"]]
    mode = "levelx" if os.path.basename(path).startswith("lvx_") else "recursive"
    out = C.run_cpu(oracle_lib, mode, m, n, ii, mt, leaf, panel, nb[0] if mode == "recursive" else None,
                    lda, ldq, seed=0, nb=nb if mode == "levelx" else None)
    err = C.compare_factor(out, (g["A"], g["T"], g["Q"]), m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "vq_*.npz"))), ids=os.path.basename)
def test_oracle_v03_q03_match_golden(oracle_lib, path):
    g = np.load(path)
    m, n, ii, mt, lda, ldq, leaf, panel = [int(v) for v in g["shape"]]
    nb = [int(v) for v in g["nb"]]
    mode = "levelx" if "_lvx_" in os.path.basename(path) else "recursive"
    out = C.run_cpu_vq(oracle_lib, mode, m, n, ii, mt, leaf, panel, nb[0] if mode == "recursive" else None,
                       lda, ldq, seed=0, nb=nb if mode == "levelx" else None)
    err = C.compare_factor(out, (g["A"], g["T"], g["Q"]), m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


def test_oracle_ormqr_golden(oracle_lib):
    m, n, ii, mt, nrhs = 87, 53, 6, 4, 8
    A, T, Q = C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, 1, 1, 7, seed=0)
    rng = np.random.default_rng(102)
    B = np.asfortranarray(rng.standard_normal((m, nrhs)))
    work = np.zeros(8 * m * (nrhs + mt))
    oracle_lib.dormqrf_z03(m, nrhs, n, ii, 0, mt, A, m, T, mt, B, m, work, work.size)
    g = np.load(os.path.join(GOLD, "ormqr_z03_87x53.npz"))
    assert C.max_rel(B, g["B"]) < C.TOL


def test_oracle_ls_golden(oracle_lib):
    m, n, k = 60, 20, 4
    rng = np.random.default_rng(400)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, n)))
    b = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, k)))
    T = np.asfortranarray(np.zeros((n, n)))
    work = np.zeros(n * k)
    oracle_lib.ls_solve(m, n, k, A, m, T, n, b, m, work)
    g = np.load(os.path.join(GOLD, "ls_60x20.npz"))
    assert C.max_rel(A, g["A"]) < C.TOL
    assert C.max_rel(np.triu(T), np.triu(g["T"])) < C.TOL
    assert C.max_rel(b[:n], g["x"]) < 1e-11


@pytest.mark.parametrize("case", C.UGLY, ids=lambda c: "x".join(map(str, c)))
def test_oracle_matches_reference_sweep(oracle_lib, ref_lib, case):
    m, n, ii, mt, lda, ldq, leaf, panel, nx = case
    out = C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=1)
    ref = C.run_cpu(ref_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=1)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("nb", [[10], [20, 5], [16, 8, 4], [7, 3]])
def test_oracle_matches_reference_levelx(oracle_lib, ref_lib, nb):
    m, n, ii, mt = 87, 53, 6, 4
    out = C.run_cpu(oracle_lib, "levelx", m, n, ii, mt, 1, 1, None, seed=2, nb=nb)
    ref = C.run_cpu(ref_lib, "levelx", m, n, ii, mt, 1, 1, None, seed=2, nb=nb)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("case", C.VQ_CASES, ids=lambda c: "x".join(map(str, c)))
def test_oracle_v03_q03_match_reference(oracle_lib, ref_lib, case):
    """V, R, T of the v03 driver and Q of the q03 driver on its output."""
    m, n, ii, mt, lda, ldq, leaf, panel, nx = case
    out = C.run_cpu_vq(oracle_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=3)
    ref = C.run_cpu_vq(ref_lib, "recursive", m, n, ii, mt, leaf, panel, nx, lda, ldq, seed=3)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("nb", [[10], [20, 5], [16, 8, 4]])
def test_oracle_v03_q03_levelx_match_reference(oracle_lib, ref_lib, nb):
    m, n, ii, mt = 87, 53, 6, 4
    out = C.run_cpu_vq(oracle_lib, "levelx", m, n, ii, mt, 1, 1, None, seed=4, nb=nb)
    ref = C.run_cpu_vq(ref_lib, "levelx", m, n, ii, mt, 1, 1, None, seed=4, nb=nb)
    err = C.compare_factor(out, ref, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("leaf,panel", [(0, 0), (1, 0), (1, 1)])
def test_oracle_v03_q03_leaves_and_panels_match_reference(oracle_lib, ref_lib, leaf, panel):
    """The leaf dispatchers (_mt) and the one-tile panels (_l, _3) of v03 /
    q03 one by one, oracle against the compiled reference."""
    m, n, ii, mt = 120, 24, 8, 8
    lw = 8 * (m + n + ii) * (n + ii + mt) + 4096
    outs = []
    for lib in (oracle_lib, ref_lib):
        A, T, Q = C.inputs(m, n, ii, mt, seed=6)
        lp = np.array([0, leaf, panel, 64], dtype=np.int32)
        w = np.zeros(lw)
        lib.dgeqrf_v03_mt(lp, m, n, ii, mt, A, m, T, mt, w, lw)
        lib.dgeqrf_q03_mt(lp, m, n, ii, mt, A, m, T, mt, Q, m, w, lw)
        outs.append((A, T, Q))
    err = C.compare_factor(outs[0], outs[1], m, n, ii, mt)
    assert max(err.values()) < C.TOL, err
    pn, pi = 6, 9
    vfn, qfn = ("dgeqr2_v03_l", "dgeqr2_q03_l") if panel == 0 else ("dgeqr2_v03_3", "dgeqr2_q03_3")
    outs = []
    for lib in (oracle_lib, ref_lib):
        A, T, Q = C.inputs(m, pn + pi, 0, mt, seed=7)
        w = np.zeros(lw)
        getattr(lib, vfn)(m, pn, pi, mt, A, m, T, mt, w, lw)
        getattr(lib, qfn)(m, pn, pi, mt, A, m, T, mt, Q, m, w, lw)
        outs.append((A, T, Q))
    err = C.compare_factor(outs[0], outs[1], m, pn, pi, mt)
    assert max(err.values()) < C.TOL, (vfn, err)


def test_oracle_v03_q03_equal_w03(oracle_lib):
    """v03 then q03 gives the w03 factorization (V, R, T and Q)."""
    m, n, ii, mt = 141, 69, 9, 7
    vq = C.run_cpu_vq(oracle_lib, "recursive", m, n, ii, mt, 1, 1, 9, seed=5)
    w = C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, 1, 1, 9, seed=5)
    err = C.compare_factor(vq, w, m, n, ii, mt)
    assert max(err.values()) < C.TOL, err


@pytest.mark.parametrize("mt", [1, 2, 3, 7, 10, 60])
def test_oracle_matches_reference_mt_sweep(oracle_lib, ref_lib, mt):
    """mt sweep of backup_test.sh_files/test_main_recursive_mt.sh, scaled down."""
    m, n, ii, nx = 141, 69, 9, 9
    for leaf, panel in ((1, 1), (1, 0), (0, 0)):
        out = C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, leaf, panel, nx, 160, 150, seed=3)
        ref = C.run_cpu(ref_lib, "recursive", m, n, ii, mt, leaf, panel, nx, 160, 150, seed=3)
        err = C.compare_factor(out, ref, m, n, ii, mt)
        assert max(err.values()) < C.TOL, (leaf, panel, err)


def test_reference_mt_hr_alias_defect_is_fixed(oracle_lib, ref_lib):
    """Leaf 2 over >= 3 mt tiles: the reference's S/work2 alias breaks R; the oracle is exact."""
    m, n, ii, mt = 87, 53, 6, 16
    A0, _, _ = C.inputs(m, n, ii, mt, seed=0)
    out = C.run_cpu(oracle_lib, "recursive", m, n, ii, mt, 2, 0, 53, seed=0)
    ref = C.run_cpu(ref_lib, "recursive", m, n, ii, mt, 2, 0, 53, seed=0)
    res_o, orth_o = C.residuals(A0, out, m, n, ii)
    res_r, _ = C.residuals(A0, ref, m, n, ii)
    assert res_o < 1e-14 and orth_o < 1e-13
    assert res_r > 1e-3  # documented reference defect


def test_oracle_queries_cover_reference(oracle_lib, ref_lib):
    """Workspace queries: the oracle's covers the reference's (plus S for mt_hr)."""
    for (m, n, ii, mt, nx) in [(87, 53, 6, 4, 7), (4000, 1000, 0, 200, 20), (1413, 692, 97, 9, 9)]:
        for leaf, panel in ((1, 1), (0, 0), (1, 2)):
            lp = C.lparam(leaf, panel, nx)
            q_o = oracle_lib.query_dgeqrf_w03_recursive(lp, m, n, ii, mt)
            q_r = ref_lib.query_dgeqrf_w03_recursive(lp, m, n, ii, mt, None, m, None, mt, None, m, None, -1)
            assert q_o >= q_r, (m, n, leaf, panel, q_o, q_r)
