"""C ABI checks that need no GPU: the library loads, exports every symbol the
headers in include/ declare, and the workspace queries behave."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"^\s*(?:int|void\s*\*|void|double|unsigned long long|long long)\s+(\w+)\s*\(", src, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_the_reference_drop_in_routines():
    names = declared_functions()
    for n in ["dgeqr3", "lila_dgeqrf_w03_recursive", "lila_dgeqrf_w03_levelx", "lila_dgeqrf_w03_mt_hr",
              "lila_dlarft_w03", "lila_dlarft_connect_w03", "lila_dormqrf_w03", "lila_dormqrbz_w03",
              "lila_dorgh2"]:
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    so = ctypes.CDLL(gpu_lib.SO_PATH)
    missing = [n for n in declared_functions() if not hasattr(so, n)]
    assert not missing, missing


def test_queries_without_gpu(gpu_lib):
    L = gpu_lib
    lp = [0, 1, 1, 20]
    q = L.query_dgeqrf_w03_recursive(lp, 4000, 1000, 0, 200, None, 4000, None, 200, None, 4000, None, -1)
    assert q >= 2 * 200 * 500  # W and its product for the largest trailing update
    q_hr = L.query_dgeqrf_w03_mt_hr(4194304, 64, 0, 32, None, 4194304, None, 32, None, 4194304, None, -1)
    assert q_hr >= 64 + 32 * 32  # S plus the second tile's coupling block
    q_lx = L.query_dgeqrf_w03_levelx([0, 1, 1, 2], 2, 0, [100, 20], 500, 300, 0, 16, None, 500, None, 16,
                                     None, 500, None, -1)
    assert q_lx > 0
    # invalid parameters give 0 rather than a size
    assert L.query_dgeqrf_w03_recursive([0, 9, 1, 20], 10, 5, 0, 4, None, 10, None, 4, None, 10, None, -1) == 0


def test_queries_cover_reference_needs(gpu_lib, ref_lib):
    """Where the GPU library's scratch plan is smaller than the reference's count it
    must still cover what the GPU routines take (checked by the lwork argument
    tests on the GPU); here we only check the queries are positive and finite."""
    L = gpu_lib
    for (m, n, ii, mt, nx) in [(87, 53, 6, 4, 7), (4000, 1000, 0, 200, 20)]:
        for leaf, panel in ((1, 1), (0, 0), (1, 2), (2, 0)):
            lp = [0, leaf, panel, nx]
            q = L.query_dgeqrf_w03_recursive(lp, m, n, ii, mt, None, m, None, mt, None, m, None, -1)
            assert 0 < q < 2 ** 31 - 1


def test_argument_checks_without_gpu(gpu_lib):
    """The v03 / q03 family, the out-of-core QR, the recursive autotuner and
    the batched handle helpers reject bad arguments before any device work,
    with the documented codes; the out-of-core workspace query follows its
    chunk plan."""
    import ctypes

    L = gpu_lib
    lib = L.lib()
    d = None  # no pointer is dereferenced before the argument checks
    # v03 / q03
    assert L.dgeqrf_v03_recursive([0, 3, 1, 8], 10, 5, 0, 4, d, 10, d, 4, d, 64) == -1   # no split leaf
    assert L.dgeqrf_v03_recursive([0, 1, 1, 8], 10, 20, 0, 4, d, 10, d, 4, d, 64) == -3  # n > m
    assert L.dgeqrf_v03_recursive([0, 1, 1, 8], 10, 5, 0, 4, d, 5, d, 4, d, 64) == -7    # lda < m
    assert L.dgeqrf_v03_recursive([0, 1, 1, 8], 10, 5, 0, 4, d, 10, d, 3, d, 64) == -9   # ldt < mt
    assert L.dgeqrf_v03_recursive([0, 1, 1, 2], 100, 50, 0, 8, d, 100, d, 8, d, 1) == -11  # lwork
    assert L.dgeqrf_q03_recursive([0, 1, 1, 8], 10, 5, 0, 4, d, 10, d, 4, d, 5, d, 64) == -11  # ldq < m
    assert L.dgeqrf_q03_recursive([0, 1, 1, 2], 100, 50, 0, 8, d, 100, d, 8, d, 100, d, 1) == -13
    assert L.dgeqrf_v03_levelx([0, 1, 1, 1], 1, 0, [0], 10, 5, 0, 4, d, 10, d, 4, d, 64) == -4  # nb <= 0
    assert L.dgeqr2_v03_3(10, 5, 2, 4, d, 10, d, 4, d, 64) == -2    # panel crosses a tile
    assert L.dgeqr2_q03_3(10, 5, 2, 4, d, 10, d, 4, d, 10, d, 64) == -2
    # out-of-core QR
    q = lib.lila_gpu_query_dgeqrf_tall_host
    assert q(0, 64, 0) == 0 and q(100, 65, 0) == 0 and q(10, 64, 0) == 0
    q_full, q_small = q(1000000, 64, 0), q(1000000, 64, 4096)
    assert q_full > q_small > 6 * 4096 * 64
    assert q_full - q_small == 6 * 64 * ((1000064 - 4096) // 1)  # six chunk buffers of C x n
    f = L.gpu_dgeqrf_tall_host
    assert f(100, 65, 32, d, 100, d, 32, d, 100, 0, d, 0) == -2
    assert f(100, 8, 0, d, 100, d, 32, d, 100, 0, d, 0) == -3
    assert f(100, 8, 32, d, 100, d, 32, d, 100, 0, d, 0) == -4
    assert f(100, 8, 32, 8, 99, 8, 32, 8, 100, 0, d, 0) == -5
    assert f(100, 8, 32, 8, 100, 8, 16, 8, 100, 0, d, 0) == -7
    assert f(100, 8, 32, 8, 100, 8, 32, 8, 100, -1, d, 0) == -10
    assert f(100, 8, 32, 8, 100, 8, 32, 8, 100, 0, 8, 1) == -12
    # recursive autotuner
    lp = (ctypes.c_int * 4)(0, 1, 1, 64)
    mt = ctypes.c_int(0)
    at = lib.lila_gpu_recursive_autotune
    assert at((ctypes.c_int * 4)(0, 7, 1, 64), 10, 5, d, 10, d, d, 32, d, 10, d, 64, ctypes.byref(mt)) == -1
    assert at(lp, 0, 5, d, 10, d, d, 32, d, 10, d, 64, ctypes.byref(mt)) == -2
    assert at(lp, 10, 5, d, 10, d, d, 32, d, 10, d, 64, ctypes.byref(mt)) == -4
    # batched handle helpers
    assert lib.lila_gels_mixed_set_trial_limit(None, 1e8) == -1
    assert lib.lila_gels_mixed_shifted(None, None) == -1


def test_c_caller_compiles_against_the_headers(gpu_lib, tmp_path):
    """A plain C caller in the reference driver's pattern (tests/c_caller/)
    compiles with -Wall -Wextra -Werror against include/ and links the
    library: the boundary is C, not C++."""
    import lila_cases as C

    exe = C.build_c_caller(tmp_path / "main_w03_gpu")
    if exe is None:
        pytest.skip("gcc or the CUDA runtime headers are not available")
    assert os.path.exists(exe)
