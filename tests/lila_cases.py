"""Shared case generators and comparisons for the parity tests.

Inputs follow the reference drivers' layout (lila-c/main_w03.c:129-183):
A is lda x (n+ii), Q is ldq x (n+ii), T is mt x (n+ii), all column-major;
entries are seeded uniform(-0.5, 0.5) (numpy PCG64, platform independent).
"""
import numpy as np

TOL = 1e-12  # elementwise, relative to max(1, max|reference|) of each output


def tile_mask(n, ii, mt):
    """Defined entries of T: upper triangle of each tile, reflectors in [ii, ii+n)."""
    M = np.zeros((mt, n + ii), dtype=bool)
    for c in range(ii, ii + n):
        tstart = c - c % mt
        first = max(ii, tstart)
        for r in range(first - tstart, c % mt + 1):
            M[r, c] = True
    return M


def inputs(m, n, ii, mt, lda=None, ldq=None, seed=0):
    lda = lda or m
    ldq = ldq or m
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (lda, n + ii)))
    Q = np.asfortranarray(rng.uniform(-0.5, 0.5, (ldq, n + ii)))
    T = np.asfortranarray(np.full((mt, n + ii), 7.0))
    return A, T, Q


def lparam(leaf, panel, nx):
    return np.array([0, leaf, panel, nx], dtype=np.int32)


def run_cpu(lib, mode, m, n, ii, mt, leaf, panel, nx, lda=None, ldq=None, seed=0, nb=None):
    """Run a driver of the oracle / compiled reference on fresh inputs."""
    lda = lda or m
    ldq = ldq or m
    A, T, Q = inputs(m, n, ii, mt, lda, ldq, seed)
    lwork = 8 * (m + n + ii) * (n + ii + mt) + 4 * (n + ii) ** 2 + 4096
    work = np.zeros(lwork)
    if mode == "recursive":
        lib.dgeqrf_w03_recursive(lparam(leaf, panel, nx), m, n, ii, mt, A, lda, T, mt, Q, ldq, work, lwork)
    elif mode == "levelx":
        nbl = np.array(nb, dtype=np.int32)
        lib.dgeqrf_w03_levelx(lparam(leaf, panel, len(nb)), len(nb), 0, nbl, m, n, ii, mt, A, lda, T,
                              mt, Q, ldq, work, lwork)
    else:
        raise ValueError(mode)
    return A, T, Q


def run_gpu(L, mode, m, n, ii, mt, leaf, panel, nx, lda=None, ldq=None, seed=0, nb=None):
    """Same through the GPU library's C ABI (device buffers, queried workspace)."""
    import torch

    lda = lda or m
    ldq = ldq or m
    A, T, Q = inputs(m, n, ii, mt, lda, ldq, seed)
    dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
    lp = [0, leaf, panel, nx if mode == "recursive" else len(nb)]
    if mode == "recursive":
        lwork = L.query_dgeqrf_w03_recursive(lp, m, n, ii, mt, None, lda, None, mt, None, ldq, None, -1)
        work = torch.empty(max(lwork, 1), dtype=torch.float64, device="cuda")
        rc = L.dgeqrf_w03_recursive(lp, m, n, ii, mt, dA, lda, dT, mt, dQ, ldq, work, lwork)
    else:
        lwork = L.query_dgeqrf_w03_levelx(lp, len(nb), 0, nb, m, n, ii, mt, None, lda, None, mt, None, ldq, None, -1)
        work = torch.empty(max(lwork, 1), dtype=torch.float64, device="cuda")
        rc = L.dgeqrf_w03_levelx(lp, len(nb), 0, nb, m, n, ii, mt, dA, lda, dT, mt, dQ, ldq, work, lwork)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return L.from_device(dA), L.from_device(dT), L.from_device(dQ)


def _vq_calls(lib, mode, lp, m, n, ii, mt, A, lda, T, Q, ldq, work, lwork, nb):
    """v03 then q03 on the same A and T (any lib exposing both)."""
    if mode == "recursive":
        rv = lib.dgeqrf_v03_recursive(lp, m, n, ii, mt, A, lda, T, mt, work, lwork)
        rq = lib.dgeqrf_q03_recursive(lp, m, n, ii, mt, A, lda, T, mt, Q, ldq, work, lwork)
    elif mode == "levelx":
        nbl = np.array(nb, dtype=np.int32) if isinstance(A, np.ndarray) else list(nb)
        rv = lib.dgeqrf_v03_levelx(lp, len(nb), 0, nbl, m, n, ii, mt, A, lda, T, mt, work, lwork)
        rq = lib.dgeqrf_q03_levelx(lp, len(nb), 0, nbl, m, n, ii, mt, A, lda, T, mt, Q, ldq, work, lwork)
    else:
        raise ValueError(mode)
    return rv, rq


def run_cpu_vq(lib, mode, m, n, ii, mt, leaf, panel, nx, lda=None, ldq=None, seed=0, nb=None):
    """V, R, T by the v03 driver, then Q from them by the q03 driver."""
    lda = lda or m
    ldq = ldq or m
    A, T, Q = inputs(m, n, ii, mt, lda, ldq, seed)
    lwork = 8 * (m + n + ii) * (n + ii + mt) + 4 * (n + ii) ** 2 + 4096
    work = np.zeros(lwork)
    lp = lparam(leaf, panel, nx if mode == "recursive" else len(nb))
    _vq_calls(lib, mode, lp, m, n, ii, mt, A, lda, T, Q, ldq, work, lwork, nb)
    return A, T, Q


def run_gpu_vq(L, mode, m, n, ii, mt, leaf, panel, nx, lda=None, ldq=None, seed=0, nb=None):
    """Same through the GPU library (workspace from the w03 query)."""
    import torch

    lda = lda or m
    ldq = ldq or m
    A, T, Q = inputs(m, n, ii, mt, lda, ldq, seed)
    dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
    lp = [0, leaf, panel, nx if mode == "recursive" else len(nb)]
    if mode == "recursive":
        lwork = L.query_dgeqrf_w03_recursive(lp, m, n, ii, mt, None, lda, None, mt, None, ldq, None, -1)
    else:
        lwork = L.query_dgeqrf_w03_levelx(lp, len(nb), 0, nb, m, n, ii, mt, None, lda, None, mt, None, ldq,
                                          None, -1)
    work = torch.empty(max(lwork, 1), dtype=torch.float64, device="cuda")
    rv, rq = _vq_calls(L, mode, lp, m, n, ii, mt, dA, lda, dT, dQ, ldq, work, lwork, nb)
    assert rv == 0 and rq == 0, (rv, rq)
    torch.cuda.synchronize()
    return L.from_device(dA), L.from_device(dT), L.from_device(dQ)


# v03 / q03 cases: leaves 0 and 1, panels 0 and 1 (leaf 2 / panel 2 are not
# implemented in the reference), nx >= 2
VQ_CASES = [
    # m,   n,  ii, mt, lda, ldq, leaf, panel, nx
    (87, 53, 6, 4, 87, 87, 1, 1, 7),
    (87, 53, 6, 4, 90, 95, 0, 0, 7),
    (87, 53, 6, 4, 87, 87, 1, 0, 7),
    (87, 53, 6, 5, 91, 88, 1, 1, 9),
    (141, 69, 9, 7, 190, 180, 1, 1, 9),
    (141, 69, 9, 70, 141, 141, 0, 1, 9),
    (141, 69, 9, 1, 141, 141, 1, 1, 9),
    (60, 60, 0, 8, 60, 60, 1, 1, 10),
    (200, 64, 0, 32, 200, 200, 1, 1, 2),
]


def max_rel(x, ref):
    return float(np.max(np.abs(x - ref)) / max(1.0, float(np.max(np.abs(ref))))) if ref.size else 0.0


def compare_factor(out, ref, m, n, ii, mt):
    """Return dict of relative max errors over the defined regions."""
    A, T, Q = out
    Ar, Tr, Qr = ref
    M = tile_mask(n, ii, mt)
    return {
        "A": max_rel(A, Ar),
        "T": max_rel(T[M], Tr[M]),
        "Q": max_rel(Q[ii:m, ii:ii + n], Qr[ii:m, ii:ii + n]),
    }


def residuals(A0, out, m, n, ii):
    """||A - QR||/||A|| and ||I - Q^T Q|| of a factorization output."""
    A, T, Q = out
    R = np.triu(A[ii:ii + n, ii:ii + n])
    Qb = Q[ii:m, ii:ii + n]
    Ab = A0[ii:m, ii:ii + n]
    res = np.linalg.norm(Qb @ R - Ab) / np.linalg.norm(Ab)
    orth = np.linalg.norm(np.eye(n) - Qb.T @ Qb)
    return res, orth


# The reference's own sweep shapes (backup_test.sh_files/test_main_recursive_mt.sh:1-60
# uses m=1413 n=692 ii=97 lda=1902 ldq=1809 nx=9; lila-c/main_w03.c:14-25 defaults
# to 87 x 53, ii=6, mt=4, nx=7) scaled down to keep the CPU suite quick.
UGLY = [
    # m,   n,  ii, mt, lda, ldq, leaf, panel, nx
    (87, 53, 6, 4, 87, 87, 1, 1, 7),
    (87, 53, 6, 4, 90, 95, 0, 0, 7),
    (87, 53, 6, 4, 87, 87, 1, 0, 7),
    (87, 53, 6, 4, 87, 87, 1, 2, 7),
    (87, 53, 6, 5, 91, 88, 1, 1, 9),
    (87, 53, 6, 16, 87, 87, 2, 0, 32),
    (120, 40, 0, 32, 120, 120, 2, 0, 64),
    (300, 64, 0, 32, 300, 300, 2, 0, 64),
    (141, 69, 9, 7, 190, 180, 1, 1, 9),
    (141, 69, 9, 70, 141, 141, 1, 1, 9),
    (141, 69, 9, 1, 141, 141, 1, 1, 9),
    (60, 60, 0, 8, 60, 60, 1, 1, 10),
]


def build_c_caller(out_path):
    """Compile tests/c_caller/main_w03_gpu.c (plain C11) against include/ and
    lila_gb300/liblila_gpu.so with gcc; returns the executable's path, or
    None when gcc or the CUDA runtime headers are not there."""
    import os
    import shutil
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if not shutil.which("gcc") or not os.path.exists(os.path.join(cuda, "include", "cuda_runtime.h")):
        return None
    libdir = os.path.join(root, "lila_gb300")
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(root, "include"),
           "-I" + os.path.join(cuda, "include"), os.path.join(root, "tests", "c_caller", "main_w03_gpu.c"),
           "-L" + libdir, "-llila_gpu", "-L" + os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + libdir, "-o", str(out_path)]
    subprocess.check_call(cmd)
    return str(out_path)

