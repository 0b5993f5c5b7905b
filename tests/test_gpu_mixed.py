"""Split-precision tall-skinny leaf (Cholesky QR 2 / shifted 3 + Householder
reconstruction on the BF16 tensor cores): accuracy gates at the condition
numbers of the tall-skinny workload, reflector consistency, and parity with
the oracle after sign normalisation."""
import numpy as np
import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu


def usv(m, n, kappa, seed_u, seed_v):
    rng = np.random.default_rng(seed_u)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    rv = np.random.default_rng(seed_v)
    V, Rv = np.linalg.qr(rv.standard_normal((n, n)))
    V = V * np.sign(np.diag(Rv))[None, :]
    sig = kappa ** (-np.arange(n) / (n - 1))
    return np.asfortranarray((U * sig[None, :]) @ V.T)


def run_mixed(L, A, mt, variant=0, i=0):
    import torch

    m = A.shape[0]
    n = A.shape[1] - i
    dA = L.to_device_colmajor(A)
    dT = L.colmajor(mt, n + i, fill=0.0)
    dQ = L.colmajor(m, n + i, fill=0.0)
    lw = L.query_dgeqrf_w03_mt_hr_mixed(m, n, i, mt, None, m, None, mt, None, m, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    rc = L.dgeqrf_w03_mt_hr_mixed_v(variant, m, n, i, mt, dA, m, dT, mt, dQ, m, dW, lw)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return dA, dT, dQ


def reflectors_reproduce_q(L, dA, dT, dQ, m, n, mt, i=0):
    """H^T Q must be [I; 0] when V, T and Q S come from the same reconstruction."""
    import torch

    dB = dQ.clone()
    lw = L.query_dormqrf_w03(m, n, n, i, i, mt, None, m, None, mt, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dormqrf_z03(m, n, n, i, i, mt, dA, m, dT, mt, dB, m, dW, lw) == 0
    B = L.from_device(dB)[i:, i:i + n]
    E = B.copy()
    E[:n] -= np.eye(n)
    return np.abs(E).max()


@pytest.mark.parametrize("kappa,variant", [(1e2, 1), (1e6, None), (1e10, 2), (1e14, 2)])
def test_mixed_accuracy_gates(gpu_lib, kappa, variant):
    L = gpu_lib
    L.gpu_clear_status()
    m, n, mt = 200000, 64, 32
    A = usv(m, n, kappa, 201, 202)
    dA, dT, dQ = run_mixed(L, A, mt)
    status = L.gpu_status()
    Ag, Qg = L.from_device(dA), L.from_device(dQ)
    R = np.triu(Ag[:n, :n])
    tol = 50 * n * 2.0 ** -53
    res = np.linalg.norm(Qg @ R - A) / np.linalg.norm(A)
    orth = np.linalg.norm(np.eye(n) - Qg.T @ Qg)
    print("kappa %g variant %d passes %d status %d res %.3g orth %.3g" % (
        kappa, L.gpu_last_variant(), L.gpu_last_passes(), status, res, orth))
    if variant is not None:
        assert L.gpu_last_variant() == variant
    assert res <= tol, res
    assert orth <= tol, orth
    assert reflectors_reproduce_q(L, dA, dT, dQ, m, n, mt) < 1e-12
    assert L.gpu_status() == 0


def test_mixed_matches_householder_after_sign_normalisation(gpu_lib, oracle_lib):
    L = gpu_lib
    m, n, mt = 20000, 64, 16
    A = usv(m, n, 1e2, 5, 6)
    dA, dT, dQ = run_mixed(L, A, mt)
    Ag, Qg = L.from_device(dA), L.from_device(dQ)
    Rg = np.triu(Ag[:n, :n])
    # oracle Householder QR (recursive, leaf 1 panel 1) of the same A
    Ao = A.copy(order="F")
    To = np.asfortranarray(np.zeros((mt, n)))
    Qo = np.asfortranarray(np.zeros((m, n)))
    work = np.zeros(8 * m * mt + 4 * n * n)
    oracle_lib.dgeqrf_w03_recursive(C.lparam(1, 1, 16), m, n, 0, mt, Ao, m, To, mt, Qo, m, work, work.size)
    Ro = np.triu(Ao[:n, :n])
    sg, so = np.sign(np.diag(Rg)), np.sign(np.diag(Ro))
    assert C.max_rel(Rg * sg[:, None], Ro * so[:, None]) < 1e-12
    assert C.max_rel(Qg * sg[None, :], Qo * so[None, :]) < 1e-12


def test_mixed_matches_plain_reconstruction(gpu_lib, oracle_lib):
    """Same V, T, S R and Q S as the FP64 Cholesky QR + reconstruction leaf on a
    well-conditioned block, with a leaf offset i and tiles that straddle it."""
    L = gpu_lib
    m, n, i, mt = 30000, 50, 6, 16
    rng = np.random.default_rng(9)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, n + i)))
    dA, dT, dQ = run_mixed(L, A, mt, variant=1, i=i)
    Ao = A.copy(order="F")
    To = np.asfortranarray(np.zeros((mt, n + i)))
    Qo = np.asfortranarray(np.zeros((m, n + i)))
    work = np.zeros(oracle_lib.query_dgeqrf_w03_mt_hr(m, n, i, mt) + 16)
    oracle_lib.dgeqrf_w03_mt_hr(m, n, i, mt, Ao, m, To, mt, Qo, m, work, work.size)
    err = C.compare_factor((L.from_device(dA), L.from_device(dT), L.from_device(dQ)), (Ao, To, Qo), m, n, i, mt)
    assert max(err.values()) < 1e-12, err


def test_recursive_with_mixed_leaves(gpu_lib, oracle_lib):
    import torch

    L = gpu_lib
    m, n, mt, nx = 6000, 256, 32, 64
    A = usv(m, n, 1e4, 11, 12)
    dA, dT, dQ = L.to_device_colmajor(A), L.colmajor(mt, n, fill=0.0), L.colmajor(m, n, fill=0.0)
    lp = [0, 3, 1, nx]
    lw = L.query_dgeqrf_w03_recursive(lp, m, n, 0, mt, None, m, None, mt, None, m, None, -1)
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dgeqrf_w03_recursive(lp, m, n, 0, mt, dA, m, dT, mt, dQ, m, dW, lw) == 0
    torch.cuda.synchronize()
    Ag, Qg = L.from_device(dA), L.from_device(dQ)
    R = np.triu(Ag[:n, :n])
    tol = 50 * n * 2.0 ** -53
    assert np.linalg.norm(Qg @ R - A) / np.linalg.norm(A) <= tol
    assert np.linalg.norm(np.eye(n) - Qg.T @ Qg) <= tol
    assert reflectors_reproduce_q(L, dA, dT, dQ, m, n, mt) < 1e-12
    assert L.gpu_status() == 0


@pytest.mark.parametrize("kappa,rows", [(1e2, 40000), (1e10, 65536), (1e14, 0)])
def test_out_of_core_matches_in_core(gpu_lib, kappa, rows):
    """lila_gpu_dgeqrf_tall_host: A and Q stay in page-locked host memory and
    stream through the device in chunks (several chunks and a short last one
    for rows > 0, one chunk for rows = 0).  The accuracy gates, H^T Q = [I; 0]
    from the written V and T, and, where the Gram's chunked summation cannot
    move the factors (kappa = 1e2), the in-core leaf's passes and elementwise
    agreement with it."""
    import torch

    L = gpu_lib
    m, n, mt = 200077, 64, 32
    A = usv(m, n, kappa, 203, 204)
    hA = torch.empty((n, m), dtype=torch.float64, pin_memory=True).t()
    hA.copy_(torch.from_numpy(A))
    hQ = torch.zeros((n, m), dtype=torch.float64, pin_memory=True).t()
    dT = L.colmajor(mt, n, fill=0.0)
    lw = L.lib().lila_gpu_query_dgeqrf_tall_host(m, n, rows)
    assert lw > 0
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    L.gpu_clear_status()
    assert L.gpu_dgeqrf_tall_host(m, n, mt, hA, m, dT, mt, hQ, m, rows, dW, lw) == 0
    torch.cuda.synchronize()
    assert L.gpu_status() == 0
    passes = L.gpu_last_passes()
    Ao, Qo = hA.numpy().copy(), hQ.numpy().copy()
    R = np.triu(Ao[:n, :n])
    res = np.linalg.norm(A - Qo @ R) / np.linalg.norm(A)
    orth = np.linalg.norm(np.eye(n) - Qo.T @ Qo)
    tol = 50 * n * 2.0 ** -53
    assert res <= tol and orth <= tol, (kappa, res, orth)
    dA, dQ = L.to_device_colmajor(Ao), L.to_device_colmajor(Qo)
    assert reflectors_reproduce_q(L, dA, dT, dQ, m, n, mt) < 1e-12
    iA, iT, iQ = run_mixed(L, A, mt)
    if kappa <= 1e2:
        assert L.gpu_last_passes() == passes == 2
        err = C.compare_factor((Ao, L.from_device(dT), Qo), (L.from_device(iA), L.from_device(iT), L.from_device(iQ)),
                               m, n, 0, mt)
        assert max(err.values()) < 1e-12, err
    # argument checks
    assert L.gpu_dgeqrf_tall_host(m, 65, mt, hA, m, dT, mt, hQ, m, rows, dW, lw) == -2
    assert L.gpu_dgeqrf_tall_host(m, n, mt, hA, m, dT, mt, hQ, m, rows, dW, 16) == -12


@pytest.mark.parametrize("m,kappa", [(300001, 1e2), (262144 + 77, 1e12)])
def test_ahead_scheduled_maps_agree_bitwise(gpu_lib, m, kappa):
    """The leaf's row maps with row scales passed between them (the default:
    the map runs one K half ahead) and without (each map finds its input's
    row scales itself, lila_prim_ozaki_map_path(1)) produce the same V, T
    and Q bit for bit."""
    L = gpu_lib
    A = usv(m, 64, kappa, 41, 42)
    outs = []
    for path in (0, 1):
        prev = L.prim_ozaki_map_path(path)
        try:
            dA, dT, dQ = run_mixed(L, A, 32)
            outs.append((L.from_device(dA), L.from_device(dT), L.from_device(dQ), L.gpu_last_passes()))
        finally:
            L.prim_ozaki_map_path(prev)
    assert outs[0][3] == outs[1][3]
    for a, b in zip(outs[0][:3], outs[1][:3]):
        assert np.array_equal(a, b)
    assert L.gpu_status() == 0
