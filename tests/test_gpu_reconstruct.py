"""GPU parity of the Householder reconstruction entry points, called directly.

lila_dorgh2_3 (lila-c/lila_dorgh2_3.c:3-55), lila_ormhr2_w03_hr
(lila-c/lila_ormhr2_w03_hr.c:3-84) and lila_dorgh2 (lila-c/lila.h:38, given
the tile contract of lila_ormhr2_w03_hr) against the oracle on the same
orthonormal Q: V and S R in A, the T tiles, Q S and the sign vector S,
elementwise to 1e-12.  The tile routines run over every tile of a leaf that
starts at a column offset i > 0 (so the rows [i, j) of R are sign-corrected
with the earlier tiles' S and the Q columns are coupled to the earlier
reflectors), with padded leading dimensions.
"""
import numpy as np
import pytest

import lila_cases as C

pytestmark = pytest.mark.gpu


def _orthonormal(m, n, seed):
    rng = np.random.default_rng(seed)
    Q, R = np.linalg.qr(rng.standard_normal((m, n)))
    return Q * np.sign(np.diag(R))[None, :]


def test_dorgh2_3_vs_oracle(gpu_lib, oracle_lib):
    import torch

    L = gpu_lib
    m, n, lda, ldt, ldq = 300, 24, 311, 29, 305
    rng = np.random.default_rng(31)
    Q0 = _orthonormal(m, n, 30)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (lda, n)))
    A[:n, :n] = np.triu(rng.uniform(0.5, 1.5, (n, n))) + np.tril(rng.uniform(-0.5, 0.5, (n, n)), -1)
    A[n:m] = Q0[n:]
    T = np.asfortranarray(np.full((ldt, n), 5.0))
    T[:n] = Q0[:n]
    Q = np.asfortranarray(rng.uniform(-0.5, 0.5, (ldq, n)))
    Q[:m] = Q0
    S = np.zeros(n)
    Ao, To, Qo, So = A.copy(order="F"), T.copy(order="F"), Q.copy(order="F"), S.copy()
    lw = max(1, L.query_dorgh2_3(m, n, None, lda, None, ldt, None, ldq, None, -1, None))
    oracle_lib.dorgh2_3(m, n, Ao, lda, To, ldt, Qo, ldq, np.zeros(lw + 16), lw + 16, So)
    dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
    dS = torch.zeros(n, dtype=torch.float64, device="cuda")
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dorgh2_3(m, n, dA, lda, dT, ldt, dQ, ldq, dW, lw, dS) == 0
    torch.cuda.synchronize()
    Ag, Tg, Qg, Sg = L.from_device(dA), L.from_device(dT), L.from_device(dQ), dS.cpu().numpy()
    assert np.array_equal(Sg, So)
    assert set(np.unique(So)) <= {-1.0, 1.0} and (So == -1.0).any() and (So == 1.0).any()
    assert C.max_rel(Ag[:m], Ao[:m]) < C.TOL
    assert C.max_rel(Tg[:n], To[:n]) < C.TOL
    assert C.max_rel(Qg[:m], Qo[:m]) < C.TOL
    # padding rows stay untouched
    assert np.array_equal(Ag[m:], A[m:]) and np.array_equal(Tg[n:], T[n:]) and np.array_equal(Qg[m:], Q[m:])
    # Q S (S R) reproduces the input product Q R
    R = np.triu(Ag[:n, :n])
    assert np.linalg.norm(Qg[:m] @ R - Q0 @ np.triu(A[:n, :n])) < 1e-12 * np.linalg.norm(R)
    assert L.gpu_status() == 0


def _leaf_state(m, n, i, mt, lda, ldq, seed):
    """A, T, Q as lila_dgeqrf_w03_mt_hr leaves them before its tile loop
    (lila-c/lila_dgeqrf_w03_mt_hr.c:19-22): an orthonormal Q(i:m, i:i+n), its R
    in A's leaf top block, arbitrary values elsewhere."""
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (lda, i + n)))
    Q = np.asfortranarray(rng.uniform(-0.5, 0.5, (ldq, i + n)))
    T = np.asfortranarray(np.full((mt, i + n), 7.0))
    Q[i:m, i:i + n] = _orthonormal(m - i, n, seed + 1)
    A[i:i + n, i:i + n] = np.triu(rng.uniform(0.5, 1.5, (n, n)))
    return A, T, Q


@pytest.mark.parametrize("name", ["ormhr2_w03_hr", "dorgh2"])
@pytest.mark.parametrize("m,n,i,mt,lda,ldq", [(300, 53, 6, 16, 307, 310), (257, 40, 13, 8, 257, 260),
                                               (500, 64, 0, 32, 500, 500)])
def test_tile_reconstruction_vs_oracle(gpu_lib, oracle_lib, name, m, n, i, mt, lda, ldq):
    import torch

    L = gpu_lib
    A, T, Q = _leaf_state(m, n, i, mt, lda, ldq, seed=40 + i)
    Ao, To, Qo = A.copy(order="F"), T.copy(order="F"), Q.copy(order="F")
    So = np.zeros(i + n)
    dA, dT, dQ = L.to_device_colmajor(A), L.to_device_colmajor(T), L.to_device_colmajor(Q)
    dS = torch.zeros(i + n, dtype=torch.float64, device="cuda")
    tiles = 0
    j = i
    while j < i + n:
        vb = min((j // mt + 1) * mt, i + n) - j
        lw = max(1, L.query_ormhr2_w03_hr(m, vb, i, j, -1, mt, None, lda, None, mt, None, ldq, None, -1, None))
        dW = torch.empty(lw, dtype=torch.float64, device="cuda")
        wo = np.zeros(lw + (j - i) * vb + 16)
        if name == "ormhr2_w03_hr":
            oracle_lib.ormhr2_w03_hr(m, vb, i, j, -1, mt, Ao, lda, To, mt, Qo, ldq, wo, wo.size, So)
            rc = L.ormhr2_w03_hr(m, vb, i, j, -1, mt, dA, lda, dT, mt, dQ, ldq, dW, lw, dS)
        else:
            oracle_lib.dorgh2(m, vb, i, j, mt, Ao, lda, To, mt, Qo, ldq, wo, wo.size, So)
            rc = L.dorgh2(m, vb, i, j, mt, dA, lda, dT, mt, dQ, ldq, dW, lw, dS)
        assert rc == 0, (j, rc)
        j += vb
        tiles += 1
    assert tiles >= 2
    torch.cuda.synchronize()
    Ag, Tg, Qg = L.from_device(dA), L.from_device(dT), L.from_device(dQ)
    Sg = dS.cpu().numpy()
    assert np.array_equal(Sg[i:], So[i:])
    err = C.compare_factor((Ag[:, :], Tg, Qg), (Ao, To, Qo), m, n, i, mt)
    assert max(err.values()) < C.TOL, err
    # columns before the leaf and padding rows stay untouched
    assert np.array_equal(Ag[:, :i], A[:, :i]) and np.array_equal(Ag[m:], A[m:])
    assert np.array_equal(Qg[:, :i], Q[:, :i]) and np.array_equal(Qg[m:], Q[m:])
    # the result is a Householder QR of Q_leaf R: the reflectors applied to
    # Q S give [I; 0] and Q S (S R) equals the input product
    R = np.triu(Ag[i:i + n, i:i + n])
    QS = Qg[i:m, i:i + n]
    assert np.linalg.norm(QS @ R - Q[i:m, i:i + n] @ A[i:i + n, i:i + n]) < 1e-12 * np.linalg.norm(R)
    lw = L.query_dormqrf_w03(m, n, n, i, i, mt, None, lda, None, mt, None, -1)
    dB = L.to_device_colmajor(np.asfortranarray(Qg[:m]))
    dW = torch.empty(lw, dtype=torch.float64, device="cuda")
    assert L.dormqrf_z03(m, n, n, i, i, mt, dA, lda, dT, mt, dB, m, dW, lw) == 0
    B = L.from_device(dB)[i:m, i:i + n]
    B[:n] -= np.eye(n)
    assert np.abs(B).max() < 1e-12
    assert L.gpu_status() == 0


def test_reconstruction_argument_checks(gpu_lib):
    import torch

    L = gpu_lib
    d = torch.zeros(256, dtype=torch.float64, device="cuda")
    # lila_dorgh2_3: n > m, lda < m, ldt < n, ldq < m, S missing
    assert L.dorgh2_3(10, 12, d, 10, d, 12, d, 10, d, 64, d) == -2
    assert L.dorgh2_3(10, 4, d, 9, d, 4, d, 10, d, 64, d) == -4
    assert L.dorgh2_3(10, 4, d, 10, d, 3, d, 10, d, 64, d) == -6
    assert L.dorgh2_3(10, 4, d, 10, d, 4, d, 9, d, 64, d) == -8
    assert L.dorgh2_3(10, 4, d, 10, d, 4, d, 10, d, 64, None) == -11
    # lila_ormhr2_w03_hr: j < i, a tile that crosses its mt boundary, ldt < mt, lwork, S missing
    assert L.ormhr2_w03_hr(40, 4, 8, 4, -1, 8, d, 40, d, 8, d, 40, d, 256, d) == -4
    assert L.ormhr2_w03_hr(40, 6, 0, 4, -1, 8, d, 40, d, 8, d, 40, d, 256, d) == -6
    assert L.ormhr2_w03_hr(40, 4, 0, 4, -1, 8, d, 40, d, 7, d, 40, d, 256, d) == -10
    assert L.ormhr2_w03_hr(40, 4, 0, 4, -1, 8, d, 40, d, 8, d, 40, d, 0, d) == -14
    assert L.ormhr2_w03_hr(40, 4, 0, 4, -1, 8, d, 40, d, 8, d, 40, d, 256, None) == -15
    # lila_dorgh2 has no `l`: the codes after it shift by one
    assert L.dorgh2(40, 4, 8, 4, 8, d, 40, d, 8, d, 40, d, 256, d) == -4
    assert L.dorgh2(40, 6, 0, 4, 8, d, 40, d, 8, d, 40, d, 256, d) == -5
    assert L.dorgh2(40, 4, 0, 4, 8, d, 40, d, 7, d, 40, d, 256, d) == -9
    assert L.dorgh2(40, 4, 0, 4, 8, d, 40, d, 8, d, 40, d, 256, None) == -14
    torch.cuda.synchronize()
    assert L.gpu_status() == 0
