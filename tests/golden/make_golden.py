"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own C code (compiled into oracle/_ref/ by
oracle/build_ref.py from the reference checkout, linked against scipy's
OpenBLAS) on seeded inputs and stores its outputs.  Inputs are not stored:
they are regenerated from the seed by tests/lila_cases.inputs (numpy PCG64).
Only runs where the reference checkout exists; the fixtures it writes are
committed so the checks also run where it does not.

    python tests/golden/make_golden.py [tag-prefix ...]

With prefixes, only the fixtures whose tag starts with one of them are
written (the others are left byte for byte as they are).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle as O  # noqa: E402
import lila_cases as C  # noqa: E402

# (tag, mode, m, n, ii, mt, lda, ldq, leaf, panel, nx_or_nb)
DRIVER_CASES = [
    ("rec_l1p1_87x53", "recursive", 87, 53, 6, 4, 87, 87, 1, 1, 7),
    ("rec_l0p0_pad", "recursive", 87, 53, 6, 4, 90, 95, 0, 0, 7),
    ("rec_l1p2_87x53", "recursive", 87, 53, 6, 4, 87, 87, 1, 2, 7),
    ("rec_l2_120x40", "recursive", 120, 40, 0, 32, 120, 120, 2, 0, 64),
    ("rec_l1p1_mt7", "recursive", 141, 69, 9, 7, 150, 145, 1, 1, 9),
    ("lvx_l1p1_20_5", "levelx", 87, 53, 6, 4, 87, 87, 1, 1, [20, 5]),
]
# the v03 driver (V, R, T) followed by the q03 driver (Q from them)
VQ_CASES = [
    ("vq_rec_l1p1_87x53", "recursive", 87, 53, 6, 4, 87, 87, 1, 1, 7),
    ("vq_rec_l0p0_pad", "recursive", 87, 53, 6, 4, 90, 95, 0, 0, 7),
    ("vq_rec_l1p0_mt7", "recursive", 141, 69, 9, 7, 150, 145, 1, 0, 9),
    ("vq_lvx_l1p1_16_8_4", "levelx", 87, 53, 6, 4, 87, 87, 1, 1, [16, 8, 4]),
]


def main(prefixes=()):
    O.ensure_built(with_ref=True)
    ref = O.load("ref")
    if ref is None:
        print("reference not available; fixtures left unchanged")
        return 1
    want = lambda tag: not prefixes or tag.startswith(tuple(prefixes))  # noqa: E731
    for tag, mode, m, n, ii, mt, lda, ldq, leaf, panel, nx in VQ_CASES:
        if not want(tag):
            continue
        nb = nx if mode == "levelx" else None
        A, T, Q = C.run_cpu_vq(ref, mode, m, n, ii, mt, leaf, panel, nx if mode == "recursive" else None,
                               lda, ldq, seed=0, nb=nb)
        np.savez_compressed(os.path.join(HERE, tag + ".npz"), A=A, T=T, Q=Q,
                            shape=np.array([m, n, ii, mt, lda, ldq, leaf, panel]),
                            nb=np.array(nb if nb else [nx], dtype=np.int32))
        print("wrote", tag)
    for tag, mode, m, n, ii, mt, lda, ldq, leaf, panel, nx in DRIVER_CASES:
        if not want(tag):
            continue
        nb = nx if mode == "levelx" else None
        A, T, Q = C.run_cpu(ref, mode, m, n, ii, mt, leaf, panel, nx if mode == "recursive" else None,
                            lda, ldq, seed=0, nb=nb)
        np.savez_compressed(os.path.join(HERE, tag + ".npz"), A=A, T=T, Q=Q,
                            shape=np.array([m, n, ii, mt, lda, ldq, leaf, panel]),
                            nb=np.array(nb if nb else [nx], dtype=np.int32))
        print("wrote", tag)
    if want("ormqr_z03_87x53"):
        write_ormqr(ref)
    if want("ls_60x20"):
        write_ls(ref)
    return 0


def write_ormqr(ref):
    # Q^T applied to a separate block B (lila_dormqrf_z03) after a recursive QR
    m, n, ii, mt, nrhs = 87, 53, 6, 4, 8
    A, T, Q = C.run_cpu(ref, "recursive", m, n, ii, mt, 1, 1, 7, seed=0)
    rng = np.random.default_rng(102)
    B = np.asfortranarray(rng.standard_normal((m, nrhs)))
    work = np.zeros(8 * m * (nrhs + mt))
    ref.dormqrf_z03(m, nrhs, n, ii, 0, mt, A, m, T, mt, B, m, work, work.size)
    np.savez_compressed(os.path.join(HERE, "ormqr_z03_87x53.npz"), B=B)
    print("wrote ormqr_z03_87x53")


def write_ls(ref):
    # least squares via dgeqr3_R + Q^T b + trsm (least-squares/main_ls_qr3.c:94-119)
    m, n, k = 60, 20, 4
    rng = np.random.default_rng(400)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, n)))
    b = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, k)))
    T = np.asfortranarray(np.zeros((n, n)))
    ref.dgeqr3_R(m, n, A, m, T, n, A, m)
    w = np.asfortranarray(np.zeros((n, k)))
    # the driver's Q^T b and solve, done with numpy on the reference's V, T, R
    V = np.tril(A, -1)[:, :n] + np.eye(m, n)
    Tu = np.triu(T)
    qtb = b - V @ (Tu.T @ (V.T @ b))
    x = np.linalg.solve(np.triu(A[:n, :n]), qtb[:n])
    np.savez_compressed(os.path.join(HERE, "ls_60x20.npz"), A=A, T=T, x=x)
    print("wrote ls_60x20")


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
