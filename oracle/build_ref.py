"""Build recipe for oracle/_ref/: the reference's own C sources compiled as a CPU checker.

Test infrastructure only.  Compiles the w03 routine set of the reference
(lila-c/*.c, the object list of the `xmain_w03.exe` target in lila-c/Makefile,
plus lila_dT2tau_w03.c, lila_dV2tau_w03.c, lila_dgeqrf_w03_appendcols.c, the
v03 / q03 routines and least-squares/dgeqr3_R.c) with gcc -O2 against the shim headers in
oracle/ref_shim/, linking scipy's bundled OpenBLAS.  Nothing is copied: the
sources are read where they lie under the read-only reference checkout and
only the resulting shared object is written, into oracle/_ref/ (git-ignored).

The checkout is looked for at $LILA_REFERENCE_DIR, else at /root/reference
(where the development container mounts it); on machines without it this
module does nothing.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("LILA_REFERENCE_DIR", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
OUT_SO = os.path.join(OUT_DIR, "liblila_ref.so")

LILA_C_FILES = [
    "dgeqr3.c",
    "lila_dormqrf_w03.c", "lila_dormqrf_z03.c", "lila_dormqrf_z00.c", "lila_dormqrbz_w03.c",
    "lila_dlarft_w03.c", "lila_dlarft_connect_w03.c",
    "lila_dgeqrf_w03_recursive.c", "lila_dgeqrf_w03_levelx.c", "lila_dgeqrf_w03_mt.c",
    "lila_dgeqrf_w03_mt_hh.c", "lila_dgeqrf_w03_mt_l.c", "lila_dgeqrf_w03_mt_hr.c",
    "lila_dgeqr2_w03.c", "lila_dgeqr2_w03_l.c", "lila_dgeqr2_w03_3.c", "lila_dgeqr2_w03_hr.c",
    "lila_dorgh2_3.c", "lila_ormhr2_w03_hr.c",
    "lila_dT2tau_w03.c", "lila_dV2tau_w03.c", "lila_dgeqrf_w03_appendcols.c",
    "lila_main_test.c",
    "lila_query_dgeqr2_w03_3.c", "lila_query_dgeqr2_w03_hr.c", "lila_query_dgeqr2_w03_l.c",
    "lila_query_dgeqrf_w03_levelx.c", "lila_query_dgeqrf_w03_mt.c",
    "lila_query_dgeqrf_w03_mt_hh.c", "lila_query_dgeqrf_w03_mt_hr.c",
    "lila_query_dgeqrf_w03_mt_l.c", "lila_query_dgeqrf_w03_recursive.c",
    "lila_query_dorgh2_3.c", "lila_query_dormqrbz_w03.c", "lila_query_dormqrf_w03.c",
    "lila_query_ormhr2_w03_hr.c",
    "lila_dgeqrf_v03_recursive.c", "lila_dgeqrf_v03_levelx.c", "lila_dgeqrf_v03_mt.c",
    "lila_dgeqrf_v03_mt_hh.c", "lila_dgeqrf_v03_mt_l.c",
    "lila_dgeqr2_v03.c", "lila_dgeqr2_v03_l.c", "lila_dgeqr2_v03_3.c",
    "lila_dgeqrf_q03_recursive.c", "lila_dgeqrf_q03_levelx.c", "lila_dgeqrf_q03_mt.c",
    "lila_dgeqrf_q03_mt_hh.c", "lila_dgeqrf_q03_mt_l.c",
    "lila_dgeqr2_q03.c", "lila_dgeqr2_q03_l.c", "lila_dgeqr2_q03_3.c",
]
LS_FILES = ["dgeqr3_R.c"]


def find_openblas():
    """Return the path of scipy's bundled LP64 OpenBLAS, or None."""
    try:
        import scipy
    except ImportError:
        return None
    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = sorted(glob.glob(os.path.join(libdir, "libscipy_openblas-*.so")))
    return cands[0] if cands else None


def available():
    return os.path.isdir(os.path.join(REF_ROOT, "lila-c"))


def build(force=False):
    """Compile the reference into oracle/_ref/liblila_ref.so; returns its path or None."""
    if not available():
        return None
    ob = find_openblas()
    if ob is None:
        return None
    srcs = [os.path.join(REF_ROOT, "lila-c", f) for f in LILA_C_FILES]
    srcs += [os.path.join(REF_ROOT, "least-squares", f) for f in LS_FILES]
    stamp = OUT_SO + ".sources"
    listing = "\n".join(srcs)
    if not force and os.path.exists(OUT_SO) and os.path.exists(stamp):
        so_mtime = os.path.getmtime(OUT_SO)
        with open(stamp) as f:
            same_list = f.read() == listing
        if same_list and all(os.path.getmtime(s) <= so_mtime for s in srcs):
            return OUT_SO
    os.makedirs(OUT_DIR, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w", "-I" + shim,
           "-I" + os.path.join(REF_ROOT, "lila-c")] + srcs + [
           ob, "-Wl,-rpath," + os.path.dirname(ob), "-lm", "-o", OUT_SO]
    subprocess.check_call(cmd)
    with open(stamp, "w") as f:
        f.write(listing)
    return OUT_SO


if __name__ == "__main__":
    p = build(force="--force" in sys.argv)
    print(p if p else "reference not available; nothing built")
