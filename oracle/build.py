"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the C restatement (oracle/lila_oracle.c + oracle/oblas.c) into
  oracle/liblila_oracle.so     -- self-contained (own BLAS loops, OpenMP);
                                  the checker used by tests and smoke()
  oracle/liblila_oracle_ob.so  -- same restatement with BLAS-1/2/3 calls
                                  forwarded to scipy's bundled OpenBLAS; only
                                  used to time the CPU baseline at full size
and, when the reference checkout is present, oracle/_ref/liblila_ref.so
(see build_ref.py).  Plain gcc; portable flags only (builds on x86-64 and
aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_ref  # noqa: E402

SRCS = [os.path.join(HERE, "lila_oracle.c"), os.path.join(HERE, "oblas.c")]
SO_SELF = os.path.join(HERE, "liblila_oracle.so")
SO_OB = os.path.join(HERE, "liblila_oracle_ob.so")


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs + [os.path.join(HERE, "oblas.h")])


def build(force=False, with_ref=True):
    base = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c99", "-I" + HERE]
    if force or _stale(SO_SELF, SRCS):
        subprocess.check_call(base + SRCS + ["-lm", "-o", SO_SELF])
    ob = build_ref.find_openblas()
    if ob is not None and (force or _stale(SO_OB, SRCS)):
        subprocess.check_call(base + ["-DORACLE_EXTERNAL_BLAS"] + SRCS + [
            ob, "-Wl,-rpath," + os.path.dirname(ob), "-lm", "-o", SO_OB])
    if with_ref:
        build_ref.build(force=force)
    return SO_SELF


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("ok")
