"""ctypes access to the CPU oracle and, where built, the compiled reference.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference leg of bench.py.  Matrices are numpy float64 arrays in
Fortran (column-major) order; pointer arguments accept an array, an
``(array, offset)`` pair (element offset into the flat column-major storage)
or None.

``load("oracle")``     -- the C restatement (oracle/liblila_oracle.so)
``load("oracle_ob")``  -- the same restatement on scipy's OpenBLAS (timing only)
``load("ref")``        -- the reference's own C compiled in oracle/_ref/ (only
                          where the reference checkout exists)
All three expose the same Python names (lila's names without the prefix).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_P = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)

# name -> (return kind, argument kinds); i = int, p = double*, I = int*
_SIGS = {
    "dgeqr3": ("i", "iipipi"),
    "dormqrf_w03": ("i", "iiiiiipipipi"),
    "dormqrf_z03": ("i", "iiiiiipipipipi"),
    "dormqrbz_w03": ("i", "iiiiiipipipipi"),
    "dlarft_w03": ("i", "iiiipipip"),
    "dlarft_connect_w03": ("i", "iiiiipipi"),
    "dT2tau_w03": ("i", "iiiipip"),
    "dV2tau_w03": ("i", "iiiipip"),
    "dorgh2_3": ("i", "iipipipipip"),
    "ormhr2_w03_hr": ("i", "iiiiiipipipipip"),
    "dgeqr2_w03": ("i", "Iiiiipipipipi"),
    "dgeqr2_w03_l": ("i", "iiiipipipipi"),
    "dgeqr2_w03_3": ("i", "iiiipipipipi"),
    "dgeqr2_w03_hr": ("i", "iiiipipipipi"),
    "dgeqrf_w03_mt": ("i", "Iiiiipipipipi"),
    "dgeqrf_w03_mt_hh": ("i", "Iiiiipipipipi"),
    "dgeqrf_w03_mt_l": ("i", "iiiipipipipi"),
    "dgeqrf_w03_mt_hr": ("i", "iiiipipipipi"),
    "dgeqrf_w03_recursive": ("i", "Iiiiipipipipi"),
    "dgeqrf_w03_levelx": ("i", "IiiIiiiipipipipi"),
    "dgeqrf_w03_appendcols": ("i", "Iiiiipipipipi"),
    "dgeqr2_v03": ("i", "Iiiiipipipi"),
    "dgeqr2_v03_l": ("i", "iiiipipipi"),
    "dgeqr2_v03_3": ("i", "iiiipipipi"),
    "dgeqrf_v03_mt": ("i", "Iiiiipipipi"),
    "dgeqrf_v03_mt_hh": ("i", "Iiiiipipipi"),
    "dgeqrf_v03_mt_l": ("i", "iiiipipipi"),
    "dgeqrf_v03_recursive": ("i", "Iiiiipipipi"),
    "dgeqrf_v03_levelx": ("i", "IiiIiiiipipipi"),
    "dgeqr2_q03": ("i", "Iiiiipipipipi"),
    "dgeqr2_q03_l": ("i", "iiiipipipipi"),
    "dgeqr2_q03_3": ("i", "iiiipipipipi"),
    "dgeqrf_q03_mt": ("i", "Iiiiipipipipi"),
    "dgeqrf_q03_mt_hh": ("i", "Iiiiipipipipi"),
    "dgeqrf_q03_mt_l": ("i", "iiiipipipipi"),
    "dgeqrf_q03_recursive": ("i", "Iiiiipipipipi"),
    "dgeqrf_q03_levelx": ("i", "IiiIiiiipipipipi"),
}
# oracle-only helpers
_ORACLE_SIGS = {
    "dorgh2": ("i", "iiiiipipipipip"),
    "ls_solve": ("i", "iiipipipip"),
    "test_qq_orth_1": ("d", "iiipi"),
    "test_qr_repres_1": ("d", "iiipipipi"),
    "query_dormqrf_w03": ("i", "iiiiii"),
    "query_dormqrbz_w03": ("i", "iiiiii"),
    "query_dgeqrf_w03_mt_hr": ("i", "iiii"),
    "query_dgeqrf_w03_mt_hh": ("i", "Iiiii"),
    "query_dgeqrf_w03_mt": ("i", "Iiiii"),
    "query_dgeqrf_w03_recursive": ("i", "Iiiii"),
    "query_dgeqrf_w03_levelx": ("i", "IiiIiiii"),
    "gemm_dd": ("i", "iiiipipipi"),
}
# reference-only: the reference's own query signatures (full lila.h argument lists)
_REF_SIGS = {
    "query_dormqrf_w03": ("i", "iiiiiipipipi"),
    "query_dormqrbz_w03": ("i", "iiiiiipipipipi"),
    "query_dgeqrf_w03_recursive": ("i", "Iiiiipipipipi"),
    "query_dgeqrf_w03_mt_hr": ("i", "iiiipipipipi"),
    "dgeqr3_R": ("i", "iipipipi"),
}

_CT = {"i": ctypes.c_int, "p": _P, "I": _IP, "d": ctypes.c_double}


def _ptr(x):
    if x is None:
        return None
    off = 0
    if isinstance(x, tuple):
        x, off = x
    if x.dtype == np.float64:
        assert x.flags.f_contiguous or x.ndim == 1, "matrices must be Fortran ordered"
        return ctypes.cast(x.ctypes.data + 8 * int(off), _P)
    if x.dtype == np.int32:
        return ctypes.cast(x.ctypes.data + 4 * int(off), _IP)
    raise TypeError("unsupported dtype %s" % x.dtype)


class _Lib:
    def __init__(self, path, prefix, sigs):
        self.path = path
        self._so = ctypes.CDLL(path)
        self._fns = {}
        for name, (ret, args) in sigs.items():
            try:
                f = getattr(self._so, prefix + name)
            except AttributeError:
                continue
            f.restype = _CT[ret]
            f.argtypes = [_CT[a] for a in args]
            self._fns[name] = (f, args)

    def has(self, name):
        return name in self._fns

    def __getattr__(self, name):
        fns = self.__dict__.get("_fns", {})
        if name not in fns:
            raise AttributeError(name)
        f, kinds = fns[name]

        def call(*args):
            assert len(args) == len(kinds), "%s takes %d arguments" % (name, len(kinds))
            conv = []
            for a, k in zip(args, kinds):
                if k == "i":
                    conv.append(int(a))
                elif k in "pI":
                    conv.append(_ptr(a))
                else:
                    conv.append(a)
            return f(*conv)

        return call


_cache = {}


def ensure_built(with_ref=True):
    import importlib.util

    spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build(with_ref=with_ref)


def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "liblila_ref.so"))


def load(kind="oracle"):
    if kind in _cache:
        return _cache[kind]
    if kind == "oracle":
        path = os.path.join(HERE, "liblila_oracle.so")
        if not os.path.exists(path):
            ensure_built(with_ref=False)
        lib = _Lib(path, "oracle_", dict(_SIGS, **_ORACLE_SIGS))
    elif kind == "oracle_ob":
        path = os.path.join(HERE, "liblila_oracle_ob.so")
        if not os.path.exists(path):
            ensure_built(with_ref=False)
        if not os.path.exists(path):
            return None
        lib = _Lib(path, "oracle_", dict(_SIGS, **_ORACLE_SIGS))
    elif kind == "ref":
        path = os.path.join(HERE, "_ref", "liblila_ref.so")
        if not os.path.exists(path):
            return None
        lib = _Lib(path, "lila_", dict(_SIGS, **_REF_SIGS))
        # dgeqr3 / dgeqr3_R are exported without the lila_ prefix
        for bare in ("dgeqr3", "dgeqr3_R"):
            f = getattr(lib._so, bare)
            ret, args = (_SIGS.get(bare) or _REF_SIGS[bare])
            f.restype = _CT[ret]
            f.argtypes = [_CT[a] for a in args]
            lib._fns[bare] = (f, args)
    else:
        raise ValueError(kind)
    _cache[kind] = lib
    return lib


def lila_param(leaf, panel, nx_or_nlvl, extra=()):
    """The reference's int lila_param[] (lila-c/main_w03.c:176-180)."""
    return np.array([0, leaf, panel, nx_or_nlvl] + list(extra), dtype=np.int32)
