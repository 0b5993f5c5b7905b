"""lila_gb300 -- GB300 (sm_103a) implementation of LILA's Householder-QR family.

Python mirror of the C ABI in include/lila.h: the same routine names as the
reference's lila-c/lila.h (without the ``lila_`` prefix where Python allows),
the same argument lists and meanings.  Matrix arguments are CUDA tensors of
dtype float64 holding column-major data (a ``(m, n)`` tensor created as
``torch.empty((n, m)).t()`` or via :func:`colmajor`), or an ``(tensor, offset)``
pair, or a raw device address (int).  ``lila_param`` / ``nb_lvl`` are host int
sequences.  Every call enqueues kernels on the current torch stream and returns
the C return code (0, or -k for an invalid argument k).

The shared library is built by :func:`build` (nvcc for sm_103a) into
lila_gb300/liblila_gpu.so; importing the package never falls back to any other
implementation -- a missing or unloadable library raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
SO_PATH = os.path.join(_HERE, "liblila_gpu.so")

_lib = None

_P = ctypes.c_void_p
_IP = ctypes.POINTER(ctypes.c_int)
_CT = {"i": ctypes.c_int, "p": _P, "I": _IP, "v": _P, "d": ctypes.c_double, "L": ctypes.c_longlong,
       "P": ctypes.POINTER(ctypes.c_void_p), "Q": ctypes.POINTER(ctypes.c_longlong), "f": ctypes.c_float}

# name -> argument kinds (i int, p device double*, I host int*)
SIGNATURES = {
    "dgeqr3": "iipipi",
    "lila_dormqrf_w03": "iiiiiipipipi",
    "lila_dormqrf_z03": "iiiiiipipipipi",
    "lila_dormqrbz_w03": "iiiiiipipipipi",
    "lila_dorgh2_3": "iipipipipip",
    "lila_dorgh2": "iiiiipipipipip",
    "lila_ormhr2_w03_hr": "iiiiiipipipipip",
    "lila_dlarft_connect_w03": "iiiiipipi",
    "lila_dlarft_w03": "iiiipipip",
    "lila_dgeqrf_w03_levelx": "IiiIiiiipipipipi",
    "lila_dgeqrf_w03_recursive": "Iiiiipipipipi",
    "lila_dgeqr2_w03": "Iiiiipipipipi",
    "lila_dgeqrf_w03_mt": "Iiiiipipipipi",
    "lila_dgeqrf_w03_mt_hh": "Iiiiipipipipi",
    "lila_dgeqrf_w03_mt_l": "iiiipipipipi",
    "lila_dgeqrf_w03_mt_hr": "iiiipipipipi",
    "lila_dgeqr2_w03_l": "iiiipipipipi",
    "lila_dgeqr2_w03_3": "iiiipipipipi",
    "lila_dgeqr2_w03_hr": "iiiipipipipi",
    "lila_query_dgeqrf_w03_levelx": "IiiIiiiipipipipi",
    "lila_query_dgeqrf_w03_recursive": "Iiiiipipipipi",
    "lila_query_dgeqrf_w03_mt": "Iiiiipipipipi",
    "lila_query_dgeqrf_w03_mt_hh": "Iiiiipipipipi",
    "lila_query_dormqrbz_w03": "iiiiiipipipipi",
    "lila_query_dgeqrf_w03_mt_hr": "iiiipipipipi",
    "lila_query_dgeqrf_w03_mt_l": "iiiipipipipi",
    "lila_query_dgeqr2_w03_hr": "iiiipipipipi",
    "lila_query_dgeqr2_w03_3": "iiiipipipipi",
    "lila_query_dgeqr2_w03_l": "iiiipipipipi",
    "lila_query_ormhr2_w03_hr": "iiiiiipipipipip",
    "lila_query_dorgh2_3": "iipipipipip",
    "lila_query_dormqrf_w03": "iiiiiipipipi",
    "lila_dT2tau_w03": "iiiipip",
    "lila_dV2tau_w03": "iiiipip",
    "lila_dgeqrf_w03_appendcols": "Iiiiipipipipi",
    "lila_gpu_dgeqrf_tall_host": "iiipipipiipL",
    "lila_dgeqrf_v03_levelx": "IiiIiiiipipipi",
    "lila_dgeqrf_v03_recursive": "Iiiiipipipi",
    "lila_dgeqrf_v03_mt": "Iiiiipipipi",
    "lila_dgeqr2_v03": "Iiiiipipipi",
    "lila_dgeqrf_v03_mt_hh": "Iiiiipipipi",
    "lila_dgeqrf_v03_mt_l": "iiiipipipi",
    "lila_dgeqr2_v03_l": "iiiipipipi",
    "lila_dgeqr2_v03_3": "iiiipipipi",
    "lila_dgeqrf_q03_levelx": "IiiIiiiipipipipi",
    "lila_dgeqrf_q03_recursive": "Iiiiipipipipi",
    "lila_dgeqrf_q03_mt_hh": "Iiiiipipipipi",
    "lila_dgeqrf_q03_mt": "Iiiiipipipipi",
    "lila_dgeqrf_q03_mt_l": "iiiipipipipi",
    "lila_dgeqr2_q03": "Iiiiipipipipi",
    "lila_dgeqr2_q03_l": "iiiipipipipi",
    "lila_dgeqr2_q03_3": "iiiipipipipi",
    "lila_gpu_set_stream": "v",
    "lila_gpu_sync": "",
    "lila_gpu_status": "",
    "lila_gpu_clear_status": "",
    "lila_gpu_version": "",
    "lila_gpu_last_variant": "",
    "lila_gpu_last_passes": "",
    "lila_gpu_last_fallback": "",
    "lila_gpu_set_check": "i",
    "lila_gpu_graph_mode": "i",
    "lila_gpu_set_precision": "i",
    "lila_gpu_graph_cache_clear": "",
    "lila_dormqrf_w03_noalloc": "iiiiiipipi",
    "lila_dgeqrf_w03_tsqr": "iiiiiipipipipi",
    "lila_query_dgeqrf_w03_tsqr": "iiiiii",
    "lila_gpu_tsqr_autotune": "iipipipipi",
    "lila_dgels_batched_prepare": "iIIiPIPIpL",
    "lila_dgels_batched_run": "iipp",
    "lila_gpu_graph_launch": "v",
    "lila_gpu_graph_destroy": "v",
    "lila_gpu_gels_autotune": "iippPPQPPQ",
    "lila_gpu_gels_config": "ii",
    "lila_dgeqrf_w03_mt_hr_mixed": "iiiipipipipi",
    "lila_dgeqrf_w03_mt_hr_mixed_v": "iiiiipipipipi",
    "lila_query_dgeqrf_w03_mt_hr_mixed": "iiiipipipipi",
    # learned variant selector (include/lila_gpu.h)
    "lila_sel_params": "",
    "lila_sel_init": "pi",
    "lila_sel_infer": "ipppp",
    "lila_sel_grad": "ippppppppL",
    "lila_sel_adam": "ppppif",
    "lila_sel_train": "ippppiifipLv",
    # device primitives (include/lila_prim.h)
    "lila_prim_gemm": "iiipiiipiiipiddiiipL",
    "lila_prim_gemm_splits": "iiiL",
    "lila_prim_ozgemm": "iiipiiipiiipiddiiipL",
    "lila_prim_ozgemm_splits": "iiiL",
    "lila_prim_trsm_right_upper": "iidpipip",
    "lila_prim_trsm_left_lower_unit": "iipipi",
    "lila_prim_trsm_right_lower_unit_trans": "iidpipi",
    "lila_prim_potrf_upper": "ipi",
    "lila_prim_lu_sign": "ipip",
    "lila_prim_larfg": "ipp",
    "lila_prim_rsqrt": "ipp",
    "lila_prim_factor_pass": "ipipipiidd",
    "lila_prim_tc_selftest": "pppii",
    "lila_prim_ozaki_gram": "iipipipL",
    "lila_prim_ozaki_map": "iipipiipi",
    "lila_prim_ozaki_gram_rows": "iipipipLi",
    "lila_prim_ozaki_map_path": "i",
    "lila_prim_panel_phantom": "iipipipi",
}


def build(force=False):
    """Compile the CUDA sources for sm_103a into lila_gb300/liblila_gpu.so."""
    from . import buildlib as _b

    return _b.build(force=force)


def lib():
    """The loaded C library (ctypes.CDLL); raises if it was never built."""
    global _lib
    if _lib is None:
        if not os.path.exists(SO_PATH):
            raise RuntimeError(
                "lila_gb300: %s is missing -- run lila_gb300.build() (nvcc, sm_103a) first" % SO_PATH)
        so = ctypes.CDLL(SO_PATH)
        for name, kinds in SIGNATURES.items():
            f = getattr(so, name)
            f.restype = ctypes.c_int
            f.argtypes = [_CT[k] for k in kinds]
        so.lila_gpu_get_stream.restype = ctypes.c_void_p
        so.lila_gpu_get_stream.argtypes = []
        so.lila_test_qq_orth_1.restype = ctypes.c_double
        so.lila_test_qq_orth_1.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int]
        so.lila_test_qr_repres_1.restype = ctypes.c_double
        so.lila_test_qr_repres_1.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int] * 3)
        so.lila_query_dgels_batched.restype = ctypes.c_longlong
        so.lila_query_dgels_batched.argtypes = [ctypes.c_int]
        so.lila_dgels_batched_graph.restype = ctypes.c_void_p
        so.lila_dgels_batched_graph.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        for nm in ("lila_sel_grad_work", "lila_sel_train_work"):
            getattr(so, nm).restype = ctypes.c_longlong
        so.lila_sel_grad_work.argtypes = [ctypes.c_int]
        so.lila_sel_train_work.argtypes = [ctypes.c_int, ctypes.c_int]
        so.lila_gels_mixed_create.restype = ctypes.c_void_p
        so.lila_gels_mixed_create.argtypes = [ctypes.c_int, _IP, _IP, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                              _IP, ctypes.POINTER(ctypes.c_void_p), _IP]
        so.lila_gels_mixed_run.restype = ctypes.c_int
        so.lila_gels_mixed_run.argtypes = [ctypes.c_void_p, _IP, ctypes.c_int, _IP, ctypes.POINTER(ctypes.c_double)]
        so.lila_gels_mixed_features.restype = ctypes.c_int
        so.lila_gels_mixed_features.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        so.lila_gels_mixed_solve.restype = ctypes.c_int
        so.lila_gels_mixed_solve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _IP,
                                             ctypes.POINTER(ctypes.c_double), _IP]
        so.lila_gels_mixed_destroy.restype = ctypes.c_int
        so.lila_gels_mixed_destroy.argtypes = [ctypes.c_void_p]
        so.lila_gels_mixed_shifted.restype = ctypes.c_int
        so.lila_gels_mixed_shifted.argtypes = [ctypes.c_void_p, _IP]
        so.lila_gpu_query_dgeqrf_tall_host.restype = ctypes.c_longlong
        so.lila_gpu_query_dgeqrf_tall_host.argtypes = [ctypes.c_int] * 3
        so.lila_gpu_recursive_autotune.restype = ctypes.c_int
        so.lila_gpu_recursive_autotune.argtypes = ([_IP, ctypes.c_int, ctypes.c_int] + [_P, ctypes.c_int, _P] +
                                                   [_P, ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_int, _IP])
        so.lila_gels_mixed_set_trial_limit.restype = ctypes.c_int
        so.lila_gels_mixed_set_trial_limit.argtypes = [ctypes.c_void_p, ctypes.c_double]
        so.lila_prim_ozaki_gram_work.restype = ctypes.c_longlong
        so.lila_prim_ozaki_gram_work.argtypes = []
        so.lila_gpu_graph_replays.restype = ctypes.c_ulonglong
        so.lila_gpu_graph_replays.argtypes = []
        so.lila_gpu_launch_count.restype = ctypes.c_ulonglong
        so.lila_gpu_launch_count.argtypes = []
        so.lila_gpu_trace.restype = ctypes.c_int
        so.lila_gpu_trace.argtypes = [ctypes.c_int]
        so.lila_gpu_trace_summary.restype = ctypes.c_int
        so.lila_gpu_trace_summary.argtypes = [ctypes.c_char_p, ctypes.c_int]
        so.lila_prim_panel_work.restype = ctypes.c_longlong
        so.lila_prim_panel_work.argtypes = [ctypes.c_int]
        so.lila_gpu_set_wait_limit.restype = ctypes.c_longlong
        so.lila_gpu_set_wait_limit.argtypes = [ctypes.c_longlong]
        so.lila_prim_fp64_probe.restype = ctypes.c_double
        so.lila_prim_fp64_probe.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        so.lila_gpu_last_check.restype = ctypes.c_int
        so.lila_gpu_last_check.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        _lib = so
    return _lib


def dptr(x):
    """Device address of a tensor (or (tensor, element_offset)), or an int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    off = 0
    if isinstance(x, tuple):
        x, off = x
    return x.data_ptr() + int(off) * x.element_size()


def _host_ints(v):
    if v is None:
        return None
    arr = (ctypes.c_int * len(v))(*[int(t) for t in v])
    return arr


def _use_torch_stream():
    try:
        import torch

        if torch.cuda.is_available():
            lib().lila_gpu_set_stream(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    except ImportError:
        pass


def call(name, *args):
    """Call a C entry point with Python arguments converted per SIGNATURES."""
    kinds = SIGNATURES[name]
    assert len(args) == len(kinds), "%s takes %d arguments" % (name, len(kinds))
    conv = []
    keep = []
    for a, k in zip(args, kinds):
        if k in "iL":
            conv.append(int(a))
        elif k in "df":
            conv.append(float(a))
        elif k == "p":
            conv.append(ctypes.c_void_p(dptr(a)) if a is not None else None)
        elif k == "I":
            arr = _host_ints(a)
            keep.append(arr)
            conv.append(ctypes.cast(arr, _IP) if arr is not None else None)
        elif k == "P":
            arr = (ctypes.c_void_p * len(a))(*[dptr(x) for x in a])
            keep.append(arr)
            conv.append(ctypes.cast(arr, ctypes.POINTER(ctypes.c_void_p)))
        elif k == "Q":
            arr = (ctypes.c_longlong * len(a))(*[int(x) for x in a])
            keep.append(arr)
            conv.append(ctypes.cast(arr, ctypes.POINTER(ctypes.c_longlong)))
        elif k == "v":
            conv.append(ctypes.c_void_p(a) if a is not None else None)
        else:
            conv.append(a)
    if not name.startswith(("lila_query", "lila_gpu_s", "lila_gpu_l", "lila_gpu_v", "lila_gpu_c",
                            "lila_prim_gemm_splits", "lila_prim_ozgemm_splits")):
        _use_torch_stream()
    return getattr(lib(), name)(*conv)


def _mk(name):
    def f(*args):
        return call(name, *args)

    f.__name__ = name
    f.__doc__ = "C entry point %s (include/lila.h)" % name
    return f


for _n in SIGNATURES:
    globals()[_n[5:] if _n.startswith("lila_") else _n] = _mk(_n)
del _n


def launch_count():
    """Kernels launched by the library so far in this process."""
    return int(lib().lila_gpu_launch_count())


def trace(on):
    """Turn per-launch CUDA-event timing on or off (clears collected records)."""
    return lib().lila_gpu_trace(1 if on else 0)


def trace_summary():
    """{kernel name: (launches, total_ms)} of the traced launches."""
    buf = ctypes.create_string_buffer(1 << 16)
    lib().lila_gpu_trace_summary(buf, len(buf))
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        out[name] = (int(cnt), float(ms))
    return out


def gpu_last_check():
    """(res, orth) of the last checked split-precision leaf (lila_gpu_last_check);
    (-1, -1) when it was not checked."""
    r = ctypes.c_double(-1.0)
    o = ctypes.c_double(-1.0)
    lib().lila_gpu_last_check(ctypes.byref(r), ctypes.byref(o))
    return r.value, o.value


def sel_grad_work(count):
    """Floats of work lila_sel_grad needs for `count` samples."""
    return int(lib().lila_sel_grad_work(count))


def sel_train_work(n, batch):
    """Floats of work lila_sel_train needs."""
    return int(lib().lila_sel_train_work(n, batch))


def recursive_autotune(lila_param, m, n, A, lda, Ascratch, T, ldt, Q, ldq, work, lwork):
    """lila_gpu_recursive_autotune: returns (rc, mt, nx); rc is the best time
    in microseconds or a negative error."""
    _use_torch_stream()
    lp = (ctypes.c_int * 4)(*[int(v) for v in lila_param])
    mt = ctypes.c_int(0)
    rc = lib().lila_gpu_recursive_autotune(lp, int(m), int(n), dptr(A), int(lda), dptr(Ascratch), dptr(T), int(ldt),
                                           dptr(Q), int(ldq), dptr(work), int(lwork), ctypes.byref(mt))
    return rc, mt.value, lp[3]


GELS_NO_FALLBACK = 1
GELS_NO_TRIAL = 2


class GelsMixed:
    """Batched least squares with per-instance variants (lila_gels_mixed_*).

    ``A`` and ``B`` are lists of column-major float64 CUDA tensors (or device
    addresses); ``m``, ``n``, ``lda``, ``ldb`` host int sequences.  ``run``
    takes a route per instance (0 Cholesky QR 2, whose trial Cholesky may
    choose the shift, 1 shifted Cholesky QR 3, 2 FP64 Householder) and
    returns ``(failed_checks, info, orth)``.
    """

    def __init__(self, m, n, nrhs, A, lda, B, ldb):
        self.count = len(m)
        self._keep = [_host_ints(m), _host_ints(n), _host_ints(lda), _host_ints(ldb),
                      (ctypes.c_void_p * self.count)(*[dptr(x) for x in A]),
                      (ctypes.c_void_p * self.count)(*[dptr(x) for x in B])]
        k = self._keep
        self.h = lib().lila_gels_mixed_create(self.count, k[0], k[1], int(nrhs), k[4], k[2], k[5], k[3])
        if not self.h:
            raise RuntimeError("lila_gels_mixed_create failed")

    def run(self, route, flags=0):
        _use_torch_stream()
        r = _host_ints(route)
        info = (ctypes.c_int * self.count)()
        orth = (ctypes.c_double * self.count)()
        rc = lib().lila_gels_mixed_run(self.h, r, int(flags), info, orth)
        return rc, list(info), list(orth)

    def solve(self, params, flags=0):
        """Features -> selector (params: float32 CUDA tensor) -> routed run;
        returns (failed_checks, info, orth, route)."""
        _use_torch_stream()
        info = (ctypes.c_int * self.count)()
        orth = (ctypes.c_double * self.count)()
        route = (ctypes.c_int * self.count)()
        rc = lib().lila_gels_mixed_solve(self.h, ctypes.c_void_p(dptr(params)), int(flags), info, orth, route)
        return rc, list(info), list(orth), list(route)

    def set_trial_limit(self, limit):
        """Condition limit of variant 0's trial factor (default 1e8)."""
        if lib().lila_gels_mixed_set_trial_limit(self.h, float(limit)) != 0:
            raise ValueError("trial limit must be positive")

    def shifted(self):
        """Per instance 1 where the last run's trial factor chose the shift."""
        out = (ctypes.c_int * self.count)()
        lib().lila_gels_mixed_shifted(self.h, out)
        return list(out)

    def features(self, F):
        """Selector inputs into F (a count x 5 float32 CUDA tensor)."""
        _use_torch_stream()
        return lib().lila_gels_mixed_features(self.h, ctypes.c_void_p(dptr(F)))

    def close(self):
        if self.h:
            lib().lila_gels_mixed_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def test_qq_orth_1(m, n, i, Q, ldq):
    """||I - Q^T Q||_F over Q(i:m, i:i+n), computed on the device."""
    _use_torch_stream()
    return lib().lila_test_qq_orth_1(m, n, i, dptr(Q), ldq)


def test_qr_repres_1(m, n, i, A, lda, Q, ldq, R, ldr):
    """||A - Q R||_F / ||A||_F over the block at (i, i), computed on the device."""
    _use_torch_stream()
    return lib().lila_test_qr_repres_1(m, n, i, dptr(A), lda, dptr(Q), ldq, dptr(R), ldr)


def colmajor(rows, cols, device="cuda", dtype=None, fill=None):
    """A column-major (Fortran-ordered) rows x cols float64 tensor on `device`."""
    import torch

    dtype = dtype or torch.float64
    t = torch.empty((cols, rows), dtype=dtype, device=device).t()
    if fill is not None:
        t.fill_(fill)
    return t


def to_device_colmajor(a_np, device="cuda"):
    """Copy a numpy (Fortran-ordered) matrix to a column-major CUDA tensor."""
    import numpy as np
    import torch

    a = np.asfortranarray(a_np, dtype=np.float64)
    return torch.from_numpy(a.T.copy()).to(device).t()


def from_device(t):
    """Column-major CUDA tensor -> numpy Fortran array."""
    import numpy as np

    return np.asfortranarray(t.t().contiguous().cpu().numpy().T)
