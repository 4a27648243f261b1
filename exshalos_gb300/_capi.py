"""ctypes binding of libexh_gb300.so (declarations in include/exh_gb300.h).

The library is built in-tree by exshalos_gb300/build.py.  There is no CPU
fallback: if the shared library or a CUDA device is missing, the calls raise.
"""
import ctypes as C
import os
import sys
import threading

import numpy as np

EXH_OK = 0
EXH_E_INVALID = 1
EXH_E_NOMEM = 2
EXH_E_CUDA = 3
EXH_E_RANGE = 4
EXH_E_TIMEOUT = 5
EXH_E_UNSUPPORTED = 6
EXH_E_NO_DEVICE = 7
EXH_MEM_HOST = 0
EXH_MEM_DEVICE = 1
EXH_FIELD_PHILOX = 1
EXH_FIELD_TAUS = 2
FIELD_STREAMS = {"philox": EXH_FIELD_PHILOX, "taus": EXH_FIELD_TAUS}


def field_stream_code(name):
    """EXH_FIELD_* code of a field stream name ("philox", "taus") or code."""
    if isinstance(name, str):
        try:
            return FIELD_STREAMS[name.lower()]
        except KeyError:
            raise ValueError(f"unknown field stream {name!r}: 'philox' or 'taus'") from None
    if int(name) not in FIELD_STREAMS.values():
        raise ValueError(f"unknown field stream {name!r}")
    return int(name)

_lib = None
_lock = threading.Lock()
_tls = threading.local()


class HaloParams(C.Structure):
    _fields_ = [
        ("R_max", C.c_float), ("ndx", C.c_int), ("ndy", C.c_int), ("ndz", C.c_int),
        ("Lc", C.c_float), ("seed", C.c_int), ("k_smooth", C.c_float),
        ("Om0", C.c_float), ("redshift", C.c_float), ("dc", C.c_float),
        ("Nmin", C.c_int), ("a", C.c_float), ("beta", C.c_float), ("alpha", C.c_float),
        ("fixed", C.c_int), ("phase", C.c_float),
        ("OUT_DEN", C.c_int), ("OUT_LPT", C.c_int), ("OUT_VEL", C.c_int), ("DO_2LPT", C.c_int),
        ("OUT_FLAG", C.c_int), ("OUT_PROF", C.c_int), ("verbose", C.c_int), ("nthreads", C.c_int),
        ("field_stream", C.c_int), ("setup_fp64", C.c_int),
    ]


class BatchItem(C.Structure):
    _fields_ = [("nd", C.c_int), ("seed", C.c_int)]


class DiffParams(C.Structure):
    _fields_ = [("nd", C.c_int), ("L", C.c_float), ("Om0", C.c_float), ("redshift", C.c_float),
                ("do_2lpt", C.c_int), ("n_knots", C.c_int), ("Nk", C.c_int), ("k_min", C.c_float),
                ("k_max", C.c_float)]


class HodParams(C.Structure):
    _fields_ = [("Lc", C.c_float), ("Om0", C.c_float), ("redshift", C.c_float),
                ("ndx", C.c_int32), ("ndy", C.c_int32), ("ndz", C.c_int32),
                ("logMmin", C.c_float), ("siglogM", C.c_float), ("logM0", C.c_float), ("logM1", C.c_float),
                ("alpha", C.c_float), ("sigma", C.c_float), ("Deltah", C.c_float), ("seed", C.c_int32)]


# every symbol the header declares, with its argument and result types
_P = C.c_void_p
SIGNATURES = {
    "exh_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "exh_ctx_destroy": (C.c_int, [_P]),
    "exh_strerror": (C.c_char_p, [C.c_int]),
    "exh_last_error": (C.c_char_p, []),
    "exh_version": (C.c_int, []),
    "exh_check_precision": (C.c_int, []),
    "exh_grid_compute": (C.c_int, [_P, _P, C.c_int64, C.c_int, C.c_float, C.c_int, C.c_int, _P, C.c_int, _P]),
    "exh_power_compute": (C.c_int, [_P, _P, C.c_int, C.c_float, C.c_int, C.c_int, C.c_float, C.c_float,
                                    _P, _P, _P, C.c_int, _P]),
    "exh_halo_params_default": (None, [C.POINTER(HaloParams)]),
    "exh_halos_box_from_pk": (C.c_int, [_P, _P, _P, C.c_int, C.POINTER(HaloParams), C.POINTER(C.c_int64), _P]),
    "exh_find_halos": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P, _P, C.c_int, C.POINTER(HaloParams),
                                 C.c_int, C.POINTER(C.c_int64), _P]),
    "exh_halos_fetch": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_int, _P]),
    "exh_halo_tables": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), _P, _P, _P, _P]),
    "exh_density_grid_compute": (C.c_int, [_P, _P, _P, C.c_int, C.POINTER(HaloParams), _P, C.c_int, _P]),
    "exh_batch_run": (C.c_int, [_P, _P, _P, C.c_int, C.POINTER(HaloParams), _P, C.c_int, C.c_int, C.c_int, _P, _P,
                                _P, _P, _P]),
    "exh_diff_forward": (C.c_int, [_P, C.POINTER(DiffParams), _P, _P, _P, _P, _P, C.POINTER(C.c_double), _P, _P,
                                   _P, _P]),
    "exh_diff_backward": (C.c_int, [_P, C.c_double, _P, _P, _P]),
    "exh_halos_box_from_grid": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P, _P, C.c_int, _P, _P,
                                          C.POINTER(HaloParams), C.c_int, C.POINTER(C.c_int64), _P]),
    "exh_grid_compute_ex": (C.c_int, [_P, _P, _P, _P, _P, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                      C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, _P, C.c_int, _P]),
    "exh_power_compute_ex": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_float, C.c_int, C.c_float, C.c_int, C.c_int,
                                       C.c_float, C.c_float, C.c_int, C.c_int, _P, _P, _P, C.c_int, _P]),
    "exh_hod_populate": (C.c_int, [_P, _P, _P, _P, _P, C.c_int64, C.POINTER(HodParams), C.c_int,
                                   C.POINTER(C.c_int64), C.c_int, _P]),
    "exh_hod_fetch": (C.c_int, [_P, _P, _P, _P, C.c_int, _P]),
    "exh_hod_split": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int64, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P,
                                C.c_int, _P]),
    "exh_abundance_compute": (C.c_int, [_P, _P, C.c_int64, C.c_float, C.c_float, C.c_int, C.c_float, C.c_int, C.c_int,
                                        C.c_int, _P, _P, _P, C.c_int, _P]),
    "exh_smoothing_ladder": (C.c_int, [_P, _P, _P, C.c_int, C.POINTER(HaloParams), C.c_int, C.c_float, _P, _P, _P,
                                       C.c_int, _P]),
    "exh_fft_r2c_3d": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P]),
    "exh_fft_c2r_3d": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P]),
    "exh_launch_count": (C.c_int64, [_P]),
    "exh_power_compute_noalloc": (C.c_int, [_P, C.c_int, C.c_float, C.c_int, C.c_int, C.c_float, C.c_float, _P, _P,
                                            _P, _P]),
    "exh_timing_enable": (C.c_int, [C.c_int]),
    "exh_timing_report": (C.c_int, [C.c_int, _P, _P, _P]),
}

TIMING_CLASSES = ["fft_strided", "fft_rows", "peaks", "sort", "grow", "mass", "lpt_stencil", "halo_disp", "cic",
                  "pk_bin", "other"]


def timing_enable(on=True):
    load().exh_timing_enable(1 if on else 0)


def timing_report():
    """{class: (ms, launches, bytes)} since timing_enable(True)."""
    n = len(TIMING_CLASSES)
    ms = np.zeros(n)
    la = np.zeros(n, dtype=np.int64)
    by = np.zeros(n)
    load().exh_timing_report(n, ptr(ms), ptr(la), ptr(by))
    return {TIMING_CLASSES[i]: (float(ms[i]), int(la[i]), float(by[i])) for i in range(n)}


def lib_path():
    from . import build
    return build.lib_path()


def load(build_if_missing=True):
    """Load the shared library (building it when absent)."""
    global _lib
    with _lock:
        if _lib is None:
            path = lib_path()
            if not os.path.exists(path):
                if not build_if_missing:
                    raise RuntimeError(f"{path} is not built; run exshalos_gb300.build.build()")
                from . import build
                build.build()
            L = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class ExhError(RuntimeError):
    pass


class HaloRangeError(ExhError):
    """EXH_E_RANGE: a halo beyond the sigma table or a mass outside the
    mass-function splines (the reference's GSL spline aborts there,
    find_halos.c:472-474)."""


def check(status):
    if status == EXH_OK:
        return
    L = load()
    msg = f"{L.exh_strerror(status).decode()}: {L.exh_last_error().decode()}"
    if status == EXH_E_INVALID:
        raise ValueError(msg)
    if status == EXH_E_NOMEM:
        raise MemoryError(msg)
    if status == EXH_E_UNSUPPORTED:
        raise NotImplementedError(msg)
    if status == EXH_E_RANGE:
        raise HaloRangeError(msg)
    raise ExhError(msg)


def context():
    """Per-thread library context on the current device (device 0 by default)."""
    ctx = getattr(_tls, "ctx", None)
    if ctx is None:
        L = load()
        h = C.c_void_p()
        dev = int(os.environ.get("EXH_DEVICE", "0"))
        check(L.exh_ctx_create(dev, C.byref(h)))
        _tls.ctx = h
        ctx = h
    return ctx


_POOL_MIN_BYTES = 1 << 20
_POOL_MAX_BUFFERS = 16


def host_empty(shape, dtype):
    """An uninitialised host array for a large output that the library fills
    completely.  Arrays of 1 MB or more are views of byte buffers from a
    per-thread pool: a buffer at least as large as the request (and at most
    twice) is handed out again only once the pool holds the last reference to
    it (the caller has dropped every array viewing it), so a result never
    shares memory with a live array.  Outputs whose length changes from call
    to call (halo catalogues) reuse the same buffers; the pool saves the page
    faults and zero-fill of a fresh allocation on every call in a loop."""
    dt = np.dtype(dtype)
    shape = tuple(int(x) for x in (shape if isinstance(shape, (tuple, list)) else (shape,)))
    nbytes = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
    if nbytes < _POOL_MIN_BYTES:
        return np.empty(shape, dtype=dt)
    pool = getattr(_tls, "pool", None)
    if pool is None:
        pool = _tls.pool = []
    pick = -1
    for i in range(len(pool)):
        cap = pool[i].nbytes
        if nbytes <= cap <= 2 * nbytes and sys.getrefcount(pool[i]) <= 2:   # list entry + argument
            if pick < 0 or cap < pool[pick].nbytes:
                pick = i
    if pick < 0:
        pool.append(np.empty(nbytes + nbytes // 8, dtype=np.uint8))
        pick = len(pool) - 1
        if len(pool) > _POOL_MAX_BUFFERS:            # drop the oldest buffer nobody holds
            for i in range(len(pool) - 1):
                if sys.getrefcount(pool[i]) <= 2:
                    del pool[i]
                    pick -= 1
                    break
    return pool[pick][:nbytes].view(dt).reshape(shape)


def ptr(a):
    """Address of a numpy array or an object exposing data_ptr() (device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, int):
        return C.c_void_p(a)
    raise TypeError(f"cannot pass {type(a)} to the C ABI")


def default_params(**kw):
    p = HaloParams()
    load().exh_halo_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def launch_count():
    return int(load().exh_launch_count(None))
