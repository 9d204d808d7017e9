"""ctypes binding of ``libkronmult_gb300.so`` (the C ABI in include/kronmult_gb300.h).

The library is loaded from this package directory.  There is no fallback: if
the shared library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkronmult_gb300.so")

_lock = threading.Lock()
_lib = None

KMX_OK = 0
STATUS = {
    0: "KMX_OK",
    1: "KMX_ERR_INVALID_ARG",
    2: "KMX_ERR_NULL_POINTER",
    3: "KMX_ERR_WORKSPACE",
    4: "KMX_ERR_UNSUPPORTED",
    5: "KMX_ERR_CUDA",
    6: "KMX_ERR_DEVICE",
    7: "KMX_ERR_OVERLAP",
}

FORMS = {"auto": 0, "plain": 1, "split": 2, "tf32x3": 3, "digits": 4, "split_raw": 5}
ENGINES = {"tuned": 0, "per_mode": 1, "tiled": 2, "small": 3, "persistent": 4, "cluster": 5,
           "lane": 6}
ACCUMULATE = {"atomic": 0, "deterministic": 1}


class KmxError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        name = STATUS.get(status, f"status {status}")
        extra = ""
        if status == 5 and _lib is not None:
            extra = f" (cuda error {int(_lib.kmx_last_cuda_error())})"
        super().__init__(f"{where}: {name}{extra}")


class Options(C.Structure):
    _fields_ = [("form", C.c_int), ("accumulate", C.c_int), ("transpose", C.c_int),
                ("engine", C.c_int), ("workspace", C.c_void_p), ("workspace_bytes", C.c_size_t),
                ("group_threads", C.c_int), ("groups_per_cta", C.c_int), ("ctas_per_sm", C.c_int)]


_vp = C.c_void_p
_i = C.c_int
_sz = C.c_size_t
_ip = C.POINTER(C.c_int)
_optp = C.POINTER(Options)

# name -> argtypes (all return int status)
_SIGS = {
    "kmx_kronmult_batched_f64": [_i, _i, _vp, _vp, _vp, _vp, _i, _vp],
    "kmx_kronmult_batched_f32": [_i, _i, _vp, _vp, _vp, _vp, _i, _vp],
    "kmx_kronmult_batched_f64_ex": [_i, _i, _vp, _vp, _vp, _vp, _i, _optp, _vp],
    "kmx_kronmult_pbatched_f64": [_i, _i, _vp, _vp, _vp, _vp, _i, _vp],
    "kmx_kronmult_pbatched_f32": [_i, _i, _vp, _vp, _vp, _vp, _i, _vp],
    "kmx_kronmult_pbatched_f64_ex": [_i, _i, _vp, _vp, _vp, _vp, _i, _optp, _vp],
    "kmx_kronmult_xbatched_f64": [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _i, _vp],
    "kmx_kronmult_xbatched_f32": [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _i, _vp],
    "kmx_kronmult_xbatched_f64_ex": [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _i, _optp, _vp],
    "kmx_kronmult_vbatched_f64": [_i, _ip, _ip, _vp, _vp, _vp, _vp, _sz, _i, _vp],
    "kmx_kronmult_vbatched_f32": [_i, _ip, _ip, _vp, _vp, _vp, _vp, _sz, _i, _vp],
    "kmx_kronmult_vbatched_f64_ex": [_i, _ip, _ip, _vp, _vp, _vp, _vp, _sz, _i, _optp, _vp],
    "kmx_kronmult_batched_f32_ex": [_i, _i, _vp, _vp, _vp, _vp, _i, _optp, _vp],
    "kmx_kronmult_pbatched_f32_ex": [_i, _i, _vp, _vp, _vp, _vp, _i, _optp, _vp],
    "kmx_kronmult_xbatched_f32_ex": [_i, _i, _vp, _i, _vp, _vp, _vp, _i, _i, _optp, _vp],
    "kmx_kronmult_vbatched_f32_ex": [_i, _ip, _ip, _vp, _vp, _vp, _vp, _sz, _i, _optp, _vp],
    "kmx_check_device_status": [_vp, _ip],
    "kmx_read_redo_counters": [_vp, C.POINTER(C.c_ulonglong)],
    "kmx_last_cuda_error": [],
    "kmx_probe_fma_rate": [_i, C.POINTER(C.c_double)],
    "kmx_release_workspace": [_vp],
    "kmx_kronmult_xbatched_f64_noalloc": [_i, _i, _vp, _i, _vp, _vp, _i, _vp],
    "kmx_kronmult_batched_grad_f64": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _i, _vp],
    "kmx_kronmult_batched_grad_f64_ex": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _i,
                                         _optp, _vp],
    "kmx_kronmult_batched_grad_f32": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _i, _vp],
    "kmx_kronmult_xbatched_wide": [_i, _i, _i, _vp, _i, _vp, _vp, _i, _optp, _vp],
    "kmx_kronmult_mixed_f64": [_i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _ip, _i, _optp, _vp],
    "kmx_xbatched_build_f64": [_i, _vp, C.c_longlong, C.c_longlong, _i, _vp, C.c_longlong, _i,
                               _vp, C.c_longlong, _i, _vp, _vp, _vp, _i, _i, _vp, _sz, _vp, _vp,
                               _vp, _vp],
    "kmx_xbatched_build_f32": [_i, _vp, C.c_longlong, C.c_longlong, _i, _vp, C.c_longlong, _i,
                               _vp, C.c_longlong, _i, _vp, _vp, _vp, _i, _i, _vp, _sz, _vp, _vp,
                               _vp, _vp],
    "kmx_kgemm_nn_batched_f64": [_i, _i, _i, C.c_double, _vp, _vp, _vp, _vp, C.c_double, _vp, _vp,
                                 _i, _vp],
    "kmx_kgemm_nt_batched_f64": [_i, _i, _i, C.c_double, _vp, _vp, _vp, _vp, C.c_double, _vp, _vp,
                                 _i, _vp],
    "kmx_kgemm_nn_batched_f32": [_i, _i, _i, C.c_float, _vp, _vp, _vp, _vp, C.c_float, _vp, _vp,
                                 _i, _vp],
    "kmx_kgemm_nt_batched_f32": [_i, _i, _i, C.c_float, _vp, _vp, _vp, _vp, C.c_float, _vp, _vp,
                                 _i, _vp],
    "kmx_kronmult_mixed_f32": [_i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _ip, _i, _optp, _vp],
    "kmx_kronmult_vmixed_f64": [_i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _ip, _i, _optp, _vp],
    "kmx_kronmult_vmixed_f32": [_i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _ip, _i, _optp, _vp],
    "kmx_set_default_options": [_optp],
    "kmx_get_default_options": [_optp],
}


def exported_symbols() -> list[str]:
    """Every function include/kronmult_gb300.h declares."""
    import re

    hdr = os.path.join(_HERE, "..", "include", "kronmult_gb300.h")
    with open(hdr) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(kmx_[a-z0-9_]+)\s*\(", text)))


def lib():
    """Load the CUDA library (raises if it is missing: there is no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'`")
            L = C.CDLL(LIB_PATH)
            for name, args in _SIGS.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = C.c_int
            L.kmx_kron_flops.argtypes = [_i, _ip, _ip]
            L.kmx_kron_flops.restype = C.c_double
            L.kmx_status_string.argtypes = [_i]
            L.kmx_status_string.restype = C.c_char_p
            L.kmx_grad_workspace_bytes.argtypes = [_i, _i, _i, _i]
            L.kmx_grad_workspace_bytes.restype = C.c_size_t
            L.kmx_deterministic_workspace_bytes.argtypes = [_i]
            L.kmx_xbatched_build_workspace_bytes.restype = _sz
            L.kmx_xbatched_build_workspace_bytes.argtypes = [_i]
            L.kmx_deterministic_workspace_bytes.restype = C.c_size_t
            L.kmx_cached_workspace_bytes.argtypes = []
            L.kmx_cached_workspace_bytes.restype = C.c_size_t
            L.kmx_version.argtypes = []
            L.kmx_version.restype = C.c_char_p
            _lib = L
        return _lib


def check(status: int, where: str) -> None:
    if status != KMX_OK:
        raise KmxError(status, where)


def options(form: str | int = "auto", accumulate: str | int = "atomic", transpose: bool = False,
            engine: str | int = "tuned", launch=None):
    """launch: (group_threads, groups_per_cta, ctas_per_sm), 0 = tuned/default."""
    f = FORMS[form] if isinstance(form, str) else int(form)
    a = ACCUMULATE[accumulate] if isinstance(accumulate, str) else int(accumulate)
    g = ENGINES[engine] if isinstance(engine, str) else int(engine)
    gt, ge, gs = (int(v) for v in launch) if launch else (0, 0, 0)
    return Options(f, a, 1 if transpose else 0, g, None, 0, gt, ge, gs)
