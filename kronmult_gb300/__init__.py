"""kronmult_gb300 -- batched Kronecker mat-vec on GB300 (sm_103a).

    Y(:,k) += kron(A1(:,:,k), ..., Ad(:,:,k)) * X(:,k),   d = 1..6

Python host side of the C ABI in ``include/kronmult_gb300.h``.  Arrays are
torch CUDA tensors (or raw device addresses); pointer arrays are int64 CUDA
tensors holding device addresses, as the reference's pointer-array entry
points expect device-resident ``T*[]`` arrays.

The per-dimension names of the reference (``kronmult6_xbatched`` ...) are
provided with the reference's argument order (kronmult6_xbatched.cpp:5-13 and
siblings); ``kronmult_batched`` etc. take d explicitly.  Every call launches
asynchronously on the current torch stream (or ``stream=``) and raises
``KmxError`` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C

from ._lib import KmxError, check, exported_symbols, lib, options  # noqa: F401

__all__ = [
    "KmxError", "lib", "options", "kron_flops", "pointer_array", "check_device_status",
    "kronmult_batched", "kronmult_pbatched", "kronmult_xbatched", "kronmult_vbatched",
    "set_default_form", "kronmult_mixed", "kronmult_vmixed", "kronmult_xbatched_wide",
]


def _torch():
    import torch

    return torch


def _addr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    t = _torch()
    if not isinstance(x, t.Tensor):
        raise TypeError(f"expected a CUDA tensor or an address, got {type(x)}")
    if not x.is_cuda:
        raise ValueError("arrays must be CUDA tensors (device memory)")
    return x.data_ptr()


def _stream(stream) -> int:
    if stream is None:
        return _torch().cuda.current_stream().cuda_stream
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def _is_f64(dtype) -> bool:
    t = _torch()
    if dtype in (t.float64, "f64", "float64"):
        return True
    if dtype in (t.float32, "f32", "float32"):
        return False
    raise TypeError(f"unsupported dtype {dtype}")


def pointer_array(base, offsets, itemsize: int | None = None):
    """int64 CUDA tensor of device addresses ``base + offsets * itemsize``."""
    t = _torch()
    offs = t.as_tensor(offsets, dtype=t.int64, device=base.device)
    isz = base.element_size() if itemsize is None else itemsize
    return offs * isz + base.data_ptr()


def kron_flops(d, m, n=None) -> float:
    """Flops of one entry (kroncommon.hpp:204-234)."""
    if isinstance(m, int):
        m = [m] * d
    n = m if n is None else ([n] * d if isinstance(n, int) else n)
    mm = (C.c_int * d)(*m)
    nn = (C.c_int * d)(*n)
    return float(lib().kmx_kron_flops(d, mm, nn))


def set_default_form(form: str = "auto", accumulate: str = "atomic") -> None:
    """Process-wide defaults of the drop-in entry points."""
    o = options(form, accumulate)
    lib().kmx_set_default_options(C.byref(o))


def check_device_status(stream=None) -> int:
    """Read and clear the device status word; raises KmxError if set."""
    flags = C.c_int(0)
    rc = lib().kmx_check_device_status(C.c_void_p(_stream(stream)), C.byref(flags))
    check(rc, "kmx_check_device_status")
    return flags.value


def read_redo_counters(stream=None) -> tuple[int, int]:
    """Read and clear the device's diagnostic counters: (entries the
    cancellation guard recomputed in FP64, digits-form entries handed to the
    double-float pass)."""
    c = (C.c_ulonglong * 2)()
    rc = lib().kmx_read_redo_counters(C.c_void_p(_stream(stream)), c)
    check(rc, "kmx_read_redo_counters")
    return int(c[0]), int(c[1])


def _opt(form, accumulate, transpose, engine=None, workspace=None, launch=None):
    if form is None and accumulate is None and not transpose and engine is None and not launch:
        return None
    o = options(form or "auto", accumulate or "atomic", transpose, engine or "tuned", launch)
    return C.byref(o)


def kronmult_batched(d, n, A, X, Y, W=None, batchCount=None, *, form=None, accumulate=None,
                     transpose=False, engine=None, launch=None, stream=None):
    """kronmult{d}_batched: A (n,n,d,batch) column-major, X/Y/W (n^d, batch).
    launch: (group_threads, groups_per_cta, ctas_per_sm) overrides, 0 = tuned."""
    f64 = _is_f64(A.dtype)
    b = batchCount if batchCount is not None else X.numel() // (n ** d)
    s = C.c_void_p(_stream(stream))
    L = lib()
    if f64:
        rc = L.kmx_kronmult_batched_f64_ex(d, n, _addr(A), _addr(X), _addr(Y), _addr(W), b,
                                           _opt(form, accumulate, transpose, engine,
                                                launch=launch), s)
    else:
        if form not in (None, "auto", "plain", "split", "tf32x3"):
            raise KmxError(4, "kmx_kronmult_batched_f32")
        rc = L.kmx_kronmult_batched_f32_ex(d, n, _addr(A), _addr(X), _addr(Y), _addr(W), b,
                                           _opt(form, accumulate, transpose, engine,
                                                launch=launch), s)
    check(rc, f"kronmult{d}_batched")


def kronmult_pbatched(d, n, A, pX, pY, pW=None, batchCount=None, *, form=None, accumulate=None,
                      transpose=False, engine=None, stream=None):
    """kronmult{d}_pbatched: A (n,n,d,batch); pX/pY/pW int64 address tensors."""
    f64 = _is_f64(A.dtype)
    b = batchCount if batchCount is not None else pX.numel()
    s = C.c_void_p(_stream(stream))
    L = lib()
    if f64:
        rc = L.kmx_kronmult_pbatched_f64_ex(d, n, _addr(A), _addr(pX), _addr(pY), _addr(pW), b,
                                            _opt(form, accumulate, transpose, engine), s)
    else:
        rc = L.kmx_kronmult_pbatched_f32_ex(d, n, _addr(A), _addr(pX), _addr(pY), _addr(pW), b,
                                            _opt(form, accumulate, transpose, engine), s)
    check(rc, f"kronmult{d}_pbatched")


def kronmult_xbatched(d, n, Aarray, lda, pX, pY, pW=None, batchCount=None, subbatchCount=0, *,
                      dtype=None, form=None, accumulate=None, transpose=False, engine=None,
                      launch=None, stream=None):
    """kronmult{d}_xbatched: Aarray (d, batch) factor addresses with leading
    dimension lda; pX/pY/pW address arrays.  dtype is float64 unless given."""
    t = _torch()
    f64 = _is_f64(dtype if dtype is not None else t.float64)
    b = batchCount if batchCount is not None else pX.numel()
    s = C.c_void_p(_stream(stream))
    L = lib()
    if f64:
        rc = L.kmx_kronmult_xbatched_f64_ex(d, n, _addr(Aarray), lda, _addr(pX), _addr(pY),
                                            _addr(pW), b, subbatchCount,
                                            _opt(form, accumulate, transpose, engine,
                                                 launch=launch), s)
    else:
        rc = L.kmx_kronmult_xbatched_f32_ex(d, n, _addr(Aarray), lda, _addr(pX), _addr(pY),
                                            _addr(pW), b, subbatchCount,
                                            _opt(form, accumulate, transpose, engine,
                                                 launch=launch), s)
    check(rc, f"kronmult{d}_xbatched")


def xbatched_build(d, Apool, a_level_stride, a_pool_stride, n_pool, Xpool, x_stride, n_x, Ypool,
                   y_stride, n_y, y_idx, x_idx, a_idx, *, sort_by_y=False, workspace=None,
                   stream=None):
    """Device-side construction of the xbatched arrays from index triples.

    Apool/Xpool/Ypool are CUDA tensors (float64 or float32); strides are in
    elements; y_idx, x_idx (count,) and a_idx (count, d) are int32 CUDA
    tensors.  Returns (Aarray, pX, pY) as int64 CUDA tensors of addresses
    (d*count, count, count), entries ordered by y when sort_by_y."""
    t = _torch()
    count = int(y_idx.numel())
    f64 = _is_f64(Xpool.dtype)
    dev = Xpool.device
    pA = t.empty(d * count, dtype=t.int64, device=dev)
    pX = t.empty(count, dtype=t.int64, device=dev)
    pY = t.empty(count, dtype=t.int64, device=dev)
    ws_bytes = 0
    if sort_by_y and workspace is None:
        ws_bytes = int(lib().kmx_xbatched_build_workspace_bytes(count))
        workspace = t.empty(ws_bytes, dtype=t.uint8, device=dev)
    elif workspace is not None:
        ws_bytes = workspace.numel() * workspace.element_size()
    fn = lib().kmx_xbatched_build_f64 if f64 else lib().kmx_xbatched_build_f32
    rc = fn(d, _addr(Apool), int(a_level_stride), int(a_pool_stride), int(n_pool), _addr(Xpool),
            int(x_stride), int(n_x), _addr(Ypool), int(y_stride), int(n_y), _addr(y_idx),
            _addr(x_idx), _addr(a_idx), count, 1 if sort_by_y else 0, _addr(workspace), ws_bytes,
            _addr(pA), _addr(pX), _addr(pY), C.c_void_p(_stream(stream)))
    check(rc, "xbatched_build")
    return pA, pX, pY


def _kgemm(trans, mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray, beta, Carray, ldCarray,
           batchCount, dtype, stream):
    t = _torch()
    f64 = _is_f64(dtype if dtype is not None else t.float64)
    b = batchCount if batchCount is not None else Carray.numel()
    fn = getattr(lib(), f"kmx_kgemm_{trans}_batched_{'f64' if f64 else 'f32'}")
    rc = fn(mm, nn, kk, float(alpha), _addr(Aarray), _addr(ldAarray), _addr(Barray),
            _addr(ldBarray), float(beta), _addr(Carray), _addr(ldCarray), b,
            C.c_void_p(_stream(stream)))
    check(rc, f"kgemm_{trans}_batched")


def kgemm_nn_batched(mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray, beta, Carray, ldCarray,
                     batchCount=None, *, dtype=None, stream=None):
    """kgemm_nn_batched (kgemm_nn_batched.cpp:8-41): C_e = alpha*A_e*B_e + beta*C_e
    for every entry; pointer arrays (int64 device tensors of addresses) and
    int32 leading-dimension arrays live on the device."""
    _kgemm("nn", mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray, beta, Carray, ldCarray,
           batchCount, dtype, stream)


def kgemm_nt_batched(mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray, beta, Carray, ldCarray,
                     batchCount=None, *, dtype=None, stream=None):
    """kgemm_nt_batched (kgemm_nt_batched.cpp:8-41): C_e = alpha*A_e*B_e^T + beta*C_e."""
    _kgemm("nt", mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray, beta, Carray, ldCarray,
           batchCount, dtype, stream)


def kronmult_vbatched(d, m, n, Aarray, pX, pY, W=None, Wcapacity_bytes=None, batchCount=None, *,
                      dtype=None, form=None, accumulate=None, transpose=False, engine=None,
                      stream=None):
    """kronmult{d}_vbatched: factor l is m[l] x n[l] (ld = m[l]) for every entry."""
    t = _torch()
    f64 = _is_f64(dtype if dtype is not None else t.float64)
    b = batchCount if batchCount is not None else pX.numel()
    mm = (C.c_int * d)(*[int(v) for v in m])
    nn = (C.c_int * d)(*[int(v) for v in n])
    cap = Wcapacity_bytes if Wcapacity_bytes is not None else (
        W.numel() * W.element_size() if W is not None else 0)
    s = C.c_void_p(_stream(stream))
    L = lib()
    if f64:
        rc = L.kmx_kronmult_vbatched_f64_ex(d, mm, nn, _addr(Aarray), _addr(pX), _addr(pY),
                                            _addr(W), cap, b, _opt(form, accumulate, transpose, engine), s)
    else:
        rc = L.kmx_kronmult_vbatched_f32_ex(d, mm, nn, _addr(Aarray), _addr(pX), _addr(pY),
                                            _addr(W), cap, b, _opt(form, accumulate, transpose, engine), s)
    check(rc, f"kronmult{d}_vbatched")


def kronmult_xbatched_wide(d, n, Aarray, lda, pX, pY, batchCount=None, *, in_dtype="f32",
                           form=None, accumulate=None, engine=None, stream=None):
    """xbatched with FP32 ("f32") or bfloat16 ("bf16") X and factors, FP32
    arithmetic (form "tf32x3": tensor cores) and FP64 Y accumulation."""
    code = {"f32": 1, "bf16": 2}[in_dtype]
    b = batchCount if batchCount is not None else pX.numel()
    rc = lib().kmx_kronmult_xbatched_wide(code, d, n, _addr(Aarray), lda, _addr(pX), _addr(pY), b,
                                          _opt(form, accumulate, False, engine),
                                          C.c_void_p(_stream(stream)))
    check(rc, f"kronmult{d}_xbatched_wide")


def kronmult_mixed(dims, Aarray, a_off, pX, pY, classes, W=None, Wcapacity_bytes=None, *,
                   dtype=None, form=None, accumulate=None, transpose=False, engine=None,
                   stream=None):
    """Instances of mixed (d, n) in one call.  dims: int32 CUDA tensor (count, 2)
    of (d, n); Aarray: factor addresses, instance i's at a_off[i] .. a_off[i]+d-1
    (a_off int64 CUDA tensor); pX/pY: block addresses; classes: host list of
    (d, n) pairs covering every instance (processed in this order)."""
    t = _torch()
    f64 = _is_f64(dtype if dtype is not None else t.float64)
    count = int(dims.shape[0])
    flat = [int(v) for c in classes for v in c]
    cl = (C.c_int * len(flat))(*flat)
    cap = Wcapacity_bytes if Wcapacity_bytes is not None else (
        W.numel() * W.element_size() if W is not None else 0)
    s = C.c_void_p(_stream(stream))
    fn = lib().kmx_kronmult_mixed_f64 if f64 else lib().kmx_kronmult_mixed_f32
    rc = fn(count, _addr(dims), _addr(Aarray), _addr(a_off), _addr(pX), _addr(pY), _addr(W), cap,
            cl, len(classes), _opt(form if f64 else None, accumulate, transpose, engine), s)
    check(rc, "kmx_kronmult_mixed")


def kronmult_vmixed(cls, Aarray, a_off, pX, pY, classes, W=None, Wcapacity_bytes=None, *,
                    dtype=None, form=None, accumulate=None, transpose=False, engine=None,
                    stream=None):
    """Instances of mixed rectangular shapes in one call.  cls: int32 CUDA tensor
    of class ids; classes: host list of (m, n) pairs of per-mode sizes (factor l
    is m[l] x n[l], leading dimension m[l]); Aarray: factor addresses,
    instance i's at a_off[i] .. a_off[i]+d-1; pX/pY: block addresses."""
    t = _torch()
    f64 = _is_f64(dtype if dtype is not None else t.float64)
    count = int(cls.numel())
    flat = []
    for m, n in classes:
        d = len(m)
        if len(n) != d or not 1 <= d <= 6:
            raise KmxError(1, "kmx_kronmult_vmixed")
        flat += [d] + [int(v) for v in m] + [1] * (6 - d) + [int(v) for v in n] + [1] * (6 - d)
    cl = (C.c_int * max(1, len(flat)))(*flat)
    cap = Wcapacity_bytes if Wcapacity_bytes is not None else (
        W.numel() * W.element_size() if W is not None else 0)
    s = C.c_void_p(_stream(stream))
    fn = lib().kmx_kronmult_vmixed_f64 if f64 else lib().kmx_kronmult_vmixed_f32
    rc = fn(count, _addr(cls), _addr(Aarray), _addr(a_off), _addr(pX), _addr(pY), _addr(W), cap,
            cl, len(classes), _opt(form if f64 else None, accumulate, transpose, engine), s)
    check(rc, "kmx_kronmult_vmixed")


# Reference names, one per d, reference argument order.
def _make(d):
    def batched(n, Aarray_, Xarray_, Yarray_, Warray_, batchCount, **kw):
        kronmult_batched(d, n, Aarray_, Xarray_, Yarray_, Warray_, batchCount, **kw)

    def pbatched(n, Aarray_, pX_, pY_, pW_, batchCount, **kw):
        kronmult_pbatched(d, n, Aarray_, pX_, pY_, pW_, batchCount, **kw)

    def xbatched(n, Aarray_, lda, pX_, pY_, pW_, batchCount, subbatchCount=0, **kw):
        kronmult_xbatched(d, n, Aarray_, lda, pX_, pY_, pW_, batchCount, subbatchCount, **kw)

    def vbatched(*args, **kw):
        mn = args[: 2 * d]
        rest = args[2 * d:]
        m = list(mn[0::2])
        n = list(mn[1::2])
        Aarray_, pX_, pY_, W_, Wcap, batchCount = rest
        kronmult_vbatched(d, m, n, Aarray_, pX_, pY_, W_, Wcap, batchCount, **kw)

    return batched, pbatched, xbatched, vbatched


for _d in range(1, 7):
    _b, _p, _x, _v = _make(_d)
    for _kind, _fn in (("batched", _b), ("pbatched", _p), ("xbatched", _x), ("vbatched", _v)):
        _fn.__name__ = f"kronmult{_d}_{_kind}"
        globals()[_fn.__name__] = _fn
        __all__.append(_fn.__name__)
del _d, _b, _p, _x, _v, _kind, _fn
