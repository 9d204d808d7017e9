"""numpy front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/libkron_oracle.so`` (the C restatement in ``kron_oracle.c``)
and, when it was built, ``oracle/_ref/libkron_ref.so`` (the reference's own
CPU/OpenMP templates compiled from its source tree).  Only the tests, the
smoke check and the benchmark's CPU-baseline leg import this module; the CUDA
product path never does.

Array conventions follow hipdac-lab/kronmult: factors are column-major with a
leading dimension, X/Y blocks are flat vectors whose LAST Kronecker index runs
fastest (test_kronmult6_batched.cpp:418-436).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "libkron_oracle.so")
_REF_SO = os.path.join(_HERE, "_ref", "libkron_ref.so")
_lock = threading.Lock()
_libs: dict = {}

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)


def build(ref: bool = True) -> None:
    """Compile the oracle (and, when the reference tree exists, oracle/_ref)."""
    targets = ["libkron_oracle.so"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", _HERE] + targets, check=True)


def _load(path: str, key: str):
    with _lock:
        if key not in _libs:
            _libs[key] = C.CDLL(path)
        return _libs[key]


def oracle_lib():
    if not os.path.exists(_ORACLE_SO):
        build(ref=False)
    return _load(_ORACLE_SO, "oracle")


def ref_lib():
    """The reference's own CPU build, or None where it was not compiled."""
    if not os.path.exists(_REF_SO):
        return None
    return _load(_REF_SO, "ref")


def set_threads(n: int) -> None:
    oracle_lib().kmo_set_threads(C.c_int(int(n)))


def max_threads() -> int:
    return int(oracle_lib().kmo_max_threads())


def _ptr(a: np.ndarray):
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.float32:
        return a.ctypes.data_as(_fp)
    raise TypeError(a.dtype)


def _suffix(dt) -> str:
    return {np.dtype(np.float64): "f64", np.dtype(np.float32): "f32"}[np.dtype(dt)]


def _ptr_array(base: np.ndarray, offsets) -> C.Array:
    """C array of pointers base + offset (offsets in elements)."""
    addr = base.ctypes.data
    it = base.itemsize
    arr = (C.c_void_p * len(offsets))()
    for i, o in enumerate(offsets):
        arr[i] = addr + int(o) * it
    return arr


def _ints(v) -> C.Array:
    v = [int(x) for x in v]
    return (C.c_int * len(v))(*v)


# ---------------------------------------------------------------------------
# Drivers mirroring the four reference entry points.
# ---------------------------------------------------------------------------

def batched(d, n, A, X, Y, W, batch, lib=None):
    """kronmult{d}_batched (kronmult6_batched.hpp:14-94); X and W are clobbered."""
    s = _suffix(A.dtype)
    if lib == "ref":
        fn = getattr(ref_lib(), f"ref_batched_{s}")
        rc = fn(C.c_int(d), C.c_int(n), _ptr(A), _ptr(X), _ptr(Y), _ptr(W), C.c_int(batch))
        assert rc == 0
    else:
        getattr(oracle_lib(), f"kmo_batched_{s}")(C.c_int(d), C.c_int(n), _ptr(A), _ptr(X),
                                                  _ptr(Y), _ptr(W), C.c_int(batch))


def pbatched(d, n, A, Xbuf, xoff, Ybuf, yoff, Wbuf, woff, lib=None):
    """kronmult{d}_pbatched (kronmult6_pbatched.hpp:14-81); pointers are
    base + offset (in elements) into the given buffers."""
    s = _suffix(A.dtype)
    batch = len(xoff)
    pX, pY, pW = _ptr_array(Xbuf, xoff), _ptr_array(Ybuf, yoff), _ptr_array(Wbuf, woff)
    if lib == "ref":
        rc = getattr(ref_lib(), f"ref_pbatched_{s}")(C.c_int(d), C.c_int(n), _ptr(A), pX, pY, pW,
                                                      C.c_int(batch))
        assert rc == 0
    else:
        getattr(oracle_lib(), f"kmo_pbatched_{s}")(C.c_int(d), C.c_int(n), _ptr(A), pX, pY, pW,
                                                   C.c_int(batch))


def xbatched(d, n, Abuf, aoff, lda, Xbuf, xoff, Ybuf, yoff, Wbuf, woff, subbatch=0, lib=None):
    """kronmult{d}_xbatched (kronmult_xbatched.hpp:19-157).  aoff is (batch, d)
    element offsets of each factor in Abuf; woff must provide the workspace
    slots the reference uses (2*subbatch when batch > 1, else 1)."""
    s = _suffix(Abuf.dtype)
    batch = len(xoff)
    aoff = np.asarray(aoff).reshape(batch * d)
    pA = _ptr_array(Abuf, aoff)
    pX, pY, pW = _ptr_array(Xbuf, xoff), _ptr_array(Ybuf, yoff), _ptr_array(Wbuf, woff)
    if lib == "ref":
        rc = getattr(ref_lib(), f"ref_xbatched_{s}")(C.c_int(d), C.c_int(n), pA, C.c_int(lda), pX,
                                                      pY, pW, C.c_int(batch), C.c_int(subbatch))
        assert rc == 0
    else:
        getattr(oracle_lib(), f"kmo_xbatched_{s}")(C.c_int(d), C.c_int(n), pA, C.c_int(lda), pX,
                                                   pY, pW, C.c_int(batch), C.c_int(subbatch))


def vbatched(d, m, nn, Abuf, aoff, Xbuf, xoff, Ybuf, yoff, W, lib=None):
    """kronmult{d}_vbatched (kronmult_vbatched.hpp:19-248); W is the single
    workspace, its byte size the capacity."""
    s = _suffix(Abuf.dtype)
    batch = len(xoff)
    aoff = np.asarray(aoff).reshape(batch * d)
    pA = _ptr_array(Abuf, aoff)
    pX, pY = _ptr_array(Xbuf, xoff), _ptr_array(Ybuf, yoff)
    cap = C.c_size_t(W.nbytes)
    if lib == "ref":
        rc = getattr(ref_lib(), f"ref_vbatched_{s}")(C.c_int(d), _ints(m), _ints(nn), pA, pX, pY,
                                                      _ptr(W), cap, C.c_int(batch))
    else:
        rc = getattr(oracle_lib(), f"kmo_vbatched_{s}")(C.c_int(d), _ints(m), _ints(nn), pA, pX,
                                                        pY, _ptr(W), cap, C.c_int(batch))
    assert rc == 0, "workspace holds no (X, W) slot pair"


def size_xw(d, m, nn) -> int:
    oracle_lib().kmo_size_xw.restype = C.c_size_t
    return int(oracle_lib().kmo_size_xw(C.c_int(d), _ints(m), _ints(nn)))


def kron_flops(d, m, nn) -> float:
    f = oracle_lib().kmo_kron_flops
    f.restype = C.c_double
    return float(f(C.c_int(d), _ints(m), _ints(nn)))


def xbatched_idx(d, n, Apool, lda, pool, Xpool, Ypool, y_idx, x_idx, a_idx):
    """Index-triple xbatched on the oracle: Apool is (d, pool, n, lda) in C
    order (each factor column-major lda x n), Xpool (nx, N), Ypool (ny, N)."""
    lib = oracle_lib()
    y_idx = np.ascontiguousarray(y_idx, dtype=np.int32)
    x_idx = np.ascontiguousarray(x_idx, dtype=np.int32)
    a_idx = np.ascontiguousarray(a_idx, dtype=np.int32)
    lib.kmo_xbatched_idx_f64(C.c_int(d), C.c_int(n), _ptr(Apool), C.c_int(lda), C.c_int(pool),
                             _ptr(Xpool), _ptr(Ypool), y_idx.ctypes.data_as(_ip),
                             x_idx.ctypes.data_as(_ip), a_idx.ctypes.data_as(_ip),
                             C.c_int(len(y_idx)))


def explicit_kron(d, m, nn, factors, lds, x):
    """Explicit-Kronecker product (test_kronmult6_batched.cpp:394-458) in long
    double, returned as float64.  factors[l] is a flat column-major array."""
    lib = oracle_lib()
    fs = [np.ascontiguousarray(f, dtype=np.float64) for f in factors]
    pA = (C.c_void_p * d)(*[f.ctypes.data for f in fs])
    x = np.ascontiguousarray(x, dtype=np.float64)
    M = int(np.prod(m))
    out = np.zeros(M, dtype=np.float64)
    lib.kmo_explicit_f64(C.c_int(d), _ints(m), _ints(nn), pA, _ints(lds), _ptr(x), _ptr(out))
    return out


def kron_batched_extended(d, n, A, X, absolute=False):
    """Y = kron(A_1, ..., A_d) X for every entry of a batched layout, evaluated
    mode by mode (the recursion of kronmultv.hpp:19-148) in numpy's extended
    precision (np.longdouble: 64-bit significand on x86, binary128 on aarch64),
    returned in that precision.  A is (batch, d, n, n) with A[b, l, j, i] =
    A_l(i, j) (column-major factors), X is (batch, n**d).  With absolute=True
    it returns |K| |X|, the magnitude the rounding errors scale with."""
    A = np.asarray(A, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[0]
    V = X.astype(np.longdouble).reshape((B,) + (n,) * d)
    if absolute:
        V = np.abs(V)
    for m in range(d):
        Am = A[:, m].astype(np.longdouble)  # [b, j, i]
        if absolute:
            Am = np.abs(Am)
        W = np.moveaxis(V, 1 + m, -1)         # [b, ..., j]
        W = np.einsum("bji,b...j->b...i", Am, W)
        V = np.moveaxis(W, -1, 1 + m)
    return V.reshape(B, -1)


def xbatched_idx_extended(d, n, Apool, Xpool, ny, y_idx, x_idx, a_idx):
    """Index-triple xbatched (pool layout of xbatched_idx, lda = n) in extended
    precision: Y[y_idx[e]] += kron(Apool[l, a_idx[e, l]]) Xpool[x_idx[e]],
    summed in np.longdouble from a zero Y and returned in that precision."""
    Ab = np.stack([Apool[np.arange(d), a_idx[e]] for e in range(len(y_idx))])
    contrib = kron_batched_extended(d, n, Ab, Xpool[x_idx])
    Y = np.zeros((ny, n ** d), dtype=np.longdouble)
    np.add.at(Y, y_idx, contrib)
    return Y


def kronmultv(d, m, nn, factors, lds, x, y):
    """One entry of the recursion, y += kron(...) x (x preserved)."""
    lib = oracle_lib()
    s = _suffix(x.dtype)
    fs = [np.ascontiguousarray(f, dtype=x.dtype) for f in factors]
    pA = (C.c_void_p * d)(*[f.ctypes.data for f in fs])
    getattr(lib, f"kmo_kronmultv_{s}")(C.c_int(d), _ints(m), _ints(nn), pA, _ints(lds), _ptr(x),
                                       _ptr(y))


# ---------------------------------------------------------------------------
# Input generators of the reference tests.
# ---------------------------------------------------------------------------

def ramp_x(N, batch, dtype=np.float64):
    """X(i,k) = (i + (k-1)*N) / (N*batch), 1-based (test_kronmult6_batched.cpp:148-161).
    Returned as (batch, N) C-order == (N, batch) column-major."""
    i = np.arange(1, N + 1, dtype=np.float64)
    k = np.arange(1, batch + 1, dtype=np.float64)
    r1 = i[None, :] + (k[:, None] - 1) * N
    return (r1 / (N * batch)).astype(dtype)


def ramp_a(n, d, batch, lda=None, dtype=np.float64):
    """A(i,j,l,k) = (i + (j-1)*n + (l-1)*n^2 + (k-1)*batch) / (n^2*d*batch)
    (test_kronmult6_batched.cpp:165-175, test_kronmult6_xbatched.cpp:265-279).
    Returned as (batch, d, n, lda) C-order == (lda, n, d, batch) column-major;
    rows n..lda-1 of the padded leading dimension are zero."""
    lda = n if lda is None else lda
    out = np.zeros((batch, d, n, lda), dtype=np.float64)
    i = np.arange(1, n + 1, dtype=np.float64)
    j = np.arange(1, n + 1, dtype=np.float64)
    for kb in range(batch):
        for l in range(d):
            r1 = i[None, :] + (j[:, None] - 1) * n + l * n * n + kb * batch
            out[kb, l, :, :n] = r1 / (n * n * d * batch)
    return out.astype(dtype)


def kgemm_batched(trans, mm, nn, kk, alpha, Abuf, aoff, ldA, Bbuf, boff, ldB, beta, Cbuf, coff,
                  ldC, lib=None):
    """kgemm_nn_batched / kgemm_nt_batched (kgemm_nn_batched.hpp:8-81,
    kgemm_nt_batched.hpp:8-79): for each entry, C = alpha*A*op(B) + beta*C.
    trans is "nn" or "nt"; *off are element offsets of each entry's matrix in
    its buffer; ldA/ldB/ldC are per-entry leading dimensions."""
    s = _suffix(Abuf.dtype)
    batch = len(aoff)
    pA, pB, pC = _ptr_array(Abuf, aoff), _ptr_array(Bbuf, boff), _ptr_array(Cbuf, coff)
    sc = C.c_double if s == "f64" else C.c_float
    args = (C.c_int(mm), C.c_int(nn), C.c_int(kk), sc(alpha), pA, _ints(ldA), pB, _ints(ldB),
            sc(beta), pC, _ints(ldC), C.c_int(batch))
    if lib == "ref":
        assert getattr(ref_lib(), f"ref_kgemm_{trans}_batched_{s}")(*args) == 0
    else:
        getattr(oracle_lib(), f"kmo_kgemm_{trans}_batched_{s}")(*args)


def ramp_kgemm(trans, mm, nn, kk, batch, dtype=np.float64):
    """The closed-form inputs of test_kgemm_nn_batched.cpp:181-217 (and the nt
    test): A(i,j) = 1+i+j*nrowA+ib, B(i,j) = 1/(1+i+j*nrowB+ib), C = 1, with
    1-based i, j and ld = number of rows.  Returns (A, B, C) as
    (batch, rows*cols) column-major arrays."""
    nrowB, ncolB = (kk, nn) if trans == "nn" else (nn, kk)
    A = np.empty((batch, mm * kk), dtype=np.float64)
    B = np.empty((batch, nrowB * ncolB), dtype=np.float64)
    for ib in range(batch):
        i, j = np.meshgrid(np.arange(1, mm + 1), np.arange(1, kk + 1), indexing="ij")
        A[ib] = (1.0 + i + j * mm + ib).ravel(order="F")
        i, j = np.meshgrid(np.arange(1, nrowB + 1), np.arange(1, ncolB + 1), indexing="ij")
        B[ib] = (1.0 / (1.0 + i + j * nrowB + ib)).ravel(order="F")
    Cm = np.ones((batch, mm * nn), dtype=np.float64)
    return A.astype(dtype), B.astype(dtype), Cm.astype(dtype)
