"""GPU test of kmx_kronmult_xbatched_f64_noalloc, the deterministic xbatched
entry point for callers that cannot allocate device memory (its scratch is a
fixed array in the library's device image).

It is called through the C ABI twice in a row, on two different batches, and
each result is compared with the allocating deterministic entry point
(kmx_kronmult_xbatched_f64_ex with accumulate = deterministic) on the same
inputs: the second call checks that the first call's leftovers in the shared
scratch do not leak into it.  A batch whose scratch would exceed the fixed
capacity must be refused before anything runs.

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-13  # normwise relative error per Y block, the FP64 parity bound
SCRATCH_BYTES = 16 << 20


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _case(seed, d, n, pool, nx, ny, ne):
    rng = np.random.default_rng(seed)
    N = n ** d
    A = torch.from_numpy(rng.standard_normal((d, pool, n, n)) / 2).cuda()
    X = torch.from_numpy(rng.standard_normal((nx, N))).cuda()
    Y0 = torch.from_numpy(rng.standard_normal((ny, N))).cuda()
    y_idx = torch.from_numpy(rng.geometric(0.2, ne) % ny).cuda()
    x_idx = torch.from_numpy(rng.integers(0, nx, ne)).cuda()
    a_idx = torch.from_numpy(rng.integers(0, pool, (ne, d))).cuda()
    lvl = torch.arange(d, device="cuda")[None, :]
    pA = ((lvl * pool + a_idx) * (n * n * 8) + A.data_ptr()).reshape(-1).contiguous()
    pX = x_idx * (N * 8) + X.data_ptr()
    return dict(d=d, n=n, N=N, ne=ne, A=A, X=X, Y0=Y0, y_idx=y_idx, pA=pA, pX=pX)


def _run(kmx, c, noalloc):
    L = kmx.lib()
    Y = c["Y0"].clone()
    pY = c["y_idx"] * (c["N"] * 8) + Y.data_ptr()
    stream = torch.cuda.current_stream().cuda_stream
    if noalloc:
        rc = L.kmx_kronmult_xbatched_f64_noalloc(c["d"], c["n"], c["pA"].data_ptr(), c["n"],
                                                 c["pX"].data_ptr(), pY.data_ptr(), c["ne"],
                                                 stream)
    else:
        from kronmult_gb300 import _lib

        o = _lib.options("auto", "deterministic")
        rc = L.kmx_kronmult_xbatched_f64_ex(c["d"], c["n"], c["pA"].data_ptr(), c["n"],
                                            c["pX"].data_ptr(), pY.data_ptr(), None, c["ne"], 0,
                                            C.byref(o), stream)
    torch.cuda.synchronize()
    assert rc == 0, kmx.lib().kmx_status_string(rc)
    assert kmx.check_device_status() == 0
    return Y


def _rel(y, yref):
    s = yref.abs().amax(dim=1, keepdim=True).clamp_min(1e-300)
    num = torch.linalg.vector_norm((y - yref) / s, dim=1)
    den = torch.linalg.vector_norm(yref / s, dim=1).clamp_min(1e-300)
    return float((num / den).max())


def test_noalloc_matches_allocating_entry_point_twice(kmx):
    first = _case(101, 6, 4, pool=64, nx=60, ny=40, ne=1500)
    second = _case(202, 4, 8, pool=32, nx=30, ny=9, ne=400)  # other shape, fewer segments
    # two no-allocation calls back to back, then the allocating entry point
    y1 = _run(kmx, first, noalloc=True)
    y2 = _run(kmx, second, noalloc=True)
    for c, y in ((first, y1), (second, y2)):
        y_ref = _run(kmx, c, noalloc=False)
        assert _rel(y, y_ref) <= TOL
        assert not torch.equal(y, c["Y0"])  # something was accumulated


def test_noalloc_refuses_batches_beyond_its_scratch(kmx):
    L = kmx.lib()
    big = 1
    while L.kmx_deterministic_workspace_bytes(big) <= SCRATCH_BYTES:
        big *= 2
    # valid arrays of that length, although the call must refuse before reading them
    c = _case(7, 6, 4, pool=8, nx=4, ny=4, ne=big)
    Y = c["Y0"].clone()
    pY = c["y_idx"] * (c["N"] * 8) + Y.data_ptr()
    rc = L.kmx_kronmult_xbatched_f64_noalloc(6, 4, c["pA"].data_ptr(), 4, c["pX"].data_ptr(),
                                             pY.data_ptr(), big, 0)
    torch.cuda.synchronize()
    assert kmx.lib().kmx_status_string(rc) == b"KMX_ERR_WORKSPACE"
    assert torch.equal(Y, c["Y0"])
