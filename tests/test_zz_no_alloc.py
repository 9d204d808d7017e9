"""GPU tests of kmx_kronmult_xbatched_f64_noalloc, the deterministic xbatched
entry point for callers that cannot allocate device memory (a plug-in inside
a host application that owns every device allocation, code between graph
launches, a pool-disciplined process): its sort and segment scratch is a
fixed array in the library's device image.

- Two calls in a row through the C ABI, on two different batches: each result
  equals, bit for bit, the allocating deterministic entry point's
  (kmx_kronmult_xbatched_f64_ex, accumulate = deterministic: same form, same
  kernels, same segment order) and is within 1e-13 of the oracle; the second
  call checks that the first call's leftovers in the shared scratch do not
  leak into it.
- A batch whose scratch would exceed the fixed capacity, and a shape whose
  entry needs a global workspace (n = 8, d = 6), are refused before anything
  runs: KMX_ERR_WORKSPACE and KMX_ERR_UNSUPPORTED, Y untouched.
- In a fresh process, two calls allocate nothing: device memory outside
  torch's cache is the same before and after, and the library's cached
  workspaces stay empty.

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-13  # normwise relative error per Y block against the oracle
SCRATCH_BYTES = 16 << 20
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _case(seed, d, n, pool, nx, ny, ne):
    rng = np.random.default_rng(seed)
    N = n ** d
    A = rng.standard_normal((d, pool, n, n)) / 2
    X = rng.standard_normal((nx, N))
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.geometric(0.2, ne) % ny
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    At, Xt = torch.from_numpy(A).cuda(), torch.from_numpy(X).cuda()
    lvl = np.arange(d)[None, :]
    pA = torch.from_numpy(((lvl * pool + a_idx) * (n * n * 8)).reshape(-1)).cuda() + At.data_ptr()
    pX = torch.from_numpy(x_idx * (N * 8)).cuda() + Xt.data_ptr()
    return dict(d=d, n=n, N=N, ne=ne, pool=pool, A=A, X=X, Y0=Y0, y_idx=y_idx, x_idx=x_idx,
                a_idx=a_idx, At=At, Xt=Xt, pA=pA, pX=pX)


def _run(kmx, c, noalloc):
    L = kmx.lib()
    Y = torch.from_numpy(c["Y0"]).cuda()
    pY = torch.from_numpy(c["y_idx"] * (c["N"] * 8)).cuda() + Y.data_ptr()
    stream = torch.cuda.current_stream().cuda_stream
    if noalloc:
        rc = L.kmx_kronmult_xbatched_f64_noalloc(c["d"], c["n"], c["pA"].data_ptr(), c["n"],
                                                 c["pX"].data_ptr(), pY.data_ptr(), c["ne"],
                                                 stream)
    else:
        o = kmx.options("auto", "deterministic")
        rc = L.kmx_kronmult_xbatched_f64_ex(c["d"], c["n"], c["pA"].data_ptr(), c["n"],
                                            c["pX"].data_ptr(), pY.data_ptr(), None, c["ne"], 0,
                                            C.byref(o), stream)
    torch.cuda.synchronize()
    assert rc == 0, L.kmx_status_string(rc)
    assert kmx.check_device_status() == 0
    return Y


def test_noalloc_matches_allocating_entry_point_twice(kmx, oracle):
    first = _case(101, 6, 4, pool=64, nx=60, ny=40, ne=1500)
    second = _case(202, 4, 8, pool=32, nx=30, ny=9, ne=400)  # other shape, fewer segments
    # two no-allocation calls back to back, then the allocating entry point
    y1 = _run(kmx, first, noalloc=True)
    y2 = _run(kmx, second, noalloc=True)
    for c, y in ((first, y1), (second, y2)):
        y_ref = _run(kmx, c, noalloc=False)
        assert torch.equal(y, y_ref), float((y - y_ref).abs().max())
        Yo = c["Y0"].copy()
        oracle.xbatched_idx(c["d"], c["n"], c["A"], c["n"], c["pool"], c["X"], Yo, c["y_idx"],
                            c["x_idx"], c["a_idx"])
        assert blockwise_rel_err(y.cpu().numpy() - c["Y0"], Yo - c["Y0"]) <= TOL


def test_noalloc_refuses_batches_beyond_its_scratch(kmx):
    L = kmx.lib()
    big = 1
    while L.kmx_deterministic_workspace_bytes(big) <= SCRATCH_BYTES:
        big *= 2
    # valid arrays of that length, although the call must refuse before reading them
    c = _case(7, 6, 4, pool=8, nx=4, ny=4, ne=big)
    Y = torch.from_numpy(c["Y0"]).cuda()
    pY = torch.from_numpy(c["y_idx"] * (c["N"] * 8)).cuda() + Y.data_ptr()
    rc = L.kmx_kronmult_xbatched_f64_noalloc(6, 4, c["pA"].data_ptr(), 4, c["pX"].data_ptr(),
                                             pY.data_ptr(), big, 0)
    torch.cuda.synchronize()
    assert L.kmx_status_string(rc) == b"KMX_ERR_WORKSPACE"
    assert torch.equal(Y.cpu(), torch.from_numpy(c["Y0"]))


@pytest.mark.parametrize("d,n", [(6, 8), (5, 8)])
def test_noalloc_refuses_entries_beyond_shared_memory(kmx, d, n):
    """An entry whose intermediate needs a global workspace: unsupported,
    refused before the segment sort runs (a distinct status from capacity)."""
    L = kmx.lib()
    c = _case(9, d, n, pool=4, nx=2, ny=2, ne=4)
    Y = torch.from_numpy(c["Y0"]).cuda()
    pY = torch.from_numpy(c["y_idx"] * (c["N"] * 8)).cuda() + Y.data_ptr()
    rc = L.kmx_kronmult_xbatched_f64_noalloc(d, n, c["pA"].data_ptr(), n, c["pX"].data_ptr(),
                                             pY.data_ptr(), c["ne"], 0)
    torch.cuda.synchronize()
    assert L.kmx_status_string(rc) == b"KMX_ERR_UNSUPPORTED"
    assert torch.equal(Y.cpu(), torch.from_numpy(c["Y0"]))
    assert kmx.check_device_status() == 0


_FRESH = textwrap.dedent("""
    import sys
    sys.path.insert(0, {root!r})
    import numpy as np
    import torch
    import kronmult_gb300 as kmx
    from tests.test_zz_no_alloc import _case, _run
    L = kmx.lib()
    a = _case(303, 6, 4, pool=32, nx=20, ny=12, ne=600)
    b = _case(404, 3, 8, pool=16, nx=10, ny=5, ne=200)
    _run(kmx, a, noalloc=True)   # loads the kernels' modules (lazy loading)
    _run(kmx, b, noalloc=True)
    torch.cuda.synchronize()
    # device memory outside torch's own cache: any allocation by the library
    # (cudaMalloc, cudaMallocAsync) would lower it
    free0 = torch.cuda.mem_get_info()[0] + torch.cuda.memory_reserved()
    cached0 = L.kmx_cached_workspace_bytes()
    _run(kmx, a, noalloc=True)
    _run(kmx, b, noalloc=True)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0] + torch.cuda.memory_reserved()
    cached1 = L.kmx_cached_workspace_bytes()
    print("free", free0, free1, "cached", cached0, cached1)
    assert cached0 == 0 and cached1 == 0, (cached0, cached1)
    assert free0 == free1, (free0, free1)
    print("NOALLOC_OK")
""")


def test_noalloc_allocates_nothing_in_a_fresh_process(kmx):
    env = dict(os.environ)
    env["PYTHONPATH"] = ROOT + os.pathsep + env.get("PYTHONPATH", "")
    r = subprocess.run([sys.executable, "-c", _FRESH.format(root=ROOT)], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "NOALLOC_OK" in r.stdout, r.stdout[-2000:] + r.stderr[-4000:]
