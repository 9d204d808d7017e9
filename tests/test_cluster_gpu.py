"""GPU parity of the cluster kernels: double-float entries beyond one SM's
shared memory (d=5 n=8, d=6 n=6, 7, 8), n CTAs per (entry, i1) sharing mode 2
through distributed shared memory.  Through the C ABI against the oracle:
batched and xbatched layouts (overlapping Y blocks, padded lda, transpose),
no workspace passed (the cluster kernels need none), entries with Inf/NaN or
an all-zero factor, and cancelling entries recomputed in FP64 by the guard
(counted per block of n^(d-2) outputs).  Tolerance: 1e-13 normwise per Y
block."""
import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPES = [(5, 8), (6, 6), (6, 7), (6, 8)]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("d,n", SHAPES)
def test_cluster_batched_without_workspace(kmx, oracle, d, n):
    rng = np.random.default_rng(7 * d + n)
    N = n ** d
    batch = 6 if N > 100000 else 12
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    Y0 = rng.uniform(-1, 1, (batch, N))
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = dev(Y0)
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form="split", engine="tiled")
    assert kmx.check_device_status() == 0
    assert blockwise_rel_err(Yd.cpu().numpy() - Y0, Yref - Y0) <= 1e-13


@pytest.mark.parametrize("d,n", [(5, 8), (6, 6)])
@pytest.mark.parametrize("transpose", [False, True])
def test_cluster_xbatched_overlap(kmx, oracle, d, n, transpose):
    """Pointer layout, lda = n + 1, Y blocks shared by several entries."""
    rng = np.random.default_rng(300 + d * n + transpose)
    N = n ** d
    pool, nx, ny, ne, lda = 6, 5, 3, 14, n + 1
    Apool = rng.standard_normal((d, pool, n, lda)) / 2
    Xpool = rng.standard_normal((nx, N))
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.integers(0, ny, ne)
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    Yref = Y0.copy()
    for e in range(ne):
        fs = [Apool[l, a_idx[e, l]].ravel() for l in range(d)]
        if transpose:
            fs = [np.ascontiguousarray(f.reshape(n, lda)[:, :n].T).ravel() for f in fs]
            lds = [n] * d
        else:
            lds = [lda] * d
        y = np.zeros(N)
        oracle.kronmultv(d, [n] * d, [n] * d, fs, lds, Xpool[x_idx[e]].copy(), y)
        Yref[y_idx[e]] += y
    Ad, Xd, Yd = dev(Apool), dev(Xpool), dev(Y0)
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * lda).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    pY = kmx.pointer_array(Yd, y_idx * N)
    kmx.kronmult_xbatched(d, n, pA, lda, pX, pY, None, ne, form="split", transpose=transpose,
                          engine="tiled")
    assert kmx.check_device_status() == 0
    assert blockwise_rel_err(Yd.cpu().numpy() - Y0, Yref - Y0) <= 1e-13


@pytest.mark.parametrize("d,n", [(5, 8), (6, 6)])
def test_cluster_special_entries(kmx, oracle, d, n):
    """Inf/NaN (FP64 blocks in the recursion's mode order, IEEE propagation),
    an all-zero factor (exact zero) and cancelling entries (zero row sums on
    X = 1 + 1e-2 Z: every block's rho_F is far below 1/4, so each of the n*n
    blocks is recomputed in FP64)."""
    rng = np.random.default_rng(55 + d * n)
    N = n ** d
    batch = 9
    A = rng.standard_normal((batch, d, n, n)) / 2
    X = rng.standard_normal((batch, N))
    canc = np.array([1, 4, 7])
    A[canc] -= A[canc].mean(axis=2, keepdims=True)
    X[canc] = 1.0 + 1e-2 * rng.standard_normal((len(canc), N))
    A[2, 3] = 0.0                # an all-zero factor
    X[5, 17] = np.nan            # NaN in X
    A[8, 0, 1, 2] = np.inf       # Inf in a factor
    Yx = oracle.kron_batched_extended(d, n, A, X).astype(np.float64)
    Yd = torch.zeros((batch, N), dtype=torch.float64, device="cuda")
    kmx.read_redo_counters()
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form="split", engine="tiled")
    guard, _ = kmx.read_redo_counters()
    assert kmx.check_device_status() == 0
    y = Yd.cpu().numpy()
    fin = np.all(np.isfinite(Yx), axis=1)
    assert np.array_equal(np.isnan(y[~fin]), np.isnan(Yx[~fin]))
    assert np.array_equal(np.isinf(y[~fin]), np.isinf(Yx[~fin]))
    assert not y[2].any()
    ok = fin & (np.arange(batch) != 2)
    assert blockwise_rel_err(y[ok], Yx[ok]) <= 1e-13
    assert guard == len(canc) * n * n


@pytest.mark.parametrize("engine", ["tuned", "cluster"])
def test_cluster_mixed_call_without_workspace(kmx, oracle, engine):
    """A mixed-shape call with classes beyond one SM (d=5 n=8, d=6 n=6) and no
    workspace: those classes run the cluster kernels (their class count read
    on the device), the rest their usual kernels; every instance against the
    oracle."""
    rng = np.random.default_rng(91)
    dims = [(5, 8), (6, 6), (3, 4), (5, 8), (2, 8), (6, 6), (4, 5), (5, 8)]
    factors, xs, ys, a_off, o = [], [], [], [], 0
    for d, n in dims:
        a_off.append(o)
        for _ in range(d):
            factors.append(rng.uniform(-1, 1, n * n))
            o += 1
        xs.append(rng.uniform(-1, 1, n ** d))
        ys.append(rng.uniform(-1, 1, n ** d))
    fbuf, xbuf, ybuf = dev(np.concatenate(factors)), dev(np.concatenate(xs)), dev(np.concatenate(ys))
    foffs = np.cumsum([0] + [f.size for f in factors[:-1]])
    xoffs = np.cumsum([0] + [x.size for x in xs[:-1]])
    classes = sorted(set(dims), key=lambda c: -(c[1] ** (c[0] + 1) * c[0]))
    kmx.kronmult_mixed(dev(np.array(dims, dtype=np.int32)), kmx.pointer_array(fbuf, foffs),
                       dev(np.array(a_off, dtype=np.int64)), kmx.pointer_array(xbuf, xoffs),
                       kmx.pointer_array(ybuf, xoffs), classes, None, form="split", engine=engine)
    assert kmx.check_device_status() == 0
    y = ybuf.cpu().numpy()
    for i, (d, n) in enumerate(dims):
        ref = ys[i].copy()
        oracle.kronmultv(d, [n] * d, [n] * d, factors[a_off[i]: a_off[i] + d], [n] * d,
                         xs[i].copy(), ref)
        seg = y[xoffs[i]: xoffs[i] + n ** d]
        assert blockwise_rel_err(seg - ys[i], ref - ys[i]) <= 1e-13, (i, d, n)


def test_cluster_engine_with_workspace(kmx, oracle):
    """engine="cluster" with a workspace still takes the cluster kernel; the
    tuned engine with the same workspace takes the per-mode kernels; both
    agree with the oracle."""
    d, n, batch = 5, 8, 8
    rng = np.random.default_rng(17)
    N = n ** d
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    Y0 = rng.uniform(-1, 1, (batch, N))
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    for engine in ("cluster", "tuned"):
        Yd = dev(Y0)
        W = torch.empty((batch, N), dtype=torch.float64, device="cuda")
        kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, W, batch, form="split", engine=engine)
        assert kmx.check_device_status() == 0
        assert blockwise_rel_err(Yd.cpu().numpy() - Y0, Yref - Y0) <= 1e-13, engine
