"""GPU parity of the small-entry kernels (engine KMX_ENGINE_SMALL: d <= 3 with
n^d <= 256, many entries per CTA) and of the lane kernels (engine
KMX_ENGINE_LANE: one entry per thread for n^2 <= 16 and n^d <= 16, one group
of n lanes per entry for d = 2 with n = 5..8, one group of n^(d-1) <= 32
lanes per entry for d >= 3) against the oracle, through the C ABI.

Covers the contiguous batched layout (staged with 128-bit loads, and at an
offset that breaks 16-byte alignment), the pointer layouts with overlapping Y
blocks (atomics), the transpose option, ragged chunk tails, every arithmetic
form (FP64 plain and double-float, FP32 with the reference's rounding and
FP32 FMA), and the double-float form's special entries: Inf/NaN (FP64 path),
all-zero factors (exact zero), cancelling entries (guard, counted).
Tolerances: FP64 1e-13 normwise per Y block; FP32 ulps as in
test_f32_semantics_gpu (reference form) or the reference test's 1e-5 (FMA)."""
import numpy as np
import pytest

from tests.common import blockwise_rel_err, ref_test_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPES = [(1, 2), (1, 3), (1, 4), (1, 8), (1, 16), (2, 2), (2, 3), (2, 4), (2, 5), (2, 6),
          (2, 7), (2, 8), (2, 16), (3, 2), (3, 3), (3, 4), (3, 5), (3, 6), (4, 2), (4, 3),
          (5, 2), (6, 2)]


ENGINES = ["small", "lane"]


def engine_shape(engine, d, n):
    """Skip a case whose shape the engine's kernels do not take."""
    if engine == "lane" and not ((d <= 3 and n * n <= 16 and n ** d <= 16) or
                                 (d == 2 and 5 <= n <= 8) or
                                 (3 <= d <= 6 and n ** (d - 1) <= 32)):
        pytest.skip("shape beyond the lane kernels")
    if engine == "small" and not (d <= 3 and n ** d <= 256):
        pytest.skip("shape beyond the small-entry kernels")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def ulps(y, ref):
    ref32 = np.asarray(ref, dtype=np.float32).ravel()
    sp = np.spacing(np.abs(ref32)).astype(np.float64)
    return np.abs(np.asarray(y, dtype=np.float64).ravel() - ref32.astype(np.float64)) / sp


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("d,n", SHAPES)
@pytest.mark.parametrize("form", ["plain", "split"])
def test_small_batched_f64(kmx, oracle, d, n, form, engine):
    engine_shape(engine, d, n)
    rng = np.random.default_rng(50 + 10 * d + n)
    N = n ** d
    batch = 1237  # several chunks and a ragged tail
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    Y0 = rng.uniform(-1, 1, (batch, N))
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    for offset in (0, 1):  # offset 1: X no longer 16-byte aligned
        Xd = dev(np.concatenate([np.zeros(offset), X.ravel()]))[offset:]
        Yd = dev(Y0)
        kmx.kronmult_batched(d, n, dev(A), Xd, Yd, None, batch, form=form, engine=engine)
        assert blockwise_rel_err(Yd.cpu().numpy() - Y0, Yref - Y0) <= 1e-13, offset
    assert kmx.check_device_status() == 0


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("d,n", SHAPES)
def test_small_batched_f32(kmx, oracle, d, n, engine):
    engine_shape(engine, d, n)
    rng = np.random.default_rng(70 + 10 * d + n)
    N = n ** d
    batch = 999
    A = (rng.standard_normal((batch, d, n, n)) / np.sqrt(n)).astype(np.float32)
    X = rng.standard_normal((batch, N)).astype(np.float32)
    Y0 = rng.uniform(-1, 1, (batch, N)).astype(np.float32)
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = dev(Y0)
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, engine=engine)  # reference form
    u = ulps(Yd.cpu().numpy(), Yref)
    assert np.mean(u <= 1.0) >= 0.999 and u.max() <= 8.0, (float(np.mean(u <= 1)), float(u.max()))
    Yp = dev(Y0)
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yp, None, batch, form="plain", engine=engine)
    assert ref_test_err(Yp.cpu().numpy(), Yref) <= 1e-5
    assert kmx.check_device_status() == 0


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("d,n", [(1, 4), (2, 3), (2, 5), (2, 8), (3, 2), (3, 4), (3, 5), (4, 3),
                                 (6, 2)])
@pytest.mark.parametrize("form", ["plain", "split"])
@pytest.mark.parametrize("transpose", [False, True])
def test_small_xbatched_overlap(kmx, oracle, d, n, form, transpose, engine):
    """Pointer layout, lda = n + 2, Y blocks shared by many entries (atomics)."""
    engine_shape(engine, d, n)
    rng = np.random.default_rng(90 + d * n)
    N = n ** d
    pool, nx, ny, ne, lda = 16, 40, 13, 2000, n + 2
    Apool = rng.standard_normal((d, pool, n, lda))  # column j of A at [.., j, :n] (lda rows)
    Xpool = rng.standard_normal((nx, N))
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.geometric(0.1, ne) % ny
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
    kmx.kronmult_xbatched(d, n, pA, lda, pX, pY, None, ne, form=form, transpose=transpose,
                          engine=engine)
    assert kmx.check_device_status() == 0
    assert blockwise_rel_err(Yd.cpu().numpy() - Y0, Yref - Y0) <= 1e-13


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("d,n", [(1, 3), (1, 8), (2, 2), (2, 4), (2, 5), (2, 8), (3, 2), (3, 3),
                                 (3, 4), (4, 3), (5, 2)])
def test_small_split_special_entries(kmx, oracle, d, n, engine):
    """Double-float in the small and lane kernels: entries with Inf/NaN (FP64
    path, IEEE propagation), an all-zero factor (exact zero), and cancelling
    entries (rows summing to zero on X = 1 + 1e-2 Z: recomputed in FP64 by the
    guard, counted) among ordinary ones.  Held to 1e-13 per block for n >= 3
    and blocks of 8 or more elements; n = 2 and smaller blocks to 5e-13: the
    guard keeps entries down to rho_F = 1/4, where the double-float bound
    c 2^-48 sqrt(N) / rho_F is widest relative to the block, and two-term dot
    products do not average the rounding errors (measured: d=2 n=2 3.9e-13,
    d=3 n=2 1.6e-13, d=1 n=3 1.06e-13; the automatic form runs plain FP64 for
    all of these shapes)."""
    engine_shape(engine, d, n)
    rng = np.random.default_rng(123 + d * n)
    N = n ** d
    batch = 700
    A = rng.standard_normal((batch, d, n, n)) / 2
    X = rng.standard_normal((batch, N))
    canc = np.arange(batch) % 7 == 3
    A[canc] -= A[canc].mean(axis=2, keepdims=True)
    X[canc] = 1.0 + 1e-2 * rng.standard_normal((int(canc.sum()), N))
    # special entries, none of them a cancelling one (index % 7 != 3)
    A[5, 0] = 0.0               # an all-zero factor
    X[11, 0] = np.inf           # Inf in X
    A[16, d - 1, 0, 0] = np.nan  # NaN in a factor
    Y0 = np.zeros((batch, N))
    Yx = oracle.kron_batched_extended(d, n, A, X).astype(np.float64)
    Yd = dev(Y0)
    kmx.read_redo_counters()
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form="split", engine=engine)
    guard, _ = kmx.read_redo_counters()
    assert kmx.check_device_status() == 0
    y = Yd.cpu().numpy()
    fin = np.all(np.isfinite(Yx), axis=1)
    assert np.array_equal(np.isnan(y[~fin]), np.isnan(Yx[~fin]))
    assert np.array_equal(np.isinf(y[~fin]), np.isinf(Yx[~fin]))
    assert not y[5].any()
    ok = fin & (np.arange(batch) != 5)
    assert blockwise_rel_err(y[ok], Yx[ok]) <= (1e-13 if n >= 3 and N >= 8 else 5e-13)
    assert guard >= int(canc.sum())


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("form", ["plain", "split"])
@pytest.mark.parametrize("d,n", [(1, 4), (2, 3), (2, 6), (3, 2), (3, 4)])
def test_small_null_entry_pointer_sets_device_status(kmx, d, n, form, engine):
    """A NULL inside a device pointer array: the entry is skipped, the status
    word reports it (no fault), and the other entries are computed."""
    engine_shape(engine, d, n)
    batch, N = 300, n ** d
    A = torch.rand((batch, d, n, n), dtype=torch.float64, device="cuda")
    X = torch.rand((batch, N), dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    pX = kmx.pointer_array(X, [b * N for b in range(batch)])
    pX[7] = 0
    pY = kmx.pointer_array(Y, [b * N for b in range(batch)])
    kmx.kronmult_pbatched(d, n, A, pX, pY, None, batch, form=form, engine=engine)
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()
    y = Y.cpu().numpy()
    assert not y[7].any() and y[0].any() and y[batch - 1].any()
    assert kmx.check_device_status() == 0  # cleared
