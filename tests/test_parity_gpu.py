"""GPU parity of the CUDA path against the oracle and the golden vectors of the
reference's own build.  Every call goes through the C ABI.

Tolerances:
  FP64 forms (plain and split): normwise relative error per Y block <= 1e-13.
  FP32: the reference test's min(abs, rel) metric <= 1e-5
        (test_kronmult6_xbatched.cpp:758) and normwise <= 2e-6.
"""
import numpy as np
import pytest

from tests.common import blockwise_rel_err, golden, ref_test_err, vb_cases

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F64_TOL = 1e-13
F32_TOL = 1e-5
F32_NORM_TOL = 2e-6
FORMS = ["plain", "split", "digits"]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def check_status(kmx):
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0


# ---------------------------------------------------------------------------
# golden vectors (reference's own CPU build, ramp inputs of its tests)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("d", range(1, 7))
def test_batched_golden(kmx, oracle, form, d):
    g = golden()
    for n in (1, 2, 3, 4):
        N = n ** d
        for batch in (1, 3):
            A = dev(oracle.ramp_a(n, d, batch))
            X = dev(oracle.ramp_x(N, batch))
            X0 = X.clone()
            Y = torch.zeros_like(X)
            W = torch.zeros_like(X)
            kmx.kronmult_batched(d, n, A, X, Y, W, batch, form=form)
            err = blockwise_rel_err(host(Y), g[f"batched_d{d}_n{n}_b{batch}"])
            assert err <= F64_TOL, (n, batch, err)
            assert torch.equal(X, X0)  # X is never modified
    check_status(kmx)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("d", range(1, 7))
def test_pbatched_overlap_golden(kmx, oracle, form, d):
    g = golden()
    for n in (1, 2, 3, 4):
        N = n ** d
        batch = 4
        X = dev(oracle.ramp_x(N, batch))
        A = dev(oracle.ramp_a(n, d, batch))
        Y = torch.zeros((batch, N), dtype=torch.float64, device="cuda")
        W = torch.zeros_like(Y)
        pX = kmx.pointer_array(X, [b * N for b in range(batch)])
        pY = kmx.pointer_array(Y, [0] * batch)  # every entry accumulates into Y(:,1)
        pW = kmx.pointer_array(W, [b * N for b in range(batch)])
        kmx.kronmult_pbatched(d, n, A, pX, pY, pW, batch, form=form)
        y = host(Y)
        assert blockwise_rel_err(y[0], g[f"pbatched_d{d}_n{n}_b{batch}"]) <= F64_TOL
        assert not y[1:].any()
    check_status(kmx)


@pytest.mark.parametrize("form", FORMS + ["f32"])
@pytest.mark.parametrize("d", range(1, 7))
def test_xbatched_padded_lda_overlap_golden(kmx, oracle, form, d):
    g = golden()
    f32 = form == "f32"
    T = np.float32 if f32 else np.float64
    tag = "f32" if f32 else "f64"
    for n in (1, 2, 3, 4):
        N = n ** d
        for batch in (1, 4):
            lda = n + 3
            Ab = dev(oracle.ramp_a(n, d, batch, lda=lda, dtype=T))
            X = dev(oracle.ramp_x(N, batch, dtype=T))
            X0 = X.clone()
            Y = torch.zeros(N, dtype=X.dtype, device="cuda")
            W = torch.zeros((max(batch, 2), N), dtype=X.dtype, device="cuda")
            pA = kmx.pointer_array(Ab, [(b * d + l) * n * lda for b in range(batch) for l in range(d)])
            pX = kmx.pointer_array(X, [b * N for b in range(batch)])
            pY = kmx.pointer_array(Y, [0] * batch)
            pW = kmx.pointer_array(W, [b * N for b in range(W.shape[0])])
            kmx.kronmult_xbatched(d, n, pA, lda, pX, pY, pW, batch, dtype=X.dtype,
                                  form=None if f32 else form)
            y = host(Y)
            ref = g[f"xbatched_{tag}_d{d}_n{n}_b{batch}"]
            if f32:
                assert ref_test_err(y, ref) <= F32_TOL
                assert blockwise_rel_err(y, ref) <= F32_NORM_TOL
            else:
                assert blockwise_rel_err(y, ref) <= F64_TOL, (n, batch)
            assert torch.equal(X, X0)
    check_status(kmx)


@pytest.mark.parametrize("ci,d", vb_cases())
@pytest.mark.parametrize("form", FORMS + ["f32"])
def test_vbatched_rectangular_golden(kmx, ci, d, form):
    g = golden()
    m, nn = g[f"vbatched_c{ci}_m"], g[f"vbatched_c{ci}_n"]
    A, X, Y0 = g[f"vbatched_c{ci}_A"], g[f"vbatched_c{ci}_X"], g[f"vbatched_c{ci}_Y0"]
    f32 = form == "f32"
    T = np.float32 if f32 else np.float64
    batch, Nx = X.shape
    Ny = Y0.shape[1]
    fsz = [int(m[l] * nn[l]) for l in range(d)]
    offs, o = [], 0
    for b in range(batch):
        for l in range(d):
            offs.append(o)
            o += fsz[l]
    Ad, Xd, Yd = dev(A.astype(T)), dev(X.astype(T)), dev(Y0.astype(T))
    pA = kmx.pointer_array(Ad, offs)
    pX = kmx.pointer_array(Xd, [b * Nx for b in range(batch)])
    pY = kmx.pointer_array(Yd, [b * Ny for b in range(batch)])
    W = torch.zeros(1 << 16, dtype=Xd.dtype, device="cuda")
    kmx.kronmult_vbatched(d, m, nn, pA, pX, pY, W, None, batch, dtype=Xd.dtype,
                          form=None if f32 else form)
    y = host(Yd)
    ref = g[f"vbatched_{'f32' if f32 else 'f64'}_c{ci}"]
    if f32:
        assert ref_test_err(y, ref) <= F32_TOL
    else:
        assert blockwise_rel_err(y, ref) <= F64_TOL
    check_status(kmx)


# ---------------------------------------------------------------------------
# random inputs against the oracle: larger n, accumulate into nonzero Y,
# the shared-memory and the global-workspace paths
# ---------------------------------------------------------------------------

SHAPES = [(1, 7), (2, 9), (3, 8), (3, 16), (4, 5), (4, 8), (5, 4), (5, 6), (6, 2), (6, 3),
          (6, 4), (6, 5), (2, 1), (4, 11), (5, 8)]


@pytest.mark.parametrize("d,n", SHAPES)
@pytest.mark.parametrize("form", FORMS)
def test_batched_random_vs_oracle(kmx, oracle, d, n, form):
    rng = np.random.default_rng(1000 * d + n)
    N = n ** d
    batch = 5 if N <= 40000 else 2
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    Y0 = rng.uniform(-1, 1, (batch, N))
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Xd, Yd = dev(X), dev(Y0)
    Wd = torch.zeros_like(Xd)
    kmx.kronmult_batched(d, n, dev(A), Xd, Yd, Wd, batch, form=form)
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("d,n", [(6, 4), (4, 8), (3, 16), (5, 3), (6, 8)])
def test_f32_random_vs_oracle(kmx, oracle, d, n):
    rng = np.random.default_rng(77 + d * n)
    N = n ** d
    batch = 4 if N <= 40000 else 2
    A = (rng.standard_normal((batch, d, n, n)) / np.sqrt(n)).astype(np.float32)
    X = rng.standard_normal((batch, N)).astype(np.float32)
    Yref = np.zeros((batch, N), dtype=np.float32)
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = torch.zeros((batch, N), dtype=torch.float32, device="cuda")
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, torch.zeros_like(Yd), batch)
    assert blockwise_rel_err(host(Yd), Yref) <= F32_NORM_TOL
    check_status(kmx)


@pytest.mark.parametrize("form", FORMS)
def test_xbatched_index_pool_vs_oracle(kmx, oracle, form):
    """Pool layout of the benchmark, small: entries (y, x, a[d]) into shared
    X/Y block pools and per-dimension factor pools, uneven Y counts."""
    rng = np.random.default_rng(5)
    d, n, pool, nx, ny, ne = 6, 4, 64, 40, 30, 500
    N = n ** d
    lda = n
    Apool = rng.standard_normal((d, pool, n, n)) / 2
    Xpool = rng.standard_normal((nx, N))
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.geometric(0.2, ne) % ny
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    Yref = Y0.copy()
    oracle.xbatched_idx(d, n, Apool, lda, pool, Xpool, Yref, y_idx, x_idx, a_idx)
    Ad, Xd, Yd = dev(Apool), dev(Xpool), dev(Y0)
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    pY = kmx.pointer_array(Yd, y_idx * N)
    kmx.kronmult_xbatched(d, n, pA, lda, pX, pY, None, ne, form=form)
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("d,n", [(3, 4), (6, 3), (2, 8)])
def test_transpose_option(kmx, oracle, form, d, n):
    """transpose=True applies kron(A1^T, ..., Ad^T): the backward dX product."""
    rng = np.random.default_rng(9)
    N = n ** d
    batch = 3
    A = rng.standard_normal((batch, d, n, n))
    At = np.ascontiguousarray(np.swapaxes(A, 2, 3))
    X = rng.standard_normal((batch, N))
    Yref = np.zeros_like(X)
    oracle.batched(d, n, At, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = torch.zeros((batch, N), dtype=torch.float64, device="cuda")
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form=form, transpose=True)
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL


def test_vbatched_large_rectangular_uses_workspace(kmx, oracle):
    """d=5 with 8x7 factors: the entry exceeds shared memory, so the global
    workspace slots of the reference's vbatched layout are used."""
    rng = np.random.default_rng(11)
    d = 5
    m = [8, 7, 8, 7, 8]
    nn = [7, 8, 7, 8, 8]
    batch = 3
    Nx, Ny = int(np.prod(nn)), int(np.prod(m))
    fsz = [m[l] * nn[l] for l in range(d)]
    A = rng.standard_normal(batch * sum(fsz))
    X = rng.standard_normal((batch, Nx))
    offs, o = [], 0
    for b in range(batch):
        row = []
        for l in range(d):
            row.append(o)
            o += fsz[l]
        offs.append(row)
    Yref = np.zeros((batch, Ny))
    sxw = oracle.size_xw(d, m, nn)
    oracle.vbatched(d, m, nn, A, offs, X, [b * Nx for b in range(batch)], Yref,
                    [b * Ny for b in range(batch)], np.zeros(2 * sxw * batch))
    Ad, Xd = dev(A), dev(X)
    Yd = torch.zeros((batch, Ny), dtype=torch.float64, device="cuda")
    W = torch.zeros(2 * sxw * 2, dtype=torch.float64, device="cuda")  # two slots
    kmx.kronmult_vbatched(d, m, nn, kmx.pointer_array(Ad, np.ravel(offs)),
                          kmx.pointer_array(Xd, [b * Nx for b in range(batch)]),
                          kmx.pointer_array(Yd, [b * Ny for b in range(batch)]), W, None, batch)
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


# ---------------------------------------------------------------------------
# error behaviour
# ---------------------------------------------------------------------------

def test_null_entry_pointer_sets_device_status(kmx):
    """A NULL inside a device pointer array is skipped by the kernel and
    reported through the status word (no fault)."""
    d, n, batch = 3, 4, 4
    N = n ** d
    A = torch.rand((batch, d, n, n), dtype=torch.float64, device="cuda")
    X = torch.rand((batch, N), dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    pX = kmx.pointer_array(X, [b * N for b in range(batch)])
    pX[2] = 0
    pY = kmx.pointer_array(Y, [b * N for b in range(batch)])
    kmx.kronmult_pbatched(d, n, A, pX, pY, None, batch)
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()
    y = Y.cpu().numpy()
    assert not y[2].any() and y[0].any()
    assert kmx.check_device_status() == 0  # cleared


def test_missing_workspace_for_large_entry(kmx):
    """Entries beyond shared memory need the caller's W in the per-mode path
    (the reference's contract); the plain form keeps that path."""
    d, n, batch = 6, 7, 1
    N = n ** d
    A = torch.rand((batch, d, n, n), dtype=torch.float64, device="cuda")
    X = torch.rand((batch, N), dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    with pytest.raises(kmx.KmxError, match="WORKSPACE"):
        kmx.kronmult_batched(d, n, A, X, Y, None, batch, form="plain")


@pytest.mark.parametrize("d", [5, 6])
@pytest.mark.parametrize("layout", ["batched", "xbatched"])
def test_large_entries_vs_oracle(kmx, oracle, d, layout):
    """n = 8, d = 5 and 6 (256 KB and 2 MB FP64 blocks, beyond shared memory):
    the split form on the per-mode kernels with the intermediate in the
    caller's workspace, against the oracle, including overlapping Y blocks,
    padded lda and the transposed factors."""
    n = 8
    N = n ** d
    rng = np.random.default_rng(70 + d)
    if layout == "batched":
        batch = 3
        A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
        X = rng.standard_normal((batch, N))
        Y0 = rng.standard_normal((batch, N))
        Yref = Y0.copy()
        oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
        Yd = dev(Y0)
        W = torch.zeros((batch, N), dtype=torch.float64, device="cuda")
        kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, W, batch, form="split")
        assert blockwise_rel_err(host(Yd) - Y0, Yref - Y0) <= F64_TOL
        At = np.ascontiguousarray(np.swapaxes(A, 2, 3))
        Yref = np.zeros_like(X)
        oracle.batched(d, n, At, X.copy(), Yref, np.zeros_like(X), batch)
        Yd = torch.zeros((batch, N), dtype=torch.float64, device="cuda")
        kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, W, batch, form="split", transpose=True)
        assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    else:
        pool, nx, ny, ne, lda = 6, 3, 2, 5, n + 3
        Apool = np.zeros((d, pool, n, lda))
        Apool[..., :n] = rng.standard_normal((d, pool, n, n)) / np.sqrt(n)
        Xpool = rng.standard_normal((nx, N))
        Y0 = rng.standard_normal((ny, N))
        y_idx = np.array([0, 1, 0, 0, 1])  # overlapping Y blocks
        x_idx = rng.integers(0, nx, ne)
        a_idx = rng.integers(0, pool, (ne, d))
        Yref = Y0.copy()
        oracle.xbatched_idx(d, n, Apool, lda, pool, Xpool, Yref, y_idx, x_idx, a_idx)
        Ad, Xd, Yd = dev(Apool), dev(Xpool), dev(Y0)
        pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * lda).ravel())
        Wd = torch.zeros((2 * ne, N), dtype=torch.float64, device="cuda")  # 2 slots per sub-batch
        kmx.kronmult_xbatched(d, n, pA, lda, kmx.pointer_array(Xd, x_idx * N),
                              kmx.pointer_array(Yd, y_idx * N),
                              kmx.pointer_array(Wd, [k * N for k in range(2 * ne)]), ne, ne,
                              form="split")
        assert blockwise_rel_err(host(Yd) - Y0, Yref - Y0) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("form", ["split", "digits"])
@pytest.mark.parametrize("d,n", [(6, 4), (4, 8), (5, 3), (3, 5), (4, 4), (3, 16)])
def test_split_form_extreme_magnitudes(kmx, oracle, d, n, form):
    """Factors scaled by 1e-30..1e30 each and X by 1e-60..1e60 (products stay
    inside FP64 but far outside FP32): the split form rescales every entry by
    powers of two, so its FP32 carriers never overflow or flush."""
    rng = np.random.default_rng(21)
    N = n ** d
    batch = 4
    A = rng.standard_normal((batch, d, n, n))
    A *= 10.0 ** rng.integers(-30, 31, (batch, d, 1, 1))
    X = rng.standard_normal((batch, N)) * 10.0 ** rng.integers(-60, 61, (batch, 1))
    Yref = np.zeros_like(X)
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = torch.zeros((batch, N), dtype=torch.float64, device="cuda")
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form=form)
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("form", FORMS)
def test_nonfinite_inputs_propagate_like_fp64(kmx, oracle, form):
    """Inf/NaN in X or a factor propagate exactly as in FP64 arithmetic (the
    split form evaluates such entries with native FP64)."""
    rng = np.random.default_rng(22)
    d, n, batch = 6, 4, 4
    N = n ** d
    A = rng.standard_normal((batch, d, n, n))
    X = rng.standard_normal((batch, N))
    X[1, 77] = np.inf
    A[2, 3, 1, 2] = np.nan
    Yref = np.zeros_like(X)
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = torch.zeros((batch, N), dtype=torch.float64, device="cuda")
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form=form)
    y = host(Yd)
    assert np.array_equal(np.isnan(y), np.isnan(Yref))
    assert np.array_equal(np.isinf(y), np.isinf(Yref))
    fin = np.isfinite(Yref).all(axis=1)
    assert blockwise_rel_err(y[fin], Yref[fin]) <= F64_TOL


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("d,n", [(6, 4), (3, 8), (2, 16), (4, 5)])
def test_zero_factor_times_inf_is_nan(kmx, oracle, form, d, n):
    """An all-zero factor with an Inf in X gives NaN (0 * Inf), as in FP64: the
    split and digits forms must not take their all-zero shortcut first."""
    rng = np.random.default_rng(23)
    N = n ** d
    batch = 3
    A = rng.standard_normal((batch, d, n, n))
    X = rng.standard_normal((batch, N))
    A[1, d // 2] = 0.0
    X[1, N // 3] = np.inf
    A[2, 0] = 0.0  # all-zero factor, finite X: contributes exactly zero
    Y0 = rng.uniform(-1, 1, (batch, N))
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = dev(Y0)
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form=form)
    y = host(Yd)
    assert np.isnan(Yref[1]).any()
    assert np.array_equal(np.isnan(y), np.isnan(Yref))
    assert np.array_equal(np.isinf(y), np.isinf(Yref))
    assert np.array_equal(y[2], Y0[2])
    assert blockwise_rel_err(y[0:1], Yref[0:1]) <= F64_TOL


# ---------------------------------------------------------------------------
# deterministic (sorted-segment) accumulation
# ---------------------------------------------------------------------------

def _pool_case(seed, d, n, pool=48, nx=40, ny=25, ne=700, dtype=np.float64):
    rng = np.random.default_rng(seed)
    N = n ** d
    Apool = (rng.standard_normal((d, pool, n, n)) / 2).astype(dtype)
    Xpool = rng.standard_normal((nx, N)).astype(dtype)
    Y0 = rng.standard_normal((ny, N)).astype(dtype)
    y_idx = rng.geometric(0.15, ne) % ny
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    return Apool, Xpool, Y0, y_idx, x_idx, a_idx


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("d,n", [(6, 4), (4, 8), (5, 3), (3, 6)])
def test_deterministic_xbatched_vs_oracle_and_bitwise(kmx, oracle, form, d, n):
    Apool, Xpool, Y0, y_idx, x_idx, a_idx = _pool_case(31 + d + n, d, n)
    N = n ** d
    ne = len(y_idx)
    Yref = Y0.copy()
    oracle.xbatched_idx(d, n, Apool, n, Apool.shape[1], Xpool, Yref, y_idx, x_idx, a_idx)
    Ad, Xd = dev(Apool), dev(Xpool)
    pool = Apool.shape[1]
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    outs = []
    for _ in range(3):
        Yd = dev(Y0)
        pY = kmx.pointer_array(Yd, y_idx * N)
        kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, ne, form=form, accumulate="deterministic")
        outs.append(host(Yd))
    check_status(kmx)
    assert blockwise_rel_err(outs[0], Yref) <= F64_TOL
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_deterministic_f32_xbatched(kmx, oracle):
    d, n = 4, 8
    Apool, Xpool, Y0, y_idx, x_idx, a_idx = _pool_case(5, d, n, dtype=np.float32)
    N = n ** d
    ne = len(y_idx)
    Yref = Y0.astype(np.float64)
    oracle.xbatched_idx(d, n, Apool.astype(np.float64), n, Apool.shape[1], Xpool.astype(np.float64),
                        Yref, y_idx, x_idx, a_idx)
    Ad, Xd = dev(Apool), dev(Xpool)
    pool = Apool.shape[1]
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    outs = []
    for _ in range(2):
        Yd = dev(Y0)
        kmx.kronmult_xbatched(d, n, pA, n, pX, kmx.pointer_array(Yd, y_idx * N), None, ne,
                              dtype=torch.float32, accumulate="deterministic")
        outs.append(host(Yd))
    assert blockwise_rel_err(outs[0], Yref) <= 1e-5
    assert np.array_equal(outs[0], outs[1])
    check_status(kmx)


def test_deterministic_partial_overlap_is_refused(kmx):
    """Y blocks that overlap without coinciding cannot be owned by one group:
    the call writes nothing and reports KMX_ERR_OVERLAP (status bit 16)."""
    d, n, ne = 4, 4, 6
    N = n ** d
    A = torch.rand((ne * d * n * n,), dtype=torch.float64, device="cuda")
    X = torch.rand((ne, N), dtype=torch.float64, device="cuda")
    Y = torch.zeros(4 * N, dtype=torch.float64, device="cuda")
    pA = kmx.pointer_array(A, [i * n * n for i in range(ne * d)])
    pX = kmx.pointer_array(X, [b * N for b in range(ne)])
    pY = kmx.pointer_array(Y, [0, 0, N // 2, N, N, 2 * N])
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, ne, accumulate="deterministic")
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError) as ei:
        kmx.check_device_status()
    assert "DEVICE" in str(ei.value)
    assert not Y.any()


@pytest.mark.parametrize("form", ["auto", "plain", "split"])
@pytest.mark.parametrize("d,n", [(2, 4), (1, 7), (3, 9), (2, 13), (2, 8)])
def test_deterministic_shapes_without_tiled_segment_kernel(kmx, oracle, d, n, form):
    """Shapes without a register-tiled segment kernel (d <= 2, unspecialised n):
    the generic kernels walk whole Y segments, bitwise repeatable and equal to
    the oracle."""
    Apool, Xpool, Y0, y_idx, x_idx, a_idx = _pool_case(91 + d + n, d, n, pool=20, nx=16, ny=9,
                                                       ne=300)
    N = n ** d
    ne = len(y_idx)
    Yref = Y0.copy()
    oracle.xbatched_idx(d, n, Apool, n, Apool.shape[1], Xpool, Yref, y_idx, x_idx, a_idx)
    Ad, Xd = dev(Apool), dev(Xpool)
    pool = Apool.shape[1]
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    outs = []
    for _ in range(2):
        Yd = dev(Y0)
        pY = kmx.pointer_array(Yd, y_idx * N)
        kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, ne, form=form, accumulate="deterministic")
        outs.append(host(Yd))
    check_status(kmx)
    assert np.array_equal(outs[0], outs[1])
    assert blockwise_rel_err(outs[0], Yref) <= F64_TOL


# ---------------------------------------------------------------------------
# mixed shapes in one call, and CUDA-graph capture of repeated calls
# ---------------------------------------------------------------------------

def _mixed_case(kmx, seed, count, ns=(2, 3, 4, 5, 6, 8), dmax=6, cap=262144, dtype=np.float64):
    rng = np.random.default_rng(seed)
    dims = []
    while len(dims) < count:
        d = int(rng.integers(1, dmax + 1))
        n = int(rng.choice(ns))
        if n ** d <= cap:
            dims.append((d, n))
    dims = np.array(dims, dtype=np.int32)
    factors, xs, ys, a_off = [], [], [], []
    o = 0
    for d, n in dims:
        a_off.append(o)
        for _ in range(d):
            factors.append(rng.uniform(-1, 1, n * n).astype(dtype))
            o += 1
        xs.append(rng.uniform(-1, 1, n ** d).astype(dtype))
        ys.append(rng.uniform(-1, 1, n ** d).astype(dtype))
    # pack into flat device buffers
    fbuf = dev(np.concatenate(factors))
    foffs = np.cumsum([0] + [f.size for f in factors[:-1]])
    xbuf, ybuf = dev(np.concatenate(xs)), dev(np.concatenate(ys))
    xoffs = np.cumsum([0] + [x.size for x in xs[:-1]])
    pA = kmx.pointer_array(fbuf, foffs)
    pX = kmx.pointer_array(xbuf, xoffs)
    classes = sorted({(int(d), int(n)) for d, n in dims}, key=lambda c: -(c[1] ** (c[0] + 1) * c[0]))
    return dict(dims=dims, factors=factors, xs=xs, ys=ys, a_off=np.array(a_off), fbuf=fbuf,
                xbuf=xbuf, ybuf=ybuf, xoffs=xoffs, pA=pA, pX=pX, classes=classes)


def _mixed_reference(oracle, c):
    out = []
    fi = 0
    for i, (d, n) in enumerate(c["dims"]):
        fs = c["factors"][c["a_off"][i]: c["a_off"][i] + d]
        y = c["ys"][i].astype(np.float64).copy()
        oracle.kronmultv(int(d), [int(n)] * d, [int(n)] * d, [f.astype(np.float64) for f in fs],
                         [int(n)] * d, c["xs"][i].astype(np.float64), y)
        out.append(y)
    return out


@pytest.mark.parametrize("form", FORMS)
def test_mixed_shapes_one_call(kmx, oracle, form):
    c = _mixed_case(kmx, 41, 300)
    ybuf = c["ybuf"].clone()
    pY = kmx.pointer_array(ybuf, c["xoffs"])
    W = torch.empty(4 * 2 * 8 ** 6, dtype=torch.float64, device="cuda")  # 4 slots for 8^6 entries
    kmx.kronmult_mixed(dev(c["dims"]), c["pA"], dev(c["a_off"].astype(np.int64)), c["pX"], pY,
                       c["classes"], W, form=form)
    y = host(ybuf)
    ref = _mixed_reference(oracle, c)
    for i, r in enumerate(ref):
        seg = y[c["xoffs"][i]: c["xoffs"][i] + r.size]
        assert blockwise_rel_err(seg, r) <= F64_TOL, (i, c["dims"][i])
    check_status(kmx)


@pytest.mark.parametrize("form", ["auto", "split"])
def test_mixed_shapes_persistent_engine(kmx, oracle, form):
    """KMX_ENGINE_PERSISTENT: one launch over every class, instances popped
    from a device work queue, each run by the generic double-float kernel with
    its own (d, n) -- on chip or, for the 8^6 entries, in the workspace."""
    c = _mixed_case(kmx, 44, 300)
    ybuf = c["ybuf"].clone()
    pY = kmx.pointer_array(ybuf, c["xoffs"])
    W = torch.empty(8 * 2 * 8 ** 6, dtype=torch.float64, device="cuda")  # 8 slots for 8^6 entries
    kmx.read_redo_counters()
    kmx.kronmult_mixed(dev(c["dims"]), c["pA"], dev(c["a_off"].astype(np.int64)), c["pX"], pY,
                       c["classes"], W, form=form, engine="persistent")
    y = host(ybuf)
    ref = _mixed_reference(oracle, c)
    for i, r in enumerate(ref):
        seg = y[c["xoffs"][i]: c["xoffs"][i] + r.size]
        assert blockwise_rel_err(seg, r) <= F64_TOL, (i, c["dims"][i])
    check_status(kmx)


def test_mixed_persistent_engine_large_n(kmx, oracle):
    """Square classes the persistent kernel cannot apply in place (n > 16):
    (3, 20) holds one buffer on chip but runs out of place, so it takes the
    workspace; (2, 24) keeps two buffers on chip; (4, 3) is small."""
    c = _mixed_case(kmx, 46, 60, ns=(20, 24, 3), dmax=4, cap=8000)
    assert {(3, 20), (2, 24)} <= set(c["classes"])
    ybuf = c["ybuf"].clone()
    pY = kmx.pointer_array(ybuf, c["xoffs"])
    W = torch.empty(16 * 2 * 8000, dtype=torch.float64, device="cuda")  # 16 slots
    kmx.kronmult_mixed(dev(c["dims"]), c["pA"], dev(c["a_off"].astype(np.int64)), c["pX"], pY,
                       c["classes"], W, engine="persistent")
    y = host(ybuf)
    ref = _mixed_reference(oracle, c)
    for i, r in enumerate(ref):
        seg = y[c["xoffs"][i]: c["xoffs"][i] + r.size]
        assert blockwise_rel_err(seg, r) <= F64_TOL, (i, c["dims"][i])
    check_status(kmx)


def test_mixed_unknown_class_is_flagged(kmx):
    c = _mixed_case(kmx, 42, 20, ns=(2, 3), dmax=3)
    ybuf = c["ybuf"].clone()
    pY = kmx.pointer_array(ybuf, c["xoffs"])
    kmx.kronmult_mixed(dev(c["dims"]), c["pA"], dev(c["a_off"].astype(np.int64)), c["pX"], pY,
                       c["classes"][:-1])
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()


def test_cuda_graph_of_repeated_mixed_calls(kmx, oracle):
    """A sequence of calls captured once as a CUDA graph and replayed gives the
    same result as the eager calls (one warm-up call first)."""
    c = _mixed_case(kmx, 43, 120, dmax=5)
    dims_d, aoff_d = dev(c["dims"]), dev(c["a_off"].astype(np.int64))
    reps = 10
    y_eager = c["ybuf"].clone()
    pY_e = kmx.pointer_array(y_eager, c["xoffs"])
    y_graph = c["ybuf"].clone()
    pY_g = kmx.pointer_array(y_graph, c["xoffs"])
    W = torch.empty(2 * 8 ** 5 * 4, dtype=torch.float64, device="cuda")
    # warm-up (caches workspaces and kernel attributes), then undo it
    kmx.kronmult_mixed(dims_d, c["pA"], aoff_d, c["pX"], pY_g, c["classes"], W, form="split")
    torch.cuda.synchronize()
    y_graph.copy_(c["ybuf"])
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            for _ in range(reps):
                kmx.kronmult_mixed(dims_d, c["pA"], aoff_d, c["pX"], pY_g, c["classes"], W,
                                   form="split", stream=s)
    torch.cuda.current_stream().wait_stream(s)
    g.replay()
    for _ in range(reps):
        kmx.kronmult_mixed(dims_d, c["pA"], aoff_d, c["pX"], pY_e, c["classes"], W, form="split")
    torch.cuda.synchronize()
    assert blockwise_rel_err(host(y_graph), host(y_eager)) <= 1e-12
    check_status(kmx)


# ---------------------------------------------------------------------------
# FP32 / BF16 storage with FP64 accumulation into shared Y blocks
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("in_dtype", ["f32", "bf16"])
@pytest.mark.parametrize("d,n", [(4, 8), (3, 16), (6, 4), (3, 5)])
@pytest.mark.parametrize("acc", ["atomic", "deterministic"])
def test_wide_forms_vs_fp64_oracle(kmx, oracle, in_dtype, d, n, acc):
    """The FP64 oracle runs on the same (rounded) inputs, so the error measures
    the FP32 arithmetic only; FP64 Y accumulation keeps it at FP32 level."""
    rng = np.random.default_rng(61 + d * n)
    pool, nx, ny, ne = 40, 30, 12, 400
    N = n ** d
    tdt = torch.float32 if in_dtype == "f32" else torch.bfloat16
    Apool = torch.from_numpy(rng.standard_normal((d, pool, n, n)) / np.sqrt(n)).to(tdt).cuda()
    Xpool = torch.from_numpy(rng.standard_normal((nx, N))).to(tdt).cuda()
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.geometric(1 / 16, ne) % ny
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    Yref = Y0.copy()
    oracle.xbatched_idx(d, n, Apool.double().cpu().numpy(), n, pool, Xpool.double().cpu().numpy(),
                        Yref, y_idx, x_idx, a_idx)
    esz = Apool.element_size()
    pA = kmx.pointer_array(Apool, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel(), esz)
    pX = kmx.pointer_array(Xpool, x_idx * N, esz)
    Yd = dev(Y0)
    pY = kmx.pointer_array(Yd, y_idx * N)
    kmx.kronmult_xbatched_wide(d, n, pA, n, pX, pY, ne, in_dtype=in_dtype, accumulate=acc)
    err = blockwise_rel_err(host(Yd), Yref)
    assert err <= 2e-6, err
    check_status(kmx)


@pytest.mark.parametrize("form,acc", [("auto", "atomic"), ("digits", "atomic"),
                                      ("auto", "deterministic")])
def test_xbatched_cuda_graph_replay(kmx, form, acc):
    """The xbatched call makes no host synchronisation in any form (the
    digits form's second pass reads its count on the device; the
    deterministic mode sorts on the device): after one warm-up call it
    captures into a CUDA graph, and each replay adds the same contribution."""
    rng = np.random.default_rng(33)
    d, n, pool, nb, ne = 6, 4, 32, 24, 200
    N = n ** d
    Apool = dev(rng.standard_normal((d, pool, n, n)) / 2)
    Xpool = dev(rng.standard_normal((nb, N)))
    y_idx = rng.geometric(0.2, ne) % nb
    x_idx = rng.integers(0, nb, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    pA = kmx.pointer_array(Apool, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xpool, x_idx * N)
    Y = torch.zeros((nb, N), dtype=torch.float64, device="cuda")
    pY = kmx.pointer_array(Y, y_idx * N)
    s = torch.cuda.Stream()
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, ne, form=form, accumulate=acc, stream=s)
    s.synchronize()
    once = Y.clone()
    Y.zero_()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, ne, form=form, accumulate=acc, stream=s)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    assert blockwise_rel_err(host(Y), 2 * host(once)) <= F64_TOL
