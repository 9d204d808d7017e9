"""GPU parity of the FP64 digits form (KMX_FORM_DIGITS: X and factors as
base-2^9 digits with one exponent per entry, exact FP16 tensor-core digit
products, exact FP32 level sums) against the FP64 oracle, including the
entries it hands to the double-float pass (results far below the entry's
scale, Inf/NaN).  Every call goes through the C ABI.  Tolerance: normwise
relative error per Y block <= 1e-13."""
import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F64_TOL = 1e-13
DIGIT_SHAPES = [(6, 4), (4, 4), (3, 16), (2, 16)]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _pool_run(kmx, oracle, d, n, Apool, Xpool, Y0, y_idx, x_idx, a_idx, form="digits"):
    pool = Apool.shape[1]
    N = n ** d
    Yref = Y0.copy()
    oracle.xbatched_idx(d, n, Apool, n, pool, Xpool, Yref, y_idx, x_idx, a_idx)
    Ad, Xd = torch.from_numpy(Apool).cuda(), torch.from_numpy(Xpool).cuda()
    Yd = torch.from_numpy(Y0.copy()).cuda()
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    pY = kmx.pointer_array(Yd, y_idx * N)
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, len(y_idx), form=form)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    return Yd.cpu().numpy(), Yref


@pytest.mark.parametrize("d,n", DIGIT_SHAPES)
@pytest.mark.parametrize("dist", ["normal", "uniform", "wide"])
def test_digits_xbatched_vs_oracle(kmx, oracle, d, n, dist):
    rng = np.random.default_rng(300 + 10 * d + n)
    pool, nx, ny, ne = 32, 24, 10, 300
    N = n ** d
    if dist == "normal":
        Apool = rng.standard_normal((d, pool, n, n)) / 2
        Xpool = rng.standard_normal((nx, N))
    elif dist == "uniform":
        Apool = rng.uniform(-1, 1, (d, pool, n, n))
        Xpool = rng.uniform(-1, 1, (nx, N))
    else:  # element magnitudes spread over six decades
        Apool = rng.standard_normal((d, pool, n, n)) * 10.0 ** rng.uniform(-3, 3, (d, pool, n, n))
        Xpool = rng.standard_normal((nx, N)) * 10.0 ** rng.uniform(-3, 3, (nx, N))
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.geometric(1 / 8, ne) % ny
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    y, yref = _pool_run(kmx, oracle, d, n, Apool, Xpool, Y0, y_idx, x_idx, a_idx)
    assert blockwise_rel_err(y - Y0, yref - Y0) <= F64_TOL


@pytest.mark.parametrize("d,n", [(6, 4), (3, 16)])
def test_digits_cancellation_goes_to_double_float(kmx, oracle, d, n):
    """Entries whose result cancels -- factors whose ROWS sum to zero (with
    column-major storage A[l, p, j, i] = A_l(i, j) that is the sum over axis
    2) applied to X = 1 + 1e-2 Z, which kron(...) nearly annihilates -- are
    handed to the double-float pass (counted on the device) and recomputed
    there in FP64 by its cancellation guard; mixed with ordinary entries on
    shared Y blocks.  Against the recursion in extended precision: within
    1e-13 per Y block, as plain FP64 is on the same data."""
    rng = np.random.default_rng(41)
    pool, nx, ny, ne = 16, 12, 6, 120
    N = n ** d
    Apool = rng.standard_normal((d, pool, n, n)) / 2
    # half of the factor pool: zero row sums -> kron(...) annihilates constants
    Apool[:, : pool // 2] -= Apool[:, : pool // 2].mean(axis=2, keepdims=True)
    Xpool = 1.0 + 1e-2 * rng.standard_normal((nx, N))
    y_idx = rng.integers(0, ny, ne)
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    cancels = np.any(a_idx < pool // 2, axis=1)  # one zero-row-sum factor suffices
    Yx = oracle.xbatched_idx_extended(d, n, Apool, Xpool, ny, y_idx, x_idx, a_idx)
    Yx = Yx.astype(np.float64)
    Ad, Xd = torch.from_numpy(Apool).cuda(), torch.from_numpy(Xpool).cuda()
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xd, x_idx * N)
    out = {}
    for form in ("plain", "digits"):
        Yd = torch.zeros((ny, N), dtype=torch.float64, device="cuda")
        kmx.read_redo_counters()
        kmx.kronmult_xbatched(d, n, pA, n, pX, kmx.pointer_array(Yd, y_idx * N), None, ne,
                              form=form)
        torch.cuda.synchronize()
        assert kmx.check_device_status() == 0
        out[form] = (Yd.cpu().numpy(), kmx.read_redo_counters())
    assert blockwise_rel_err(out["plain"][0], Yx) <= F64_TOL
    y, (guard, handback) = out["digits"]
    assert handback >= int(cancels.sum())
    assert guard >= int(cancels.sum())
    assert blockwise_rel_err(y, Yx) <= F64_TOL


def test_digits_zero_blocks_contribute_nothing(kmx, oracle):
    d, n = 6, 4
    rng = np.random.default_rng(5)
    pool, nx, ny, ne = 8, 6, 4, 40
    N = n ** d
    Apool = rng.standard_normal((d, pool, n, n))
    Apool[2, 0] = 0.0               # an all-zero factor
    Xpool = rng.standard_normal((nx, N))
    Xpool[0] = 0.0                  # an all-zero X block
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.integers(0, ny, ne)
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    y, yref = _pool_run(kmx, oracle, d, n, Apool, Xpool, Y0, y_idx, x_idx, a_idx)
    assert blockwise_rel_err(y, yref) <= F64_TOL


def test_digits_matches_plain_on_benchmark_sample(kmx):
    """A slice of the benchmark's workload (xbatched d=6 n=4, N(0,1)/2 factor
    pool, N(0,1) X pool, geometric Y counts): digits vs plain FP64."""
    rng = np.random.default_rng(20261203)
    d, n, pool, nb, ne = 6, 4, 1024, 512, 8192
    N = n ** d
    Apool = torch.from_numpy(rng.standard_normal((d, pool, n, n)) / 2).cuda()
    Xpool = torch.from_numpy(rng.standard_normal((nb, N))).cuda()
    y_idx = np.repeat(np.arange(nb), rng.geometric(1 / 16, nb))[:ne]
    y_idx = np.concatenate([y_idx, rng.integers(0, nb, ne - len(y_idx))]) if len(y_idx) < ne else y_idx
    x_idx = rng.integers(0, nb, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    pA = kmx.pointer_array(Apool, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    pX = kmx.pointer_array(Xpool, x_idx * N)
    out = {}
    for form in ("plain", "digits"):
        Y = torch.zeros((nb, N), dtype=torch.float64, device="cuda")
        kmx.kronmult_xbatched(d, n, pA, n, pX, kmx.pointer_array(Y, y_idx * N), None, ne, form=form)
        out[form] = Y
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    num = torch.linalg.vector_norm(out["digits"] - out["plain"], dim=1)
    den = torch.linalg.vector_norm(out["plain"], dim=1).clamp_min(1e-300)
    assert float((num / den).max()) <= F64_TOL
