"""GPU parity of the tensor-core form (KMX_FORM_TF32X3: mma.sync TF32, each
operand split into two TF32 parts, three products, FP32 accumulation) for
FP32- and BF16-stored data, against the FP64 oracle on the same (rounded)
inputs.  Every call goes through the C ABI.

Tolerance: normwise relative error per Y block <= 5e-6 (the scheme's
per-product error is about 2^-21; the FP32-FMA form of the same data reaches
about 2e-7)."""
import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TC_TOL = 5e-6
TC_SHAPES = [(4, 4), (6, 4), (3, 8), (4, 8), (5, 8), (2, 16), (3, 16)]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _case(rng, d, n, pool=24, nx=20, ny=9, ne=160):
    N = n ** d
    A = rng.standard_normal((d, pool, n, n)) / np.sqrt(n)
    X = rng.standard_normal((nx, N))
    Y0 = rng.standard_normal((ny, N))
    y_idx = rng.geometric(1 / 8, ne) % ny
    x_idx = rng.integers(0, nx, ne)
    a_idx = rng.integers(0, pool, (ne, d))
    return A, X, Y0, y_idx, x_idx, a_idx


def _pointers(kmx, Ad, Xd, Yd, y_idx, x_idx, a_idx, d, n, pool):
    N = n ** d
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel())
    return pA, kmx.pointer_array(Xd, x_idx * N), kmx.pointer_array(Yd, y_idx * N)


@pytest.mark.parametrize("d,n", TC_SHAPES)
@pytest.mark.parametrize("transpose", [False, True])
def test_tf32x3_f32_entry_point(kmx, oracle, d, n, transpose):
    """FP32 X, factors and Y (kmx_kronmult_xbatched_f32 with form TF32X3)."""
    rng = np.random.default_rng(100 + 10 * d + n)
    A, X, Y0, y_idx, x_idx, a_idx = _case(rng, d, n)
    pool = A.shape[1]
    A32, X32, Y32 = A.astype(np.float32), X.astype(np.float32), Y0.astype(np.float32)
    At = A32.transpose(0, 1, 3, 2).copy() if transpose else A32  # oracle gets A^T explicitly
    Yref = Y32.astype(np.float64)
    oracle.xbatched_idx(d, n, At.astype(np.float64), n, pool, X32.astype(np.float64), Yref,
                        y_idx, x_idx, a_idx)
    Ad, Xd, Yd = (torch.from_numpy(v).cuda() for v in (A32, X32, Y32.copy()))
    pA, pX, pY = _pointers(kmx, Ad, Xd, Yd, y_idx, x_idx, a_idx, d, n, pool)
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, len(y_idx), dtype=torch.float32,
                          form="tf32x3", transpose=transpose)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    # the reference starts from the FP32 Y0; compare the accumulated part
    err = blockwise_rel_err(Yd.cpu().numpy().astype(np.float64) - Y32, Yref - Y32)
    assert err <= TC_TOL, err


@pytest.mark.parametrize("d,n", TC_SHAPES)
@pytest.mark.parametrize("in_dtype", ["f32", "bf16"])
def test_tf32x3_wide_fp64_y(kmx, oracle, d, n, in_dtype):
    """FP32/BF16 X and factors, FP64 Y (kmx_kronmult_xbatched_wide, TF32X3)."""
    rng = np.random.default_rng(200 + 10 * d + n)
    A, X, Y0, y_idx, x_idx, a_idx = _case(rng, d, n)
    pool = A.shape[1]
    tdt = torch.float32 if in_dtype == "f32" else torch.bfloat16
    Ad = torch.from_numpy(A).to(tdt).cuda()
    Xd = torch.from_numpy(X).to(tdt).cuda()
    Yref = Y0.copy()
    oracle.xbatched_idx(d, n, Ad.double().cpu().numpy(), n, pool, Xd.double().cpu().numpy(), Yref,
                        y_idx, x_idx, a_idx)
    Yd = torch.from_numpy(Y0.copy()).cuda()
    N = n ** d
    esz = Ad.element_size()
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel(), esz)
    pX = kmx.pointer_array(Xd, x_idx * N, esz)
    pY = kmx.pointer_array(Yd, y_idx * N)
    kmx.kronmult_xbatched_wide(d, n, pA, n, pX, pY, len(y_idx), in_dtype=in_dtype, form="tf32x3")
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    err = blockwise_rel_err(Yd.cpu().numpy() - Y0, Yref - Y0)
    assert err <= TC_TOL, err


def test_tf32x3_unsupported_shape_uses_fp32_fma(kmx, oracle):
    """Shapes without a tensor-core kernel (here d=3, n=5) run the FP32-FMA
    kernels; the result is the same to FP32 accuracy."""
    d, n = 3, 5
    rng = np.random.default_rng(7)
    A, X, Y0, y_idx, x_idx, a_idx = _case(rng, d, n)
    pool = A.shape[1]
    A32, X32 = A.astype(np.float32), X.astype(np.float32)
    Yref = np.zeros_like(Y0)
    oracle.xbatched_idx(d, n, A32.astype(np.float64), n, pool, X32.astype(np.float64), Yref,
                        y_idx, x_idx, a_idx)
    Ad, Xd = torch.from_numpy(A32).cuda(), torch.from_numpy(X32).cuda()
    Yd = torch.zeros(Y0.shape, dtype=torch.float32, device="cuda")
    pA, pX, pY = _pointers(kmx, Ad, Xd, Yd, y_idx, x_idx, a_idx, d, n, pool)
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, len(y_idx), dtype=torch.float32,
                          form="tf32x3")
    torch.cuda.synchronize()
    assert blockwise_rel_err(Yd.cpu().numpy().astype(np.float64), Yref) <= 2e-6


def test_tf32x3_null_entry_flagged(kmx):
    d, n, ne = 4, 8, 6
    N = n ** d
    A = torch.rand((ne, d, n, n), dtype=torch.float32, device="cuda")
    X = torch.rand((ne, N), dtype=torch.float32, device="cuda")
    Y = torch.zeros_like(X)
    pA = kmx.pointer_array(A, [e * d * n * n + l * n * n for e in range(ne) for l in range(d)])
    pX = kmx.pointer_array(X, [e * N for e in range(ne)])
    pY = kmx.pointer_array(Y, [e * N for e in range(ne)])
    pX[3] = 0
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, ne, dtype=torch.float32, form="tf32x3")
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()
    y = Y.cpu().numpy()
    assert not y[3].any() and y[0].any() and y[5].any()


@pytest.mark.parametrize("d,n", [s for s in TC_SHAPES if s != (5, 8) and s[0] >= 3])
@pytest.mark.parametrize("in_dtype", ["f32", "bf16"])
def test_tf32x3_deterministic_segments(kmx, oracle, d, n, in_dtype):
    """Deterministic mode: entries grouped by Y block, each block's
    contributions summed in a fixed order in registers and written once;
    bitwise identical across calls.  (The deterministic mode takes d >= 3.)"""
    rng = np.random.default_rng(400 + 10 * d + n)
    A, X, Y0, y_idx, x_idx, a_idx = _case(rng, d, n)
    pool = A.shape[1]
    tdt = torch.float32 if in_dtype == "f32" else torch.bfloat16
    Ad = torch.from_numpy(A).to(tdt).cuda()
    Xd = torch.from_numpy(X).to(tdt).cuda()
    Yref = Y0.copy()
    oracle.xbatched_idx(d, n, Ad.double().cpu().numpy(), n, pool, Xd.double().cpu().numpy(), Yref,
                        y_idx, x_idx, a_idx)
    N = n ** d
    esz = Ad.element_size()
    pA = kmx.pointer_array(Ad, ((np.arange(d)[None, :] * pool + a_idx) * n * n).ravel(), esz)
    pX = kmx.pointer_array(Xd, x_idx * N, esz)
    outs = []
    for _ in range(2):
        Yd = torch.from_numpy(Y0.copy()).cuda()
        kmx.kronmult_xbatched_wide(d, n, pA, n, pX, kmx.pointer_array(Yd, y_idx * N), len(y_idx),
                                   in_dtype=in_dtype, form="tf32x3", accumulate="deterministic")
        outs.append(Yd)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    assert torch.equal(outs[0], outs[1])
    err = blockwise_rel_err(outs[0].cpu().numpy() - Y0, Yref - Y0)
    assert err <= TC_TOL, err


def test_tf32x3_deterministic_f32_entry_point(kmx, oracle):
    d, n = 4, 8
    rng = np.random.default_rng(9)
    A, X, Y0, y_idx, x_idx, a_idx = _case(rng, d, n)
    pool = A.shape[1]
    A32, X32, Y32 = A.astype(np.float32), X.astype(np.float32), Y0.astype(np.float32)
    Yref = Y32.astype(np.float64)
    oracle.xbatched_idx(d, n, A32.astype(np.float64), n, pool, X32.astype(np.float64), Yref,
                        y_idx, x_idx, a_idx)
    Ad, Xd, Yd = (torch.from_numpy(v).cuda() for v in (A32, X32, Y32.copy()))
    pA, pX, pY = _pointers(kmx, Ad, Xd, Yd, y_idx, x_idx, a_idx, d, n, pool)
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, len(y_idx), dtype=torch.float32,
                          form="tf32x3", accumulate="deterministic")
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    err = blockwise_rel_err(Yd.cpu().numpy().astype(np.float64) - Y32, Yref - Y32)
    assert err <= TC_TOL, err


def test_tf32x3_deterministic_without_segment_kernel(kmx):
    """d=5, n=8 (32768-element blocks) has no segment kernel in any form: the
    deterministic request is refused before any launch."""
    d, n = 5, 8
    A = torch.zeros((1, d, n, n), dtype=torch.float32, device="cuda")
    X = torch.zeros((1, n ** d), dtype=torch.float32, device="cuda")
    Y = torch.zeros((1, n ** d), dtype=torch.float64, device="cuda")
    pA = kmx.pointer_array(A, [l * n * n for l in range(d)])
    with pytest.raises(kmx.KmxError, match="UNSUPPORTED"):
        kmx.kronmult_xbatched_wide(d, n, pA, n, kmx.pointer_array(X, [0]),
                                   kmx.pointer_array(Y, [0]), 1, form="tf32x3",
                                   accumulate="deterministic")
