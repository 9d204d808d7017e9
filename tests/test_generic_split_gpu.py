"""GPU parity of the generic split (double-float) kernel: rectangular factors
(the reference's vbatched, kronmult_vbatched.hpp:19-248) and square n without
a compile-time specialisation, against the oracle.  Every call goes through
the C ABI.

Tolerance: normwise relative error per Y block <= 1e-13 (FP64 forms).
"""
import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F64_TOL = 1e-13


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


def kernels_of(fn):
    """Names of the CUDA kernels fn launches (None when the profiler sees no
    device activity on this build of torch)."""
    from torch.profiler import ProfilerActivity, profile

    torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        fn()
        torch.cuda.synchronize()
    names = [e.name for e in prof.events() if e.device_type == torch.autograd.DeviceType.CUDA]
    return names or None


def vb_case(seed, d, m, nn, batch, scale_exp=0, y0=True):
    rng = np.random.default_rng(seed)
    Nx, Ny = int(np.prod(nn)), int(np.prod(m))
    fsz = [m[l] * nn[l] for l in range(d)]
    A = rng.standard_normal(batch * sum(fsz))
    offs, o = [], 0
    for b in range(batch):
        for l in range(d):
            if scale_exp:
                A[o:o + fsz[l]] *= 10.0 ** rng.integers(-scale_exp, scale_exp + 1)
            offs.append(o)
            o += fsz[l]
    X = rng.standard_normal((batch, Nx))
    if scale_exp:
        X *= 10.0 ** rng.integers(-2 * scale_exp, 2 * scale_exp + 1, (batch, 1))
    Y0 = rng.uniform(-1, 1, (batch, Ny)) if y0 else np.zeros((batch, Ny))
    return A, offs, X, Y0


def run_vb(kmx, oracle, d, m, nn, A, offs, X, Y0, form, wslots=None):
    batch, Nx = X.shape
    Ny = Y0.shape[1]
    sxw = oracle.size_xw(d, m, nn)
    Yref = Y0.copy()
    oracle.vbatched(d, m, nn, A, offs, X, [b * Nx for b in range(batch)], Yref,
                    [b * Ny for b in range(batch)], np.zeros(2 * sxw * batch))
    Ad, Xd, Yd = dev(A), dev(X), dev(Y0)
    nslots = batch if wslots is None else wslots
    W = torch.zeros(2 * sxw * nslots, dtype=torch.float64, device="cuda")

    def call():
        kmx.kronmult_vbatched(d, m, nn, kmx.pointer_array(Ad, offs),
                              kmx.pointer_array(Xd, [b * Nx for b in range(batch)]),
                              kmx.pointer_array(Yd, [b * Ny for b in range(batch)]), W, None,
                              batch, form=form)

    return call, Yd, Yref


RECT = [
    (1, [5], [3]),
    (2, [3, 7], [6, 2]),
    (3, [4, 5, 6], [6, 5, 4]),
    (3, [2, 9, 3], [9, 2, 9]),
    (4, [3, 4, 3, 4], [4, 3, 4, 3]),
    (5, [2, 3, 4, 3, 2], [3, 2, 3, 4, 3]),
    (6, [4, 3, 4, 3, 4, 3], [3, 4, 3, 4, 3, 4]),
    (6, [2, 2, 3, 3, 2, 2], [3, 3, 2, 2, 3, 3]),
    (4, [17, 5, 17, 5], [5, 17, 5, 17]),
]


@pytest.mark.parametrize("d,m,nn", RECT)
def test_generic_split_rectangular_vs_oracle(kmx, oracle, d, m, nn):
    """Rectangular factors in double-float, accumulated into a nonzero Y."""
    A, offs, X, Y0 = vb_case(31 + d, d, m, nn, batch=6)
    call, Yd, Yref = run_vb(kmx, oracle, d, m, nn, A, offs, X, Y0, "split")
    names = kernels_of(call)
    if names is not None:
        assert any("gen_split_kernel" in k for k in names), names
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("d,n", [(3, 9), (4, 11), (2, 13), (3, 17), (2, 20), (3, 1), (4, 10)])
def test_generic_split_unspecialised_square_vs_oracle(kmx, oracle, d, n):
    """Square n without a compiled specialisation: n <= 16 runs in place, n > 16
    through the second buffer."""
    rng = np.random.default_rng(100 * d + n)
    N = n ** d
    batch = 4
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    Y0 = rng.uniform(-1, 1, (batch, N))
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Xd, Yd, Ad = dev(X), dev(Y0), dev(A)

    def call():
        kmx.kronmult_batched(d, n, Ad, Xd, Yd, None, batch, form="split")

    names = kernels_of(call)
    if names is not None:
        assert any("gen_split_kernel" in k for k in names), names
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


def test_generic_split_global_workspace(kmx, oracle):
    """d=5 with 8x7 / 7x8 factors: one entry exceeds shared memory, so the
    split kernel keeps its pairs in the caller's workspace slots (two slots
    for three entries: slots are reused)."""
    d, m, nn = 5, [8, 7, 8, 7, 8], [7, 8, 7, 8, 8]
    A, offs, X, Y0 = vb_case(41, d, m, nn, batch=3)
    call, Yd, Yref = run_vb(kmx, oracle, d, m, nn, A, offs, X, Y0, "split", wslots=2)
    names = kernels_of(call)
    if names is not None:
        assert any("gen_split_kernel" in k for k in names), names
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("d,m,nn", [RECT[2], RECT[6], RECT[8]])
def test_generic_split_extreme_magnitudes(kmx, oracle, d, m, nn):
    """Factors scaled by 1e-30..1e30 and X by 1e-60..1e60: per-entry power-of-
    two scaling keeps the FP32 carriers in range."""
    A, offs, X, _ = vb_case(51, d, m, nn, batch=5, scale_exp=30, y0=False)
    Y0 = np.zeros((X.shape[0], int(np.prod(m))))
    call, Yd, Yref = run_vb(kmx, oracle, d, m, nn, A, offs, X, Y0, "split")
    call()
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


def test_generic_split_nonfinite_like_fp64(kmx, oracle):
    """Inf/NaN in X or a factor: those entries run the FP64 arithmetic, so
    Inf/NaN land where FP64 puts them; the other entries stay in tolerance."""
    d, m, nn = 4, [3, 4, 3, 4], [4, 3, 4, 3]
    A, offs, X, _ = vb_case(61, d, m, nn, batch=4, y0=False)
    X[1, 17] = np.inf
    A[offs[2 * d + 2] + 3] = np.nan
    # entry 3: an all-zero factor times an Inf in X gives NaN, as in FP64
    A[offs[3 * d + 1]:offs[3 * d + 1] + m[1] * nn[1]] = 0.0
    X[3, 5] = -np.inf
    Y0 = np.zeros((4, int(np.prod(m))))
    call, Yd, Yref = run_vb(kmx, oracle, d, m, nn, A, offs, X, Y0, "split")
    call()
    y = host(Yd)
    assert np.isnan(Yref[3]).any()
    assert np.array_equal(np.isnan(y), np.isnan(Yref))
    assert np.array_equal(np.isinf(y), np.isinf(Yref))
    fin = np.isfinite(Yref).all(axis=1)
    assert fin.sum() == 1
    assert blockwise_rel_err(y[fin], Yref[fin]) <= F64_TOL
    check_status(kmx)


def test_generic_split_zero_factor_adds_nothing(kmx, oracle):
    """An all-zero factor or X block contributes exactly zero (Y unchanged)."""
    d, m, nn = 3, [4, 5, 6], [6, 5, 4]
    A, offs, X, Y0 = vb_case(71, d, m, nn, batch=3)
    A[offs[1]:offs[1] + m[1] * nn[1]] = 0.0  # entry 0, factor 1
    X[2] = 0.0
    call, Yd, Yref = run_vb(kmx, oracle, d, m, nn, A, offs, X, Y0, "split")
    call()
    y = host(Yd)
    assert np.array_equal(y[0], Y0[0]) and np.array_equal(y[2], Y0[2])
    assert blockwise_rel_err(y[1:2], Yref[1:2]) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("d,m,nn,kernel", [
    (3, [10, 12, 10], [12, 10, 12], "gen_split_kernel"),
    (2, [32, 24], [24, 32], "gen_split_kernel"),
    (2, [6, 7], [7, 6], "gen_plain_kernel"),
])
def test_auto_form_for_generic_shapes(kmx, oracle, d, m, nn, kernel):
    """The automatic form takes double-float for entries of 512 or more
    elements and FP64 below (where the per-entry scaling costs more)."""
    A, offs, X, Y0 = vb_case(81, d, m, nn, batch=4)
    call, Yd, Yref = run_vb(kmx, oracle, d, m, nn, A, offs, X, Y0, None)
    names = kernels_of(call)
    if names is not None:
        assert any(kernel in k for k in names), names
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("form", ["split", "plain"])
@pytest.mark.parametrize("d,m,nn", [RECT[2], RECT[5], RECT[8]])
def test_generic_transpose_option_rectangular(kmx, oracle, d, m, nn, form):
    """transpose=True applies A_l^T (n_l x m_l) from factors stored m_l x n_l:
    checked against the oracle on the explicitly transposed factors."""
    rng = np.random.default_rng(91 + d)
    batch = 4
    # applied operator l is n_l x m_l: X blocks have prod(m) elements, Y blocks prod(n)
    Nx, Ny = int(np.prod(m)), int(np.prod(nn))
    fsz = [m[l] * nn[l] for l in range(d)]
    F = rng.standard_normal(batch * sum(fsz))          # stored m_l x n_l, column-major
    G = np.empty_like(F)                               # the transposes, n_l x m_l
    offs, o = [], 0
    for b in range(batch):
        for l in range(d):
            blk = F[o:o + fsz[l]].reshape(nn[l], m[l]).T   # (m_l, n_l) matrix
            G[o:o + fsz[l]] = blk.T.reshape(-1, order="F")
            offs.append(o)
            o += fsz[l]
    X = rng.standard_normal((batch, Nx))
    Y0 = rng.uniform(-1, 1, (batch, Ny))
    Yref = Y0.copy()
    sxw = oracle.size_xw(d, nn, m)
    oracle.vbatched(d, nn, m, G, offs, X, [b * Nx for b in range(batch)], Yref,
                    [b * Ny for b in range(batch)], np.zeros(2 * sxw * batch))
    Fd, Xd, Yd = dev(F), dev(X), dev(Y0)
    W = torch.zeros(2 * sxw * batch, dtype=torch.float64, device="cuda")
    kmx.kronmult_vbatched(d, m, nn, kmx.pointer_array(Fd, offs),
                          kmx.pointer_array(Xd, [b * Nx for b in range(batch)]),
                          kmx.pointer_array(Yd, [b * Ny for b in range(batch)]), W, None, batch,
                          form=form, transpose=True)
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("d,n", [(3, 9), (4, 10), (2, 20)])
def test_generic_split_transpose_option_square(kmx, oracle, d, n):
    """transpose=True on square unspecialised n against the oracle on A^T."""
    rng = np.random.default_rng(95 + n)
    N = n ** d
    batch = 3
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    Y0 = rng.uniform(-1, 1, (batch, N))
    Yref = Y0.copy()
    oracle.batched(d, n, np.ascontiguousarray(np.swapaxes(A, 2, 3)), X.copy(), Yref,
                   np.zeros_like(X), batch)
    Yd = dev(Y0)
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None, batch, form="split", transpose=True)
    assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL
    check_status(kmx)


@pytest.mark.parametrize("form", [None, "plain"])
@pytest.mark.parametrize("d,m,nn,wslots", [
    (3, [4, 5, 6], [6, 5, 4], None),
    (6, [4, 3, 4, 3, 4, 3], [3, 4, 3, 4, 3, 4], None),
    (2, [32, 24], [24, 32], None),
    (5, [8, 7, 8, 7, 8], [7, 8, 7, 8, 8], 3),   # beyond shared memory: workspace slots
])
def test_deterministic_rectangular_vbatched(kmx, oracle, d, m, nn, wslots, form):
    """Deterministic mode for rectangular vbatched with Y blocks shared by
    several entries: entries grouped by Y block on the device and each block
    summed by one group in a fixed order -- bitwise repeatable, equal to the
    oracle."""
    rng = np.random.default_rng(200 + d)
    batch, nyb = 12, 4
    Nx, Ny = int(np.prod(nn)), int(np.prod(m))
    A, offs, X, _ = vb_case(201 + d, d, m, nn, batch=batch, y0=False)
    yblk = rng.integers(0, nyb, batch)
    Y0 = rng.uniform(-1, 1, (nyb, Ny))
    Yref = Y0.copy()
    sxw = oracle.size_xw(d, m, nn)
    oracle.vbatched(d, m, nn, A, offs, X, [b * Nx for b in range(batch)], Yref,
                    [int(y) * Ny for y in yblk], np.zeros(2 * sxw * batch))
    Ad, Xd = dev(A), dev(X)
    W = torch.zeros(2 * sxw * (wslots or batch), dtype=torch.float64, device="cuda")
    outs = []
    for _ in range(2):
        Yd = dev(Y0)
        kmx.kronmult_vbatched(d, m, nn, kmx.pointer_array(Ad, offs),
                              kmx.pointer_array(Xd, [b * Nx for b in range(batch)]),
                              kmx.pointer_array(Yd, [int(y) * Ny for y in yblk]), W, None, batch,
                              form=form, accumulate="deterministic")
        outs.append(host(Yd))
    check_status(kmx)
    assert np.array_equal(outs[0], outs[1])
    assert blockwise_rel_err(outs[0], Yref) <= F64_TOL


def test_deterministic_generic_f32(kmx, oracle):
    """FP32 data, a shape without a tiled segment kernel (d = 2, n = 6)."""
    rng = np.random.default_rng(301)
    d, n, ne, nyb = 2, 6, 200, 7
    N = n ** d
    A = rng.standard_normal((ne, d, n, n)).astype(np.float32)
    X = rng.standard_normal((ne, N)).astype(np.float32)
    yblk = rng.integers(0, nyb, ne)
    Y0 = rng.uniform(-1, 1, (nyb, N)).astype(np.float32)
    Yref = Y0.copy()
    # the oracle's pbatched with a Y offset per entry (it clobbers X and W)
    offs = [b * N for b in range(ne)]
    oracle.pbatched(d, n, A, X.copy().reshape(-1), offs, Yref.reshape(-1),
                    [int(y) * N for y in yblk], np.zeros(ne * N, dtype=np.float32), offs)
    Ad, Xd = dev(A), dev(X)
    outs = []
    for _ in range(2):
        Yd = dev(Y0)
        kmx.kronmult_pbatched(d, n, Ad, kmx.pointer_array(Xd, [b * N for b in range(ne)]),
                              kmx.pointer_array(Yd, [int(y) * N for y in yblk]), None, ne,
                              accumulate="deterministic")
        outs.append(host(Yd))
    check_status(kmx)
    assert np.array_equal(outs[0], outs[1])
    assert blockwise_rel_err(outs[0], Yref) <= 1e-5


def _random_shapes(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        d = int(rng.integers(1, 7))
        m = [int(v) for v in rng.integers(1, 13, d)]
        nn = [int(v) for v in rng.integers(1, 13, d)]
        sizes = [int(np.prod(nn))] + [int(np.prod(m[:k])) * int(np.prod(nn[k:]))
                                      for k in range(1, d + 1)]
        if max(sizes) <= 20000:
            out.append((d, m, nn))
    return out


@pytest.mark.parametrize("case", range(24))
def test_generic_random_shape_sweep(kmx, oracle, case):
    """Seeded random rectangular shapes (d = 1..6, extents 1..12, every
    intermediate at most 20000 elements), random batch sizes, both FP64 forms,
    atomic and deterministic accumulation, Y blocks shared between entries:
    against the oracle's vbatched."""
    d, m, nn = _random_shapes(7, 24)[case]
    rng = np.random.default_rng(1000 + case)
    batch = int(rng.integers(1, 9))
    nyb = int(rng.integers(1, batch + 1))
    Nx, Ny = int(np.prod(nn)), int(np.prod(m))
    A, offs, X, _ = vb_case(2000 + case, d, m, nn, batch=batch, y0=False)
    yblk = rng.integers(0, nyb, batch)
    Y0 = rng.uniform(-1, 1, (nyb, Ny))
    Yref = Y0.copy()
    sxw = oracle.size_xw(d, m, nn)
    oracle.vbatched(d, m, nn, A, offs, X, [b * Nx for b in range(batch)], Yref,
                    [int(y) * Ny for y in yblk], np.zeros(2 * sxw * batch))
    Ad, Xd = dev(A), dev(X)
    W = torch.zeros(2 * sxw * batch, dtype=torch.float64, device="cuda")
    for form in ("split", "plain"):
        for acc in ("atomic", "deterministic"):
            Yd = dev(Y0)
            kmx.kronmult_vbatched(d, m, nn, kmx.pointer_array(Ad, offs),
                                  kmx.pointer_array(Xd, [b * Nx for b in range(batch)]),
                                  kmx.pointer_array(Yd, [int(y) * Ny for y in yblk]), W, None,
                                  batch, form=form, accumulate=acc)
            assert blockwise_rel_err(host(Yd), Yref) <= F64_TOL, (d, m, nn, form, acc)
    check_status(kmx)
