"""Full-size properties of the headline workload: xbatched FP64, d=6, n=4,
131072 entries over 8192 X / 8192 Y blocks (256 MiB each), per-Y-block
counts geometric with mean 16 -- the size the benchmark measures, where the
CPU oracle would take minutes.  Checked through properties that hold at any
size (agreement of every arithmetic form with plain FP64, accumulation,
linearity, the adjoint identity, bitwise repeatability of the deterministic
mode) and against the oracle on a sample of Y blocks, whose contributing
entries the oracle recomputes in full.  Every call goes through the C ABI.

Tolerance: normwise relative error per Y block <= 1e-13 (FP64 forms).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F64_TOL = 1e-13


@pytest.fixture(scope="module")
def wl(kmx):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bench

    w = bench.make_workload()
    d, n, pool = bench.D, bench.NN, bench.POOL
    N = n ** d
    dev = torch.device("cuda", 0)
    Ad = torch.from_numpy(w["Apool"]).to(dev)
    Xd = torch.from_numpy(w["Xpool"]).to(dev)
    y_idx = torch.from_numpy(w["y_idx"]).to(dev).long()
    x_idx = torch.from_numpy(w["x_idx"]).to(dev).long()
    a_idx = torch.from_numpy(w["a_idx"]).to(dev).long()
    lvl = torch.arange(d, device=dev).long()[None, :]
    pA = ((lvl * pool + a_idx) * (n * n * 8) + Ad.data_ptr()).reshape(-1).contiguous()
    return dict(w=w, d=d, n=n, N=N, pool=pool, A=Ad, X=Xd, y_idx=y_idx, x_idx=x_idx, pA=pA,
                entries=int(y_idx.numel()))


def _apply(kmx, wl, X, Y, form="auto", acc="atomic", transpose=False):
    """Y[y_idx[e]] += K_e X[x_idx[e]]; with transpose the adjoint direction:
    X plays the Y-pool role and Y the X-pool role (indices swapped)."""
    N = wl["N"]
    src_idx, dst_idx = (wl["y_idx"], wl["x_idx"]) if transpose else (wl["x_idx"], wl["y_idx"])
    pX = src_idx * (N * 8) + X.data_ptr()
    pY = dst_idx * (N * 8) + Y.data_ptr()
    kmx.kronmult_xbatched(wl["d"], wl["n"], wl["pA"], wl["n"], pX, pY, None, wl["entries"],
                          form=form, accumulate=acc, transpose=transpose)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0


def _blockwise(y, yref):
    num = torch.linalg.vector_norm(y - yref, dim=1)
    den = torch.linalg.vector_norm(yref, dim=1).clamp_min(1e-300)
    return float((num / den).max())


def test_fullsize_forms_agree_with_plain_fp64(kmx, wl):
    Yp = torch.zeros_like(wl["X"])
    _apply(kmx, wl, wl["X"], Yp, form="plain")
    for form, acc in (("auto", "atomic"), ("split", "atomic"), ("digits", "atomic"),
                      ("auto", "deterministic")):
        Y = torch.zeros_like(wl["X"])
        _apply(kmx, wl, wl["X"], Y, form=form, acc=acc)
        assert _blockwise(Y, Yp) <= F64_TOL, (form, acc)


def test_fullsize_accumulates_into_y(kmx, wl):
    """Y is accumulated into: two calls on a nonzero Y add twice the product."""
    g = torch.Generator(device="cuda").manual_seed(3)
    Y0 = torch.rand(wl["X"].shape, dtype=torch.float64, device="cuda", generator=g)
    Y1 = Y0.clone()
    _apply(kmx, wl, wl["X"], Y1)
    Y2 = Y1.clone()
    _apply(kmx, wl, wl["X"], Y2)
    assert _blockwise(Y2 - Y0, 2 * (Y1 - Y0)) <= F64_TOL


def test_fullsize_linearity_in_x(kmx, wl):
    g = torch.Generator(device="cuda").manual_seed(4)
    X2 = torch.randn(wl["X"].shape, dtype=torch.float64, device="cuda", generator=g)
    al, be = 0.75, -1.25
    Ya = torch.zeros_like(wl["X"])
    Yb = torch.zeros_like(wl["X"])
    Yc = torch.zeros_like(wl["X"])
    _apply(kmx, wl, wl["X"], Ya)
    _apply(kmx, wl, X2, Yb)
    _apply(kmx, wl, al * wl["X"] + be * X2, Yc)
    assert _blockwise(Yc, al * Ya + be * Yb) <= F64_TOL


@pytest.mark.parametrize("form", ["auto", "plain"])
def test_fullsize_adjoint_identity(kmx, wl, form):
    """<G, K X> = <K^T G, X>: the forward over all entries against the
    transposed product with x and y indices swapped."""
    g = torch.Generator(device="cuda").manual_seed(5)
    G = torch.randn(wl["X"].shape, dtype=torch.float64, device="cuda", generator=g)
    KX = torch.zeros_like(wl["X"])
    _apply(kmx, wl, wl["X"], KX, form=form)
    KtG = torch.zeros_like(wl["X"])
    _apply(kmx, wl, G, KtG, form=form, transpose=True)
    lhs = float((G * KX).sum())
    rhs = float((KtG * wl["X"]).sum())
    scale = float(torch.linalg.vector_norm(G) * torch.linalg.vector_norm(KX))
    assert abs(lhs - rhs) <= 1e-13 * scale, (lhs, rhs, scale)


def test_fullsize_deterministic_is_bitwise_repeatable(kmx, wl):
    Y1 = torch.zeros_like(wl["X"])
    Y2 = torch.zeros_like(wl["X"])
    _apply(kmx, wl, wl["X"], Y1, acc="deterministic")
    _apply(kmx, wl, wl["X"], Y2, acc="deterministic")
    assert torch.equal(Y1, Y2)


def test_fullsize_sampled_blocks_vs_oracle(kmx, oracle, wl):
    """48 Y blocks of the full run against the oracle, which recomputes every
    entry that contributes to them (about 770 entries)."""
    Y = torch.zeros_like(wl["X"])
    _apply(kmx, wl, wl["X"], Y)
    w = wl["w"]
    rng = np.random.default_rng(6)
    blocks = rng.choice(w["Xpool"].shape[0], 48, replace=False)
    remap = -np.ones(w["Xpool"].shape[0], dtype=np.int64)
    remap[blocks] = np.arange(len(blocks))
    sel = np.nonzero(remap[w["y_idx"]] >= 0)[0]
    Yref = np.zeros((len(blocks), wl["N"]))
    oracle.xbatched_idx(wl["d"], wl["n"], w["Apool"], wl["n"], wl["pool"], w["Xpool"], Yref,
                        remap[w["y_idx"][sel]], w["x_idx"][sel], w["a_idx"][sel])
    got = Y[torch.from_numpy(blocks).cuda()].cpu().numpy()
    num = np.linalg.norm(got - Yref, axis=1)
    den = np.maximum(np.linalg.norm(Yref, axis=1), 1e-300)
    assert float((num / den).max()) <= F64_TOL


# ---------------------------------------------------------------------------
# the precision-form workload at full size: xbatched d=4 n=8 and d=3 n=16,
# 262144 entries over 16384 X/Y blocks, factors N(0,1)/sqrt(n), X N(0,1)
# ---------------------------------------------------------------------------

F32_FORM_TOL = 1e-6   # FP32-stored forms, against FP64 on the unrounded inputs
BF16_FORM_TOL = 1e-2  # BF16 storage: the error of rounding inputs to 8 bits


def _precision_case(d, n, seed):
    entries, nblocks, pool = 262144, 16384, 1024
    N = n ** d
    rng = np.random.default_rng(seed)
    counts = rng.geometric(1.0 / 16, nblocks)
    y_idx = np.repeat(np.arange(nblocks), counts)[:entries]
    if len(y_idx) < entries:
        y_idx = np.concatenate([y_idx, rng.integers(0, nblocks, entries - len(y_idx))])
    rng.shuffle(y_idx)
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn((d, pool, n, n), dtype=torch.float64, device="cuda", generator=g) / n ** 0.5
    X = torch.randn((nblocks, N), dtype=torch.float64, device="cuda", generator=g)
    return dict(d=d, n=n, N=N, pool=pool, entries=entries, A=A, X=X,
                ai=torch.from_numpy(rng.integers(0, pool, (entries, d))).cuda(),
                xi=torch.from_numpy(rng.integers(0, nblocks, entries)).cuda(),
                yi=torch.from_numpy(y_idx).cuda())


def _pc_ptrs(c, A, X, Y):
    lvl = torch.arange(c["d"], device="cuda")[None, :]
    n, N = c["n"], c["N"]
    return (((lvl * c["pool"] + c["ai"]) * (n * n * A.element_size()) + A.data_ptr())
            .reshape(-1).contiguous(),
            c["xi"] * (N * X.element_size()) + X.data_ptr(),
            c["yi"] * (N * Y.element_size()) + Y.data_ptr())


def _scaled_blockwise(y, yref):
    s = yref.abs().amax(dim=1, keepdim=True).clamp_min(1e-300)
    return float((torch.linalg.vector_norm((y - yref) / s, dim=1) /
                  torch.linalg.vector_norm(yref / s, dim=1).clamp_min(1e-300)).max())


@pytest.mark.parametrize("d,n", [(4, 8), (3, 16)])
def test_fullsize_precision_forms(kmx, d, n):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = _precision_case(d, n, 31 + n)
    Yref = torch.zeros_like(c["X"])
    pA, pX, pY = _pc_ptrs(c, c["A"], c["X"], Yref)
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, c["entries"], form="plain")
    Y = torch.zeros_like(Yref)
    pA, pX, pY = _pc_ptrs(c, c["A"], c["X"], Y)
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, c["entries"])
    torch.cuda.synchronize()
    assert _blockwise(Y, Yref) <= F64_TOL
    for tdt, tol in ((torch.float32, F32_FORM_TOL), (torch.bfloat16, BF16_FORM_TOL)):
        A, X = c["A"].to(tdt), c["X"].to(tdt)
        ind = "f32" if tdt == torch.float32 else "bf16"
        for form, acc in ((None, None), ("tf32x3", None), ("tf32x3", "deterministic")):
            Y.zero_()
            pA, pX, pY = _pc_ptrs(c, A, X, Y)
            kmx.kronmult_xbatched_wide(d, n, pA, n, pX, pY, c["entries"], in_dtype=ind,
                                       form=form, accumulate=acc)
            torch.cuda.synchronize()
            assert _scaled_blockwise(Y, Yref) <= tol, (ind, form, acc)
            if acc == "deterministic":
                Y2 = torch.zeros_like(Y)
                kmx.kronmult_xbatched_wide(d, n, pA, n, pX, c["yi"] * (c["N"] * 8) + Y2.data_ptr(),
                                           c["entries"], in_dtype=ind, form=form, accumulate=acc)
                torch.cuda.synchronize()
                assert torch.equal(Y, Y2)
        del A, X
    # the FP32 entry point proper (FP32 X, factors and Y)
    A32, X32 = c["A"].float(), c["X"].float()
    Y32 = torch.zeros(c["X"].shape, dtype=torch.float32, device="cuda")
    pA, pX, pY = _pc_ptrs(c, A32, X32, Y32)
    for form in (None, "plain", "tf32x3"):
        Y32.zero_()
        kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, c["entries"], dtype=torch.float32,
                              form=form)
        torch.cuda.synchronize()
        assert _scaled_blockwise(Y32.double(), Yref) <= F32_FORM_TOL, form
    assert kmx.check_device_status() == 0
