"""GPU parity of the rectangular mixed-shape call (kmx_kronmult_vmixed_*):
instances of several rectangular shape classes in one call, checked against
the oracle's vbatched (kronmult_vbatched.hpp:19-248) run class by class on the
same inputs.  Every call goes through the C ABI.

Tolerances: FP64 normwise relative error per Y block <= 1e-13; FP32 <= 1e-5.
"""
import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F64_TOL = 1e-13
F32_TOL = 1e-5

# (m, n) per class: rectangular, a specialised square shape (register-tiled
# kernel), unspecialised square, d = 1, and one entry beyond shared memory
CLASSES = [
    ([4, 3, 4], [3, 4, 3]),
    ([5], [7]),
    ([3, 2, 3, 2, 3, 2], [2, 3, 2, 3, 2, 3]),
    ([4, 4, 4, 4], [4, 4, 4, 4]),
    ([10, 12], [12, 10]),
    ([9, 9, 9], [9, 9, 9]),
    ([8, 7, 8, 7, 8], [7, 8, 7, 8, 8]),
]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _case(seed, classes, count, dtype=np.float64, big_share=0.01):
    """Random instances: class ids, own factors and X blocks, Y blocks drawn
    from a per-class pool so that several instances add into one block."""
    rng = np.random.default_rng(seed)
    nbig = len(classes) - 1 if np.prod(classes[-1][1]) > 20000 else None
    p = np.ones(len(classes))
    if nbig is not None:
        p[nbig] = big_share * (len(classes) - 1) / (1 - big_share)
    cls = rng.choice(len(classes), count, p=p / p.sum()).astype(np.int32)
    ypool = [max(1, int((cls == c).sum()) // 3) for c in range(len(classes))]
    yoff_class, o = [], 0
    for c, (m, _) in enumerate(classes):
        yoff_class.append(o)
        o += ypool[c] * int(np.prod(m))
    Y0 = rng.uniform(-1, 1, o).astype(dtype)
    A, X, aoff, xoff, yoff, a_first = [], [], [], [], [], []
    na = nx = 0
    for i in range(count):
        m, n = classes[cls[i]]
        a_first.append(len(aoff))
        for l in range(len(m)):
            A.append((rng.standard_normal(m[l] * n[l]) / np.sqrt(n[l])).astype(dtype))
            aoff.append(na)
            na += m[l] * n[l]
        X.append(rng.standard_normal(int(np.prod(n))).astype(dtype))
        xoff.append(nx)
        nx += int(np.prod(n))
        c = cls[i]
        yoff.append(yoff_class[c] + int(rng.integers(0, ypool[c])) * int(np.prod(m)))
    return dict(cls=cls, A=np.concatenate(A), X=np.concatenate(X), Y0=Y0, aoff=aoff, xoff=xoff,
                yoff=yoff, a_first=a_first)


def _oracle(oracle, classes, cs):
    """The oracle's vbatched per class, instances in their original order."""
    Y = cs["Y0"].copy()
    for c, (m, n) in enumerate(classes):
        idx = np.nonzero(cs["cls"] == c)[0]
        if len(idx) == 0:
            continue
        d = len(m)
        aoff = [cs["aoff"][cs["a_first"][i] + l] for i in idx for l in range(d)]
        sxw = oracle.size_xw(d, m, n)
        oracle.vbatched(d, m, n, cs["A"], aoff, cs["X"], [cs["xoff"][i] for i in idx], Y,
                        [cs["yoff"][i] for i in idx],
                        np.zeros(2 * sxw * len(idx), dtype=cs["A"].dtype))
    return Y


def _device(kmx, cs, classes):
    dA = torch.from_numpy(cs["A"]).cuda()
    dX = torch.from_numpy(cs["X"]).cuda()
    dY = torch.from_numpy(cs["Y0"].copy()).cuda()
    pA = kmx.pointer_array(dA, cs["aoff"])
    pX = kmx.pointer_array(dX, cs["xoff"])
    pY = kmx.pointer_array(dY, cs["yoff"])
    a_off = torch.tensor(cs["a_first"], dtype=torch.int64, device="cuda")
    cls = torch.from_numpy(cs["cls"]).cuda()
    big = max(kmx_sxw(m, n) for m, n in classes)
    W = torch.zeros(2 * big * 64, dtype=dA.dtype, device="cuda")  # 64 slots
    return dict(dA=dA, dX=dX, dY=dY, pA=pA, pX=pX, pY=pY, a_off=a_off, cls=cls, W=W)


def kmx_sxw(m, n):
    d = len(m)
    best = int(np.prod(n))
    for k in range(1, d + 1):
        best = max(best, int(np.prod(m[:k])) * int(np.prod(n[k:])))
    return best


def _blocks(Y, cs, classes):
    """Rows = the Y blocks of every class (for the per-block error)."""
    out = []
    o = 0
    for c, (m, _) in enumerate(classes):
        nb = int(np.prod(m))
        used = sorted({cs["yoff"][i] for i in np.nonzero(cs["cls"] == c)[0]})
        out += [Y[u:u + nb] for u in used]
    return out


def _err(y, yref, cs, classes):
    return max(blockwise_rel_err(a[None, :], b[None, :])
               for a, b in zip(_blocks(y, cs, classes), _blocks(yref, cs, classes)))


@pytest.mark.parametrize("form", [None, "plain", "split"])
def test_vmixed_vs_oracle(kmx, oracle, form):
    cs = _case(5, CLASSES, 700)
    ref = _oracle(oracle, CLASSES, cs)
    dv = _device(kmx, cs, CLASSES)
    kmx.kronmult_vmixed(dv["cls"], dv["pA"], dv["a_off"], dv["pX"], dv["pY"], CLASSES, dv["W"],
                        form=form)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    assert _err(dv["dY"].cpu().numpy(), ref, cs, CLASSES) <= F64_TOL


def test_vmixed_f32_vs_oracle(kmx, oracle):
    classes = CLASSES[:6]
    cs = _case(6, classes, 500, dtype=np.float32)
    ref = _oracle(oracle, classes, cs)
    dv = _device(kmx, cs, classes)
    kmx.kronmult_vmixed(dv["cls"], dv["pA"], dv["a_off"], dv["pX"], dv["pY"], classes, dv["W"],
                        dtype=torch.float32)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    assert _err(dv["dY"].cpu().numpy(), ref, cs, classes) <= F32_TOL


def test_vmixed_cuda_graph_replay(kmx):
    """No host synchronisation inside the call: it captures into a CUDA graph;
    two replays add twice the contribution of one call."""
    classes = CLASSES[:6]
    cs = _case(7, classes, 400)
    dv = _device(kmx, cs, classes)
    s = torch.cuda.Stream()
    args = (dv["cls"], dv["pA"], dv["a_off"], dv["pX"], dv["pY"], classes, dv["W"])
    with torch.cuda.stream(s):
        kmx.kronmult_vmixed(*args, stream=s)  # warm-up (workspace, kernel attributes)
    s.synchronize()
    once = dv["dY"].clone() - torch.from_numpy(cs["Y0"]).cuda()
    dv["dY"].copy_(torch.from_numpy(cs["Y0"]).cuda())
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        kmx.kronmult_vmixed(*args, stream=s)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    twice = dv["dY"] - torch.from_numpy(cs["Y0"]).cuda()
    err = ((twice - 2 * once).norm() / (2 * once).norm()).item()
    assert err < 1e-13
    assert kmx.check_device_status() == 0


def test_vmixed_unknown_class_is_flagged(kmx, oracle):
    """An instance whose class id is outside the list is skipped and flagged;
    the others are computed."""
    classes = CLASSES[:3]
    cs = _case(8, classes, 60)
    bad = 17
    ref_cs = dict(cs)
    ref_cs["cls"] = cs["cls"].copy()
    ref_cs["cls"][bad] = 99  # the oracle skips it too (no class 99)
    ref = _oracle(oracle, classes, ref_cs)
    dv = _device(kmx, cs, classes)
    dv["cls"][bad] = 99
    kmx.kronmult_vmixed(dv["cls"], dv["pA"], dv["a_off"], dv["pX"], dv["pY"], classes, dv["W"])
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()
    assert _err(dv["dY"].cpu().numpy(), ref, cs, classes) <= F64_TOL
    assert kmx.check_device_status() == 0


def test_vmixed_missing_workspace_for_large_class(kmx):
    """A class whose entries exceed shared memory needs the caller's W (as in
    vbatched): without it the call returns KMX_ERR_WORKSPACE."""
    classes = [CLASSES[0], CLASSES[6]]
    cs = _case(9, classes, 20, big_share=0.3)
    dv = _device(kmx, cs, classes)
    with pytest.raises(kmx.KmxError):
        kmx.kronmult_vmixed(dv["cls"], dv["pA"], dv["a_off"], dv["pX"], dv["pY"], classes, None)


def _shared_y_case(seed, classes, count, blocks_per_size, sizes, rng_dtype=np.float64):
    """Instances of random classes whose Y blocks come from one pool per block
    size, so that instances of one class -- and of different classes with
    equal block sizes -- add into the same block."""
    rng = np.random.default_rng(seed)
    cls = rng.integers(0, len(classes), count).astype(np.int32)
    pools, o = {}, 0
    for sz in sorted(set(sizes)):
        pools[sz] = [o + k * sz for k in range(blocks_per_size)]
        o += blocks_per_size * sz
    Y0 = rng.uniform(-1, 1, o)
    yoff = [int(rng.choice(pools[sizes[c]])) for c in cls]
    return cls, Y0, yoff, rng


def _run_twice(call, Y0):
    outs = []
    for _ in range(2):
        Yd = torch.from_numpy(Y0.copy()).cuda()
        call(Yd)
        torch.cuda.synchronize()
        outs.append(Yd.cpu().numpy())
    return outs


def test_mixed_square_deterministic_vs_oracle(kmx, oracle):
    """kmx_kronmult_mixed_f64, deterministic: instances of several (d, n)
    classes share Y blocks (also across classes of equal block size); the
    result is bitwise repeatable and equals the oracle's contributions summed
    per block."""
    classes = [(2, 4), (4, 2), (3, 4), (6, 2), (2, 8), (1, 16), (5, 3)]
    sizes = [n ** d for d, n in classes]
    cls, Y0, yoff, rng = _shared_y_case(11, classes, 400, 6, sizes)
    factors, xs, ptr_offs, aoff, xoff, dims = [], [], [], [], [], []
    Yref = Y0.copy()
    fo = xo = 0
    for i, c in enumerate(cls):
        d, n = classes[c]
        dims.append((d, n))
        A = rng.standard_normal((1, d, n, n)) / np.sqrt(n)
        X = rng.standard_normal((1, n ** d))
        contrib = np.zeros_like(X)
        oracle.batched(d, n, A, X.copy(), contrib, np.zeros_like(X), 1)
        Yref[yoff[i]:yoff[i] + n ** d] += contrib[0]
        aoff.append(len(ptr_offs))
        ptr_offs += [fo + l * n * n for l in range(d)]  # factor l of instance i
        factors.append(A.reshape(-1))
        fo += d * n * n
        xs.append(X.reshape(-1))
        xoff.append(xo)
        xo += n ** d
    fbuf = torch.from_numpy(np.concatenate(factors)).cuda()
    xbuf = torch.from_numpy(np.concatenate(xs)).cuda()
    pA = kmx.pointer_array(fbuf, ptr_offs)
    pX = kmx.pointer_array(xbuf, xoff)
    dims_d = torch.from_numpy(np.array(dims, dtype=np.int32)).cuda()
    a_off = torch.tensor(aoff, dtype=torch.int64, device="cuda")

    def call(Yd):
        kmx.kronmult_mixed(dims_d, pA, a_off, pX, kmx.pointer_array(Yd, yoff), classes, None,
                           accumulate="deterministic")

    outs = _run_twice(call, Y0)
    assert kmx.check_device_status() == 0
    assert np.array_equal(outs[0], outs[1])
    rows = sorted(set((o, sizes[c]) for o, c in zip(yoff, cls)))
    worst = max(blockwise_rel_err(outs[0][o:o + sz][None, :], Yref[o:o + sz][None, :])
                for o, sz in rows)
    assert worst <= F64_TOL


@pytest.mark.parametrize("form", [None, "plain"])
def test_vmixed_deterministic_vs_oracle(kmx, oracle, form):
    """kmx_kronmult_vmixed_f64, deterministic, rectangular classes (one beyond
    shared memory) sharing Y blocks, also across classes of equal block size:
    bitwise repeatable, equal to the oracle's vbatched run class by class."""
    classes = [([4, 3], [3, 4]), ([3, 4], [5, 2]), ([4, 3, 4], [3, 4, 3]),
               ([2, 3, 8], [3, 4, 4]), ([8, 7, 8, 7, 8], [7, 8, 7, 8, 8])]
    sizes = [int(np.prod(m)) for m, _ in classes]
    cs = _case(13, classes, 300, big_share=0.02)
    rng = np.random.default_rng(14)
    pools, o = {}, 0
    for sz in sorted(set(sizes)):
        pools[sz] = [o + k * sz for k in range(5)]
        o += 5 * sz
    cs["Y0"] = rng.uniform(-1, 1, o)
    cs["yoff"] = [int(rng.choice(pools[sizes[c]])) for c in cs["cls"]]
    ref = _oracle(oracle, classes, cs)
    dv = _device(kmx, cs, classes)

    def call(Yd):
        kmx.kronmult_vmixed(dv["cls"], dv["pA"], dv["a_off"], dv["pX"],
                            kmx.pointer_array(Yd, cs["yoff"]), classes, dv["W"], form=form,
                            accumulate="deterministic")

    outs = _run_twice(call, cs["Y0"])
    assert kmx.check_device_status() == 0
    assert np.array_equal(outs[0], outs[1])
    assert _err(outs[0], ref, cs, classes) <= F64_TOL


@pytest.mark.parametrize("form", [None, "split"])
def test_vmixed_persistent_engine(kmx, oracle, form):
    """KMX_ENGINE_PERSISTENT on rectangular classes: one launch over every
    class, instances from a device work queue, each run by the generic
    double-float kernel with its own shape (two buffers on chip, or in the
    caller's workspace for the class beyond shared memory)."""
    cs = _case(15, CLASSES, 600, big_share=0.03)
    ref = _oracle(oracle, CLASSES, cs)
    dv = _device(kmx, cs, CLASSES)
    kmx.kronmult_vmixed(dv["cls"], dv["pA"], dv["a_off"], dv["pX"], dv["pY"], CLASSES, dv["W"],
                        form=form, engine="persistent")
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    assert _err(dv["dY"].cpu().numpy(), ref, cs, CLASSES) <= F64_TOL


def test_vmixed_persistent_unknown_class_is_flagged(kmx, oracle):
    classes = CLASSES[:3]
    cs = _case(16, classes, 60)
    bad = 11
    ref_cs = dict(cs)
    ref_cs["cls"] = cs["cls"].copy()
    ref_cs["cls"][bad] = 99
    ref = _oracle(oracle, classes, ref_cs)
    dv = _device(kmx, cs, classes)
    dv["cls"][bad] = 99
    kmx.kronmult_vmixed(dv["cls"], dv["pA"], dv["a_off"], dv["pX"], dv["pY"], classes, dv["W"],
                        engine="persistent")
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()
    assert _err(dv["dY"].cpu().numpy(), ref, cs, classes) <= F64_TOL
    assert kmx.check_device_status() == 0
