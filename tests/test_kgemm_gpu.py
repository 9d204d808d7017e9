"""GPU parity of the batched tiny-GEMM entry points kgemm_{nn,nt}_batched
(kgemm_nn_batched.cpp:8-41, kgemm_nt_batched.cpp:8-41) against the golden
outputs of the reference's own CPU build and against the oracle.  Every call
goes through the C ABI.

Tolerances:
  FP64: normwise relative error per entry <= 1e-13 on the golden inputs; on
        random inputs (long dot products that cancel) the componentwise GEMM
        measure |dC| <= 1e-13 (|alpha| |A||op(B)| + |beta| |C|) (the
        reference test's own bound is max abs error < 1e-9,
        test_kgemm_nn_batched.cpp:563).
  FP32: the reference test's max abs error < 5e-4 (:562) on its closed-form
        inputs and normwise <= 1e-5 per entry (both paths accumulate to about
        48 bits and round once).
"""
import os

import numpy as np
import pytest

from tests.common import blockwise_rel_err
from tests.golden import make_kgemm_golden as mk

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F64_TOL = 1e-13
F64_CW_TOL = 1e-13  # componentwise, relative to |alpha| |A| |op(B)| + |beta| |C|
F32_NORM_TOL = 1e-5
F32_ABS_TOL = 5e-4


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _golden():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "kgemm_golden.npz"))


def _run_gpu(kmx, trans, A, aoff, ldA, B, boff, ldB, C, coff, ldC, mm, nn, kk, alpha, beta):
    """A, B, C host arrays (flat); returns C after the GPU call."""
    dA, dB, dC = (torch.from_numpy(np.ascontiguousarray(v).reshape(-1)).cuda() for v in (A, B, C))
    pA = kmx.pointer_array(dA, aoff)
    pB = kmx.pointer_array(dB, boff)
    pC = kmx.pointer_array(dC, coff)
    i32 = lambda v: torch.tensor(v, dtype=torch.int32, device="cuda")  # noqa: E731
    fn = kmx.kgemm_nn_batched if trans == "nn" else kmx.kgemm_nt_batched
    fn(mm, nn, kk, alpha, pA, i32(ldA), pB, i32(ldB), beta, pC, i32(ldC), len(aoff),
       dtype=dA.dtype)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    return dC.cpu().numpy().reshape(np.shape(C))


def _err_ok(tag, got, ref, ncols):
    got = got.reshape(-1, ncols) if ncols else got
    ref = ref.reshape(-1, ncols) if ncols else ref
    g64, r64 = got.astype(np.float64), ref.astype(np.float64)
    err = blockwise_rel_err(g64.reshape(g64.shape[0], -1), r64.reshape(r64.shape[0], -1))
    if tag == "f64":
        return err <= F64_TOL, err
    return err <= F32_NORM_TOL and np.abs(g64 - r64).max() < F32_ABS_TOL, err


@pytest.mark.parametrize("trans", ["nn", "nt"])
@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_kgemm_golden(kmx, trans, tag):
    g = _golden()
    T = np.float64 if tag == "f64" else np.float32
    for (mm, nn, kk, batch) in mk.SHAPES:
        for bname, beta in mk.BETAS:
            if bname != "b12" and (mm, nn, kk, batch) not in mk.ALL_BETAS:
                continue
            A, B, C0 = mk.po.ramp_kgemm(trans, mm, nn, kk, batch, dtype=T)
            got = _run_gpu(kmx, trans, A, [i * mm * kk for i in range(batch)], [mm] * batch,
                           B, [i * B.shape[1] for i in range(batch)],
                           [mk.ld_b(trans, nn, kk)] * batch, C0,
                           [i * mm * nn for i in range(batch)], [mm] * batch, mm, nn, kk,
                           mk.ALPHA, beta)
            ok, err = _err_ok(tag, got, g[mk.case_key(trans, tag, mm, nn, kk, batch, bname)],
                              mm * nn)
            assert ok, (mm, nn, kk, batch, bname, err)


@pytest.mark.parametrize("trans", ["nn", "nt"])
@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_kgemm_shared_c_golden(kmx, trans, tag):
    """beta == 1: every entry adds into the same C with atomics."""
    g = _golden()
    T = np.float64 if tag == "f64" else np.float32
    mm, nn, kk, batch = 8, 15, 22, 8
    A, B, C0 = mk.po.ramp_kgemm(trans, mm, nn, kk, batch, dtype=T)
    got = _run_gpu(kmx, trans, A, [i * mm * kk for i in range(batch)], [mm] * batch,
                   B, [i * B.shape[1] for i in range(batch)], [mk.ld_b(trans, nn, kk)] * batch,
                   C0[:1].copy(), [0] * batch, [mm] * batch, mm, nn, kk, mk.ALPHA, 1.0)
    ok, err = _err_ok(tag, got, g[f"{trans}_{tag}_shared_8x15x22_b8"], mm * nn)
    assert ok, err


def _componentwise_err(trans, got, ref, A, aoff, ldA, B, boff, ldB, C0, coff, ldC, mm, nn, kk,
                       alpha, beta):
    """max over C elements of |got - ref| / (|alpha| (|A| |op(B)|) + |beta| |C0|):
    the standard GEMM error measure, meaningful where a long dot product
    cancels (a normwise relative error of a 1 x 1 output is not)."""
    worst = 0.0
    for b in range(len(aoff)):
        Ab = A[aoff[b]:aoff[b] + ldA[b] * kk].reshape(kk, ldA[b]).T[:mm, :].astype(np.float64)
        if trans == "nn":
            Bb = B[boff[b]:boff[b] + ldB[b] * nn].reshape(nn, ldB[b]).T[:kk, :]
        else:
            Bb = B[boff[b]:boff[b] + ldB[b] * kk].reshape(kk, ldB[b]).T[:nn, :].T
        Bb = Bb.astype(np.float64)

        def cm(X):
            return X[coff[b]:coff[b] + ldC[b] * nn].reshape(nn, ldC[b]).T[:mm, :].astype(np.float64)

        scale = abs(alpha) * (np.abs(Ab) @ np.abs(Bb)) + abs(beta) * np.abs(cm(C0))
        diff = np.abs(cm(got) - cm(ref))
        worst = max(worst, float((diff / np.maximum(scale, 1e-300)).max()))
    return worst


def _random_case(rng, trans, T, mm, nn, kk, batch, pad):
    ldA, ldC = mm + pad, mm + pad
    ldB = (kk if trans == "nn" else nn) + pad
    colsB = nn if trans == "nn" else kk
    A = rng.standard_normal(batch * ldA * kk).astype(T)
    B = rng.standard_normal(batch * ldB * colsB).astype(T)
    C = rng.standard_normal(batch * ldC * nn).astype(T)
    offs = lambda ld, cols: [i * ld * cols for i in range(batch)]  # noqa: E731
    return (A, offs(ldA, kk), [ldA] * batch, B, offs(ldB, colsB), [ldB] * batch, C,
            offs(ldC, nn), [ldC] * batch)


@pytest.mark.parametrize("trans", ["nn", "nt"])
@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_kgemm_random_sweep_vs_oracle(kmx, oracle, trans, tag):
    """The reference's size sweep (mm, nn, kk over 1..65, test_kgemm_nn_batched.cpp:
    525-560, every other step here) with padded leading dimensions, random
    inputs, and the kronmult contraction shapes (short-wide and tall-narrow)."""
    T = np.float64 if tag == "f64" else np.float32
    rng = np.random.default_rng(11)
    sizes = [(mm, nn, kk) for mm in (1, 15, 29, 50, 65) for nn in (1, 22, 65) for kk in (1, 8, 36, 65)]
    sizes += [(4, 1024, 4), (1024, 4, 4), (5, 3125, 5), (3125, 5, 5), (8, 512, 8), (512, 8, 8),
              (16, 4096, 16), (300, 17, 3)]
    for (mm, nn, kk) in sizes:
        batch = 5
        args = _random_case(rng, trans, T, mm, nn, kk, batch, pad=3)
        A, aoff, ldA, B, boff, ldB, C, coff, ldC = args
        ref = C.copy()
        oracle.kgemm_batched(trans, mm, nn, kk, 0.7, A, aoff, ldA, B, boff, ldB, -0.4, ref, coff, ldC)
        got = _run_gpu(kmx, trans, A, aoff, ldA, B, boff, ldB, C, coff, ldC, mm, nn, kk, 0.7, -0.4)
        # compare the matrices; the padding rows below mm must be untouched
        gv = got.reshape(batch, nn, mm + 3)[:, :, :mm].reshape(batch, -1)
        rv = ref.reshape(batch, nn, mm + 3)[:, :, :mm].reshape(batch, -1)
        assert np.array_equal(got.reshape(batch, nn, mm + 3)[:, :, mm:],
                              C.reshape(batch, nn, mm + 3)[:, :, mm:])  # padding kept
        g64, r64 = gv.astype(np.float64), rv.astype(np.float64)
        if tag == "f64":
            err = _componentwise_err(trans, got, ref, A, aoff, ldA, B, boff, ldB, C, coff, ldC,
                                     mm, nn, kk, 0.7, -0.4)
            assert err <= F64_CW_TOL, (mm, nn, kk, err)
        else:
            err = blockwise_rel_err(g64, r64)
            assert err <= F32_NORM_TOL, (mm, nn, kk, err)


@pytest.mark.parametrize("beta", [0.0, 1.0, -0.4])
def test_kgemm_f32_dense_streaming_vs_oracle(kmx, oracle, beta):
    """FP32 nn with dense B and C (ldB == kk, ldC == mm) and a long column
    dimension: the chunk's columns move through shared memory as contiguous
    runs.  Ragged last chunks, kk = 1, and (beta == 1) every entry adding into
    one shared C."""
    rng = np.random.default_rng(12)
    T = np.float32
    for (mm, nn, kk) in [(4, 1024, 4), (5, 3125, 5), (16, 4096, 16), (6, 7776, 6), (1, 4097, 1),
                         (7, 2000, 3), (16, 300, 16), (3, 2187, 3), (12, 700, 9)]:
        batch = 4
        A = rng.standard_normal(batch * mm * kk).astype(T)
        B = rng.standard_normal(batch * kk * nn).astype(T)
        shared = beta == 1.0
        C = rng.standard_normal((1 if shared else batch) * mm * nn).astype(T)
        aoff = [i * mm * kk for i in range(batch)]
        boff = [i * kk * nn for i in range(batch)]
        coff = [0] * batch if shared else [i * mm * nn for i in range(batch)]
        ref = C.copy()
        oracle.kgemm_batched("nn", mm, nn, kk, 0.7, A, aoff, [mm] * batch, B, boff, [kk] * batch,
                             beta, ref, coff, [mm] * batch)
        got = _run_gpu(kmx, "nn", A, aoff, [mm] * batch, B, boff, [kk] * batch, C, coff,
                       [mm] * batch, mm, nn, kk, 0.7, beta)
        rows = 1 if shared else batch
        err = blockwise_rel_err(got.astype(np.float64).reshape(rows, -1),
                                ref.astype(np.float64).reshape(rows, -1))
        assert err <= F32_NORM_TOL, (mm, nn, kk, beta, err)


def test_kgemm_kk_zero_scales_c(kmx):
    """kk == 0: the product is empty and C becomes beta*C (beta == 0: zero)."""
    C = np.arange(1, 13, dtype=np.float64)
    for beta, expect in ((2.0, 2 * C), (0.0, 0 * C), (1.0, C)):
        got = _run_gpu(kmx, "nn", np.zeros(1), [0, 0], [3, 3], np.zeros(1), [0, 0], [1, 1],
                       C.copy(), [0, 6], [3, 3], 3, 2, 0, 1.5, beta)
        assert np.array_equal(got, expect)


def test_kgemm_null_entry_and_bad_ld_flagged(kmx):
    """A NULL entry pointer or a leading dimension below the row count is
    skipped and reported through the device status word; other entries run."""
    mm, nn, kk, batch = 4, 6, 3, 3
    A = torch.rand(batch * mm * kk, dtype=torch.float64, device="cuda")
    B = torch.rand(batch * kk * nn, dtype=torch.float64, device="cuda")
    C = torch.zeros(batch * mm * nn, dtype=torch.float64, device="cuda")
    pA = kmx.pointer_array(A, [i * mm * kk for i in range(batch)])
    pB = kmx.pointer_array(B, [i * kk * nn for i in range(batch)])
    pC = kmx.pointer_array(C, [i * mm * nn for i in range(batch)])
    pB[1] = 0
    i32 = lambda v: torch.tensor(v, dtype=torch.int32, device="cuda")  # noqa: E731
    kmx.kgemm_nn_batched(mm, nn, kk, 1.0, pA, i32([mm] * batch), pB, i32([kk] * batch), 0.0, pC,
                         i32([mm, mm, mm - 1]), batch)
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()
    c = C.cpu().numpy().reshape(batch, -1)
    assert c[0].any() and not c[1].any() and not c[2].any()
    assert kmx.check_device_status() == 0


def test_kgemm_graph_capture_replays(kmx):
    """The entry point makes no host synchronisation: it captures into a CUDA
    graph and a replay repeats the accumulation."""
    mm, nn, kk, batch = 4, 256, 4, 64
    A = torch.rand(batch * mm * kk, dtype=torch.float64, device="cuda")
    B = torch.rand(batch * kk * nn, dtype=torch.float64, device="cuda")
    C = torch.zeros(mm * nn, dtype=torch.float64, device="cuda")
    pA = kmx.pointer_array(A, [i * mm * kk for i in range(batch)])
    pB = kmx.pointer_array(B, [i * kk * nn for i in range(batch)])
    pC = kmx.pointer_array(C, [0] * batch)
    lA = torch.full((batch,), mm, dtype=torch.int32, device="cuda")
    lB = torch.full((batch,), kk, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    kmx.kgemm_nn_batched(mm, nn, kk, 1.0, pA, lA, pB, lB, 1.0, pC, lA, batch, stream=s)  # warm-up
    s.synchronize()
    once = C.clone()
    C.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        kmx.kgemm_nn_batched(mm, nn, kk, 1.0, pA, lA, pB, lB, 1.0, pC, lA, batch, stream=s)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    err = (C - 2 * once).abs().max().item() / once.abs().max().item()
    assert err < 1e-13


@pytest.mark.parametrize("trans", ["nn", "nt"])
@pytest.mark.parametrize("mm,nn,kk", [(4, 1024, 4), (1024, 4, 4), (3, 5, 7), (40, 70, 20)])
def test_kgemm_fp64_extreme_magnitudes_and_nonfinite(kmx, oracle, trans, mm, nn, kk):
    """Entries scaled by 1e-150..1e150 stay within the FP64 bound; an Inf in
    one entry's A and a NaN in another's B propagate as in the oracle; an
    all-zero A gives beta * C."""
    rng = np.random.default_rng(17 + mm)
    batch = 6
    args = _random_case(rng, trans, np.float64, mm, nn, kk, batch, pad=0)
    A, aoff, ldA, B, boff, ldB, C, coff, ldC = args
    sa = 10.0 ** rng.integers(-150, 151, batch)
    sb = 10.0 ** rng.integers(-150, 151, batch)
    na, nb = len(A) // batch, len(B) // batch
    for b in range(batch):
        A[b * na:(b + 1) * na] *= sa[b]
        B[b * nb:(b + 1) * nb] *= sb[b]
    C *= 1e-3
    A[1 * na + 2] = np.inf
    B[2 * nb + 1] = np.nan
    A[3 * na:4 * na] = 0.0
    ref = C.copy()
    oracle.kgemm_batched(trans, mm, nn, kk, 1.3, A, aoff, ldA, B, boff, ldB, 1.2, ref, coff, ldC)
    got = _run_gpu(kmx, trans, A, aoff, ldA, B, boff, ldB, C, coff, ldC, mm, nn, kk, 1.3, 1.2)
    g2, r2 = got.reshape(batch, -1), ref.reshape(batch, -1)
    assert np.array_equal(np.isnan(g2), np.isnan(r2))
    assert np.array_equal(np.isinf(g2), np.isinf(r2))
    fin = np.isfinite(r2).all(axis=1)
    assert fin.sum() >= 4
    idx = np.nonzero(fin)[0]
    sub = lambda X, off, n: np.concatenate([X[off[b]:off[b] + n] for b in idx])  # noqa: E731
    na_, nb_, nc_ = len(A) // batch, len(B) // batch, len(C) // batch
    offs = lambda n: [i * n for i in range(len(idx))]  # noqa: E731
    err = _componentwise_err(trans, sub(got, coff, nc_), sub(ref, coff, nc_), sub(A, aoff, na_),
                             offs(na_), [ldA[0]] * len(idx), sub(B, boff, nb_), offs(nb_),
                             [ldB[0]] * len(idx), sub(C, coff, nc_), offs(nc_),
                             [ldC[0]] * len(idx), mm, nn, kk, 1.3, 1.2)
    assert err <= F64_CW_TOL
