"""CPU tests of the oracle: pinned against the golden vectors produced by the
reference's own CPU build, and against an explicit-Kronecker evaluation."""
import os

import numpy as np
import pytest

from tests.common import blockwise_rel_err, golden, vb_cases


@pytest.fixture(scope="module")
def po1(oracle):
    oracle.set_threads(1)
    yield oracle
    oracle.set_threads(0)


@pytest.mark.parametrize("d", range(1, 7))
@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_batched_matches_golden_bitwise(po1, d, n):
    g = golden()
    N = n ** d
    for batch in (1, 3):
        A = po1.ramp_a(n, d, batch)
        X = po1.ramp_x(N, batch)
        Y = np.zeros_like(X)
        W = np.zeros_like(X)
        po1.batched(d, n, A, X.copy(), Y, W, batch)
        assert np.array_equal(Y, g[f"batched_d{d}_n{n}_b{batch}"])


@pytest.mark.parametrize("d", range(1, 7))
@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_pbatched_overlap_matches_golden(po1, d, n):
    g = golden()
    N = n ** d
    batch = 4
    A = po1.ramp_a(n, d, batch)
    X = po1.ramp_x(N, batch)
    Y = np.zeros((batch, N))
    W = np.zeros((batch, N))
    po1.pbatched(d, n, A, X.copy(), [b * N for b in range(batch)], Y, [0] * batch, W,
                 [b * N for b in range(batch)])
    assert np.array_equal(Y[0], g[f"pbatched_d{d}_n{n}_b{batch}"])
    assert not Y[1:].any()


@pytest.mark.parametrize("dtype,tag", [(np.float64, "f64"), (np.float32, "f32")])
@pytest.mark.parametrize("d", range(1, 7))
def test_xbatched_padded_lda_matches_golden(po1, dtype, tag, d):
    g = golden()
    for n in (1, 2, 3, 4):
        N = n ** d
        for batch in (1, 4):
            lda = n + 3
            A = po1.ramp_a(n, d, batch, lda=lda, dtype=dtype)
            X = po1.ramp_x(N, batch, dtype=dtype)
            X0 = X.copy()
            aoff = [[(b * d + l) * n * lda for l in range(d)] for b in range(batch)]
            Y = np.zeros(N, dtype=dtype)
            W = np.zeros((max(batch, 2), N), dtype=dtype)
            po1.xbatched(d, n, A, aoff, lda, X, [b * N for b in range(batch)], Y, [0] * batch, W,
                         [b * N for b in range(W.shape[0])])
            assert np.array_equal(Y, g[f"xbatched_{tag}_d{d}_n{n}_b{batch}"])
            if batch > 1:  # the reference preserves X when batch > 1
                assert np.array_equal(X, X0)


def _vb_inputs(g, ci, d):
    m, nn = g[f"vbatched_c{ci}_m"], g[f"vbatched_c{ci}_n"]
    A, X, Y0 = g[f"vbatched_c{ci}_A"], g[f"vbatched_c{ci}_X"], g[f"vbatched_c{ci}_Y0"]
    fsz = [int(m[l] * nn[l]) for l in range(d)]
    aoff, o = [], 0
    for b in range(X.shape[0]):
        row = []
        for l in range(d):
            row.append(o)
            o += fsz[l]
        aoff.append(row)
    return m, nn, A, X, Y0, aoff, fsz


@pytest.mark.parametrize("ci,d", vb_cases())
def test_vbatched_rectangular_matches_golden(po1, ci, d):
    g = golden()
    m, nn, A, X, Y0, aoff, fsz = _vb_inputs(g, ci, d)
    batch, Nx = X.shape
    Ny = Y0.shape[1]
    for T, tag in ((np.float64, "f64"), (np.float32, "f32")):
        Y = Y0.astype(T).copy()
        W = np.zeros(2 * po1.size_xw(d, m, nn) * 2, dtype=T)
        po1.vbatched(d, m, nn, A.astype(T), aoff, X.astype(T), [b * Nx for b in range(batch)], Y,
                     [b * Ny for b in range(batch)], W)
        assert np.array_equal(Y, g[f"vbatched_{tag}_c{ci}"])
    # and the recursion agrees with the explicit Kronecker product
    for b in range(batch):
        fs = [A[aoff[b][l]: aoff[b][l] + fsz[l]] for l in range(d)]
        ye = po1.explicit_kron(d, m, nn, fs, m, X[b])
        assert blockwise_rel_err(g[f"vbatched_f64_c{ci}"][b], Y0[b] + ye) < 1e-14


@pytest.mark.parametrize("d", range(1, 7))
def test_recursion_matches_explicit_kron_random(po1, d):
    rng = np.random.default_rng(7 + d)
    for n in (2, 3, 4) if d <= 4 else (2, 3):
        fs = [rng.standard_normal(n * n) for _ in range(d)]
        x = rng.standard_normal(n ** d)
        y = np.zeros(n ** d)
        po1.kronmultv(d, [n] * d, [n] * d, fs, [n] * d, x, y)
        ye = po1.explicit_kron(d, [n] * d, [n] * d, fs, [n] * d, x)
        assert blockwise_rel_err(y, ye) < 1e-14


def test_oracle_matches_reference_build_random(oracle):
    """The C restatement and the reference's own templates agree bit for bit
    on non-overlapping random inputs (where the reference tree was built)."""
    if oracle.ref_lib() is None:
        pytest.skip("reference CPU build not available on this machine")
    rng = np.random.default_rng(3)
    for d in range(1, 7):
        n = 3 if d > 4 else 4
        N = n ** d
        batch = 5
        A = rng.standard_normal((batch, d, n, n))
        X = rng.standard_normal((batch, N))
        outs = []
        for lib in (None, "ref"):
            Y = np.zeros_like(X)
            oracle.batched(d, n, A, X.copy(), Y, np.zeros_like(X), batch, lib=lib)
            outs.append(Y)
        assert np.array_equal(outs[0], outs[1])


def test_kron_flops_square(oracle):
    for d in range(1, 7):
        for n in (1, 2, 4, 5):
            assert oracle.kron_flops(d, [n] * d, [n] * d) == 2.0 * d * n ** (d + 1)


def test_planted_mistake_is_caught(po1):
    """A one-ulp change in one factor entry of the oracle's input must move the
    result away from the golden vector: the comparison is not vacuous."""
    g = golden()
    d, n, batch = 4, 3, 3
    N = n ** d
    A = po1.ramp_a(n, d, batch)
    A[1, 2, 1, 0] = np.nextafter(A[1, 2, 1, 0], 1.0)
    X = po1.ramp_x(N, batch)
    Y = np.zeros_like(X)
    po1.batched(d, n, A, X.copy(), Y, np.zeros_like(X), batch)
    assert not np.array_equal(Y, g[f"batched_d{d}_n{n}_b{batch}"])


# ---------------------------------------------------------------------------
# kgemm_{nn,nt}_batched
# ---------------------------------------------------------------------------

def _kgemm_cases():
    from tests.golden import make_kgemm_golden as mk

    for trans in ("nn", "nt"):
        for tag in ("f64", "f32"):
            for shape in mk.SHAPES:
                for bname, beta in mk.BETAS:
                    if bname != "b12" and shape not in mk.ALL_BETAS:
                        continue
                    yield trans, tag, shape, bname, beta


def test_kgemm_oracle_matches_golden_bitwise(po1):
    from tests.golden import make_kgemm_golden as mk

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "kgemm_golden.npz"))
    n = 0
    for trans, tag, (mm, nn, kk, batch), bname, beta in _kgemm_cases():
        T = np.float64 if tag == "f64" else np.float32
        got = mk.run(trans, T, mm, nn, kk, batch, beta, lib=None)
        ref = g[mk.case_key(trans, tag, mm, nn, kk, batch, bname)]
        assert got.dtype == ref.dtype and np.array_equal(got, ref), (trans, tag, mm, nn, kk, bname)
        n += 1
    for trans in ("nn", "nt"):
        for tag, T in (("f64", np.float64), ("f32", np.float32)):
            got = mk.run(trans, T, 8, 15, 22, 8, 1.0, shared_c=True, lib=None)
            assert np.array_equal(got, g[f"{trans}_{tag}_shared_8x15x22_b8"])
    assert n == 56


@pytest.mark.parametrize("trans", ["nn", "nt"])
def test_kgemm_oracle_closed_form_sweep(oracle, trans):
    """The reference test's own check (test_kgemm_nn_batched.cpp:458-487,
    main_func :525-560): C = alpha*A*op(B) + beta*1 against a direct sum,
    max abs error below 1e-9 (FP64) / 5e-4 (FP32), alpha 1.3, beta 1.2, over
    mm, nn, kk in 1..65 step 7 (every other step here) and batch 1, 8, 15."""
    for T, tol in ((np.float64, 1e-9), (np.float32, 5e-4)):
        for batch in (1, 8, 15):
            for kk in range(1, 66, 14):
                for nn in range(1, 66, 14):
                    for mm in range(1, 66, 14):
                        A, B, Cm = oracle.ramp_kgemm(trans, mm, nn, kk, batch, dtype=T)
                        C = Cm.copy()
                        ldb = kk if trans == "nn" else nn
                        oracle.kgemm_batched(trans, mm, nn, kk, 1.3, A.reshape(-1),
                                             [i * mm * kk for i in range(batch)], [mm] * batch,
                                             B.reshape(-1), [i * B.shape[1] for i in range(batch)],
                                             [ldb] * batch, 1.2, C.reshape(-1),
                                             [i * mm * nn for i in range(batch)], [mm] * batch)
                        Ad = A.astype(np.float64).reshape(batch, kk, mm).transpose(0, 2, 1)
                        Bd = B.astype(np.float64)
                        # op(B) indexed [b, k, j]: B is kk x nn (nn) or nn x kk (nt), column-major
                        Bm = (Bd.reshape(batch, nn, kk).transpose(0, 2, 1) if trans == "nn"
                              else Bd.reshape(batch, kk, nn))
                        exact = 1.3 * np.einsum("bik,bkj->bij", Ad, Bm) + 1.2
                        got = C.astype(np.float64).reshape(batch, nn, mm).transpose(0, 2, 1)
                        assert np.abs(got - exact).max() < tol, (T, batch, mm, nn, kk)
