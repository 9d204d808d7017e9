"""FP32 entry points against the reference's float semantics, per element in
FP32 ulps.

The reference's float kernels accumulate every dot product in double and
round it once when storing (kgemm_nt.hpp:557-571, kgemm_nn.hpp:688-701),
stage by stage in its mode order (A1 first), and add each entry's
contribution to Y with a float atomic.  The FP32 entry points' default form
does the same rounding (exact products summed as an FP32 pair, rounded once),
so against the golden outputs of the reference's own build:
  - within one FP32 ulp per element, with overlapping Y blocks summed in the
    reference's entry order (deterministic mode);
and against the oracle (the same semantics, restated in C) on random data:
  - at most one ulp on all but a few elements (a one-ulp tie difference in a
    middle stage can grow to a few ulps where the next stages cancel).
Form PLAIN (FP32 fused multiply-add) is the fast form and only holds the
reference test's 1e-5 metric.  Every call goes through the C ABI."""
import numpy as np
import pytest

from tests.common import golden, ref_test_err, vb_cases

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def ulps(y, ref):
    """|y - ref| in units of the FP32 spacing at |ref| (exact zeros must match)."""
    y = np.asarray(y, dtype=np.float64).ravel()
    ref32 = np.asarray(ref, dtype=np.float32).ravel()
    sp = np.spacing(np.abs(ref32)).astype(np.float64)
    return np.abs(y - ref32.astype(np.float64)) / sp


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("d", range(1, 7))
def test_f32_xbatched_golden_within_one_ulp(kmx, oracle, d):
    g = golden()
    for n in (1, 2, 3, 4):
        N = n ** d
        for batch in (1, 4):
            lda = n + 3
            Ab = dev(oracle.ramp_a(n, d, batch, lda=lda, dtype=np.float32))
            X = dev(oracle.ramp_x(N, batch, dtype=np.float32))
            Y = torch.zeros(N, dtype=torch.float32, device="cuda")
            pA = kmx.pointer_array(Ab, [(b * d + l) * n * lda for b in range(batch) for l in range(d)])
            pX = kmx.pointer_array(X, [b * N for b in range(batch)])
            pY = kmx.pointer_array(Y, [0] * batch)  # every entry adds to one block
            kmx.kronmult_xbatched(d, n, pA, lda, pX, pY, None, batch, dtype=torch.float32,
                                  accumulate="deterministic")
            y = Y.cpu().numpy()
            ref = g[f"xbatched_f32_d{d}_n{n}_b{batch}"]
            assert ulps(y, ref).max() <= 1.0, (n, batch, float(ulps(y, ref).max()))
    assert kmx.check_device_status() == 0


@pytest.mark.parametrize("ci,d", vb_cases())
def test_f32_vbatched_golden_within_one_ulp(kmx, ci, d):
    g = golden()
    m, nn = g[f"vbatched_c{ci}_m"], g[f"vbatched_c{ci}_n"]
    A, X, Y0 = g[f"vbatched_c{ci}_A"], g[f"vbatched_c{ci}_X"], g[f"vbatched_c{ci}_Y0"]
    batch, Nx = X.shape
    Ny = Y0.shape[1]
    fsz = [int(m[l] * nn[l]) for l in range(d)]
    offs, o = [], 0
    for b in range(batch):
        for l in range(d):
            offs.append(o)
            o += fsz[l]
    Ad, Xd, Yd = dev(A.astype(np.float32)), dev(X.astype(np.float32)), dev(Y0.astype(np.float32))
    pA = kmx.pointer_array(Ad, offs)
    pX = kmx.pointer_array(Xd, [b * Nx for b in range(batch)])
    pY = kmx.pointer_array(Yd, [b * Ny for b in range(batch)])
    W = torch.zeros(1 << 16, dtype=torch.float32, device="cuda")
    kmx.kronmult_vbatched(d, m, nn, pA, pX, pY, W, None, batch, dtype=torch.float32)
    y = Yd.cpu().numpy()
    ref = g[f"vbatched_f32_c{ci}"]
    assert ulps(y, ref).max() <= 1.0, float(ulps(y, ref).max())
    assert kmx.check_device_status() == 0


@pytest.mark.parametrize("d,n", [(1, 8), (2, 9), (3, 8), (4, 5), (5, 4), (6, 4), (3, 16), (5, 8)])
def test_f32_random_vs_oracle_in_ulps(kmx, oracle, d, n):
    rng = np.random.default_rng(4100 + 10 * d + n)
    N = n ** d
    batch = 6 if N <= 40000 else 2
    A = (rng.standard_normal((batch, d, n, n)) / np.sqrt(n)).astype(np.float32)
    X = rng.standard_normal((batch, N)).astype(np.float32)
    Y0 = rng.uniform(-1, 1, (batch, N)).astype(np.float32)
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    Yd = dev(Y0)
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, torch.zeros_like(Yd), batch)
    u = ulps(Yd.cpu().numpy(), Yref)
    assert np.mean(u <= 1.0) >= 0.999, (float(np.mean(u <= 1.0)), float(u.max()))
    assert u.max() <= 8.0, float(u.max())
    # the fast form: FP32 FMA, the reference test's metric only
    Yp = dev(Y0)
    kmx.kronmult_batched(d, n, dev(A), dev(X), Yp, torch.zeros_like(Yp), batch, form="plain")
    assert ref_test_err(Yp.cpu().numpy(), Yref) <= 1e-5
    assert kmx.check_device_status() == 0
