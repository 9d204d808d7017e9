"""Device-side construction of the xbatched arrays from (y, x, a) index
triples, and the xbatched call on the arrays it builds, against the oracle's
index-triple driver (kmo_xbatched_idx_f64)."""
import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _triples(rng, count, d, pool, nx, ny):
    y = (rng.geometric(0.2, count) * 7) % ny
    x = rng.integers(0, nx, count)
    a = rng.integers(0, pool, (count, d))
    return y.astype(np.int32), x.astype(np.int32), a.astype(np.int32)


@pytest.mark.parametrize("sort_by_y", [False, True])
def test_build_addresses(kmx, sort_by_y):
    rng = np.random.default_rng(5)
    d, n, pool, nx, ny, count = 4, 3, 7, 11, 13, 500
    N = n ** d
    Ap = torch.zeros((d, pool, n, n), dtype=torch.float64, device="cuda")
    Xp = torch.zeros((nx, N), dtype=torch.float64, device="cuda")
    Yp = torch.zeros((ny, N), dtype=torch.float64, device="cuda")
    y, x, a = _triples(rng, count, d, pool, nx, ny)
    pA, pX, pY = kmx.xbatched_build(d, Ap, pool * n * n, n * n, pool, Xp, N, nx, Yp, N, ny,
                                    torch.from_numpy(y).cuda(), torch.from_numpy(x).cuda(),
                                    torch.from_numpy(a).cuda(), sort_by_y=sort_by_y)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    order = np.argsort(y, kind="stable") if sort_by_y else np.arange(count)
    exp_y = Yp.data_ptr() + y[order].astype(np.int64) * N * 8
    exp_x = Xp.data_ptr() + x[order].astype(np.int64) * N * 8
    lvl = np.arange(d)[None, :]
    exp_a = Ap.data_ptr() + (lvl * pool * n * n + a[order].astype(np.int64) * n * n) * 8
    assert np.array_equal(pY.cpu().numpy(), exp_y)
    assert np.array_equal(pX.cpu().numpy(), exp_x)
    assert np.array_equal(pA.cpu().numpy(), exp_a.reshape(-1))


def test_build_out_of_range_index_is_null_and_flagged(kmx):
    d, n, pool, nx, ny = 3, 2, 4, 5, 6
    N = n ** d
    Ap = torch.zeros((d, pool, n, n), dtype=torch.float64, device="cuda")
    Xp = torch.zeros((nx, N), dtype=torch.float64, device="cuda")
    Yp = torch.zeros((ny, N), dtype=torch.float64, device="cuda")
    y = torch.tensor([0, 6, 2], dtype=torch.int32, device="cuda")   # 6 is out of range
    x = torch.tensor([1, 1, -1], dtype=torch.int32, device="cuda")  # -1 is out of range
    a = torch.tensor([[0, 1, 2], [3, 3, 3], [0, 0, 4]], dtype=torch.int32, device="cuda")
    pA, pX, pY = kmx.xbatched_build(d, Ap, pool * n * n, n * n, pool, Xp, N, nx, Yp, N, ny,
                                    y, x, a)
    torch.cuda.synchronize()
    with pytest.raises(kmx.KmxError):
        kmx.check_device_status()
    assert pY[1].item() == 0 and pX[2].item() == 0 and pA[2 * d + 2].item() == 0
    assert pY[0].item() != 0 and pA[2 * d + 1].item() != 0


@pytest.mark.parametrize("form", ["plain", "split"])
@pytest.mark.parametrize("sort_by_y", [False, True])
def test_build_then_xbatched_matches_oracle(kmx, oracle, form, sort_by_y):
    rng = np.random.default_rng(8)
    d, n, pool, nx, ny, count = 6, 4, 16, 24, 20, 600
    N = n ** d
    Apool = rng.standard_normal((d, pool, n, n)) / 2
    Xpool = rng.standard_normal((nx, N))
    y, x, a = _triples(rng, count, d, pool, nx, ny)
    Yref = np.zeros((ny, N))
    oracle.xbatched_idx(d, n, Apool, n, pool, Xpool, Yref, y, x, a)
    Ap = torch.from_numpy(Apool).cuda()
    Xp = torch.from_numpy(Xpool).cuda()
    Yp = torch.zeros((ny, N), dtype=torch.float64, device="cuda")
    pA, pX, pY = kmx.xbatched_build(d, Ap, pool * n * n, n * n, pool, Xp, N, nx, Yp, N, ny,
                                    torch.from_numpy(y).cuda(), torch.from_numpy(x).cuda(),
                                    torch.from_numpy(a).cuda(), sort_by_y=sort_by_y)
    kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, count, form=form)
    torch.cuda.synchronize()
    assert kmx.check_device_status() == 0
    err = blockwise_rel_err(Yp.cpu().numpy(), Yref)
    assert err <= 1e-13, err
