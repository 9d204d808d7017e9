"""Every row of the committed tuning table, run on the GPU through the C ABI
and checked against the oracle: once as a default call (engine TUNED, so the
library applies the row's engine and launch shape itself) and once with the
row's engine and launch shape passed explicitly.  Batched rows use the batched
entry point; pointer rows use xbatched with Y blocks shared by two entries
(atomic accumulation).  Tolerances: 1e-13 normwise per Y block for FP64 (plain
and double-float), 1e-5 for FP32 fused multiply-add."""
import json

import numpy as np
import pytest

from kronmult_gb300 import tune
from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

with open(tune.TABLE) as _f:
    ROWS = json.load(_f)["rows"]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _row_id(r):
    return f"{r['form']}-{r.get('layout', 'batched')}-d{r['d']}n{r['n']}-{r['engine']}"


@pytest.mark.parametrize("row", ROWS, ids=[_row_id(r) for r in ROWS])
def test_table_row_matches_oracle(kmx, oracle, row):
    d, n, form, layout = row["d"], row["n"], row["form"], row.get("layout", "batched")
    N = n ** d
    f32 = form == "f32"
    dt = np.float32 if f32 else np.float64
    kform = "plain" if f32 else form
    tol = 1e-5 if f32 else 1e-13
    launch = tuple(int(row.get(k, 0)) for k in ("group_threads", "groups_per_cta", "ctas_per_sm"))
    rng = np.random.default_rng(1000 * d + 10 * n + len(form) + (layout == "pointer"))
    batch = max(2, min(24, 131072 // N))
    A = (rng.standard_normal((batch, d, n, n)) / 2).astype(dt)
    X = rng.standard_normal((batch, N)).astype(dt)
    W = np.zeros_like(X) if N * X.itemsize > 200 * 1024 else None
    if layout == "batched":
        Y0 = rng.uniform(-1, 1, (batch, N)).astype(dt)
        Yref = Y0.astype(np.float64)
        oracle.batched(d, n, A.astype(np.float64), X.astype(np.float64), Yref,
                       np.zeros((batch, N)), batch)
        for engine, lt in (("tuned", None), (row["engine"], launch)):
            Yd = dev(Y0)
            kmx.kronmult_batched(d, n, dev(A), dev(X), Yd, None if W is None else dev(W), batch,
                                 form=kform, engine=engine, launch=lt)
            assert kmx.check_device_status() == 0
            y = Yd.cpu().numpy().astype(np.float64)
            assert blockwise_rel_err(y - Y0, Yref - Y0) <= tol, (engine, lt)
    else:
        ny = max(1, batch // 2)
        y_idx = np.arange(batch) % ny
        Y0 = rng.uniform(-1, 1, (ny, N)).astype(dt)
        Yref = Y0.astype(np.float64)
        for e in range(batch):
            y = np.zeros(N)
            oracle.kronmultv(d, [n] * d, [n] * d, [A[e, l].astype(np.float64).ravel() for l in range(d)],
                             [n] * d, X[e].astype(np.float64).copy(), y)
            Yref[y_idx[e]] += y
        Ad, Xd = dev(A), dev(X)
        pA = kmx.pointer_array(Ad, np.arange(batch * d) * n * n)
        pX = kmx.pointer_array(Xd, np.arange(batch) * N)
        Wd = None if W is None else dev(W)
        pW = None if Wd is None else kmx.pointer_array(Wd, np.arange(batch) * N)
        for engine, lt in (("tuned", None), (row["engine"], launch)):
            Yd = dev(Y0)
            pY = kmx.pointer_array(Yd, y_idx * N)
            kmx.kronmult_xbatched(d, n, pA, n, pX, pY, pW, batch, dtype=torch.float32 if f32 else None,
                                  form=kform, engine=engine, launch=lt)
            assert kmx.check_device_status() == 0
            y = Yd.cpu().numpy().astype(np.float64)
            assert blockwise_rel_err(y - Y0, Yref - Y0) <= tol, (engine, lt)
