"""The bounded wait of the register-tiled kernels, made to run out.

Each group of the register-tiled kernels waits (on an mbarrier, at most about
2 s of %globaltimer) for the bulk copy that stages its next X block in shared
memory.  When a wait runs out the group must not leave with that copy still
in flight: it waits for the copy once more under the same bound, sets
DF_WAIT_TIMEOUT in the device status word and returns without touching Y.

The host-side test hook KMX_TEST_EXPIRE_WAITS=1 makes every group's first
wait report that it ran out (no real stall, no fault), so the whole path runs:
afterwards the status word holds DF_WAIT_TIMEOUT, every Y block is bitwise
unchanged, and the next call (hook off) is correct against the oracle."""
import ctypes as C

import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

DF_WAIT_TIMEOUT = 2


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _status_flags(kmx):
    flags = C.c_int(0)
    kmx.lib().kmx_check_device_status(None, C.byref(flags))  # reads and clears
    return flags.value


@pytest.mark.parametrize("form", ["split", "plain"])
def test_expired_wait_drains_the_copy_and_leaves_y_untouched(kmx, oracle, monkeypatch, form):
    d, n, batch = 6, 4, 96  # register-tiled kernel, X blocks staged by bulk copy
    N = n ** d
    rng = np.random.default_rng(61)
    A = rng.standard_normal((batch, d, n, n)) / 2
    X = rng.standard_normal((batch, N))
    Y0 = rng.standard_normal((batch, N))
    At, Xt = torch.from_numpy(A).cuda(), torch.from_numpy(X).cuda()
    Y = torch.from_numpy(Y0).cuda()
    _status_flags(kmx)
    monkeypatch.setenv("KMX_TEST_EXPIRE_WAITS", "1")
    kmx.kronmult_batched(d, n, At, Xt, Y, None, batch, form=form)
    torch.cuda.synchronize()
    assert _status_flags(kmx) & DF_WAIT_TIMEOUT
    assert torch.equal(Y.cpu(), torch.from_numpy(Y0))
    # the context stays usable: the same call without the hook is correct
    monkeypatch.delenv("KMX_TEST_EXPIRE_WAITS")
    kmx.kronmult_batched(d, n, At, Xt, Y, None, batch, form=form)
    torch.cuda.synchronize()
    assert _status_flags(kmx) == 0
    Yref = Y0.copy()
    oracle.batched(d, n, A, X.copy(), Yref, np.zeros_like(X), batch)
    assert blockwise_rel_err(Y.cpu().numpy() - Y0, Yref - Y0) <= 1e-13
