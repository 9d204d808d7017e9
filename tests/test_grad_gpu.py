"""Backward pass: the fused kernel against an explicit-Kronecker gradient,
FP64 central differences, and torch.autograd.gradcheck."""
import numpy as np
import pytest

from tests.common import blockwise_rel_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def explicit_grads(A, X, G):
    """dX, dA of sum(G * (K X)) with K = kron(A_1..A_d) built explicitly.
    A: (batch, d, n, n) with A[b, l].T the factor (column-major storage)."""
    batch, d, n, _ = A.shape
    dX = np.zeros_like(X)
    dA = np.zeros_like(A)
    for b in range(batch):
        mats = [A[b, l].T for l in range(d)]
        K = mats[0]
        for m in mats[1:]:
            K = np.kron(K, m)
        dX[b] = K.T @ G[b]
        dK = np.outer(G[b], X[b]).reshape([n] * (2 * d))  # [i_1..i_d, j_1..j_d]
        for k in range(d):
            t = dK
            # contract every mode l != k with A_l(i_l, j_l)
            letters = "abcdefghijklmnopqrstuvwxyz"
            ii, jj = letters[:d], letters[d:2 * d]
            ops, subs = [t], [ii + jj]
            for l in range(d):
                if l != k:
                    ops.append(mats[l])
                    subs.append(ii[l] + jj[l])
            g = np.einsum(",".join(subs) + "->" + ii[k] + jj[k], *ops)
            dA[b, k] = g.T  # column-major storage
    return dX, dA


GRAD_FORMS = ["split", "plain"]  # double-float (the default for FP64) and native FP64


@pytest.mark.parametrize("form", GRAD_FORMS)
@pytest.mark.parametrize("d,n", [(1, 3), (2, 4), (3, 3), (4, 2), (3, 5), (2, 7), (3, 8), (4, 6)])
def test_fused_grad_vs_explicit_kron(kmx, d, n, form):
    from kronmult_gb300.autograd import kronmult_fused_grad

    rng = np.random.default_rng(d * 10 + n)
    batch, N = 3, n ** d
    A = rng.standard_normal((batch, d, n, n))
    X = rng.standard_normal((batch, N))
    G = rng.standard_normal((batch, N))
    Y, dX, dA = kronmult_fused_grad(*(torch.from_numpy(t).cuda() for t in (A, X, G)), form=form)
    ex_dX, ex_dA = explicit_grads(A, X, G)
    assert blockwise_rel_err(dX.cpu().numpy(), ex_dX) <= 1e-13
    assert blockwise_rel_err(dA.cpu().numpy().reshape(batch, -1), ex_dA.reshape(batch, -1)) <= 1e-13
    # forward output of the fused kernel equals the forward entry point
    Y2 = torch.zeros_like(Y)
    kmx.kronmult_batched(d, n, torch.from_numpy(A).cuda(), torch.from_numpy(X).cuda(), Y2, None,
                         batch, form="plain")
    assert blockwise_rel_err(Y.cpu().numpy(), Y2.cpu().numpy()) <= (1e-14 if form == "plain"
                                                                     else 1e-13)


@pytest.mark.parametrize("form", GRAD_FORMS)
@pytest.mark.parametrize("d,n,batch", [(6, 5, 3), (3, 8, 8), (6, 4, 4)])
def test_fused_grad_central_differences(kmx, d, n, batch, form):
    """64 random coordinates of X and of each A_i, h = 1e-6: the loss is linear
    in every single coordinate, so central differences are exact up to rounding."""
    from kronmult_gb300.autograd import kronmult_fused_grad

    rng = np.random.default_rng(100 + d * n)
    N = n ** d
    A = torch.from_numpy(rng.standard_normal((batch, d, n, n)) / np.sqrt(n)).cuda()
    X = torch.from_numpy(rng.standard_normal((batch, N))).cuda()
    G = torch.from_numpy(rng.standard_normal((batch, N))).cuda()
    _, dX, dA = kronmult_fused_grad(A, X, G, want_y=False, form=form)

    def loss(Av, Xv, b):
        # only entry b depends on the perturbed coordinate
        Y = torch.zeros_like(Xv)
        kmx.kronmult_batched(d, n, Av, Xv, Y, None, batch, form="plain")
        return float((G[b] * Y[b]).sum())

    h = 1e-6
    for name, T, grad in [("X", X, dX)] + [(f"A{k}", A, dA) for k in range(d)]:
        idx = []
        for _ in range(64):
            if name == "X":
                idx.append((int(rng.integers(batch)), int(rng.integers(N))))
            else:
                k = int(name[1:])
                idx.append((int(rng.integers(batch)), k, int(rng.integers(n)), int(rng.integers(n))))
        for ix in idx:
            old = float(T[ix])
            T[ix] = old + h
            lp = loss(A, X, ix[0])
            T[ix] = old - h
            lm = loss(A, X, ix[0])
            T[ix] = old
            fd = (lp - lm) / (2 * h)
            g = float(grad[ix])
            assert abs(fd - g) <= 1e-6 * (1 + abs(g)), (name, ix, fd, g)


def test_autograd_function_gradcheck(kmx):
    from kronmult_gb300.autograd import kronmult

    rng = np.random.default_rng(3)
    A = torch.from_numpy(rng.standard_normal((2, 3, 2, 2))).cuda().requires_grad_()
    X = torch.from_numpy(rng.standard_normal((2, 8))).cuda().requires_grad_()
    assert torch.autograd.gradcheck(lambda a, x: kronmult(a, x, "plain"), (A, X), eps=1e-6,
                                    atol=1e-8, rtol=1e-6)


def test_autograd_backward_matches_fused(kmx):
    from kronmult_gb300.autograd import kronmult, kronmult_fused_grad

    rng = np.random.default_rng(4)
    A = torch.from_numpy(rng.standard_normal((5, 4, 3, 3))).cuda().requires_grad_()
    X = torch.from_numpy(rng.standard_normal((5, 81))).cuda().requires_grad_()
    G = torch.from_numpy(rng.standard_normal((5, 81))).cuda()
    Y = kronmult(A, X)
    Y.backward(G)
    _, dX, dA = kronmult_fused_grad(A.detach(), X.detach(), G)
    # the Gram reductions use shared-memory atomics: equal up to summation order
    assert blockwise_rel_err(X.grad.cpu().numpy(), dX.cpu().numpy()) <= 1e-14
    assert blockwise_rel_err(A.grad.reshape(5, -1).cpu().numpy(),
                             dA.reshape(5, -1).cpu().numpy()) <= 1e-14


@pytest.mark.parametrize("form", GRAD_FORMS)
@pytest.mark.parametrize("d,n,batch", [(6, 5, 1024), (3, 8, 4096)])
def test_fused_grad_fullsize_identities(kmx, d, n, batch, form):
    """At the benchmark sizes, exact identities instead of differences:
    Y equals the forward, dX equals the transposed forward of G, and for each
    mode k, K is linear in A_k, so sum(G * K(A with A_k := E) X) = <dA_k, E>
    entry by entry."""
    from kronmult_gb300.autograd import kronmult_fused_grad

    g = torch.Generator(device="cuda").manual_seed(40 + d)
    A = torch.randn((batch, d, n, n), dtype=torch.float64, device="cuda", generator=g) / n ** 0.5
    X = torch.randn((batch, n ** d), dtype=torch.float64, device="cuda", generator=g)
    G = torch.randn((batch, n ** d), dtype=torch.float64, device="cuda", generator=g)
    Y, dX, dA = kronmult_fused_grad(A, X, G, form=form)
    torch.cuda.synchronize()
    Yf = torch.zeros_like(X)
    kmx.kronmult_batched(d, n, A, X, Yf, None, batch, form="plain")
    dXf = torch.zeros_like(X)
    kmx.kronmult_batched(d, n, A, G, dXf, None, batch, form="plain", transpose=True)
    torch.cuda.synchronize()

    def rel(a, b):
        return float((torch.linalg.vector_norm(a - b, dim=1) /
                      torch.linalg.vector_norm(b, dim=1).clamp_min(1e-300)).max())

    assert rel(Y, Yf) <= 1e-13
    assert rel(dX, dXf) <= 1e-13
    E = torch.randn((batch, n, n), dtype=torch.float64, device="cuda", generator=g)
    for k in range(d):
        Ak = A.clone()
        Ak[:, k] = E
        Z = torch.zeros_like(X)
        kmx.kronmult_batched(d, n, Ak, X, Z, None, batch, form="plain")
        torch.cuda.synchronize()
        lhs = (G * Z).sum(dim=1)
        rhs = (dA[:, k] * E).sum(dim=(1, 2))
        scale = torch.linalg.vector_norm(G, dim=1) * torch.linalg.vector_norm(Z, dim=1)
        assert float(((lhs - rhs).abs() / scale).max()) <= 1e-13, k
    assert kmx.check_device_status() == 0


def test_split_grad_special_entries_run_fp64(kmx):
    """Entries with Inf/NaN, or an all-zero X, G or factor, are evaluated in FP64
    by the double-float kernel: NaN/Inf land where FP64 puts them and the zero
    cases match the FP64 kernel; the other entries stay within tolerance."""
    from kronmult_gb300.autograd import kronmult_fused_grad

    rng = np.random.default_rng(77)
    d, n, batch = 4, 5, 6
    N = n ** d
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    G = rng.standard_normal((batch, N))
    X[1, 7] = np.inf
    A[2, 1, 0, 3] = np.nan
    A[3, 2] = 0.0     # zero factor: dA_2 of entry 3 is still nonzero
    X[4] = 0.0        # zero X: dX of entry 4 is still nonzero
    G[5] = 0.0
    T = [torch.from_numpy(t).cuda() for t in (A, X, G)]
    Ys, dXs, dAs = kronmult_fused_grad(*T, form="split")
    Yp, dXp, dAp = kronmult_fused_grad(*T, form="plain")
    for s_, p_ in ((Ys, Yp), (dXs, dXp), (dAs.reshape(batch, -1), dAp.reshape(batch, -1))):
        s_, p_ = s_.cpu().numpy(), p_.cpu().numpy()
        assert np.array_equal(np.isnan(s_), np.isnan(p_))
        assert np.array_equal(np.isinf(s_), np.isinf(p_))
        for b in (0, 3, 4, 5):
            assert np.array_equal(s_[b], p_[b]) or blockwise_rel_err(s_[b:b + 1], p_[b:b + 1]) <= 1e-13
    assert np.array_equal(dAs[3].cpu().numpy(), dAp[3].cpu().numpy())  # FP64 path taken
    assert np.abs(dAs[3, 2].cpu().numpy()).max() > 0


# Shapes the warp-per-entry fused kernel takes (d >= 3 with the entry's
# factors and intermediates in 32 KB of shared memory).
WARP_SHAPES = [(3, 2), (3, 3), (3, 4), (3, 5), (3, 6), (3, 7), (3, 8), (4, 2), (4, 3), (4, 4),
               (4, 5), (5, 2), (5, 3), (6, 2)]


@pytest.mark.parametrize("form", GRAD_FORMS)
@pytest.mark.parametrize("d,n", WARP_SHAPES)
def test_warp_kernel_vs_explicit_and_cta_kernel(kmx, d, n, form):
    """The warp-per-entry kernel (the default for these shapes) against the
    explicit-Kronecker gradient, and against the CTA-per-entry kernel (engine
    "per_mode") on a batch that leaves the last CTA's warps partly idle, with
    nonzero outputs to accumulate into."""
    from kronmult_gb300.autograd import _grad_call

    rng = np.random.default_rng(1000 + 10 * d + n)
    batch, N = 37, n ** d
    A = rng.standard_normal((batch, d, n, n)) / np.sqrt(n)
    X = rng.standard_normal((batch, N))
    G = rng.standard_normal((batch, N))
    Y0 = rng.standard_normal((batch, N))
    dX0 = rng.standard_normal((batch, N))
    dA0 = rng.standard_normal((batch, d, n, n))
    At, Xt, Gt = (torch.from_numpy(t).cuda() for t in (A, X, G))
    out = {}
    for eng in ("tuned", "per_mode"):
        Y, dX, dA = (torch.from_numpy(t.copy()).cuda() for t in (Y0, dX0, dA0))
        _grad_call(d, n, At, Xt, Gt, Y, dX, dA, None, form, eng)
        torch.cuda.synchronize()
        out[eng] = [t.cpu().numpy() for t in (Y, dX, dA)]
    assert kmx.check_device_status() == 0
    ex_dX, ex_dA = explicit_grads(A[:5], X[:5], G[:5])
    w = out["tuned"]
    assert blockwise_rel_err(w[1][:5] - dX0[:5], ex_dX) <= 1e-13
    assert blockwise_rel_err((w[2][:5] - dA0[:5]).reshape(5, -1), ex_dA.reshape(5, -1)) <= 1e-13
    for a, b in zip(out["tuned"], out["per_mode"]):
        assert blockwise_rel_err(a.reshape(batch, -1), b.reshape(batch, -1)) <= 1e-13
