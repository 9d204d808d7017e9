"""torch.autograd.Function over the C ABI's forward and fused backward.

Layout (the reference's batched layout, kronmult6_batched.hpp:14-94):
  A: (batch, d, n, n) tensor whose [b, l] slice holds factor A_l of entry b in
     COLUMN-major order, i.e. A[b, l, j, i] = A_l(i, j) (A[b, l].T is the matrix);
  X: (batch, n**d); the result Y has the same shape.

Forward runs the tuned forward kernel; backward runs the fused kernel that
recomputes the forward intermediates on chip (nothing is stored between the
two) and returns dA, dX -- in double-float for FP64 data unless the forward
asked for form="plain".
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib, kronmult_batched


def _grad_call(d, n, A, X, G, Y, dX, dA, W, form=None, engine=None):
    L = _lib.lib()
    f64 = A.dtype == torch.float64

    def a(t):
        return t.data_ptr() if t is not None else None

    cap = W.numel() * W.element_size() if W is not None else 0
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if f64:
        opt = None
        if form is not None or engine is not None:
            opt = C.byref(_lib.options(form if form is not None else "auto",
                                       engine=engine if engine is not None else "tuned"))
        rc = L.kmx_kronmult_batched_grad_f64_ex(d, n, a(A), a(X), a(G), a(Y), a(dX), a(dA), a(W),
                                                cap, A.shape[0], opt, s)
    else:
        rc = L.kmx_kronmult_batched_grad_f32(d, n, a(A), a(X), a(G), a(Y), a(dX), a(dA), a(W),
                                             cap, A.shape[0], s)
    _lib.check(rc, "kmx_kronmult_batched_grad")


def grad_workspace(d, n, batch, dtype=torch.float64, device="cuda"):
    """Workspace for the fused backward (None when an entry's intermediates
    fit in shared memory); the library reports the size it wants."""
    f64 = dtype == torch.float64
    nbytes = _lib.lib().kmx_grad_workspace_bytes(d, n, batch, 1 if f64 else 0)
    if nbytes == 0:
        return None
    esz = 8 if f64 else 4
    return torch.empty((nbytes + esz - 1) // esz, dtype=dtype, device=device)


def kronmult_fused_grad(A, X, G, want_y=True, form=None, engine=None):
    """Y, dX, dA of loss = sum(G * Y) in one launch.  form: None (the library
    default: double-float for FP64), "split", or "plain" (native FP64).
    engine: None (one warp per entry where the entry fits, else a CTA per
    entry) or "per_mode" (a CTA per entry)."""
    batch, d, n, _ = A.shape
    Y = torch.zeros_like(X) if want_y else None
    dX = torch.zeros_like(X)
    dA = torch.zeros_like(A)
    _grad_call(d, n, A.contiguous(), X.contiguous(), G.contiguous(), Y, dX, dA,
               grad_workspace(d, n, batch, A.dtype), form, engine)
    return Y, dX, dA


class KronmultFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, X, form=None):
        batch, d, n, _ = A.shape
        A = A.contiguous()
        X = X.contiguous()
        Y = torch.zeros_like(X)
        kronmult_batched(d, n, A, X, Y, None, batch, form=form)
        ctx.save_for_backward(A, X)
        ctx.form = form
        return Y

    @staticmethod
    def backward(ctx, G):
        A, X = ctx.saved_tensors
        batch, d, n, _ = A.shape
        need_a, need_x = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        dX = torch.zeros_like(X) if need_x else None
        dA = torch.zeros_like(A) if need_a else None
        # the backward follows the forward's arithmetic form ("plain": FP64)
        form = "plain" if ctx.form == "plain" else None
        _grad_call(d, n, A, X, G.contiguous(), None, dX, dA, grad_workspace(d, n, batch, A.dtype),
                   form)
        return dA, dX, None


def kronmult(A, X, form=None):
    """Differentiable Y = kron(A_1, ..., A_d) X per entry (see module doc)."""
    return KronmultFunction.apply(A, X, form)
