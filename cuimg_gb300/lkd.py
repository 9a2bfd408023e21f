"""Differentiable LK residual with the hand-written CUDA adjoint.

``LKResidual.apply(I0, I1, u0, pts, nlevels, window, iters)`` returns the
per-point loss (sum of squared level-0 photometric residuals after coarse-to-
fine Gauss-Newton); its backward calls gbt_lkd_backward, which recomputes the
pyramids.  The torch.autograd.Function exists for gradient checks: the
forward and backward are the C ABI calls gbt_lkd_forward / gbt_lkd_backward.
"""
import ctypes

import torch

from ._native import check, cuda_lib


def _lib():
    lib = cuda_lib()
    if not getattr(lib, "_lkd_typed", False):
        P, I32, I64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        lib.gbt_lkd_scratch_bytes.argtypes = [I32, I32, I32, I32]
        lib.gbt_lkd_scratch_bytes.restype = I64
        lib.gbt_lkd_forward.argtypes = [P, P, I64, I64, I32, I32, I32, I32, I32, I32, P, P, I32, P, P, P]
        lib.gbt_lkd_backward.argtypes = [P, P, I64, I64, I32, I32, I32, I32, I32, I32, P, P, I32, P, P, P, P, P]
        lib._lkd_typed = True
    return lib


def _prep(I0, I1, u0, pts):
    if I0.dim() == 2:
        I0, I1, u0, pts = I0[None], I1[None], u0[None], pts[None]
    return (I0.contiguous().float(), I1.contiguous().float(), u0.contiguous().float(), pts.contiguous().float())


def forward(I0, I1, u0, pts, nlevels=5, window=9, iters=10):
    lib = _lib()
    I0, I1, u0, pts = _prep(I0, I1, u0, pts)
    P, H, W = I0.shape
    n = pts.shape[1]
    loss = torch.empty((P, n), device=I0.device)
    vf = torch.empty((P, n, 2), device=I0.device)
    st = torch.cuda.current_stream().cuda_stream
    check(lib.gbt_lkd_forward(I0.data_ptr(), I1.data_ptr(), W * 4, H * W * 4, H, W, nlevels, window, iters, P,
                              pts.data_ptr(), u0.data_ptr(), n, loss.data_ptr(), vf.data_ptr(), st))
    return loss, vf


def backward(I0, I1, u0, pts, dloss, nlevels=5, window=9, iters=10):
    lib = _lib()
    I0, I1, u0, pts = _prep(I0, I1, u0, pts)
    P, H, W = I0.shape
    n = pts.shape[1]
    dloss = dloss.reshape(P, n).contiguous().float()
    dI0 = torch.empty_like(I0)
    dI1 = torch.empty_like(I1)
    du0 = torch.empty_like(u0)
    st = torch.cuda.current_stream().cuda_stream
    check(lib.gbt_lkd_backward(I0.data_ptr(), I1.data_ptr(), W * 4, H * W * 4, H, W, nlevels, window, iters, P,
                               pts.data_ptr(), u0.data_ptr(), n, dloss.data_ptr(), dI0.data_ptr(), dI1.data_ptr(),
                               du0.data_ptr(), st))
    return dI0, dI1, du0


class LKResidual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, I0, I1, u0, pts, nlevels=5, window=9, iters=10):
        loss, _ = forward(I0, I1, u0, pts, nlevels, window, iters)
        ctx.save_for_backward(I0, I1, u0, pts)
        ctx.cfg = (nlevels, window, iters)
        return loss.reshape(pts.shape[:-1])

    @staticmethod
    def backward(ctx, gloss):
        I0, I1, u0, pts = ctx.saved_tensors
        dI0, dI1, du0 = backward(I0, I1, u0, pts, gloss, *ctx.cfg)
        return dI0.reshape(I0.shape), dI1.reshape(I1.shape), du0.reshape(u0.shape), None, None, None, None
