"""Differentiable LK residual with the hand-written CUDA adjoint.

``LKResidual.apply(I0, I1, u0, pts, nlevels, window, iters)`` returns the
per-point loss (sum of squared level-0 photometric residuals after coarse-to-
fine Gauss-Newton).  Its forward records a tape (per point: each level's
normal-matrix inverse and the iterates with their right-hand sides) and its
backward reads that tape instead of replaying the forward; both recompute the
pyramids.  The torch.autograd.Function exists for gradient checks: the
forward and backward are the C ABI calls gbt_lkd_forward_tape /
gbt_lkd_backward_tape (gbt_lkd_forward / gbt_lkd_backward without a tape).
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
        lib.gbt_lkd_tape_bytes.argtypes = [I32, I32, I32, I32]
        lib.gbt_lkd_tape_bytes.restype = I64
        lib.gbt_lkd_forward.argtypes = [P, P, I64, I64, I32, I32, I32, I32, I32, I32, P, P, I32, P, P, P]
        lib.gbt_lkd_backward.argtypes = [P, P, I64, I64, I32, I32, I32, I32, I32, I32, P, P, I32, P, P, P, P, P]
        lib.gbt_lkd_forward_tape.argtypes = [P, P, I64, I64, I32, I32, I32, I32, I32, I32, P, P, I32, P, P, P, P]
        lib.gbt_lkd_backward_tape.argtypes = [P, P, I64, I64, I32, I32, I32, I32, I32, I32, P, P, I32, P, P, P, P,
                                              P, P]
        lib._lkd_typed = True
    return lib


def _prep(I0, I1, u0, pts):
    if I0.dim() == 2:
        I0, I1, u0, pts = I0[None], I1[None], u0[None], pts[None]
    return (I0.contiguous().float(), I1.contiguous().float(), u0.contiguous().float(), pts.contiguous().float())


def tape_bytes(nlevels, iters, npairs, npts):
    return int(_lib().gbt_lkd_tape_bytes(nlevels, iters, npairs, npts))


def forward(I0, I1, u0, pts, nlevels=5, window=9, iters=10, tape=False):
    """Loss per point and final positions; with tape=True also the tape for backward()."""
    lib = _lib()
    I0, I1, u0, pts = _prep(I0, I1, u0, pts)
    P, H, W = I0.shape
    n = pts.shape[1]
    loss = torch.empty((P, n), device=I0.device)
    vf = torch.empty((P, n, 2), device=I0.device)
    t = None
    if tape:
        nb = tape_bytes(nlevels, iters, P, n)
        if nb < 0:
            raise ValueError("bad adjoint configuration")
        t = torch.empty(max(nb, 16), dtype=torch.uint8, device=I0.device)
    st = torch.cuda.current_stream().cuda_stream
    check(lib.gbt_lkd_forward_tape(I0.data_ptr(), I1.data_ptr(), W * 4, H * W * 4, H, W, nlevels, window, iters, P,
                                   pts.data_ptr(), u0.data_ptr(), n, loss.data_ptr(), vf.data_ptr(),
                                   t.data_ptr() if t is not None else None, st))
    return (loss, vf, t) if tape else (loss, vf)


def backward(I0, I1, u0, pts, dloss, nlevels=5, window=9, iters=10, tape=None):
    """Gradients of sum(dloss * loss) w.r.t. I0, I1 and u0 (tape: from forward(..., tape=True))."""
    lib = _lib()
    I0, I1, u0, pts = _prep(I0, I1, u0, pts)
    P, H, W = I0.shape
    n = pts.shape[1]
    dloss = dloss.reshape(P, n).contiguous().float()
    dI0 = torch.empty_like(I0)
    dI1 = torch.empty_like(I1)
    du0 = torch.empty_like(u0)
    st = torch.cuda.current_stream().cuda_stream
    check(lib.gbt_lkd_backward_tape(I0.data_ptr(), I1.data_ptr(), W * 4, H * W * 4, H, W, nlevels, window, iters, P,
                                    pts.data_ptr(), u0.data_ptr(), n, dloss.data_ptr(), dI0.data_ptr(),
                                    dI1.data_ptr(), du0.data_ptr(), tape.data_ptr() if tape is not None else None,
                                    st))
    return dI0, dI1, du0


class LKResidual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, I0, I1, u0, pts, nlevels=5, window=9, iters=10):
        loss, _, tape = forward(I0, I1, u0, pts, nlevels, window, iters, tape=True)
        ctx.save_for_backward(I0, I1, u0, pts, tape)
        ctx.cfg = (nlevels, window, iters)
        return loss.reshape(pts.shape[:-1])

    @staticmethod
    def backward(ctx, gloss):
        I0, I1, u0, pts, tape = ctx.saved_tensors
        dI0, dI1, du0 = backward(I0, I1, u0, pts, gloss, *ctx.cfg, tape=tape)
        return dI0.reshape(I0.shape), dI1.reshape(I1.shape), du0.reshape(u0.shape), None, None, None, None
