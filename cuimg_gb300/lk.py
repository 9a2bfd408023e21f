"""Pyramidal Lucas-Kanade over batches of frame pairs (C ABI wrapper).

    out, status, err = lk.track(prev, cur, points, nlevels=3)

prev / cur: torch tensors on the GPU, (P, H, W) uint8 (the reference's gl8u
path: 2x2 floor-mean pyramid, uint8 template) or float32 (sigma-1 Gaussian
pyramid); points: (P, N, 2) float32 (row, col) in level-0 pixels.  Parameters
default to the reference's iterative_lk_match_5x5 constants (window 11, 25
masked pixels, 30 iterations, step 0.1, error bound 300).
"""
import ctypes

from ._native import check, cuda_lib


class gbt_lk_params(ctypes.Structure):
    _fields_ = [("window", ctypes.c_int32), ("npix", ctypes.c_int32), ("max_iter", ctypes.c_int32),
                ("eps", ctypes.c_float), ("max_err", ctypes.c_float), ("warps_per_block", ctypes.c_int32)]


def params(window=11, npix=25, max_iter=30, eps=0.1, max_err=300.0, warps_per_block=0):
    """warps_per_block: CTA size of the tracking kernel (2, 4, 8; 0 = 8), speed only;
    cuimg_gb300.autotune.tune_lk picks it for a workload."""
    return gbt_lk_params(window, npix, max_iter, eps, max_err, warps_per_block)


def _declare(lib):
    if getattr(lib, "_lk_typed", False):
        return
    P = ctypes.c_void_p
    I32 = ctypes.c_int32
    lib.gbt_lk_params_default.argtypes = [P]
    lib.gbt_lk_params_default.restype = None
    lib.gbt_lk_scratch_bytes.argtypes = [I32, I32, I32, I32]
    lib.gbt_lk_scratch_bytes.restype = ctypes.c_int64
    lib.gbt_lk_track_batch.argtypes = [P, P, ctypes.c_int64, ctypes.c_int64, I32, I32, I32, I32,
                                       ctypes.POINTER(gbt_lk_params), I32, P, I32, P, P, P, P]
    lib._lk_typed = True


def track(prev, cur, points, nlevels=3, prm=None, stream=None):
    import torch
    lib = cuda_lib()
    _declare(lib)
    if prev.dim() == 2:
        prev, cur, points = prev[None], cur[None], points[None]
    assert prev.is_cuda and cur.is_cuda and points.is_cuda
    assert prev.shape == cur.shape and prev.dtype == cur.dtype
    is_u8 = prev.dtype == torch.uint8
    prev, cur = prev.contiguous(), cur.contiguous()
    points = points.contiguous().float()
    P, H, W = prev.shape
    N = points.shape[1]
    es = 1 if is_u8 else 4
    out = torch.empty_like(points)
    status = torch.empty((P, N), dtype=torch.int32, device=points.device)
    err = torch.empty((P, N), dtype=torch.float32, device=points.device)
    prm = prm or params()
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    check(lib.gbt_lk_track_batch(prev.data_ptr(), cur.data_ptr(), W * es, H * W * es, H, W, int(is_u8), nlevels,
                                 ctypes.byref(prm), P, points.data_ptr(), N, out.data_ptr(), status.data_ptr(),
                                 err.data_ptr(), st))
    return out, status, err
