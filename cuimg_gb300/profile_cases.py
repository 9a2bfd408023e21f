"""Small, self-contained cases of each kernel, for profiler captures.

    python -m cuimg_gb300.profile_cases gaussian   # 8 fp32 1920x1080 images, sigma 4
    python -m cuimg_gb300.profile_cases lk         # 4 fp32 640x480 pairs, 5 levels, 20k points each
    python -m cuimg_gb300.profile_cases adjoint    # LK residual forward (tape) + backward, same batch
    python -m cuimg_gb300.profile_cases tracker    # 4 streams of 1920x1080, 6 frames
    python -m cuimg_gb300.profile_cases tracker_det  # the same with the detector every third frame
    python -m cuimg_gb300.profile_cases tracker16  # 16 streams of 1920x1080 in one group, 4 frames

Each case runs its kernels a few times on inputs larger than L2 but a few GB
at most on the device, so a capture of one or two launches ends quickly.
"""
import ctypes
import sys

import numpy as np


def gaussian(reps=3):
    import torch

    from . import synth
    from ._native import check, cuda_lib
    lib = cuda_lib()
    H, W, n = 1080, 1920, 8
    x = torch.from_numpy(synth.Stream(7, H, W).frame_f32(0)).cuda().repeat(n, 1, 1).contiguous()
    y = torch.empty_like(x)
    for _ in range(reps):
        check(lib.gbt_gaussian_f32_batch(x.data_ptr(), W * 4, H * W * 4, y.data_ptr(), W * 4, H * W * 4, H, W, n,
                                         ctypes.c_float(4.0), None))
    torch.cuda.synchronize()


def _lk_batch(P=4, n=20000):
    import torch

    from . import synth
    H, W = 480, 640
    rng = np.random.default_rng(0)
    f0 = np.empty((P, H, W), np.float32)
    f1 = np.empty((P, H, W), np.float32)
    for p in range(P):
        s = synth.Stream(300 + p, H, W)
        f0[p], f1[p] = s.frame_f32(0), s.frame_f32(1)
    pts = np.stack([rng.uniform(30, H - 30, (P, n)), rng.uniform(30, W - 30, (P, n))], -1).astype(np.float32)
    u0 = rng.uniform(-2, 2, (P, n, 2)).astype(np.float32)
    t = lambda a: torch.from_numpy(a).cuda()
    return t(f0), t(f1), t(pts), t(u0)


def lk_case(reps=3):
    import torch

    from . import lk
    A, B, X, _ = _lk_batch()
    prm = lk.params(window=9, npix=81, max_iter=10)
    for _ in range(reps):
        lk.track(A, B, X, nlevels=5, prm=prm)
    torch.cuda.synchronize()


def adjoint(reps=2):
    import torch

    from . import lkd
    A, B, X, U = _lk_batch()
    ones = torch.ones(X.shape[:2], device="cuda")
    for _ in range(reps):
        tape = lkd.forward(A, B, U, X, 5, 9, 10, tape=True)[2]
        lkd.backward(A, B, U, X, ones, 5, 9, 10, tape=tape)
    torch.cuda.synchronize()


def tracker(frames=6):
    from . import BatchTracker, synth
    cfg = [dict(rows=1080, cols=1920, nscales=4, detector_threshold=20, detector_frequency=10)] * 4
    vids = [synth.frames(1000 + i, 1080, 1920, frames) for i in range(4)]
    bt = BatchTracker(cfg, graphs=False, groups=1)  # one launch per stage over all four streams
    for t in range(frames):
        bt.run([v[t] for v in vids])
    bt.sync()
    bt.close()


def tracker_det(frames=8):
    """4 streams of 1920x1080 with the detector every third frame (frames 0, 3, 6)."""
    from . import BatchTracker, synth
    cfg = [dict(rows=1080, cols=1920, nscales=4, detector_threshold=20, detector_frequency=3)] * 4
    vids = [synth.frames(1000 + i, 1080, 1920, frames) for i in range(4)]
    bt = BatchTracker(cfg, graphs=False, groups=1)  # one launch per stage over all four streams
    for t in range(frames):
        bt.run([v[t] for v in vids])
    bt.sync()
    bt.close()


def tracker16(frames=4):
    """16 streams of 1920x1080 in one stream group, blur strips of 32 rows."""
    from . import BatchTracker, synth
    cfg = [dict(rows=1080, cols=1920, nscales=4, detector_threshold=20, detector_frequency=10)] * 16
    vids = [synth.frames(1000 + i, 1080, 1920, frames) for i in range(16)]
    bt = BatchTracker(cfg, graphs=False, groups=1)
    bt.set_tuning(1, 32)
    for t in range(frames):
        bt.run([v[t] for v in vids])
    bt.sync()
    bt.close()


CASES = {"gaussian": gaussian, "lk": lk_case, "adjoint": adjoint, "tracker": tracker, "tracker_det": tracker_det,
         "tracker16": tracker16}

if __name__ == "__main__":
    for name in sys.argv[1:] or list(CASES):
        CASES[name]()
    print("ok")
