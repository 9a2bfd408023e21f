"""Seeded synthetic video streams (wrapper over csrc/synth.c).

Texture = 128 + Gaussian blobs + 4-octave value noise, each frame warped by
a per-frame affine motion with bilinear sampling plus sigma-2 Gaussian noise;
one seed per stream.  Stands in for camera video, which the reference's
sample reads (samples/tracking/main.cc:61-117).
"""
import ctypes

import numpy as np

from ._native import synth_lib


class Stream:
    def __init__(self, seed, rows, cols):
        self._lib = synth_lib()
        self.rows, self.cols = rows, cols
        self._h = self._lib.synth_create(int(seed), int(rows), int(cols))
        if not self._h:
            raise ValueError("bad stream size %dx%d" % (rows, cols))

    def frame(self, t):
        out = np.empty((self.rows, self.cols), np.uint8)
        self._lib.synth_frame_u8(self._h, int(t), out.ctypes.data)
        return out

    def frame_rgb(self, t):
        out = np.empty((self.rows, self.cols, 3), np.uint8)
        self._lib.synth_frame_rgb(self._h, int(t), out.ctypes.data)
        return out

    def frame_f32(self, t, noise_sigma=2.0):
        out = np.empty((self.rows, self.cols), np.float32)
        self._lib.synth_frame_f32(self._h, int(t), ctypes.c_float(noise_sigma), out.ctypes.data)
        return out

    def true_flow(self, t, points):
        """Displacement (drow, dcol) of frame t-1 points into frame t."""
        out = np.zeros((len(points), 2), np.float64)
        dy, dx = ctypes.c_double(), ctypes.c_double()
        for i, (y, x) in enumerate(points):
            self._lib.synth_true_flow(self._h, int(t), float(y), float(x), ctypes.byref(dy), ctypes.byref(dx))
            out[i] = dy.value, dx.value
        return out

    def close(self):
        if self._h:
            self._lib.synth_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def frames(seed, rows, cols, n, start=0):
    s = Stream(seed, rows, cols)
    out = np.empty((n, rows, cols), np.uint8)
    for t in range(n):
        out[t] = s.frame(start + t)
    s.close()
    return out
