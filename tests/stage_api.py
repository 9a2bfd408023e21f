"""Uniform ctypes view over libraries that export the tracker stage-dump API.

Three libraries export the same getters under different prefixes:
  * ``ref_``    -- the reference's own CPU tracker (oracle/_ref, this container only),
  * ``oracle_`` -- the C restatement in oracle/tracker_oracle.c,
and the CUDA tracker exposes the same stage images through its C ABI
(``cuimg_gb300.tracker.Tracker.state``).  Tests compare them stage by stage.
"""
import ctypes

import numpy as np

c_int_p = ctypes.POINTER(ctypes.c_int)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class StageLib:
    def __init__(self, lib, prefix):
        self.lib = lib
        self.p = prefix
        f = self._f
        f("create").restype = ctypes.c_void_p
        f("create").argtypes = [ctypes.c_int] * 6
        f("destroy").argtypes = [ctypes.c_void_p]
        f("run").argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        for name in ("dims", "bins"):
            f(name).argtypes = [ctypes.c_void_p, ctypes.c_int, c_int_p, c_int_p]
        for name in ("get_input", "get_s1", "get_s2"):
            f(name).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        for name in ("get_saliency", "get_mask", "get_contrast", "get_sparse"):
            f(name).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        f("get_bins").argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4
        for name in ("nparticles", "compact_has_run", "frame_count"):
            f(name).argtypes = [ctypes.c_void_p, ctypes.c_int]
            f(name).restype = ctypes.c_int
        f("get_particles").argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 5 + [c_int_p]
        self.h = None

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def create(self, rows, cols, nscales, threshold=20, det_freq=10, filt_freq=1):
        self.h = self._f("create")(rows, cols, nscales, threshold, det_freq, filt_freq)
        if not self.h:
            raise RuntimeError("create failed")
        self.L = nscales
        return self

    def set_param(self, scale, key, value):
        """The library's setter of one scale between frames (keys of
        gbt_set_param; see oracle_set_param / ref_set_param)."""
        f = self._f("set_param")
        f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        if f(self.h, scale, key, value) != 0:
            raise RuntimeError("set_param failed")

    def destroy(self):
        if self.h:
            self._f("destroy")(self.h)
            self.h = None

    def run(self, frame):
        frame = np.ascontiguousarray(frame, dtype=np.uint8)
        r = self._f("run")(self.h, _ptr(frame))
        if r not in (None, 0):
            raise RuntimeError("run failed: %r" % r)

    def dims(self, s):
        r, c = ctypes.c_int(), ctypes.c_int()
        self._f("dims")(self.h, s, ctypes.byref(r), ctypes.byref(c))
        return r.value, c.value

    def _img(self, name, s, b, dtype=np.uint8):
        H, W = self.dims(s)
        out = np.zeros((H + 2 * b, W + 2 * b), dtype)
        self._f(name)(self.h, s, b, _ptr(out))
        return out

    def input(self, s, b=0):
        return self._img("get_input", s, b)

    def s1(self, s, b=0):
        return self._img("get_s1", s, b)

    def s2(self, s, b=0):
        return self._img("get_s2", s, b)

    def _plain(self, name, s, dtype):
        H, W = self.dims(s)
        out = np.zeros((H, W), dtype)
        self._f(name)(self.h, s, _ptr(out))
        return out

    def saliency(self, s):
        return self._plain("get_saliency", s, np.uint8)

    def mask(self, s):
        return self._plain("get_mask", s, np.uint8)

    def contrast(self, s):
        return self._plain("get_contrast", s, np.uint32)

    def sparse(self, s):
        return self._plain("get_sparse", s, np.uint32)

    def bins(self, s):
        r, c = ctypes.c_int(), ctypes.c_int()
        self._f("bins")(self.h, s, ctypes.byref(r), ctypes.byref(c))
        BH, BW = r.value, c.value
        flow = np.zeros((BH, BW, 2), np.float32)
        count = np.zeros((BH, BW), np.uint32)
        st_n = np.zeros((BH, BW), np.int32)
        st_sp = np.zeros((BH, BW, 2), np.int32)
        self._f("get_bins")(self.h, s, _ptr(flow), _ptr(count), _ptr(st_n), _ptr(st_sp))
        return dict(flow=flow, count=count, stat_n=st_n, stat_speed=st_sp)

    def nparticles(self, s):
        return self._f("nparticles")(self.h, s)

    def compact_has_run(self, s):
        return bool(self._f("compact_has_run")(self.h, s))

    def frame_count(self, s):
        return self._f("frame_count")(self.h, s)

    def particles(self, s):
        n = self.nparticles(s)
        speed = np.zeros((n, 2), np.float32)
        pos = np.zeros((n, 2), np.int16)
        age = np.zeros(n, np.uint16)
        feat = np.zeros((n, 32), np.uint8)
        nm = ctypes.c_int()
        self._f("get_particles")(self.h, s, _ptr(speed), _ptr(pos), _ptr(age), _ptr(feat), None, ctypes.byref(nm))
        matches = np.zeros(max(nm.value, 1), np.int32)
        self._f("get_particles")(self.h, s, _ptr(speed), _ptr(pos), _ptr(age), _ptr(feat), _ptr(matches),
                                 ctypes.byref(nm))
        return dict(speed=speed, pos=pos, age=age, feat=feat, matches=matches[: nm.value])


def snapshot(lib, L, borders=True):
    """Every stage of every scale after the last run(), as numpy arrays."""
    out = []
    for s in range(L):
        d = dict(
            input=lib.input(s, 6 if borders else 0),
            s1=lib.s1(s, 3 if borders else 0),
            s2=lib.s2(s, 6 if borders else 0),
            contrast=lib.contrast(s),
            saliency=lib.saliency(s),
            mask=lib.mask(s),
            sparse=lib.sparse(s),
            compact=lib.compact_has_run(s),
        )
        d.update(lib.bins(s))
        d.update(lib.particles(s))
        out.append(d)
    return out


def diff_snapshots(a, b, detector_frame, keys=None, fast_detector=True):
    """Names of the stages that differ between two snapshots (empty = equal).
    The FAST saliency and mask stages are compared on detector frames of the
    FAST detector only."""
    bad = []
    for s, (x, y) in enumerate(zip(a, b)):
        ks = keys or [k for k in x if k not in ("compact", "matches", "mask", "saliency")]
        for k in ks:
            if k in ("mask", "saliency") and not detector_frame:
                continue
            if k == "feat":
                xv, yv = x[k][:, :16], y[k][:, :16]
            else:
                xv, yv = x[k], y[k]
            if xv.shape != yv.shape or not np.array_equal(xv, yv):
                bad.append("scale %d: %s" % (s, k))
        if detector_frame:
            for k in ("mask", "saliency") if fast_detector else ():
                if not np.array_equal(x[k], y[k]):
                    bad.append("scale %d: %s" % (s, k))
            if x["compact"] != y["compact"]:
                bad.append("scale %d: compact flag" % s)
            elif x["compact"] and not np.array_equal(x["matches"], y["matches"]):
                bad.append("scale %d: matches" % s)
    return bad


# Setter calls made between frames, as the reference's own setters of one
# scale: (before frame, scale, key, value), keys of gbt_set_param (0 FAST
# threshold, 1 arc length n, 2 detector frequency, 3 filtering frequency,
# 4 k, 5 with_merge).  The frequency and k setters also set every coarser
# scale (tracking_strategies.hpp:56-82); the others set their scale only.
SETTER_SCHEDULE = [
    (2, 0, 2, 3),    # detector every 3 frames, all scales
    (4, 1, 0, 35),   # per-scale thresholds
    (4, 2, 0, 12),
    (6, 1, 5, 0),    # no merge on scale 1
    (8, 1, 2, 2),    # detector every 2 frames on scales 1 and up
    (9, 0, 4, 60),   # k = 60 everywhere: many more matches rejected
    (11, 2, 3, 2),   # filter every 2 frames on scale 2
    (12, 0, 1, 12),  # arc length 12 on scale 0
    (14, 0, 4, 300),
]
UPWARD_KEYS = (2, 3, 4)


def scales_set_by(L, scale, key):
    """Scales one reference setter call changes."""
    return list(range(scale, L)) if key in UPWARD_KEYS else [scale]


class SettingsTrack:
    """The per-scale settings a SETTER_SCHEDULE has produced so far."""

    def __init__(self, L, det_freq, filt_freq):
        self.det = [det_freq] * L
        self.filt = [filt_freq] * L

    def apply(self, L, scale, key, value):
        for s in scales_set_by(L, scale, key):
            if key == 2:
                self.det[s] = value
            elif key == 3:
                self.filt[s] = value

    def all_detect(self, frame):
        return all(frame % d == 0 for d in self.det)

