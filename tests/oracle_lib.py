"""Loads the oracle libraries (test infrastructure only)."""
import ctypes
import os

import numpy as np

from stage_api import StageLib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF = os.path.join(ROOT, "oracle", "_ref", "libcuimg_ref.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")

_lib = None


def oracle():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(ORACLE)
        _lib.oracle_sizes_ok.argtypes = [ctypes.c_int] * 3
        _lib.oracle_gauss_taps.argtypes = [ctypes.c_float, ctypes.c_void_p]
        _lib.oracle_gauss_taps.restype = ctypes.c_int
        _lib.oracle_gauss_sep_f32.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p]
        _lib.oracle_gauss_pyramid_f32.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [
            ctypes.c_void_p] * 4
        for n in ("oracle_set_k", "oracle_set_with_merge", "oracle_set_n"):
            getattr(_lib, n).argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib.oracle_set_detector.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 3
    return _lib


def tracker_oracle(rows, cols, nscales, threshold=20, det_freq=10, filt_freq=1):
    return StageLib(oracle(), "oracle_").create(rows, cols, nscales, threshold, det_freq, filt_freq)


def reference_available():
    return os.path.exists(REF)


def tracker_reference(rows, cols, nscales, threshold=20, det_freq=10, filt_freq=1):
    return StageLib(ctypes.CDLL(REF), "ref_").create(rows, cols, nscales, threshold, det_freq, filt_freq)


def gauss_taps(sigma):
    taps = np.zeros(2 * 200 + 1, np.float32)
    R = oracle().oracle_gauss_taps(sigma, taps.ctypes.data)
    return R, taps[: 2 * R + 1].copy()


def gauss_sep(img, sigma):
    img = np.ascontiguousarray(img, np.float32)
    H, W = img.shape
    R, taps = gauss_taps(sigma)
    tmp = np.zeros_like(img)
    out = np.zeros_like(img)
    oracle().oracle_gauss_sep_f32(img.ctypes.data, H, W, taps.ctypes.data, R, tmp.ctypes.data, out.ctypes.data)
    return out


def gauss_pyramid(img, nlevels):
    img = np.ascontiguousarray(img, np.float32)
    H, W = img.shape
    total = sum((H >> l) * (W >> l) for l in range(1, nlevels))
    out = np.zeros(total, np.float32)
    tmp, blur, work = (np.zeros_like(img) for _ in range(3))
    oracle().oracle_gauss_pyramid_f32(img.ctypes.data, H, W, nlevels, tmp.ctypes.data, blur.ctypes.data,
                                      work.ctypes.data, out.ctypes.data)
    levels, off = [], 0
    for l in range(1, nlevels):
        n = (H >> l) * (W >> l)
        levels.append(out[off:off + n].reshape(H >> l, W >> l))
        off += n
    return levels


def box_pyramid_u8(img, nlevels):
    """2x2 floor-mean pyramid (mipmap_kernel, cuimg/gpu/mipmap.h:24-49)."""
    levels, cur = [], img.astype(np.int32)
    for _ in range(1, nlevels):
        h, w = cur.shape[0] // 2, cur.shape[1] // 2
        c = cur[: 2 * h, : 2 * w]
        nxt = (c[0::2, 0::2] + c[0::2, 1::2] + c[1::2, 0::2] + c[1::2, 1::2]) // 4
        levels.append(nxt.astype(np.uint8))
        cur = nxt
    return levels


def alt_tracker_oracle(kind, rows, cols, nscales, det_freq, filt_freq, step=1, grad_th=1):
    """Oracle with the regular (kind 1) or dense (kind 2) detector."""
    o = tracker_oracle(rows, cols, nscales, 20, det_freq, filt_freq)
    oracle().oracle_set_detector(o.h, kind, step, grad_th)
    return o


def alt_golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("altdet_") and f.endswith(".npz"))


def alt_reference(kind, rows, cols, nscales, det_freq, filt_freq, step=1, grad_th=1):
    """The reference's generic strategy with regular_detector / dense_detector
    (oracle/_ref, built here only): returns (lib, handle)."""
    lib = ctypes.CDLL(REF)
    lib.refx_create.restype = ctypes.c_void_p
    lib.refx_create.argtypes = [ctypes.c_int] * 8
    lib.refx_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.refx_nparticles.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.refx_compact_has_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.refx_get_particles.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 6
    lib.refx_destroy.argtypes = [ctypes.c_void_p]
    return lib, lib.refx_create(kind, rows, cols, nscales, det_freq, filt_freq, step, grad_th)


def alt_reference_particles(lib, h, s):
    """Particle state of scale s of an alt_reference tracker."""
    n = lib.refx_nparticles(h, s)
    speed = np.zeros((n, 2), np.float32)
    pos = np.zeros((n, 2), np.int16)
    age = np.zeros(n, np.uint16)
    feat = np.zeros((n, 32), np.uint8)
    nm = ctypes.c_int()
    lib.refx_get_particles(h, s, speed.ctypes.data, pos.ctypes.data, age.ctypes.data, feat.ctypes.data, None,
                           ctypes.byref(nm))
    matches = np.zeros(max(nm.value, 1), np.int32)
    lib.refx_get_particles(h, s, speed.ctypes.data, pos.ctypes.data, age.ctypes.data, feat.ctypes.data,
                           matches.ctypes.data, ctypes.byref(nm))
    return dict(speed=speed, pos=pos, age=age, feat=feat, matches=matches[: nm.value],
                compact=bool(lib.refx_compact_has_run(h, s)))


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("tracker_") and f.endswith(".npz"))


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def lk_track(prev, cur, pts, nlevels, pyr=0, window=11, npix=25, max_iter=30, eps=0.1, max_err=300.0):
    """Oracle pyramidal LK (oracle/lk_oracle.c); pyr 0 = uint8 box path, 1 = fp32 Gaussian."""
    lib = oracle()
    if not getattr(lib, "_lk_typed", False):
        lib.oracle_lk_track.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 7 + [
            ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
        lib._lk_typed = True
    A = np.ascontiguousarray(prev, np.float32)
    B = np.ascontiguousarray(cur, np.float32)
    p = np.ascontiguousarray(pts, np.float32)
    n = len(p)
    out = np.zeros((n, 2), np.float32)
    st = np.zeros(n, np.int32)
    er = np.zeros(n, np.float32)
    H, W = A.shape
    assert lib.oracle_lk_track(A.ctypes.data, B.ctypes.data, H, W, nlevels, pyr, window, npix, max_iter, eps, max_err,
                               p.ctypes.data, n, out.ctypes.data, st.ctypes.data, er.ctypes.data) == 0
    return out, st, er


def lkd_forward64(I0, I1, pts, u0, L, window, iters):
    lib = oracle()
    if not getattr(lib, "_lkd_typed", False):
        lib.oracle_lkd_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_lkd_grad_fd.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_double] + [ctypes.c_void_p] * 3
        lib._lkd_typed = True
    a = np.ascontiguousarray(I0, np.float64)
    b = np.ascontiguousarray(I1, np.float64)
    p = np.ascontiguousarray(pts, np.float64)
    u = np.ascontiguousarray(u0, np.float64)
    n = len(p)
    loss = np.zeros(n)
    vf = np.zeros((n, 2))
    H, W = a.shape
    lib.oracle_lkd_forward(a.ctypes.data, b.ctypes.data, H, W, L, window, iters, p.ctypes.data, u.ctypes.data, n,
                           loss.ctypes.data, vf.ctypes.data)
    return loss, vf


def lkd_grad_fd64(I0, I1, pts, u0, L, window, iters, wts, h=1e-3):
    lkd_forward64(I0[:16, :16] * 0 + 1, I1[:16, :16] * 0 + 1, pts[:0], u0[:0], 1, 3, 0)  # declares types
    lib = oracle()
    a = np.ascontiguousarray(I0, np.float64)
    b = np.ascontiguousarray(I1, np.float64)
    p = np.ascontiguousarray(pts, np.float64)
    u = np.ascontiguousarray(u0, np.float64)
    w = np.ascontiguousarray(wts, np.float64)
    H, W = a.shape
    g0, g1, gu = np.zeros((H, W)), np.zeros((H, W)), np.zeros_like(u)
    lib.oracle_lkd_grad_fd(a.ctypes.data, b.ctypes.data, H, W, L, window, iters, p.ctypes.data, u.ctypes.data,
                           len(p), w.ctypes.data, h, g0.ctypes.data, g1.ctypes.data, gu.ctypes.data)
    return g0, g1, gu


class PyrlkLib:
    """The pyramidal LK tracker strategy (pyrlk_cpu<fast_detector<cpu>,
    iterative_lk_match_5x5>) from the oracle (prefix oracle_pyrlk_) or the
    reference built from its own sources (reflk_)."""

    def __init__(self, which, rows, cols, nscales, threshold=20, det_freq=10, filt_freq=1, with_merge=1):
        self.L = nscales
        self.dims = [(rows >> s, cols >> s) for s in range(nscales)]
        P, I = ctypes.c_void_p, ctypes.c_int
        if which == "oracle":
            lib = oracle()
            lib.oracle_pyrlk_create.restype = P
            lib.oracle_pyrlk_create.argtypes = [I] * 6
            lib.oracle_pyrlk_run.argtypes = [P, P]
            lib.oracle_pyrlk_nparticles.argtypes = [P, I]
            lib.oracle_pyrlk_get.argtypes = [P, I] + [P] * 6
            lib.oracle_pyrlk_get_sparse.argtypes = [P, I, P]
            lib.oracle_pyrlk_destroy.argtypes = [P]
            lib.oracle_pyrlk_set_param.argtypes = [P, I, I, I]
            self.h = lib.oracle_pyrlk_create(rows, cols, nscales, threshold, det_freq, filt_freq)
            if not with_merge:
                lib.oracle_pyrlk_set_param(self.h, -1, 5, 0)
            self._run, self._n, self._get = lib.oracle_pyrlk_run, lib.oracle_pyrlk_nparticles, lib.oracle_pyrlk_get
            self._sparse, self._destroy = lib.oracle_pyrlk_get_sparse, lib.oracle_pyrlk_destroy
            self.set_param = lambda s, key, value: lib.oracle_pyrlk_set_param(self.h, s, key, value)
        else:
            lib = ctypes.CDLL(REF)
            lib.reflk_create_full.restype = P
            lib.reflk_create_full.argtypes = [I] * 7
            lib.reflk_run.argtypes = [P, P]
            lib.reflk_nparticles.argtypes = [P, I]
            lib.reflk_get_full.argtypes = [P, I] + [P] * 6
            lib.reflk_get_sparse.argtypes = [P, I, P]
            lib.reflk_destroy.argtypes = [P]
            self.h = lib.reflk_create_full(rows, cols, nscales, threshold, det_freq, filt_freq, with_merge)
            self._run, self._n, self._get = lib.reflk_run, lib.reflk_nparticles, lib.reflk_get_full
            self._sparse, self._destroy = lib.reflk_get_sparse, lib.reflk_destroy

    def run(self, frame):
        f = np.ascontiguousarray(frame, np.uint8)
        self._run(self.h, f.ctypes.data)

    def particles(self, s):
        n = self._n(self.h, s)
        pos = np.zeros((n, 2), np.float32)
        speed = np.zeros((n, 2), np.float32)
        age = np.zeros(n, np.uint16)
        nm, comp = ctypes.c_int(), ctypes.c_int()
        self._get(self.h, s, None, None, None, None, ctypes.byref(nm), ctypes.byref(comp))
        matches = np.zeros(max(nm.value, 1), np.int32)
        self._get(self.h, s, pos.ctypes.data, speed.ctypes.data, age.ctypes.data, matches.ctypes.data,
                  ctypes.byref(nm), ctypes.byref(comp))
        return dict(pos=pos, speed=speed, age=age, matches=matches[: nm.value], compact=bool(comp.value))

    def sparse(self, s):
        H, W = self.dims[s]
        out = np.zeros((H, W), np.uint32)
        self._sparse(self.h, s, out.ctypes.data)
        return out

    def destroy(self):
        if self.h:
            self._destroy(self.h)
            self.h = None


def black_margin_frames(seed, rows, cols, n, margin):
    """Seeded synthetic frames with a black margin of `margin` pixels on every
    side: the LK windows of every particle then stay inside the image at every
    scale (the reference reads outside its images otherwise)."""
    from cuimg_gb300 import synth
    f = synth.frames(seed, rows, cols, n)
    f[:, :margin] = 0
    f[:, rows - margin:] = 0
    f[:, :, :margin] = 0
    f[:, :, cols - margin:] = 0
    return f


def diff_pyrlk(a, b, L, with_sparse=True):
    """Names of what differs between two PyrlkLib-like states (empty = equal)."""
    bad = []
    for s in range(L):
        x, y = a.particles(s), b.particles(s)
        for k in ("pos", "speed", "age"):
            if x[k].shape != y[k].shape or not np.array_equal(x[k], y[k]):
                bad.append("scale %d %s" % (s, k))
        if x["compact"] != y["compact"]:
            bad.append("scale %d compact" % s)
        elif x["compact"] and not np.array_equal(x["matches"], y["matches"]):
            bad.append("scale %d matches" % s)
        if with_sparse and not np.array_equal(a.sparse(s), b.sparse(s)):
            bad.append("scale %d sparse" % s)
    return bad
