"""Pins the LK oracle against the reference's own pyramidal LK tracker
(golden fixture from pyrlk_cpu<fast_detector<cpu>, iterative_lk_match_5x5>)."""
import numpy as np
import pytest

from oracle_lib import box_pyramid_u8, load_golden, lk_track, reference_available


def test_lk_oracle_matches_reference_golden():
    g = load_golden("lk_240x320_s3")
    rows, cols, L, seed = [int(x) for x in g["meta"]]
    f0, f1 = g["frames"][0], g["frames"][1]
    p0 = [f0] + box_pyramid_u8(f0, L)
    p1 = [f1] + box_pyramid_u8(f1, L)
    for s in range(L):
        pts = g["born_s%d_pos" % s]
        ref_pos, ref_age = g["tracked_s%d_pos" % s], g["tracked_s%d_age" % s]
        out, st, _ = lk_track(p0[s], p1[s], pts, L - s, pyr=0)
        H, W = p0[s].shape
        m = 12 * 2 ** (L - 1 - s)  # windows of every level stay inside (the reference reads outside otherwise)
        inner = (pts[:, 0] >= m) & (pts[:, 1] >= m) & (pts[:, 0] < H - m) & (pts[:, 1] < W - m)
        assert inner.sum() > 50
        np.testing.assert_array_equal(st[inner] > 0, ref_age[inner] > 0)
        both = inner & (st > 0)
        # The restatement computes in the reference's order and selects the
        # mask with the reference's std::nth_element order among equal norms,
        # so the tracked positions are identical, not just within 0.01 px.
        np.testing.assert_array_equal(out[both], ref_pos[both], err_msg="scale %d" % s)


def test_lk_oracle_recovers_known_translation():
    rng = np.random.default_rng(0)
    base = rng.uniform(0, 255, (140, 180)).astype(np.float32)
    from oracle_lib import gauss_sep
    tex = gauss_sep(base, 2.0)
    prev = tex[10:130, 10:170]
    cur = tex[12:132, 7:167]  # content moves by (-2, +3)
    pts = np.array([[60.0, 80.0], [50.5, 70.25], [70.0, 100.0]], np.float32)
    out, st, _ = lk_track(prev, cur, pts, 2, pyr=1, window=11, npix=121, max_iter=30, eps=0.01)
    assert st.all()
    np.testing.assert_allclose(out - pts, [[-2.0, 3.0]] * 3, atol=0.05)


def _reference_lk(rows, cols, L, frames):
    """The reference's pyrlk_cpu tracker (compiled from its sources into
    oracle/_ref) on a frame pair: births on frame 0, one LK step."""
    import ctypes

    from oracle_lib import REF
    lib = ctypes.CDLL(REF)
    lib.reflk_create.restype = ctypes.c_void_p
    lib.reflk_create.argtypes = [ctypes.c_int] * 4
    lib.reflk_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.reflk_nparticles.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.reflk_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.reflk_destroy.argtypes = [ctypes.c_void_p]
    h = lib.reflk_create(rows, cols, L, 20)
    out = {}

    def grab(tag):
        for s in range(L):
            n = lib.reflk_nparticles(h, s)
            pos = np.zeros((n, 2), np.float32)
            age = np.zeros(n, np.uint16)
            lib.reflk_get(h, s, pos.ctypes.data, age.ctypes.data)
            out[tag, s] = (pos, age)

    lib.reflk_run(h, np.ascontiguousarray(frames[0]).ctypes.data)
    grab("born")
    lib.reflk_run(h, np.ascontiguousarray(frames[1]).ctypes.data)
    grab("tracked")
    lib.reflk_destroy(h)
    return out


@pytest.mark.skipif(not reference_available(), reason="reference not built here (oracle/_ref)")
@pytest.mark.parametrize("rows,cols,L,seed", [(180, 260, 2, 3), (257, 391, 3, 8), (320, 480, 3, 40), (211, 603, 2, 77)])
def test_lk_oracle_matches_reference_live(rows, cols, L, seed):
    from cuimg_gb300 import synth
    frames = synth.frames(seed, rows, cols, 2)
    ref = _reference_lk(rows, cols, L, frames)
    p0 = [frames[0]] + box_pyramid_u8(frames[0], L)
    p1 = [frames[1]] + box_pyramid_u8(frames[1], L)
    for s in range(L):
        pts = ref["born", s][0]
        ref_pos, ref_age = ref["tracked", s]
        out, st, _ = lk_track(p0[s], p1[s], pts, L - s, pyr=0)
        H, W = p0[s].shape
        m = 12 * 2 ** (L - 1 - s)
        inner = (pts[:, 0] >= m) & (pts[:, 1] >= m) & (pts[:, 0] < H - m) & (pts[:, 1] < W - m)
        if inner.sum() < 20:
            continue
        np.testing.assert_array_equal(st[inner] > 0, ref_age[inner] > 0)
        both = inner & (st > 0)
        np.testing.assert_array_equal(out[both], ref_pos[both], err_msg="scale %d" % s)


@pytest.mark.skipif(not reference_available(), reason="reference not built here (oracle/_ref)")
@pytest.mark.parametrize("rows,cols,L,det,filt,merge,seed,n", [
    (320, 480, 3, 3, 1, 1, 5, 16),
    (256, 384, 2, 1, 1, 1, 6, 10),
    (480, 640, 3, 10, 2, 1, 7, 22),
    (300, 420, 3, 4, 1, 0, 8, 12),
])
def test_pyrlk_tracker_oracle_matches_reference_live(rows, cols, L, det, filt, merge, seed, n):
    # The whole LK tracker strategy over frames (pyrlk_cpu: LK matching with
    # the coarse-to-fine prediction, FAST births, compaction, merge) against
    # the reference's own, on frames with a black margin wide enough that no
    # window ever reads outside an image at any scale (which the reference
    # leaves undefined): every particle's position, speed and age, the
    # compaction map and the sparse index equal on every frame and scale.
    from oracle_lib import PyrlkLib, black_margin_frames, diff_pyrlk
    frames = black_margin_frames(seed, rows, cols, n, 16 << (L - 1))
    o = PyrlkLib("oracle", rows, cols, L, 20, det, filt, merge)
    r = PyrlkLib("ref", rows, cols, L, 20, det, filt, merge)
    for t in range(n):
        o.run(frames[t])
        r.run(frames[t])
        bad = diff_pyrlk(o, r, L)
        assert not bad, "frame %d: %s" % (t, bad)
    live = [int((o.particles(s)["age"] > 0).sum()) for s in range(L)]
    assert live[0] > 500
    o.destroy()
    r.destroy()
