"""The pyramidal LK tracker strategy on the GPU (gbt_config.matcher =
GBT_MATCHER_LK) against the oracle's restatement of the reference's
pyrlk_cpu<fast_detector<cpu>, iterative_lk_match_5x5>, which the CPU tests pin
bit for bit against the reference itself.  Every frame and scale: positions,
speeds and ages of every particle slot, the compaction map and the sparse
index -- bit-exact, since the GPU path evaluates the LK in the reference's
floating-point order."""
import numpy as np
import pytest

from oracle_lib import PyrlkLib, black_margin_frames, diff_pyrlk

pytestmark = pytest.mark.gpu


class GpuView:
    """diff_pyrlk's view of one stream of a GPU LK tracker."""

    def __init__(self, bt, stream=0):
        self.bt, self.stream = bt, stream

    def particles(self, s):
        return self.bt.particles_f(self.stream, s)

    def sparse(self, s):
        return self.bt.stage(self.stream, s, "sparse")


def _lk_tracker(rows, cols, L, det, filt, merge):
    from cuimg_gb300 import Tracker
    tr = Tracker((rows, cols), L, matcher="lk", detector_threshold=20, detector_frequency=det,
                 filtering_frequency=filt, with_merge=merge)
    return tr


@pytest.mark.parametrize("rows,cols,L,det,filt,merge,seed,n,margin", [
    (240, 320, 3, 3, 1, 1, 3, 14, 0),
    (480, 640, 3, 10, 1, 1, 1, 30, 0),     # the plain tracker configuration's geometry
    (320, 480, 3, 3, 1, 1, 5, 16, 64),     # a clip the oracle is pinned on against the reference
    (257, 391, 2, 1, 2, 0, 8, 10, 0),
    (1080, 1920, 4, 10, 1, 1, 2, 12, 0),
])
def test_lk_tracker_matches_oracle_every_frame(rows, cols, L, det, filt, merge, seed, n, margin):
    from cuimg_gb300 import synth
    frames = black_margin_frames(seed, rows, cols, n, margin) if margin else synth.frames(seed, rows, cols, n)
    tr = _lk_tracker(rows, cols, L, det, filt, merge)
    o = PyrlkLib("oracle", rows, cols, L, 20, det, filt, merge)
    g = GpuView(tr)
    for t in range(n):
        tr.run(frames[t])
        o.run(frames[t])
        bad = diff_pyrlk(o, g, L)
        assert not bad, "frame %d: %s" % (t, bad)
    live = int((tr.particles_f(0, 0)["age"] > 0).sum())
    assert live > 200
    tr.close()
    o.destroy()


def test_lk_tracker_batch_of_uneven_streams():
    from cuimg_gb300 import BatchTracker, synth
    shapes = [(240, 320, 3), (480, 640, 3), (200, 288, 2)]
    n = 12
    vids = [synth.frames(60 + i, r, c, n) for i, (r, c, L) in enumerate(shapes)]
    bt = BatchTracker([dict(rows=r, cols=c, nscales=L, matcher=1, detector_threshold=20, detector_frequency=4)
                       for r, c, L in shapes])
    os_ = [PyrlkLib("oracle", r, c, L, 20, 4, 1, 1) for r, c, L in shapes]
    for t in range(n):
        bt.run([v[t] for v in vids])
        for i, (r, c, L) in enumerate(shapes):
            os_[i].run(vids[i][t])
            bad = diff_pyrlk(os_[i], GpuView(bt, i), L)
            assert not bad, "stream %d frame %d: %s" % (i, t, bad)
    bt.close()
    for o in os_:
        o.destroy()


def test_lk_tracker_runtime_setters():
    # The strategy's setters between frames: per-scale thresholds and arc
    # length, frequencies forwarded to the coarser scales, k and merge per
    # scale (pyrlk_cpu's set_k does not forward).
    from cuimg_gb300 import synth
    rows, cols, L, n = 240, 320, 3, 16
    frames = synth.frames(21, rows, cols, n)
    tr = _lk_tracker(rows, cols, L, 10, 1, 1)
    o = PyrlkLib("oracle", rows, cols, L, 20, 10, 1, 1)
    sched = {2: [(0, "detector_frequency", 2, 3)], 4: [(1, "threshold", 0, 35), (2, "threshold", 0, 12)],
             6: [(1, "with_merge", 5, 0)], 8: [(1, "k", 4, 30)], 11: [(2, "filtering_frequency", 3, 2)],
             12: [(0, "n", 1, 12)]}
    for t in range(n):
        for scale, what, key, value in sched.get(t, []):
            st = tr.scale(scale).strategy()
            if what == "threshold":
                st.detector().set_fast_threshold(value)
            elif what == "n":
                st.detector().set_n(value)
            elif what == "detector_frequency":
                st.set_detector_frequency(value)
            elif what == "filtering_frequency":
                st.set_filtering_frequency(value)
            elif what == "k":
                st.set_k(value)
            else:
                st.set_with_merge(bool(value))
            for s in (range(scale, L) if key in (2, 3) else [scale]):
                o.set_param(s, key, value)
        tr.run(frames[t])
        o.run(frames[t])
        bad = diff_pyrlk(o, GpuView(tr), L)
        assert not bad, "frame %d: %s" % (t, bad)
    assert tr.get_param("k", 0, 1) == 30 and tr.get_param("k", 0, 2) == 300
    tr.close()
    o.destroy()


def test_lk_context_refuses_what_it_does_not_keep():
    import ctypes

    from cuimg_gb300._native import cuda_lib
    tr = _lk_tracker(120, 160, 2, 1, 1, 1)
    ctx = tr._ensure()
    lib = cuda_lib()
    assert lib.gbt_use_graphs(ctx, 1) == 1
    buf = ctypes.create_string_buffer(256)
    lib.gbt_last_error(ctx, buf, 256)
    assert b"LK matcher" in buf.value
    assert lib.gbt_trajectories_enable(ctx, 10) == 1
    tr.close()
