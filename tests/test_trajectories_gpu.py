"""Device-side trajectories against the reference's host-side bookkeeping:
particle_container::sync_attributes (particle_container.hpp:514-553) followed
by the sample's update_trajectories (samples/tracking/main.cc:39-57), replayed
in Python on the oracle's particles, matches and compaction flags, frame by
frame.  Bit-exact."""
import numpy as np
import pytest

from oracle_lib import tracker_oracle

pytestmark = pytest.mark.gpu


def sync_and_update(v, parts, compact, T):
    """One frame of the sample's trajectory bookkeeping on a list of lists."""
    n = len(parts["age"])
    if compact:
        tmp = [[] for _ in range(n)]
        for i, ni in enumerate(parts["matches"]):
            if ni >= 0 and i < len(v):
                tmp[ni] = v[i]
        v = tmp
    else:
        v = (v + [[] for _ in range(n - len(v))])[:n]
    for i in range(n):
        if parts["age"][i] > 0:
            v[i] = v[i] + [tuple(int(x) for x in parts["pos"][i])]
            if len(v[i]) > T:
                v[i] = v[i][1:]
        else:
            v[i] = []
    return v


@pytest.mark.parametrize("rows,cols,L,n,detf,T,graphs", [
    (240, 320, 3, 26, 5, 20, False),
    (203, 317, 3, 14, 3, 6, True),
])
def test_trajectories_match_sync_attributes(rows, cols, L, n, detf, T, graphs):
    from cuimg_gb300 import Tracker, synth
    frames = synth.frames(31, rows, cols, n)
    tr = Tracker((rows, cols), L, graphs=graphs)
    tr.strategy().set_detector_frequency(detf).set_filtering_frequency(1)
    tr.enable_trajectories(T)
    o = tracker_oracle(rows, cols, L, 20, detf, 1)
    hist = [[] for _ in range(L)]
    for t in range(n):
        tr.run(frames[t])
        o.run(frames[t])
        for s in range(L):
            parts = o.particles(s)
            hist[s] = sync_and_update(hist[s], parts, o.compact_has_run(s), T)
            xy, ln = tr.trajectories(0, s)
            assert len(ln) == len(hist[s]), (t, s)
            want_len = np.array([len(h) for h in hist[s]], np.uint8)
            np.testing.assert_array_equal(ln, want_len, err_msg="frame %d scale %d lengths" % (t, s))
            for j, h in enumerate(hist[s]):
                if h:
                    np.testing.assert_array_equal(xy[j, :len(h)], np.array(h, np.int16),
                                                  err_msg="frame %d scale %d slot %d" % (t, s, j))
    assert max(len(h) for h in hist[0]) >= min(T, 6)  # histories long enough to wrap the ring at T = 6
    tr.close()
    o.destroy()
