"""Checkpoint / resume through the C ABI: a tracker restored from a blob
continues bit for bit like the one that saved it (particles, features,
matches, stages, trajectories), also in a context that has run other frames
before, and a blob is refused by a context of another configuration."""
import numpy as np
import pytest

from stage_api import diff_snapshots

pytestmark = pytest.mark.gpu


def _cfgs():
    return [dict(rows=240, cols=320, nscales=3, detector_frequency=4),
            dict(rows=203, cols=317, nscales=3, detector_frequency=3)]


def _frames(n):
    from cuimg_gb300 import synth
    return [synth.frames(40, 240, 320, n), synth.frames(41, 203, 317, n)]


@pytest.mark.parametrize("graphs", [False, True])
def test_resume_continues_bit_for_bit(graphs):
    from cuimg_gb300 import BatchTracker
    n0, n1 = 9, 8
    vids = _frames(n0 + n1)
    a = BatchTracker(_cfgs(), graphs=graphs).enable_trajectories(12)
    for t in range(n0):
        a.run([v[t] for v in vids])
    blob = a.checkpoint()
    # b has a history of its own (other frames) before it loads the blob.
    b = BatchTracker(_cfgs(), graphs=graphs)
    other = _frames(5)
    for t in range(5):
        b.run([v[4 - t] for v in other])
    b.restore(blob)
    for t in range(n0, n0 + n1):
        a.run([v[t] for v in vids])
        b.run([v[t] for v in vids])
        for s in range(2):
            det = t % _cfgs()[s]["detector_frequency"] == 0
            bad = diff_snapshots(a.snapshot(s), b.snapshot(s), det)
            assert not bad, (t, s, bad)
            for l in range(3):
                xa, la = a.trajectories(s, l)
                xb, lb = b.trajectories(s, l)
                np.testing.assert_array_equal(la, lb)
                np.testing.assert_array_equal(xa, xb)
    assert a.nparticles(0) > 0
    a.close()
    b.close()


def test_blob_of_another_configuration_is_refused():
    from cuimg_gb300 import BatchTracker
    from cuimg_gb300._native import GbtError
    vids = _frames(2)
    a = BatchTracker(_cfgs())
    a.run([v[0] for v in vids])
    blob = a.checkpoint()
    c = BatchTracker([dict(rows=240, cols=320, nscales=3, detector_frequency=5),
                      dict(rows=203, cols=317, nscales=3, detector_frequency=3)])
    with pytest.raises(GbtError):
        c.restore(blob)
    with pytest.raises(GbtError):
        a.restore(blob[:100])
    a.close()
    c.close()
