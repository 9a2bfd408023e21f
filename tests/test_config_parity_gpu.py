"""GPU parity on the configurations the benchmark measures.

* The plain tracker configuration: 640x480 gray, 3 scales, FAST threshold 20,
  30 frames, every stage of every frame (detector every 10 frames as the
  reference's sample, and every frame as a stress case).
* 1920x1080 RGB through the fused ingest (channel 0 tracked, as the sample's
  get_x), 4 scales, all 120 frames, one stream.
* The benchmark's own workload: 16 streams of 1920x1080 in the default stream
  groups with CUDA-graph replay, two streams of every group checked against
  their own oracles on every frame.

Bit-exact against the oracle (which is bit-exact against the reference's own
CPU tracker).  The oracles of several streams run in threads (their C calls
release the interpreter lock).
"""
import concurrent.futures as cf

import numpy as np
import pytest

from oracle_lib import tracker_oracle
from stage_api import diff_snapshots, snapshot

pytestmark = pytest.mark.gpu

PARTICLE_KEYS = ("pos", "speed", "age", "feat")


def _frames(seeds, rows, cols, n):
    from cuimg_gb300 import synth
    with cf.ThreadPoolExecutor(max_workers=16) as ex:
        return list(ex.map(lambda s: synth.frames(s, rows, cols, n), seeds))


def _same_particles(o, gpu_snap_particles, s):
    p = o.particles(s)
    g = gpu_snap_particles
    for k in ("pos", "speed", "age"):
        if not np.array_equal(p[k], g[k]):
            return k
    if not np.array_equal(p["feat"][:, :16], g["feat"]):
        return "feat"
    if o.compact_has_run(s) != g["compact"]:
        return "compact"
    if g["compact"] and not np.array_equal(p["matches"], g["matches"]):
        return "matches"
    return None


@pytest.mark.parametrize("detf", [10, 1])
def test_plain_640x480_30_frames(detf):
    from cuimg_gb300 import Tracker
    rows, cols, L, n = 480, 640, 3, 30
    frames = _frames([1], rows, cols, n)[0]
    tr = Tracker((rows, cols), L, detector_threshold=20, detector_frequency=detf)
    o = tracker_oracle(rows, cols, L, 20, detf, 1)
    for t in range(n):
        tr.run(frames[t])
        o.run(frames[t])
        bad = diff_snapshots(snapshot(o, L), tr.snapshot(), detector_frame=(t % detf == 0))
        assert not bad, "frame %d: %s" % (t, bad)
    assert tr.nparticles() > 10000
    tr.close()
    o.destroy()


def test_rgb_1080p_120_frames_fused_ingest():
    from cuimg_gb300 import Tracker
    rows, cols, L, n = 1080, 1920, 4, 120
    gray, g2, g3 = _frames([2, 502, 902], rows, cols, n)
    tr = Tracker((rows, cols), L, detector_threshold=20, detector_frequency=10, graphs=True)
    o = tracker_oracle(rows, cols, L, 20, 10, 1)
    rgb = np.empty((rows, cols, 3), np.uint8)
    for t in range(n):
        rgb[..., 0], rgb[..., 1], rgb[..., 2] = gray[t], g2[t], g3[t]  # channel 0 is tracked
        tr.run(rgb)
        o.run(gray[t])
        for s in range(L):
            bad = _same_particles(o, tr._particles(0, s), s)
            assert bad is None, "frame %d scale %d: %s" % (t, s, bad)
        if t % 10 == 9 or t == n - 1:
            bad = diff_snapshots(snapshot(o, L), tr.snapshot(), detector_frame=(t % 10 == 0))
            assert not bad, "frame %d: %s" % (t, bad)
    live = sum(int((tr._particles(0, s)["age"] > 0).sum()) for s in range(L))
    assert live > 10000
    tr.close()
    o.destroy()


def test_benchmark_workload_16_streams_in_groups_with_graphs():
    from cuimg_gb300 import BatchTracker
    rows, cols, L, B, n = 1080, 1920, 4, 16, 40
    vids = _frames([1000 + i for i in range(B)], rows, cols, n)  # the benchmark's seeds
    cfg = [dict(rows=rows, cols=cols, nscales=L, detector_threshold=20, detector_frequency=10,
                filtering_frequency=1)] * B
    bt = BatchTracker(cfg, graphs=True)  # default grouping, as the benchmark
    groups = bt.groups()
    assert groups == 4
    # The library balances streams over groups by pixels (equal here): stream
    # i goes to group i % 4 in that case, so streams 0..7 cover every group twice.
    checked = list(range(8))
    oracles = {i: tracker_oracle(rows, cols, L, 20, 10, 1) for i in checked}
    with cf.ThreadPoolExecutor(max_workers=len(checked)) as ex:
        for t in range(n):
            bt.run([v[t] for v in vids])
            list(ex.map(lambda i: oracles[i].run(vids[i][t]), checked))
            for i in checked:
                for s in range(L):
                    bad = _same_particles(oracles[i], bt._particles(i, s), s)
                    assert bad is None, "stream %d frame %d scale %d: %s" % (i, t, s, bad)
    for i in checked[:2]:
        bad = diff_snapshots(snapshot(oracles[i], L), bt.snapshot(i), detector_frame=False)
        assert not bad, "stream %d last frame: %s" % (i, bad)
    bt.close()
    for o in oracles.values():
        o.destroy()
