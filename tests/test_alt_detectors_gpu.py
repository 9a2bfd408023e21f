"""The reference's other detectors on the GPU: regular_detector
(bc2s_regular_gradient_cpu) and dense_detector (bc2s_dense_gradient_cpu),
bit-exact against the reference's golden outputs and the oracle, alone and
mixed with FAST streams in one context."""
import numpy as np
import pytest

from oracle_lib import alt_golden_cases, alt_tracker_oracle, load_golden, tracker_oracle
from stage_api import diff_snapshots, snapshot

pytestmark = pytest.mark.gpu


def _gpu(kind, rows, cols, L, detf, step=1, grad_th=1):
    from cuimg_gb300 import Tracker
    return Tracker((rows, cols), L, detector_frequency=detf, filtering_frequency=1, detector=kind,
                   detector_step=step, detector_grad_th=grad_th)


@pytest.mark.parametrize("case", alt_golden_cases())
def test_gpu_alt_detector_matches_reference_golden(case):
    g = load_golden(case)
    kind, rows, cols, L, detf, filtf, n, seed, step, grad_th = [int(x) for x in g["meta"]]
    tr = _gpu(kind, rows, cols, L, detf, step, grad_th)
    for t in range(n):
        tr.run(g["frames"][t])
        for s in range(L):
            p = tr._particles(0, s)
            for k in ("pos", "speed", "age"):
                np.testing.assert_array_equal(p[k], g["f%d_s%d_%s" % (t, s, k)], err_msg="f%d s%d %s" % (t, s, k))
            np.testing.assert_array_equal(p["feat"], g["f%d_s%d_feat" % (t, s)], err_msg="f%d s%d feat" % (t, s))
            key = "f%d_s%d_matches" % (t, s)
            assert p["compact"] == (key in g.files)
            if key in g.files:
                np.testing.assert_array_equal(p["matches"], g[key])
    tr.close()


@pytest.mark.parametrize("kind,rows,cols,L,detf,n,step,grad_th", [
    (1, 240, 320, 3, 3, 10, 2, 5),
    (1, 203, 317, 3, 4, 9, 3, 12),
    (2, 96, 128, 2, 2, 6, 1, 1),
    (2, 125, 167, 3, 5, 8, 1, 1),
])
def test_gpu_alt_detector_matches_oracle(kind, rows, cols, L, detf, n, step, grad_th):
    from cuimg_gb300 import synth
    frames = synth.frames(50 + kind, rows, cols, n)
    tr = _gpu(kind, rows, cols, L, detf, step, grad_th)
    o = alt_tracker_oracle(kind, rows, cols, L, detf, 1, step, grad_th)
    for t in range(n):
        tr.run(frames[t])
        o.run(frames[t])
        bad = diff_snapshots(snapshot(o, L), tr.snapshot(), t % detf == 0, fast_detector=False)
        assert not bad, "frame %d: %s" % (t, bad)
    assert tr.nparticles() > 0
    tr.close()
    o.destroy()


def test_mixed_detectors_in_one_context():
    from cuimg_gb300 import BatchTracker, synth
    specs = [(0, 240, 320, 3, 3, 1, 1), (1, 203, 317, 3, 2, 3, 8), (2, 96, 128, 2, 3, 1, 1)]
    cfgs = [dict(rows=r, cols=c, nscales=L, detector_frequency=d, detector=k, detector_step=st, detector_grad_th=gt)
            for k, r, c, L, d, st, gt in specs]
    bt = BatchTracker(cfgs, graphs=True)
    oracles = [tracker_oracle(r, c, L, 20, d, 1) if k == 0 else alt_tracker_oracle(k, r, c, L, d, 1, st, gt)
               for k, r, c, L, d, st, gt in specs]
    vids = [synth.frames(60 + i, r, c, 8) for i, (k, r, c, L, d, st, gt) in enumerate(specs)]
    for t in range(8):
        bt.run([v[t] for v in vids])
        for i, (k, r, c, L, d, st, gt) in enumerate(specs):
            oracles[i].run(vids[i][t])
            bad = diff_snapshots(snapshot(oracles[i], L), bt.snapshot(i), t % d == 0, fast_detector=(k == 0))
            assert not bad, "stream %d frame %d: %s" % (i, t, bad)
    bt.close()
    for o in oracles:
        o.destroy()


def test_capacity_overflow_is_reported():
    # The regular detector with step 1 and grad_th 0 adds a particle at every
    # pixel of every detector frame; without merging or filtering the set
    # outgrows its capacity (4 x pixels + 4096) on the fifth frame.  The
    # births beyond it are dropped and gbt_sync reports GBT_E_CAPACITY.
    from cuimg_gb300 import Tracker, synth
    from cuimg_gb300._native import GbtError
    rows, cols = 120, 160
    frames = synth.frames(71, rows, cols, 6)
    tr = Tracker((rows, cols), 1, detector_frequency=1, filtering_frequency=1000, with_merge=0, detector=1,
                 detector_step=1, detector_grad_th=0)
    for t in range(4):
        tr.run(frames[t])
    tr.sync()
    assert tr.nparticles() > 3 * rows * cols
    with pytest.raises(GbtError) as e:
        for t in range(4, 6):
            tr.run(frames[t])
        tr.sync()
    assert e.value.code == 4
    tr.close()
