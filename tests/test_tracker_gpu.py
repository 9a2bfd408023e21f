"""GPU tracker parity: the CUDA path through the C ABI against the reference's
golden outputs and the oracle restatement, bit-exact, stage by stage."""
import numpy as np
import pytest

from oracle_lib import golden_cases, load_golden, tracker_oracle
from stage_api import diff_snapshots, snapshot

pytestmark = pytest.mark.gpu

STAGE_KEYS = ("input", "s1", "s2", "contrast", "saliency", "mask", "sparse", "flow", "count", "stat_n", "stat_speed")


def _gpu_tracker(rows, cols, L, th=20, detf=10, filtf=1, graphs=False):
    from cuimg_gb300 import Tracker
    tr = Tracker((rows, cols), L, graphs=graphs)
    tr.strategy().set_detector_frequency(detf).set_filtering_frequency(filtf)
    for s in range(L):
        tr.scale(s).strategy().detector().set_n(9).set_fast_threshold(th)
    return tr


@pytest.mark.parametrize("case", golden_cases())
def test_gpu_matches_reference_golden(case):
    g = load_golden(case)
    rows, cols, L, th, detf, filtf, n, seed = [int(x) for x in g["meta"]]
    tr = _gpu_tracker(rows, cols, L, th, detf, filtf)
    for t in range(n):
        tr.run(g["frames"][t])
        for s in range(L):
            p = tr._particles(0, s)
            for k in ("pos", "speed", "age"):
                np.testing.assert_array_equal(p[k], g["f%d_s%d_%s" % (t, s, k)], err_msg="frame %d scale %d %s" % (t, s, k))
            np.testing.assert_array_equal(p["feat"], g["f%d_s%d_feat" % (t, s)], err_msg="frame %d scale %d feat" % (t, s))
            key = "f%d_s%d_matches" % (t, s)
            assert p["compact"] == (key in g.files)
            if key in g.files:
                np.testing.assert_array_equal(p["matches"], g[key])
    snap = tr.snapshot()
    last_was_detector = (n - 1) % detf == 0
    for s in range(L):
        for k in STAGE_KEYS:
            if k in ("saliency", "mask") and not last_was_detector:
                continue  # the stage dump recomputes these from the current frame
            np.testing.assert_array_equal(snap[s][k], g["last_s%d_%s" % (s, k)], err_msg="scale %d %s" % (s, k))
    tr.close()


def _compare_run(rows, cols, L, n, seed, detf=10, filtf=1, graphs=False, matcher=None, blur_rows=None,
                 match_tile=None, frames=None, stats=None, tile_cap=None):
    from cuimg_gb300 import synth
    from cuimg_gb300._native import cuda_lib
    if frames is None:
        frames = synth.frames(seed, rows, cols, n)
    tr = _gpu_tracker(rows, cols, L, 20, detf, filtf, graphs)
    if tile_cap is not None:
        assert cuda_lib().gbt_test_tile_capacity(tr._ensure(), tile_cap) == 0
    if matcher is not None:
        tr.set_tuning(0, matcher)
    if blur_rows is not None:
        tr.set_tuning(1, blur_rows)
    if match_tile is not None:
        tr.set_tuning(2, match_tile)
    o = tracker_oracle(rows, cols, L, 20, detf, filtf)
    for t in range(n):
        tr.run(frames[t])
        o.run(frames[t])
        bad = diff_snapshots(snapshot(o, L), tr.snapshot(), detector_frame=(t % detf == 0))
        assert not bad, "frame %d: %s" % (t, bad)
    total = tr.nparticles()
    if stats is not None:
        stats["fallbacks"] = tr.tile_fallbacks()
    tr.close()
    o.destroy()
    return total


@pytest.mark.parametrize("rows,cols,L,n,seed,detf", [
    (480, 640, 3, 24, 1, 10),
    (240, 320, 3, 16, 2, 1),
    (203, 317, 4, 12, 9, 3),
    (101, 133, 3, 10, 12, 1),
])
def test_gpu_matches_oracle(rows, cols, L, n, seed, detf):
    assert _compare_run(rows, cols, L, n, seed, detf) > 0


@pytest.mark.parametrize("n_fast,th", [(7, 10), (12, 35), (16, 5)])
def test_detector_arc_lengths_and_thresholds(n_fast, th):
    # FAST arc lengths other than 9 take the generic run test; the oracle keeps
    # the reference's branchy scan with its pre-test.
    from cuimg_gb300 import Tracker, synth
    rows, cols, L, n = 240, 320, 3, 8
    frames = synth.frames(21, rows, cols, n)
    tr = Tracker((rows, cols), L)
    tr.strategy().set_detector_frequency(2).set_filtering_frequency(1)
    for s in range(L):
        tr.scale(s).strategy().detector().set_n(n_fast).set_fast_threshold(th)
    o = tracker_oracle(rows, cols, L, th, 2, 1)
    o.lib.oracle_set_n(o.h, n_fast)
    for t in range(n):
        tr.run(frames[t])
        o.run(frames[t])
        bad = diff_snapshots(snapshot(o, L), tr.snapshot(), detector_frame=(t % 2 == 0))
        assert not bad, "frame %d: %s" % (t, bad)
    assert tr.nparticles() > 0 or n_fast == 16
    tr.close()
    o.destroy()


def test_gpu_matches_oracle_4k():
    # 3840x2160 with 5 scales: the largest benchmark geometry (fixed s1/s2 pitch).
    total = _compare_run(2160, 3840, 5, 3, 33, 10)
    assert total > 0


def test_gpu_matches_oracle_wider_than_the_fixed_pitch():
    # Levels wider than 4064 pixels take the runtime-pitch matcher.
    total = _compare_run(64, 4200, 2, 4, 34, 2)
    assert total > 0


def test_gpu_matches_oracle_1080p():
    # The headline geometry: 1920x1080, 4 scales, detector every 10 frames.
    total = _compare_run(1080, 1920, 4, 12, 5, 10)
    assert total > 50000


@pytest.mark.parametrize("matcher", [0, 1, 2, 3])
def test_matcher_variants_match_oracle(matcher):
    _compare_run(480, 640, 3, 14, 6, detf=5, matcher=matcher)


@pytest.mark.parametrize("match_tile", range(8))
def test_tile_shapes_match_oracle(match_tile):
    # Every CTA shape of the tiled matcher, with full (0..3) and slim (4..6)
    # staged margins.
    stats = {}
    _compare_run(480, 640, 3, 12, 6, detf=5, matcher=0, match_tile=match_tile, stats=stats)
    if match_tile < 4:
        assert stats["fallbacks"] == 0


def _jittered_frames(seed, rows, cols, n, amp):
    """A synthetic scene shifted by a random offset of up to `amp` pixels in
    each axis on every frame, so that predictions miss and descents run long."""
    from cuimg_gb300 import synth
    base = synth.frames(seed, rows + 2 * amp, cols + 2 * amp, 1)[0]
    rng = np.random.default_rng(seed)
    out = np.empty((n, rows, cols), np.uint8)
    for t in range(n):
        dy, dx = rng.integers(0, 2 * amp + 1, size=2)
        out[t] = base[dy:dy + rows, dx:dx + cols]
    return out


@pytest.mark.parametrize("match_tile", [4, 5, 6, 7])
def test_slim_tile_fallbacks_match_oracle(match_tile):
    # Long descents: the particles whose descent leaves the slim staged margins
    # are matched again from global memory, with the oracle's results.
    rows, cols, L, n = 480, 640, 3, 10
    stats = {}
    frames = _jittered_frames(41, rows, cols, n, 9)
    assert _compare_run(rows, cols, L, n, 41, detf=2, matcher=0, match_tile=match_tile, frames=frames,
                        stats=stats) > 0
    assert stats["fallbacks"] > 0


@pytest.mark.parametrize("tile_cap,graphs", [(1, False), (4, True), (64, False)])
def test_tile_list_overflow_matches_oracle(tile_cap, graphs):
    # Tile lists of 1, 4 or 64 particles: the particles beyond a tile's list
    # are matched by the overflow kernel from global memory, bit-exactly.
    assert _compare_run(480, 640, 3, 12, 7, detf=3, graphs=graphs, tile_cap=tile_cap) > 0


def test_tile_capacity_hook_rejects_bad_values():
    from cuimg_gb300._native import cuda_lib
    tr = _gpu_tracker(120, 160, 3)
    lib = cuda_lib()
    assert lib.gbt_test_tile_capacity(tr._ensure(), 0) != 0
    assert lib.gbt_test_tile_capacity(tr._ensure(), 1025) != 0
    assert lib.gbt_test_tile_capacity(tr._ensure(), 1024) == 0
    tr.close()


@pytest.mark.parametrize("blur_rows", [16, 32, 64])
def test_blur_strip_heights_match_oracle(blur_rows):
    # Strips of 16 / 32 / 64 rows: interior strips (no row checks) and the
    # strips at each level's first and last rows, on four uneven levels.
    assert _compare_run(203, 317, 4, 6, 9, detf=3, blur_rows=blur_rows) > 0


def test_graph_replay_matches_oracle():
    _compare_run(240, 320, 3, 14, 4, detf=3, graphs=True)


@pytest.mark.parametrize("groups", [1, 2, 0])
def test_batched_uneven_streams_match_per_stream_oracles(groups):
    # groups: the context's stream groups (0 = the default, here one per stream).
    from cuimg_gb300 import BatchTracker, synth
    shapes = [(240, 320, 3), (480, 640, 3), (135, 201, 2), (360, 480, 4)]
    cfgs = [dict(rows=r, cols=c, nscales=L, detector_threshold=20, detector_frequency=4) for r, c, L in shapes]
    bt = BatchTracker(cfgs, graphs=True, groups=groups)
    assert bt.groups() == (groups or 4)
    streams = [synth.Stream(100 + i, r, c) for i, (r, c, L) in enumerate(shapes)]
    oracles = [tracker_oracle(r, c, L, 20, 4, 1) for r, c, L in shapes]
    for t in range(9):
        frames = [s.frame(t) for s in streams]
        bt.run(frames)
        for i, (r, c, L) in enumerate(shapes):
            oracles[i].run(frames[i])
            bad = diff_snapshots(snapshot(oracles[i], L), bt.snapshot(i), detector_frame=(t % 4 == 0))
            assert not bad, "stream %d frame %d: %s" % (i, t, bad)
    bt.close()


def test_counts_read_sync_and_async_agree_across_groups():
    import ctypes
    from cuimg_gb300 import BatchTracker, synth
    from cuimg_gb300._native import check
    shapes = [(240, 320, 3), (120, 160, 2), (480, 640, 4)]
    cfgs = [dict(rows=r, cols=c, nscales=L, detector_threshold=20, detector_frequency=3) for r, c, L in shapes]
    bt = BatchTracker(cfgs, graphs=True, groups=2)
    streams = [synth.Stream(300 + i, r, c) for i, (r, c, L) in enumerate(shapes)]
    for t in range(7):
        bt.run([s.frame(t) for s in streams])
    n = sum(L for _, _, L in shapes)
    a = np.zeros(n, np.int32)
    b = np.full(n, -1, np.int32)
    check(bt._lib.gbt_read_counts(bt._ctx, a.ctypes.data, n), bt._ctx)
    check(bt._lib.gbt_read_counts_async(bt._ctx, b.ctypes.data, n), bt._ctx)
    bt.sync()
    want = [bt.nparticles(s, l) for s, (_, _, L) in enumerate(shapes) for l in range(L)]
    assert a.tolist() == want and b.tolist() == want
    bt.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_resident_input_slots_alternate_and_match_gbt_run(graphs):
    # Frames written by the caller into the input slots (on the context stream)
    # and run with gbt_run_resident give the same tracks as gbt_run; the slot
    # of the next frame alternates between two buffers (frame pipeline).
    torch = pytest.importorskip("torch")
    from cuimg_gb300 import BatchTracker, synth
    shapes = [(240, 320, 3), (120, 160, 2), (200, 300, 3)]
    cfgs = [dict(rows=r, cols=c, nscales=L, detector_threshold=20, detector_frequency=3) for r, c, L in shapes]
    a = BatchTracker(cfgs, graphs=graphs, groups=2)
    b = BatchTracker(cfgs, graphs=graphs, groups=2)
    streams = [synth.Stream(500 + i, r, c) for i, (r, c, L) in enumerate(shapes)]
    stream = torch.cuda.ExternalStream(b.cuda_stream())
    import ctypes
    from cuimg_gb300._native import cuda_lib
    memcpy2d = cuda_lib().cudaMemcpy2DAsync  # the runtime the library links
    memcpy2d.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                         ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    slots = []
    for t in range(8):
        frames = [s.frame(t) for s in streams]
        a.run(frames)
        with torch.cuda.stream(stream):
            for k, f in enumerate(frames):
                ptr, pitch = b.input_slot(k)
                if k == 0:
                    slots.append(ptr)
                h, w = f.shape
                src = torch.from_numpy(f).to("cuda")
                torch.cuda.current_stream().synchronize()
                # Into the pitched slot, ordered on the context stream (cudaMemcpyDeviceToDevice = 3).
                assert memcpy2d(ptr, pitch, src.data_ptr(), w, w, h, 3, stream.cuda_stream) == 0
        b.run_resident()
        for k, (r, c, L) in enumerate(shapes):
            bad = diff_snapshots(a.snapshot(k), b.snapshot(k), detector_frame=(t % 3 == 0))
            assert not bad, "stream %d frame %d: %s" % (k, t, bad)
    assert slots[0] != slots[1] and slots[0] == slots[2]
    a.close()
    b.close()


def test_rgb_input_tracks_channel_zero():
    from cuimg_gb300 import synth
    s = synth.Stream(7, 120, 160)
    a = _gpu_tracker(120, 160, 2, detf=2)
    b = _gpu_tracker(120, 160, 2, detf=2)
    for t in range(5):
        a.run(s.frame(t))
        b.run(s.frame_rgb(t))
    assert not diff_snapshots(a.snapshot(), b.snapshot(), True)


@pytest.mark.parametrize("where", ["host", "host_pinned", "device"])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("rows,cols,L", [(120, 160, 2), (121, 163, 1), (133, 301, 3)])
def test_rgb_ingest_fused_in_pyramid(where, mode, rows, cols, L):
    # RGB frames go to the device as they are and become gray inside the
    # pyramid kernel; the result must equal tracking the gray image directly.
    torch = pytest.importorskip("torch")
    from cuimg_gb300 import synth
    from cuimg_gb300.tracker import GBT_FRAMES_DEVICE_RGB, GBT_FRAMES_HOST_RGB
    s = synth.Stream(17, rows, cols)
    rng = np.random.default_rng(3)
    a = _gpu_tracker(rows, cols, L, detf=2)
    b = _gpu_tracker(rows, cols, L, detf=2)
    b.set_rgb_to_gray(mode)
    for t in range(5):
        rgb = s.frame_rgb(t).copy()
        rgb[..., 1] = rng.integers(0, 256, rgb.shape[:2])  # make the channels differ
        r, g, bl = (rgb[..., k].astype(np.int32) for k in range(3))
        gray = rgb[..., 0] if mode == 0 else ((77 * r + 150 * g + 29 * bl + 128) >> 8).astype(np.uint8)
        a.run(np.ascontiguousarray(gray))
        if where == "host":
            b.run(rgb)
        elif where == "host_pinned":
            h = torch.from_numpy(rgb).pin_memory()
            b.run((h.data_ptr(), cols * 3), location=GBT_FRAMES_HOST_RGB)
            b.sync()
        else:
            d = torch.from_numpy(rgb).cuda()
            b.run((d.data_ptr(), cols * 3), location=GBT_FRAMES_DEVICE_RGB)
            b.sync()
        assert not diff_snapshots(a.snapshot(), b.snapshot(), t % 2 == 0), t
    a.close()
    b.close()


def test_deterministic_across_runs():
    from cuimg_gb300 import synth
    frames = synth.frames(8, 240, 320, 8)
    snaps = []
    for _ in range(2):
        tr = _gpu_tracker(240, 320, 3, detf=2)
        for f in frames:
            tr.run(f)
        snaps.append(tr.snapshot())
        tr.close()
    assert not diff_snapshots(snaps[0], snaps[1], True)


def test_flat_and_empty_frames():
    tr = _gpu_tracker(64, 96, 2, detf=1)
    for _ in range(3):
        tr.run(np.full((64, 96), 77, np.uint8))
    assert tr.nparticles() == 0
    assert tr.stage(0, 0, "contrast").max() == 0
    tr.close()


def test_bounded_tile_wait_reports_timeout_and_the_device_stays_usable():
    # The tiled matcher waits for its TMA-staged tile on an mbarrier with a
    # time limit.  With the copies withheld nothing completes the barrier:
    # every tile's wait gives up, the next gbt_sync reports GBT_E_TIMEOUT, and
    # no fault follows -- a fresh context on the same device then tracks
    # bit-exactly.
    import time

    from cuimg_gb300 import GbtError, synth
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    frames = synth.frames(5, 240, 320, 3)
    tr = _gpu_tracker(240, 320, 2, detf=10, graphs=True)
    for t in range(2):
        tr.run(frames[t])
    tr.sync()
    assert tr.nparticles() > 0
    assert lib.gbt_test_withhold_tile_copies(tr._ensure(), 1) == 0
    t0 = time.perf_counter()
    with pytest.raises(GbtError) as e:
        tr.run(frames[2])
        tr.sync()
    assert e.value.code == 5
    assert time.perf_counter() - t0 < 30.0
    tr.close()
    # Another matcher variant has no tile copies to withhold.
    tr = _gpu_tracker(64, 96, 1)
    tr.set_tuning(0, 2)
    assert lib.gbt_test_withhold_tile_copies(tr._ensure(), 1) == 1
    tr.close()
    assert _compare_run(240, 320, 2, 4, 5) > 0


def test_invalid_geometry_rejected():
    from cuimg_gb300 import GbtError, Tracker
    tr = Tracker((97, 131), 3)
    with pytest.raises(GbtError):
        tr.run(np.zeros((97, 131), np.uint8))


def _apply_setter(strategy, key, value):
    """One of the reference's setters on a scale's strategy() (keys of
    gbt_set_param)."""
    if key == 0:
        strategy.detector().set_fast_threshold(value)
    elif key == 1:
        strategy.detector().set_n(value)
    elif key == 2:
        strategy.set_detector_frequency(value)
    elif key == 3:
        strategy.set_filtering_frequency(value)
    elif key == 4:
        strategy.set_k(value)
    else:
        strategy.set_with_merge(bool(value))


@pytest.mark.parametrize("graphs", [False, True])
def test_runtime_setters_match_oracle(graphs):
    # Settings changed between frames through the reference-style setters
    # (gbt_set_param): per-scale thresholds and arc length, frequencies and k
    # forwarded to the coarser scales, merge off on one scale; every stage of
    # every frame bit-exact with the oracle given the same calls, with and
    # without graph replay.
    from cuimg_gb300 import synth
    from stage_api import SETTER_SCHEDULE, SettingsTrack, scales_set_by
    rows, cols, L, n = 240, 320, 3, 18
    frames = synth.frames(12, rows, cols, n)
    tr = _gpu_tracker(rows, cols, L, 20, 10, 1, graphs)
    o = tracker_oracle(rows, cols, L, 20, 10, 1)
    track = SettingsTrack(L, 10, 1)
    for t in range(n):
        for (ft, scale, key, value) in SETTER_SCHEDULE:
            if ft == t:
                _apply_setter(tr.scale(scale).strategy(), key, value)
                for s in scales_set_by(L, scale, key):
                    o.set_param(s, key, value)
                track.apply(L, scale, key, value)
        tr.run(frames[t])
        o.run(frames[t])
        bad = diff_snapshots(snapshot(o, L), tr.snapshot(), detector_frame=track.all_detect(t))
        assert not bad, "frame %d: %s" % (t, bad)
    assert tr.get_param("detector_threshold", 0, 1) == 35
    assert tr.get_param("detector_frequency", 0, 2) == 2 and tr.get_param("detector_frequency", 0, 0) == 3
    tr.close()
    o.destroy()


def test_runtime_setter_on_one_stream_of_a_batch():
    # A setter on one stream of a batch changes that stream only.
    from cuimg_gb300 import BatchTracker, synth
    rows, cols, L, n = 240, 320, 3, 12
    vids = [synth.frames(30 + i, rows, cols, n) for i in range(2)]
    bt = BatchTracker([dict(rows=rows, cols=cols, nscales=L, detector_threshold=20, detector_frequency=10)] * 2,
                      graphs=True, groups=1)
    os_ = [tracker_oracle(rows, cols, L, 20, 10, 1) for _ in range(2)]
    for t in range(n):
        if t == 3:
            bt._set_param(1, 0, "detector_frequency", 2)
            for s in range(L):
                os_[1].set_param(s, 2, 2)
        bt.run([v[t] for v in vids])
        for i in range(2):
            os_[i].run(vids[i][t])
            bad = diff_snapshots(snapshot(os_[i], L), bt.snapshot(i), detector_frame=False)
            assert not bad, "stream %d frame %d: %s" % (i, t, bad)
    bt.close()
    for o in os_:
        o.destroy()
