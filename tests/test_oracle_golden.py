"""Pins the oracle: the C restatement against the reference's own outputs.

Golden fixtures (tests/golden/*.npz, *.json) were produced by running the
reference code itself (tests/golden/make_golden.py).  Where the reference is
built in this container (oracle/_ref), extra seeds and sizes are compared live.
"""
import json
import os

import numpy as np
import pytest

from oracle_lib import (GOLDEN, alt_golden_cases, alt_reference, alt_reference_particles, alt_tracker_oracle, box_pyramid_u8, gauss_pyramid,
                        gauss_sep, gauss_taps, golden_cases, load_golden, oracle, reference_available, tracker_oracle,
                        tracker_reference)
from stage_api import diff_snapshots, snapshot

STAGE_KEYS = ("input", "s1", "s2", "contrast", "saliency", "mask", "sparse", "flow", "count", "stat_n", "stat_speed")


def _check_against_golden(lib, g):
    rows, cols, L, th, detf, filtf, n, seed = [int(x) for x in g["meta"]]
    for t in range(n):
        lib.run(g["frames"][t])
        for s in range(L):
            p = lib.particles(s)
            for k in ("pos", "speed", "age"):
                np.testing.assert_array_equal(p[k], g["f%d_s%d_%s" % (t, s, k)], err_msg="frame %d scale %d %s" % (t, s, k))
            np.testing.assert_array_equal(p["feat"][:, :16], g["f%d_s%d_feat" % (t, s)])
            key = "f%d_s%d_matches" % (t, s)
            assert lib.compact_has_run(s) == (key in g.files)
            if key in g.files:
                np.testing.assert_array_equal(p["matches"], g[key])
    snap = snapshot(lib, L)
    for s in range(L):
        for k in STAGE_KEYS:
            np.testing.assert_array_equal(snap[s][k], g["last_s%d_%s" % (s, k)], err_msg="scale %d %s" % (s, k))


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_matches_reference_golden(case):
    g = load_golden(case)
    rows, cols, L, th, detf, filtf, n, seed = [int(x) for x in g["meta"]]
    o = tracker_oracle(rows, cols, L, th, detf, filtf)
    try:
        _check_against_golden(o, g)
    finally:
        o.destroy()


def test_golden_weights_constant_255():
    # The restatement (and the CUDA path) store 16 feature bytes because the
    # reference's 16 weights are never anything but 255 on this path.
    for case in golden_cases():
        g = load_golden(case)
        for k in g.files:
            if k.endswith("weights_all_255"):
                assert bool(g[k])


@pytest.mark.skipif(not reference_available(), reason="reference not built here (oracle/_ref)")
@pytest.mark.parametrize("rows,cols,L,detf,n,seed", [
    (240, 320, 3, 10, 22, 11),
    (135, 201, 2, 2, 12, 4),
    (203, 317, 4, 1, 8, 9),
])
def test_oracle_matches_reference_live(rows, cols, L, detf, n, seed):
    from cuimg_gb300 import synth
    frames = synth.frames(seed, rows, cols, n)
    ref = tracker_reference(rows, cols, L, 20, detf, 1)
    o = tracker_oracle(rows, cols, L, 20, detf, 1)
    for t in range(n):
        ref.run(frames[t])
        o.run(frames[t])
        bad = diff_snapshots(snapshot(ref, L), snapshot(o, L), detector_frame=(t % detf == 0))
        assert not bad, "frame %d: %s" % (t, bad)
    ref.destroy()
    o.destroy()


@pytest.mark.skipif(not reference_available(), reason="reference not built here (oracle/_ref)")
@pytest.mark.parametrize("rows,cols,L,seed", [(240, 320, 3, 12), (480, 640, 3, 1)])
def test_oracle_runtime_setters_match_reference_live(rows, cols, L, seed):
    # The reference's setters called between frames (per-scale thresholds,
    # frequencies, k, merge, arc length; SETTER_SCHEDULE) and the oracle's
    # oracle_set_param on the scales each call sets: every stage of every
    # frame equal.
    from cuimg_gb300 import synth
    from stage_api import SETTER_SCHEDULE, SettingsTrack, scales_set_by
    n = 18
    frames = synth.frames(seed, rows, cols, n)
    ref = tracker_reference(rows, cols, L, 20, 10, 1)
    o = tracker_oracle(rows, cols, L, 20, 10, 1)
    track = SettingsTrack(L, 10, 1)
    for t in range(n):
        for (ft, scale, key, value) in SETTER_SCHEDULE:
            if ft == t and scale < L:
                ref.set_param(scale, key, value)
                for s in scales_set_by(L, scale, key):
                    o.set_param(s, key, value)
                track.apply(L, scale, key, value)
        ref.run(frames[t])
        o.run(frames[t])
        bad = diff_snapshots(snapshot(ref, L), snapshot(o, L), detector_frame=track.all_detect(t))
        assert not bad, "frame %d: %s" % (t, bad)
    ref.destroy()
    o.destroy()


@pytest.mark.skipif(not reference_available(), reason="reference not built here (oracle/_ref)")
def test_oracle_matches_reference_live_random_geometries():
    # Seeded random geometries, scale counts, thresholds and detector periods
    # (GBT_REF_SWEEP cases, default 40; larger sweeps: GBT_REF_SWEEP=300),
    # every stage of every frame compared.
    from cuimg_gb300 import synth
    rng = np.random.default_rng(20261203)
    lib = oracle()
    done, total = 0, int(os.environ.get("GBT_REF_SWEEP", "40"))
    while done < total:
        rows, cols, L = int(rng.integers(40, 400)), int(rng.integers(40, 600)), int(rng.integers(1, 5))
        detf, n, seed = int(rng.choice([1, 2, 3, 5, 10])), int(rng.integers(4, 12)), int(rng.integers(0, 1000))
        th = int(rng.choice([10, 20, 30]))
        if not lib.oracle_sizes_ok(rows, cols, L):
            continue
        frames = synth.frames(seed, rows, cols, n)
        ref = tracker_reference(rows, cols, L, th, detf, 1)
        o = tracker_oracle(rows, cols, L, th, detf, 1)
        for t in range(n):
            ref.run(frames[t])
            o.run(frames[t])
            bad = diff_snapshots(snapshot(ref, L), snapshot(o, L), detector_frame=(t % detf == 0))
            assert not bad, "%dx%d L%d det/%d th%d seed %d frame %d: %s" % (rows, cols, L, detf, th, seed, t, bad)
        ref.destroy()
        o.destroy()
        done += 1


def _alt_check(get, g, L, n, tag):
    for t in range(n):
        for s in range(L):
            p = get(t, s)
            for k in ("pos", "speed", "age"):
                np.testing.assert_array_equal(p[k], g["f%d_s%d_%s" % (t, s, k)], err_msg="%s f%d s%d %s" % (tag, t, s, k))
            np.testing.assert_array_equal(p["feat"][:, :16], g["f%d_s%d_feat" % (t, s)], err_msg="%s f%d s%d feat" % (tag, t, s))
            key = "f%d_s%d_matches" % (t, s)
            if key in g.files:
                np.testing.assert_array_equal(p["matches"], g[key], err_msg="%s f%d s%d matches" % (tag, t, s))


@pytest.mark.parametrize("case", alt_golden_cases())
def test_alt_detector_oracle_matches_reference_golden(case):
    # The regular and dense detectors of the reference's generic strategy.
    g = load_golden(case)
    kind, rows, cols, L, detf, filtf, n, seed, step, grad_th = [int(x) for x in g["meta"]]
    o = alt_tracker_oracle(kind, rows, cols, L, detf, filtf, step, grad_th)
    snaps = []
    for t in range(n):
        o.run(g["frames"][t])
        snaps.append([o.particles(s) for s in range(L)])
    _alt_check(lambda t, s: snaps[t][s], g, L, n, case)
    o.destroy()


@pytest.mark.skipif(not reference_available(), reason="reference not built here (oracle/_ref)")
@pytest.mark.parametrize("kind,rows,cols,L,detf,n,step,grad_th", [
    (1, 101, 133, 3, 2, 7, 2, 5),
    (2, 60, 90, 2, 3, 6, 1, 1),
])
def test_alt_detector_oracle_matches_reference_live(kind, rows, cols, L, detf, n, step, grad_th):
    from cuimg_gb300 import synth
    frames = synth.frames(13, rows, cols, n)
    lib, h = alt_reference(kind, rows, cols, L, detf, 1, step, grad_th)
    o = alt_tracker_oracle(kind, rows, cols, L, detf, 1, step, grad_th)
    for t in range(n):
        lib.refx_run(h, frames[t].ctypes.data)
        o.run(frames[t])
        for s in range(L):
            r, p = alt_reference_particles(lib, h, s), o.particles(s)
            for k in ("pos", "speed", "age", "feat"):
                np.testing.assert_array_equal(p[k], r[k], err_msg="f%d s%d %s" % (t, s, k))
            if r["compact"]:
                np.testing.assert_array_equal(p["matches"], r["matches"])
    lib.refx_destroy(h)
    o.destroy()


def test_oracle_size_rule():
    lib = oracle()
    assert lib.oracle_sizes_ok(1080, 1920, 4) == 1
    assert lib.oracle_sizes_ok(2160, 3840, 5) == 1
    assert lib.oracle_sizes_ok(97, 131, 3) == 0    # bin parent outside the upper level
    assert lib.oracle_sizes_ok(20, 20, 2) == 0     # second level below 16 px
    assert lib.oracle_sizes_ok(64, 64, 10) == 0


def test_meta_gaussian_taps_match_generator():
    with open(os.path.join(GOLDEN, "meta_gaussian_taps.json")) as f:
        gold = json.load(f)
    for sigma in range(1, 51):
        R, taps = gauss_taps(float(sigma))
        assert R == int(np.ceil(3 * sigma))
        for x_s, v in gold[str(sigma)].items():
            x = int(x_s)
            if abs(x) <= R:
                assert np.float32(v) == taps[x + R], (sigma, x)
    R, taps = gauss_taps(0.5)
    assert R == 2
    for x_s, v in gold["0.5"].items():
        assert np.float32(v) == taps[int(x_s) + R]


def test_gaussian_oracle_properties():
    rng = np.random.default_rng(0)
    img = rng.uniform(0, 255, (37, 53)).astype(np.float32)
    for sigma in (0.5, 1.0, 2.0, 4.0):
        R, taps = gauss_taps(sigma)
        np.testing.assert_array_equal(taps, taps[::-1])
        const = np.full((23, 29), 7.0, np.float32)
        out = gauss_sep(const, sigma)
        np.testing.assert_allclose(out, 7.0 * float(np.sum(taps, dtype=np.float64)) ** 2, rtol=1e-5)
        # separable == 2-D convolution with the outer product (clamped)
        out = gauss_sep(img, sigma)
        H, W = img.shape
        ref = np.zeros((H, W), np.float64)
        for dy in range(-R, R + 1):
            for dx in range(-R, R + 1):
                rr = np.clip(np.arange(H) + dy, 0, H - 1)
                cc = np.clip(np.arange(W) + dx, 0, W - 1)
                ref += taps[dy + R] * taps[dx + R] * img[rr][:, cc]
        np.testing.assert_allclose(out, ref, rtol=1e-5, atol=1e-3)


def test_gaussian_pyramid_oracle():
    rng = np.random.default_rng(1)
    img = rng.uniform(0, 255, (61, 90)).astype(np.float32)
    levels = gauss_pyramid(img, 4)
    assert [l.shape for l in levels] == [(30, 45), (15, 22), (7, 11)]
    np.testing.assert_allclose(levels[0], gauss_sep(img, 1.0)[0::2, 0::2][:30, :45], rtol=1e-6)
    np.testing.assert_allclose(levels[1], gauss_sep(levels[0], 1.0)[0::2, 0::2][:15, :22], rtol=1e-6)


@pytest.mark.parametrize("case", golden_cases())
def test_box_pyramid_matches_reference_levels(case):
    g = load_golden(case)
    rows, cols, L = [int(x) for x in g["meta"][:3]]
    levels = box_pyramid_u8(g["frames"][-1], L)
    for s in range(1, L):
        np.testing.assert_array_equal(levels[s - 1], g["last_s%d_input" % s][6:-6, 6:-6])


def test_oracle_deterministic_and_edge_cases():
    from cuimg_gb300 import synth
    frames = synth.frames(21, 64, 80, 4)
    a = tracker_oracle(64, 80, 2, 20, 1, 1)
    b = tracker_oracle(64, 80, 2, 20, 1, 1)
    for f in frames:
        a.run(f)
        b.run(f)
    assert not diff_snapshots(snapshot(a, 2), snapshot(b, 2), True)
    # flat frames: no corners, no particles, contrast 0 everywhere
    c = tracker_oracle(48, 64, 2, 20, 1, 1)
    c.run(np.full((48, 64), 128, np.uint8))
    assert c.nparticles(0) == 0 and c.contrast(0).max() == 0
    for x in (a, b, c):
        x.destroy()
