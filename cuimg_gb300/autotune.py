"""Autotuner for the tracker's launch shapes.

The tracker's results do not depend on its tuning knobs (GBT_TUNE_* in
include/cuimg_gb300.h); only speed does, and the best setting depends on the
GPU and on the streams' resolutions.  ``tune`` times every setting of each
knob on the caller's own workload -- a throwaway one-group context per
setting, a few warm-up frames, then per-kernel CUDA-event time of the knob's
kernel over the timed frames -- keeps the fastest, and caches the choice in a
JSON file keyed by GPU name and stream geometry.  ``apply`` puts the cached
choice on a tracker.
"""
import ctypes
import json
import os

from ._native import check, cuda_lib

KNOBS = {
    # knob id: (name, settings, kernel names whose time decides)
    0: ("matcher", (0, 1, 2, 3), ("k_match", "k_match_warp", "k_match_tiled", "k_mt_list", "k_match_overflow")),
    1: ("blur_rows", (16, 32, 64), ("k_blur",)),
    2: ("match_tile", (0, 1, 2, 3, 4, 5, 6, 7), ("k_match_tiled",)),
}
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _load_cache(cache_path):
    if os.path.exists(cache_path):
        try:
            with open(cache_path) as f:
                return json.load(f)
        except (OSError, ValueError):
            pass
    return {}


def _store(cache_path, key, value):
    """Adds one entry to the cache file, written to a temporary file first and
    renamed over the old one, so that processes tuning at the same time (one per
    GPU) never leave a partial file."""
    os.makedirs(os.path.dirname(cache_path), exist_ok=True)
    cache = _load_cache(cache_path)
    cache[key] = value
    tmp = "%s.%d.tmp" % (cache_path, os.getpid())
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, cache_path)


def _gpu_name(device):
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return "cuda:%d" % device


def signature(configs, device=0):
    geo = sorted("%dx%dx%d" % (c["rows"], c["cols"], c["nscales"]) for c in configs)
    return "%s|%s" % (_gpu_name(device), ",".join(geo))


def _kernel_ms(bt, names):
    lib = cuda_lib()
    buf = ctypes.create_string_buffer(64)
    tot, cnt = ctypes.c_double(), ctypes.c_int32()
    ms, k = 0.0, 0
    while True:
        n = lib.gbt_profile_read(bt._ctx, k, buf, 64, ctypes.byref(tot), ctypes.byref(cnt))
        if k >= n:
            break
        if buf.value.decode() in names:
            ms += tot.value
        k += 1
    return ms


def tune(configs, frames, warmup=3, timed=8, device=0, cache_path=DEFAULT_CACHE, force=False):
    """frames[t][s]: frame t of stream s (numpy uint8).  Returns {knob: value}."""
    from .tracker import BatchTracker
    key = signature(configs, device)
    cache = _load_cache(cache_path)
    if key in cache and not force:
        return {int(k): v for k, v in cache[key].items()}
    lib = cuda_lib()
    choice = {}
    for knob, (name, settings, kernels) in KNOBS.items():
        best = None
        for value in settings:
            # One stream group: each launch then covers every stream, so a
            # setting is charged the work it does for the whole frame.  (Split
            # into groups, per-kernel timing would time small launches one
            # after another, which favours the setting with the most CTAs --
            # e.g. 16-row blur strips -- over the one that costs least when the
            # groups run together.)
            bt = BatchTracker(configs, device=device, graphs=False, groups=1)
            bt._ensure()
            for k2, v2 in choice.items():
                bt.set_tuning(k2, v2)
            bt.set_tuning(knob, value)
            for t in range(warmup):
                bt.run(frames[t % len(frames)])
            check(lib.gbt_profile_enable(bt._ctx, 1), bt._ctx)
            for t in range(timed):
                bt.run(frames[(warmup + t) % len(frames)])
            bt.sync()
            ms = _kernel_ms(bt, kernels)
            bt.close()
            if best is None or ms < best[0]:
                best = (ms, value)
        choice[knob] = best[1]
    _store(cache_path, key, {str(k): v for k, v in choice.items()})
    return choice


def apply(bt, choice):
    for knob, value in choice.items():
        bt.set_tuning(int(knob), int(value))
    return bt


LK_WARPS = (2, 4, 8)


def tune_lk(prev, cur, points, nlevels, prm, reps=3, cache_path=DEFAULT_CACHE, force=False):
    """Warps per CTA of the LK tracking kernel for this workload: each setting
    timed with CUDA events over `reps` calls of lk.track on the caller's own
    batch, the fastest cached by GPU name, batch geometry and LK parameters.
    Returns params equal to `prm` with warps_per_block set."""
    import torch

    from . import lk
    dev = prev.device.index or 0
    key = "lk|%s|%s|%s|%d|%d|%d|%d|%d" % (_gpu_name(dev), "x".join(map(str, prev.shape)), str(prev.dtype),
                                         points.shape[-2], nlevels, prm.window, prm.npix, prm.max_iter)
    best = _load_cache(cache_path).get(key) if not force else None
    if best is None:
        times = {}
        for w in LK_WARPS:
            p = lk.params(prm.window, prm.npix, prm.max_iter, prm.eps, prm.max_err, w)
            lk.track(prev, cur, points, nlevels=nlevels, prm=p)  # warm-up
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                lk.track(prev, cur, points, nlevels=nlevels, prm=p)
            e1.record()
            e1.synchronize()
            times[w] = e0.elapsed_time(e1)
        best = min(times, key=times.get)
        _store(cache_path, key, best)
    return lk.params(prm.window, prm.npix, prm.max_iter, prm.eps, prm.max_err, int(best))
