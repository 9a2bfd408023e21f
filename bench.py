"""Benchmark: cuimg semi-dense tracker at 1920x1080 on GB300.

Workload (one "step" = one frame of every stream): B independent 1920x1080
uint8 gray video streams from the seeded generator, 4 scales, FAST threshold
20, detector every 10 frames, filtering every frame, advanced by one launch
per stage replayed as a CUDA graph.  Every stream first runs PREROLL frames
untimed (the 120 frames of the 1080p configuration), so the timed frames see
the steady-state particle population, not the ramp-up after the first
detection.  Where a clip is replayed longer than it was generated, frames are
played back and forth (palindromic order), so the motion stays coherent.

Prints one JSON line:
  value      tracked frames/s over all streams (batched), frames resident in HBM
  e2e        same metric through the C ABI from pinned host frames: H2D copy of
             every frame and a D2H read of every stream's particle counts inside
             the timed region
  plain      frames/s of the single-stream (B = 1) path, and the speed-up
  roofline   the dominant kernel's algorithmic bytes / its CUDA-event time
  cpu_baseline  the oracle port (C restatement of the reference CPU tracker)
             on the host cores, bounded sample
`--impl reference` times that CPU implementation alone on the same workload.
`--profile-case NAME` runs one small case of a kernel family for profiler
captures (no timing, no JSON).
"""
import argparse
import concurrent.futures as cf
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ROWS, COLS, NSCALES = 1080, 1920, 4
DET_FREQ, FILT_FREQ, THRESHOLD = 10, 1, 20
PREROLL = 120  # frames run before any timed region
METRIC = "tracked_frames_per_s_1080p"
UNIT = "frames/s"
PER_PARTICLE_BYTES = 84  # state read/write, template read/write, sparse index
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch per
# 1080p stream (4 scales), measured by ncu on launches over four 1080p streams
# at steady state (k_match_tiled with its default 192-thread, slim-margin
# tiles: 81.1 and 88.9 MB for two consecutive frames after 120 untimed ones;
# k_match: 76.8 MB); a launch's traffic grows with the streams it covers.
DRAM_BYTES_PER_STREAM = {"k_match_tiled": 21.3e6, "k_match": 19.2e6}
# The unit that limits the tiled matcher and its utilisation in the same ncu
# capture (l1tex__data_pipe_lsu_wavefronts: shared-memory byte gathers; 61.9%
# and 70.1% of peak for the two frames).
LIMITER = {"k_match_tiled": ("L1 / shared-memory data pipe (byte gathers at the ring offsets)", 0.66)}


def pal(t, n):
    """Frame index of step t when a clip of n frames is played back and forth
    (0, 1, .., n-1, n-2, .., 1, 0, 1, ..)."""
    if n <= 1:
        return 0
    p = 2 * n - 2
    t %= p
    return t if t < n else p - t


def level_pixels(rows=ROWS, cols=COLS, nscales=NSCALES):
    return [(rows >> l) * (cols >> l) for l in range(nscales)]


def frame_bytes_model(live_particles, rows=ROWS, cols=COLS, nscales=NSCALES):
    """Algorithmic HBM bytes of one tracked frame (one stream)."""
    P = level_pixels(rows, cols, nscales)
    Pt = sum(P)
    return P[0] + sum(P[1:]) + 2 * Pt + Pt + 2 * Pt + Pt / 8 + PER_PARTICLE_BYTES * live_particles


def kernel_bytes_model(name, live_particles, nstreams):
    P = level_pixels()
    Pt = sum(P)
    per = {
        "k_blur": 3 * Pt,
        "k_match": 2 * Pt + PER_PARTICLE_BYTES * live_particles,  # s1 + s2 read once, per-particle state
        "k_match_tiled": 2 * Pt + PER_PARTICLE_BYTES * live_particles,
        "k_pyramid": P[0] + sum(P[1:]),
        "k_detect": Pt + Pt / 4 + Pt / 9,
    }.get(name)
    return None if per is None else per * nstreams


def gen_clips(specs, workers=None):
    """specs: (seed, rows, cols, nframes) per clip.  Every clip's generator is
    made once and its frames are generated in threads (frame generation only
    reads the generator's texture, and its C calls release the interpreter
    lock)."""
    import numpy as np

    from cuimg_gb300 import synth
    outs = [np.empty((n, r, c), np.uint8) for (_, r, c, n) in specs]
    with cf.ThreadPoolExecutor(max_workers=workers or min(32, os.cpu_count() or 4)) as ex:
        streams = list(ex.map(lambda sp: synth.Stream(sp[0], sp[1], sp[2]), specs))

        def one(job):
            k, t = job
            outs[k][t] = streams[k].frame(t)

        list(ex.map(one, [(k, t) for k, sp in enumerate(specs) for t in range(sp[3])]))
    for s in streams:
        s.close()
    return outs


def gen_streams(nstreams, nframes, seed0=1000):
    return gen_clips([(seed0 + i, ROWS, COLS, nframes) for i in range(nstreams)])


class ClockSampler:
    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                parts = [p.strip() for p in out.stdout.strip().split(",")]
                if len(parts) == 6:
                    self.samples.append(parts)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_model():
    """Host CPU description (lscpu's model name, or the architecture)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def _cpu_stream_worker(i, preroll, nframes, barrier, out):
    """One stream of the CPU tracker (oracle port, one thread) in its own
    process: `preroll` frames untimed, then `nframes` timed frames, started
    together by a barrier shared by all streams.  Reports the time spent in
    the timed frames' tracker calls and the live particles (age > 0, summed
    over the scales) averaged over those frames, counted between the calls."""
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np

    from cuimg_gb300 import synth
    from oracle_lib import tracker_oracle
    frames = synth.frames(1000 + i, ROWS, COLS, preroll + nframes)
    o = tracker_oracle(ROWS, COLS, NSCALES, THRESHOLD, DET_FREQ, FILT_FREQ)
    for t in range(preroll):
        o.run(frames[t])
    barrier.wait()
    dt, live = 0.0, []
    for t in range(preroll, preroll + nframes):
        t0 = time.perf_counter()
        o.run(frames[t])
        dt += time.perf_counter() - t0
        live.append(sum(int((o.particles(s)["age"] > 0).sum()) for s in range(NSCALES)))
    barrier.wait()
    out.put((i, dt, float(np.mean(live))))
    o.destroy()


def run_cpu_streams(nstreams, steps, preroll):
    """The CPU tracker on `nstreams` 1080p streams at once, one process and
    one core per stream (the streams are independent, as on the GPU); returns
    frames/s over all streams, the time of the timed frames (the slowest
    stream's), the cores used and the live particles (age > 0) per stream,
    averaged over the timed frames and the streams."""
    import multiprocessing as mp

    import numpy as np
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    workers = max(1, min(nstreams, os.cpu_count() or 1))
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(workers)
    out = ctx.Queue()
    procs = [ctx.Process(target=_cpu_stream_worker, args=(i, preroll, steps, barrier, out)) for i in range(workers)]
    for pr in procs:
        pr.start()
    res = [out.get() for _ in procs]
    for pr in procs:
        pr.join()
    wall = max(r[1] for r in res)
    return workers * steps / wall, wall, workers, float(np.mean([r[2] for r in res]))


def _cpu_pyrlk_worker(i, rows, cols, nscales, preroll, nframes, barrier, out):
    """One stream of the oracle's LK tracker (one thread) in its own process:
    `preroll` frames untimed, then `nframes` timed, started together by a
    barrier shared by all streams; reports the time of the timed calls."""
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from cuimg_gb300 import synth
    from oracle_lib import PyrlkLib
    frames = synth.frames(900 + i, rows, cols, preroll + nframes)  # the GPU row's clips (gen_clips, seeds 900 + i)
    o = PyrlkLib("oracle", rows, cols, nscales, THRESHOLD, DET_FREQ, FILT_FREQ)
    for t in range(preroll):
        o.run(frames[t])
    barrier.wait()
    t0 = time.perf_counter()
    for t in range(preroll, preroll + nframes):
        o.run(frames[t])
    dt = time.perf_counter() - t0
    barrier.wait()
    out.put((i, dt))
    o.destroy()


def run_cpu_pyrlk_streams(nstreams, rows, cols, nscales, preroll, steps):
    """The oracle's LK tracker on `nstreams` streams at once, one process
    and core per stream; returns frames/s over all streams, the slowest
    stream's timed seconds and the cores used."""
    import multiprocessing as mp
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    workers = max(1, min(nstreams, os.cpu_count() or 1))
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(workers)
    out = ctx.Queue()
    procs = [ctx.Process(target=_cpu_pyrlk_worker, args=(i, rows, cols, nscales, preroll, steps, barrier, out))
             for i in range(workers)]
    for pr in procs:
        pr.start()
    res = [out.get() for _ in procs]
    for pr in procs:
        pr.join()
    wall = max(r[1] for r in res)
    return workers * steps / wall, wall, workers


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = os.environ.get("BENCH_BACKEND", "nccl")
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def workload_name(nstreams):
    return ("%d streams x 1920x1080 gray, 4 scales, FAST th 20, detector every 10 frames, filter every frame; "
            "%d frames of every stream before timing; one frame of every stream per step" % (nstreams, PREROLL))


def bench_reference(args):
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return
    fps, wall, cores, n = run_cpu_streams(args.streams, args.steps, PREROLL + args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(fps, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * wall / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": workload_name(cores), "streams": cores, "live_particles_per_stream": round(n)},
        "cpu_baseline": {"value": round(fps, 3), "unit": UNIT, "cores": cores, "kind": "port",
                         "per_core": round(fps / cores, 3), "cpu": cpu_model(),
                         "sample": "%d timed frames of each of %d streams after %d untimed frames, one process and "
                                   "core per stream" % (args.steps, cores, PREROLL + args.warmup)},
        "e2e": {"value": round(fps, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_ours(args):
    import numpy as np
    import torch

    from cuimg_gb300 import BatchTracker
    from cuimg_gb300._native import check, cuda_lib

    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = cuda_lib()
    B = args.streams
    W0 = PREROLL + args.warmup  # untimed frames before every timed region
    nfr = W0 + args.steps
    frames = gen_streams(B, nfr, seed0=1000 + rank * B)
    cfg = [dict(rows=ROWS, cols=COLS, nscales=NSCALES, detector_threshold=THRESHOLD, detector_frequency=DET_FREQ,
                filtering_frequency=FILT_FREQ) for _ in range(B)]

    from cuimg_gb300 import autotune
    if args.matcher >= 0:
        tuning = {0: args.matcher}
    else:
        # Tuned at steady state: every setting runs the pre-roll, then is timed.
        tuning = autotune.tune(cfg, [[frames[s][pal(t, nfr)] for s in range(B)] for t in range(PREROLL + 8)],
                               warmup=PREROLL, timed=8, device=local)

    def make(nstreams, graphs=True, groups=0):
        bt = BatchTracker(cfg[:nstreams], device=local, graphs=graphs, groups=groups)
        bt._ensure()
        autotune.apply(bt, tuning)
        return bt

    dev_frames = [torch.from_numpy(f).to(dev) for f in frames]  # resident in HBM
    torch.cuda.synchronize()

    launches = [0]  # kernels launched inside the last timed region
    step_stats = [None]  # per-step milliseconds of the last timed region

    def resident_step(bt, nstreams, t, ptrs, pitches):
        for s in range(nstreams):
            ptrs[s] = dev_frames[s][pal(t, nfr)].data_ptr()
        check(lib.gbt_run(bt._ctx, ptrs, pitches, 1), bt._ctx)

    def preroll(bt, nstreams, n):
        ptrs = (ctypes.c_void_p * nstreams)()
        pitches = (ctypes.c_int64 * nstreams)(*([COLS] * nstreams))
        for t in range(n):
            resident_step(bt, nstreams, t, ptrs, pitches)
        bt.sync()

    def timed_resident(bt, nstreams, steps, sustain_s=0.0):
        """Frames 0 .. W0 - 1 untimed, then `steps` timed frames."""
        stream = torch.cuda.ExternalStream(bt.cuda_stream(), device=dev)
        ptrs = (ctypes.c_void_p * nstreams)()
        pitches = (ctypes.c_int64 * nstreams)(*([COLS] * nstreams))
        preroll(bt, nstreams, W0)
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        k0 = bt.kernel_launches()
        ev[0].record(stream)
        for t in range(steps):
            resident_step(bt, nstreams, W0 + t, ptrs, pitches)
            ev[t + 1].record(stream)
        launches[0] = bt.kernel_launches() - k0
        ev[-1].synchronize()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[-1])
        per = sorted(ev[t].elapsed_time(ev[t + 1]) for t in range(steps))
        step_stats[0] = {"median": round(per[len(per) // 2], 4), "p10": round(per[len(per) // 10], 4),
                         "p90": round(per[min(len(per) - 1, (9 * len(per)) // 10)], 4)}
        # Keep the same step running so the clock sampler sees the GPU under
        # this load for longer than the (short) timed region; not timed.
        t_end, t = time.perf_counter() + sustain_s, W0 + steps
        while time.perf_counter() < t_end:
            for _ in range(32):
                resident_step(bt, nstreams, t, ptrs, pitches)
                t += 1
            bt.sync()
        if pg:
            tt = torch.tensor([ms], device=dev)
            pg.all_reduce(tt, op=pg.ReduceOp.MAX)
            ms = float(tt.item())
        return ms

    def live_per_stream(bt, nstreams):
        return float(np.mean([sum(int((bt._particles(s, l)["age"] > 0).sum()) for l in range(NSCALES))
                              for s in range(nstreams)]))

    # Batched, resident.
    bt = make(B)
    with ClockSampler(local) as clk:
        ms = timed_resident(bt, B, args.steps, sustain_s=1.5)
    timed_launches = launches[0]
    batched_steps = step_stats[0]
    clocks = clk.summary()
    clocks["window"] = "timed region + 1.5 s more of the same step"
    value = B * world * args.steps / (ms / 1000.0)
    ngroups = bt.groups()
    bt.close()

    # The same with device-side trajectories (20 positions per particle).
    btt = make(B)
    btt.enable_trajectories(20)
    ms_t = timed_resident(btt, B, args.steps)
    traj_fps = B * world * args.steps / (ms_t / 1000.0)
    btt.close()

    # Plain single stream, resident.
    bt1 = make(1)
    ms1 = timed_resident(bt1, 1, args.steps)
    plain = args.steps / (ms1 / 1000.0)
    bt1.close()

    # Per-kernel device time (eager, CUDA events on the context stream), over
    # the frames the timed region ran, after the same pre-roll.
    btp = make(B, graphs=False, groups=1)  # one launch per kernel over all streams, serialised
    nprof = max(args.steps, DET_FREQ)
    preroll(btp, B, W0)
    lib.gbt_profile_enable(btp._ctx, 1)
    preroll_ptrs = (ctypes.c_void_p * B)()
    pitches = (ctypes.c_int64 * B)(*([COLS] * B))
    live_hist = []
    for t in range(nprof):
        resident_step(btp, B, W0 + t, preroll_ptrs, pitches)
        btp.sync()
        live_hist.append(live_per_stream(btp, B))  # between frames: the per-kernel events are unaffected
    btp.sync()
    prof = {}
    nameb = ctypes.create_string_buffer(64)
    tot = ctypes.c_double()
    cnt = ctypes.c_int32()
    k = 0
    while True:
        nent = lib.gbt_profile_read(btp._ctx, k, nameb, 64, ctypes.byref(tot), ctypes.byref(cnt))
        if k >= nent:
            break
        prof[nameb.value.decode()] = (tot.value, cnt.value)
        k += 1
    # Live particles (age > 0) per stream, averaged over the profiled frames --
    # the timed region's frames (the count swings about 3x with the detector
    # period, so a single frame's count depends on where it falls).
    live_mean = float(np.mean(live_hist))
    btp.close()
    total_ms = sum(v[0] for v in prof.values())
    shares = {n: round(v[0] / total_ms, 4) for n, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    modeled = [(n, v) for n, v in prof.items() if kernel_bytes_model(n, live_mean, B) is not None]
    dom, (dom_ms, dom_launches) = max(modeled, key=lambda kv: kv[1][0])
    dom_avg_s = dom_ms / dom_launches / 1000.0
    dom_bytes = kernel_bytes_model(dom, live_mean, B)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_source = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"
    achieved = dom_bytes / dom_avg_s / 1e9
    frame_bytes = frame_bytes_model(live_mean) * B
    frame_gbs = frame_bytes * args.steps / (ms / 1000.0) / 1e9

    # End to end through the C ABI: pinned host frames in, every step's
    # per-unit particle counts out, H2D and D2H inside the timed region, on
    # the frames the resident rate is timed on.  "e2e" reads step t's counts
    # while step t + 1 runs (gbt_read_counts_async into pinned memory, an
    # event per step); "blocking" waits for each step's counts before queuing
    # the next.  One context runs the pre-roll from resident frames (untimed)
    # and saves a checkpoint; every repeat restores it (untimed) and times
    # frames W0 .. W0 + steps - 1 from the host.  Host clock, max over ranks;
    # the median of the repeats (the host shares its cores with other work).
    nunits = B * NSCALES
    E2E_REPEATS = 15

    def timed_e2e(host_frames, pitch_bytes, location, pipelined):
        ptrs_ = (ctypes.c_void_p * B)()
        pitch_ = (ctypes.c_int64 * B)(*([pitch_bytes] * B))
        outs = [torch.zeros(nunits, dtype=torch.int32).pin_memory() for _ in range(2)]
        evs = [torch.cuda.Event() for _ in range(2)]
        rates = []
        bt_ = make(B)
        preroll(bt_, B, W0)
        blob = bt_.checkpoint()
        stream = torch.cuda.ExternalStream(bt_.cuda_stream(), device=dev)
        for rep_ in range(E2E_REPEATS):
            bt_.restore(blob)
            bt_.sync()
            torch.cuda.synchronize()
            seen = [0]

            def consume(k):
                evs[k].synchronize()
                seen[0] += int(outs[k].sum())

            def run(t, k):
                for s_ in range(B):
                    ptrs_[s_] = host_frames[s_][t].data_ptr()
                check(lib.gbt_run(bt_._ctx, ptrs_, pitch_, location), bt_._ctx)
                if pipelined:
                    check(lib.gbt_read_counts_async(bt_._ctx, outs[k].data_ptr(), nunits), bt_._ctx)
                    evs[k].record(stream)
                else:
                    check(lib.gbt_read_counts(bt_._ctx, outs[k].data_ptr(), nunits), bt_._ctx)
                    seen[0] += int(outs[k].sum())

            if pg:
                pg.barrier()
            t0 = time.perf_counter()
            for t in range(args.steps):
                run(t, t & 1)
                if pipelined and t > 0:
                    consume((t - 1) & 1)
            if pipelined:
                consume((args.steps - 1) & 1)
            el = time.perf_counter() - t0
            if pg:
                tt = torch.tensor([el], device=dev)
                pg.all_reduce(tt, op=pg.ReduceOp.MAX)
                el = float(tt.item())
            rates.append(B * world * args.steps / el)
        bt_.close()
        return sorted(rates)[len(rates) // 2], rates

    host = [torch.from_numpy(np.ascontiguousarray(frames[s][W0:W0 + args.steps])).pin_memory() for s in range(B)]
    e2e, e2e_all = timed_e2e(host, COLS, 0, True)
    e2e_block, _ = timed_e2e(host, COLS, 0, False)
    del host
    # RGB frames of the same timed frames: 3 bytes per pixel go to the device
    # and the pyramid kernel makes them gray (channel 0, as the reference's
    # sample).
    host_rgb = [torch.from_numpy(np.ascontiguousarray(np.repeat(frames[s][W0:W0 + args.steps, :, :, None], 3,
                                                                axis=3))).pin_memory() for s in range(B)]
    e2e_rgb, _ = timed_e2e(host_rgb, COLS * 3, 2, True)
    del host_rgb

    extras = {} if args.no_extras else measure_extras(args, dev, local, peak)

    cpu = None
    if rank == 0 and not args.no_cpu:
        fps_cpu, wall_cpu, cores_cpu, live_cpu = run_cpu_streams(B, args.cpu_frames, PREROLL)
        cpu = {"value": round(fps_cpu, 3), "unit": UNIT, "cores": cores_cpu, "kind": "port",
               "per_core": round(fps_cpu / cores_cpu, 3), "cpu": cpu_model(),
               "live_particles_per_stream": round(live_cpu),
               "sample": "%d frames of each of %d 1080p streams after %d untimed frames (%.1f s wall), one process "
                         "and core per stream" % (args.cpu_frames, cores_cpu, PREROLL, wall_cpu)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": workload_name(B) + ", CUDA-graph replay",
                       "streams_per_gpu": B, "stream_groups": ngroups, "preroll_frames": PREROLL,
                       "live_particles_per_stream": round(live_mean),
                       "live_particles_note": "age > 0, all scales, mean over the timed frames",
                       "l2": "working set per step > L2 (inputs larger than L2)",
                       "parallelism": "replicas only (independent streams per GPU)"},
            "plain": {"value": round(plain, 2), "unit": UNIT, "streams": 1, "ms_per_frame": round(ms1 / args.steps, 4),
                      "batched_speedup": round(value / world / plain, 2)},
            "mpix_per_s": round(value * ROWS * COLS / 1e6, 1),
            "frame_roofline": {"achieved": round(frame_gbs, 1), "peak": peak, "unit": "GB/s",
                               "frac": round(frame_gbs / peak, 4),
                               "bytes_per_frame_model": round(frame_bytes / B)},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4),
                         "traffic": round(DRAM_BYTES_PER_STREAM[dom] * B) if dom in DRAM_BYTES_PER_STREAM else None,
                         "traffic_source": "ncu dram__bytes_read+write of a 4-stream 1080p launch, scaled by streams",
                         "avg_launch_ms": round(dom_avg_s * 1000, 5), "peak_source": peak_source,
                         "limiter": LIMITER.get(dom, (None, None))[0],
                         "limiter_frac_ncu": LIMITER.get(dom, (None, None))[1]},
            "kernel_time_shares": shares,
            "gpu_launches": timed_launches,
            "step_ms": batched_steps,
            "trajectories": {"history": 20, "frames_per_s": round(traj_fps, 2),
                             "relative_to_value": round(traj_fps / value, 3)},
            "clocks": clocks,
            "e2e_rgb": {"value": round(e2e_rgb, 2), "unit": UNIT, "h2d_bytes_per_step": B * ROWS * COLS * 3,
                        "d2h_bytes_per_step": nunits * 4, "steps": args.steps, "repeats": E2E_REPEATS,
                        "note": "pinned RGB host frames of the timed frames, gray made on the GPU; results read "
                                "one step behind"},
            "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": B * ROWS * COLS,
                    "d2h_bytes_per_step": 4 * nunits, "steps": args.steps, "repeats": E2E_REPEATS,
                    "all": [round(x, 1) for x in e2e_all],
                    "note": "gbt_run from pinned host frames: the frames the resident rate is timed on, after the "
                            "same untimed pre-roll (restored from a checkpoint before every repeat); each step's "
                            "per-unit counts read with gbt_read_counts_async while the next step runs",
                    "blocking": round(e2e_block, 2)},
            "cpu_baseline": cpu,
            "tuning": {autotune.KNOBS[int(k)][0]: v for k, v in tuning.items()},
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


def _events_ms(fn, reps, stream):
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def measure_extras(args, dev, local, peak):
    """The other measured rows: isolated Gaussian (8 B/px), pyramidal LK,
    the LK/pyramid adjoint, batched streams of uneven resolution and the
    large combined 4K workload."""
    import numpy as np
    import torch

    from cuimg_gb300 import BatchTracker, autotune, lk, lkd, synth
    from cuimg_gb300._native import check, cuda_lib
    lib = cuda_lib()
    out = {}
    stream = torch.cuda.current_stream()
    # Isolated separable Gaussian: 32 fp32 1920x1080 images per launch (> L2).
    n_img = 32
    base = torch.from_numpy(synth.Stream(7, ROWS, COLS).frame_f32(0)).to(dev)
    x = base.repeat(n_img, 1, 1).contiguous()
    y = torch.empty_like(x)
    g = {}
    for sigma in (0.5, 1.0, 2.0, 4.0):
        def run():
            check(lib.gbt_gaussian_f32_batch(x.data_ptr(), COLS * 4, ROWS * COLS * 4, y.data_ptr(), COLS * 4,
                                             ROWS * COLS * 4, ROWS, COLS, n_img, ctypes.c_float(sigma),
                                             stream.cuda_stream))
        ms = _events_ms(run, 10, stream)
        gbs = n_img * ROWS * COLS * 8 / (ms / 1000) / 1e9
        g[str(sigma)] = {"ms_per_image": round(ms / n_img, 5), "GB_s": round(gbs, 1), "frac": round(gbs / peak, 4)}
    out["gaussian_1080p_f32"] = {"images_per_launch": n_img, "bytes_per_px": 8, "by_sigma": g}
    # Pyramidal LK: 16 fp32 pairs 640x480, 5 levels, 9x9 full window, 10
    # iterations, 20k points per pair; and the reference constants on uint8.
    P, H, W, n = 16, 480, 640, 20000
    rng = np.random.default_rng(0)
    f0 = np.empty((P, H, W), np.float32)
    f1 = np.empty((P, H, W), np.float32)
    for p in range(P):
        st = synth.Stream(300 + p, H, W)
        f0[p], f1[p] = st.frame_f32(0), st.frame_f32(1)
    pts = np.stack([rng.uniform(30, H - 30, (P, n)), rng.uniform(30, W - 30, (P, n))], -1).astype(np.float32)
    A, Bt, X = torch.from_numpy(f0).to(dev), torch.from_numpy(f1).to(dev), torch.from_numpy(pts).to(dev)
    # Warps per CTA of the LK kernel chosen by the autotuner on each batch.
    prm = autotune.tune_lk(A, Bt, X, 5, lk.params(window=9, npix=81, max_iter=10))
    ms = _events_ms(lambda: lk.track(A, Bt, X, nlevels=5, prm=prm), 3, stream)
    A8 = A.clamp(0, 255).to(torch.uint8)
    B8 = Bt.clamp(0, 255).to(torch.uint8)
    prm8 = autotune.tune_lk(A8, B8, X, 3, lk.params())
    ms8 = _events_ms(lambda: lk.track(A8, B8, X, nlevels=3, prm=prm8), 3, stream)
    out["lk_640x480_x16"] = {"points": P * n,
                             "f32_5lvl_9x9_10it": {"ms": round(ms, 3), "points_per_s": round(P * n / (ms / 1000)),
                                                   "warps_per_block": prm.warps_per_block},
                             "u8_3lvl_11x11_30it_top25": {"ms": round(ms8, 3),
                                                          "points_per_s": round(P * n / (ms8 / 1000)),
                                                          "warps_per_block": prm8.warps_per_block}}
    # Adjoint: forward recording the tape, backward reading it (pyramids
    # recomputed by both); the backward without a tape replays the forward.
    U0 = torch.from_numpy(rng.uniform(-2, 2, (P, n, 2)).astype(np.float32)).to(dev)
    ones = torch.ones((P, n), device=dev)
    tape = [None]

    def fwd():
        tape[0] = lkd.forward(A, Bt, U0, X, 5, 9, 10, tape=True)[2]

    msf = _events_ms(fwd, 3, stream)
    msb = _events_ms(lambda: lkd.backward(A, Bt, U0, X, ones, 5, 9, 10, tape=tape[0]), 3, stream)
    msr = _events_ms(lambda: lkd.backward(A, Bt, U0, X, ones, 5, 9, 10), 3, stream)
    out["lk_adjoint_640x480_x16"] = {"forward_ms": round(msf, 3), "backward_ms": round(msb, 3),
                                     "backward_replay_ms": round(msr, 3),
                                     "tape_bytes": tape[0].numel(),
                                     "pairs_per_s": round(P / ((msf + msb) / 1000), 1)}
    del tape
    del A, Bt, X, A8, B8, U0, x, y
    torch.cuda.empty_cache()
    out["batched_uneven_64"] = measure_uneven(dev, local)
    out["combined_4k"] = measure_combined_4k(dev)
    out["lk_tracker"] = measure_lk_tracker(dev)
    if local == 0 and not args.no_cpu:
        # The same 640x480 streams through the oracle's LK tracker (a
        # restatement of pyrlk_cpu, bit-exact with it), one process and core
        # per stream: 40 frames untimed, then one detector period timed.
        fps, wall, cores = run_cpu_pyrlk_streams(16, 480, 640, 3, 40, DET_FREQ)
        out["lk_tracker"]["640x480_x16"]["cpu_baseline"] = {
            "frames_per_s": round(fps, 2), "cores": cores, "kind": "port", "cpu": cpu_model(),
            "sample": "%d frames of each of %d streams after 40 untimed frames (%.1f s wall), one process and core "
                      "per stream" % (DET_FREQ, cores, wall)}
    return out


def measure_lk_tracker(dev, cases=((480, 640, 3, 16), (1080, 1920, 4, 4)), pre=40, timed=20):
    """The pyramidal LK tracker strategy (gbt_config.matcher = GBT_MATCHER_LK):
    B streams of one size, `pre` frames untimed, then `timed` frames timed
    with CUDA events on the context stream; frames resident in HBM."""
    import numpy as np
    import torch

    from cuimg_gb300 import BatchTracker
    from cuimg_gb300._native import check, cuda_lib
    lib = cuda_lib()
    res = {}
    for rows, cols, L, B in cases:
        vids = gen_clips([(900 + i, rows, cols, pre + timed) for i in range(B)])
        dv = [torch.from_numpy(v).to(dev) for v in vids]
        bt = BatchTracker([dict(rows=rows, cols=cols, nscales=L, matcher=1, detector_threshold=THRESHOLD,
                                detector_frequency=DET_FREQ, filtering_frequency=FILT_FREQ)] * B,
                          device=dev.index or 0)
        bt._ensure()
        cst = torch.cuda.ExternalStream(bt.cuda_stream(), device=dev)
        ptrs = (ctypes.c_void_p * B)()
        pit = (ctypes.c_int64 * B)(*([cols] * B))

        def step(t):
            for s in range(B):
                ptrs[s] = dv[s][t].data_ptr()
            check(lib.gbt_run(bt._ctx, ptrs, pit, 1), bt._ctx)

        for t in range(pre):
            step(t)
        bt.sync()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(timed + 1)]
        ev[0].record(cst)
        for t in range(timed):
            step(pre + t)
            ev[t + 1].record(cst)
        ev[-1].synchronize()
        ms = ev[0].elapsed_time(ev[-1]) / timed
        live = float(np.mean([sum(int((bt.particles_f(s, l)["age"] > 0).sum()) for l in range(L)) for s in range(B)]))
        bt.close()
        del dv
        res["%dx%d_x%d" % (cols, rows, B)] = {
            "streams": B, "scales": L, "ms_per_step": round(ms, 3), "frames_per_s": round(B / (ms / 1000), 1),
            "mpix_per_s": round(B * rows * cols / (ms / 1000) / 1e6, 1), "live_particles_per_stream_end": round(live)}
    res["note"] = ("pyrlk_cpu on the GPU: 11x11 window, 25 strongest gradients, 30 iterations, detector every 10 "
                   "frames; %d frames untimed, %d timed (CUDA events)" % (pre, timed))
    return res


def measure_uneven(dev, local, nstreams=64, nf=60, timed=20):
    """64 streams drawn from five resolutions, 60-frame clips: frames 0..39
    untimed, 20 timed steps on frames 40..59 (one launch per stage over every
    stream, graph replay, launch shapes autotuned on the same streams)."""
    import numpy as np
    import torch

    from cuimg_gb300 import BatchTracker, autotune
    from cuimg_gb300._native import check, cuda_lib
    lib = cuda_lib()
    shapes = [(240, 320, 3), (480, 640, 3), (720, 1280, 4), (1080, 1920, 4), (2160, 3840, 5)]
    rs = np.random.default_rng(4)
    picks = [shapes[i] for i in rs.integers(0, 5, nstreams)]
    cfgs = [dict(rows=r, cols=c, nscales=L, detector_threshold=THRESHOLD, detector_frequency=DET_FREQ,
                 filtering_frequency=FILT_FREQ) for r, c, L in picks]
    vids = gen_clips([(5000 + i, r, c, nf) for i, (r, c, L) in enumerate(picks)])
    dvid = [torch.from_numpy(v).to(dev) for v in vids]
    pre = nf - timed
    tuning = autotune.tune(cfgs, [[vids[s][t] for s in range(nstreams)] for t in range(pre + 6)], warmup=pre,
                           timed=6, device=local)
    bt = BatchTracker(cfgs, device=local, graphs=True)
    bt._ensure()
    autotune.apply(bt, tuning)
    ptrs = (ctypes.c_void_p * nstreams)()
    pit = (ctypes.c_int64 * nstreams)(*[c for r, c, L in picks])
    cst = torch.cuda.ExternalStream(bt.cuda_stream(), device=dev)

    def step(t):
        for s in range(nstreams):
            ptrs[s] = dvid[s][t].data_ptr()
        check(lib.gbt_run(bt._ctx, ptrs, pit, 1), bt._ctx)

    for t in range(pre):
        step(t)
    bt.sync()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(timed + 1)]
    ev[0].record(cst)
    for t in range(timed):
        step(pre + t)
        ev[t + 1].record(cst)
    ev[-1].synchronize()
    ms = ev[0].elapsed_time(ev[-1]) / timed
    px = sum(r * c for r, c, L in picks)
    live = sum(int((bt._particles(s, l)["age"] > 0).sum()) for s in range(nstreams) for l in range(picks[s][2]))
    bt.close()
    return {"streams": nstreams, "ms_per_step": round(ms, 3), "frames_per_s": round(nstreams / (ms / 1000), 1),
            "mpix_per_s": round(px / (ms / 1000) / 1e6, 1), "live_particles": live,
            "resolutions": {"%dx%d" % (c, r): sum(1 for p in picks if p[:2] == (r, c)) for r, c, L in shapes},
            "tuning": {autotune.KNOBS[int(k)][0]: v for k, v in tuning.items()},
            "note": "%d-frame clips: frames 0..%d untimed, %d timed steps (CUDA events)" % (nf, pre - 1, timed)}


def measure_combined_4k(dev, nf=300, every=10):
    """One 3840x2160 stream (5 scales) tracked for 300 frames, with the LK
    residual and its adjoint through the Gaussian pyramid (fp32, 5 levels,
    9x9, 10 steps; pyramids recomputed in the backward pass) on every 10th
    frame pair, over the level-0 particles alive at that frame.  Tracker
    frames and adjoint pairs timed with CUDA events."""
    import numpy as np
    import torch

    from cuimg_gb300 import BatchTracker, lkd
    from cuimg_gb300._native import check, cuda_lib
    lib = cuda_lib()
    H4, W4 = 2160, 3840
    v4 = gen_clips([(7000, H4, W4, nf)])[0]
    d4 = torch.from_numpy(v4).to(dev)
    del v4
    bt4 = BatchTracker([dict(rows=H4, cols=W4, nscales=5, detector_threshold=THRESHOLD,
                             detector_frequency=DET_FREQ, filtering_frequency=FILT_FREQ)], device=dev.index or 0,
                       graphs=True)
    bt4._ensure()
    cst = torch.cuda.ExternalStream(bt4.cuda_stream(), device=dev)
    ts = torch.cuda.current_stream()
    p4 = (ctypes.c_void_p * 1)()
    pit4 = (ctypes.c_int64 * 1)(W4)
    t_trk, t_adj, npairs, npts = 0.0, 0.0, 0, []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for t in range(nf):
        p4[0] = d4[t].data_ptr()
        e0.record(cst)
        check(lib.gbt_run(bt4._ctx, p4, pit4, 1), bt4._ctx)
        e1.record(cst)
        e1.synchronize()
        t_trk += e0.elapsed_time(e1)
        if t > 0 and t % every == 0:
            parts = bt4._particles(0, 0)  # the points: level-0 particles alive now (read outside the timing)
            pts = torch.from_numpy(parts["pos"][parts["age"] > 0].astype(np.float32)).to(dev)[None]
            u0 = torch.zeros_like(pts)
            ones = torch.ones(pts.shape[:2], device=dev)
            a, b = d4[t - 1].float()[None], d4[t].float()[None]
            torch.cuda.synchronize()
            e0.record(ts)
            tp = lkd.forward(a, b, u0, pts, 5, 9, 10, tape=True)[2]
            lkd.backward(a, b, u0, pts, ones, 5, 9, 10, tape=tp)
            e1.record(ts)
            e1.synchronize()
            t_adj += e0.elapsed_time(e1)
            npairs += 1
            npts.append(int(pts.shape[1]))
            del tp, a, b
    live = sum(int((bt4._particles(0, l)["age"] > 0).sum()) for l in range(5))
    bt4.close()
    del d4
    torch.cuda.empty_cache()
    return {"frames": nf, "tracker_ms_per_frame": round(t_trk / nf, 4), "adjoint_pairs": npairs,
            "adjoint_ms_per_pair": round(t_adj / max(1, npairs), 3), "points_per_pair_mean": round(float(np.mean(npts))),
            "live_particles_final": live, "frames_per_s": round(nf / ((t_trk + t_adj) / 1000), 1),
            "note": "CUDA events: each tracked frame on the context stream, each adjoint pair (forward with tape + "
                    "backward) on the torch stream; particle read-back between them untimed"}


# --- profiler capture cases -------------------------------------------------
# Each runs its kernels a few times on inputs larger than L2 but a few GB at
# most on the device, so a capture of one or two launches ends quickly.

def _case_gaussian(reps=3, sigma=4.0):
    """8 fp32 1920x1080 images, sigma 4 (or `sigma`)."""
    import torch

    from cuimg_gb300 import synth
    from cuimg_gb300._native import check, cuda_lib
    lib = cuda_lib()
    n = 8
    x = torch.from_numpy(synth.Stream(7, ROWS, COLS).frame_f32(0)).cuda().repeat(n, 1, 1).contiguous()
    y = torch.empty_like(x)
    for _ in range(reps):
        check(lib.gbt_gaussian_f32_batch(x.data_ptr(), COLS * 4, ROWS * COLS * 4, y.data_ptr(), COLS * 4,
                                         ROWS * COLS * 4, ROWS, COLS, n, ctypes.c_float(sigma), None))
    torch.cuda.synchronize()


def _lk_batch(P=4, n=20000):
    import numpy as np
    import torch

    from cuimg_gb300 import synth
    H, W = 480, 640
    rng = np.random.default_rng(0)
    f0 = np.empty((P, H, W), np.float32)
    f1 = np.empty((P, H, W), np.float32)
    for p in range(P):
        s = synth.Stream(300 + p, H, W)
        f0[p], f1[p] = s.frame_f32(0), s.frame_f32(1)
    pts = np.stack([rng.uniform(30, H - 30, (P, n)), rng.uniform(30, W - 30, (P, n))], -1).astype(np.float32)
    u0 = rng.uniform(-2, 2, (P, n, 2)).astype(np.float32)
    t = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    return t(f0), t(f1), t(pts), t(u0)


def _case_lk(reps=3):
    """4 fp32 640x480 pairs, 5 levels, 9x9, 10 steps, 20k points each."""
    import torch

    from cuimg_gb300 import lk
    A, B, X, _ = _lk_batch()
    prm = lk.params(window=9, npix=81, max_iter=10)
    for _ in range(reps):
        lk.track(A, B, X, nlevels=5, prm=prm)
    torch.cuda.synchronize()


def _case_adjoint(reps=2):
    """LK residual forward (tape) + backward on the same batch."""
    import torch

    from cuimg_gb300 import lkd
    A, B, X, U = _lk_batch()
    ones = torch.ones(X.shape[:2], device="cuda")
    for _ in range(reps):
        tape = lkd.forward(A, B, U, X, 5, 9, 10, tape=True)[2]
        lkd.backward(A, B, U, X, ones, 5, 9, 10, tape=tape)
    torch.cuda.synchronize()


def _case_tracker(nstreams, frames, det_freq, blur_rows=None):
    from cuimg_gb300 import BatchTracker
    cfg = [dict(rows=ROWS, cols=COLS, nscales=NSCALES, detector_threshold=THRESHOLD, detector_frequency=det_freq)]
    vids = gen_streams(nstreams, frames)
    bt = BatchTracker(cfg * nstreams, graphs=False, groups=1)  # one launch per stage over every stream
    if blur_rows:
        bt.set_tuning(1, blur_rows)
    for t in range(frames):
        bt.run([v[t] for v in vids])
    bt.sync()
    bt.close()


def _case_steady(nstreams, det_freq, frames, lk=False, rows=ROWS, cols=COLS, nscales=NSCALES, preroll=PREROLL):
    """`nstreams` streams in one group, `preroll` frames untimed, then `frames`
    frames between cudaProfilerStart / Stop: with ncu --profile-from-start off
    only the steady-state frames are captured."""
    import torch

    from cuimg_gb300 import BatchTracker
    cfg = [dict(rows=rows, cols=cols, nscales=nscales, detector_threshold=THRESHOLD, detector_frequency=det_freq,
                matcher=1 if lk else 0)]
    vids = gen_clips([(1000 + i, rows, cols, preroll + frames) for i in range(nstreams)])
    bt = BatchTracker(cfg * nstreams, graphs=False, groups=1)  # one launch per stage over every stream
    if not lk:
        bt.set_tuning(1, 32)
    for t in range(preroll):
        bt.run([v[t] for v in vids])
    bt.sync()
    torch.cuda.profiler.start()
    for t in range(preroll, preroll + frames):
        bt.run([v[t] for v in vids])
    bt.sync()
    torch.cuda.profiler.stop()
    bt.close()


PROFILE_CASES = {
    "gaussian": _case_gaussian,
    "gaussian_s2": lambda: _case_gaussian(sigma=2.0),
    "lk": _case_lk,
    "adjoint": _case_adjoint,
    "tracker": lambda: _case_tracker(4, 6, 10),        # 4 streams of 1920x1080, 6 frames
    "tracker_det": lambda: _case_tracker(4, 8, 3),     # the same with the detector every third frame
    "tracker16": lambda: _case_tracker(16, 4, 10, 32),  # 16 streams in one group, 32-row blur strips
    # steady state (120 frames before the captured ones):
    "tracker16_steady": lambda: _case_steady(16, DET_FREQ, 10),  # the benchmark's streams, one detector period
    "tracker4_steady": lambda: _case_steady(4, 3, 3),             # 4 streams, detector every third frame
    "lk_tracker_steady": lambda: _case_steady(2, DET_FREQ, 2, lk=True, preroll=30),  # LK strategy, 2 x 1080p
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--streams", type=int, default=16)
    ap.add_argument("--cpu-frames", type=int, default=DET_FREQ,
                    help="timed frames per stream of the CPU baseline (default: one detector period)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--matcher", type=int, default=-1, help="matcher variant (default: autotuned)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the Gaussian / LK / adjoint / uneven-batch / 4K lines")
    ap.add_argument("--profile-case", nargs="+", choices=sorted(PROFILE_CASES),
                    help="run these small cases for a profiler capture and exit")
    args = ap.parse_args()
    if args.profile_case:
        for name in args.profile_case:
            PROFILE_CASES[name]()
        print("ok")
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
