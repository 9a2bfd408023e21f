"""Host-side mirror of cuimg's tracker API, backed by the GB300 C ABI.

    tr = Tracker((rows, cols), nscales)                 # tracker<F>(obox2d, nscales)
    tr.strategy().set_detector_frequency(10)            # generic_strategy setters
    tr.scale(s).strategy().detector().set_n(9).set_fast_threshold(20)
    tr.run(frame)                                       # tracker<F>::run(const I&)
    ps = tr.scale(s).pset()                             # particle_container view
    ps.dense_particles(), ps.features(), ps.matches(), ps.sync_attributes(v, new)

(cuimg/tracking2/tracker.h:10-47, tracking_strategies.h:28-107,
particle_container.h:62-183.)  Setters work at any time, per scale as in the
reference: the frequencies and k set on scale s apply to s and every coarser
scale (tracking_strategies.hpp:56-82), with_merge and the detector's n and
threshold to scale s only.  ``BatchTracker`` advances many independent streams
of any resolution with one launch per stage.
"""
import ctypes

import numpy as np

from ._native import GbtError, check, cuda_lib, gbt_config

GBT_FRAMES_HOST, GBT_FRAMES_DEVICE, GBT_FRAMES_HOST_RGB, GBT_FRAMES_DEVICE_RGB = 0, 1, 2, 3
GBT_RGB_CHANNEL0, GBT_RGB_BT601 = 0, 1
GBT_MATCHER_BC2S, GBT_MATCHER_LK = 0, 1
STAGES = dict(input=0, s1=1, s2=2, contrast=3, saliency=4, mask=5, sparse=6)


def sizes_ok(rows, cols, nscales):
    return bool(cuda_lib().gbt_sizes_ok(rows, cols, nscales))


# gbt_set_param keys, and whether a setter on scale s also sets the coarser
# scales (as generic_strategy's setters forward to upper_).
PARAMS = dict(detector_threshold=(0, False), detector_n=(1, False), detector_frequency=(2, True),
              filtering_frequency=(3, True), k=(4, True), with_merge=(5, False), detector_grad_th=(6, False))


class _Detector:
    def __init__(self, owner):
        self._o = owner

    def set_n(self, n):
        self._o._set("detector_n", int(n))
        return self

    def set_fast_threshold(self, th):
        if float(th) != int(th) or th < 0:
            raise ValueError("the FAST threshold must be a whole number >= 0")
        self._o._set("detector_threshold", int(th))
        return self

    def saliency(self):
        return self._o._stage("saliency")


class _Strategy:
    def __init__(self, owner):
        self._o = owner
        self._det = _Detector(owner)

    def set_detector_frequency(self, n):
        self._o._set("detector_frequency", int(n))
        return self

    def set_filtering_frequency(self, n):
        self._o._set("filtering_frequency", int(n))
        return self

    def set_k(self, k):
        self._o._set("k", int(k))
        return self

    def set_with_merge(self, b):
        self._o._set("with_merge", 1 if b else 0)
        return self

    def detector(self):
        return self._det


class ParticleSet:
    """particle_container view of one (stream, scale) after the last frame."""

    def __init__(self, tracker, stream, scale):
        self._t, self._s, self._l = tracker, stream, scale
        self._cache = None

    def _fetch(self):
        if self._cache is None:
            self._cache = self._t._particles(self._s, self._l)
        return self._cache

    def size(self):
        return len(self._fetch()["age"])

    def dense_particles(self):
        """Structured array with fields speed (2 float32), pos (2 int16), age."""
        d = self._fetch()
        out = np.zeros(len(d["age"]), dtype=[("speed", np.float32, 2), ("pos", np.int16, 2), ("age", np.uint16)])
        out["speed"], out["pos"], out["age"] = d["speed"], d["pos"], d["age"]
        return out

    def features(self):
        return self._fetch()["feat"]

    def matches(self):
        return self._fetch()["matches"]

    def compact_has_run(self):
        return self._fetch()["compact"]

    def sync_attributes(self, v, new_value=None, die_fun=None):
        """particle_container::sync_attributes (particle_container.hpp:511-545)."""
        n = self.size()
        if self.compact_has_run():
            m = self.matches()
            tmp = [new_value] * n
            for i, ni in enumerate(m):
                if ni >= 0:
                    if i < len(v):
                        tmp[ni] = v[i]
                elif die_fun is not None and i < len(v):
                    die_fun(v[i])
            v[:] = tmp
        else:
            v.extend([new_value] * (n - len(v)))
        return v


class _Scale:
    def __init__(self, tracker, stream, scale):
        self._t, self._s, self._l = tracker, stream, scale

    def pset(self):
        return ParticleSet(self._t, self._s, self._l)

    def strategy(self):
        return _Strategy(_ScaleSetter(self._t, self._s, self._l))

    def input(self, border=0):
        return self._t.stage(self._s, self._l, "input", border)

    def domain(self):
        return self._t.dims(self._s, self._l)


class _ScaleSetter:
    def __init__(self, t, s, l):
        self.t, self.s, self.l = t, s, l

    def _set(self, key, value):
        self.t._set_param(self.s, 0 if self.l is None else self.l, key, value)

    def _stage(self, name):
        return self.t.stage(self.s, self.l, name)


class BatchTracker:
    """Many independent streams advanced one frame per run() call."""

    def __init__(self, configs, device=0, graphs=False, groups=0):
        """groups: stream groups (gbt_create_ex; 0 = the library's default)."""
        self._lib = cuda_lib()
        self._cfgs = []
        for c in configs:
            cfg = gbt_config()
            self._lib.gbt_config_default(ctypes.byref(cfg), int(c["rows"]), int(c["cols"]), int(c["nscales"]))
            for k, v in c.items():
                if k not in ("rows", "cols", "nscales"):
                    setattr(cfg, k, int(v))
            self._cfgs.append(cfg)
        self._device = device
        self._graphs = graphs
        self._groups = groups
        self._ctx = None
        self._pending = []  # per-scale settings made before the context exists
        self.nstreams = len(self._cfgs)

    # -- settings (the reference's setters, at any time) --
    def _set_param(self, stream, scale, key, value):
        """Sets `key` on `scale` (and the coarser scales for the frequencies
        and k) of `stream` (every stream when None), through gbt_set_param
        once the context runs."""
        pid, upward = PARAMS[key]
        if key == "k" and self._cfgs[0].matcher == GBT_MATCHER_LK:
            upward = False  # pyrlk_cpu::set_k sets its own scale only (pyrlk_tracker.h:44)
        streams = range(self.nstreams) if stream is None else [stream]
        for s in streams:
            L = self._cfgs[s].nscales
            scales = range(scale, L) if upward else [scale]
            if self._ctx is None:
                if len(scales) == L:  # every scale: the stream's configuration, replacing earlier per-scale values
                    setattr(self._cfgs[s], key, value)
                    self._pending = [e for e in self._pending if not (e[0] == s and e[2] == pid)]
                else:
                    self._pending.append((s, list(scales), pid, value))
            else:
                for l in scales:
                    check(self._lib.gbt_set_param(self._ctx, s, l, pid, value), self._ctx)

    def get_param(self, key, stream=0, scale=0):
        v = ctypes.c_int32()
        check(self._lib.gbt_get_param(self._ensure(), stream, scale, PARAMS[key][0], ctypes.byref(v)), self._ctx)
        return v.value

    def _ensure(self):
        if self._ctx is None:
            arr = (gbt_config * self.nstreams)(*self._cfgs)
            ctx = ctypes.c_void_p()
            code = self._lib.gbt_create_ex(arr, self.nstreams, self._device, self._groups, ctypes.byref(ctx))
            if code:
                raise GbtError(code, "gbt_create failed (sizes ok: %s)" % [
                    sizes_ok(c.rows, c.cols, c.nscales) for c in self._cfgs])
            self._ctx = ctx
            for s, scales, pid, value in self._pending:
                for l in scales:
                    check(self._lib.gbt_set_param(ctx, s, l, pid, value), ctx)
            self._pending = []
            if self._graphs:
                check(self._lib.gbt_use_graphs(self._ctx, 1), self._ctx)
        return self._ctx

    def close(self):
        if self._ctx is not None:
            self._lib.gbt_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dims(self, stream, scale):
        c = self._cfgs[stream]
        return (c.rows >> scale, c.cols >> scale)

    def run(self, frames, location=None):
        """One frame per stream: numpy uint8 arrays (gray, or HxWx3 RGB whose
        channel 0 is tracked), or device pointers with location=DEVICE."""
        ctx = self._ensure()
        n = self.nstreams
        ptrs = (ctypes.c_void_p * n)()
        pitches = (ctypes.c_int64 * n)()
        keep = []
        loc = location
        for s, f in enumerate(frames):
            if isinstance(f, np.ndarray):
                f = np.ascontiguousarray(f, dtype=np.uint8)
                keep.append(f)
                ptrs[s] = f.ctypes.data
                pitches[s] = f.strides[0]
                if loc is None:
                    loc = GBT_FRAMES_HOST_RGB if f.ndim == 3 else GBT_FRAMES_HOST
            else:
                ptr, pitch = f
                ptrs[s] = ptr
                pitches[s] = pitch
        check(self._lib.gbt_run(ctx, ptrs, pitches, GBT_FRAMES_HOST if loc is None else loc), ctx)
        return self

    def run_resident(self):
        check(self._lib.gbt_run_resident(self._ensure()), self._ctx)

    def sync(self):
        check(self._lib.gbt_sync(self._ensure()), self._ctx)

    def input_slot(self, stream):
        p, pitch = ctypes.c_void_p(), ctypes.c_int64()
        check(self._lib.gbt_input_slot(self._ensure(), stream, ctypes.byref(p), ctypes.byref(pitch)), self._ctx)
        return p.value, pitch.value

    def cuda_stream(self):
        p = ctypes.c_void_p()
        check(self._lib.gbt_stream(self._ensure(), ctypes.byref(p)), self._ctx)
        return p.value

    def set_tuning(self, knob, value):
        check(self._lib.gbt_set_tuning(self._ensure(), knob, value), self._ctx)

    def get_tuning(self, knob):
        v = ctypes.c_int32()
        check(self._lib.gbt_get_tuning(self._ensure(), knob, ctypes.byref(v)), self._ctx)
        return v.value

    def tile_fallbacks(self):
        """Particles the slim-margin tiled matcher matched again from global
        memory, over the frames run so far (test and diagnostic hook)."""
        v = ctypes.c_int64()
        check(self._lib.gbt_test_tile_fallbacks(self._ensure(), ctypes.byref(v)), self._ctx)
        return v.value

    def kernels_per_frame(self):
        n = ctypes.c_int32()
        check(self._lib.gbt_kernels_per_frame(self._ensure(), ctypes.byref(n)), self._ctx)
        return n.value

    def groups(self):
        """Stream groups of the context (each runs on its own CUDA streams)."""
        n = ctypes.c_int32()
        check(self._lib.gbt_groups(self._ensure(), ctypes.byref(n)), self._ctx)
        return n.value

    def kernel_launches(self):
        """Kernels launched by this tracker so far (graph replays included)."""
        n = ctypes.c_int64()
        check(self._lib.gbt_kernel_launches(self._ensure(), ctypes.byref(n)), self._ctx)
        return n.value

    def nparticles(self, stream=0, scale=None):
        if scale is None:
            return sum(self.nparticles(stream, s) for s in range(self._cfgs[stream].nscales))
        n = ctypes.c_int32()
        check(self._lib.gbt_nparticles(self._ensure(), stream, scale, ctypes.byref(n)), self._ctx)
        return n.value

    def is_lk(self):
        """True for a context of the LK matcher (gbt_config.matcher == GBT_MATCHER_LK)."""
        return self._cfgs[0].matcher == GBT_MATCHER_LK

    def particles_f(self, stream, scale):
        """Particle state with float positions and speeds (gbt_get_particles_f)."""
        ctx = self._ensure()
        n = self.nparticles(stream, scale)
        pos = np.zeros((n, 2), np.float32)
        speed = np.zeros((n, 2), np.float32)
        age = np.zeros(n, np.uint16)
        nm, comp = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.gbt_get_particles_f(ctx, stream, scale, None, None, None, None, ctypes.byref(nm),
                                            ctypes.byref(comp)), ctx)
        matches = np.zeros(max(nm.value, 1), np.int32)
        check(self._lib.gbt_get_particles_f(ctx, stream, scale, pos.ctypes.data, speed.ctypes.data, age.ctypes.data,
                                            matches.ctypes.data, ctypes.byref(nm), ctypes.byref(comp)), ctx)
        return dict(pos=pos, speed=speed, age=age, matches=matches[: nm.value], compact=bool(comp.value))

    def _particles(self, stream, scale):
        if self.is_lk():
            return self.particles_f(stream, scale)
        ctx = self._ensure()
        n = self.nparticles(stream, scale)
        speed = np.zeros((n, 2), np.float32)
        pos = np.zeros((n, 2), np.int16)
        age = np.zeros(n, np.uint16)
        feat = np.zeros((n, 16), np.uint8)
        nm, comp = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.gbt_get_particles(ctx, stream, scale, None, None, None, None, None, ctypes.byref(nm),
                                          ctypes.byref(comp)), ctx)
        matches = np.zeros(max(nm.value, 1), np.int32)
        check(self._lib.gbt_get_particles(ctx, stream, scale, speed.ctypes.data, pos.ctypes.data, age.ctypes.data,
                                          feat.ctypes.data, matches.ctypes.data, ctypes.byref(nm),
                                          ctypes.byref(comp)), ctx)
        return dict(speed=speed, pos=pos, age=age, feat=feat, matches=matches[: nm.value], compact=bool(comp.value))

    def checkpoint(self):
        """The carried state of every stream as bytes (gbt_checkpoint_save)."""
        ctx = self._ensure()
        n = ctypes.c_size_t()
        check(self._lib.gbt_checkpoint_size(ctx, ctypes.byref(n)), ctx)
        buf = ctypes.create_string_buffer(n.value)
        w = ctypes.c_size_t()
        check(self._lib.gbt_checkpoint_save(ctx, buf, n.value, ctypes.byref(w)), ctx)
        return buf.raw[: w.value]

    def restore(self, blob):
        """Continue from a checkpoint of a tracker with the same configuration."""
        ctx = self._ensure()
        check(self._lib.gbt_checkpoint_load(ctx, blob, len(blob)), ctx)
        return self

    def set_rgb_to_gray(self, mode):
        """GBT_RGB_CHANNEL0 (the reference's get_x) or GBT_RGB_BT601 for RGB frames."""
        check(self._lib.gbt_set_rgb_to_gray(self._ensure(), int(mode)), self._ctx)
        return self

    def enable_trajectories(self, history=20):
        """Keep every particle's last `history` positions on the GPU, in step
        with the slots (gbt_trajectories_enable)."""
        check(self._lib.gbt_trajectories_enable(self._ensure(), int(history)), self._ctx)
        return self

    def trajectories(self, stream=0, scale=0):
        """(xy[n, history, 2] oldest first and zero padded, length[n]) for the
        current particle slots."""
        ctx = self._ensure()
        n, T = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.gbt_get_trajectories(ctx, stream, scale, None, None, ctypes.byref(n), ctypes.byref(T)), ctx)
        xy = np.zeros((n.value, T.value, 2), np.int16)
        ln = np.zeros(n.value, np.uint8)
        check(self._lib.gbt_get_trajectories(ctx, stream, scale, xy.ctypes.data, ln.ctypes.data, ctypes.byref(n),
                                             ctypes.byref(T)), ctx)
        return xy, ln

    def stage(self, stream, scale, name, border=0):
        ctx = self._ensure()
        H, W = self.dims(stream, scale)
        kind = STAGES[name]
        if name in ("contrast", "sparse"):
            out = np.zeros((H, W), np.uint32)
            border = 0
        elif name in ("saliency", "mask"):
            out = np.zeros((H, W), np.uint8)
            border = 0
        else:
            out = np.zeros((H + 2 * border, W + 2 * border), np.uint8)
        check(self._lib.gbt_get_stage(ctx, stream, scale, kind, border, out.ctypes.data), ctx)
        return out

    def bins(self, stream, scale):
        ctx = self._ensure()
        r, c = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.gbt_bins(ctx, stream, scale, ctypes.byref(r), ctypes.byref(c)), ctx)
        BH, BW = r.value, c.value
        flow = np.zeros((BH, BW, 2), np.float32)
        count = np.zeros((BH, BW), np.uint32)
        st_n = np.zeros((BH, BW), np.int32)
        st_sp = np.zeros((BH, BW, 2), np.int32)
        check(self._lib.gbt_get_bins(ctx, stream, scale, flow.ctypes.data, count.ctypes.data, st_n.ctypes.data,
                                     st_sp.ctypes.data), ctx)
        return dict(flow=flow, count=count, stat_n=st_n, stat_speed=st_sp)

    def snapshot(self, stream=0, borders=True):
        """Every stage of every scale, in the layout of tests/stage_api.snapshot."""
        out = []
        for s in range(self._cfgs[stream].nscales):
            d = dict(
                input=self.stage(stream, s, "input", 6 if borders else 0),
                s1=self.stage(stream, s, "s1", 3 if borders else 0),
                s2=self.stage(stream, s, "s2", 6 if borders else 0),
                contrast=self.stage(stream, s, "contrast"),
                saliency=self.stage(stream, s, "saliency"),
                mask=self.stage(stream, s, "mask"),
                sparse=self.stage(stream, s, "sparse"),
            )
            d.update(self.bins(stream, s))
            p = self._particles(stream, s)
            feat32 = np.concatenate([p["feat"], np.full_like(p["feat"], 255)], axis=1)
            d.update(speed=p["speed"], pos=p["pos"], age=p["age"], feat=feat32, matches=p["matches"],
                     compact=p["compact"])
            out.append(d)
        return out


class Tracker(BatchTracker):
    """Single-stream tracker with the reference's tracker<F> interface.
    matcher="lk" selects the pyramidal LK tracker strategy (pyrlk_cpu)."""

    def __init__(self, domain, nscales, device=0, graphs=False, matcher="bc2s", **settings):
        rows, cols = domain
        cfg = dict(rows=rows, cols=cols, nscales=nscales, matcher={"bc2s": GBT_MATCHER_BC2S, "lk": GBT_MATCHER_LK}[matcher])
        cfg.update(settings)
        super().__init__([cfg], device=device, graphs=graphs)

    def run(self, frame, location=None):
        return super().run([frame], location)

    def strategy(self):
        return _Strategy(_ScaleSetter(self, None, None))

    def scale(self, s):
        return _Scale(self, 0, s)

    def pset(self):
        return ParticleSet(self, 0, 0)

    def domain(self):
        return self.dims(0, 0)

    def nparticles(self, stream=0, scale=None):
        return super().nparticles(stream, scale)
