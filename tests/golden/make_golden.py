"""Generates the committed golden fixtures from the reference itself.

Run where the reference sources are mounted (default /root/reference):

    python tests/golden/make_golden.py [REF_SRC]

Outputs (small, committed):
  meta_gaussian_taps.json -- sigma -> {x: float} for the generated
      meta_kernel<meta_gaussian<0, sigma>, x>::coef() tables (integer sigma
      1..50, from running the reference's tools/make_meta_gaussian generator)
      and the float taps of cuimg/gaussian_kernel.h for sigma 0.5;
  tracker_*.npz -- input frames and the reference CPU tracker's state after
      every frame (particles, features, matches) plus every stage image after
      the last frame, from oracle/_ref/libcuimg_ref.so (built by
      `make -C oracle ref`);
  altdet_*.npz -- the same particle state for the generic strategy with the
      reference's regular_detector and dense_detector;
  lk_*.npz -- the reference's pyramidal LK tracker on a frame pair.
"""
import ctypes
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
from stage_api import StageLib, snapshot  # noqa: E402
from oracle_lib import alt_reference, alt_reference_particles  # noqa: E402

CASES = [
    # name, rows, cols, nscales, detector_frequency, frames, seed
    ("tracker_120x160_s3_d10", 120, 160, 3, 10, 14, 1),
    ("tracker_101x133_s3_d1", 101, 133, 3, 1, 8, 3),
    ("tracker_96x128_s2_d3", 96, 128, 2, 3, 10, 5),
]


def make_taps(ref):
    out = {}
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "mmg")
        subprocess.check_call(["g++", "-O0", "-o", exe, os.path.join(ref, "tools/make_meta_gaussian/make_meta_gaussian.cpp")])
        gen = os.path.join(td, "gen")
        os.makedirs(gen)
        subprocess.check_call([exe, "-s", gen])
        pat = re.compile(r"meta_kernel<meta_gaussian<0, (\d+)>, (-?\d+)>.*?return ([-0-9.e+]+)f;")
        for fn in os.listdir(gen):
            with open(os.path.join(gen, fn)) as f:
                for line in f:
                    m = pat.search(line)
                    if m:
                        s, x, v = int(m.group(1)), int(m.group(2)), m.group(3)
                        out.setdefault(str(s), {})[str(x)] = float(np.float32(v))
        # float taps of cuimg/gaussian_kernel.h for sigma = 0.5
        src = os.path.join(td, "half.cpp")
        with open(src, "w") as f:
            f.write('#include <cstdio>\n#include <cassert>\n#include <cuimg/profiler.h>\n#include <cuimg/dsl/all.h>\n#include <cuimg/gaussian_kernel.h>\n'
                    'int main(){for(int x=-2;x<=2;x++) printf("%d %a\\n", x, (double)cuimg::gaussian_derivative<0>(0.5f, x));}\n')
        exe2 = os.path.join(td, "half")
        subprocess.check_call(["g++", "-O0", "-I" + ref, "-I" + os.path.join(ROOT, "oracle/shim"), "-DNO_CUDA", "-std=c++11", "-w",
                               src, "-o", exe2])
        half = {}
        for line in subprocess.check_output([exe2], text=True).split("\n"):
            if line.strip():
                x, v = line.split()
                half[x] = float.fromhex(v)
        out["0.5"] = half
    return out


def synth_frames(rows, cols, n, seed):
    lib = ctypes.CDLL(os.path.join(ROOT, "cuimg_gb300/_build/libgbt_synth.so"))
    lib.synth_create.restype = ctypes.c_void_p
    lib.synth_create.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
    lib.synth_frame_u8.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.synth_destroy.argtypes = [ctypes.c_void_p]
    h = lib.synth_create(seed, rows, cols)
    frames = np.zeros((n, rows, cols), np.uint8)
    for t in range(n):
        lib.synth_frame_u8(h, t, frames[t].ctypes.data)
    lib.synth_destroy(h)
    return frames


def make_tracker_case(name, rows, cols, L, detf, n, seed):
    os.environ["OMP_NUM_THREADS"] = "1"
    ref = StageLib(ctypes.CDLL(os.path.join(ROOT, "oracle/_ref/libcuimg_ref.so")), "ref_").create(rows, cols, L, 20, detf, 1)
    frames = synth_frames(rows, cols, n, seed)
    d = dict(frames=frames, meta=np.array([rows, cols, L, 20, detf, 1, n, seed], np.int32))
    for t in range(n):
        ref.run(frames[t])
        for s in range(L):
            p = ref.particles(s)
            d["f%d_s%d_pos" % (t, s)] = p["pos"]
            d["f%d_s%d_speed" % (t, s)] = p["speed"]
            d["f%d_s%d_age" % (t, s)] = p["age"]
            d["f%d_s%d_feat" % (t, s)] = p["feat"][:, :16]
            d["f%d_s%d_weights_all_255" % (t, s)] = np.array(bool((p["feat"][:, 16:] == 255).all()))
            if ref.compact_has_run(s):
                d["f%d_s%d_matches" % (t, s)] = p["matches"]
    snap = snapshot(ref, L)
    for s, st in enumerate(snap):
        for k in ("input", "s1", "s2", "contrast", "saliency", "mask", "sparse", "flow", "count", "stat_n",
                  "stat_speed"):
            d["last_s%d_%s" % (s, k)] = st[k]
    ref.destroy()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)


ALT_CASES = [
    # name, detector (1 regular, 2 dense), rows, cols, nscales, detector_frequency, frames, seed, step, grad_th
    ("altdet_regular_120x160_s2", 1, 120, 160, 2, 3, 8, 7, 3, 8),
    ("altdet_dense_64x80_s2", 2, 64, 80, 2, 2, 5, 8, 1, 1),
]


def make_alt_case(name, kind, rows, cols, L, detf, n, seed, step, grad_th):
    """The reference's generic strategy with regular_detector or dense_detector."""
    os.environ["OMP_NUM_THREADS"] = "1"
    lib, h = alt_reference(kind, rows, cols, L, detf, 1, step, grad_th)
    frames = synth_frames(rows, cols, n, seed)
    d = dict(frames=frames, meta=np.array([kind, rows, cols, L, detf, 1, n, seed, step, grad_th], np.int32))
    for t in range(n):
        lib.refx_run(h, frames[t].ctypes.data)
        for s in range(L):
            p = alt_reference_particles(lib, h, s)
            d["f%d_s%d_pos" % (t, s)] = p["pos"]
            d["f%d_s%d_speed" % (t, s)] = p["speed"]
            d["f%d_s%d_age" % (t, s)] = p["age"]
            d["f%d_s%d_feat" % (t, s)] = p["feat"][:, :16]
            if p["compact"]:
                d["f%d_s%d_matches" % (t, s)] = p["matches"]
    lib.refx_destroy(h)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)


LK_CASES = [
    # name, rows, cols, nscales, seed
    ("lk_240x320_s3", 240, 320, 3, 21),
]


def make_lk_case(name, rows, cols, L, seed):
    """The reference's own pyramidal LK tracker (pyrlk_cpu) on a frame pair:
    detector births on frame 0, then one LK step; no filtering or merging."""
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle/_ref/libcuimg_ref.so"))
    lib.reflk_create.restype = ctypes.c_void_p
    lib.reflk_create.argtypes = [ctypes.c_int] * 4
    lib.reflk_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.reflk_nparticles.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.reflk_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.reflk_destroy.argtypes = [ctypes.c_void_p]
    frames = synth_frames(rows, cols, 2, seed)
    h = lib.reflk_create(rows, cols, L, 20)
    d = dict(frames=frames, meta=np.array([rows, cols, L, seed], np.int32))

    def grab(tag):
        for s in range(L):
            n = lib.reflk_nparticles(h, s)
            pos = np.zeros((n, 2), np.float32)
            age = np.zeros(n, np.uint16)
            lib.reflk_get(h, s, pos.ctypes.data, age.ctypes.data)
            d["%s_s%d_pos" % (tag, s)] = pos
            d["%s_s%d_age" % (tag, s)] = age

    lib.reflk_run(h, frames[0].ctypes.data)
    grab("born")
    lib.reflk_run(h, frames[1].ctypes.data)
    grab("tracked")
    lib.reflk_destroy(h)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    taps = make_taps(ref)
    with open(os.path.join(HERE, "meta_gaussian_taps.json"), "w") as f:
        json.dump(taps, f, indent=0, sort_keys=True)
    for case in CASES:
        make_tracker_case(*case)
    for case in ALT_CASES:
        make_alt_case(*case)
    for case in LK_CASES:
        make_lk_case(*case)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
