"""The C and C++ boundary, compiled.

* include/cuimg_gb300.h is valid C (C99, pedantic) and C++, and its struct
  layouts and host-only calls agree with the ctypes mirror.
* include/cuimg_gb300_strategy.hpp compiles against the reference's own
  headers: the sample's tracking loop with tracker<bc2s_fast_gradient_gb300>
  and with tracker<pyrlk_gb300> builds and links against libcuimg_gb300.so,
  and the strategies' particle-set loaders reproduce the reference trackers'
  pset() (bc2s_fast_gradient_cpu's and pyrlk_cpu's) of every scale on every
  frame, bit for bit (particles, features, matches, compact_has_run, the
  sparse index, the sample's trajectories through sync_attributes).

The reference sources are needed for the C++ checks, so they are skipped where
the reference is not mounted.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "cuimg_gb300", "_build")
SHIM = os.path.join(ROOT, "oracle", "shim")
REF_SRC = os.environ.get("CUIMG_REF_SRC", "/root/reference")
CUDA_LIB = "/usr/local/cuda/lib64"
LINK_GBT = ["-L" + BUILD, "-lcuimg_gb300", "-Wl,-rpath," + BUILD, "-L" + CUDA_LIB, "-Wl,-rpath," + CUDA_LIB]
REF_FLAGS = ["-std=c++11", "-O1", "-DNO_CUDA", "-DNDEBUG", "-DCUIMG_RIGID_TRANSFORM_H_", "-fopenmp",
             "-I" + SHIM, "-I" + REF_SRC, "-I" + INCLUDE]

needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF_SRC, "cuimg")),
                               reason="reference sources not mounted")


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, "compile failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:])


def _run(exe, *args, env=None):
    e = dict(os.environ, OMP_NUM_THREADS="1")
    e.update(env or {})
    return subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, env=e, timeout=600)


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_c_header_is_valid_c_and_matches_the_ctypes_mirror(tmp_path, lang):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    exe = str(tmp_path / "c_abi_check")
    src = os.path.join(CPP, "c_abi_check.c")
    if lang == "c":
        cmd = ["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I" + INCLUDE, src, "-o", exe]
    else:
        cmd = ["g++", "-x", "c++", "-std=c++11", "-Wall", "-Wextra", "-Werror", "-I" + INCLUDE, src, "-x", "none",
               "-o", exe]
    _compile(cmd + LINK_GBT)
    r = _run(exe)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in r.stdout.splitlines():
        k, v = line.split(" ", 1)
        out[k] = v
    from cuimg_gb300 import lk
    from cuimg_gb300._native import gbt_config
    assert int(out["sizeof.gbt_config"]) == ctypes.sizeof(gbt_config)
    for name, _ in gbt_config._fields_:
        assert int(out["gbt_config." + name]) == getattr(gbt_config, name).offset, name
    assert int(out["sizeof.gbt_lk_params"]) == ctypes.sizeof(lk.gbt_lk_params)
    for name, _ in lk.gbt_lk_params._fields_:
        assert int(out["gbt_lk_params." + name]) == getattr(lk.gbt_lk_params, name).offset, name
    # host-only calls give the same answers through C as through ctypes
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    c = gbt_config()
    lib.gbt_config_default(ctypes.byref(c), 480, 640, 3)
    assert [int(x) for x in out["default"].split()] == [getattr(c, n) for n, _ in gbt_config._fields_]
    assert [int(x) for x in out["sizes_ok"].split()] == [1, 0, 0]
    assert int(out["lk_scratch"]) == lib.gbt_lk_scratch_bytes(480, 640, 3, 2)
    R, t0, tc = out["taps4"].split()
    assert int(R) == 12
    from oracle_lib import gauss_taps
    Ro, taps = gauss_taps(4.0)
    assert Ro == 12 and np.float32(t0) == taps[0] and np.float32(tc) == taps[12]


def _clip(rows, cols, n, seed):
    from cuimg_gb300 import synth
    return np.ascontiguousarray(synth.frames(seed, rows, cols, n))


@needs_ref
@pytest.mark.parametrize("rows,cols,L,det,n,seed", [(120, 160, 3, 3, 14, 1), (203, 317, 3, 10, 24, 9),
                                                    (480, 640, 3, 10, 30, 1)])
def test_strategy_loader_reproduces_the_reference_psets(tmp_path, rows, cols, L, det, n, seed):
    exe = str(tmp_path / "pset_load_check")
    _compile(["g++"] + REF_FLAGS + [os.path.join(CPP, "pset_load_check.cpp"),
                                    os.path.join(ROOT, "oracle", "_build", "liboracle.so"),
                                    "-Wl,-rpath," + os.path.join(ROOT, "oracle", "_build"), "-o", exe] + LINK_GBT)
    raw = str(tmp_path / "clip.raw")
    _clip(rows, cols, n, seed).tofile(raw)
    r = _run(exe, rows, cols, L, det, n, raw)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout
    comp = int(r.stdout.split("compactions=")[1].split()[0])
    assert comp >= L * ((n + det - 1) // det)  # every detector frame compacted every scale


@needs_ref
@pytest.mark.parametrize("rows,cols,L,det,n,seed", [(320, 480, 3, 3, 16, 5), (256, 384, 2, 1, 10, 6)])
def test_lk_strategy_loader_reproduces_the_reference_psets(tmp_path, rows, cols, L, det, n, seed):
    from oracle_lib import black_margin_frames
    exe = str(tmp_path / "pyrlk_load_check")
    _compile(["g++"] + REF_FLAGS + [os.path.join(CPP, "pyrlk_load_check.cpp"),
                                    os.path.join(ROOT, "oracle", "_build", "liboracle.so"),
                                    "-Wl,-rpath," + os.path.join(ROOT, "oracle", "_build"), "-o", exe] + LINK_GBT)
    raw = str(tmp_path / "clip.raw")
    np.ascontiguousarray(black_margin_frames(seed, rows, cols, n, 16 << (L - 1))).tofile(raw)
    r = _run(exe, rows, cols, L, det, n, raw)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout


@needs_ref
@pytest.mark.parametrize("strategy", ["bc2s", "pyrlk"])
def test_sample_loop_with_the_gb300_strategy_builds_and_links(tmp_path, strategy):
    """The sample's loop compiles unchanged but for the strategy name, links
    against libcuimg_gb300.so and reaches the C ABI.  Without a GPU the first
    frame's gbt_create fails and the strategy throws, as the reference throws on
    a CUDA error; with one, the run tracks."""
    exe = str(tmp_path / "sample_loop")
    extra = ["-DSAMPLE_STRATEGY=pyrlk_gb300"] if strategy == "pyrlk" else []
    _compile(["g++"] + REF_FLAGS + extra + [os.path.join(CPP, "sample_loop.cpp"), "-o", exe] + LINK_GBT)
    rows, cols, L, n = 120, 160, 3, 6
    raw = str(tmp_path / "clip.raw")
    _clip(rows, cols, n, 1).tofile(raw)
    r = _run(exe, rows, cols, L, 20, n, raw, tmp_path / "out.txt")
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stdout + r.stderr
    else:
        assert r.returncode == 3, r.stdout + r.stderr
        assert "error: cuimg_gb300: gbt_create failed" in r.stdout, r.stdout
