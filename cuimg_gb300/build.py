"""Build recipe for the native libraries (no CMake, no setuptools).

Produces, in-tree under cuimg_gb300/_build/:
  libcuimg_gb300.so  -- every CUDA kernel and the C ABI of include/cuimg_gb300.h,
                        compiled for sm_103a only;
  libgbt_synth.so    -- the seeded synthetic video generator (host C).
Translation units compile in parallel; a unit is rebuilt only when a source or
header it may include is newer than its object.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

CUDA_SOURCES = ["tracker.cu", "gaussian.cu", "lk.cu", "lkd.cu", "pyrlk.cu"]
# Per-file flags: the LK solvers keep separate multiply/add roundings, as the
# reference's C++ evaluates them.
EXTRA_FLAGS = {"lk.cu": ["--fmad=false"], "pyrlk.cu": ["--fmad=false"]}
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC,
]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cuimg_gb300")
    return cand


def _newest_dep():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(p) for p in paths)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    newest = _newest_dep()
    nvcc = _nvcc()
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < newest:
            jobs.append([nvcc] + NVCC_FLAGS + EXTRA_FLAGS.get(src, []) + ["-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    lib = os.path.join(OUT, "libcuimg_gb300.so")
    if force or jobs or not os.path.exists(lib):
        _run([nvcc, "-shared", "-o", lib] + objs + ["-lcudart"])
    synth = os.path.join(OUT, "libgbt_synth.so")
    src = os.path.join(CSRC, "synth.c")
    if force or not os.path.exists(synth) or os.path.getmtime(synth) < os.path.getmtime(src):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", src, "-o", synth, "-lm"])
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
