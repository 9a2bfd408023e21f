"""The C ABI library loads and exports every symbol include/*.h declares;
host-only entry points (no GPU needed) behave like the oracle."""
import ctypes
import glob
import json
import os
import re

import numpy as np

from oracle_lib import GOLDEN, ROOT, oracle


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(?:int|void|int32_t)\s+\**\s*(gbt_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    names = declared_symbols()
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_gaussian_taps_entry_point_matches_generator():
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    with open(os.path.join(GOLDEN, "meta_gaussian_taps.json")) as f:
        gold = json.load(f)
    taps = np.zeros(64, np.float32)
    R = ctypes.c_int32()
    for sigma in [0.5] + list(range(1, 9)):
        assert lib.gbt_gaussian_taps(ctypes.c_float(sigma), taps.ctypes.data, ctypes.byref(R)) == 0
        assert R.value == int(np.ceil(3 * sigma))
        for x_s, v in gold[str(sigma) if sigma != int(sigma) else str(int(sigma))].items():
            x = int(x_s)
            if abs(x) <= R.value:
                assert np.float32(v) == taps[x + R.value], (sigma, x)
    assert lib.gbt_gaussian_taps(ctypes.c_float(-1.0), taps.ctypes.data, ctypes.byref(R)) == 1


def test_size_rule_matches_oracle():
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    o = oracle()
    rng = np.random.default_rng(3)
    for _ in range(300):
        H, W, L = int(rng.integers(8, 600)), int(rng.integers(8, 600)), int(rng.integers(1, 7))
        assert bool(lib.gbt_sizes_ok(H, W, L)) == bool(o.oracle_sizes_ok(H, W, L)), (H, W, L)


def test_config_defaults_are_reference_defaults():
    from cuimg_gb300._native import cuda_lib, gbt_config
    cfg = gbt_config()
    cuda_lib().gbt_config_default(ctypes.byref(cfg), 480, 640, 3)
    # generic_strategy ctor (tracking_strategies.hpp:33-49), fast_detector ctor (fast_detector.hpp:161-168)
    assert (cfg.detector_frequency, cfg.filtering_frequency, cfg.k, cfg.with_merge, cfg.detector_n) == (1, 1, 300, 1, 9)


def test_invalid_arguments_fail_cleanly_without_gpu_work():
    from cuimg_gb300._native import cuda_lib, gbt_config
    lib = cuda_lib()
    out = ctypes.c_void_p()
    cfg = gbt_config()
    lib.gbt_config_default(ctypes.byref(cfg), 97, 131, 3)   # unsupported geometry
    assert lib.gbt_create(ctypes.byref(cfg), 1, 0, ctypes.byref(out)) == 1
    assert not out.value
    assert lib.gbt_create(None, 1, 0, ctypes.byref(out)) == 1
    assert lib.gbt_destroy(None) == 1
    assert lib.gbt_gaussian_f32(None, 0, None, 0, 10, 10, ctypes.c_float(1.0), None) == 1
