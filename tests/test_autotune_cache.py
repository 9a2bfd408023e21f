"""The autotuner's cache file stays valid JSON when several processes (one per
GPU under torchrun) store their choices at the same time."""
import json
import multiprocessing as mp
import os


def _writer(path, k):
    from cuimg_gb300 import autotune
    for j in range(20):
        autotune._store(path, "gpu%d|%d" % (k, j), {"0": k, "1": j})


def test_concurrent_stores_leave_a_valid_cache(tmp_path):
    from cuimg_gb300 import autotune
    path = str(tmp_path / "sub" / "autotune.json")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_writer, args=(path, k)) for k in range(4)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    with open(path) as f:
        cache = json.load(f)  # never a partial file
    assert cache and all(k.startswith("gpu") for k in cache)
    assert not [n for n in os.listdir(os.path.dirname(path)) if n.endswith(".tmp")]
    autotune._store(path, "k", 7)
    assert autotune._load_cache(path)["k"] == 7


def test_knob_settings_match_the_header():
    # The autotuner tries every setting the C ABI accepts for each knob, and no
    # other: the match-tile range and the blur strip heights in
    # include/cuimg_gb300.h.
    import re

    from cuimg_gb300 import autotune
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = open(os.path.join(root, "include", "cuimg_gb300.h")).read()
    m = re.search(r"#define GBT_TUNE_MATCH_TILE 2\s*/\*.*?(\d+)\.\.(\d+)", hdr)
    assert m, "GBT_TUNE_MATCH_TILE range not documented"
    lo, hi = int(m.group(1)), int(m.group(2))
    assert tuple(autotune.KNOBS[2][1]) == tuple(range(lo, hi + 1))
    m = re.search(r"#define GBT_TUNE_BLUR_ROWS 1\s*/\*.*?(\d+), (\d+) or (\d+)", hdr)
    assert m, "GBT_TUNE_BLUR_ROWS settings not documented"
    assert tuple(autotune.KNOBS[1][1]) == tuple(int(x) for x in m.groups())
