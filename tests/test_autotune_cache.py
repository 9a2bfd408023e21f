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
