"""Host-side assignment of independent video streams to GPUs (replicas).

Streams never exchange data, so multi-GPU tracking is one context per GPU with
a disjoint subset of the streams and no collective.  ``assign`` balances the
per-frame work (pixels over all pyramid levels) greedily: largest stream
first, onto the least-loaded rank; ties go to the lower rank, so every rank
computes the same assignment without communicating.
"""


def stream_cost(rows, cols, nscales, frames=1):
    return frames * sum((rows >> l) * (cols >> l) for l in range(nscales))


def assign(streams, world):
    """streams: list of dicts with rows, cols, nscales (and optional frames).
    Returns a list (one per rank) of stream indices."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(streams)),
                   key=lambda i: (-stream_cost(streams[i]["rows"], streams[i]["cols"], streams[i]["nscales"],
                                               streams[i].get("frames", 1)), i))
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in order:
        s = streams[i]
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += stream_cost(s["rows"], s["cols"], s["nscales"], s.get("frames", 1))
    for r in out:
        r.sort()
    return out


def my_streams(streams, rank, world):
    return assign(streams, world)[rank]
