"""The allocation-free LK entry point against the allocating one.

gbt_lk_track_batch_noalloc serves callers that cannot allocate device memory
(an application owning the device heap or budget, a plugin forbidden to call
cudaMalloc): it runs the same tracker out of a fixed static device arena.
Both entry points launch the same kernels on the same inputs, so their
outputs must be bitwise equal -- for two calls in a row on different inputs,
and for two calls queued back to back on one stream with a single wait at the
end (the arena is shared; stream order must keep the second call from
overwriting it under the first).  Oversized requests must be refused.  This
file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GBT_E_TOO_LARGE = 6


def _lib():
    from cuimg_gb300 import lk
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    lk._declare(lib)
    P, I32 = ctypes.c_void_p, ctypes.c_int32
    lib.gbt_lk_track_batch_noalloc.argtypes = [P, P, ctypes.c_int64, ctypes.c_int64, I32, I32, I32, I32,
                                               ctypes.POINTER(lk.gbt_lk_params), I32, P, I32, P, P, P, P]
    lib.gbt_lk_noalloc_max_bytes.restype = ctypes.c_int64
    return lib, lk


def _queue(fn, prev, cur, pts, L, prm, is_u8):
    """Queues one call on the current stream; returns (code, out, status, err)
    as device tensors (not yet waited for)."""
    import torch
    npairs, H, W = prev.shape
    n = pts.shape[1]
    es = 1 if is_u8 else 4
    out = torch.full((npairs, n, 2), -7.0, device="cuda")
    st = torch.full((npairs, n), -7, dtype=torch.int32, device="cuda")
    err = torch.full((npairs, n), -7.0, device="cuda")
    code = fn(prev.data_ptr(), cur.data_ptr(), W * es, H * W * es, H, W, int(is_u8), L, ctypes.byref(prm), npairs,
              pts.data_ptr(), n, out.data_ptr(), st.data_ptr(), err.data_ptr(),
              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return code, out, st, err


def _run(fn, *args):
    import torch
    code, out, st, err = _queue(fn, *args)
    torch.cuda.synchronize()
    return code, out.cpu().numpy(), st.cpu().numpy(), err.cpu().numpy()


def _inputs(seed, npairs, H, W, n, is_u8):
    import torch
    from cuimg_gb300 import synth
    rng = np.random.default_rng(seed)
    prevs, curs = [], []
    for p in range(npairs):
        s = synth.Stream(seed * 10 + p, H, W)
        prevs.append(s.frame(1) if is_u8 else s.frame_f32(1))
        curs.append(s.frame(2) if is_u8 else s.frame_f32(2))
    pts = np.stack([np.stack([rng.uniform(20, H - 20, n), rng.uniform(20, W - 20, n)], 1) for _ in range(npairs)])
    # half the points on integer pixels, where equal gradient norms are common
    pts[:, : n // 2] = np.floor(pts[:, : n // 2])
    dt = torch.uint8 if is_u8 else torch.float32
    return (torch.from_numpy(np.stack(prevs)).to("cuda", dt), torch.from_numpy(np.stack(curs)).to("cuda", dt),
            torch.from_numpy(pts.astype(np.float32)).cuda())


def _assert_same(a, b):
    for x, y in zip(a[1:], b[1:]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("is_u8,L,window", [(True, 3, 11), (False, 4, 9)])
def test_noalloc_matches_allocating_entry_point_twice(is_u8, L, window):
    pytest.importorskip("torch")
    lib, lk = _lib()
    prm = lk.params(window=window)
    for call, seed in enumerate((3, 4)):  # two calls in a row, different inputs
        prev, cur, pts = _inputs(seed, 2, 240, 320, 300, is_u8)
        r0 = _run(lib.gbt_lk_track_batch, prev, cur, pts, L, prm, is_u8)
        r1 = _run(lib.gbt_lk_track_batch_noalloc, prev, cur, pts, L, prm, is_u8)
        assert r0[0] == 0 and r1[0] == 0, (call, r0[0], r1[0])
        assert (r0[2] > 0).sum() > 100
        _assert_same(r1, r0)


def test_noalloc_calls_queued_back_to_back_on_one_stream():
    torch = pytest.importorskip("torch")
    lib, lk = _lib()
    prm = lk.params()
    a = _inputs(6, 2, 240, 320, 400, True)
    b = _inputs(7, 3, 200, 288, 500, True)  # another geometry: the arena's layout changes between the calls
    ref_a = _run(lib.gbt_lk_track_batch, *a, 3, prm, True)
    ref_b = _run(lib.gbt_lk_track_batch, *b, 3, prm, True)
    qa = _queue(lib.gbt_lk_track_batch_noalloc, *a, 3, prm, True)
    qb = _queue(lib.gbt_lk_track_batch_noalloc, *b, 3, prm, True)
    torch.cuda.synchronize()
    assert qa[0] == 0 and qb[0] == 0
    _assert_same([0] + [t.cpu().numpy() for t in qa[1:]], ref_a)
    _assert_same([0] + [t.cpu().numpy() for t in qb[1:]], ref_b)


def test_noalloc_rejects_requests_beyond_its_arena():
    pytest.importorskip("torch")
    lib, lk = _lib()
    limit = lib.gbt_lk_noalloc_max_bytes()
    assert limit == 48 << 20
    prev, cur, pts = _inputs(5, 1, 240, 320, 8, True)
    # 64 pairs of 1080p would need far more than the fixed arena.
    need = lib.gbt_lk_scratch_bytes(1080, 1920, 4, 64)
    assert need > limit
    out = ctypes.c_void_p(pts.data_ptr())
    code = lib.gbt_lk_track_batch_noalloc(prev.data_ptr(), cur.data_ptr(), 1920, 1080 * 1920, 1080, 1920, 1, 4,
                                          ctypes.byref(lk.params()), 64, pts.data_ptr(), 8, out, out, out, None)
    assert code == GBT_E_TOO_LARGE
