"""GPU pyramidal LK against the oracle (and the reference's own LK golden):
at least 99.5% of tracks must agree within 0.01 px."""
import numpy as np
import pytest

from oracle_lib import box_pyramid_u8, load_golden, lk_track

pytestmark = pytest.mark.gpu

TOL_PX = 0.01
MIN_AGREE = 0.995


def _torch():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def _points(rng, H, W, n, margin):
    ints = np.stack([rng.integers(margin, H - margin, n // 2), rng.integers(margin, W - margin, n // 2)], 1)
    flts = np.stack([rng.uniform(margin, H - margin, n - n // 2), rng.uniform(margin, W - margin, n - n // 2)], 1)
    return np.concatenate([ints, flts]).astype(np.float32)


def _agreement(gpu_out, gpu_st, ora_out, ora_st):
    status_agree = (gpu_st > 0) == (ora_st > 0)
    both = (gpu_st > 0) & (ora_st > 0)
    d = np.abs(gpu_out[both] - ora_out[both]).max(axis=1)
    return status_agree.mean(), (d < TOL_PX).mean() if both.any() else 1.0, both.sum()


@pytest.mark.parametrize("is_u8,L,window,npix,iters", [
    (True, 3, 11, 25, 30),      # the reference's constants, gl8u path
    (True, 3, 7, 25, 5),        # 7x7 window, 5 iterations per level
    (False, 5, 9, 81, 10),      # fp32 Gaussian pyramid, 9x9 full window, 10 iterations
])
def test_lk_matches_oracle(is_u8, L, window, npix, iters):
    torch = _torch()
    from cuimg_gb300 import lk, synth
    rng = np.random.default_rng(1)
    H, W, npairs, n = 480, 640, 3, 600
    prevs, curs, pts = [], [], []
    for p in range(npairs):
        s = synth.Stream(40 + p, H, W)
        if is_u8:
            prevs.append(s.frame(3))
            curs.append(s.frame(4))
        else:
            prevs.append(s.frame_f32(3))
            curs.append(s.frame_f32(4))
        pts.append(_points(rng, H, W, n, 24))
    dt = torch.uint8 if is_u8 else torch.float32
    P = torch.from_numpy(np.stack(prevs)).to("cuda", dt)
    C = torch.from_numpy(np.stack(curs)).to("cuda", dt)
    X = torch.from_numpy(np.stack(pts)).cuda()
    prm = lk.params(window=window, npix=npix, max_iter=iters)
    out, st, err = lk.track(P, C, X, nlevels=L, prm=prm)
    torch.cuda.synchronize()
    out, st = out.cpu().numpy(), st.cpu().numpy()
    for p in range(npairs):
        o_out, o_st, _ = lk_track(prevs[p], curs[p], pts[p], L, pyr=0 if is_u8 else 1, window=window, npix=npix,
                                  max_iter=iters)
        sa, pa, nboth = _agreement(out[p], st[p], o_out, o_st)
        assert nboth > n // 2
        assert sa >= MIN_AGREE and pa >= MIN_AGREE, (p, sa, pa)


def test_lk_matches_reference_golden():
    torch = _torch()
    from cuimg_gb300 import lk
    g = load_golden("lk_240x320_s3")
    rows, cols, L, seed = [int(x) for x in g["meta"]]
    f0, f1 = g["frames"][0], g["frames"][1]
    p0 = [f0] + box_pyramid_u8(f0, L)
    p1 = [f1] + box_pyramid_u8(f1, L)
    for s in range(L):
        pts = g["born_s%d_pos" % s]
        ref_pos, ref_age = g["tracked_s%d_pos" % s], g["tracked_s%d_age" % s]
        A = torch.from_numpy(np.ascontiguousarray(p0[s])).cuda()
        B = torch.from_numpy(np.ascontiguousarray(p1[s])).cuda()
        out, st, _ = lk.track(A, B, torch.from_numpy(pts).cuda(), nlevels=L - s)
        out, st = out.cpu().numpy()[0], st.cpu().numpy()[0]
        H, W = p0[s].shape
        m = 12 * 2 ** (L - 1 - s)
        inner = (pts[:, 0] >= m) & (pts[:, 1] >= m) & (pts[:, 0] < H - m) & (pts[:, 1] < W - m)
        np.testing.assert_array_equal(st[inner] > 0, ref_age[inner] > 0)
        both = inner & (st > 0)
        d = np.abs(out[both] - ref_pos[both]).max(axis=1)
        assert (d < TOL_PX).mean() >= MIN_AGREE, (s, (d < TOL_PX).mean())


def test_lk_edge_points_and_empty():
    torch = _torch()
    from cuimg_gb300 import lk, synth
    s = synth.Stream(9, 120, 160)
    A = torch.from_numpy(s.frame(0)).cuda()
    B = torch.from_numpy(s.frame(1)).cuda()
    pts = np.array([[0, 0], [2.5, 80], [119, 159], [60, 1], [-5, 40], [60.5, 80.25]], np.float32)
    out, st, err = lk.track(A, B, torch.from_numpy(pts).cuda(), nlevels=2)
    o_out, o_st, _ = lk_track(s.frame(0), s.frame(1), pts, 2, pyr=0)
    np.testing.assert_array_equal(st.cpu().numpy()[0], o_st)
    assert st.cpu().numpy()[0][:5].sum() == 0  # outside domain - border(3)
    out, st, err = lk.track(A, B, torch.zeros((0, 2)).cuda(), nlevels=2)
    assert out.numel() == 0


def test_lk_block_sizes_give_identical_tracks():
    # warps_per_block (the autotuned CTA size) changes speed only.
    torch = _torch()
    from cuimg_gb300 import autotune, lk, synth
    H, W, n = 240, 320, 500
    rng = np.random.default_rng(5)
    s = synth.Stream(41, H, W)
    A = torch.from_numpy(np.stack([s.frame_f32(0), s.frame_f32(2)])).cuda()
    B = torch.from_numpy(np.stack([s.frame_f32(1), s.frame_f32(3)])).cuda()
    X = torch.from_numpy(np.stack([_points(rng, H, W, n, 20), _points(rng, H, W, n, 20)])).cuda()
    runs = [lk.track(A, B, X, nlevels=3, prm=lk.params(window=9, npix=81, max_iter=10, warps_per_block=w))
            for w in (2, 4, 8, 0)]
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            assert torch.equal(a, b)
    p = autotune.tune_lk(A, B, X, 3, lk.params(window=9, npix=81, max_iter=10), force=True)
    assert p.warps_per_block in autotune.LK_WARPS
