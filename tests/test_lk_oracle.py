"""Pins the LK oracle against the reference's own pyramidal LK tracker
(golden fixture from pyrlk_cpu<fast_detector<cpu>, iterative_lk_match_5x5>)."""
import numpy as np

from oracle_lib import box_pyramid_u8, load_golden, lk_track


def test_lk_oracle_matches_reference_golden():
    g = load_golden("lk_240x320_s3")
    rows, cols, L, seed = [int(x) for x in g["meta"]]
    f0, f1 = g["frames"][0], g["frames"][1]
    p0 = [f0] + box_pyramid_u8(f0, L)
    p1 = [f1] + box_pyramid_u8(f1, L)
    for s in range(L):
        pts = g["born_s%d_pos" % s]
        ref_pos, ref_age = g["tracked_s%d_pos" % s], g["tracked_s%d_age" % s]
        out, st, _ = lk_track(p0[s], p1[s], pts, L - s, pyr=0)
        H, W = p0[s].shape
        m = 12 * 2 ** (L - 1 - s)  # windows of every level stay inside (the reference reads outside otherwise)
        inner = (pts[:, 0] >= m) & (pts[:, 1] >= m) & (pts[:, 0] < H - m) & (pts[:, 1] < W - m)
        assert inner.sum() > 50
        np.testing.assert_array_equal(st[inner] > 0, ref_age[inner] > 0)
        both = inner & (st > 0)
        d = np.abs(out[both] - ref_pos[both]).max(axis=1)
        # Residual differences come from std::nth_element's unspecified order
        # among equal gradient norms (frequent at integer positions, where the
        # window samples the Sobel grid exactly); the oracle takes the lower
        # window index.
        assert (d < 0.01).mean() >= 0.97, (s, (d < 0.01).mean())
        assert np.median(d) < 1e-4


def test_lk_oracle_recovers_known_translation():
    rng = np.random.default_rng(0)
    base = rng.uniform(0, 255, (140, 180)).astype(np.float32)
    from oracle_lib import gauss_sep
    tex = gauss_sep(base, 2.0)
    prev = tex[10:130, 10:170]
    cur = tex[12:132, 7:167]  # content moves by (-2, +3)
    pts = np.array([[60.0, 80.0], [50.5, 70.25], [70.0, 100.0]], np.float32)
    out, st, _ = lk_track(prev, cur, pts, 2, pyr=1, window=11, npix=121, max_iter=30, eps=0.01)
    assert st.all()
    np.testing.assert_allclose(out - pts, [[-2.0, 3.0]] * 3, atol=0.05)
