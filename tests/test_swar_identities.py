"""The exact integer identities the BC2S blur and the pyramid kernels compute
with (cuimg_gb300/csrc/tracker_kernels.cuh: havg4 / row_pass4 / col_pass4 and
pyr_mean2), checked over every byte value.  The reference's passes are
(x[c-1] + 2 x[c] + x[c+1]) / 4 and (a + b + c + d) / 4 in C++ integer division
(cuimg/cpu/gaussian_blur.h:9-47, cuimg/gpu/mipmap.h:24-49)."""
import numpy as np

M = 0xFFFFFFFF


def havg4(a, b):
    # per-byte floor((a + b) / 2), four bytes per 32-bit word
    return ((a & b) + (((a ^ b) >> 1) & 0x7F7F7F7F)) & M


def test_three_tap_pass_is_two_floor_averages():
    a = np.arange(256, dtype=np.int64)
    A, B, C = np.meshgrid(a, a, a, indexing="ij")
    assert np.array_equal((A + 2 * B + C) // 4, havg4(havg4(A, C), B))


def test_bytewise_average_does_not_carry_between_bytes():
    rng = np.random.default_rng(3)
    x = rng.integers(0, 1 << 32, 200000, dtype=np.int64)
    y = rng.integers(0, 1 << 32, 200000, dtype=np.int64)
    got = havg4(x, y)
    for j in range(4):
        xb, yb = (x >> (8 * j)) & 255, (y >> (8 * j)) & 255
        assert np.array_equal((got >> (8 * j)) & 255, (xb + yb) // 2)


def test_pyramid_mean_in_16_bit_lanes():
    lo = 0x00FF00FF
    rng = np.random.default_rng(4)
    x = rng.integers(0, 1 << 32, 200000, dtype=np.int64)
    y = rng.integers(0, 1 << 32, 200000, dtype=np.int64)
    x[:2], y[:2] = M, M  # all 255: the largest lane sum, 1020
    got = ((((x & lo) + ((x >> 8) & lo) + (y & lo) + ((y >> 8) & lo)) >> 2) & lo)
    byte = lambda v, j: (v >> (8 * j)) & 255
    for k in range(2):  # output k from bytes 2k, 2k + 1 of both rows
        want = (byte(x, 2 * k) + byte(x, 2 * k + 1) + byte(y, 2 * k) + byte(y, 2 * k + 1)) // 4
        assert np.array_equal(byte(got, 2 * k), want)
        assert not np.any(byte(got, 2 * k + 1))
