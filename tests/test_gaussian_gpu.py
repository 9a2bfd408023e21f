"""GPU Gaussian / pyramid parity against the oracle (fp32 within 1e-5
relative; uint8 pyramid bit-exact), called through the C ABI."""
import ctypes

import numpy as np
import pytest

from oracle_lib import box_pyramid_u8, gauss_pyramid, gauss_sep

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # fp32 tolerance for Gaussian and pyramid outputs


def _torch():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def _gauss_gpu(img, sigma):
    torch = _torch()
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    x = torch.from_numpy(np.ascontiguousarray(img, np.float32)).cuda()
    y = torch.empty_like(x)
    H, W = img.shape
    assert lib.gbt_gaussian_f32(x.data_ptr(), W * 4, y.data_ptr(), W * 4, H, W, ctypes.c_float(sigma), None) == 0
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("sigma", [0.5, 1.0, 2.0, 3.0, 4.0, 1.5])
@pytest.mark.parametrize("shape", [(1080, 1920), (37, 53), (5, 300), (130, 7), (300, 129)])
def test_gaussian_matches_oracle(sigma, shape):
    from cuimg_gb300 import synth
    H, W = shape
    img = synth.Stream(3, max(H, 16), max(W, 16)).frame_f32(1)[:H, :W].copy()
    out = _gauss_gpu(img, sigma)
    ref = gauss_sep(img, sigma)
    np.testing.assert_allclose(out, ref, rtol=RTOL, atol=0)


def test_gaussian_batch_and_pitch():
    torch = _torch()
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    rng = np.random.default_rng(0)
    n, H, W, pitch = 5, 67, 90, 128
    imgs = rng.uniform(0, 255, (n, H, W)).astype(np.float32)
    x = torch.zeros((n, H, pitch), dtype=torch.float32, device="cuda")
    x[:, :, :W] = torch.from_numpy(imgs).cuda()
    y = torch.zeros_like(x)
    assert lib.gbt_gaussian_f32_batch(x.data_ptr(), pitch * 4, H * pitch * 4, y.data_ptr(), pitch * 4, H * pitch * 4,
                                      H, W, n, ctypes.c_float(2.0), None) == 0
    torch.cuda.synchronize()
    out = y.cpu().numpy()[:, :, :W]
    for i in range(n):
        np.testing.assert_allclose(out[i], gauss_sep(imgs[i], 2.0), rtol=RTOL)
    assert float(y[:, :, W:].abs().max()) == 0.0  # padding untouched


def test_gaussian_linearity_full_size():
    # Size-independent property at the benchmark size: G(a x + b y) = a G(x) + b G(y).
    torch = _torch()
    rng = np.random.default_rng(2)
    a = rng.uniform(0, 255, (1080, 1920)).astype(np.float32)
    b = rng.uniform(0, 255, (1080, 1920)).astype(np.float32)
    lhs = _gauss_gpu(0.25 * a + 0.75 * b, 4.0)
    rhs = 0.25 * _gauss_gpu(a, 4.0) + 0.75 * _gauss_gpu(b, 4.0)
    np.testing.assert_allclose(lhs, rhs, rtol=1e-5, atol=1e-4)


def test_gaussian_pyramid_matches_oracle():
    torch = _torch()
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    from cuimg_gb300 import synth
    H, W, L = 480, 640, 5
    img = synth.Stream(4, H, W).frame_f32(0)
    x = torch.from_numpy(img).cuda()
    total = sum((H >> l) * (W >> l) for l in range(1, L))
    y = torch.zeros(total, dtype=torch.float32, device="cuda")
    assert lib.gbt_gaussian_pyramid_f32(x.data_ptr(), W * 4, H, W, L, y.data_ptr(), None) == 0
    torch.cuda.synchronize()
    out = y.cpu().numpy()
    ref = gauss_pyramid(img, L)
    off = 0
    for l, lv in enumerate(ref, 1):
        n = lv.size
        np.testing.assert_allclose(out[off:off + n].reshape(lv.shape), lv, rtol=RTOL)
        off += n


def test_box_pyramid_u8_bit_exact():
    torch = _torch()
    from cuimg_gb300._native import cuda_lib
    lib = cuda_lib()
    from cuimg_gb300 import synth
    H, W, L = 1080, 1920, 4
    img = synth.Stream(5, H, W).frame(0)
    x = torch.from_numpy(img).cuda()
    total = sum((H >> l) * (W >> l) for l in range(1, L))
    y = torch.zeros(total, dtype=torch.uint8, device="cuda")
    assert lib.gbt_pyramid_u8(x.data_ptr(), W, H, W, L, y.data_ptr(), None) == 0
    torch.cuda.synchronize()
    out = y.cpu().numpy()
    off = 0
    for lv in box_pyramid_u8(img, L):
        np.testing.assert_array_equal(out[off:off + lv.size].reshape(lv.shape), lv)
        off += lv.size
