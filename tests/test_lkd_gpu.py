"""Adjoint of the LK photometric residual and the Gaussian pyramid, against
the FP64 oracle (oracle/lk_adjoint_oracle.c): forward loss, and gradients with
respect to both frames and the initial flow against FP64 central differences
with h = 1e-3 -- within 1e-3 relative."""
import numpy as np
import pytest

from oracle_lib import lkd_forward64, lkd_grad_fd64

pytestmark = pytest.mark.gpu

RTOL_GRAD = 1e-3


def _torch():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def _problem(seed, H, W, n, margin, flow=1.0):
    from cuimg_gb300 import synth
    rng = np.random.default_rng(seed)
    s = synth.Stream(seed, H, W)
    I0, I1 = s.frame_f32(1, 0.0), s.frame_f32(2, 0.0)
    pts = np.stack([rng.uniform(margin, H - margin, n), rng.uniform(margin, W - margin, n)], 1).astype(np.float32)
    u0 = rng.uniform(-flow, flow, (n, 2)).astype(np.float32)
    return I0, I1, pts, u0


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("L,window,iters", [(3, 7, 4), (2, 9, 6)])
def test_adjoint_matches_fp64_central_differences(L, window, iters):
    torch = _torch()
    from cuimg_gb300 import lkd
    H, W, n = 48, 64, 4
    I0, I1, pts, u0 = _problem(11 + L, H, W, n, 14)
    wts = np.linspace(0.5, 1.5, n)
    loss64, _ = lkd_forward64(I0, I1, pts, u0, L, window, iters)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    loss, vf = lkd.forward(t(I0), t(I1), t(u0), t(pts), L, window, iters)
    np.testing.assert_allclose(loss.cpu().numpy()[0], loss64, rtol=1e-4)
    dI0, dI1, du0 = lkd.backward(t(I0), t(I1), t(u0), t(pts), t(wts.astype(np.float32)), L, window, iters)
    g0, g1, gu = lkd_grad_fd64(I0, I1, pts, u0, L, window, iters, wts, h=1e-3)
    assert _rel(dI0.cpu().numpy()[0], g0) < RTOL_GRAD
    assert _rel(dI1.cpu().numpy()[0], g1) < RTOL_GRAD
    assert _rel(du0.cpu().numpy()[0], gu) < RTOL_GRAD


def test_adjoint_config_scale_batch_and_directional_derivative():
    # 16 fp32 frame pairs at 640x480, 5 levels, 9x9 windows, 10 Gauss-Newton
    # steps, 20k points per pair; pyramids are recomputed in the backward.
    torch = _torch()
    from cuimg_gb300 import lkd, synth
    P, H, W, n, L, ws, K = 16, 480, 640, 20000, 5, 9, 10
    rng = np.random.default_rng(0)
    I0 = np.empty((P, H, W), np.float32)
    I1 = np.empty((P, H, W), np.float32)
    for p in range(P):
        s = synth.Stream(200 + p, H, W)
        I0[p], I1[p] = s.frame_f32(0), s.frame_f32(1)
    pts = np.stack([rng.uniform(40, H - 40, (P, n)), rng.uniform(40, W - 40, (P, n))], -1).astype(np.float32)
    u0 = rng.uniform(-2, 2, (P, n, 2)).astype(np.float32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    loss, vf = lkd.forward(t(I0), t(I1), t(u0), t(pts), L, ws, K)
    dI0, dI1, du0 = lkd.backward(t(I0), t(I1), t(u0), t(pts), torch.ones((P, n), device="cuda"), L, ws, K)
    torch.cuda.synchronize()
    for x in (loss, vf, dI0, dI1, du0):
        assert torch.isfinite(x).all()
    # One pair, a subset of points, against the FP64 oracle: loss and the
    # derivative along a random image direction.
    k = 64
    sub_p, sub_u = pts[0, :k], u0[0, :k]
    l64, _ = lkd_forward64(I0[0], I1[0], sub_p, sub_u, L, ws, K)
    lg, _ = lkd.forward(t(I0[:1]), t(I1[:1]), t(sub_u[None]), t(sub_p[None]), L, ws, K)
    np.testing.assert_allclose(lg.cpu().numpy()[0], l64, rtol=2e-4)
    g0, g1, gu = lkd.backward(t(I0[:1]), t(I1[:1]), t(sub_u[None]), t(sub_p[None]), torch.ones((1, k), device="cuda"),
                              L, ws, K)
    d0 = rng.standard_normal((H, W))
    d1 = rng.standard_normal((H, W))
    du = rng.standard_normal((k, 2))
    h = 1e-3
    lp, _ = lkd_forward64(I0[0] + h * d0, I1[0] + h * d1, sub_p, sub_u + h * du, L, ws, K)
    lm, _ = lkd_forward64(I0[0] - h * d0, I1[0] - h * d1, sub_p, sub_u - h * du, L, ws, K)
    fd = (lp.sum() - lm.sum()) / (2 * h)
    an = float((g0.cpu().numpy()[0] * d0).sum() + (g1.cpu().numpy()[0] * d1).sum() + (gu.cpu().numpy()[0] * du).sum())
    assert abs(an - fd) / abs(fd) < RTOL_GRAD, (an, fd)


def test_backward_from_the_tape_equals_the_replay():
    # The tape the forward records replaces the backward's replay: same
    # gradients up to the order of the float atomics.
    torch = _torch()
    from cuimg_gb300 import lkd
    for L, ws, K, seed in ((3, 7, 4, 21), (2, 9, 6, 22), (5, 9, 10, 23)):
        H, W = (48, 64) if L < 5 else (96, 128)
        I0, I1, pts, u0 = _problem(seed, H, W, 40, 14)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        wts = t(np.linspace(0.5, 1.5, 40).astype(np.float32))
        loss, vf, tape = lkd.forward(t(I0), t(I1), t(u0), t(pts), L, ws, K, tape=True)
        assert tape.numel() == lkd.tape_bytes(L, K, 1, 40)
        l2, v2 = lkd.forward(t(I0), t(I1), t(u0), t(pts), L, ws, K)
        assert torch.equal(loss, l2) and torch.equal(vf, v2)
        a = lkd.backward(t(I0), t(I1), t(u0), t(pts), wts, L, ws, K, tape=tape)
        b = lkd.backward(t(I0), t(I1), t(u0), t(pts), wts, L, ws, K)
        for got, want in zip(a, b):
            torch.testing.assert_close(got, want, rtol=1e-5, atol=1e-6 * float(want.abs().max()))


def test_autograd_function_routes_to_the_adjoint():
    torch = _torch()
    from cuimg_gb300 import lkd
    I0, I1, pts, u0 = _problem(5, 48, 64, 3, 14)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    a, b, u = t(I0).requires_grad_(), t(I1).requires_grad_(), t(u0).requires_grad_()
    loss = lkd.LKResidual.apply(a, b, u, t(pts), 3, 7, 4)
    loss.sum().backward()
    dI0, dI1, du0 = lkd.backward(t(I0), t(I1), t(u0), t(pts), torch.ones(3, device="cuda"), 3, 7, 4)
    # Same adjoint; the float atomics of the image scatter may sum in another order.
    for got, want in ((a.grad, dI0[0]), (b.grad, dI1[0]), (u.grad, du0[0])):
        torch.testing.assert_close(got, want, rtol=1e-5, atol=1e-6 * float(want.abs().max()))
