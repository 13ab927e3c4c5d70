"""The differentiable warp residual on the GPU (sst_warp_residual and the
torch.autograd Function over it) against the FP64 oracle, central finite
differences (h = 1e-3), the analytic ECC Jacobian, and a joint template +
warp refinement.

Tolerances: loss 1e-5 relative; parameter gradients 1e-4 relative to the
largest component; template / flow gradients 1e-4 of their scale (FP32
sampling against FP64) except at samples within FP32 rounding of a pixel-grid
line, where the bilinear derivative jumps (at most 0.2 % of the pixels).
Finite differences: 5e-3 relative (samples that cross a grid line within the
step).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tex(w, h, dx=0.0, dy=0.0):
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    X, Y = x - dx, y - dy
    return (10 + 4 * np.sin(2 * np.pi * X / 17.0) * np.cos(2 * np.pi * Y / 13.0)
            + 3 * np.sin(2 * np.pi * (X + Y) / 23.0))


def _problem(n=3, w=96, h=64, seed=1):
    rng = np.random.default_rng(seed)
    tmpl = _tex(w, h)
    frames, params = [], []
    for _ in range(n):
        d = rng.uniform(-1.5, 1.5, size=2)
        frames.append(_tex(w, h, -d[0], -d[1]) + rng.normal(0, 0.05, size=(h, w)))
        params.append([1 + rng.normal(0, 2e-3), rng.normal(0, 2e-3), d[0] + rng.normal(0, 0.2),
                       rng.normal(0, 2e-3), 1 + rng.normal(0, 2e-3), d[1] + rng.normal(0, 0.2)])
    flow = rng.normal(0, 0.05, size=(n, h, w, 2))
    return (np.stack(frames).astype(np.float32), tmpl.astype(np.float32), np.array(params, np.float32),
            flow.astype(np.float32))


def _gpu(*arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def test_forward_and_gradients_match_oracle(gpu, oracle):
    import torch
    from serstacker_gb300 import adjoint
    frames, tmpl, params, flow = _problem()
    fr, T, p, fl = _gpu(frames, tmpl, params, flow)
    T.requires_grad_(True)
    p.requires_grad_(True)
    fl.requires_grad_(True)
    loss = adjoint.warp_residual(fr, T, p, gpu.AFFINE, fl)
    loss.sum().backward()
    m = oracle.model(oracle.AFFINE)
    gt_sum = np.zeros(tmpl.shape)
    for i in range(len(frames)):
        st = oracle.set_params(m, oracle.identity(m), params[i].astype(np.float64))
        L, gp, gt, gu = oracle.warp_residual(m, st, frames[i].astype(np.float64), tmpl.astype(np.float64),
                                             flow[i].astype(np.float64))
        gt_sum += gt
        assert abs(float(loss[i].detach()) - L) <= 1e-5 * L
        g = p.grad[i].cpu().numpy().astype(np.float64)
        assert np.abs(g - gp).max() <= 1e-4 * np.abs(gp).max(), (i, g, gp)
        gug = fl.grad[i].cpu().numpy()
        off = np.abs(gug - gu) > 1e-4 * max(1.0, np.abs(gu).max())
        assert off.mean() <= 2e-3, off.mean()
    dT = np.abs(T.grad.cpu().numpy() - gt_sum)
    assert (dT > 1e-4 * max(1.0, np.abs(gt_sum).max())).mean() <= 2e-3


def test_parameter_gradient_matches_central_differences(gpu):
    import torch
    from serstacker_gb300 import adjoint
    frames, tmpl, params, flow = _problem(n=2, seed=4)
    # generic parameters: no sample sits exactly on a pixel-grid line
    params = params + np.float32(1.37e-4)
    fr, T, fl = _gpu(frames, tmpl, flow)
    p = torch.from_numpy(params).cuda().requires_grad_(True)
    adjoint.warp_residual(fr, T, p, gpu.AFFINE, fl).sum().backward()
    g = p.grad.cpu().numpy().astype(np.float64)
    h = 1e-3
    for i in range(2):
        for k in range(6):
            pp, pm = params.astype(np.float64).copy(), params.astype(np.float64).copy()
            pp[i, k] += h
            pm[i, k] -= h
            Lp = float(adjoint.warp_residual(fr, T, torch.from_numpy(pp).float().cuda(), gpu.AFFINE, fl).sum())
            Lm = float(adjoint.warp_residual(fr, T, torch.from_numpy(pm).float().cuda(), gpu.AFFINE, fl).sum())
            fd = (Lp - Lm) / (2 * h)
            assert abs(fd - g[i, k]) <= 5e-3 * np.abs(g[i]).max(), (i, k, fd, g[i, k])


def test_template_gradient_matches_central_differences(gpu):
    import torch
    from serstacker_gb300 import adjoint
    frames, tmpl, params, _ = _problem(n=2, seed=6)
    fr, p = _gpu(frames, params)
    T = torch.from_numpy(tmpl).cuda().requires_grad_(True)
    adjoint.warp_residual(fr, T, p, gpu.AFFINE).sum().backward()
    g = T.grad.cpu().numpy()
    h = 1e-3
    for (y, x) in [(10, 12), (33, 50), (60, 90)]:
        tp, tm = tmpl.astype(np.float64).copy(), tmpl.astype(np.float64).copy()
        tp[y, x] += h
        tm[y, x] -= h
        Lp = float(adjoint.warp_residual(fr, torch.from_numpy(tp).float().cuda(), p, gpu.AFFINE).sum())
        Lm = float(adjoint.warp_residual(fr, torch.from_numpy(tm).float().cuda(), p, gpu.AFFINE).sum())
        assert abs((Lp - Lm) / (2 * h) - g[y, x]) <= 1e-2 * max(1.0, abs(g[y, x]))


def test_gradient_agrees_with_the_analytic_ecc_jacobian(gpu, oracle):
    """J^T r with J from the steepest-descent images of the warped frame
    (ecc_differentiate gradients, as FA / LM form it) against the adjoint's
    J^T r over the same interior pixels (away from the replicated border).
    They differ by the derivative used: the 5x3 stencil of the warped image
    against the exact derivative of the bilinear interpolant, which is what
    the finite differences of the discrete objective see; the two gradients
    must point the same way (cosine > 0.98)."""
    import torch
    from serstacker_gb300 import adjoint
    frames, tmpl, params, _ = _problem(n=1, w=72, h=56, seed=9)
    h, w = tmpl.shape
    fr, T = _gpu(frames, tmpl)
    p = torch.from_numpy(params).cuda()
    u = torch.zeros((1, h, w, 2), dtype=torch.float32, device="cuda", requires_grad=True)
    adjoint.warp_residual(fr, T, p, gpu.AFFINE, u).sum().backward()
    gu = u.grad[0].cpu().numpy().astype(np.float64)        # r grad I per pixel
    m = oracle.model(oracle.AFFINE)
    st = oracle.set_params(m, oracle.identity(m), params[0].astype(np.float64))
    warped = oracle.remap(m, st, frames[0].astype(np.float64), w, h, border=oracle.BORDER_REPLICATE)
    gx, gy = oracle.differentiate(warped)
    r = warped - tmpl
    ecc, exact = np.zeros(6), np.zeros(6)
    for y in range(4, h - 4):
        for x in range(4, w - 4):
            ecc += r[y, x] * oracle.sd(m, st, x, y, gx[y, x], gy[y, x])
            exact += oracle.sd(m, st, x, y, gu[y, x, 0], gu[y, x, 1])
    cos = float(ecc @ exact / (np.linalg.norm(ecc) * np.linalg.norm(exact)))
    assert cos > 0.98, (cos, ecc, exact)


def test_joint_template_and_warp_refinement_decreases_the_loss(gpu):
    import torch
    from serstacker_gb300 import adjoint
    frames, tmpl, params, _ = _problem(n=4, seed=11)
    fr, T, p = _gpu(frames, tmpl + np.float32(0.3), params)
    T2, p2, hist = adjoint.refine(fr, T, p, gpu.AFFINE, iterations=5)
    assert all(b <= a * (1 + 1e-6) for a, b in zip(hist, hist[1:])), hist
    assert hist[-1] < 0.5 * hist[0], hist
