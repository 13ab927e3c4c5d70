"""Known-answer tests pinning the FP64 oracle (CPU only).

The reference ships no tests or golden data, so the oracle is pinned to the
mathematics it restates: motion-model formulas (c_image_transform.cc),
OpenCV primitive semantics (pyrDown, sepFilter2D, remap), the ECC solvers'
fixed points on exactly-known warps, and the integer Bayer operations
(debayer.cc) against independent numpy formulations.
"""
import math

import numpy as np
import pytest

from serstacker_gb300 import synth

MOTIONS = [0, 1, 2, 3, 4, 5, 6]


def rand_state(O, rng, t):
    m = O.model(t)
    s = O.identity(m)
    n = O.nparams(m)
    p = O.get_params(m, s)
    p = p + rng.normal(0, 1, size=n) * np.array({
        0: [2, 2], 1: [2, 2, 0.01], 2: [2, 2, 0.01, 0.01], 3: [1e-3, 1e-3, 2, 1e-3, 1e-3, 2],
        4: [1e-3, 1e-3, 2, 1e-3, 1e-3, 2, 1e-6, 1e-6], 5: [1e-3, 1e-3, 2, 1e-6, 1e-3, 1e-3, 2, 1e-6],
        6: [1e-3, 1e-3, 2, 1e-6, 1e-6, 1e-6, 1e-3, 1e-3, 2, 1e-6, 1e-6, 1e-6]}[t])
    return m, O.set_params(m, s, p)


@pytest.mark.parametrize("t", MOTIONS)
def test_sd_images_match_finite_differences(oracle, t):
    """create_steepest_descent_images == gx dWx/dp + gy dWy/dp (central FD of W)."""
    O = oracle
    rng = np.random.default_rng(t)
    m, s = rand_state(O, rng, t)
    n = O.nparams(m)
    p0 = O.get_params(m, s)
    for (x, y) in [(0.0, 0.0), (37.0, 11.0), (300.0, 200.0)]:
        gx, gy = 0.7, -1.3
        J = O.sd(m, s, x, y, gx, gy)
        for i in range(n):
            h = 1e-6 * max(1.0, abs(p0[i]))
            pp, pm = p0.copy(), p0.copy()
            pp[i] += h
            pm[i] -= h
            Xp, Yp = O.warp(m, O.set_params(m, s, pp), x, y)
            Xm, Ym = O.warp(m, O.set_params(m, s, pm), x, y)
            fd = gx * (Xp - Xm) / (2 * h) + gy * (Yp - Ym) / (2 * h)
            if t in (1, 2) and i == 2:   # reference's rotation SD carries the scale factor (c_image_transform.cc:647)
                pass
            assert J[i] == pytest.approx(fd, rel=1e-5, abs=1e-6), (t, i, x, y)


@pytest.mark.parametrize("t", MOTIONS)
def test_scale_transform_is_coordinate_scaling(oracle, t):
    """scale_transfrom(f): W_f(f x) = f W(x)"""
    O = oracle
    rng = np.random.default_rng(10 + t)
    m, s = rand_state(O, rng, t)
    f = 0.5
    sf = O.scale(m, s, f)
    for (x, y) in [(3.0, 4.0), (100.0, 50.0)]:
        X, Y = O.warp(m, s, x, y)
        Xf, Yf = O.warp(m, sf, f * x, f * y)
        assert Xf == pytest.approx(f * X, abs=1e-9)
        assert Yf == pytest.approx(f * Y, abs=1e-9)


@pytest.mark.parametrize("t", [0, 1, 2, 3, 4])
def test_invert_and_compose(oracle, t):
    """invert_and_compose(p, dp) (c_image_transform.h:159-167, 309-317, 372-377; .cc:737-833):
    translation / euclidean compose exactly W(p) o W(dp)^-1; affine / homography use the
    reference's first-order form inv(inv(M(p)) + M(dp)). dp = 0 returns p."""
    O = oracle
    rng = np.random.default_rng(20 + t)
    m, s = rand_state(O, rng, t)
    n = O.nparams(m)
    out = O.invert_and_compose(m, s, np.zeros(n))
    X0, Y0 = O.warp(m, s, 12.0, 34.0)
    X1, Y1 = O.warp(m, out, 12.0, 34.0)
    assert X1 == pytest.approx(X0, abs=1e-7) and Y1 == pytest.approx(Y0, abs=1e-7)
    dp = rng.normal(0, 1e-3, size=n)
    if t in (0, 1, 2):
        dp[:2] *= 1000
    out = O.invert_and_compose(m, s, dp)
    if t in (0, 1, 2):
        mid = O.identity(m)
        sinc = O.set_params(m, mid, O.get_params(m, mid) + dp if t else dp)
        for (x, y) in [(5.0, 7.0), (200.0, 150.0)]:
            xi, yi = O.warp(m, sinc, x, y)
            Xa, Ya = O.warp(m, out, xi, yi)
            Xb, Yb = O.warp(m, s, x, y)
            assert Xa == pytest.approx(Xb, abs=1e-6) and Ya == pytest.approx(Yb, abs=1e-6)
    else:
        Mp = synth.homography_from_state(t, s)
        D = np.zeros((3, 3))
        D.flat[:n] = dp
        R = np.linalg.inv(np.linalg.inv(Mp) + D)
        if t == 4:
            R = R / R[2, 2]
        assert np.allclose(R.flat[:n], out[:n], rtol=1e-9, atol=1e-12)


def test_euclidean_fixed_scale_eps_quirk(oracle):
    """eps() of EUCLIDEAN (fixed scale) includes max(W,H)*scale: it never drops below max(W,H)."""
    O = oracle
    m = O.model(O.EUCLIDEAN)
    s = O.identity(m)
    e = O.eps(m, s, np.zeros(3), 640, 480)
    assert e == pytest.approx(640.0)


def test_gaussian_kernel(oracle):
    k = oracle.gaussian_kernel(1.0)
    assert len(k) == 7 and k.sum() == pytest.approx(1.0)
    assert np.allclose(k, k[::-1])
    x = np.arange(7) - 3.0
    ref = np.exp(-x * x / 2)
    assert np.allclose(k, ref / ref.sum())
    assert len(oracle.gaussian_kernel(0.2)) == 3


def test_pyrdown_semantics(oracle):
    rng = np.random.default_rng(0)
    img = rng.random((37, 50))
    d = oracle.pyrdown(img)
    assert d.shape == (18, 24)   # ((w+1)>>1)&~1
    k = np.array([1, 4, 6, 4, 1]) / 16.0

    def refl(p, n):
        while p < 0 or p >= n:
            p = -p if p < 0 else 2 * (n - 1) - p
        return p
    for (y, x) in [(0, 0), (5, 7), (17, 23)]:
        v = sum(k[i] * k[j] * img[refl(2 * y + j - 2, 37), refl(2 * x + i - 2, 50)] for i in range(5) for j in range(5))
        assert d[y, x] == pytest.approx(v, abs=1e-12)
    assert np.allclose(oracle.pyrdown(np.full((16, 16), 3.5)), 3.5)


def test_differentiate_linear_ramp(oracle):
    y, x = np.mgrid[0:20, 0:30].astype(float)
    gx, gy = oracle.differentiate(2.0 * x - 3.0 * y + 1.0)
    assert np.allclose(gx[:, 2:-2], 2.0) and np.allclose(gy[2:-2, :], -3.0)
    valid = np.ones((20, 30), np.uint8)
    valid[5, 6] = 0
    gx, gy = oracle.differentiate(2.0 * x, valid)
    assert gx[5, 6] == 0 and gy[5, 6] == 0


def test_bilinear_and_borders(oracle):
    img = np.arange(12, dtype=float).reshape(3, 4)
    lib = oracle.lib()
    a = img.ctypes.data
    assert lib.orc_sample_bilinear(a, 4, 3, 1.5, 1.0, oracle.BORDER_REPLICATE, 0) == pytest.approx(5.5)
    assert lib.orc_sample_bilinear(a, 4, 3, -1.0, 0.0, oracle.BORDER_REPLICATE, 0) == 0.0
    assert lib.orc_sample_bilinear(a, 4, 3, -1.0, 0.0, oracle.BORDER_REFLECT101, 0) == 1.0
    assert lib.orc_sample_bilinear(a, 4, 3, 4.0, 0.0, oracle.BORDER_REFLECT101, 0) == 2.0
    assert lib.orc_sample_bilinear(a, 4, 3, -0.5, 0.0, oracle.BORDER_CONSTANT, 0) == pytest.approx(0.0)


def test_erode5(oracle):
    m = np.full((12, 12), 255, np.uint8)
    m[6, 6] = 0
    e = oracle.erode5(m)
    assert (e[4:9, 4:9] == 0).all() and e[3, 6] == 255 and e[0, 0] == 255


@pytest.mark.parametrize("method", [0, 1, 2, 3])
def test_align_recovers_known_translation(oracle, method):
    """Every ECC method recovers an exactly-rendered sub-pixel shift."""
    O = oracle
    sc = synth.Scene(160, 120, 45.0, edge_sigma=2.0)
    ref = synth.reference_np(sc)
    H = np.array([[1, 0, 2.3], [0, 1, -1.7], [0, 0, 1.0]])
    cur = synth.render_frame_np(sc, H)
    m = O.model(O.AFFINE)
    ok, s, it, e = O.ecc_align(m, O.identity(m), ref, cur, method=method, max_iterations=60, max_eps=1e-3)
    assert ok
    assert s[2] == pytest.approx(2.3, abs=0.01) and s[5] == pytest.approx(-1.7, abs=0.01)


def test_identity_warp_first_update_is_zero(oracle):
    O = oracle
    sc = synth.Scene(96, 80, 30.0)
    ref = synth.reference_np(sc)
    m = O.model(O.AFFINE)
    ok, s, it, e = O.ecc_align(m, O.identity(m), ref, ref.copy(), method=O.IC, max_iterations=1, max_eps=1e-9)
    assert np.allclose(s[:6], O.identity(m)[:6], atol=1e-9)


def test_ecch_pyramid_homography(oracle):
    O = oracle
    sc = synth.Scene(256, 192, 70.0)
    ref = synth.reference_np(sc)
    Hs = np.array([[1.002, 0.004, 5.2], [-0.003, 0.998, -3.1], [1e-6, -2e-6, 1.0]])
    cur = synth.render_frame_np(sc, Hs)
    o = O.ecch_opts(method=O.IC, maxlevel=3, epsx=1e-3)
    m = O.model(O.HOMOGRAPHY)
    s, it, e = O.ecch_align(m, O.identity(m), ref, cur, o)
    mx, my = O.warp_grid(m, s, 256, 192)
    y, x = np.mgrid[0:192, 0:256].astype(float)
    w = Hs[2, 0] * x + Hs[2, 1] * y + 1
    tx = (Hs[0, 0] * x + Hs[0, 1] * y + Hs[0, 2]) / w
    ty = (Hs[1, 0] * x + Hs[1, 1] * y + Hs[1, 2]) / w
    rms = math.sqrt(np.mean((mx - tx) ** 2 + (my - ty) ** 2))
    assert rms < 0.05   # bilinear-interpolation bias of ECC on a 2 px edge; not a parity bound


def test_correlation_of_identical_images(oracle):
    O = oracle
    sc = synth.Scene(96, 80, 30.0)
    ref = synth.reference_np(sc)
    m = O.model(O.AFFINE)
    assert O.correlation(m, O.identity(m), ref, ref) == pytest.approx(1.0, abs=1e-12)


def test_extract_bayer_planes_matches_slicing(oracle):
    rng = np.random.default_rng(3)
    raw = rng.integers(0, 4096, size=(20, 30), dtype=np.uint16)
    planes = oracle.extract_bayer_planes(raw)
    assert np.array_equal(planes[..., 0], raw[0::2, 0::2])
    assert np.array_equal(planes[..., 1], raw[0::2, 1::2])
    assert np.array_equal(planes[..., 2], raw[1::2, 0::2])
    assert np.array_equal(planes[..., 3], raw[1::2, 1::2])
    avg = oracle.average_bayer_planes(raw)
    s = raw[0::2, 0::2].astype(int) + raw[0::2, 1::2] + raw[1::2, 0::2] + raw[1::2, 1::2]
    assert np.array_equal(avg, ((2 + s) // 4).astype(np.uint16))


def test_bayer_pattern_mask(oracle):
    m = oracle.bayer_pattern_mask(8, 4, 4)   # RGGB: R=2, G=1, B=0
    assert m[0, 0] == 2 and m[0, 1] == 1 and m[1, 0] == 1 and m[1, 1] == 0
    cells = {9: [[1, 2], [0, 1]], 10: [[1, 0], [2, 1]], 11: [[0, 1], [1, 2]]}   # GRBG, GBRG, BGGR
    for cid, q in cells.items():
        assert np.array_equal(oracle.bayer_pattern_mask(cid, 2, 2), np.array(q, np.uint8))
    # odd sizes: the pattern continues by parity into the last row / column
    m = oracle.bayer_pattern_mask(8, 5, 3)
    assert np.array_equal(m, np.tile(np.array([[2, 1], [1, 0]], np.uint8), (2, 3))[:3, :5])


def test_bayer_accumulate_constant_channels(oracle):
    """Each raw sample lands in its own cell's channel, so a mosaic with one
    constant per channel averages to those constants under any warp."""
    h, w = 40, 50
    pat = oracle.bayer_pattern_mask(8, w, h)
    raw = np.choose(pat, [300.0, 200.0, 100.0])          # B, G, R
    acc = np.zeros((h, w, 3))
    cntr = np.zeros((h, w, 3))
    m = oracle.model(oracle.AFFINE)
    st = oracle.set_params(m, oracle.identity(m), [1.01, 0.02, 3.3, -0.01, 0.99, -2.7])
    mx, my = oracle.warp_grid(m, st, w, h)
    oracle.bayer_accumulate(raw, mx, my, pat, None, acc, cntr)
    sel = cntr > 1e-9
    assert sel.mean() > 0.5
    avg = np.where(sel, acc / np.where(sel, cntr, 1), 0)
    for ch, v in ((0, 300.0), (1, 200.0), (2, 100.0)):
        assert np.allclose(avg[..., ch][sel[..., ch]], v, rtol=1e-12)
    # the four bilinear weights of a gathered pixel sum to 1 across channels
    inside = cntr.sum(axis=2) > 0
    assert np.allclose(cntr.sum(axis=2)[inside], 1.0, atol=1e-12)


def test_bayer_accumulate_truncates_toward_zero(oracle):
    """(int) p truncates: a position in (-1, 0) gathers from column 0 with a
    negative right-hand weight, as the reference's interpolate lambda does."""
    h, w = 4, 4
    pat = oracle.bayer_pattern_mask(8, w, h)
    raw = np.arange(16, dtype=np.float64).reshape(h, w)
    mx = np.full((h, w), -0.25)
    my = np.full((h, w), 1.0)
    acc = np.zeros((h, w, 3))
    cntr = np.zeros((h, w, 3))
    oracle.bayer_accumulate(raw, mx, my, pat, None, acc, cntr)
    # sx = 0, ax = 1.25, bx = -0.25; sy = 1, ay = 1, by = 0: row 1 holds G (x=0) and B (x=1)
    assert np.allclose(cntr[0, 0], [-0.25, 1.25, 0.0])
    assert np.allclose(acc[0, 0], [-0.25 * raw[1, 1], 1.25 * raw[1, 0], 0.0])


def test_running_mean_equals_weighted_sum(oracle):
    """The reference's running mean A += (I - A) w / W equals sum(w I) / sum(w)."""
    rng = np.random.default_rng(4)
    h, w, n = 8, 9, 50
    acc32 = np.zeros((h, w), np.float32)
    accw32 = np.zeros((h, w), np.float32)
    acc = np.zeros((h, w))
    accw = np.zeros((h, w))
    lib = oracle.lib()
    for _ in range(n):
        img = rng.random((h, w)).astype(np.float32)
        wt = (rng.random((h, w)) * (rng.random((h, w)) > 0.2)).astype(np.float32)
        lib.orc_running_mean_add_f32(acc32.ctypes.data, accw32.ctypes.data, w, h, img.ctypes.data, wt.ctypes.data)
        img64, wt64 = img.astype(float), wt.astype(float)
        oracle.lib().orc_weighted_average_add(acc.ctypes.data, accw.ctypes.data, w, h, img64.ctypes.data,
                                              wt64.ctypes.data)
    ok = accw > 0
    assert np.allclose(acc32[ok], (acc / np.where(ok, accw, 1))[ok], rtol=1e-5)


def test_stack_remap_mask_is_eroded(oracle):
    O = oracle
    img = np.ones((40, 50))
    m = O.model(O.TRANSLATION)
    s = O.identity(m)
    s[0], s[1] = 3.25, 0.0
    dst, msk = O.stack_remap(m, s, img, 50, 40)
    # both taps inside needs x + 4 <= 49 -> x <= 45; the 5x5 erosion removes 2 more columns
    assert msk[20, 43] == 255 and msk[20, 44] == 0
    assert msk[20, 0] == 255


# ----------------------------------------------------------------- c_eccflow

def test_resize_area_integer_factor_is_block_mean(oracle):
    rng = np.random.default_rng(21)
    img = rng.uniform(0, 1, size=(32, 48))
    out = oracle.resize_area(img, 12, 8)
    assert np.allclose(out, img.reshape(8, 4, 12, 4).mean(axis=(1, 3)), atol=1e-12)


def test_resize_area_fractional_preserves_constants_and_mean(oracle):
    img = np.full((37, 53), 3.25)
    assert np.allclose(oracle.resize_area(img, 20, 14), 3.25, atol=1e-12)
    ramp = np.add.outer(np.arange(37.0), np.arange(53.0))
    out = oracle.resize_area(ramp, 40, 28)       # scale 1.325: partial cells on both ends
    assert abs(out.mean() - ramp.mean()) < 0.05


def _keys(t, a=-0.75):
    t = abs(t)
    if t <= 1:
        return (a + 2) * t ** 3 - (a + 3) * t ** 2 + 1
    if t < 2:
        return a * t ** 3 - 5 * a * t ** 2 + 8 * a * t - 4 * a
    return 0.0


def test_resize_cubic_matches_the_keys_kernel(oracle):
    """INTER_CUBIC: Keys convolution (a = -0.75) at (x + 0.5) s - 0.5, taps clamped"""
    rng = np.random.default_rng(8)
    img = rng.uniform(0, 1, size=(9, 11))
    out = oracle.resize_cubic(img, 17, 13)
    sx, sy = 11 / 17, 9 / 13

    def axis(n_src, d, s):
        f = (d + 0.5) * s - 0.5
        i0 = int(np.floor(f))
        return [(min(max(i0 - 1 + k, 0), n_src - 1), _keys(f - (i0 - 1 + k))) for k in range(4)]

    for dy in range(13):
        for dx in range(17):
            v = sum(wy * wx * img[iy, ix] for iy, wy in axis(9, dy, sy) for ix, wx in axis(11, dx, sx))
            assert abs(out[dy, dx] - v) < 1e-12
    assert np.allclose(oracle.resize_cubic(np.full((9, 11), 2.5), 17, 13), 2.5, atol=1e-12)


def test_eccflow_levels_follow_the_reference_rule(oracle):
    o = oracle.flow_opts(scale_factor=0.75, support_scale=4, min_image_size=-1)
    lv = oracle.eccflow_levels(100, 80, o)
    assert lv[0] == (100, 80)
    for (pw, ph), (nw, nh) in zip(lv, lv[1:]):
        assert (nw, nh) == (int((pw + 1) * 0.75), int((ph + 1) * 0.75))
    assert max(lv[-1]) > 4
    nw, nh = int((lv[-1][0] + 1) * 0.75), int((lv[-1][1] + 1) * 0.75)
    assert max(nw, nh) <= 4                      # the next level would be at or below the minimum
    assert len(oracle.eccflow_levels(100, 80, oracle.flow_opts(max_pyramid_level=2))) == 3


def _textured(w, h, dx=0.0, dy=0.0):
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    X, Y = x - dx, y - dy
    return (10 + 4 * np.sin(2 * np.pi * X / 17.0) * np.cos(2 * np.pi * Y / 13.0) + 3 * np.sin(2 * np.pi * (X + Y) / 23.0))


def test_eccflow_identical_images_give_zero_flow(oracle):
    img = _textured(96, 64)
    flow = oracle.eccflow(oracle.flow_opts(scale_factor=0.75, support_scale=3, max_iterations=2), img, img)
    assert np.abs(flow).max() < 1e-9


def test_eccflow_recovers_a_translation(oracle):
    """current(x) = reference(x - d): the flow (rmap - x) is +d where the
    warped current matches the reference"""
    ref = _textured(128, 96)
    cur = _textured(128, 96, dx=1.2, dy=-0.7)
    o = oracle.flow_opts(scale_factor=0.5, support_scale=3, max_iterations=3)
    flow = oracle.eccflow(o, ref, cur)
    inner = flow[16:-16, 16:-16]
    assert abs(np.median(inner[..., 0]) - 1.2) < 0.1
    assert abs(np.median(inner[..., 1]) + 0.7) < 0.1


def test_warp_residual_gradients_match_finite_differences(oracle):
    """Exact gradients of the bilinear warp residual vs central differences.
    The bilinear interpolant has kinks on the pixel grid, so the parameters are
    generic (no sample lands exactly on a grid line) and the tolerance covers
    the samples that cross a grid line within the step: 1e-3 relative at
    h = 1e-6, 5e-3 relative at the h = 1e-3 of the adjoint checks."""
    rng = np.random.default_rng(5)
    h, w = 40, 50
    img = _textured(w, h) + rng.normal(0, 0.1, size=(h, w))
    tmpl = _textured(w, h, 0.6, -0.3)
    m = oracle.model(oracle.AFFINE)
    p0 = np.array([1.0103217, 0.0201387, 0.4137113, -0.0103911, 0.9903187, -0.2171393])
    st = oracle.set_params(m, oracle.identity(m), p0)
    L, gp, gt, gu = oracle.warp_residual(m, st, img, tmpl)
    for h_fd, tol in ((1e-6, 1e-3), (1e-3, 5e-3)):
        for k in range(6):
            pp, pm = p0.copy(), p0.copy()
            pp[k] += h_fd
            pm[k] -= h_fd
            Lp = oracle.warp_residual(m, oracle.set_params(m, oracle.identity(m), pp), img, tmpl)[0]
            Lm = oracle.warp_residual(m, oracle.set_params(m, oracle.identity(m), pm), img, tmpl)[0]
            fd = (Lp - Lm) / (2 * h_fd)
            assert abs(fd - gp[k]) <= tol * abs(gp[k]), (h_fd, k, fd, gp[k])
    # template gradient: dL/dT = -r (L is quadratic in T: central differences are exact)
    t2, t3 = tmpl.copy(), tmpl.copy()
    t2[7, 9] += 1e-3
    t3[7, 9] -= 1e-3
    fd_t = (oracle.warp_residual(m, st, img, t2)[0] - oracle.warp_residual(m, st, img, t3)[0]) / 2e-3
    assert abs(fd_t - gt[7, 9]) < 1e-6


def test_focus_weights_known_answers(oracle):
    m = oracle.model(oracle.TRANSLATION)
    st = oracle.identity(m)
    flat = np.full((30, 40), 7.0)
    assert np.abs(oracle.focus_weights(m, st, flat, 40, 30)).max() < 1e-20     # no structure, no weight
    y, x = np.mgrid[0:30, 0:40].astype(np.float64)
    ramp = 0.5 * x                                  # |grad| = 0.5, lap = 0 away from the borders
    wgt = oracle.focus_weights(m, st, ramp, 40, 30)
    assert abs(wgt[15, 20] - 0.25 ** 2) < 1e-12
    quad = 0.25 * x * x                             # lap = 0.5, grad = (0.5 x, 0)
    e = (6 * 0.25 + (0.5 * x) ** 2) ** 2
    raw = oracle.focus_weights(m, st, quad, 40, 30)
    k = oracle.gaussian_kernel(3.0)
    assert len(k) == 19
    assert abs(raw[15, 20] - sum(k[i] * e[15, 20 + i - 9] for i in range(19))) < 1e-6 * raw[15, 20]


def test_resize_linear_known_answers(oracle):
    # cv::resize INTER_LINEAR of [0, 1] to 4: f = (d + 0.5) / 2 - 0.5, clamped at both ends
    out = oracle.resize_linear(np.array([[0.0, 1.0]]), 4, 1)
    assert np.allclose(out, [[0.0, 0.25, 0.75, 1.0]], atol=1e-15)
    img = np.arange(12.0).reshape(3, 4)
    assert np.array_equal(oracle.resize_linear(img, 4, 3), img)           # equal sizes copy
    # linear data stays linear away from the clamped ends
    ramp = np.tile(np.arange(8.0), (2, 1))
    up = oracle.resize_linear(ramp, 16, 2)
    assert np.allclose(up[0, 1:15], (np.arange(1, 15) + 0.5) / 2 - 0.5, atol=1e-12)


def test_local_variance_map_sizes_follow_the_reference(oracle):
    assert oracle.local_variance_size(1280, 960, 1, 3) == (1280, 960)    # upscaled back to the frame
    assert oracle.local_variance_size(1280, 960, 0, 0) == (1280, 960)
    assert oracle.local_variance_size(1280, 960, 0, 3) == (160, 120)     # the reference keeps the reduced map
    assert oracle.local_variance_size(16, 10, 0, 3) == (8, 5)            # dscaleSize stops before a side < 4
    assert oracle.local_variance_size(3, 9, 2, 0) == (3, 9)              # pdownscale keeps images below 4


def test_local_variance_map_known_answers(oracle):
    # no structure: no map and Q = 0
    m, q = oracle.local_variance_map(np.full((30, 40), 3.0))
    assert m is None and q == 0.0
    # vertical step a -> b at x = 20, radius 2: G = |b - a| on columns 18..21, 0 elsewhere
    a, b, ds = 0.25, 0.75, 20.0
    img = np.full((30, 40), a)
    img[:, 20:] = b
    m, q = oracle.local_variance_map(img, kradius=2, dscale=0, uscale=0, depth_scale=ds)
    d3 = (ds * (b - a)) ** 3
    assert abs(q - d3) < 1e-12 * d3                          # Q = ds^3 sum G^4 / sum G
    want = np.full((30, 40), 0.05 * d3)
    want[:, 18:22] += d3
    assert np.allclose(m, want, rtol=1e-14, atol=0)
    # radius 0 acts as 1: columns 19..20
    m1, _ = oracle.local_variance_map(img, kradius=0, dscale=0, uscale=0, depth_scale=ds)
    assert np.allclose(m1[0, 18:22], [0.05 * d3, 1.05 * d3, 1.05 * d3, 0.05 * d3])


def test_local_variance_map_is_scale_invariant_and_area_reduced(oracle):
    rng = np.random.default_rng(7)
    img = rng.random((96, 128))
    m1, q1 = oracle.local_variance_map(img)
    m2, q2 = oracle.local_variance_map(img * 7.0, depth_scale=20.0 / 7.0)
    assert m1.shape == (96, 128)
    assert abs(q1 - q2) < 1e-12 * q1 and np.abs(m1 - m2).max() < 1e-12 * m1.max()
    # dscale 0, uscale 1: the reference returns the INTER_AREA-halved map + 0.05 Q
    m3, q3 = oracle.local_variance_map(img, kradius=1, dscale=0, uscale=1, depth_scale=1.0)
    assert m3.shape == (48, 64)
    p = np.pad(img, 1, mode="edge")
    win = np.lib.stride_tricks.sliding_window_view(p, (3, 3))
    g = win.max(axis=(2, 3)) - win.min(axis=(2, 3))
    assert abs(q3 - (g ** 4).sum() / g.sum()) < 1e-12 * q3
    want = (g ** 3).reshape(48, 2, 64, 2).mean(axis=(1, 3)) + 0.05 * q3
    assert np.abs(m3 - want).max() < 1e-12 * want.max()


def test_average_pyramid_inpaint_known_answers(oracle):
    rng = np.random.default_rng(3)
    img = rng.random((24, 20))
    full = np.full((24, 20), 255, np.uint8)
    out, om = oracle.average_pyramid_inpaint(img, full)
    assert np.array_equal(out, img) and np.array_equal(om, full)            # nothing to fill: a copy
    # nothing to fill from: zeros, yet every pixel comes back valid, since
    # upject_even marks each copied position valid whether or not its value was
    out, om = oracle.average_pyramid_inpaint(img, np.zeros_like(full))
    assert not out.any() and om.min() == 255
    # a 3 x 3 image with its centre missing: the centre becomes the mean of its 8 neighbours
    s = np.arange(9.0).reshape(3, 3) ** 2
    m = np.full((3, 3), 255, np.uint8)
    m[1, 1] = 0
    out, om = oracle.average_pyramid_inpaint(s, m)
    assert abs(out[1, 1] - (s.sum() - s[1, 1]) / 8) < 1e-12 and om.min() == 255
    assert np.array_equal(np.delete(out.ravel(), 4), np.delete(s.ravel(), 4))
    # a constant image keeps its value over a large hole; a linear ramp over a one-pixel hole
    c = np.full((40, 33), 2.5)
    m = np.full((40, 33), 255, np.uint8)
    m[5:30, 3:25] = 0
    out, om = oracle.average_pyramid_inpaint(c, m)
    assert np.abs(out - 2.5).max() < 1e-12 and om.min() == 255
    y, x = np.mgrid[0:17, 0:19].astype(np.float64)
    ramp = 0.5 * x - 0.25 * y
    m = np.full((17, 19), 255, np.uint8)
    m[8, 9] = 0
    out, _ = oracle.average_pyramid_inpaint(ramp, m)
    assert abs(out[8, 9] - ramp[8, 9]) < 1e-12
    # no pyramid levels: the holes stay empty
    out, om = oracle.average_pyramid_inpaint(ramp, m, max_levels=0)
    assert out[8, 9] == 0 and om[8, 9] == 0 and om.sum() == 255 * (17 * 19 - 1)


def test_stack_error_report_separates_arithmetic_from_registration(oracle):
    """The checker of the end-to-end stack comparisons: a stack built in FP64
    from transforms moved by a few thousandths of a pixel has no arithmetic
    error against its own transforms, an end-to-end error well above 1e-5 at
    the disk's rim, and that error stays inside the registration bound."""
    from serstacker_gb300 import synth
    O = oracle
    w, h, n = 128, 96, 3
    sc = synth.Scene(w, h, 30.0)
    frames, _, _ = synth.make_sequence_np(sc, n, seed=5, kind="config1", dtype=np.uint16, gain=64.0,
                                          blur_range=(0.8, 2.0))
    scale = 1.0 / 65535.0
    ref = synth.reference_np(sc) * 64.0 * scale
    po = O.pipeline_opts(passes=(O.AFFINE, O.HOMOGRAPHY), method=O.IC, maxlevel=2, max_iterations=30, epsx=0.01,
                         min_rho=0.0, minimum_image_size=16)
    states, status, rho, S, W = O.register_and_stack(po, ref, frames, scale)
    m = O.model(O.HOMOGRAPHY)
    params = np.zeros((n, 12), np.float32)
    weights = np.zeros(n, np.float32)
    S2 = np.zeros((h, w))
    W2 = np.zeros((h, w))
    for i in range(n):
        p = O.get_params(m, states[i]).copy()
        p[2] += 0.003 * (i + 1)
        p[5] -= 0.002
        params[i, :8] = p
        img = frames[i].astype(np.float64) * scale
        weights[i] = O.laplacian_energy(O.pyrdown(O.smooth(img, 1.0)))
        st = O.set_params(m, O.identity(m), params[i, :8].astype(np.float64))
        dst, msk = O.stack_remap(m, st, img, w, h)
        wt = np.where(msk > 0, float(weights[i]), 0.0)
        S2 += wt * dst
        W2 += wt
    avg = np.where(W2 > 0, S2 / np.where(W2 > 0, W2, 1), 0).astype(np.float32)
    rep = O.stack_error_report(frames, scale, O.HOMOGRAPHY, params, status, weights, avg, states, status, S, W)
    assert rep["arith_max"] < 1e-6, rep
    assert rep["e2e_max"] > 1e-5, rep
    assert rep["e2e_bound_frac"] <= 1.0, rep
    assert 0.005 < rep["warp_disp_max"] < 0.02, rep


def test_pyrup_known_answers(oracle):
    """cv::pyrUp: zero insertion + 4 x [1 4 6 4 1] / 16, BORDER_REFLECT_101 on the
    2w grid, a 2w - 1 destination keeps the first 2w - 1 samples."""
    O = oracle
    assert np.allclose(O.pyrup(np.full((5, 7), 3.25), 14, 10), 3.25)
    assert np.allclose(O.pyrup(np.full((5, 7), 3.25), 13, 9), 3.25)
    s = np.zeros((1, 8))
    s[0, 3] = 1.0
    up = O.pyrup(np.repeat(s, 4, axis=0), 16, 8)[3]
    assert np.allclose(up[4:9], [1 / 8, 1 / 2, 6 / 8, 1 / 2, 1 / 8]) and np.allclose(up[:4], 0) and np.allclose(up[9:], 0)
    r = np.arange(1.0, 9.0)[None].repeat(4, axis=0)          # right edge: reflect on the 2w grid
    up = O.pyrup(r, 16, 8)[0]
    assert np.isclose(up[14], (7 + 7 * 8) / 8) and np.isclose(up[15], 8.0)
    assert np.isclose(up[0], (2 + 6 * 1 + 2) / 8)
    up_odd = O.pyrup(r, 15, 8)[0]
    assert np.allclose(up_odd, up[:15])
    ramp = np.add.outer(np.arange(6.0) * 0.5, np.arange(9.0) * 2.0)
    assert np.allclose(O.pyrup(ramp, 18, 12)[2:-2, 2:-2],
                       np.add.outer(np.arange(12.0) * 0.25, np.arange(18.0))[2:-2, 2:-2])


def test_pyrdown_border_and_mask_threshold(oracle):
    O = oracle
    a = np.arange(30, dtype=np.float64).reshape(5, 6)
    rep = O.pyrdown_border(a, O.BORDER_REPLICATE)
    r101 = O.pyrdown_border(a, O.BORDER_REFLECT101)
    assert rep.shape == (3, 3) and r101.shape == (3, 3)
    k = np.array([1, 4, 6, 4, 1]) / 16.0

    def ref(border):
        idx = lambda p, n: (min(max(p, 0), n - 1) if border == O.BORDER_REPLICATE else
                            (abs(p) if p < 0 else (2 * (n - 1) - p if p >= n else p)))
        out = np.zeros((3, 3))
        for y in range(3):
            for x in range(3):
                out[y, x] = sum(k[j] * k[i] * a[idx(2 * y + j - 2, 5), idx(2 * x + i - 2, 6)]
                                for j in range(5) for i in range(5))
        return out
    assert np.allclose(rep, ref(O.BORDER_REPLICATE)) and np.allclose(r101, ref(O.BORDER_REFLECT101))
    # u8 pyrDown ((sum + 128) >> 8) then >= 250: one zero pixel under a tap of weight
    # 1 or 4 keeps the output, weight 6 or more clears it
    for (j, i), keep in [((0, 0), True), ((0, 1), True), ((0, 2), False), ((1, 1), False), ((2, 2), False)]:
        m = np.full((12, 12), 255, np.uint8)
        m[4 + j - 2, 4 + i - 2] = 0       # tap (j, i) of output (2, 2), weight k_j k_i of 1 4 6 4 1
        out = O.mask_pyrdown_ge250(m)
        assert (out[2, 2] == 255) == keep, (j, i)
        assert (out == 0).sum() <= 5


def test_ecc_normalize_known_answers(oracle):
    """ecc_normalize removes the pyramid background: zero on constant images,
    zero on linear ramps away from the border, zero outside the mask."""
    O = oracle
    assert np.allclose(O.ecc_normalize(np.full((40, 56), 7.0), 2), 0)
    ramp = np.add.outer(np.arange(48.0) * 0.3, np.arange(64.0) * 0.7)
    nz = O.ecc_normalize(ramp, 2)
    assert np.abs(nz[12:-12, 12:-12]).max() < 1e-12
    rng = np.random.default_rng(3)
    img = rng.random((33, 47))
    mask = (rng.random((33, 47)) > 0.2).astype(np.uint8) * 255
    out = O.ecc_normalize(img, 1, mask)
    assert np.all(out[mask == 0] == 0)
    assert np.allclose(out[mask > 0], (img - O.ecc_normalize(img, 1) * 0 - (img - O.ecc_normalize(img, 1)))[mask > 0])


def test_register_frame_scaled_recovers_warps(oracle):
    """register_frame with the reference's defaults (scale 0.5: registration on
    the pyrDown'ed images, the transform scaled back; eps tightened to 0.01) and
    with translation-first on a 3-level IC pyramid (step 1: the default step
    of 1.5 overshoots) recovers exactly rendered warps; a frame of noise is
    rejected by the correlation gate."""
    from serstacker_gb300 import synth
    O = oracle
    w, h = 192, 144
    sc = synth.Scene(w, h, 45.0, band_period=16.0)
    ref = synth.reference_np(sc)
    m = O.model(O.AFFINE)
    H = np.array([[1.002, -0.004, 2.6], [0.003, 0.999, -1.7], [0, 0, 1.0]])
    cur = synth.render_frame_np(sc, H)
    for kw in (dict(eps=0.01), dict(method=O.IC, ecch_max_level=3, eps=0.01, update_step_scale=1.0),
               dict(method=O.IC, ecch_max_level=3, eps=0.01, update_step_scale=1.0, normalization_scale=2, scale=1.0)):
        o = O.registration_opts(**kw)
        status, st, rho, it = O.register_frame(o, ref, cur)
        assert status == 0 and rho > 0.99, (kw, status, rho)
        gx, gy = O.warp_grid(m, st, w, h)
        yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
        tx = H[0, 0] * xx + H[0, 1] * yy + H[0, 2]
        ty = H[1, 0] * xx + H[1, 1] * yy + H[1, 2]
        rms = np.sqrt(np.mean((gx - tx) ** 2 + (gy - ty) ** 2))
        assert rms < 0.02, (kw, rms)
    noise = np.random.default_rng(4).random((h, w)) * 200
    status, _, rho, _ = O.register_frame(O.registration_opts(method=O.IC, ecch_max_level=3), ref, noise)
    assert status == 3 and rho < 0.6


def test_fp32_baseline_restatement_matches_oracle(oracle):
    """The timed CPU baseline (oracle/sst_refcpu.cc: FP32 images, the
    reference's sequence of full-image passes, FP32 running mean) registers
    like the FP64 oracle (0.02 px) and stacks within FP32 running-mean error."""
    from serstacker_gb300 import synth
    O = oracle
    w, h, n = 192, 144, 3
    sc = synth.Scene(w, h, 0.28 * min(w, h))
    frames, _, _ = synth.make_sequence_np(sc, n, seed=12, kind="config1", dtype=np.uint16, gain=64.0,
                                          blur_range=(0.8, 2.0))
    scale = 1.0 / 65535.0
    ref = synth.reference_np(sc) * 64.0 * scale
    po = O.pipeline_opts(passes=(O.AFFINE, O.HOMOGRAPHY), method=O.IC, maxlevel=3, max_iterations=40, epsx=0.01,
                         min_rho=0.5, minimum_image_size=16)
    st_o, s_o, r_o, S, W = O.register_and_stack(po, ref, frames, scale)
    st_r, s_r, r_r, A, Wr = O.refcpu_register_and_stack(po, ref, frames, scale)
    assert np.array_equal(s_o, s_r)
    m = O.model(O.HOMOGRAPHY)
    for i in range(n):
        xa, ya = O.warp_grid(m, st_o[i], w, h)
        xb, yb = O.warp_grid(m, st_r[i], w, h)
        assert np.sqrt(((xa - xb) ** 2 + (ya - yb) ** 2).mean()) < 0.02
        assert abs(r_o[i] - r_r[i]) < 1e-4
    assert ((W > 0) == (Wr > 0)).mean() > 0.995
    both = (W > 0) & (Wr > 0)
    rel = O.stack_rel_err(A[both], S[both] / W[both])
    assert np.median(rel) < 1e-4


def test_eccflow_masks_known_answers(oracle):
    """c_eccflow masks: an all-valid reference mask changes nothing; an empty
    one stops every update (the flow stays at its start); half a reference
    mask changes the flow."""
    O = oracle
    rng = np.random.default_rng(2)
    h, w = 64, 80
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    ref = 10 + 4 * np.sin(x / 3.1) * np.cos(y / 2.3) + np.sin((x + y) / 5.0)
    cur = 10 + 4 * np.sin((x - 0.6) / 3.1) * np.cos((y + 0.4) / 2.3) + np.sin((x + y - 0.2) / 5.0)
    o = O.flow_opts(support_scale=2, max_iterations=2, scale_factor=0.5, min_image_size=8)
    base = O.eccflow(o, ref, cur)
    assert np.array_equal(O.eccflow(o, ref, cur, ref_mask=np.full((h, w), 255, np.uint8)), base)
    assert np.array_equal(O.eccflow(o, ref, cur, ref_mask=np.zeros((h, w), np.uint8)), np.zeros((h, w, 2)))
    init = np.stack([np.full((h, w), 0.3), np.full((h, w), -0.2)], axis=-1)
    assert np.allclose(O.eccflow(o, ref, cur, init_flow=init, ref_mask=np.zeros((h, w), np.uint8)), init)
    # an all-valid current mask still drops samples whose nearest source pixel lies
    # outside the frame: the flow changes, but only from the border inwards
    full = O.eccflow(o, ref, cur, cur_mask=np.full((h, w), 255, np.uint8))
    assert np.abs(full - base).max() > 0
    m = np.full((h, w), 255, np.uint8)
    m[:, : w // 2] = 0
    half = O.eccflow(o, ref, cur, ref_mask=m)
    assert np.abs(half - base).max() > 1e-3


def test_lpg_known_answers(oracle):
    """lpg() (core/proc/lpg.cc:223-291): a flat image gives the map eps
    (1e-9) scaled by (uscale - dscale) and raised to p; a ramp a x has no
    Laplacian and the extended-Sobel gradient 56 a, so with no scaling and
    p = 1 the map is beta (100 / 36)^2 (56 a)^2 + eps everywhere (the edge
    rows and columns copy their inner neighbours)."""
    O = oracle
    m, met = O.lpg(np.full((40, 56), 0.3))
    assert np.allclose(m, (4 * 1e-9) ** 2, rtol=1e-9) and np.isclose(met, (4e-9) ** 2, rtol=1e-9)
    a, k = 0.01, 2.0
    ramp = np.tile(np.arange(56) * a, (40, 1))
    m, met = O.lpg(ramp, k=k, p=1.0, dscale=0, uscale=0)
    want = 1.0 / (k + 1) * (100.0 / 36.0) ** 2 * (56 * a) ** 2 + 1e-9
    assert np.allclose(m, want, rtol=1e-12) and np.isclose(met, want, rtol=1e-12)
    # the map has the image's size for every dscale / uscale, and the metric is its (masked) mean
    img = np.random.default_rng(3).random((100, 140))
    for ds, us in ((0, 0), (1, 3), (2, 6), (3, 3)):
        m, met = O.lpg(img, dscale=ds, uscale=us)
        assert m.shape == img.shape and np.isclose(met, m.mean())
    mask = np.zeros((100, 140), np.uint8)
    mask[20:60, 30:90] = 255
    m, met = O.lpg(img, mask=mask)
    assert np.isclose(met, m[mask > 0].mean())


def test_debayer_nn2_known_answers(oracle):
    """debayer NN2 (core/io/debayer.cc:828-1161) against a direct restatement
    of the reference's per-position formulas on an RGGB mosaic, including the
    reflected first / last rows and columns and the integer rounding; the
    other patterns are the RGGB rule on the mosaic shifted by their cell
    offset."""
    O = oracle
    rng = np.random.default_rng(6)
    h, w = 6, 8
    raw = rng.integers(0, 4096, size=(h, w)).astype(np.uint16)
    out = O.debayer_nn2(raw, 8)
    r = lambda v: 2 * (h - 1) - v if v >= h else abs(v)
    c = lambda v: 2 * (w - 1) - v if v >= w else abs(v)
    s = lambda x, y: int(raw[r(y), c(x)])
    for y in range(h):
        for x in range(w):
            q = (s(x, y - 1) + s(x - 1, y) + s(x + 1, y) + s(x, y + 1) + 2) // 4
            d = (s(x - 1, y - 1) + s(x + 1, y - 1) + s(x - 1, y + 1) + s(x + 1, y + 1) + 2) // 4
            hz = (s(x - 1, y) + s(x + 1, y) + 1) // 2
            vt = (s(x, y - 1) + s(x, y + 1) + 1) // 2
            if y % 2 == 0 and x % 2 == 0:      # R
                want = (d, q, s(x, y))
            elif y % 2 == 0:                   # G in an R row: R horizontal, B vertical
                want = (vt, s(x, y), hz)
            elif x % 2 == 0:                   # G in a B row: B horizontal, R vertical
                want = (hz, s(x, y), vt)
            else:                              # B
                want = (s(x, y), q, d)
            assert tuple(out[y, x]) == want, (x, y, tuple(out[y, x]), want)
    big = rng.integers(0, 4096, size=(12, 16)).astype(np.uint16)
    for cid, (dy, dx) in ((9, (0, 1)), (10, (1, 0)), (11, (1, 1))):
        a = O.debayer_nn2(big, cid)
        b = O.debayer_nn2(big[dy:dy + 10, dx:dx + 14], 8)
        assert np.array_equal(a[dy + 1:dy + 9, dx + 1:dx + 13], b[1:9, 1:13]), cid
    fl = rng.random((6, 8)).astype(np.float32)
    assert np.array_equal(O.debayer_nn2(fl, 8)[..., 2][0::2, 0::2], fl[0::2, 0::2])


def test_optimal_dft_size_known_answers(oracle):
    O = oracle
    for n, m in [(1, 1), (7, 8), (11, 12), (13, 15), (17, 18), (29, 30), (37, 40), (960, 960), (1021, 1024),
                 (1280, 1280), (2049, 2160)]:
        assert O.optimal_dft_size(n) == m, n


def test_fft_average_known_answers(oracle):
    """c_frame_accumulation_with_fft: one frame or identical frames give the
    frame back; two constant frames c, d give (c^7 + d^7) / (c^6 + d^6), the
    DC bins weighted by (|F|^2 / area^2)^3 = c^6 and d^6 (the other bins are
    zero in both)"""
    O = oracle
    rng = np.random.default_rng(3)
    f = rng.random((29, 37))
    assert np.abs(O.fft_average(f[None]) - f).max() < 1e-10
    assert np.abs(O.fft_average(np.stack([f, f, f])) - f).max() < 1e-10
    c, d = 0.6, 0.9
    frames = np.stack([np.full((30, 40), c), np.full((30, 40), d)])
    want = (c ** 7 + d ** 7) / (c ** 6 + d ** 6)
    assert np.abs(O.fft_average(frames) - want).max() < 1e-10
    col = rng.random((2, 17, 23, 3))
    out = O.fft_average(np.stack([col[0], col[0]]))
    assert out.shape == (17, 23, 3) and np.abs(out - col[0]).max() < 1e-10


def test_linear_inpaint_known_answers(oracle):
    """linear_interpolation_inpaint: a run of holes between s and e takes
    sv + (x - s) (ev - sv) / (run length) (the slope over the run length, as
    the reference computes it), a single hole its right / lower neighbour;
    both directions mix as (h dv + v dh) / (dh + dv)"""
    O = oracle
    row = np.array([[1.0, 0.0, 0.0, 4.0]])
    out = O.linear_inpaint(row, np.array([[255, 0, 0, 255]], np.uint8))
    assert np.allclose(out, [[1.0, 2.5, 4.0, 4.0]])
    img = np.arange(9, dtype=np.float64).reshape(3, 3) ** 2
    m = np.full((3, 3), 255, np.uint8)
    m[1, 1] = 0
    out = O.linear_inpaint(img, m)
    assert out[1, 1] == pytest.approx((img[1, 2] + img[2, 1]) / 2)
    # an all-hole row and column: filled in a second sweep from the first one's values
    img = np.random.default_rng(1).random((6, 7))
    m = np.full((6, 7), 255, np.uint8)
    m[2, :] = 0
    m[:, 3] = 0
    out = O.linear_inpaint(img, m)
    assert np.isfinite(out).all()
    assert np.array_equal(out[m > 0], img[m > 0])


def test_focus_stack_known_answers(oracle):
    """c_laplacian_pyramid_focus_stacking: one frame, or identical frames,
    reconstruct the frame (both fusing policies)"""
    O = oracle
    rng = np.random.default_rng(4)
    f = rng.random((70, 90))
    for policy in (0, 1):
        assert np.abs(O.focus_stack(f[None], policy=policy) - f).max() < 1e-10
        assert np.abs(O.focus_stack(np.stack([f, f, f]), policy=policy) - f).max() < 1e-10
    c = rng.random((50, 66, 3))
    for policy in (0, 1):
        assert np.abs(O.focus_stack(np.stack([c, c]), policy=policy) - c).max() < 1e-10


def test_canvas_average_known_answers(oracle):
    """c_canvas_average: the first frame is centred on a 3/2-size canvas; a
    frame without remap lands on the last box; an identity remap places the
    frame at its box; a box within 32 px of the left edge shifts the canvas
    contents 64 px right (when the shifted copy is not empty)"""
    O = oracle
    rng = np.random.default_rng(6)
    n, h, w = 3, 40, 60
    fr = rng.random((n, h, w))
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    rm = np.stack([xx, yy], axis=-1)
    boxes = np.zeros((n, 4), np.int32)
    boxes[2] = (20, 12, w, h)
    acc, W, st, last = O.canvas_average(fr, boxes=boxes, rmaps=[None, None, rm])
    assert acc.shape == (60, 90) and list(st) == [0, 0, 0] and list(last) == [20, 12, w, h]
    # frames 0 and 1 at (15, 10); frame 2 at (20, 12): the 90 x 60 canvas is too
    # small for the 64 px shift in y, so nothing moves
    assert W[10, 15] == 2 and W[12, 20] == 3 and W[51, 79] == 1 and W.sum() == 3 * w * h
    assert acc[10, 15] == pytest.approx((fr[0, 0, 0] + fr[1, 0, 0]) / 2)
    assert acc[51, 79] == pytest.approx(fr[2, 39, 59])
    assert acc[12, 20] == pytest.approx((fr[0, 2, 5] + fr[1, 2, 5] + fr[2, 0, 0]) / 3)
    acc3, W3, st3, last3 = O.canvas_average(fr[:2], boxes=np.array([[0, 0, 0, 0], [10, 50, w, h]], np.int32),
                                            rmaps=[None, rm], canvas=(300, 200))
    assert acc3.shape == (200, 300) and list(st3) == [0, 0] and list(last3) == [74, 50, w, h]
    assert np.all(W3[80:120, 184:244] == 1) and np.all(W3[50:90, 74:134] == 1) and W3.sum() == 2 * w * h
    assert np.allclose(acc3[80:120, 184:244], fr[0]) and np.allclose(acc3[50:90, 74:134], fr[1])


def test_filter_bad_pixels_known_answers(oracle):
    """median_filter_bad_pixels / bayer_denoise: on a flat frame a hot and a
    cold pixel take the window median (the flat value), nothing else moves;
    in a Bayer mosaic only the pixel's own plane counts"""
    O = oracle
    f = np.full((30, 40), 1000, np.uint16)
    f[7, 9], f[20, 31] = 9000, 3
    g = O.filter_bad_pixels(f, 0, 3.0)
    assert g[7, 9] == 1000 and g[20, 31] == 1000 and (g != f).sum() == 2
    # RGGB cells of values 100, 200, 300, 400; a hot pixel in the G1 plane (x odd, y even)
    m = np.zeros((30, 40), np.uint16)
    m[0::2, 0::2], m[0::2, 1::2], m[1::2, 0::2], m[1::2, 1::2] = 100, 200, 300, 400
    m[10, 13] = 5000
    b = O.filter_bad_pixels(m, 8, 3.0)
    assert b[10, 13] == 200 and (b != m).sum() == 1
    # a pixel within k * mad + 1 of the median stays
    n = np.full((30, 40), 1000, np.uint16)
    n[15, 15] = 1001
    assert np.array_equal(O.filter_bad_pixels(n, 0, 3.0), n)
