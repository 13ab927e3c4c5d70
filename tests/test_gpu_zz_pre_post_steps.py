"""The steps on either side of the stacking loop, on the GPU.

Post-stack hole filling (sst_average_pyramid_inpaint) against the FP64
oracle of average_pyramid_inpaint (average_pyramid_inpaint.cc:18-126):
2e-6 of the image's largest magnitude (FP32 3 x 3 means over the pyramid
against FP64), masks exact.

Dark / flat calibration of raw frames (sst_calibrate_frames,
c_image_stacking_pipeline_base.cc:142-183) against the same sequence of
rounded FP32 operations in numpy: bitwise."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _case(h, w, kind, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    img = (1000 + 300 * np.sin(x / 9) * np.cos(y / 13) + rng.standard_normal((h, w))).astype(np.float32)
    if kind == "ring":          # the master frame's uncovered border and a hole in the middle
        r = np.hypot(x - w / 2, y - h / 2)
        mask = ((r < 0.42 * (w + h)) & (r > 30)).astype(np.uint8) * 255
    elif kind == "blobs":
        mask = np.full((h, w), 255, np.uint8)
        mask[20:90, 40:200] = 0
        mask[150:, 300:] = 0
        mask[:, :3] = 0
    elif kind == "sparse":
        mask = (rng.random((h, w)) > 0.97).astype(np.uint8) * 255
    elif kind == "frac":        # mask values other than 0 / 255 weigh the means
        mask = (rng.integers(1, 256, (h, w)) * (rng.random((h, w)) > 0.5)).astype(np.uint8)
    elif kind == "none":
        mask = np.full((h, w), 255, np.uint8)
    elif kind == "empty":
        mask = np.zeros((h, w), np.uint8)
    else:
        mask = (rng.random((h, w)) > 0.5).astype(np.uint8) * 255
    return img, mask


@pytest.mark.parametrize("h,w,kind", [
    (960, 1280, "ring"), (277, 333, "blobs"), (64, 64, "sparse"), (129, 65, "frac"), (300, 200, "none"),
    (33, 47, "empty"), (1, 17, "rand"), (2, 2, "rand"), (5, 1, "rand"), (31, 2, "rand")])
@pytest.mark.parametrize("max_levels", [100, 3, 0])
def test_inpaint_matches_oracle(gpu, oracle, h, w, kind, max_levels):
    img, mask = _case(h, w, kind, seed=h * 7 + w)
    got, gm = gpu.average_pyramid_inpaint(img, mask, max_levels)
    want, wm = oracle.average_pyramid_inpaint(img.astype(np.float64), mask, max_levels)
    assert np.array_equal(gm, wm)
    err = np.abs(got.astype(np.float64) - want).max()
    assert err <= TOL * max(np.abs(want).max(), 1.0), err


def test_inpaint_device_buffers(gpu, oracle):
    import torch
    C = gpu
    img, mask = _case(130, 170, "blobs", 4)
    s = torch.from_numpy(img).cuda()
    m = torch.from_numpy(mask).cuda()
    d = torch.zeros_like(s)
    dm = torch.zeros_like(m)
    C._check(C.lib().sst_average_pyramid_inpaint(s.data_ptr(), 170 * 4, m.data_ptr(), 170, 170, 130, 100,
                                                 d.data_ptr(), 170 * 4, dm.data_ptr(), 170, 1, None), "inpaint")
    torch.cuda.synchronize()
    want, wm = oracle.average_pyramid_inpaint(img.astype(np.float64), mask, 100)
    assert np.array_equal(dm.cpu().numpy(), wm)
    assert np.abs(d.cpu().numpy().astype(np.float64) - want).max() <= TOL * np.abs(want).max()


@pytest.mark.parametrize("dtype,scale", [(np.uint16, 1.0 / 4096), (np.uint8, 1.0 / 256), (np.float32, 1.0)])
@pytest.mark.parametrize("use_dark,use_flat", [(True, True), (True, False), (False, True), (False, False)])
def test_calibration_is_the_reference_sequence_in_fp32(gpu, dtype, scale, use_dark, use_flat):
    import torch
    rng = np.random.default_rng(11)
    n, h, w = 3, 37, 70
    if dtype == np.float32:
        raw = rng.random((n, h, w)).astype(np.float32)
        t = torch.from_numpy(raw).cuda()
    else:
        raw = rng.integers(0, 4096 if dtype == np.uint16 else 256, (n, h, w)).astype(dtype)
        t = torch.from_numpy(raw.view(np.int16) if dtype == np.uint16 else raw).cuda()
    dark = (rng.random((h, w)) * 0.05).astype(np.float32)
    flat = (0.5 + rng.random((h, w))).astype(np.float32)
    out = gpu.calibrate_frames(t, scale, torch.from_numpy(dark).cuda() if use_dark else None,
                               torch.from_numpy(flat).cuda() if use_flat else None).cpu().numpy()
    want = raw.astype(np.float32) * np.float32(scale)
    if use_dark:
        want = want - dark
    if use_flat:
        want = (want * np.float32(5)) / flat
    assert want.dtype == np.float32
    assert np.array_equal(out, want)


@pytest.mark.parametrize("colorid", [8, 9, 10, 11])
@pytest.mark.parametrize("dtype", [np.uint16, np.float32])
def test_debayer_nn2_bit_exact(gpu, oracle, colorid, dtype):
    """read_input_frame's DEBAYER_NN2 (nninterpolation, core/debayer.cc:
    828-1161) of raw Bayer frames against the oracle: bitwise."""
    C, O = gpu, oracle
    rng = np.random.default_rng(colorid)
    n, h, w = 3, 62, 90
    if dtype == np.uint16:
        raw = rng.integers(0, 65536, (n, h, w)).astype(np.uint16)
    else:
        raw = rng.random((n, h, w)).astype(np.float32)
    got = C.debayer_nn2(raw, colorid)
    for i in range(n):
        want = O.debayer_nn2(raw[i], colorid)
        assert got[i].dtype == want.dtype
        assert np.array_equal(got[i].view(np.uint8), want.view(np.uint8)), i


@pytest.mark.parametrize("colorid", [0, 8, 11])
@pytest.mark.parametrize("dtype", [np.uint16, np.float32, np.uint8])
def test_filter_bad_pixels_bit_exact(gpu, oracle, colorid, dtype):
    """read_input_frame's bad-pixel filter (median_filter_bad_pixels 5 x 5 /
    bayer_denoise 3 x 3 per Bayer plane) against the oracle: bitwise"""
    C, O = gpu, oracle
    rng = np.random.default_rng(colorid + 3)
    n, h, w = 3, 58, 84
    if dtype == np.float32:
        raw = rng.normal(0.4, 0.01, (n, h, w)).astype(np.float32)
        hot = 0.9
    else:
        top = 65535 if dtype == np.uint16 else 255
        raw = np.clip(rng.normal(0.4 * top, 0.01 * top, (n, h, w)), 0, top).astype(dtype)
        hot = top
    for i in range(n):
        raw[i, rng.integers(0, h, 25), rng.integers(0, w, 25)] = hot
        raw[i, rng.integers(0, h, 10), rng.integers(0, w, 10)] = 0
    got = C.filter_bad_pixels(raw, colorid, 3.0)
    for i in range(n):
        if dtype == np.uint8:
            want = O.filter_bad_pixels(raw[i].astype(np.uint16), colorid, 3.0).astype(np.uint8)
        else:
            want = O.filter_bad_pixels(raw[i], colorid, 3.0)
        assert np.array_equal(got[i].view(np.uint8), want.view(np.uint8)), (i, (got[i] != want).sum())
        assert (got[i] != raw[i]).sum() >= 20
