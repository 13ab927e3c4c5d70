"""The engine's pyramids on the GPU against the FP64 oracle: convert (x
scale), Gaussian pre-smooth (sepFilter2D, REPLICATE) and pyrDown levels
(5-tap, REFLECT_101, c_ecch::compute_next_pyramid_layer_size).

Levels 0 and 1 come from the fused convert + pre-smooth + pyrDown pass when
the frames meet its layout rules (7-tap Gaussian, rows whose base and stride
allow a lane's four-cell loads), else from the two-kernel path; both are
covered. The fused pass works in strips of 120 columns by 96 rows (interior
and edge strips launched apart); the cases include strips cut by the right
edge, bands cut by the bottom edge, frames narrower than one strip and
shorter than one band.

Tolerance: 2e-6 of the level's largest magnitude per pixel (FP32 sums of 7
and 5 taps against FP64).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _image(w, h, dtype, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    base = 0.5 + 0.3 * np.sin(x / 7.0) * np.cos(y / 11.0) + 0.05 * rng.standard_normal((h, w))
    if dtype == np.uint8:
        return np.clip(base * 200, 0, 255).astype(np.uint8)
    if dtype == np.uint16:
        return np.clip(base * 50000, 0, 65535).astype(np.uint16)
    return (base * 100).astype(np.float32)


def _oracle_levels(oracle, img, scale, sigma, L):
    lv = [oracle.smooth(img.astype(np.float64) * scale, sigma)]
    for _ in range(1, L):
        lv.append(oracle.pyrdown(lv[-1]))
    return lv


def _check(got, want, what):
    assert got.shape == want.shape, (what, got.shape, want.shape)
    err = np.abs(got.astype(np.float64) - want).max()
    assert err <= TOL * np.abs(want).max(), (what, err, np.abs(want).max())


@pytest.mark.parametrize("w,h,dtype", [
    (1280, 960, np.uint16),      # fused: the headline frame size, whole tiles
    (328, 277, np.float32),      # fused: partial tiles at the right and bottom edges
    (208, 150, np.uint8),        # fused: u8 window alignment
    (136, 70, np.uint16),        # fused: 8 columns / 6 rows in the last tiles
    (132, 40, np.float32),       # fused: 4 level-0 and 2 level-1 columns in the last tile
    (121, 97, np.uint16),        # fused: a one-column second strip, a one-row second band
    (244, 193, np.uint8),        # fused: one interior strip, 244-byte rows (4-byte, not 16-byte multiples)
    (364, 17, np.float32),       # fused: 17 rows (two levels), one band cut short
    (100, 300, np.uint16),       # fused: narrower than one strip (edge launch only), four bands
    (333, 277, np.float32),      # two-kernel path: 1332-byte rows
    (1283, 101, np.uint16),      # two-kernel path: 2566-byte rows
])
def test_reference_pyramid_matches_oracle(gpu, oracle, w, h, dtype):
    img = _image(w, h, dtype, seed=w + h)
    scale = 1.0 / 256 if dtype == np.uint16 else 1.0
    eng = gpu.c_ecch(reference_smooth_sigma=1.0, input_smooth_sigma=1.0)
    eng.set_reference_image(img, scale=scale)
    L = eng.num_levels()
    want = _oracle_levels(oracle, img, scale, 1.0, L)
    for lvl in range(L):
        _check(eng.reference_image(lvl), want[lvl], ("reference", lvl))


@pytest.mark.parametrize("w,h,dtype", [(1280, 960, np.uint16), (328, 277, np.float32), (333, 277, np.float32)])
def test_frame_pyramids_of_a_batch_match_oracle(gpu, oracle, w, h, dtype):
    ref = _image(w, h, dtype, seed=5)
    frames = np.stack([_image(w, h, dtype, seed=10 + k) for k in range(3)])
    eng = gpu.c_ecch(reference_smooth_sigma=1.0, input_smooth_sigma=1.0, max_iterations=2)
    eng.set_reference_image(ref)
    eng.align(frames, [gpu.TRANSLATION])
    L = eng.num_levels()
    for k in range(len(frames)):
        want = _oracle_levels(oracle, frames[k], 1.0, 1.0, L)
        for lvl in range(L):
            _check(eng.current_image(k, lvl), want[lvl], ("frame", k, lvl))
