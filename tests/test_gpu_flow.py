"""GPU parity of c_eccflow (dense smooth flow, ecc2.cc:2220-2865) with the
FP64 oracle. Tolerance: the flow within 2e-3 px RMS and 2e-2 px max of the
oracle's over the whole frame (FP32 against FP64 through every level and
iteration of the coarse-to-fine loop)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RMS_TOL, MAX_TOL = 2e-3, 2e-2


def _scene(w, h, seed, n=3):
    """a 2-D texture everywhere (the flow's 2x2 systems stay well conditioned)
    and n frames under smooth deformations of up to ~1.5 px; returns the
    reference, the frames and the true flows"""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)

    def tex(X, Y):
        return (10 + 4 * np.sin(2 * np.pi * X / 17.0) * np.cos(2 * np.pi * Y / 13.0)
                + 3 * np.sin(2 * np.pi * (X + Y) / 23.0) + 2 * np.cos(2 * np.pi * (X - 2 * Y) / 31.0))

    ref = tex(x, y)
    frames, truth = [], []
    for _ in range(n):
        a = rng.normal(0, 0.6, size=4)
        u = a[0] * np.sin(2 * np.pi * y / h) + a[1] * np.cos(2 * np.pi * x / w)
        v = a[2] * np.cos(2 * np.pi * y / h) + a[3] * np.sin(2 * np.pi * x / w)
        frames.append(tex(x - u, y - v) + rng.normal(0, 0.05, size=(h, w)))
        truth.append(np.stack([u, v], axis=-1))
    return ref.astype(np.float32), np.stack(frames).astype(np.float32), truth


def _flow(rm):
    h, w = rm.shape[:2]
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    return np.stack([rm[..., 0] - x, rm[..., 1] - y], axis=-1)


CASES = [
    # w, h, scale_factor, support_scale, downscale, max_pyramid_level
    (256, 192, 0.75, 4, 0, -1),      # the registration defaults (c_frame_registration.h:88-100)
    (192, 144, 0.5, 3, 0, 3),        # recursive INTER_AREA
    (192, 144, 0.75, 3, 1, 4),       # full resize from level 0
    (128, 96, 0.5, 3, 2, 3),         # pyrDown
]


@pytest.mark.parametrize("w,h,scale_factor,support_scale,downscale,max_level", CASES)
def test_eccflow_matches_oracle(gpu, oracle, w, h, scale_factor, support_scale, downscale, max_level):
    C, O = gpu, oracle
    ref, frames, truth = _scene(w, h, 3)
    kw = dict(scale_factor=scale_factor, support_scale=support_scale, max_iterations=3, min_image_size=4,
              downscale=downscale, max_pyramid_level=max_level)
    fl = C.c_eccflow(C.eccflow_options(**kw))
    fl.set_reference_image(ref)
    oo = O.flow_opts(**kw)
    assert fl.num_levels() == len(O.eccflow_levels(w, h, oo))
    rm = fl.compute(frames)
    for i in range(len(frames)):
        f_o = O.eccflow(oo, ref.astype(np.float64), frames[i].astype(np.float64))
        err = np.hypot(*(f_o - truth[i])[8:-8, 8:-8].transpose(2, 0, 1))
        assert np.median(err) < 0.15            # a well-posed case: the oracle finds the deformation
        d = _flow(rm[i]) - f_o
        rms = float(np.sqrt(np.mean(d ** 2)))
        assert rms <= RMS_TOL and np.abs(d).max() <= MAX_TOL, (i, rms, np.abs(d).max())


def test_eccflow_with_initial_rmap_matches_oracle(gpu, oracle):
    C, O = gpu, oracle
    w, h = 112, 80
    ref, frames, _ = _scene(w, h, 9, n=1)
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    init_flow = np.stack([0.3 + 0.002 * x, -0.2 + 0.001 * y], axis=-1).astype(np.float32)
    init_rm = np.stack([x, y], axis=-1) + init_flow
    kw = dict(scale_factor=0.75, support_scale=3, max_iterations=2, max_pyramid_level=4)
    fl = C.c_eccflow(C.eccflow_options(**kw))
    fl.set_reference_image(ref)
    rm = fl.compute(frames[:1], init_rmap=init_rm[None])
    oo = O.flow_opts(**kw)
    f_o = O.eccflow(oo, ref.astype(np.float64), frames[0].astype(np.float64), init_flow.astype(np.float64))
    d = _flow(rm[0]) - f_o
    assert float(np.sqrt(np.mean(d ** 2))) <= RMS_TOL and np.abs(d).max() <= MAX_TOL


def test_eccflow_identical_frames_give_identity(gpu):
    C = gpu
    ref, _, _ = _scene(96, 64, 1, n=1)
    fl = C.c_eccflow(C.eccflow_options(scale_factor=0.75, support_scale=3, max_iterations=2))
    fl.set_reference_image(ref)
    rm = fl.compute(np.stack([ref, ref]))
    assert np.abs(_flow(rm[0])).max() < 1e-5 and np.abs(_flow(rm[1])).max() < 1e-5


@pytest.mark.parametrize("ref_masked,cur_masked", [(True, False), (False, True), (True, True)])
def test_eccflow_masks_match_oracle(gpu, oracle, ref_masked, cur_masked):
    """Masks (set_reference_image(reference, mask), compute(current, rmap,
    mask)): per level INTER_NEAREST mask pyramids; in each update the current
    mask remapped INTER_NEAREST by the flow and ANDed with the reference mask
    zeroes It gx, It gy (ecc2.cc:2253-2335)."""
    C, O = gpu, oracle
    w, h = 160, 112
    ref, frames, _ = _scene(w, h, 21, n=2)
    rng = np.random.default_rng(4)
    rmask = np.full((h, w), 255, np.uint8)
    rmask[20:60, 30:90] = 0
    rmask[rng.integers(0, h, 200), rng.integers(0, w, 200)] = 0
    cmasks = np.full((2, h, w), 255, np.uint8)
    cmasks[:, :, :12] = 0
    cmasks[1, 70:, 100:] = 0
    kw = dict(scale_factor=0.5, support_scale=3, max_iterations=2, min_image_size=8)
    fl = C.c_eccflow(C.eccflow_options(**kw))
    fl.set_reference_image(ref, mask=rmask if ref_masked else None)
    rm = fl.compute(frames, masks=cmasks if cur_masked else None)
    oo = O.flow_opts(**kw)
    for i in range(2):
        f_o = O.eccflow(oo, ref.astype(np.float64), frames[i].astype(np.float64),
                        ref_mask=rmask if ref_masked else None, cur_mask=cmasks[i] if cur_masked else None)
        d = _flow(rm[i]) - f_o
        rms = float(np.sqrt(np.mean(d ** 2)))
        assert rms <= RMS_TOL and np.abs(d).max() <= MAX_TOL, (i, rms, np.abs(d).max())
