"""c_frame_registration on the GPU (sst_frame_registration_*, sst_remap_rmap)
against the FP64 oracle (oracle/sst_oracle_reg.cc).

Tolerances:
  - ECC images (scaleImage: pyrDown at 0.5, INTER_AREA otherwise;
    ecc_normalize): 2e-6 of the image's largest magnitude (FP32 sums of a
    few taps against FP64); scaled masks bit-exact (integer pyrDown);
  - registration: status equal, warp within 0.02 px RMS of the oracle's over
    the frame grid, rho within 1e-4;
  - current remaps: within 1e-3 px of the parameters' warp;
  - eccflow-refined remaps: within 5e-3 px RMS of the oracle's c_eccflow run
    from the oracle's ECC transform;
  - base_remap by a dense map: values 2e-5 of the maximum (FP32 map positions
    on a random source), masks on >= 99.9 % of the pixels (the >= 255
    coverage threshold).
"""
import math

import numpy as np
import pytest

from serstacker_gb300 import synth

pytestmark = pytest.mark.gpu

WARP_RMS_TOL = 0.02
SCALE = 1.0 / 65535.0


def _sequence(w, h, n, seed):
    sc = synth.Scene(w, h, 0.3 * min(w, h), band_period=16.0)
    frames, Hs, _ = synth.make_sequence_np(sc, n, seed=seed, kind="config1", dtype=np.uint16, gain=64.0,
                                           blur_range=(0.8, 2.0))
    ref = synth.reference_np(sc) * 64.0
    return ref, frames


def _rms(O, m, s_a, s_b, w, h):
    xa, ya = O.warp_grid(m, s_a, w, h)
    xb, yb = O.warp_grid(m, s_b, w, h)
    return math.sqrt(float(((xa - xb) ** 2 + (ya - yb) ** 2)[::4, ::4].mean()))


@pytest.mark.parametrize("scale,norm", [(0.5, 0), (0.4, 0), (0.5, 2), (1.0, 3)])
def test_ecc_images_match_oracle(gpu, oracle, scale, norm):
    C, O = gpu, oracle
    w, h = 203, 150
    ref, frames = _sequence(w, h, 2, seed=31)
    rng = np.random.default_rng(5)
    mask = np.full((h, w), 255, np.uint8)
    mask[rng.integers(0, h, 40), rng.integers(0, w, 40)] = 0
    mask[:, :7] = 0
    reg = C.c_frame_registration(ecc=dict(scale=scale, normalization_scale=norm, ecc_method=C.IC, ecch_max_level=2))
    reg.setup_reference_frame(ref.astype(np.float32), mask=mask, scale=SCALE)
    eref, emask = reg.ecc_image(-1, with_mask=True)
    oref, omask = O.scale_image(ref * SCALE, scale, mask) if scale != 1.0 else (ref * SCALE, mask)
    assert eref.shape == oref.shape
    assert np.array_equal(emask, omask)
    if norm:
        oref = O.ecc_normalize(oref, norm, omask)
    tol = 2e-6 * np.abs(oref).max()
    assert np.abs(eref - oref).max() <= tol, np.abs(eref - oref).max() / np.abs(oref).max()
    reg.register_frames(frames, scale=SCALE)
    for i in range(2):
        ocur, _ = O.scale_image(frames[i].astype(np.float64) * SCALE, scale) if scale != 1.0 else \
            (frames[i].astype(np.float64) * SCALE, None)
        if norm:
            ocur = O.ecc_normalize(ocur, norm)
        got = reg.ecc_image(i)
        assert np.abs(got - ocur).max() <= 2e-6 * np.abs(ocur).max(), i


CASES = [
    # motion, ecc options
    (3, dict()),                                                               # the reference defaults (LM, scale 0.5, 1 level)
    (3, dict(ecc_method=1, ecch_max_level=3, eps=0.01)),                        # IC, translation first, step 1.5
    (4, dict(ecc_method=3, ecch_max_level=3, eps=0.01, update_step_scale=1.0)),  # IC-LM homography
    (3, dict(ecc_method=1, ecch_max_level=2, eps=0.01, scale=1.0, normalization_scale=2,
             ecch_estimate_translation_first=0)),                              # normalized, full scale
    (4, dict(ecc_method=0, ecch_max_level=2, eps=0.01, scale=0.4, update_step_scale=1.0)),  # FA on INTER_AREA
    (1, dict(ecc_method=1, ecch_max_level=3, eps=0.01)),                        # euclidean (fixed scale)
]


@pytest.mark.parametrize("motion,ecc", CASES)
def test_register_frames_matches_oracle(gpu, oracle, motion, ecc):
    C, O = gpu, oracle
    w, h, n = 256, 192, 4
    ref, frames = _sequence(w, h, n, seed=40 + motion)
    reg = C.c_frame_registration(motion_type=motion, ecc=ecc)
    reg.setup_reference_frame(ref.astype(np.float32), scale=SCALE)
    out = reg.register_frames(frames, scale=SCALE, rmap=True)
    e = reg.options.ecc
    oo = O.registration_opts(motion_type=motion, method=e.ecc_method, scale=e.scale, eps=e.eps, min_rho=e.min_rho,
                             input_smooth_sigma=e.input_smooth_sigma,
                             reference_smooth_sigma=e.reference_smooth_sigma,
                             update_step_scale=e.update_step_scale, max_iterations=e.max_iterations,
                             ecch_max_level=e.ecch_max_level, ecch_minimum_image_size=e.ecch_minimum_image_size,
                             normalization_scale=e.normalization_scale, normalization_noise=e.normalization_noise,
                             estimate_translation_first=e.ecch_estimate_translation_first)
    m = O.model(motion)
    for i in range(n):
        status, st, rho, it = O.register_frame(oo, ref * SCALE, frames[i].astype(np.float64) * SCALE)
        assert out["status"][i] == status, (i, out["status"][i], status, out["rho"][i], rho)
        assert out["rho"][i] == pytest.approx(rho, abs=1e-4), i
        if status != 0:
            continue
        s_g = O.set_params(m, O.identity(m), out["params"][i][:O.nparams(m)].astype(np.float64))
        rms = _rms(O, m, st, s_g, w, h)
        assert rms <= WARP_RMS_TOL, (i, rms, out["iterations"][i], it)
        X, Y = O.warp_grid(m, s_g, w, h)
        assert np.abs(out["rmap"][i, ..., 0] - X).max() < 1e-3
        assert np.abs(out["rmap"][i, ..., 1] - Y).max() < 1e-3


def test_register_frames_gates_low_correlation(gpu, oracle):
    """A frame of noise fails the translation estimate's 0.75 min_rho gate
    (status LOW_RHO) in both; its neighbours register."""
    C, O = gpu, oracle
    w, h = 256, 192
    ref, frames = _sequence(w, h, 3, seed=50)
    frames[1] = np.random.default_rng(1).integers(0, 13000, size=(h, w)).astype(np.uint16)
    reg = C.c_frame_registration(ecc=dict(ecc_method=1, ecch_max_level=3, eps=0.01))
    reg.setup_reference_frame(ref.astype(np.float32), scale=SCALE)
    out = reg.register_frames(frames, scale=SCALE)
    oo = O.registration_opts(method=O.IC, ecch_max_level=3, eps=0.01)
    for i in range(3):
        status, _, rho, _ = O.register_frame(oo, ref * SCALE, frames[i].astype(np.float64) * SCALE)
        assert out["status"][i] == status, i
    assert out["status"][1] == C.FRAME_LOW_RHO and out["status"][0] == 0 and out["status"][2] == 0


def _textured_sequence(w, h, n, seed):
    """a 2-D texture everywhere (c_eccflow's 2 x 2 systems stay well
    conditioned) under an affine warp plus a smooth deformation of ~1 px"""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)

    def tex(X, Y):
        return (10 + 4 * np.sin(2 * np.pi * X / 17.0) * np.cos(2 * np.pi * Y / 13.0)
                + 3 * np.sin(2 * np.pi * (X + Y) / 23.0) + 2 * np.cos(2 * np.pi * (X - 2 * Y) / 31.0))

    frames = []
    for _ in range(n):
        a = rng.normal(0, 0.5, size=4)
        tx, ty = rng.uniform(-3, 3, size=2)
        u = tx + 0.002 * (x - w / 2) + a[0] * np.sin(2 * np.pi * y / h) + a[1] * np.cos(2 * np.pi * x / w)
        v = ty - 0.002 * (y - h / 2) + a[2] * np.cos(2 * np.pi * y / h) + a[3] * np.sin(2 * np.pi * x / w)
        frames.append(tex(x - u, y - v) + rng.normal(0, 0.05, size=(h, w)))
    return tex(x, y).astype(np.float32), np.stack(frames).astype(np.float32)


def test_eccflow_registration_refines_the_ecc_remap(gpu, oracle):
    """enable_eccflow_registration: the ECC transform's remap refined by
    c_eccflow on the full-size frame, against the oracle's c_eccflow run from
    the oracle's ECC transform."""
    C, O = gpu, oracle
    w, h, n = 256, 192, 2
    ref, frames = _textured_sequence(w, h, n, seed=61)
    flow = dict(max_iterations=2, support_scale=3, scale_factor=0.5, min_image_size=8)
    reg = C.c_frame_registration(motion_type=3, ecc=dict(ecc_method=1, ecch_max_level=3, eps=0.01, min_rho=0.5),
                                 eccflow=flow, enable_eccflow_registration=1)
    reg.setup_reference_frame(ref)
    out = reg.register_frames(frames, rmap=True)
    oo = O.registration_opts(method=O.IC, ecch_max_level=3, eps=0.01, min_rho=0.5)
    fo = O.flow_opts(update_multiplier=1.5, scale_factor=0.5, max_iterations=2, support_scale=3, min_image_size=8)
    m = O.model(O.AFFINE)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    for i in range(n):
        status, st, _, _ = O.register_frame(oo, ref.astype(np.float64), frames[i].astype(np.float64))
        assert status == 0 and out["status"][i] == 0
        X, Y = O.warp_grid(m, st, w, h)
        init = np.stack([X - xx, Y - yy], axis=-1)
        fl = O.eccflow(fo, ref.astype(np.float64), frames[i].astype(np.float64), init_flow=init)
        d = out["rmap"][i] - np.stack([xx + fl[..., 0], yy + fl[..., 1]], axis=-1)
        rms = math.sqrt(float((d ** 2).sum(axis=-1).mean()))
        assert rms < 5e-3, (i, rms)
        # the refinement moved the remap away from the affine transform's
        assert math.sqrt(float(((out["rmap"][i, ..., 0] - X) ** 2).mean())) > 0.05


@pytest.mark.parametrize("border", [0, 1, 2, 4])
def test_remap_rmap_matches_oracle(gpu, oracle, border):
    C, O = gpu, oracle
    rng = np.random.default_rng(11)
    src = rng.random((90, 120)).astype(np.float32)
    m = O.model(O.AFFINE)
    st = O.set_params(m, O.identity(m), np.array([1.01, 0.02, -6.3, -0.015, 0.99, 4.7]))
    X, Y = O.warp_grid(m, st, 110, 80)
    rmap = np.stack([X, Y], axis=-1).astype(np.float32)
    dst, msk = C.remap_rmap(src, rmap, border=border, border_value=0.25 if border == 0 else 0.0)
    want = O.remap(m, st, src.astype(np.float64), 110, 80, border=border, bval=0.25 if border == 0 else 0.0)
    _, want_m = O.stack_remap(m, st, src.astype(np.float64), 110, 80)
    # the map holds FP32 positions (4e-6 px at x ~ 100) of a random source
    assert np.abs(dst - want).max() < 2e-5 * np.abs(want).max()
    assert (msk == want_m).mean() > 0.999
