"""Local-variance sharpness maps on the GPU against the FP64 oracle
(compute_local_variance_map, c_local_variance_sharpness_measure.cc:193-249),
and the stacking pipeline's weighting 3, which warps each frame's map like
the frame (bilinear, BORDER_CONSTANT 0) and multiplies it by the remapped
mask (c_image_stacking_pipeline.cc:1653-1658, 1704-1713).

Tolerances: maps within 2e-5 of the frame's largest map value and Q within
1e-5 relative (FP32 pyrDown values and cubes against FP64); stacked pixels
within 2e-5 relative of the FP64 weighted sums.
"""
import numpy as np
import pytest

from serstacker_gb300 import synth

pytestmark = pytest.mark.gpu

MAP_TOL = 2e-5
Q_TOL = 1e-5
STACK_TOL = 2e-5


def _image(w, h, dtype, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    base = 0.5 + 0.3 * np.sin(x / 7.0) * np.cos(y / 11.0) + 0.05 * rng.standard_normal((h, w))
    if dtype == np.uint8:
        return np.clip(base * 200, 0, 255).astype(np.uint8)
    if dtype == np.uint16:
        return np.clip(base * 50000, 0, 65535).astype(np.uint16)
    return base.astype(np.float32)


_SCALE = {np.uint8: 1.0 / 255, np.uint16: 1.0 / 65535, np.float32: 1.0}


@pytest.mark.parametrize("w,h,dtype,kradius,dscale,uscale", [
    (1280, 960, np.uint16, 2, 1, 3),     # the stacking defaults at the headline frame size (8 x 8 cells folded)
    (333, 277, np.float32, 1, 2, 2),     # two pyrDowns, non-integer INTER_AREA factors
    (160, 120, np.uint8, 3, 0, 0),       # full resolution, no reduction
    (100, 75, np.float32, 2, 1, 0),      # pyrDown only, INTER_LINEAR back
    (61, 47, np.uint16, 2, 1, 3),        # partial tiles, dscaleSize stops early
    (200, 150, np.float32, 16, 1, 1),    # the largest supported radius (general two-kernel path)
    (150, 97, np.uint8, 1, 1, 2),        # fused pyrDown + gradient, radius 1
    (257, 129, np.uint16, 3, 1, 2),      # fused pyrDown + gradient, radius 3
    (130, 66, np.uint16, 4, 1, 0),       # pyrDown kernel, then the staged gradient of radius 4
    (96, 40, np.float32, 4, 0, 0),       # staged gradient of radius 4 on the frame itself
    (1024, 512, np.uint16, 1, 1, 4),     # 16 x 16 INTER_AREA cells folded into the gradient tiles
])
def test_local_variance_maps_match_oracle(gpu, oracle, w, h, dtype, kradius, dscale, uscale):
    frames = np.stack([_image(w, h, dtype, seed=w + k) for k in range(2)])
    lv = gpu.c_local_variance_sharpness_measure(kradius=kradius, dscale=dscale, uscale=uscale)
    maps, q = lv.create_maps(frames, scale=_SCALE[dtype])
    for k in range(len(frames)):
        want, q_o = oracle.local_variance_map(frames[k].astype(np.float64) * _SCALE[dtype], kradius, dscale, uscale)
        assert want.shape == (h, w)
        err = np.abs(maps[k].astype(np.float64) - want).max()
        assert err <= MAP_TOL * want.max(), (k, err, want.max())
        assert abs(q[k] - q_o) <= Q_TOL * q_o, (k, q[k], q_o)


def test_flat_frames_have_no_map(gpu):
    frames = np.stack([_image(96, 64, np.float32, 3), np.full((64, 96), 0.25, np.float32)])
    maps, q = gpu.c_local_variance_sharpness_measure().create_maps(frames)
    assert q[0] > 0 and maps[0].min() > 0
    assert q[1] == 0 and not maps[1].any()


def test_reduced_reference_map_is_upscaled(gpu, oracle):
    """dscale 0 with uscale > 0: the reference returns the INTER_AREA-reduced
    map; the library upscales it to the frame's size with INTER_LINEAR."""
    img = _image(200, 150, np.float32, 11)
    maps, q = gpu.c_local_variance_sharpness_measure(dscale=0, uscale=2).create_maps(img)
    small, q_o = oracle.local_variance_map(img.astype(np.float64), 2, 0, 2)
    assert small.shape == (38, 50)
    want = oracle.resize_linear(small, 200, 150)
    assert np.abs(maps[0] - want).max() <= MAP_TOL * want.max()
    assert abs(q[0] - q_o) <= Q_TOL * q_o


def _state(O, m, p):
    return O.set_params(m, O.identity(m), np.asarray(p, np.float64))


def test_pipeline_local_variance_weights_match_oracle(gpu, oracle):
    C, O = gpu, oracle
    w, h, n = 160, 120, 4
    sc = synth.Scene(w, h, 0.3 * min(w, h))
    frames, _, _ = synth.make_sequence_np(sc, n, seed=23, kind="config1", dtype=np.uint16, gain=64.0,
                                          blur_range=(0.8, 2.0))
    ref = synth.reference_np(sc) * 64.0
    scale = 1.0 / 65535.0
    reg = C.c_ecch(C.default_options(method=1, maxlevel=2, max_iterations=30, epsx=0.01, minimum_image_size=16))
    reg.set_reference_image(ref.astype(np.float32), scale=scale)
    acc = C.c_weigthed_average(w, h)
    acc.set_local_variance(kradius=2, dscale=1, uscale=2)
    out = C.stack_frames(reg, acc, frames, [3, 4], scale, weighting=3)
    avg, mask = acc.compute()
    m = O.model(4)
    S = np.zeros((h, w))
    W = np.zeros((h, w))
    for i in range(n):
        assert out["status"][i] == 0
        st = _state(O, m, out["params"][i][:8])
        img = frames[i].astype(np.float64) * scale
        dst, msk = O.stack_remap(m, st, img, w, h)
        lvm, _ = O.local_variance_map(img, 2, 1, 2)
        wmap = O.remap(m, st, lvm, w, h, border=O.BORDER_CONSTANT, bval=0.0)
        wt = np.where(msk > 0, wmap, 0.0)
        S += wt * dst
        W += wt
    both = (mask > 0) & (W > 0)
    assert ((mask > 0) == (W > 0)).mean() > 0.999
    ref_avg = S[both] / W[both]
    rel = np.abs(avg[both] - ref_avg) / np.maximum(np.abs(ref_avg), 0.01 * float(ref_avg.max()))
    assert rel.max() <= STACK_TOL, rel.max()


def test_pipeline_local_variance_disabled_by_zero_radius(gpu):
    """kradius <= 0: weights_required is false and the frames stack unweighted."""
    C = gpu
    w, h, n = 128, 96, 3
    sc = synth.Scene(w, h, 0.3 * min(w, h))
    frames, _, _ = synth.make_sequence_np(sc, n, seed=5, kind="config1", dtype=np.uint16, gain=64.0)
    ref = synth.reference_np(sc) * 64.0
    scale = 1.0 / 65535.0
    res = []
    for weighting, kr in ((3, 0), (0, 2)):
        reg = C.c_ecch(C.default_options(method=1, maxlevel=2, max_iterations=30, epsx=0.01, minimum_image_size=16))
        reg.set_reference_image(ref.astype(np.float32), scale=scale)
        acc = C.c_weigthed_average(w, h)
        acc.set_local_variance(kradius=kr)
        C.stack_frames(reg, acc, frames, [3], scale, weighting=weighting)
        res.append(acc.save_state()[0])
    assert np.array_equal(res[0], res[1])


def test_stack_bayer_frames_local_variance_weights(gpu, oracle):
    """weighting = 3 on the Bayer pipeline: the local-variance map of the
    binned luminance, warped to the plane grid, weights all four planes."""
    from test_gpu_bayer import _raw_sequence
    C, O = gpu, oracle
    W_, H_, n = 192, 128, 4
    pw, ph = W_ // 2, H_ // 2
    frames, ref_raw, _ = _raw_sequence(n, W_, H_, 31)
    scale = 1.0 / 4096
    reg = C.c_ecch(C.default_options(method=C.IC, maxlevel=2, max_iterations=30, epsx=0.01, minimum_image_size=16))
    reg.set_reference_image(O.average_bayer_planes(ref_raw).astype(np.float32), scale=scale)
    accs = [C.c_weigthed_average(pw, ph) for _ in range(4)]
    accs[0].set_local_variance(kradius=1, dscale=1, uscale=1)
    out = C.stack_bayer_frames(reg, accs, frames, [C.TRANSLATION], scale, weighting=3)
    m = O.model(C.TRANSLATION)
    planes = np.stack([O.extract_bayer_planes(frames[i]) for i in range(n)])
    wts = []
    for i in range(n):
        st = _state(O, m, out["params"][i][:2])
        lvm, _ = O.local_variance_map(O.average_bayer_planes(frames[i]).astype(np.float64) * scale, 1, 1, 1)
        wts.append((st, O.remap(m, st, lvm, pw, ph, border=O.BORDER_CONSTANT, bval=0.0)))
    for k in range(4):
        S = np.zeros((ph, pw))
        Wt = np.zeros((ph, pw))
        for i in range(n):
            st, wmap = wts[i]
            dst, msk = O.stack_remap(m, st, planes[i, ..., k].astype(np.float64) * scale, pw, ph)
            wt = np.where(msk > 0, wmap, 0.0)
            S += wt * dst
            Wt += wt
        st_g, _ = accs[k].save_state()
        Sg = st_g[0].astype(np.float64) + st_g[1]
        Wg = st_g[2].astype(np.float64) + st_g[3]
        ok = (Wt > 0) & (Wg > 0)
        assert ((Wt > 0) == (Wg > 0)).mean() > 0.999
        a_o, a_g = S[ok] / Wt[ok], Sg[ok] / Wg[ok]
        rel = np.abs(a_g - a_o) / np.maximum(np.abs(a_o), 0.01 * float(a_o.max()))
        assert rel.max() <= STACK_TOL, (k, rel.max())
