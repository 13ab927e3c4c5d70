"""GPU parity of ROI batches (crops of different sizes, each against its own
reference crop) with the FP64 oracle's c_ecch run crop by crop.

Tolerance: the registered warp within 0.02 px RMS of the oracle's over the
crop's pixel grid, per crop.
"""
import math

import numpy as np
import pytest

from serstacker_gb300 import synth

pytestmark = pytest.mark.gpu

WARP_RMS_TOL = 0.02


def _crops(n, seed, lo=64, hi=220):
    """n (reference, current) crop pairs cut from one banded-disk scene; the
    current crop is the scene under a small random affine + quadratic map."""
    rng = np.random.default_rng(seed)
    W = H = 900
    sc = synth.Scene(W, H, 380.0)
    refs, curs = [], []
    for _ in range(n):
        w, h = int(rng.integers(lo, hi + 1)), int(rng.integers(lo, hi + 1))
        ox = float(rng.uniform(150, W - 150 - w))
        oy = float(rng.uniform(150, H - 150 - h))
        y, x = np.mgrid[0:h, 0:w].astype(np.float64)
        refs.append(synth.render_np(sc, x + ox, y + oy, 0.5).astype(np.float32))
        a = rng.normal(0, 4e-3, size=4)
        t = rng.uniform(-3, 3, size=2)
        q = rng.normal(0, 2e-5, size=2)
        X = (1 + a[0]) * x + a[1] * y + t[0] + q[0] * x * y
        Y = a[2] * x + (1 + a[3]) * y + t[1] + q[1] * x * x
        img = synth.render_np(sc, X + ox, Y + oy, 0.5)
        curs.append(synth.add_noise_np(rng, img, 1.0, 1.0, 1e9).astype(np.float32))
    return refs, curs


def _grid_rms(O, m, s_a, s_b, w, h, step=4):
    d2 = []
    for y in range(0, h, step):
        for x in range(0, w, step):
            xa, ya = O.warp(m, s_a, float(x), float(y))
            xb, yb = O.warp(m, s_b, float(x), float(y))
            d2.append((xa - xb) ** 2 + (ya - yb) ** 2)
    return math.sqrt(float(np.mean(d2)))


@pytest.mark.parametrize("method,motion", [(0, 6), (2, 6), (0, 3), (2, 4)])
def test_roi_batch_matches_oracle(gpu, oracle, method, motion):
    C, O = gpu, oracle
    refs, curs = _crops(6, 40 + 7 * method + motion)
    opts = C.default_options(method=method, maxlevel=3, max_iterations=40, epsx=0.01, minimum_image_size=16)
    rb = C.c_roi_batch(opts)
    out = rb.align(refs, curs, [motion])
    oo = O.ecch_opts(method=method, maxlevel=3, max_iterations=40, epsx=0.01, minimum_image_size=16)
    m = O.model(motion)
    for i, (r, c) in enumerate(zip(refs, curs)):
        h, w = r.shape
        s_o, it_o, _ = O.ecch_align(m, O.identity(m), r.astype(np.float64), c.astype(np.float64), oo)
        s_g = O.set_params(m, O.identity(m), out["params"][i][:O.nparams(m)].astype(np.float64))
        rms = _grid_rms(O, m, s_o, s_g, w, h)
        assert out["status"][i] == 0, out["status"]
        assert rms <= WARP_RMS_TOL, (method, motion, i, (w, h), rms, out["iterations"][i], it_o)


def test_roi_batch_equal_sizes_match_uniform_engine(gpu):
    """Crops that all share one reference and one size: the ROI schedule and
    the uniform batched engine agree."""
    C = gpu
    w, h, n = 160, 128, 5
    sc = synth.Scene(w, h, 0.3 * min(w, h))
    frames, _, _ = synth.make_sequence_np(sc, n, seed=8, kind="config1", dtype=np.uint16, gain=50.0,
                                          blur_range=(0.8, 1.5))
    ref = (synth.reference_np(sc) * 50.0).astype(np.float32)
    f32 = [f.astype(np.float32) for f in frames]
    for method in (0, 2):
        opts = C.default_options(method=method, maxlevel=2, max_iterations=30, epsx=0.01, minimum_image_size=16)
        reg = C.c_ecch(opts)
        reg.set_reference_image(ref)
        a = reg.align(np.stack(f32), [3])
        b = C.c_roi_batch(opts).align([ref] * n, f32, [3])
        assert np.array_equal(a["status"], b["status"])
        M = a["params"].shape[1]
        assert np.abs(a["params"] - b["params"][:, :M]).max() < 2e-3, method
        assert np.array_equal(a["iterations"], b["iterations"]), method


def test_roi_batch_rejects_ic_and_bad_rois(gpu):
    C = gpu
    with pytest.raises(C.SSTError):
        C.c_roi_batch(C.default_options(method=1))
    rb = C.c_roi_batch(C.default_options(method=0, maxlevel=2, minimum_image_size=16))
    tiny = np.zeros((8, 8), np.float32)
    with pytest.raises(C.SSTError):
        rb.align([tiny], [tiny], [0])                    # below minimum_image_size
