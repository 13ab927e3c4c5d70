"""The other frame accumulators on the GPU against the FP64 oracle
(oracle/sst_oracle_accum.cc):

  - c_frame_accumulation_with_fft (sst_fft_average_*): FP32 cuFFT transforms
    against FP64 DFTs, within 2e-5 of the average's largest magnitude;
  - c_canvas_average (sst_canvas_average_*): the running mean in FP32 with the
    remaps at the FP32 map positions, within 2e-6 of the largest value;
    weight sums within 1e-6 relative (exact for masks), canvas geometry
    (size, last box, shifts) exact;
  - c_laplacian_pyramid_focus_stacking (sst_focus_stack_*): FP32 pyramids
    against FP64, within 2e-5 of the largest magnitude.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _smooth_frames(n, h, w, cn, seed, dtype=np.float32, scale=1.0):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    out = []
    for i in range(n):
        planes = []
        for c in range(cn):
            p = 0.5 + 0.3 * np.sin(x / (3.0 + i + c)) * np.cos(y / (4.0 + 0.5 * i)) + 0.05 * rng.standard_normal((h, w))
            planes.append(p)
        out.append(np.stack(planes, axis=-1) if cn > 1 else planes[0])
    a = np.stack(out)
    if dtype == np.float32:
        return a.astype(np.float32)
    return np.clip(np.rint(a * scale), 0, np.iinfo(dtype).max).astype(dtype)


@pytest.mark.parametrize("n,h,w,cn,dtype", [
    (6, 29, 37, 1, np.float32),      # padded to 30 x 40
    (4, 48, 64, 1, np.uint16),       # already optimal: no padding
    (3, 34, 50, 3, np.float32),      # colour, padded to 36 x 50
    (70, 30, 41, 1, np.float32),     # two transform batches (64 + 6 frames)
])
def test_fft_average_matches_oracle(gpu, oracle, n, h, w, cn, dtype):
    C, O = gpu, oracle
    scale = 1.0 / 65535.0 if dtype == np.uint16 else 1.0
    frames = _smooth_frames(n, h, w, cn, seed=n + h, dtype=dtype, scale=65535.0)
    avg, mask = C.fft_average(frames, scale=scale)
    want = O.fft_average(frames.astype(np.float64) * scale)
    assert avg.shape == want.shape and mask.shape == (h, w) and (mask == 255).all()
    err = np.abs(avg - want).max() / np.abs(want).max()
    assert err <= 2e-5, err


def test_fft_average_accumulates_over_calls(gpu, oracle):
    C, O = gpu, oracle
    frames = _smooth_frames(5, 26, 33, 1, seed=3)
    acc = C.c_frame_accumulation_with_fft()
    acc.add_batch(frames[:2])
    for i in range(2, 5):
        acc.add(frames[i])
    assert acc.accumulated_frames() == 5 and acc.fft_size() == (36, 27)
    avg, _ = acc.compute()
    want = O.fft_average(frames.astype(np.float64))
    assert np.abs(avg - want).max() <= 2e-5 * np.abs(want).max()


def _affine_map(bw, bh, a, rng):
    y, x = np.mgrid[0:bh, 0:bw].astype(np.float64)
    X = a[0] * x + a[1] * y + a[2] + 0.3 * np.sin(y / 17.0)
    Y = a[3] * x + a[4] * y + a[5]
    return np.stack([X, Y], axis=-1).astype(np.float32)


@pytest.mark.parametrize("cn,wkind", [(1, "none"), (1, "mask"), (3, "weights"), (1, "weights")])
def test_canvas_average_matches_oracle(gpu, oracle, cn, wkind):
    """a sequence: the first frame, a frame without remap, frames remapped to
    boxes around the canvas (two of them within 32 px of an edge, which
    shifts the canvas), one box clipped by the canvas (counted, not added)"""
    C, O = gpu, oracle
    rng = np.random.default_rng(10 + cn)
    n, h, w = 7, 60, 80
    frames = _smooth_frames(n, h, w, cn, seed=5)
    weights = None
    if wkind == "mask":
        weights = (rng.random((n, h, w)) > 0.2).astype(np.uint8) * 255
    elif wkind == "weights":
        weights = rng.uniform(0.2, 2.0, (n, h, w)).astype(np.float32)
    canvas = (400, 300)
    boxes = [None, None, (150, 120, 70, 50), (20, 140, 80, 60), (260, 200, 64, 48), (330, 10, 60, 40),
             (380, 150, 60, 40)]
    maps = [None, None]
    for b in boxes[2:]:
        a = (1.0 + rng.normal(0, 0.01), rng.normal(0, 0.01), rng.uniform(0, 6), rng.normal(0, 0.01),
             1.0 + rng.normal(0, 0.01), rng.uniform(0, 8))
        maps.append(_affine_map(b[2], b[3], a, rng))
    acc = C.c_canvas_average(canvas)
    statuses = []
    for i in range(n):
        acc.add(frames[i], None if weights is None else weights[i], maps[i], boxes[i])
    (cw, ch), last, nf = acc.state()
    avg, mask = acc.compute()
    W = acc.counter()
    ob = np.array([b if b is not None else (0, 0, 0, 0) for b in boxes], np.int32)
    ow = None if weights is None else (weights if weights.dtype == np.uint8 else weights.astype(np.float64))
    oacc, oW, ost, olast = O.canvas_average(frames.astype(np.float64), weights=ow, boxes=ob,
                                            rmaps=[None if m is None else m.astype(np.float64) for m in maps],
                                            canvas=canvas)
    assert (cw, ch) == (oW.shape[1], oW.shape[0]) and nf == n
    assert list(last) == list(olast)
    assert 1 in list(ost) and (np.asarray(ost) >= 0).all()   # the clipped box is counted only
    if wkind == "weights":
        assert np.abs(W - oW).max() <= 1e-6 * oW.max()
    else:
        assert np.array_equal(W, oW.astype(np.float32))
    assert np.array_equal(mask > 0, oW > 0)
    err = np.abs(avg - oacc).max() / np.abs(oacc).max()
    assert err <= 2e-6, err
    sub, smask = acc.compute(dscale=2.0, rbbox=(10, 20, 50, 40))
    assert np.allclose(sub, 2.0 * avg[20:60, 10:60], rtol=1e-6) and np.array_equal(smask, mask[20:60, 10:60])


def test_canvas_average_rejects_empty_box(gpu):
    C = gpu
    acc = C.c_canvas_average()
    f = np.ones((20, 30), np.float32)
    acc.add(f)
    with pytest.raises(C.SSTError):
        acc.add(f, rmap=np.zeros((10, 10, 2), np.float32), bbox=(5000, 5000, 10, 10))
    assert acc.state()[2] == 1


def _gauss(k, sigma):
    """cv::getGaussianKernel(k, sigma) from its documented formula"""
    if sigma <= 0:
        sigma = 0.3 * ((k - 1) * 0.5 - 1) + 0.8
    x = np.arange(k) - (k - 1) * 0.5
    g = np.exp(-x * x / (2 * sigma * sigma))
    return g / g.sum()


def _holes(n, h, w, seed):
    rng = np.random.default_rng(seed)
    m = np.full((n, h, w), 255, np.uint8)
    for i in range(n):
        m[i, :, : 2 + i] = 0                          # a registration border
        y0, x0 = rng.integers(5, h - 12), rng.integers(5, w - 12)
        m[i, y0:y0 + 6, x0:x0 + 9] = 0                # a hole in the middle
        m[i, rng.integers(0, h, 20), rng.integers(0, w, 20)] = 0
    return m


@pytest.mark.parametrize("policy,cn,masked,smooth", [
    (0, 1, False, None),                 # the reference defaults
    (0, 1, True, None),                  # mask holes: inpaint + masked levels
    (1, 1, False, None),                 # weighted average
    (1, 3, True, None),                  # colour, channel-sum weights
    (0, 3, False, (2, 1.0)),             # select with smoothed magnitudes, frame by frame
    (1, 1, True, (1, 0.0)),              # weighted with smoothed energies (default sigma)
])
def test_focus_stack_matches_oracle(gpu, oracle, policy, cn, masked, smooth):
    C, O = gpu, oracle
    n, h, w = 5, 70, 90
    frames = _smooth_frames(n, h, w, cn, seed=21 + cn)
    masks = _holes(n, h, w, seed=3) if masked else None
    if masked and policy == 1:
        # a coefficient masked in every frame has no weight (0 / 0 in both);
        # keep every other frame whole
        masks[0::2] = 255
    kw = dict(fusing_policy=policy)
    G = None
    if smooth:
        kw.update(kradius=smooth[0], ksigma=smooth[1])
        G = _gauss(2 * smooth[0] + 1, smooth[1])
    fs = C.c_laplacian_pyramid_focus_stacking(**kw)
    if G is not None:
        assert np.abs(fs.kernel() - G).max() < 1e-7
    fs.add_batch(frames[:2], None if masks is None else masks[:2])
    for i in range(2, n):
        fs.add(frames[i], None if masks is None else masks[i])
    got = fs.compute()
    want = O.focus_stack(frames.astype(np.float64), masks, policy=policy, G=G)
    assert got.shape == want.shape
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err <= 2e-5, err


@pytest.mark.parametrize("cn", [1, 3])
def test_linear_inpaint_matches_oracle(gpu, oracle, cn):
    C, O = gpu, oracle
    h, w = 64, 77
    img = _smooth_frames(1, h, w, cn, seed=8)[0]
    m = _holes(1, h, w, seed=9)[0]
    m[20, :] = 0                                       # a whole row: filled from the columns
    m[:, 40] = 0
    got = C.linear_interpolation_inpaint(img, m)
    want = O.linear_inpaint(img.astype(np.float64), m)
    assert got.shape == want.shape
    assert np.abs(got - want).max() <= 2e-6 * np.abs(want).max()
    assert np.array_equal(got[m > 0], img[m > 0])
