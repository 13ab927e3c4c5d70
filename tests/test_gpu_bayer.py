"""GPU parity of the Bayer mosaic accumulator (c_bayer_average) against the
FP64 oracle fed the way the stacking pipeline feeds the reference
(c_image_stacking_pipeline.cc:1704-1749: remapped mask x frame weight, then
_bayer_accumulate, c_frame_accumulation.cc:988-1126).

Tolerance: channel averages within 1e-5 relative of the FP64 sums (relative
to max(|avg|, 1% of full scale)), channel weight sums within 1e-5 relative.
The >= 255 mask test can flip on a pixel whose coverage sits at the threshold
between FP32 and FP64 positions; pixels whose weight sums disagree are
counted and must stay below 0.1 %.
"""
import numpy as np
import pytest

from serstacker_gb300 import synth

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def _mosaic_sequence(n, w, h, seed, noise=False):
    rng = np.random.default_rng(seed)
    if noise:
        return rng.integers(0, 4096, size=(n, h, w), dtype=np.uint16)
    sc = synth.Scene(w, h, 0.3 * min(w, h))
    frames, _, _ = synth.make_sequence_np(sc, n, seed=seed, kind="config1", dtype=np.uint16, gain=12.0,
                                          blur_range=(0.8, 2.0))
    # per-channel gains on the mosaic positions (R, G, G, B cells)
    g = np.array([[1.0, 0.7], [0.7, 0.45]])
    tile = np.tile(g, (h // 2 + 1, w // 2 + 1))[:h, :w]
    return np.minimum(frames * tile, 4095).astype(np.uint16)


def _params(rng, n, motion):
    if motion == 0:
        return rng.uniform(-6, 6, size=(n, 2)).astype(np.float32)
    p = np.zeros((n, 8 if motion == 4 else 6), np.float32)
    for i in range(n):
        row = [1 + rng.normal(0, 1e-3), rng.normal(0, 1e-3), rng.uniform(-6, 6), rng.normal(0, 1e-3),
               1 + rng.normal(0, 1e-3), rng.uniform(-6, 6)]
        if motion == 4:
            row += [rng.normal(0, 1e-6), rng.normal(0, 1e-6)]
        p[i] = row
    return p


def _check(acc_g, w_g, acc_o, w_o):
    """acc/w: (h, w, 3) channel sums and weights (GPU f32, oracle f64)."""
    floor_w = 1e-30 + 0.0
    wagree = np.abs(w_g - w_o) <= REL_TOL * np.maximum(np.abs(w_o), 1e-3)
    assert wagree.mean() > 0.999, wagree.mean()
    both = wagree & (w_o > 0)
    assert both.any()
    avg_o = acc_o[both] / w_o[both]
    avg_g = acc_g[both] / w_g[both]
    floor = 0.01 * float(np.abs(avg_o).max()) + floor_w
    rel = np.abs(avg_g - avg_o) / np.maximum(np.abs(avg_o), floor)
    assert rel.max() <= REL_TOL, rel.max()


def _gpu_sums(acc):
    st, frames = acc.save_state()
    S = st[:, 0].astype(np.float64) + st[:, 1]
    W = st[:, 2].astype(np.float64) + st[:, 3]
    return np.moveaxis(S, 0, -1), np.moveaxis(W, 0, -1), frames


@pytest.mark.parametrize("motion,colorid,size,noise", [
    (3, 8, (200, 150), False),      # affine, RGGB
    (4, 8, (200, 150), True),       # homography, RGGB, noise mosaic
    (0, 11, (160, 120), False),     # translation, BGGR
    (3, 10, (203, 151), True),      # odd size, GBRG
    (4, 9, (128, 96), False),       # GRBG
])
def test_bayer_average_matches_oracle(gpu, oracle, motion, colorid, size, noise):
    C, O = gpu, oracle
    w, h = size
    n = 7
    rng = np.random.default_rng(31 + motion + colorid)
    frames = _mosaic_sequence(n, w, h, 11 + colorid, noise)
    params = _params(rng, n, motion)
    weights = rng.uniform(0.3, 2.0, size=n).astype(np.float32)
    status = np.zeros(n, np.int32)
    status[2] = 3                      # a rejected frame is skipped
    scale = 1.0 / 4096
    acc = C.c_bayer_average(w, h, colorid)
    acc.add(frames[:4], motion, params[:4], status=status[:4], weights=weights[:4], scale=scale)
    acc.add(frames[4:], motion, params[4:], status=status[4:], weights=weights[4:], scale=scale)
    S_o, W_o = O.bayer_average(colorid, frames, motion, params, weights, status, scale)
    S_g, W_g, nf = _gpu_sums(acc)
    assert nf == n and acc.accumulated_frames() == n
    _check(S_g, W_g, S_o, W_o)
    avg, mask, accw = acc.compute()
    ok = W_o > 0
    assert np.array_equal(mask > 0, ok.any(axis=2)) or (np.mean((mask > 0) == ok.any(axis=2)) > 0.999)
    ref = np.where(ok, S_o / np.where(ok, W_o, 1), 0)
    sel = ok & (np.abs(W_g - W_o) <= REL_TOL * np.maximum(W_o, 1e-3))
    floor = 0.01 * float(ref.max())
    assert (np.abs(avg[sel] - ref[sel]) / np.maximum(np.abs(ref[sel]), floor)).max() <= REL_TOL
    half = np.array([1.0, 0.5, 1.0])
    assert np.allclose(accw, (W_g * half).astype(np.float32), rtol=1e-6, atol=0)


def test_bayer_average_without_remap(gpu, oracle):
    """Empty rmap: each raw sample goes to the channel of its own mosaic cell."""
    C, O = gpu, oracle
    w, h, n = 96, 64, 5
    frames = _mosaic_sequence(n, w, h, 3, noise=True)
    weights = np.linspace(0.5, 1.5, n).astype(np.float32)
    acc = C.c_bayer_average(w, h, 8)
    acc.add(frames, None, weights=weights, scale=1.0 / 4096)
    S_o, W_o = O.bayer_average(8, frames, None, None, weights, None, 1.0 / 4096)
    S_g, W_g, _ = _gpu_sums(acc)
    assert np.array_equal(W_g > 0, W_o > 0)
    _check(S_g, W_g, S_o, W_o)
    avg, mask, _ = acc.compute()
    # RGGB: R at (even, even), B at (odd, odd); channel order B, G, R
    assert (avg[0::2, 0::2, 2] > 0).all() and (avg[0::2, 0::2, 0] == 0).all()
    assert (avg[1::2, 1::2, 0] > 0).all() and (avg[1::2, 1::2, 2] == 0).all()
    assert (mask == 255).all()


def test_bayer_constant_channels_reproduced(gpu):
    """A mosaic whose every channel is constant averages to those constants
    wherever a channel received weight, for any warp."""
    C = gpu
    w, h, n = 120, 90, 4
    val = {2: 1000.0, 1: 2000.0, 0: 3000.0}        # R, G, B raw values
    pat = np.zeros((h, w), np.int64)
    pat[0::2, 0::2], pat[0::2, 1::2], pat[1::2, 0::2], pat[1::2, 1::2] = 2, 1, 1, 0
    raw = np.vectorize(val.get)(pat).astype(np.uint16)
    frames = np.repeat(raw[None], n, axis=0)
    rng = np.random.default_rng(9)
    acc = C.c_bayer_average(w, h, 8)
    acc.add(frames, 4, _params(rng, n, 4), scale=1.0)
    avg, _, accw = acc.compute()
    for ch, v in ((0, 3000.0), (1, 2000.0), (2, 1000.0)):
        sel = accw[..., ch] > 1e-3
        assert sel.mean() > 0.8
        assert np.abs(avg[..., ch][sel] - v).max() <= 1e-5 * v


def test_bayer_state_roundtrip(gpu):
    C = gpu
    w, h = 64, 48
    frames = _mosaic_sequence(3, w, h, 5, noise=True)
    a = C.c_bayer_average(w, h, 8)
    a.add(frames, 3, _params(np.random.default_rng(1), 3, 3))
    st, nf = a.save_state()
    b = C.c_bayer_average(w, h, 8)
    b.load_state(st, nf)
    assert b.accumulated_frames() == 3
    assert np.array_equal(a.compute()[0], b.compute()[0])
    b.clear()
    assert b.accumulated_frames() == 0
    with pytest.raises(C.SSTError):
        b.compute()
