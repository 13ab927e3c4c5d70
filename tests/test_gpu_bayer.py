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


def _raw_sequence(n, W, H, seed):
    """raw RGGB u16 12-bit mosaic frames of a scene translated by up to
    +-6 raw px, Poisson-like noise; returns frames, reference mosaic, shifts"""
    rng = np.random.default_rng(seed)
    sc = synth.Scene(W, H, 0.3 * min(W, H))
    g = np.array([[1.0, 0.7], [0.7, 0.45]])
    gains = np.tile(g, (H // 2, W // 2))
    shifts = rng.uniform(-6, 6, size=(n, 2))
    frames = np.empty((n, H, W), np.uint16)
    for i in range(n):
        Hm = np.eye(3)
        Hm[0, 2], Hm[1, 2] = shifts[i]
        img = synth.render_frame_np(sc, Hm, 1.0) * 12.0 * gains
        img = rng.poisson(np.maximum(img, 0)).astype(np.float64) + rng.normal(0, 2.0, size=img.shape)
        frames[i] = np.clip(np.rint(img), 0, 4095).astype(np.uint16)
    ref = np.clip(np.rint(synth.reference_np(sc) * 12.0 * gains), 0, 4095).astype(np.uint16)
    return frames, ref, shifts


def test_stack_bayer_frames_matches_oracle(gpu, oracle):
    """Binned-luminance registration + four-plane stack (sst_stack_bayer_frames)
    against the oracle: registration within 0.02 px RMS of the oracle's
    c_ecch on the same binned frames, plane stacks within 1e-5 relative of
    FP64 sums of the bit-exact extracted planes under the same transforms."""
    C, O = gpu, oracle
    W, H, n = 256, 192, 6
    pw, ph = W // 2, H // 2
    frames, ref_raw, shifts = _raw_sequence(n, W, H, 21)
    scale = 1.0 / 4096
    ref_bin = O.average_bayer_planes(ref_raw)
    opts = C.default_options(method=C.IC, maxlevel=2, max_iterations=40, epsx=0.01, minimum_image_size=16,
                             min_rho=0.5)
    reg = C.c_ecch(opts)
    reg.set_reference_image(ref_bin.astype(np.float32), scale=scale)
    accs = [C.c_weigthed_average(pw, ph) for _ in range(4)]
    out = C.stack_bayer_frames(reg, accs, frames, [C.TRANSLATION], scale, weighting=1)
    assert (out["status"] == 0).all(), out["status"]
    # registration: GPU vs the oracle's c_ecch on the oracle-binned frames
    oo = O.ecch_opts(method=1, maxlevel=2, max_iterations=40, epsx=0.01, minimum_image_size=16)
    m = O.model(C.TRANSLATION)
    for i in range(n):
        b = O.average_bayer_planes(frames[i]).astype(np.float64) * scale
        s_o, _, _ = O.ecch_align(m, O.identity(m), ref_bin.astype(np.float64) * scale, b, oo)
        p_o = O.get_params(m, s_o)
        assert np.hypot(*(p_o - out["params"][i][:2])) <= 0.02, (i, p_o, out["params"][i][:2])
        # and close to the true shift (raw px / 2)
        assert np.hypot(*(out["params"][i][:2] - shifts[i] / 2)) <= 0.1
    # stacks: the same transforms applied to the extracted planes, in FP64
    planes = np.stack([O.extract_bayer_planes(frames[i]) for i in range(n)])     # (n, ph, pw, 4)
    for k in range(4):
        S = np.zeros((ph, pw))
        Wt = np.zeros((ph, pw))
        for i in range(n):
            st = O.set_params(m, O.identity(m), out["params"][i][:2].astype(np.float64))
            dst, msk = O.stack_remap(m, st, planes[i, ..., k].astype(np.float64) * scale, pw, ph)
            wt = np.where(msk > 0, float(out["weight"][i]), 0.0)
            S += wt * dst
            Wt += wt
        st_g, nf = accs[k].save_state()
        assert nf == n
        Sg = st_g[0].astype(np.float64) + st_g[1]
        Wg = st_g[2].astype(np.float64) + st_g[3]
        _check(Sg[..., None], Wg[..., None], S[..., None], Wt[..., None])


def test_stack_bayer_frames_device_and_host_inputs_agree(gpu):
    """The streamed host path and the device-resident path give identical
    planes for the same chunking (chunks of 3 frames: the compensated
    register sums are folded into the planes once per chunk)."""
    import torch
    C = gpu
    W, H, n = 128, 96, 7
    frames, ref_raw, _ = _raw_sequence(n, W, H, 4)
    scale = 1.0 / 4096
    from oracle import average_bayer_planes
    ref_bin = average_bayer_planes(ref_raw)
    opts = C.default_options(method=C.IC, maxlevel=2, max_iterations=30, epsx=0.01, minimum_image_size=16)
    states = []
    for dev in (False, True):
        reg = C.c_ecch(opts)
        reg.set_reference_image(ref_bin.astype(np.float32), scale=scale)
        reg.set_chunk_frames(3)
        accs = [C.c_weigthed_average(W // 2, H // 2) for _ in range(4)]
        if dev:
            d = torch.from_numpy(frames.view(np.int16)).cuda()
            outs = {"params": torch.zeros((n, 12), dtype=torch.float32, device="cuda"),
                    "status": torch.zeros(n, dtype=torch.int32, device="cuda"),
                    "rho": torch.zeros(n, dtype=torch.float32, device="cuda"),
                    "weight": torch.zeros(n, dtype=torch.float32, device="cuda")}
            C.stack_bayer_frames(reg, accs, d, [C.TRANSLATION], scale, on_device=True, n=n, width=W, height=H,
                                 row_stride=W * 2, frame_stride=W * H * 2, outputs=outs)
            torch.cuda.synchronize()
        else:
            C.stack_bayer_frames(reg, accs, frames, [C.TRANSLATION], scale)
        states.append([a.save_state()[0] for a in accs])
    for k in range(4):
        assert np.array_equal(states[0][k], states[1][k]), k


def test_stack_bayer_frames_focus_weights(gpu, oracle):
    """weighting = 2 on the Bayer pipeline: the focus map of the warped binned
    luminance weights all four planes (1e-4 relative, FP32 Laplacians)."""
    C, O = gpu, oracle
    W_, H_, n = 192, 128, 4
    pw, ph = W_ // 2, H_ // 2
    frames, ref_raw, _ = _raw_sequence(n, W_, H_, 31)
    scale = 1.0 / 4096
    ref_bin = O.average_bayer_planes(ref_raw)
    reg = C.c_ecch(C.default_options(method=C.IC, maxlevel=2, max_iterations=30, epsx=0.01, minimum_image_size=16))
    reg.set_reference_image(ref_bin.astype(np.float32), scale=scale)
    accs = [C.c_weigthed_average(pw, ph) for _ in range(4)]
    out = C.stack_bayer_frames(reg, accs, frames, [C.TRANSLATION], scale, weighting=2)
    m = O.model(C.TRANSLATION)
    planes = np.stack([O.extract_bayer_planes(frames[i]) for i in range(n)])
    for k in range(4):
        S = np.zeros((ph, pw))
        Wt = np.zeros((ph, pw))
        for i in range(n):
            st = O.set_params(m, O.identity(m), out["params"][i][:2].astype(np.float64))
            dst, msk = O.stack_remap(m, st, planes[i, ..., k].astype(np.float64) * scale, pw, ph)
            fw = O.focus_weights(m, st, O.average_bayer_planes(frames[i]).astype(np.float64) * scale, pw, ph)
            wt = np.where(msk > 0, fw, 0.0)
            S += wt * dst
            Wt += wt
        st_g, _ = accs[k].save_state()
        Sg = st_g[0].astype(np.float64) + st_g[1]
        Wg = st_g[2].astype(np.float64) + st_g[3]
        ok = (Wt > 0) & (Wg > 0)
        assert ((Wt > 0) == (Wg > 0)).mean() > 0.999
        a_o, a_g = S[ok] / Wt[ok], Sg[ok] / Wg[ok]
        rel = np.abs(a_g - a_o) / np.maximum(np.abs(a_o), 0.01 * float(a_o.max()))
        assert rel.max() <= 1e-4, (k, rel.max())
