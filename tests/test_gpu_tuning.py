"""Tunable launch shapes (sst_tuning) and the project's autotuner.

Shapes that only change which CTA handles which item (CTAs per SM of the
Gauss-Newton passes and of the correlation) must give bitwise-identical
results. Shapes that regroup sums (the IC pass tile width, the stack's frame
chunks) must stay within the parity tolerances: 0.02 px warp RMS against the
default shapes and 1e-6 relative on stacked pixels.
"""
import math

import numpy as np
import pytest

from serstacker_gb300 import synth

pytestmark = pytest.mark.gpu

SCALE = 1.0 / 65535.0


def _workload(n=48, w=800, h=600):
    sc = synth.Scene(w, h, 0.3 * min(w, h))
    frames, _, _ = synth.make_sequence_np(sc, n, seed=91, kind="config1", dtype=np.uint16, gain=64.0,
                                          blur_range=(0.8, 2.0))
    ref = (synth.reference_np(sc) * 64.0).astype(np.float32)
    return frames, ref


def _run(C, frames, ref, tuning):
    h, w = ref.shape
    reg = C.c_ecch(C.default_options(method=C.IC, maxlevel=4, max_iterations=50, epsx=0.01, minimum_image_size=16,
                                     min_rho=0.5))
    reg.set_reference_image(ref, scale=SCALE)
    acc = C.c_weigthed_average(w, h)
    if tuning is not None:
        reg.set_tuning(tuning)
        acc.set_tuning(tuning)
    out = C.stack_frames(reg, acc, frames, [C.AFFINE, C.HOMOGRAPHY], SCALE, weighting=1)
    state, _ = acc.save_state()
    return out, state


def _grid_rms(p, q, w, h):
    ys, xs = np.mgrid[0:h:8, 0:w:8].astype(np.float64)

    def warp(a):
        d = a[6] * xs + a[7] * ys + 1
        return (a[0] * xs + a[1] * ys + a[2]) / d, (a[3] * xs + a[4] * ys + a[5]) / d
    xa, ya = warp(p.astype(np.float64))
    xb, yb = warp(q.astype(np.float64))
    return math.sqrt(float(((xa - xb) ** 2 + (ya - yb) ** 2).mean()))


def test_cta_counts_are_bitwise_neutral(gpu):
    C = gpu
    frames, ref = _workload()
    base, st0 = _run(C, frames, ref, None)
    for t in ({"pass_ctas_per_sm": 1}, {"pass_ctas_per_sm": 5, "corr_ctas_per_sm": 1}, {"corr_ctas_per_sm": 8}):
        out, st = _run(C, frames, ref, t)
        for k in ("params", "status", "rho", "weight"):
            assert np.array_equal(out[k], base[k]), (t, k)
        assert np.array_equal(st, st0), t


def test_regrouping_shapes_stay_within_tolerance(gpu):
    C = gpu
    frames, ref = _workload()
    h, w = ref.shape
    base, st0 = _run(C, frames, ref, None)
    S0 = st0[0].astype(np.float64) + st0[1]
    W0 = st0[2].astype(np.float64) + st0[3]
    for t in ({"pass_tile_w": [128, 128, 64, 64]}, {"pass_tile_w": [64, 64, 64, 64]},
              {"stack_max_chunks": 1}, {"stack_max_chunks": 8, "stack_items_per_slot": 8}):
        out, st = _run(C, frames, ref, t)
        assert np.array_equal(out["status"], base["status"]), t
        for i in range(frames.shape[0]):
            assert _grid_rms(out["params"][i], base["params"][i], w, h) <= 0.02, (t, i)
        if "stack_max_chunks" in t:
            assert np.array_equal(out["params"], base["params"]), t
            S = st[0].astype(np.float64) + st[1]
            W = st[2].astype(np.float64) + st[3]
            ok = W0 > 0
            assert np.array_equal(W > 0, ok)
            rel = np.abs(S[ok] / W[ok] - S0[ok] / W0[ok]) / np.maximum(np.abs(S0[ok] / W0[ok]), 1e-3)
            assert rel.max() <= 1e-6, (t, rel.max())


def test_autotuner_searches_caches_and_applies(gpu, tmp_path, monkeypatch):
    import torch
    C = gpu
    from serstacker_gb300 import autotune
    monkeypatch.setenv("SST_TUNE_CACHE", str(tmp_path / "tune.json"))
    frames, ref = _workload(n=64)
    n, h, w = frames.shape
    d = torch.from_numpy(frames.view(np.int16)).cuda()
    reg = C.c_ecch(C.default_options(method=C.IC, maxlevel=4, max_iterations=50, epsx=0.01, minimum_image_size=16,
                                     min_rho=0.5))
    reg.set_reference_image(ref, scale=SCALE)
    acc = C.c_weigthed_average(w, h)
    r1 = autotune.tune_stack_frames(reg, acc, d, n, w, h, C.DEPTH_U16, w * 2, w * h * 2, [C.AFFINE, C.HOMOGRAPHY],
                                    SCALE, sample=32, reps=1)
    assert r1["source"] == "search" and r1["candidates"] >= 5 and r1["ms"] <= r1["default_ms"]
    assert reg.get_tuning() == r1["tuning"]
    r2 = autotune.tune_stack_frames(reg, acc, d, n, w, h, C.DEPTH_U16, w * 2, w * h * 2, [C.AFFINE, C.HOMOGRAPHY],
                                    SCALE, sample=32, reps=1)
    assert r2["source"] == "cache" and r2["tuning"] == r1["tuning"]
