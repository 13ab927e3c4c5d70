"""The CPU-runnable configuration on the GPU: plain forward-additive ECC,
EUCLIDEAN (rotation about (0, 0), fixed scale), one pyramid level, on u8
640x480 frames of the banded-disk scene, then the unweighted stack.

The reference's euclidean transform with a fixed scale never converges by
eps: c_euclidean_image_transform::eps adds the stored absolute scale (1) as
a parameter step (c_image_transform.cc:407-421, 509-523), so every frame runs
max_iterations (its counter then reads max_iterations + 1, ecc2.cc:1295).
The GPU keeps that quirk: every frame's iteration count must equal the
oracle's, which must be max_iterations + 1.

Tolerances: warp within 0.02 px RMS of the oracle's; the stack within 1e-5
relative (1 % floor) of FP64 sums with the GPU's transforms, settled pixels.
"""
import math

import numpy as np
import pytest

from serstacker_gb300 import synth

pytestmark = pytest.mark.gpu


def test_config0_fa_euclidean_matches_oracle(gpu, oracle):
    C, O = gpu, oracle
    w, h, n, max_it = 640, 480, 6, 30
    sc = synth.scene_config0()
    frames, Hs, _ = synth.make_sequence_np(sc, n, seed=1000, kind="config0", dtype=np.uint8)
    ref = synth.reference_np(sc).astype(np.float32)
    opts = C.default_options(method=C.FA, maxlevel=0, max_iterations=max_it, epsx=0.2, minimum_image_size=16,
                             min_rho=0.0)
    reg = C.c_ecch(opts)
    reg.set_reference_image(ref)
    assert reg.num_levels() == 1
    out = reg.align(frames, [C.EUCLIDEAN])
    acc = C.c_weigthed_average(w, h)
    st_out = C.stack_frames(reg, acc, frames, [C.EUCLIDEAN], 1.0, weighting=0)
    avg, mask = acc.compute()
    assert np.array_equal(st_out["params"][:, :3], out["params"][:, :3])
    m = O.model(O.EUCLIDEAN)
    oo = O.ecch_opts(method=O.FA, maxlevel=0, max_iterations=max_it, epsx=0.2, minimum_image_size=16)
    S = np.zeros((h, w))
    W = np.zeros((h, w))
    ms = []
    for i in range(n):
        st, it, _ = O.ecch_align(m, O.identity(m), ref.astype(np.float64), frames[i].astype(np.float64), oo)
        # every frame runs all max_iterations updates; the reference's counter
        # `while (_num_iterations++ < _max_iterations)` then reads max_iterations + 1
        assert it == max_it + 1, it
        assert out["iterations"][i] == it, (out["iterations"][i], it)
        s_g = O.set_params(m, O.identity(m), out["params"][i][:3].astype(np.float64))
        xa, ya = O.warp_grid(m, s_g, w, h)
        xb, yb = O.warp_grid(m, st, w, h)
        rms = math.sqrt(float(((xa - xb) ** 2 + (ya - yb) ** 2)[::4, ::4].mean()))
        assert out["status"][i] == 0 and rms <= 0.02, (i, rms)
        ms.append((m, s_g))
        dst, msk = O.stack_remap(m, s_g, frames[i].astype(np.float64), w, h)
        wt = (msk > 0).astype(np.float64)
        S += wt * dst
        W += wt
    keep = O.stack_compare_region(ms, w, h, w, h)
    assert np.array_equal((mask > 0)[keep], (W > 0)[keep])
    both = keep & (W > 0)
    rel = O.stack_rel_err(avg[both], S[both] / W[both])
    assert rel.max() <= 1e-5, rel.max()
