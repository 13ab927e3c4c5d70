"""LPG sharpness maps on the GPU (sst_lpg_compute) against the FP64 oracle of
lpg() (core/proc/lpg.cc:223-291, oracle/sst_oracle_lpg.cc).

Tolerances: maps within 2e-5 of the map's largest value (FP32 pyrDowns,
5 x 5 operators, squares, powers and pyrUps against FP64), metrics within
2e-5 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-5
MAXVAL = {np.uint8: 255.0, np.uint16: 65535.0, np.float32: 1.0}


def _frames(n, w, h, dtype, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    out = []
    for i in range(n):
        img = 0.4 + 0.25 * np.sin(x / (5.0 + i)) * np.cos(y / 7.0) + 0.05 * rng.standard_normal((h, w))
        img[(x - w / 2) ** 2 + (y - h / 2) ** 2 < (0.2 * min(w, h)) ** 2] += 0.2
        img = np.clip(img, 0, 1)
        out.append(img * MAXVAL[dtype] if dtype != np.float32 else img)
    a = np.stack(out)
    if dtype == np.float32:
        return a.astype(np.float32)
    return np.rint(a).astype(dtype)


CASES = [
    (320, 240, np.uint16, {}),                                             # the reference defaults
    (333, 251, np.uint8, {}),                                              # odd sizes
    (256, 192, np.float32, dict(k=0.5, p=1.0, dscale=0, uscale=0)),         # full scale, no power
    (200, 150, np.uint16, dict(k=4.0, p=1.5, dscale=1, uscale=3)),
    (180, 130, np.float32, dict(k=2.0, p=0.0, dscale=3, uscale=2)),         # uscale below dscale
]


@pytest.mark.parametrize("w,h,dtype,opts", CASES)
def test_lpg_maps_match_oracle(gpu, oracle, w, h, dtype, opts):
    C, O = gpu, oracle
    n = 3
    frames = _frames(n, w, h, dtype, seed=w + h)
    lpg = C.c_lpg_sharpness_measure(**opts)
    o = lpg.options
    maps, metrics = lpg.compute(frames)
    for i in range(n):
        want, met = O.lpg(frames[i].astype(np.float64) / MAXVAL[dtype], k=o.k, p=o.p, dscale=o.dscale,
                          uscale=o.uscale)
        err = np.abs(maps[i] - want).max() / np.abs(want).max()
        assert err <= TOL, (i, err)
        assert metrics[i] == pytest.approx(met, rel=TOL), i


def test_lpg_masked_metric_matches_oracle(gpu, oracle):
    C, O = gpu, oracle
    w, h = 240, 180
    frames = _frames(2, w, h, np.uint16, seed=3)
    rng = np.random.default_rng(9)
    masks = (rng.random((2, h, w)) > 0.3).astype(np.uint8) * 255
    masks[1, :, : w // 2] = 0
    lpg = C.c_lpg_sharpness_measure()
    _, metrics = lpg.compute(frames, masks)
    for i in range(2):
        _, met = O.lpg(frames[i].astype(np.float64) / 65535.0, mask=masks[i])
        assert metrics[i] == pytest.approx(met, rel=TOL), i
