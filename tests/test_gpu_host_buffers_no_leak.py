"""Entry points that take host buffers stage them in device temporaries; each
call must give those back. Repeated calls leave the device's free memory
where it was after the first call (which may grow buffers kept with the
accumulator)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 1024, 768
CALLS = 24
# a leak of one call's temporaries would be megabytes per call; allow 8 MiB of
# allocator rounding over all calls
SLACK = 8 << 20


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _check_flat(fn):
    fn()
    before = _free_bytes()
    for _ in range(CALLS):
        fn()
    after = _free_bytes()
    assert before - after <= SLACK, (before - after) / 2**20


def test_accumulator_host_calls_release_their_temporaries(gpu):
    rng = np.random.default_rng(3)
    acc = gpu.c_weigthed_average(W, H)
    acc.add(rng.random((H, W), dtype=np.float32))
    _check_flat(acc.compute)
    _check_flat(acc.get_acc_counters)
    avg, _ = acc.compute()
    accw = acc.get_acc_counters()
    _check_flat(lambda: acc.reinitialize(avg, accw))


def test_remap_and_inpaint_host_calls_release_their_temporaries(gpu):
    rng = np.random.default_rng(4)
    img = rng.random((H, W), dtype=np.float32)
    params = np.array([0.01, 0.002, 1.5, -0.003, 0.01, -2.0], np.float32)
    _check_flat(lambda: gpu.remap(img, gpu.AFFINE, params))
    _check_flat(lambda: gpu.create_remap(gpu.AFFINE, params, W, H))
    rmap = gpu.create_remap(gpu.AFFINE, params, W, H)
    _check_flat(lambda: gpu.remap_rmap(img, rmap))
    mask = (rng.random((H, W)) > 0.05).astype(np.uint8) * 255
    _check_flat(lambda: gpu.average_pyramid_inpaint(img, mask))
