"""The allocation-free stacking entry point against the allocating one.

sst_weighted_average_add_warped_batch_noalloc serves callers that cannot let
the library call cudaMalloc (a host whose own pool owns all device memory, a
real-time loop that cannot take cudaMalloc's device-wide synchronisation): it
runs the same warp + weight + compensated accumulate kernels with its
per-frame scratch in a fixed device array and the accumulator planes owned by
the caller, and returns SST_OK only when the kernels' error flag stayed
clear. This test feeds both entry points the same device-resident frames,
parameters and weights, twice in a row, and
checks the caller-owned planes against the object's planes after each call.
It is collected last so a stop-at-first-failure run has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STACK_REL_TOL = 1e-5


def _batch(rng, n, h, w):
    frames = rng.integers(0, 60000, size=(n, h, w), dtype=np.uint16)
    params = np.zeros((n, 12), np.float32)
    for i in range(n):
        params[i, :8] = [1 + rng.normal(0, 1e-3), rng.normal(0, 1e-3), rng.uniform(-6, 6), rng.normal(0, 1e-3),
                         1 + rng.normal(0, 1e-3), rng.uniform(-6, 6), rng.normal(0, 1e-6), rng.normal(0, 1e-6)]
    weights = rng.uniform(0.25, 2.0, size=n).astype(np.float32)
    status = np.zeros(n, np.int32)
    status[n // 3] = 3          # a rejected frame is skipped by both entry points
    return frames, params, weights, status


def _rel(a, b):
    scale = np.maximum(np.abs(b), 0.01 * float(np.abs(b).max()) + 1e-30)
    return float((np.abs(a - b) / scale).max())


def test_noalloc_matches_allocating_entry_point():
    import torch
    from serstacker_gb300 import capi as CA
    assert torch.cuda.is_available()
    lib = CA.lib()
    h, w = 150, 200
    rng = np.random.default_rng(2024)
    model = CA.motion(CA.HOMOGRAPHY)
    acc = CA.c_weigthed_average(w, h)
    acc_state = torch.zeros((4, h, w), dtype=torch.float32, device="cuda")
    for call in range(2):
        frames, params, weights, status = _batch(rng, 9, h, w)
        d_frames = torch.from_numpy(frames.view(np.int16)).cuda()
        d_params = torch.from_numpy(params).cuda()
        d_weights = torch.from_numpy(weights).cuda()
        d_status = torch.from_numpy(status).cuda()
        n = frames.shape[0]
        rs, fs = frames.strides[1], frames.strides[0]
        rc = lib.sst_weighted_average_add_warped_batch(
            acc.handle, d_frames.data_ptr(), CA.DEPTH_U16, n, w, h, rs, fs, 1.0 / 65535, 1, C.byref(model),
            d_params.data_ptr(), d_status.data_ptr(), d_weights.data_ptr(), CA.BORDER_REFLECT101, None)
        assert rc == 0, CA.last_error()
        rc = lib.sst_weighted_average_add_warped_batch_noalloc(
            d_frames.data_ptr(), CA.DEPTH_U16, n, w, h, rs, fs, 1.0 / 65535, C.byref(model), d_params.data_ptr(),
            d_status.data_ptr(), d_weights.data_ptr(), CA.BORDER_REFLECT101, acc_state.data_ptr(), w, h, None)
        assert rc == 0, CA.last_error()
        torch.cuda.synchronize()
        ref_state, _ = acc.save_state()
        got = acc_state.cpu().numpy()
        S_ref = ref_state[0].astype(np.float64) + ref_state[1]
        W_ref = ref_state[2].astype(np.float64) + ref_state[3]
        S_got = got[0].astype(np.float64) + got[1]
        W_got = got[2].astype(np.float64) + got[3]
        assert np.array_equal(W_ref > 0, W_got > 0), call
        ok = W_ref > 0
        assert ok.mean() > 0.5
        assert _rel(S_got[ok] / W_got[ok], S_ref[ok] / W_ref[ok]) <= STACK_REL_TOL, call
        assert _rel(W_got[ok], W_ref[ok]) <= STACK_REL_TOL, call


def test_noalloc_rejects_oversized_batches():
    import torch
    from serstacker_gb300 import capi as CA
    lib = CA.lib()
    model = CA.motion(CA.AFFINE)
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    n = 4096 + 1
    rc = lib.sst_weighted_average_add_warped_batch_noalloc(
        dummy.data_ptr(), CA.DEPTH_F32, n, 4, 4, 16, 64, 1.0, C.byref(model), dummy.data_ptr(), None, None,
        CA.BORDER_REFLECT101, dummy.data_ptr(), 4, 4, None)
    assert rc == -1
    assert "SST_NOALLOC_MAX_FRAMES" in CA.last_error()
