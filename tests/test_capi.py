"""The C-ABI library loads and exports every symbol the header declares;
host-side argument checking works without a GPU (no compute calls)."""
import ctypes as C

import numpy as np
import pytest


def test_library_exports_every_header_symbol(capi):
    lib = capi.lib()
    names = capi.exported_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_default_options_match_reference(capi):
    """c_ecch_options defaults (ecc2.h:158-172)."""
    o = capi.default_options()
    assert o.epsx == pytest.approx(1e-5)
    assert o.reference_smooth_sigma == 1 and o.input_smooth_sigma == 1
    assert o.update_step_scale == 1
    assert o.method == capi.ICLM
    assert o.max_iterations == 50 and o.minimum_image_size == 8 and o.maxlevel == 0


def test_invalid_arguments_are_rejected_without_gpu(capi):
    lib = capi.lib()
    h = C.c_void_p()
    o = capi.default_options(interpolation=3)
    assert lib.sst_ecch_create(C.byref(h), C.byref(o)) == -3
    assert "LINEAR" in capi.last_error()
    o = capi.default_options()
    assert lib.sst_ecch_create(C.byref(h), C.byref(o)) == 0
    # no reference image yet
    frames = np.zeros((1, 8, 8), np.float32)
    models = (capi.MotionModel * 1)(capi.motion(capi.AFFINE))
    rc = lib.sst_ecch_align_batch(h, frames.ctypes.data, 5, 1, 8, 8, 32, 256, 1.0, 0, 1, models, 0,
                                  None, None, None, None, None, None, None)
    assert rc == -4 and "reference" in capi.last_error()
    assert lib.sst_ecch_destroy(h) == 0
    assert lib.sst_extract_bayer_planes_u16(None, 4, 4, 8, None, None) == -1


def test_device_count_without_gpu_is_safe(capi):
    assert capi.lib().sst_device_count() >= 0


def test_kernel_launch_counter(capi):
    capi.kernel_launch_count(reset=True)
    assert capi.kernel_launch_count() == 0
