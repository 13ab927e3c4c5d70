"""ctypes binding of the C ABI in ``include/serstacker_gb300.h``.

Thin Python classes with the reference's names (``c_ecch``,
``c_weigthed_average``, ``c_bayer_average``, ``c_eccflow``,
``c_local_variance_sharpness_measure``, ``c_ser_reader``, ``c_ser_writer``)
over ``libsst_gb300.so``. Host numpy buffers are
passed with ``on_device=0``; device buffers (e.g. torch CUDA tensors) with
``on_device=1`` and their ``data_ptr()``. Errors raise ``SSTError`` carrying
``sst_last_error()``. There is no CPU fallback: if the library cannot be
loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build

# status / enums (serstacker_gb300.h)
SST_OK = 0
ERR_INVALID_ARG, ERR_CUDA, ERR_UNSUPPORTED, ERR_STATE, ERR_NOMEM, ERR_TIMEOUT, ERR_IO = -1, -2, -3, -4, -5, -6, -7
FRAME_OK, FRAME_SINGULAR, FRAME_EMPTY_MASK, FRAME_LOW_RHO, FRAME_NAN, FRAME_NOT_INVERTIBLE = range(6)
TRANSLATION, EUCLIDEAN, SCALED_EUCLIDEAN, AFFINE, HOMOGRAPHY, SEMI_QUADRATIC, QUADRATIC, EPIPOLAR = range(8)
FA, IC, LM, ICLM = range(4)
BORDER_CONSTANT, BORDER_REPLICATE, BORDER_REFLECT, BORDER_REFLECT101 = 0, 1, 2, 4
COLORID_BAYER_RGGB, COLORID_BAYER_GRBG, COLORID_BAYER_GBRG, COLORID_BAYER_BGGR = 8, 9, 10, 11
DEPTH_U8, DEPTH_U16, DEPTH_F32 = 0, 2, 5
DEPTH_S32, DEPTH_F64 = 4, 6           # reported by SER files only

_NP_DEPTH = {np.dtype(np.uint8): DEPTH_U8, np.dtype(np.uint16): DEPTH_U16, np.dtype(np.float32): DEPTH_F32}


class SSTError(RuntimeError):
    pass


class MotionModel(C.Structure):
    _fields_ = [("type", C.c_int32), ("fix_translation", C.c_int32), ("fix_rotation", C.c_int32),
                ("fix_scale", C.c_int32)]


def motion(t: int) -> MotionModel:
    """create_image_transform(t): EUCLIDEAN fixes the scale (image_transform.cc:35-39)."""
    return MotionModel(t, 0, 0, 1 if t == EUCLIDEAN else 0)


def nparams(t: int) -> int:
    return {TRANSLATION: 2, EUCLIDEAN: 3, SCALED_EUCLIDEAN: 4, AFFINE: 6, HOMOGRAPHY: 8, SEMI_QUADRATIC: 8,
            QUADRATIC: 12, EPIPOLAR: 8}[t]


class EcchOptions(C.Structure):
    """c_ecch_options (ecc2.h:158-172) + the registration's min_rho."""
    _fields_ = [("epsx", C.c_double), ("reference_smooth_sigma", C.c_double), ("input_smooth_sigma", C.c_double),
                ("update_step_scale", C.c_double), ("method", C.c_int32), ("interpolation", C.c_int32),
                ("max_iterations", C.c_int32), ("minimum_image_size", C.c_int32), ("maxlevel", C.c_int32),
                ("min_rho", C.c_double), ("ic_jacobian_at_identity", C.c_int32), ("reserved", C.c_int32)]


class Tuning(C.Structure):
    """sst_tuning: launch shapes of the engine and the accumulator (0 = default)."""
    _fields_ = [("pass_ctas_per_sm", C.c_int32), ("pass_tile_w", C.c_int32 * 4), ("corr_ctas_per_sm", C.c_int32),
                ("stack_max_chunks", C.c_int32), ("stack_items_per_slot", C.c_int32)]

    @classmethod
    def from_dict(cls, d: dict) -> "Tuning":
        t = cls()
        for k, v in (d or {}).items():
            if k == "pass_tile_w":
                for i, x in enumerate(v):
                    t.pass_tile_w[i] = int(x)
            else:
                setattr(t, k, int(v))
        return t

    def to_dict(self) -> dict:
        return {"pass_ctas_per_sm": self.pass_ctas_per_sm, "pass_tile_w": list(self.pass_tile_w),
                "corr_ctas_per_sm": self.corr_ctas_per_sm, "stack_max_chunks": self.stack_max_chunks,
                "stack_items_per_slot": self.stack_items_per_slot}


class EccRegistrationOptions(C.Structure):
    """c_ecc_registration_options (c_frame_registration.h:47-63)."""
    _fields_ = [("scale", C.c_double), ("eps", C.c_double), ("min_rho", C.c_double),
                ("input_smooth_sigma", C.c_double), ("reference_smooth_sigma", C.c_double),
                ("update_step_scale", C.c_double), ("normalization_noise", C.c_double), ("se_radius", C.c_int32),
                ("ecc_method", C.c_int32), ("max_iterations", C.c_int32), ("ecch_max_level", C.c_int32),
                ("ecch_minimum_image_size", C.c_int32), ("normalization_scale", C.c_int32),
                ("ecch_estimate_translation_first", C.c_int32), ("replace_planetary_disk_with_mask", C.c_int32)]


class EccflowRegistrationOptions(C.Structure):
    """c_eccflow_registration_options (c_frame_registration.h:88-100)."""
    _fields_ = [("update_multiplier", C.c_double), ("input_smooth_sigma", C.c_double),
                ("reference_smooth_sigma", C.c_double), ("noise_level", C.c_double), ("scale_factor", C.c_double),
                ("max_iterations", C.c_int32), ("support_scale", C.c_int32), ("min_image_size", C.c_int32),
                ("max_pyramid_level", C.c_int32), ("downscale_method", C.c_int32), ("reserved", C.c_int32)]


class ImageRegistrationOptions(C.Structure):
    """c_image_registration_options (c_frame_registration.h:119-137)."""
    _fields_ = [("motion_type", C.c_int32), ("ecc_registration_channel", C.c_int32), ("interpolation", C.c_int32),
                ("border_mode", C.c_int32), ("border_value", C.c_double), ("ecc", EccRegistrationOptions),
                ("eccflow", EccflowRegistrationOptions), ("enable_feature_registration", C.c_int32),
                ("enable_ecc_registration", C.c_int32), ("enable_eccflow_registration", C.c_int32),
                ("accumulate_and_compensate_turbulent_flow", C.c_int32)]


_lib = None
LIB_PATH = _build.LIB


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        p, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
        sigs = {
            "sst_last_error": (C.c_char_p, []),
            "sst_version": (C.c_char_p, []),
            "sst_device_count": (i, []),
            "sst_kernel_launch_count": (C.c_longlong, [i]),
            "sst_ecch_options_default": (None, [p]),
            "sst_ecch_create": (i, [p, p]),
            "sst_ecch_destroy": (i, [p]),
            "sst_ecch_set_reference_image": (i, [p, p, i, i, i, sz, d, p, sz, i, p]),
            "sst_ecch_num_levels": (i, [p]),
            "sst_ecch_align_batch": (i, [p, p, i, i, i, i, sz, sz, d, i, i, p, i, p, p, p, p, p, p, p]),
            "sst_ecch_align_plain": (i, [p, p, i, i, i, i, sz, sz, d, i, i, p, i, p, p, p, p, p, p, p]),
            "sst_set_chunk_frames": (i, [p, i]),
            "sst_ecch_set_level_loops": (i, [p, i]),
            "sst_ecch_level_stats": (i, [p, i, i, p, p, p]),
            "sst_ecch_reference_image": (i, [p, i, p, i]),
            "sst_ecch_current_image": (i, [p, i, i, p, i]),
            "sst_weighted_average_create": (i, [p, i, i]),
            "sst_weighted_average_destroy": (i, [p]),
            "sst_weighted_average_clear": (i, [p, p]),
            "sst_weighted_average_add": (i, [p, p, i, sz, d, p, i, sz, i, p]),
            "sst_weighted_average_add_warped_batch": (i, [p, p, i, i, i, i, sz, sz, d, i, p, p, p, p, i, p]),
            "sst_weighted_average_compute": (i, [p, p, p, i, p]),
            "sst_weighted_average_get_acc_counters": (i, [p, p, i, p]),
            "sst_weighted_average_reinitialize": (i, [p, p, p, i, p]),
            "sst_weighted_average_accumulated_frames": (i, [p]),
            "sst_weighted_average_save_state": (i, [p, p, p, p]),
            "sst_weighted_average_load_state": (i, [p, p, C.c_int32, p]),
            "sst_stack_frames": (i, [p, p, p, i, i, i, i, sz, sz, d, i, i, p, i, i, p, p, p, p, p]),
            "sst_remap": (i, [p, i, i, i, sz, d, p, p, i, p, p, i, i, p]),
            "sst_extract_bayer_planes_u16": (i, [p, i, i, sz, p, p]),
            "sst_average_bayer_planes_u16": (i, [p, i, i, sz, p, p]),
            "sst_weighted_average_add_warped_batch_noalloc": (i, [p, i, i, i, i, sz, sz, d, p, p, p, p, i, p, i, i,
                                                                  p]),
            "sst_state_merge": (i, [p, p, i, sz]),
            "sst_warp_residual": (i, [p, i, i, i, sz, p, p, p, p, p, p, p, p, p, p, p]),
            "sst_eccflow_options_default": (None, [p]),
            "sst_eccflow_create": (i, [p, p]),
            "sst_eccflow_destroy": (i, [p]),
            "sst_eccflow_set_reference_image": (i, [p, p, i, i, i, sz, d, i, p]),
            "sst_eccflow_num_levels": (i, [p]),
            "sst_eccflow_compute_batch": (i, [p, p, i, i, sz, sz, d, i, p, p, p]),
            "sst_eccflow_set_reference_image_masked": (i, [p, p, i, i, i, sz, d, p, sz, i, p]),
            "sst_eccflow_compute_batch_masked": (i, [p, p, i, i, sz, sz, d, p, sz, sz, i, p, p, p]),
            "sst_roi_batch_create": (i, [p, p]),
            "sst_roi_batch_destroy": (i, [p]),
            "sst_roi_batch_align": (i, [p, i, p, p, p, i, d, i, i, p, p, p, p, p, p, p, p]),
            "sst_roi_batch_level_stats": (i, [p, i, i, p, p, p, p]),
            "sst_stack_bayer_frames": (i, [p, p, p, i, i, i, sz, sz, d, i, i, p, i, i, p, p, p, p, p]),
            "sst_bayer_average_create": (i, [p, i, i, i]),
            "sst_bayer_average_destroy": (i, [p]),
            "sst_bayer_average_clear": (i, [p, p]),
            "sst_bayer_average_add_batch": (i, [p, p, i, i, sz, sz, d, i, p, p, p, p, p]),
            "sst_bayer_average_compute": (i, [p, p, p, p, i, p]),
            "sst_bayer_average_accumulated_frames": (i, [p]),
            "sst_bayer_average_save_state": (i, [p, p, p, p]),
            "sst_bayer_average_load_state": (i, [p, p, C.c_int32, p]),
            "sst_local_variance_options_default": (None, [p]),
            "sst_local_variance_create": (i, [p, p]),
            "sst_local_variance_destroy": (i, [p]),
            "sst_local_variance_compute": (i, [p, p, i, i, i, i, sz, sz, d, i, p, p, p]),
            "sst_weighted_average_set_local_variance": (i, [p, p]),
            "sst_ser_open": (i, [p, C.c_char_p]),
            "sst_ser_close": (i, [p]),
            "sst_ser_get_info": (i, [p, p]),
            "sst_ser_timestamps": (i, [p, p, i]),
            "sst_ser_curpos": (i, [p]),
            "sst_ser_seek": (i, [p, i]),
            "sst_ser_read": (i, [p, i, p, sz, p]),
            "sst_stack_ser": (i, [p, p, p, i, i, i, i, p, i, i, p, p, p, p, p]),
            "sst_ser_writer_create": (i, [p, C.c_char_p, i, i, i, i]),
            "sst_ser_write": (i, [p, p, i, sz, p]),
            "sst_ser_writer_close": (i, [p]),
            "sst_average_pyramid_inpaint": (i, [p, sz, p, sz, i, i, i, p, sz, p, sz, i, p]),
            "sst_calibrate_frames": (i, [p, i, i, i, i, sz, sz, d, p, sz, p, sz, p, sz, sz, p]),
            "sst_debayer_nn2": (i, [p, i, i, i, i, sz, sz, i, p, sz, sz, p]),
            "sst_filter_bad_pixels": (i, [p, i, i, i, i, sz, sz, i, d, p, sz, sz, p]),
            "sst_lpg_options_default": (None, [p]),
            "sst_optimal_dft_size": (i, [i]),
            "sst_focus_stack_options_default": (None, [p]),
            "sst_focus_stack_create": (i, [p, p]),
            "sst_focus_stack_destroy": (i, [p]),
            "sst_focus_stack_clear": (i, [p]),
            "sst_focus_stack_accumulated_frames": (i, [p]),
            "sst_focus_stack_kernel": (i, [p, p, p]),
            "sst_focus_stack_add": (i, [p, p, i, i, i, i, i, sz, sz, d, p, sz, sz, i, p]),
            "sst_focus_stack_compute": (i, [p, p, sz, i, p]),
            "sst_linear_interpolation_inpaint": (i, [p, sz, i, i, i, p, sz, i, p]),
            "sst_fft_average_create": (i, [p]),
            "sst_fft_average_destroy": (i, [p]),
            "sst_fft_average_clear": (i, [p]),
            "sst_fft_average_accumulated_frames": (i, [p]),
            "sst_fft_average_size": (i, [p, p, p]),
            "sst_fft_average_add": (i, [p, p, i, i, i, i, i, sz, sz, d, i, p]),
            "sst_fft_average_compute": (i, [p, p, sz, p, sz, i, p]),
            "sst_canvas_average_create": (i, [p, i, i]),
            "sst_canvas_average_destroy": (i, [p]),
            "sst_canvas_average_clear": (i, [p]),
            "sst_canvas_average_set_canvas_size": (i, [p, i, i]),
            "sst_canvas_average_state": (i, [p, p, p, p, p]),
            "sst_canvas_average_add": (i, [p, p, i, i, i, i, sz, d, p, i, sz, p, p, i, p]),
            "sst_canvas_average_compute": (i, [p, p, sz, p, sz, d, p, p, i, p]),
            "sst_canvas_average_counter": (i, [p, p, sz, i, p]),
            "sst_lpg_create": (i, [p, p]),
            "sst_lpg_destroy": (i, [p]),
            "sst_lpg_compute": (i, [p, p, i, i, i, i, sz, sz, p, sz, sz, i, p, p, p]),
            "sst_ecch_set_tuning": (i, [p, p]),
            "sst_ecch_get_tuning": (i, [p, p]),
            "sst_weighted_average_set_tuning": (i, [p, p]),
            "sst_image_registration_options_default": (None, [p]),
            "sst_frame_registration_create": (i, [p, p]),
            "sst_frame_registration_destroy": (i, [p]),
            "sst_frame_registration_setup_reference_frame": (i, [p, p, i, i, i, sz, d, p, sz, i, p]),
            "sst_frame_registration_register_frames": (i, [p, p, i, i, i, i, sz, sz, d, i, p, p, p, p, p, p]),
            "sst_frame_registration_set_chunk_frames": (i, [p, i]),
            "sst_frame_registration_ecc_size": (i, [p, p, p]),
            "sst_frame_registration_ecc_image": (i, [p, i, p, p, i]),
            "sst_remap_rmap": (i, [p, i, i, i, sz, d, p, i, i, i, d, p, sz, p, p, i, p]),
            "sst_image_transform_scale": (i, [p, p, d]),
            "sst_image_transform_create_remap": (i, [p, p, i, i, p, i, p]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def exported_symbols() -> list:
    """Names of every entry point declared in include/serstacker_gb300.h."""
    import re
    hdr = os.path.join(os.path.dirname(_build.HERE), "include", "serstacker_gb300.h")
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(sst_\w+)\s*\(", open(hdr).read(), re.M)
    return sorted(set(names))


def _check(rc: int, what: str):
    if rc != SST_OK:
        raise SSTError(f"{what} failed ({rc}): {lib().sst_last_error().decode(errors='replace')}")


def last_error() -> str:
    return lib().sst_last_error().decode(errors="replace")


def kernel_launch_count(reset: bool = False) -> int:
    return lib().sst_kernel_launch_count(1 if reset else 0)


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if isinstance(a, int):
        return a
    return a.data_ptr()   # torch tensor


def default_options(**kw) -> EcchOptions:
    o = EcchOptions()
    lib().sst_ecch_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class c_ecch:
    """Batched c_ecch (ecc2.h:193-308) over the C ABI."""

    def __init__(self, options: Optional[EcchOptions] = None, **kw):
        self.options = options if options is not None else default_options(**kw)
        self._h = C.c_void_p()
        _check(lib().sst_ecch_create(C.byref(self._h), C.byref(self.options)), "sst_ecch_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_ecch_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def set_reference_image(self, image: np.ndarray, mask: Optional[np.ndarray] = None, scale: float = 1.0):
        img = np.ascontiguousarray(image)
        depth = _NP_DEPTH[img.dtype]
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        _check(lib().sst_ecch_set_reference_image(self._h, _ptr(img), depth, img.shape[1], img.shape[0],
                                                  img.strides[0], scale, _ptr(m), 0 if m is None else m.strides[0],
                                                  0, None), "set_reference_image")
        self._ref_shape = img.shape[:2]

    def level_shape(self, level: int):
        """(height, width) of a pyramid level: c_ecch::compute_next_pyramid_layer_size per level."""
        hh, ww = self._ref_shape
        for _ in range(level):
            hh, ww = ((hh + 1) // 2) & ~1, ((ww + 1) // 2) & ~1
        return hh, ww

    def reference_image(self, level: int = 0) -> np.ndarray:
        """The engine's reference pyramid level (converted, pre-smoothed, pyrDown'ed)."""
        out = np.empty(self.level_shape(level), np.float32)
        _check(lib().sst_ecch_reference_image(self._h, level, _ptr(out), 0), "reference_image")
        return out

    def current_image(self, frame: int, level: int = 0) -> np.ndarray:
        """Frame `frame`'s pyramid level from the last registration call."""
        out = np.empty(self.level_shape(level), np.float32)
        _check(lib().sst_ecch_current_image(self._h, frame, level, _ptr(out), 0), "current_image")
        return out

    def num_levels(self) -> int:
        return lib().sst_ecch_num_levels(self._h)

    def set_tuning(self, tuning):
        t = tuning if isinstance(tuning, Tuning) else Tuning.from_dict(tuning)
        _check(lib().sst_ecch_set_tuning(self._h, C.byref(t)), "sst_ecch_set_tuning")

    def get_tuning(self) -> dict:
        t = Tuning()
        _check(lib().sst_ecch_get_tuning(self._h, C.byref(t)), "sst_ecch_get_tuning")
        return t.to_dict()

    def set_chunk_frames(self, n: int):
        _check(lib().sst_set_chunk_frames(self._h, n), "set_chunk_frames")

    def set_level_loops(self, enable: bool):
        """Level iterations as graph WHILE loops (default) or the unrolled schedule."""
        _check(lib().sst_ecch_set_level_loops(self._h, 1 if enable else 0), "set_level_loops")

    def level_stats(self, pass_index: int, level: int):
        """(ms, frame_iterations, algorithmic_bytes) of the last call at one pass / level."""
        ms, fi, ab = C.c_float(), C.c_double(), C.c_double()
        _check(lib().sst_ecch_level_stats(self._h, pass_index, level, C.byref(ms), C.byref(fi), C.byref(ab)),
               "level_stats")
        return ms.value, fi.value, ab.value

    def align(self, frames: np.ndarray, passes: Sequence[int], scale: float = 1.0, init_params=None,
              plain: bool = False):
        """Register a (n, h, w) stack of host frames. Returns a dict of arrays."""
        fr = np.ascontiguousarray(frames)
        if fr.ndim == 2:
            fr = fr[None]
        n, hh, ww = fr.shape
        depth = _NP_DEPTH[fr.dtype]
        models = (MotionModel * len(passes))(*[motion(t) for t in passes])
        params = np.zeros((n, 12), np.float32)
        if init_params is not None:
            ip = np.asarray(init_params, np.float32)
            params[:, :ip.shape[-1]] = ip
        status = np.zeros(n, np.int32)
        iters = np.zeros(n, np.int32)
        eps = np.zeros(n, np.float32)
        rho = np.zeros(n, np.float32)
        weight = np.zeros(n, np.float32)
        fn = lib().sst_ecch_align_plain if plain else lib().sst_ecch_align_batch
        _check(fn(self._h, _ptr(fr), depth, n, ww, hh, fr.strides[1], fr.strides[0], scale, 0, len(passes), models,
                  1 if init_params is not None else 0, _ptr(params), _ptr(status), _ptr(iters), _ptr(eps), _ptr(rho),
                  _ptr(weight), None), "align")
        M = nparams(passes[-1])
        return {"params": params[:, :M], "status": status, "iterations": iters, "eps": eps, "rho": rho,
                "weight": weight}


class EccflowOptions(C.Structure):
    """c_eccflow_options (ecc2.h:515-527)"""
    _fields_ = [("update_multiplier", C.c_double), ("scale_factor", C.c_double), ("noise_level", C.c_double),
                ("input_smooth_sigma", C.c_double), ("reference_smooth_sigma", C.c_double),
                ("max_iterations", C.c_int32), ("support_scale", C.c_int32), ("min_image_size", C.c_int32),
                ("max_pyramid_level", C.c_int32), ("downscale", C.c_int32), ("reserved", C.c_int32)]


def eccflow_options(**kw) -> EccflowOptions:
    o = EccflowOptions()
    lib().sst_eccflow_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class c_eccflow:
    """c_eccflow (ecc2.h:548-662) over sst_eccflow_*: dense flow of a batch of
    frames against one reference."""

    def __init__(self, options: Optional[EccflowOptions] = None):
        self._h = C.c_void_p()
        o = options if options is not None else eccflow_options()
        _check(lib().sst_eccflow_create(C.byref(self._h), C.byref(o)), "sst_eccflow_create")
        self.shape = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_eccflow_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def set_reference_image(self, img: np.ndarray, scale: float = 1.0, mask: Optional[np.ndarray] = None):
        a = np.ascontiguousarray(img)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        _check(lib().sst_eccflow_set_reference_image_masked(
            self._h, _ptr(a), _NP_DEPTH[a.dtype], a.shape[1], a.shape[0], a.strides[0], scale, _ptr(m),
            0 if m is None else m.strides[0], 0, None), "set_reference_image")
        self.shape = a.shape

    def num_levels(self) -> int:
        return lib().sst_eccflow_num_levels(self._h)

    def compute(self, frames: np.ndarray, init_rmap=None, scale: float = 1.0, masks: Optional[np.ndarray] = None):
        """frames (n, h, w) (+ masks (n, h, w) u8) -> rmaps (n, h, w, 2) = identity + flow"""
        fr = np.ascontiguousarray(frames)
        if fr.ndim == 2:
            fr = fr[None]
        n, hh, ww = fr.shape
        out = np.zeros((n, hh, ww, 2), np.float32)
        init = None if init_rmap is None else np.ascontiguousarray(init_rmap, np.float32).reshape(n, hh, ww, 2)
        m = None if masks is None else np.ascontiguousarray(masks, np.uint8).reshape(n, hh, ww)
        _check(lib().sst_eccflow_compute_batch_masked(
            self._h, _ptr(fr), _NP_DEPTH[fr.dtype], n, fr.strides[1], fr.strides[0], scale, _ptr(m),
            0 if m is None else m.strides[1], 0 if m is None else m.strides[0], 0, _ptr(init), _ptr(out), None),
            "sst_eccflow_compute_batch")
        return out

    def compute_device(self, frames, n, depth, row_stride, frame_stride, rmap_out, init_rmap=None, scale=1.0):
        _check(lib().sst_eccflow_compute_batch(self._h, _ptr(frames), depth, n, row_stride, frame_stride, scale, 1,
                                               _ptr(init_rmap), _ptr(rmap_out), None), "sst_eccflow_compute_batch")
        return rmap_out


class Roi(C.Structure):
    _fields_ = [("ref_offset", C.c_int64), ("cur_offset", C.c_int64), ("ref_row_stride", C.c_int64),
                ("cur_row_stride", C.c_int64), ("width", C.c_int32), ("height", C.c_int32)]


def pack_rois(refs, curs):
    """Pack lists of same-dtype 2D crops (reference i and current i of equal
    size) into two contiguous pools; returns (ref_pool, cur_pool, Roi array)."""
    if len(refs) != len(curs) or not refs:
        raise ValueError("refs and curs must be non-empty lists of equal length")
    dt = np.asarray(refs[0]).dtype
    sizes = [np.asarray(r).size for r in refs]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    ref_pool = np.empty(int(offs[-1]), dt)
    cur_pool = np.empty(int(offs[-1]), dt)
    rois = (Roi * len(refs))()
    for i, (r, c) in enumerate(zip(refs, curs)):
        r = np.asarray(r, dt)
        c = np.asarray(c, dt)
        if r.shape != c.shape:
            raise ValueError(f"crop {i}: reference and current sizes differ")
        hh, ww = r.shape
        ref_pool[offs[i]:offs[i + 1]] = r.ravel()
        cur_pool[offs[i]:offs[i + 1]] = c.ravel()
        b = dt.itemsize
        rois[i] = Roi(int(offs[i]) * b, int(offs[i]) * b, ww * b, ww * b, ww, hh)
    return ref_pool, cur_pool, rois


class c_roi_batch:
    """A batch of independent c_ecch problems of different sizes (crop i
    registered against reference crop i) over sst_roi_batch_*."""

    def __init__(self, options: EcchOptions):
        self._h = C.c_void_p()
        _check(lib().sst_roi_batch_create(C.byref(self._h), C.byref(options)), "sst_roi_batch_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_roi_batch_destroy(h)
            self._h = C.c_void_p()

    def align(self, refs, curs, passes: Sequence[int], scale: float = 1.0, init_params=None):
        ref_pool, cur_pool, rois = pack_rois(refs, curs)
        n = len(refs)
        models = (MotionModel * len(passes))(*[motion(t) for t in passes])
        ip = None
        if init_params is not None:
            ip = np.zeros((n, 12), np.float32)
            pp = np.asarray(init_params, np.float32).reshape(n, -1)
            ip[:, :pp.shape[1]] = pp
        out = {"params": np.zeros((n, 12), np.float32), "status": np.zeros(n, np.int32),
               "iterations": np.zeros(n, np.int32), "eps": np.zeros(n, np.float32), "rho": np.zeros(n, np.float32)}
        _check(lib().sst_roi_batch_align(self._h, n, rois, _ptr(ref_pool), _ptr(cur_pool), _NP_DEPTH[ref_pool.dtype],
                                         scale, 0, len(passes), models, _ptr(ip), _ptr(out["params"]),
                                         _ptr(out["status"]), _ptr(out["iterations"]), _ptr(out["eps"]),
                                         _ptr(out["rho"]), None), "sst_roi_batch_align")
        return out

    def align_device(self, n, rois, ref_pool, cur_pool, depth, passes: Sequence[int], scale: float, outputs,
                     init_params=None):
        """Device-resident pools (torch tensors or pointers) and outputs."""
        models = (MotionModel * len(passes))(*[motion(t) for t in passes])
        _check(lib().sst_roi_batch_align(self._h, n, rois, _ptr(ref_pool), _ptr(cur_pool), depth, scale, 1,
                                         len(passes), models, _ptr(init_params), _ptr(outputs.get("params")),
                                         _ptr(outputs.get("status")), _ptr(outputs.get("iterations")),
                                         _ptr(outputs.get("eps")), _ptr(outputs.get("rho")), None),
               "sst_roi_batch_align")
        return outputs

    def level_stats(self, pass_index: int, level: int):
        ms = C.c_float()
        fi, px, ab = C.c_double(), C.c_double(), C.c_double()
        _check(lib().sst_roi_batch_level_stats(self._h, pass_index, level, C.byref(ms), C.byref(fi), C.byref(px),
                                               C.byref(ab)), "level_stats")
        return ms.value, fi.value, px.value, ab.value


class LocalVarianceOptions(C.Structure):
    """c_local_variance_map_options (c_local_variance_sharpness_measure.h:17-23)"""
    _fields_ = [("kradius", C.c_int), ("dscale", C.c_int), ("uscale", C.c_int)]


def local_variance_options(**kw) -> LocalVarianceOptions:
    o = LocalVarianceOptions()
    lib().sst_local_variance_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class c_local_variance_sharpness_measure:
    """c_local_variance_sharpness_measure::create_map over the C ABI."""

    def __init__(self, options: Optional[LocalVarianceOptions] = None, **kw):
        self.options = options if options is not None else local_variance_options(**kw)
        self._h = C.c_void_p()
        _check(lib().sst_local_variance_create(C.byref(self._h), C.byref(self.options)), "sst_local_variance_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_local_variance_destroy(h)
            self._h = C.c_void_p()

    def create_maps(self, frames: np.ndarray, scale: float = 1.0):
        """frames (n, h, w) or (h, w) -> (maps (n, h, w) float32, q (n,) float64)"""
        f = np.ascontiguousarray(frames)
        if f.ndim == 2:
            f = f[None]
        n, h, w = f.shape
        maps = np.zeros((n, h, w), np.float32)
        q = np.zeros(n, np.float64)
        _check(lib().sst_local_variance_compute(self._h, _ptr(f), _NP_DEPTH[f.dtype], n, w, h, f.strides[1],
                                                 f.strides[0], scale, 0, _ptr(maps), _ptr(q), None),
               "sst_local_variance_compute")
        return maps, q


class LpgOptions(C.Structure):
    """c_lpg_options (c_lpg_sharpness_measure.h:22-28)"""
    _fields_ = [("k", C.c_double), ("p", C.c_double), ("dscale", C.c_int32), ("uscale", C.c_int32)]


def lpg_options(**kw) -> LpgOptions:
    o = LpgOptions()
    lib().sst_lpg_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class c_lpg_sharpness_measure:
    """c_lpg_sharpness_measure (c_lpg_sharpness_measure.h:44-80) over the C
    ABI: lpg() maps and metrics of batches of mono frames."""

    def __init__(self, options: Optional[LpgOptions] = None, **kw):
        self.options = options if options is not None else lpg_options(**kw)
        self._h = C.c_void_p()
        _check(lib().sst_lpg_create(C.byref(self._h), C.byref(self.options)), "sst_lpg_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_lpg_destroy(h)
            self._h = C.c_void_p()

    def compute(self, frames: np.ndarray, masks: Optional[np.ndarray] = None):
        """frames (n, h, w) or (h, w) u8 / u16 / f32, masks of the same shape
        (u8, nonzero = valid) or None -> (maps (n, h, w) float32, metrics (n,)
        float64)"""
        f = np.ascontiguousarray(frames)
        if f.ndim == 2:
            f = f[None]
        n, h, w = f.shape
        mk = None
        if masks is not None:
            mk = np.ascontiguousarray(masks, dtype=np.uint8).reshape(n, h, w)
        maps = np.zeros((n, h, w), np.float32)
        metrics = np.zeros(n, np.float64)
        _check(lib().sst_lpg_compute(self._h, _ptr(f), _NP_DEPTH[f.dtype], n, w, h, f.strides[1], f.strides[0],
                                     None if mk is None else _ptr(mk), w, w * h, 0, _ptr(maps), _ptr(metrics), None),
               "sst_lpg_compute")
        return maps, metrics


def _hwc(a):
    """(h, w) or (h, w, cn) -> contiguous array and (h, w, cn)"""
    a = np.ascontiguousarray(a)
    h, w = a.shape[:2]
    return a, h, w, (a.shape[2] if a.ndim == 3 else 1)


class c_frame_accumulation_with_fft:
    """c_frame_accumulation_with_fft (c_frame_accumulation.h:168-199) over the
    C ABI: frames (h, w) or (h, w, cn) u8 / u16 / f32."""

    def __init__(self):
        self._h = C.c_void_p()
        _check(lib().sst_fft_average_create(C.byref(self._h)), "sst_fft_average_create")
        self._cn, self._shape = 1, None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_fft_average_destroy(h)
            self._h = C.c_void_p()

    def add(self, frame, scale: float = 1.0):
        """one frame (h, w) or (h, w, cn)"""
        a, h, w, cn = _hwc(frame)
        self.add_batch(a.reshape(1, h, w, cn), scale)

    def add_batch(self, frames, scale: float = 1.0):
        """frames (n, h, w) or (n, h, w, cn)"""
        f = np.ascontiguousarray(frames)
        n, h, w = f.shape[:3]
        cn = f.shape[3] if f.ndim == 4 else 1
        _check(lib().sst_fft_average_add(self._h, _ptr(f), _NP_DEPTH[f.dtype], n, w, h, cn, f.strides[1],
                                         f.strides[0], scale, 0, None), "sst_fft_average_add")
        self._cn, self._shape = cn, (h, w)

    def compute(self):
        if not self.accumulated_frames():
            raise SSTError("c_frame_accumulation_with_fft: accumulator is empty")
        cn = self._cn
        h, w = self._shape
        avg = np.zeros((h, w, cn), np.float32)
        mask = np.zeros((h, w), np.uint8)
        _check(lib().sst_fft_average_compute(self._h, _ptr(avg), 0, _ptr(mask), 0, 0, None), "sst_fft_average_compute")
        return (avg[..., 0] if cn == 1 else avg), mask

    def fft_size(self):
        fw, fh = C.c_int(), C.c_int()
        _check(lib().sst_fft_average_size(self._h, C.byref(fw), C.byref(fh)), "sst_fft_average_size")
        return fw.value, fh.value

    def accumulated_frames(self) -> int:
        return lib().sst_fft_average_accumulated_frames(self._h)

    def clear(self):
        _check(lib().sst_fft_average_clear(self._h), "clear")


def fft_average(frames, scale: float = 1.0):
    """c_frame_accumulation_with_fft over a batch: frames (n, h, w) or
    (n, h, w, cn) -> (avg, mask)"""
    acc = c_frame_accumulation_with_fft()
    acc.add_batch(frames, scale)
    return acc.compute()


SELECT_MAX_ENERGY, WEIGHTED_AVERAGE = 0, 1


class FocusStackOptions(C.Structure):
    """c_laplacian_pyramid_focus_stacking::options (c_frame_accumulation.h:158-164)"""
    _fields_ = [("fusing_policy", C.c_int32), ("inpaint_mask_holes", C.c_int32), ("avgchannel", C.c_int32),
                ("kradius", C.c_int32), ("ksigma", C.c_double)]


def focus_stack_options(**kw) -> FocusStackOptions:
    o = FocusStackOptions()
    lib().sst_focus_stack_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class c_laplacian_pyramid_focus_stacking:
    """c_laplacian_pyramid_focus_stacking (c_frame_accumulation.h:149-191)
    over the C ABI: frames (h, w) or (h, w, cn)."""

    def __init__(self, options: Optional[FocusStackOptions] = None, **kw):
        self.options = options if options is not None else focus_stack_options(**kw)
        self._h = C.c_void_p()
        _check(lib().sst_focus_stack_create(C.byref(self._h), C.byref(self.options)), "sst_focus_stack_create")
        self._cn, self._shape = 1, None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_focus_stack_destroy(h)
            self._h = C.c_void_p()

    def add(self, frame, mask=None, scale: float = 1.0):
        a, h, w, cn = _hwc(frame)
        self.add_batch(a.reshape(1, h, w, cn), None if mask is None else np.asarray(mask)[None], scale)

    def add_batch(self, frames, masks=None, scale: float = 1.0):
        """frames (n, h, w) or (n, h, w, cn); masks (n, h, w) u8 or None"""
        f = np.ascontiguousarray(frames)
        n, h, w = f.shape[:3]
        cn = f.shape[3] if f.ndim == 4 else 1
        m = None if masks is None else np.ascontiguousarray(masks, np.uint8).reshape(n, h, w)
        _check(lib().sst_focus_stack_add(self._h, _ptr(f), _NP_DEPTH[f.dtype], n, w, h, cn, f.strides[1], f.strides[0],
                                         scale, _ptr(m), w, w * h, 0, None), "sst_focus_stack_add")
        self._cn, self._shape = cn, (h, w)

    def compute(self):
        h, w = self._shape
        avg = np.zeros((h, w, self._cn), np.float32)
        _check(lib().sst_focus_stack_compute(self._h, _ptr(avg), 0, 0, None), "sst_focus_stack_compute")
        return avg[..., 0] if self._cn == 1 else avg

    def kernel(self):
        n = C.c_int()
        _check(lib().sst_focus_stack_kernel(self._h, None, C.byref(n)), "kernel")
        k = np.zeros(n.value, np.float32)
        if n.value:
            _check(lib().sst_focus_stack_kernel(self._h, _ptr(k), C.byref(n)), "kernel")
        return k

    def accumulated_frames(self) -> int:
        return lib().sst_focus_stack_accumulated_frames(self._h)

    def clear(self):
        _check(lib().sst_focus_stack_clear(self._h), "clear")


def linear_interpolation_inpaint(image, mask):
    """sst_linear_interpolation_inpaint: image (h, w) or (h, w, cn) f32, u8
    mask (0 = hole) -> the filled image"""
    a, h, w, cn = _hwc(np.asarray(image, np.float32))
    a = a.copy()
    m = np.ascontiguousarray(mask, np.uint8)
    _check(lib().sst_linear_interpolation_inpaint(_ptr(a), a.strides[0], w, h, cn, _ptr(m), m.strides[0], 0, None),
           "sst_linear_interpolation_inpaint")
    return a


class c_canvas_average:
    """c_canvas_average (c_frame_accumulation.h:65-146) over the C ABI."""

    def __init__(self, canvas_size=(0, 0)):
        self._h = C.c_void_p()
        _check(lib().sst_canvas_average_create(C.byref(self._h), int(canvas_size[0]), int(canvas_size[1])),
               "sst_canvas_average_create")
        self._cn = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_canvas_average_destroy(h)
            self._h = C.c_void_p()

    def set_canvas_size(self, size):
        _check(lib().sst_canvas_average_set_canvas_size(self._h, int(size[0]), int(size[1])), "set_canvas_size")

    def add(self, image, weights=None, rmap=None, bbox=None, scale: float = 1.0):
        """image (h, w[, cn]); weights None, u8 mask or f32 (h, w); rmap
        (bh, bw, 2) f32 with bbox (x, y, bw, bh)"""
        a, h, w, cn = _hwc(image)
        self._cn = cn
        wt = None if weights is None else np.ascontiguousarray(weights)
        wd = 0 if wt is None else _NP_DEPTH[wt.dtype]
        rm = None if rmap is None else np.ascontiguousarray(rmap, np.float32)
        bb = None if bbox is None else np.ascontiguousarray(bbox, np.int32)
        _check(lib().sst_canvas_average_add(self._h, _ptr(a), _NP_DEPTH[a.dtype], w, h, cn, a.strides[0], scale,
                                            _ptr(wt), wd, 0 if wt is None else wt.strides[0], _ptr(rm), _ptr(bb), 0,
                                            None), "sst_canvas_average_add")

    def state(self):
        cw, ch, fr = C.c_int(), C.c_int(), C.c_int()
        bb = np.zeros(4, np.int32)
        _check(lib().sst_canvas_average_state(self._h, C.byref(cw), C.byref(ch), _ptr(bb), C.byref(fr)), "state")
        return (cw.value, ch.value), bb, fr.value

    def compute(self, dscale: float = 1.0, rbbox=None):
        (cw, ch), _, _ = self.state()
        rb = None if rbbox is None else np.ascontiguousarray(rbbox, np.int32)
        bw, bh = (cw, ch) if rb is None else (int(rb[2]), int(rb[3]))
        bw, bh = min(bw, cw), min(bh, ch)
        cn = self._cn or 1
        avg = np.zeros((bh, bw, cn), np.float32)
        mask = np.zeros((bh, bw), np.uint8)
        ob = np.zeros(4, np.int32)
        _check(lib().sst_canvas_average_compute(self._h, _ptr(avg), avg.strides[0], _ptr(mask), mask.strides[0], dscale,
                                                _ptr(rb), _ptr(ob), 0, None), "sst_canvas_average_compute")
        avg, mask = avg[:ob[3], :ob[2]], mask[:ob[3], :ob[2]]
        return (avg[..., 0] if cn == 1 else avg), mask

    def counter(self):
        (cw, ch), _, _ = self.state()
        W = np.zeros((ch, cw), np.float32)
        _check(lib().sst_canvas_average_counter(self._h, _ptr(W), 0, 0, None), "counter")
        return W


class c_weigthed_average:
    """c_weigthed_average (c_frame_accumulation.h:39-63) over the C ABI."""

    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self._h = C.c_void_p()
        _check(lib().sst_weighted_average_create(C.byref(self._h), width, height), "sst_weighted_average_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_weighted_average_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def clear(self):
        _check(lib().sst_weighted_average_clear(self._h, None), "clear")

    def set_tuning(self, tuning):
        t = tuning if isinstance(tuning, Tuning) else Tuning.from_dict(tuning)
        _check(lib().sst_weighted_average_set_tuning(self._h, C.byref(t)), "sst_weighted_average_set_tuning")

    def set_local_variance(self, options: Optional[LocalVarianceOptions] = None, **kw):
        """sharpness-map options of stack_frames(weighting=3)"""
        o = options if options is not None else local_variance_options(**kw)
        _check(lib().sst_weighted_average_set_local_variance(self._h, C.byref(o)), "set_local_variance")

    def add(self, src: np.ndarray, weights: Optional[np.ndarray] = None, scale: float = 1.0):
        s = np.ascontiguousarray(src)
        w = None if weights is None else np.ascontiguousarray(weights)
        wd = 0 if w is None else _NP_DEPTH[w.dtype]
        _check(lib().sst_weighted_average_add(self._h, _ptr(s), _NP_DEPTH[s.dtype], s.strides[0], scale, _ptr(w), wd,
                                              0 if w is None else w.strides[0], 0, None), "add")

    def add_warped(self, frames: np.ndarray, motion_type: int, params: np.ndarray, status=None, weights=None,
                   scale: float = 1.0, border: int = BORDER_REFLECT101):
        fr = np.ascontiguousarray(frames)
        if fr.ndim == 2:
            fr = fr[None]
        n, hh, ww = fr.shape
        p = np.zeros((n, 12), np.float32)
        pp = np.asarray(params, np.float32).reshape(n, -1)
        p[:, :pp.shape[1]] = pp
        st = None if status is None else np.ascontiguousarray(status, np.int32)
        wt = None if weights is None else np.ascontiguousarray(weights, np.float32)
        m = motion(motion_type)
        _check(lib().sst_weighted_average_add_warped_batch(self._h, _ptr(fr), _NP_DEPTH[fr.dtype], n, ww, hh,
                                                           fr.strides[1], fr.strides[0], scale, 0, C.byref(m),
                                                           _ptr(p), _ptr(st), _ptr(wt), border, None), "add_warped")

    def compute(self):
        avg = np.zeros((self.height, self.width), np.float32)
        mask = np.zeros((self.height, self.width), np.uint8)
        _check(lib().sst_weighted_average_compute(self._h, _ptr(avg), _ptr(mask), 0, None), "compute")
        return avg, mask

    def get_acc_counters(self):
        w = np.zeros((self.height, self.width), np.float32)
        _check(lib().sst_weighted_average_get_acc_counters(self._h, _ptr(w), 0, None), "get_acc_counters")
        return w

    def reinitialize(self, avg: np.ndarray, accw: np.ndarray):
        a = np.ascontiguousarray(avg, np.float32)
        w = np.ascontiguousarray(accw, np.float32)
        _check(lib().sst_weighted_average_reinitialize(self._h, _ptr(a), _ptr(w), 0, None), "reinitialize")

    def accumulated_frames(self) -> int:
        return lib().sst_weighted_average_accumulated_frames(self._h)

    def save_state(self):
        st = np.zeros((4, self.height, self.width), np.float32)
        fr = C.c_int32()
        _check(lib().sst_weighted_average_save_state(self._h, _ptr(st), C.byref(fr), None), "save_state")
        return st, fr.value

    def load_state(self, state: np.ndarray, frames: int):
        s = np.ascontiguousarray(state, np.float32)
        _check(lib().sst_weighted_average_load_state(self._h, _ptr(s), frames, None), "load_state")


class c_bayer_average:
    """c_bayer_average (c_frame_accumulation.h:222-262) over the C ABI: raw
    mosaic frames in, a 3-channel (B, G, R) average out."""

    def __init__(self, width: int, height: int, colorid: int = COLORID_BAYER_RGGB):
        self.width, self.height, self.colorid = width, height, colorid
        self._h = C.c_void_p()
        _check(lib().sst_bayer_average_create(C.byref(self._h), width, height, colorid), "sst_bayer_average_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_bayer_average_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def clear(self):
        _check(lib().sst_bayer_average_clear(self._h, None), "clear")

    def add(self, frames: np.ndarray, motion_type: Optional[int] = None, params=None, status=None, weights=None,
            scale: float = 1.0):
        """set_remap(transform of params) + add(frame, mask * weight) for each
        frame; motion_type None adds the frames without a remap."""
        fr = np.ascontiguousarray(frames)
        if fr.ndim == 2:
            fr = fr[None]
        n = fr.shape[0]
        m, p = None, None
        if motion_type is not None:
            m = motion(motion_type)
            p = np.zeros((n, 12), np.float32)
            pp = np.asarray(params, np.float32).reshape(n, -1)
            p[:, :pp.shape[1]] = pp
        st = None if status is None else np.ascontiguousarray(status, np.int32)
        wt = None if weights is None else np.ascontiguousarray(weights, np.float32)
        _check(lib().sst_bayer_average_add_batch(self._h, _ptr(fr), _NP_DEPTH[fr.dtype], n, fr.strides[1],
                                                 fr.strides[0], scale, 0, None if m is None else C.byref(m),
                                                 _ptr(p), _ptr(st), _ptr(wt), None), "add")

    def compute(self):
        """(avg (h, w, 3) f32, mask (h, w) u8, accw (h, w, 3) f32 with green halved)"""
        avg = np.zeros((self.height, self.width, 3), np.float32)
        mask = np.zeros((self.height, self.width), np.uint8)
        accw = np.zeros((self.height, self.width, 3), np.float32)
        _check(lib().sst_bayer_average_compute(self._h, _ptr(avg), _ptr(mask), _ptr(accw), 0, None), "compute")
        return avg, mask, accw

    def accumulated_frames(self) -> int:
        return lib().sst_bayer_average_accumulated_frames(self._h)

    def save_state(self):
        st = np.zeros((3, 4, self.height, self.width), np.float32)
        fr = C.c_int32()
        _check(lib().sst_bayer_average_save_state(self._h, _ptr(st), C.byref(fr), None), "save_state")
        return st, fr.value

    def load_state(self, state: np.ndarray, frames: int):
        s = np.ascontiguousarray(state, np.float32)
        _check(lib().sst_bayer_average_load_state(self._h, _ptr(s), frames, None), "load_state")


def stack_frames(reg: c_ecch, acc: c_weigthed_average, frames, passes: Sequence[int], scale: float,
                 weighting: int = 1, border: int = BORDER_REFLECT101, on_device: bool = False, n=None,
                 width=None, height=None, depth=None, row_stride=None, frame_stride=None, outputs=None,
                 host_input: bool = False):
    """sst_stack_frames: register + warp + stack a sequence.

    frames: a numpy (n, h, w) array (host), or a raw pointer / torch tensor with
    explicit n, width, height, depth and strides. `on_device` says where the
    frames and the outputs live; `host_input` marks a raw host pointer (e.g. a
    pinned torch tensor's data_ptr()) whose outputs are host buffers too.
    """
    if isinstance(frames, np.ndarray):
        fr = np.ascontiguousarray(frames)
        n, height, width = fr.shape
        depth = _NP_DEPTH[fr.dtype]
        row_stride, frame_stride = fr.strides[1], fr.strides[0]
        ptr = _ptr(fr)
        dev = 0
    else:
        ptr = _ptr(frames)
        dev = 0 if host_input else (1 if on_device else 0)
    models = (MotionModel * len(passes))(*[motion(t) for t in passes])
    if outputs is None:
        outputs = {"params": np.zeros((n, 12), np.float32), "status": np.zeros(n, np.int32),
                   "rho": np.zeros(n, np.float32), "weight": np.zeros(n, np.float32)}
    _check(lib().sst_stack_frames(reg.handle, acc.handle, ptr, depth, n, width, height, row_stride, frame_stride,
                                  scale, dev, len(passes), models, border, weighting,
                                  _ptr(outputs["params"]), _ptr(outputs["status"]), _ptr(outputs["rho"]),
                                  _ptr(outputs["weight"]), None), "sst_stack_frames")
    return outputs


def stack_bayer_frames(reg: c_ecch, accs: Sequence[c_weigthed_average], frames, passes: Sequence[int],
                       scale: float, weighting: int = 1, border: int = BORDER_REFLECT101, on_device: bool = False,
                       n=None, width=None, height=None, row_stride=None, frame_stride=None, outputs=None,
                       host_input: bool = False):
    """sst_stack_bayer_frames: register the binned luminance of raw u16 mosaic
    frames and stack their four Bayer planes into accs[0..3]."""
    if isinstance(frames, np.ndarray):
        fr = np.ascontiguousarray(frames, np.uint16)
        n, height, width = fr.shape
        row_stride, frame_stride = fr.strides[1], fr.strides[0]
        ptr = _ptr(fr)
        dev = 0
    else:
        ptr = _ptr(frames)
        dev = 0 if host_input else (1 if on_device else 0)
    if len(accs) != 4:
        raise ValueError("four plane accumulators are required")
    handles = (C.c_void_p * 4)(*[a.handle.value for a in accs])
    models = (MotionModel * len(passes))(*[motion(t) for t in passes])
    if outputs is None:
        outputs = {"params": np.zeros((n, 12), np.float32), "status": np.zeros(n, np.int32),
                   "rho": np.zeros(n, np.float32), "weight": np.zeros(n, np.float32)}
    _check(lib().sst_stack_bayer_frames(reg.handle, handles, ptr, n, width, height, row_stride, frame_stride, scale,
                                        dev, len(passes), models, border, weighting, _ptr(outputs["params"]),
                                        _ptr(outputs["status"]), _ptr(outputs["rho"]), _ptr(outputs["weight"]),
                                        None), "sst_stack_bayer_frames")
    return outputs


class SerInfo(C.Structure):
    """sst_ser_info: the SER header as c_ser_reader reads it (c_ser_file.h:42-56)"""
    _fields_ = [("luid", C.c_int32), ("color_id", C.c_int32), ("data_little_endian", C.c_int32),
                ("width", C.c_int32), ("height", C.c_int32), ("bits_per_plane", C.c_int32), ("frames", C.c_int32),
                ("channels", C.c_int32), ("bytes_per_plane", C.c_int32), ("depth", C.c_int32),
                ("has_timestamps", C.c_int32), ("observer", C.c_char * 41), ("instrument", C.c_char * 41),
                ("telescope", C.c_char * 41), ("date_time", C.c_uint64), ("date_time_utc", C.c_uint64)]


_SER_DTYPE = {1: np.uint8, 2: np.uint16}


class c_ser_reader:
    """c_ser_reader (core/io/c_ser_file.h:136-174) over the C ABI."""

    def __init__(self, path: str):
        self._h = C.c_void_p()
        _check(lib().sst_ser_open(C.byref(self._h), os.fsencode(path)), "sst_ser_open")
        self.info = SerInfo()
        _check(lib().sst_ser_get_info(self._h, C.byref(self.info)), "sst_ser_get_info")

    def __del__(self):
        self.close()

    def close(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.sst_ser_close(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def dtype(self):
        if self.info.depth == DEPTH_F32:
            return np.float32
        if self.info.depth == DEPTH_F64:
            return np.float64
        if self.info.depth == DEPTH_S32:
            return np.int32
        return _SER_DTYPE[self.info.bytes_per_plane]

    def curpos(self) -> int:
        return lib().sst_ser_curpos(self._h)

    def seek(self, frame: int):
        _check(lib().sst_ser_seek(self._h, frame), "sst_ser_seek")

    def read(self, n: int = 1) -> np.ndarray:
        """up to n frames from the current position: (m, h, w[, channels])"""
        i = self.info
        shape = (n, i.height, i.width) + ((i.channels,) if i.channels > 1 else ())
        out = np.zeros(shape, self.dtype())
        got = C.c_int()
        _check(lib().sst_ser_read(self._h, n, _ptr(out), 0, C.byref(got)), "sst_ser_read")
        return out[:got.value]

    def timestamps(self) -> np.ndarray:
        ts = np.zeros(self.info.frames, np.uint64)
        m = lib().sst_ser_timestamps(self._h, _ptr(ts), len(ts))
        if m < 0:
            _check(m, "sst_ser_timestamps")
        return ts[:m]


class c_ser_writer:
    """c_ser_writer (core/io/c_ser_file.h:183-213) over the C ABI."""

    def __init__(self, path: str, width: int, height: int, color_id: int = 0, bits_per_plane: int = 16):
        self._h = C.c_void_p()
        _check(lib().sst_ser_writer_create(C.byref(self._h), os.fsencode(path), width, height, color_id,
                                           bits_per_plane), "sst_ser_writer_create")

    def write(self, frames: np.ndarray, timestamps=None):
        """appends frames (n, h, w[, c]) in the file's format, with n timestamps or none"""
        f = np.ascontiguousarray(frames)
        n = f.shape[0]
        ts = None if timestamps is None else np.ascontiguousarray(timestamps, np.uint64)
        if ts is not None and ts.size != n:
            raise ValueError("one timestamp per frame")
        _check(lib().sst_ser_write(self._h, _ptr(f), n, 0, _ptr(ts)), "sst_ser_write")

    def close(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            self._h = C.c_void_p()
            _check(_lib.sst_ser_writer_close(h), "sst_ser_writer_close")

    def __del__(self):
        try:
            self.close()
        except SSTError:
            pass


def stack_ser(reg: c_ecch, accs, ser: c_ser_reader, passes: Sequence[int], first: int = 0, count: int = -1,
              chunk: int = 0, weighting: int = 1, border: int = BORDER_REFLECT101):
    """sst_stack_ser: register + stack frames of a SER file (accs: one
    accumulator for mono files, four for Bayer files)."""
    accs = list(accs) if isinstance(accs, (list, tuple)) else [accs]
    n = ser.info.frames - first if count < 0 else min(count, ser.info.frames - first)
    handles = (C.c_void_p * len(accs))(*[a.handle.value for a in accs])
    models = (MotionModel * len(passes))(*[motion(t) for t in passes])
    outputs = {"params": np.zeros((n, 12), np.float32), "status": np.zeros(n, np.int32),
               "rho": np.zeros(n, np.float32), "weight": np.zeros(n, np.float32)}
    _check(lib().sst_stack_ser(reg.handle, handles, ser.handle, first, count, chunk, len(passes), models, border,
                               weighting, _ptr(outputs["params"]), _ptr(outputs["status"]), _ptr(outputs["rho"]),
                               _ptr(outputs["weight"]), None), "sst_stack_ser")
    return outputs


def calibrate_frames(frames, scale: float, dark=None, flat=None):
    """sst_calibrate_frames on torch CUDA tensors: frames (n, h, w) u8 / int16
    (u16 bits) / f32, dark and flat (h, w) f32 or None -> (n, h, w) f32"""
    import torch
    n, h, w = frames.shape
    depth = {torch.uint8: DEPTH_U8, torch.int16: DEPTH_U16, torch.float32: DEPTH_F32}[frames.dtype]
    es = frames.element_size()
    out = torch.empty((n, h, w), dtype=torch.float32, device=frames.device)
    _check(lib().sst_calibrate_frames(frames.data_ptr(), depth, n, w, h, frames.stride(1) * es, frames.stride(0) * es,
                                      scale, None if dark is None else dark.data_ptr(), 0,
                                      None if flat is None else flat.data_ptr(), 0, out.data_ptr(), 0, 0, None),
           "sst_calibrate_frames")
    return out


def debayer_nn2(raw, colorid: int):
    """sst_debayer_nn2: raw (n, h, w) or (h, w) Bayer frames, numpy u8 / u16 /
    f32 -> (n, h, w, 3) BGR frames of the same dtype (through device
    buffers)"""
    import torch
    r = np.ascontiguousarray(raw)
    if r.ndim == 2:
        r = r[None]
    n, h, w = r.shape
    dev = torch.from_numpy(r.view(np.int16) if r.dtype == np.uint16 else r).cuda()
    out = torch.empty((n, h, w, 3), dtype=dev.dtype, device=dev.device)
    _check(lib().sst_debayer_nn2(dev.data_ptr(), _NP_DEPTH[r.dtype], n, w, h, w * r.itemsize, w * h * r.itemsize,
                                 colorid, out.data_ptr(), 0, 0, None), "sst_debayer_nn2")
    res = out.cpu().numpy()
    return res.view(np.uint16) if r.dtype == np.uint16 else res


def filter_bad_pixels(frames, colorid: int = 0, threshold: float = 3.0):
    """sst_filter_bad_pixels: frames (n, h, w) or (h, w) numpy u8 / u16 / f32
    (colorid 8..11: Bayer mosaics) -> filtered frames of the same dtype
    (through device buffers)"""
    import torch
    r = np.ascontiguousarray(frames)
    single = r.ndim == 2
    if single:
        r = r[None]
    n, h, w = r.shape
    dev = torch.from_numpy(r.view(np.int16) if r.dtype == np.uint16 else r).cuda()
    out = torch.empty_like(dev)
    _check(lib().sst_filter_bad_pixels(dev.data_ptr(), _NP_DEPTH[r.dtype], n, w, h, w * r.itemsize,
                                       w * h * r.itemsize, colorid, threshold, out.data_ptr(), 0, 0, None),
           "sst_filter_bad_pixels")
    res = out.cpu().numpy()
    res = res.view(np.uint16) if r.dtype == np.uint16 else res
    return res[0] if single else res


def average_pyramid_inpaint(image: np.ndarray, mask: np.ndarray, max_levels: int = 100):
    """average_pyramid_inpaint of a float32 image and its u8 mask -> (image, mask)"""
    img = np.ascontiguousarray(image, np.float32)
    msk = np.ascontiguousarray(mask, np.uint8)
    h, w = img.shape
    out = np.zeros((h, w), np.float32)
    om = np.zeros((h, w), np.uint8)
    _check(lib().sst_average_pyramid_inpaint(_ptr(img), img.strides[0], _ptr(msk), msk.strides[0], w, h, max_levels,
                                             _ptr(out), out.strides[0], _ptr(om), om.strides[0], 0, None),
           "sst_average_pyramid_inpaint")
    return out, om


def remap(src: np.ndarray, motion_type: int, params, dst_shape=None, border=BORDER_REFLECT101, scale=1.0):
    """base_remap of one frame on the device (numpy in/out via torch device buffers)."""
    import torch
    s = np.ascontiguousarray(src)
    h, w = s.shape if dst_shape is None else dst_shape
    ds = torch.from_numpy(s.view(np.uint8) if s.dtype != np.float32 else s).cuda()
    dst = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    msk = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
    p = np.zeros(12, np.float32)
    pp = np.asarray(params, np.float32).ravel()
    p[:pp.size] = pp
    m = motion(motion_type)
    _check(lib().sst_remap(ds.data_ptr(), _NP_DEPTH[s.dtype], s.shape[1], s.shape[0], s.strides[0], scale,
                           C.byref(m), _ptr(p), border, dst.data_ptr(), msk.data_ptr(), w, h, None), "sst_remap")
    torch.cuda.synchronize()
    return dst.cpu().numpy(), msk.cpu().numpy()


def bayer_planes(raw: np.ndarray, average: bool = False):
    import torch
    r = np.ascontiguousarray(raw, np.uint16)
    h, w = r.shape
    d = torch.from_numpy(r.view(np.int16)).cuda()
    if average:
        out = torch.zeros((h // 2, w // 2), dtype=torch.int16, device="cuda")
        _check(lib().sst_average_bayer_planes_u16(d.data_ptr(), w, h, r.strides[0], out.data_ptr(), None), "bayer")
    else:
        out = torch.zeros((h // 2, w // 2, 4), dtype=torch.int16, device="cuda")
        _check(lib().sst_extract_bayer_planes_u16(d.data_ptr(), w, h, r.strides[0], out.data_ptr(), None), "bayer")
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint16)


# ------------------------------------------------------------ frame registration

def image_registration_options(ecc=None, eccflow=None, **kw) -> ImageRegistrationOptions:
    """The reference defaults (sst_image_registration_options_default), then
    `kw` on the top level, `ecc` / `eccflow` dicts on the nested options.
    Feature registration is switched off and ECC registration on unless kw says
    otherwise."""
    o = ImageRegistrationOptions()
    lib().sst_image_registration_options_default(C.byref(o))
    o.enable_feature_registration = 0
    o.enable_ecc_registration = 1
    for k, v in kw.items():
        setattr(o, k, v)
    for k, v in (ecc or {}).items():
        setattr(o.ecc, k, v)
    for k, v in (eccflow or {}).items():
        setattr(o.eccflow, k, v)
    return o


class c_frame_registration:
    """c_frame_registration (c_frame_registration.h:210-356) over the C ABI."""

    def __init__(self, options: Optional[ImageRegistrationOptions] = None, **kw):
        self.options = options if options is not None else image_registration_options(**kw)
        self._h = C.c_void_p()
        _check(lib().sst_frame_registration_create(C.byref(self._h), C.byref(self.options)),
               "sst_frame_registration_create")
        self.width = self.height = 0

    def __del__(self):
        try:
            if self._h:
                lib().sst_frame_registration_destroy(self._h)
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def setup_reference_frame(self, image: np.ndarray, mask: Optional[np.ndarray] = None, scale: float = 1.0):
        a = np.ascontiguousarray(image)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        _check(lib().sst_frame_registration_setup_reference_frame(
            self._h, _ptr(a), _NP_DEPTH[a.dtype], a.shape[1], a.shape[0], a.strides[0], scale, _ptr(m),
            0 if m is None else m.strides[0], 0, None), "setup_reference_frame")
        self.height, self.width = a.shape

    def register_frames(self, frames: np.ndarray, scale: float = 1.0, rmap: bool = False):
        fr = np.ascontiguousarray(frames)
        if fr.ndim == 2:
            fr = fr[None]
        n, hh, ww = fr.shape
        out = {"params": np.zeros((n, 12), np.float32), "status": np.zeros(n, np.int32),
               "rho": np.zeros(n, np.float32), "iterations": np.zeros(n, np.int32),
               "rmap": np.zeros((n, hh, ww, 2), np.float32) if rmap else None}
        _check(lib().sst_frame_registration_register_frames(
            self._h, _ptr(fr), _NP_DEPTH[fr.dtype], n, ww, hh, fr.strides[1], fr.strides[0], scale, 0,
            _ptr(out["params"]), _ptr(out["status"]), _ptr(out["rho"]), _ptr(out["iterations"]), _ptr(out["rmap"]),
            None), "register_frames")
        return out

    def set_chunk_frames(self, n: int):
        _check(lib().sst_frame_registration_set_chunk_frames(self._h, n), "set_chunk_frames")

    def ecc_size(self):
        w, h = C.c_int(), C.c_int()
        _check(lib().sst_frame_registration_ecc_size(self._h, C.byref(w), C.byref(h)), "ecc_size")
        return w.value, h.value

    def ecc_image(self, frame: int = -1, with_mask: bool = False):
        w, h = self.ecc_size()
        out = np.zeros((h, w), np.float32)
        m = np.zeros((h, w), np.uint8) if with_mask else None
        _check(lib().sst_frame_registration_ecc_image(self._h, frame, _ptr(out), _ptr(m), 0), "ecc_image")
        return (out, m) if with_mask else out


def remap_rmap(src: np.ndarray, rmap: np.ndarray, border: int = BORDER_REFLECT101, border_value: float = 0.0,
               src_mask=None, scale: float = 1.0):
    """sst_remap_rmap on host arrays: (dst, dst_mask)."""
    s = np.ascontiguousarray(src)
    rm = np.ascontiguousarray(rmap, np.float32)
    dh, dw = rm.shape[:2]
    msk = None if src_mask is None else np.ascontiguousarray(src_mask, np.uint8)
    dst = np.zeros((dh, dw), np.float32)
    dmask = np.zeros((dh, dw), np.uint8)
    _check(lib().sst_remap_rmap(_ptr(s), _NP_DEPTH[s.dtype], s.shape[1], s.shape[0], s.strides[0], scale, _ptr(rm),
                                dw, dh, border, border_value, _ptr(msk), 0 if msk is None else msk.strides[0],
                                _ptr(dst), _ptr(dmask), 0, None), "sst_remap_rmap")
    return dst, dmask


def create_remap(motion_type: int, params, width: int, height: int) -> np.ndarray:
    """sst_image_transform_create_remap: (height, width, 2) map of W(x, y; params)."""
    m = motion(motion_type)
    p = np.zeros(12, np.float32)
    pp = np.asarray(params, np.float32).ravel()
    p[:pp.size] = pp
    out = np.zeros((height, width, 2), np.float32)
    _check(lib().sst_image_transform_create_remap(C.byref(m), _ptr(p), width, height, _ptr(out), 0, None),
           "create_remap")
    return out


def scale_transform(motion_type: int, params, factor: float) -> np.ndarray:
    """sst_image_transform_scale: scale_transfrom(factor) of a parameter vector."""
    m = motion(motion_type)
    p = np.zeros(12, np.float32)
    pp = np.asarray(params, np.float32).ravel()
    p[:pp.size] = pp
    _check(lib().sst_image_transform_scale(C.byref(m), _ptr(p), factor), "scale_transform")
    return p[:nparams(motion_type)]
