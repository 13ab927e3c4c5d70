"""FP64 oracle for the registration + stacking hot path (test infrastructure).

ctypes binding of ``oracle/_build/libsst_oracle.so`` (built by ``make -C oracle``).
Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import this module; the product never does.

Parity status: unpinned by the reference (it ships no tests or golden data and
cannot be built without OpenCV/TBB). The restatement is pinned by known-answer
tests in ``tests/test_oracle.py``.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsst_oracle.so")

# IMAGE_MOTION_TYPE (image_transform.h:15-26)
TRANSLATION, EUCLIDEAN, SCALED_EUCLIDEAN, AFFINE, HOMOGRAPHY, SEMI_QUADRATIC, QUADRATIC, EPIPOLAR = range(8)
# ECC_ALIGN_METHOD (ecc2.h:57-62)
FA, IC, LM, ICLM = range(4)
BORDER_CONSTANT, BORDER_REPLICATE, BORDER_REFLECT, BORDER_REFLECT101 = 0, 1, 2, 4


def build(force: bool = False) -> str:
    srcs = [os.path.join(_HERE, f) for f in sorted(os.listdir(_HERE)) if f.endswith((".cc", ".h")) or f == "Makefile"]
    if force or not os.path.exists(_LIB_PATH) or any(
            os.path.getmtime(s) > os.path.getmtime(_LIB_PATH) for s in srcs):
        subprocess.check_call(["make", "-s", "-j8", "-C", _HERE])
    return _LIB_PATH


class Model(C.Structure):
    _fields_ = [("type", C.c_int), ("fix_translation", C.c_int), ("fix_rotation", C.c_int),
                ("fix_scale", C.c_int)]


class AlignOpts(C.Structure):
    _fields_ = [("method", C.c_int), ("max_iterations", C.c_int), ("max_eps", C.c_double),
                ("update_step_scale", C.c_double), ("ic_jacobian_at_identity", C.c_int)]


class Level(C.Structure):
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("ref", C.c_void_p), ("ref_mask", C.c_void_p),
                ("cur", C.c_void_p), ("cw", C.c_int), ("ch", C.c_int), ("cur_mask", C.c_void_p)]


class EcchOpts(C.Structure):
    _fields_ = [("epsx", C.c_double), ("reference_smooth_sigma", C.c_double),
                ("input_smooth_sigma", C.c_double), ("update_step_scale", C.c_double),
                ("method", C.c_int), ("max_iterations", C.c_int), ("minimum_image_size", C.c_int),
                ("maxlevel", C.c_int), ("ic_jacobian_at_identity", C.c_int)]


class PipelineOpts(C.Structure):
    _fields_ = [("ecch", EcchOpts), ("num_passes", C.c_int), ("pass_motion", C.c_int * 3),
                ("min_rho", C.c_double), ("border_mode", C.c_int), ("use_laplacian_weights", C.c_int)]


class RegistrationOpts(C.Structure):
    """c_ecc_registration_options (c_frame_registration.h:47-63) + motion type."""
    _fields_ = [("motion_type", C.c_int), ("method", C.c_int), ("scale", C.c_double), ("eps", C.c_double),
                ("min_rho", C.c_double), ("input_smooth_sigma", C.c_double), ("reference_smooth_sigma", C.c_double),
                ("update_step_scale", C.c_double), ("max_iterations", C.c_int), ("ecch_max_level", C.c_int),
                ("ecch_minimum_image_size", C.c_int), ("normalization_scale", C.c_int),
                ("normalization_noise", C.c_double), ("estimate_translation_first", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        d, i, p = C.c_double, C.c_int, C.c_void_p
        sig = {
            "orc_model_nparams": (i, [p]),
            "orc_model_identity": (None, [p, p]),
            "orc_model_get_params": (None, [p, p, p]),
            "orc_model_set_params": (None, [p, p, p]),
            "orc_model_warp": (None, [p, p, d, d, p, p]),
            "orc_model_sd": (None, [p, p, d, d, d, d, p]),
            "orc_model_eps": (d, [p, p, p, i, i]),
            "orc_model_scale": (None, [p, p, d]),
            "orc_model_invert_and_compose": (i, [p, p, p, p]),
            "orc_gaussian_kernel": (i, [d, p]),
            "orc_smooth": (None, [p, i, i, d, p]),
            "orc_pyrdown": (None, [p, i, i, p, i, i]),
            "orc_differentiate": (None, [p, i, i, p, p, p]),
            "orc_sample_bilinear": (d, [p, i, i, d, d, i, d]),
            "orc_erode5": (None, [p, i, i, i, p]),
            "orc_remap_model": (None, [p, p, p, i, i, i, i, i, d, p]),
            "orc_ecc_align": (i, [p, p, p, p, p, p]),
            "orc_ecch_num_levels": (i, [i, i, p]),
            "orc_ecch_align": (i, [p, p, p, p, p, i, i, p, p, i, i, p, p]),
            "orc_correlation": (d, [p, p, i, i, p, p, i, i, p, p]),
            "orc_stack_remap": (None, [p, p, p, i, i, i, i, i, p, p]),
            "orc_weighted_average_add": (None, [p, p, i, i, p, p]),
            "orc_running_mean_add_f32": (None, [p, p, i, i, p, p]),
            "orc_extract_bayer_planes_u16": (None, [p, i, i, p]),
            "orc_average_bayer_planes_u16": (None, [p, i, i, p]),
            "orc_bayer_pattern_mask": (None, [i, i, i, p]),
            "orc_bayer_accumulate": (None, [p, i, i, p, p, p, p, p, p]),
            "orc_warp_grid": (None, [p, p, i, i, p, p]),
            "orc_resize_area": (None, [p, i, i, p, i, i]),
            "orc_resize_cubic": (None, [p, i, i, p, i, i]),
            "orc_eccflow_levels": (i, [i, i, p, p, p, i]),
            "orc_eccflow": (i, [p, p, p, i, i, p, p]),
            "orc_warp_residual": (d, [p, p, p, p, p, i, i, p, p, p]),
            "orc_focus_weights": (None, [p, p, p, i, i, i, i, p]),
            "orc_laplacian_energy": (d, [p, i, i]),
            "orc_resize_linear": (None, [p, i, i, p, i, i]),
            "orc_local_variance_size": (i, [i, i, i, i, p, p]),
            "orc_local_variance_map": (i, [p, i, i, i, i, i, d, p, p, p, p]),
            "orc_average_pyramid_inpaint": (None, [p, p, i, i, i, p, p]),
            "orc_register_and_stack": (i, [p, p, i, i, p, i, d, p, p, p, p, p]),
            "orc_pyrdown_border": (None, [p, i, i, p, i, i, i]),
            "orc_pyrup": (None, [p, i, i, p, i, i]),
            "orc_mask_pyrdown_ge250": (None, [p, i, i, p, i, i]),
            "orc_scale_image_size": (None, [i, i, d, p, p]),
            "orc_scale_image": (None, [p, p, i, i, d, p, p]),
            "orc_ecc_normalize": (None, [p, p, i, i, i, p]),
            "orc_register_frame": (i, [p, p, p, i, i, p, p, p, p]),
            "ref_register_and_stack": (i, [p, p, i, i, p, i, d, p, p, p, p, p]),
            "orc_eccflow_masked": (i, [p, p, p, p, p, i, i, p, p]),
            "orc_lpg": (i, [p, p, i, i, d, d, i, i, p, p]),
            "orc_debayer_nn2_u16": (i, [p, i, i, i, p]),
            "orc_debayer_nn2_f32": (i, [p, i, i, i, p]),
            "orc_optimal_dft_size": (i, [i]),
            "orc_linear_inpaint": (None, [p, p, i, i, i]),
            "orc_filter_bad_pixels_u16": (i, [p, i, i, i, d, p]),
            "orc_filter_bad_pixels_f32": (i, [p, i, i, i, d, p]),
            "orc_fft_average": (i, [p, i, i, i, i, p]),
            "orc_focus_stack": (i, [p, p, i, i, i, i, i, i, i, p, i, p]),
            "orc_canvas_average": (i, [p, i, i, i, i, i, p, p, p, p, p, p, p, p]),
            "orc_set_num_threads": (None, [i]),
            "orc_get_num_threads": (i, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _u8(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint8)


def model(motion: int, fix_translation=0, fix_rotation=0, fix_scale=None) -> Model:
    """create_image_transform (image_transform.cc:32-60): EUCLIDEAN fixes the scale."""
    if fix_scale is None:
        fix_scale = 1 if motion == EUCLIDEAN else 0
    return Model(motion, fix_translation, fix_rotation, fix_scale)


def nparams(m: Model) -> int:
    return lib().orc_model_nparams(C.byref(m))


def identity(m: Model) -> np.ndarray:
    s = np.zeros(16)
    lib().orc_model_identity(C.byref(m), _ptr(s))
    return s


def get_params(m: Model, state) -> np.ndarray:
    p = np.zeros(16)
    s = _f64(state)
    lib().orc_model_get_params(C.byref(m), _ptr(s), _ptr(p))
    return p[:nparams(m)]


def set_params(m: Model, state, p) -> np.ndarray:
    s = _f64(state).copy()
    pp = np.zeros(16)
    pp[:len(p)] = p
    lib().orc_model_set_params(C.byref(m), _ptr(s), _ptr(pp))
    return s


def warp(m: Model, state, x: float, y: float):
    s = _f64(state)
    X, Y = C.c_double(), C.c_double()
    lib().orc_model_warp(C.byref(m), _ptr(s), x, y, C.byref(X), C.byref(Y))
    return X.value, Y.value


def warp_grid(m: Model, state, w: int, h: int):
    """W(x;p) over the w x h grid (create_remap) -> (mapx, mapy)."""
    mx = np.empty((h, w))
    my = np.empty((h, w))
    s = _f64(state)
    lib().orc_warp_grid(C.byref(m), _ptr(s), w, h, _ptr(mx), _ptr(my))
    return mx, my


def sd(m: Model, state, x, y, gx, gy) -> np.ndarray:
    s = _f64(state)
    J = np.zeros(12)
    lib().orc_model_sd(C.byref(m), _ptr(s), x, y, gx, gy, _ptr(J))
    return J[:nparams(m)]


def eps(m: Model, state, dp, w, h) -> float:
    s = _f64(state)
    d = np.zeros(16)
    d[:len(dp)] = dp
    return lib().orc_model_eps(C.byref(m), _ptr(s), _ptr(d), w, h)


def scale(m: Model, state, f) -> np.ndarray:
    s = _f64(state).copy()
    lib().orc_model_scale(C.byref(m), _ptr(s), f)
    return s


def invert_and_compose(m: Model, state, dp) -> np.ndarray:
    s = _f64(state)
    d = np.zeros(16)
    d[:len(dp)] = dp
    out = np.zeros(16)
    lib().orc_model_invert_and_compose(C.byref(m), _ptr(s), _ptr(d), _ptr(out))
    return out


def gaussian_kernel(sigma: float) -> np.ndarray:
    k = np.zeros(512)
    n = lib().orc_gaussian_kernel(sigma, _ptr(k))
    return k[:n]


def smooth(img, sigma):
    a = _f64(img)
    out = np.empty_like(a)
    lib().orc_smooth(_ptr(a), a.shape[1], a.shape[0], sigma, _ptr(out))
    return out


def next_size(w, h):
    """c_ecch::compute_next_pyramid_layer_size (ecc2.h:290-293)"""
    return ((w + 1) >> 1) & ~1, ((h + 1) >> 1) & ~1


def pyrdown(img, dw=None, dh=None):
    a = _f64(img)
    h, w = a.shape
    if dw is None:
        dw, dh = next_size(w, h)
    out = np.empty((dh, dw))
    lib().orc_pyrdown(_ptr(a), w, h, _ptr(out), dw, dh)
    return out


def differentiate(img, valid=None):
    a = _f64(img)
    gx = np.empty_like(a)
    gy = np.empty_like(a)
    lib().orc_differentiate(_ptr(a), a.shape[1], a.shape[0], _ptr(_u8(valid)), _ptr(gx), _ptr(gy))
    return gx, gy


def erode5(mask):
    m = _u8(mask)
    out = np.empty_like(m)
    lib().orc_erode5(_ptr(m), m.shape[1], m.shape[0], 1, _ptr(out))
    return out


def remap(m: Model, state, src, dw, dh, border=BORDER_REPLICATE, bval=0.0):
    s = _f64(state)
    a = _f64(src)
    out = np.empty((dh, dw))
    lib().orc_remap_model(C.byref(m), _ptr(s), _ptr(a), a.shape[1], a.shape[0], dw, dh, border, bval, _ptr(out))
    return out


def ecc_align(m: Model, state, ref, cur, method=IC, max_iterations=50, max_eps=0.2, step=1.0,
              ref_mask=None, cur_mask=None, ic_jacobian_at_identity=1):
    """Single-level c_ecc_align::align(). Returns (ok, state, iterations, eps)."""
    s = _f64(state).copy()
    r, c = _f64(ref), _f64(cur)
    rm, cm = _u8(ref_mask), _u8(cur_mask)
    lv = Level(r.shape[1], r.shape[0], _ptr(r), _ptr(rm), _ptr(c), c.shape[1], c.shape[0], _ptr(cm))
    o = AlignOpts(method, max_iterations, max_eps, step, ic_jacobian_at_identity)
    it, e = C.c_int(), C.c_double()
    ok = lib().orc_ecc_align(C.byref(m), _ptr(s), C.byref(lv), C.byref(o), C.byref(it), C.byref(e))
    return bool(ok), s, it.value, e.value


def ecch_opts(method=IC, maxlevel=4, max_iterations=50, epsx=0.2, ref_sigma=1.0, in_sigma=1.0, step=1.0,
              minimum_image_size=16, ic_jacobian_at_identity=1) -> EcchOpts:
    return EcchOpts(epsx, ref_sigma, in_sigma, step, method, max_iterations, minimum_image_size, maxlevel,
                    ic_jacobian_at_identity)


def ecch_num_levels(w, h, o: EcchOpts) -> int:
    return lib().orc_ecch_num_levels(w, h, C.byref(o))


def ecch_align(m: Model, state, ref, cur, o: EcchOpts, ref_mask=None, cur_mask=None):
    s = _f64(state).copy()
    r, c = _f64(ref), _f64(cur)
    rm, cm = _u8(ref_mask), _u8(cur_mask)
    it, e = C.c_int(), C.c_double()
    lib().orc_ecch_align(C.byref(m), _ptr(s), C.byref(o), _ptr(r), _ptr(rm), r.shape[1], r.shape[0],
                         _ptr(c), _ptr(cm), c.shape[1], c.shape[0], C.byref(it), C.byref(e))
    return s, it.value, e.value


def correlation(m: Model, state, cur, ref, cur_mask=None, ref_mask=None) -> float:
    s = _f64(state)
    c, r = _f64(cur), _f64(ref)
    return lib().orc_correlation(_ptr(c), _ptr(_u8(cur_mask)), c.shape[1], c.shape[0], _ptr(r),
                                 _ptr(_u8(ref_mask)), r.shape[1], r.shape[0], C.byref(m), _ptr(s))


def stack_remap(m: Model, state, src, dw, dh, border=BORDER_REFLECT101):
    s = _f64(state)
    a = _f64(src)
    out = np.empty((dh, dw))
    msk = np.empty((dh, dw), np.uint8)
    lib().orc_stack_remap(C.byref(m), _ptr(s), _ptr(a), a.shape[1], a.shape[0], dw, dh, border, _ptr(out),
                          _ptr(msk))
    return out, msk


def laplacian_energy(img) -> float:
    a = _f64(img)
    return lib().orc_laplacian_energy(_ptr(a), a.shape[1], a.shape[0])


def extract_bayer_planes(raw):
    a = np.ascontiguousarray(raw, dtype=np.uint16)
    h, w = a.shape
    out = np.empty((h // 2, w // 2, 4), np.uint16)
    lib().orc_extract_bayer_planes_u16(_ptr(a), w, h, _ptr(out))
    return out


def average_bayer_planes(raw):
    a = np.ascontiguousarray(raw, dtype=np.uint16)
    h, w = a.shape
    out = np.empty((h // 2, w // 2), np.uint16)
    lib().orc_average_bayer_planes_u16(_ptr(a), w, h, _ptr(out))
    return out


def bayer_pattern_mask(colorid, w, h):
    out = np.empty((h, w), np.uint8)
    lib().orc_bayer_pattern_mask(colorid, w, h, _ptr(out))
    return out


def bayer_accumulate(src, mapx, mapy, pattern, weights, acc, cntr):
    a = _f64(src)
    h, w = a.shape
    mx = None if mapx is None else _f64(mapx)
    my = None if mapy is None else _f64(mapy)
    wt = None if weights is None else _f64(weights)
    lib().orc_bayer_accumulate(_ptr(a), w, h, _ptr(mx), _ptr(my), _ptr(_u8(pattern)), _ptr(wt), _ptr(acc),
                               _ptr(cntr))


def bayer_average(colorid, frames, motion_type=None, params=None, weights=None, status=None, scale=1.0):
    """c_bayer_average fed as the stacking pipeline feeds it
    (c_image_stacking_pipeline.cc:1704-1749): per frame the remap of the
    transform of params[f], the per-pixel weight = remapped frame mask
    (>= 255, 5x5 erode) x weights[f], then _bayer_accumulate. Returns the
    channel sums (h, w, 3) and channel weights (h, w, 3), B, G, R order."""
    fr = np.asarray(frames)
    if fr.ndim == 2:
        fr = fr[None]
    n, h, w = fr.shape
    pat = bayer_pattern_mask(colorid, w, h)
    acc = np.zeros((h, w, 3))
    cntr = np.zeros((h, w, 3))
    for f in range(n):
        wf = 1.0 if weights is None else float(weights[f])
        if status is not None and status[f] != 0:
            continue
        if not wf > 0:
            continue
        img = fr[f].astype(np.float64) * scale
        if motion_type is None:
            bayer_accumulate(img, None, None, pat, np.full((h, w), wf), acc, cntr)
            continue
        m = model(motion_type)
        st = set_params(m, identity(m), np.asarray(params[f], np.float64)[:nparams(m)])
        _, msk = stack_remap(m, st, img, w, h)
        mx, my = warp_grid(m, st, w, h)
        bayer_accumulate(img, mx, my, pat, np.where(msk > 0, wf, 0.0), acc, cntr)
    return acc, cntr


class FlowOpts(C.Structure):
    """c_eccflow_options (ecc2.h:515-527); downscale 0 recursive resize, 1 full resize, 2 pyrDown"""
    _fields_ = [("update_multiplier", C.c_double), ("scale_factor", C.c_double), ("noise_level", C.c_double),
                ("max_iterations", C.c_int), ("support_scale", C.c_int), ("min_image_size", C.c_int),
                ("max_pyramid_level", C.c_int), ("downscale", C.c_int)]


def flow_opts(update_multiplier=1.5, scale_factor=0.5, noise_level=-1.0, max_iterations=1, support_scale=5,
              min_image_size=4, max_pyramid_level=-1, downscale=0) -> FlowOpts:
    """defaults of c_eccflow_options (ecc2.h:515-527)"""
    return FlowOpts(update_multiplier, scale_factor, noise_level, max_iterations, support_scale, min_image_size,
                    max_pyramid_level, downscale)


def resize_area(img, dw, dh):
    a = _f64(img)
    out = np.empty((dh, dw))
    lib().orc_resize_area(_ptr(a), a.shape[1], a.shape[0], _ptr(out), dw, dh)
    return out


def resize_cubic(img, dw, dh):
    a = _f64(img)
    out = np.empty((dh, dw))
    lib().orc_resize_cubic(_ptr(a), a.shape[1], a.shape[0], _ptr(out), dw, dh)
    return out


def eccflow_levels(w, h, o: FlowOpts):
    ws = np.zeros(64, np.int32)
    hs = np.zeros(64, np.int32)
    n = lib().orc_eccflow_levels(w, h, C.byref(o), _ptr(ws), _ptr(hs), 64)
    return list(zip(ws[:n].tolist(), hs[:n].tolist()))


def eccflow(o: FlowOpts, ref, cur, init_flow=None, ref_mask=None, cur_mask=None):
    """c_eccflow: reference + current (+ masks) -> flow (h, w, 2) (rmap = identity + flow)"""
    r, c = _f64(ref), _f64(cur)
    h, w = r.shape
    init = None if init_flow is None else _f64(init_flow)
    out = np.empty((h, w, 2))
    lib().orc_eccflow_masked(C.byref(o), _ptr(r), _ptr(_u8(ref_mask)), _ptr(c), _ptr(_u8(cur_mask)), w, h,
                             _ptr(init), _ptr(out))
    return out


def focus_weights(m: Model, state, src, dw, dh):
    """focus weights (6 lap^2 + |grad|^2)^2 of the warped frame, Gaussian sigma 3"""
    s, a = _f64(state), _f64(src)
    out = np.empty((dh, dw))
    lib().orc_focus_weights(C.byref(m), _ptr(s), _ptr(a), a.shape[1], a.shape[0], dw, dh, _ptr(out))
    return out


def resize_linear(img, dw, dh):
    """cv::resize INTER_LINEAR"""
    a = _f64(img)
    out = np.empty((dh, dw))
    lib().orc_resize_linear(_ptr(a), a.shape[1], a.shape[0], _ptr(out), dw, dh)
    return out


def local_variance_size(w, h, dscale=1, uscale=3):
    """(width, height) of the map compute_local_variance_map returns"""
    mw, mh = C.c_int(), C.c_int()
    lib().orc_local_variance_size(w, h, dscale, uscale, C.byref(mw), C.byref(mh))
    return mw.value, mh.value


def local_variance_map(img, kradius=2, dscale=1, uscale=3, depth_scale=20.0):
    """compute_local_variance_map -> (map or None, Q); depth_scale 20 is the
    CV_32F case (20 * maxval(CV_32F) / maxval(depth))"""
    a = _f64(img)
    h, w = a.shape
    out = np.empty((h, w))
    mw, mh, q = C.c_int(), C.c_int(), C.c_double()
    ok = lib().orc_local_variance_map(_ptr(a), w, h, kradius, dscale, uscale, depth_scale, _ptr(out),
                                      C.byref(mw), C.byref(mh), C.byref(q))
    if not ok:
        return None, 0.0
    return out.ravel()[:mw.value * mh.value].reshape(mh.value, mw.value).copy(), q.value


def average_pyramid_inpaint(img, mask, max_levels=100):
    """average_pyramid_inpaint -> (image, mask)"""
    a = _f64(img)
    m = np.ascontiguousarray(mask, np.uint8)
    h, w = a.shape
    out = np.empty((h, w))
    om = np.empty((h, w), np.uint8)
    lib().orc_average_pyramid_inpaint(_ptr(a), _ptr(m), w, h, max_levels, _ptr(out), _ptr(om))
    return out, om


def warp_residual(m: Model, state, img, tmpl, flow=None):
    """L = 1/2 sum (I(W(x; p) + u(x)) - T(x))^2 and its exact gradients (p, T, u)."""
    s, a, t = _f64(state), _f64(img), _f64(tmpl)
    h, w = a.shape
    f = None if flow is None else _f64(flow)
    gp = np.zeros(16)
    gt = np.zeros((h, w))
    gu = np.zeros((h, w, 2))
    L = lib().orc_warp_residual(C.byref(m), _ptr(s), _ptr(a), _ptr(t), _ptr(f), w, h, _ptr(gp), _ptr(gt), _ptr(gu))
    return L, gp[:nparams(m)], gt, gu


def pipeline_opts(passes=(AFFINE, HOMOGRAPHY), method=IC, maxlevel=4, max_iterations=50, epsx=0.2,
                  min_rho=0.8, border=BORDER_REFLECT101, laplacian_weights=1, ic_jacobian_at_identity=1,
                  minimum_image_size=16) -> PipelineOpts:
    o = PipelineOpts()
    o.ecch = ecch_opts(method, maxlevel, max_iterations, epsx, 1.0, 1.0, 1.0, minimum_image_size,
                       ic_jacobian_at_identity)
    o.num_passes = len(passes)
    for k, p in enumerate(passes):
        o.pass_motion[k] = p
    o.min_rho = min_rho
    o.border_mode = border
    o.use_laplacian_weights = laplacian_weights
    return o


def register_and_stack(o: PipelineOpts, ref, frames, frame_scale):
    """CPU restatement of register_frame + the stacking loop body for n frames."""
    r = _f64(ref)
    fr = np.ascontiguousarray(frames, dtype=np.uint16)
    n = fr.shape[0]
    h, w = r.shape
    states = np.zeros((n, 16))
    status = np.zeros(n, np.int32)
    rho = np.zeros(n)
    acc = np.zeros((h, w))
    accw = np.zeros((h, w))
    lib().orc_register_and_stack(C.byref(o), _ptr(r), w, h, _ptr(fr), n, frame_scale, _ptr(states),
                                 _ptr(status), _ptr(rho), _ptr(acc), _ptr(accw))
    return states, status, rho, acc, accw


def set_num_threads(n: int):
    lib().orc_set_num_threads(n)


def get_num_threads() -> int:
    return lib().orc_get_num_threads()


def stack_compare_region(models_states, dw, dh, sw, sh, delta=0.05):
    """Pixels of a dw x dh stack whose per-frame validity is settled.

    The stacked mask of a frame is its remapped coverage (>= 255 of 255, i.e.
    coverage >= 0.998) eroded 5 x 5 (c_frame_registration.cc:1315-1340).
    A registration that differs by up to 0.02 px can flip a pixel whose 5 x 5
    window maps within that distance of the source frame's edge, which moves
    that pixel's stacked value by a whole frame's share. A pixel is kept
    when, for every frame (motion model, oracle state), the warped positions
    of its clipped 5 x 5 window lie all at least `delta` px inside the source
    frame [0, sw - 1] x [0, sh - 1] or at least one of them `delta` px
    outside it. models_states: iterable of (Model, state) of accepted frames.
    """
    from scipy.ndimage import maximum_filter, minimum_filter
    keep = np.ones((dh, dw), bool)
    for m, s in models_states:
        X, Y = warp_grid(m, s, dw, dh)
        x0, x1 = minimum_filter(X, 5, mode="nearest"), maximum_filter(X, 5, mode="nearest")
        y0, y1 = minimum_filter(Y, 5, mode="nearest"), maximum_filter(Y, 5, mode="nearest")
        inside = (x0 >= delta) & (x1 <= sw - 1 - delta) & (y0 >= delta) & (y1 <= sh - 1 - delta)
        outside = (x0 <= -delta) | (x1 >= sw - 1 + delta) | (y0 <= -delta) | (y1 >= sh - 1 + delta)
        keep &= inside | outside
    return keep


def stack_rel_err(avg, ref_avg, floor_frac=0.01):
    """|avg - ref| / max(|ref|, floor_frac * max |ref|) elementwise (the floor
    keeps the black sky of the synthetic scenes from dividing by ~0)."""
    ref_avg = np.asarray(ref_avg, np.float64)
    den = np.maximum(np.abs(ref_avg), floor_frac * float(np.abs(ref_avg).max()))
    return np.abs(np.asarray(avg, np.float64) - ref_avg) / den


def stack_error_report(frames, frame_scale, motion, gpu_params, gpu_status, gpu_weights, gpu_avg, orc_states,
                       orc_status, orc_S, orc_W, input_sigma=1.0, laplacian_weights=True, border=BORDER_REFLECT101,
                       arith_tol=1e-5, floor_frac=0.01):
    """Errors of a GPU stack against the FP64 oracle, split by cause.

    arith   : the GPU stack against FP64 sums of the same frames warped with
              the GPU's own transforms and weighted by the GPU's own frame
              weights: the error of the warp + accumulate arithmetic alone.
    e2e     : the GPU stack against the oracle pipeline's stack (its own
              registration and FP64 Laplacian-energy weights).
    e2e_bound_frac : the largest ratio of the end-to-end error to the error
              the registration differences explain. For pixel p the bound is
                arith_tol * den(p)
                + 2 * sum_f w_f * g_f(p) * sqrt(2) * d_f / sum_f w_f
                + 2 * sum_f w_f * |I_f(p) - avg(p)| * dw_f / sum_f w_f
              with d_f the largest displacement between the GPU's and the
              oracle's warp of frame f over the image, g_f(p) the largest
              forward difference of source frame f over the 5 x 5 source
              pixels around the oracle's sample position of p (within a
              bilinear cell the interpolant's slope along x or y is a blend
              of two such differences, so a sample moved by d < 1 px changes
              by at most sqrt(2) d g_f), and dw_f the relative difference of
              the two frame weights (the derivative of the weighted mean by
              w_f is (I_f - avg) / sum w). The factor 2 covers second-order
              terms. A value <= 1 means the whole end-to-end difference is
              accounted for.
    Every maximum is over the pixels that stack_compare_region keeps (of the
    oracle's transforms for e2e, of the GPU's for arith) where both stacks
    have weight. Relative errors use stack_rel_err's floor.
    """
    from scipy.ndimage import maximum_filter
    n, h, w = frames.shape
    m = model(motion)
    orc_avg = np.where(orc_W > 0, orc_S / np.where(orc_W > 0, orc_W, 1.0), 0.0)
    S_g = np.zeros((h, w))
    W_g = np.zeros((h, w))
    G = np.zeros((h, w))
    T = np.zeros((h, w))
    Wb = np.zeros((h, w))
    ms_g, ms_o = [], []
    warp_rms, disp_max, dw_max = 0.0, 0.0, 0.0
    for i in range(n):
        img = frames[i].astype(np.float64) * frame_scale
        if gpu_status[i] == 0:
            s_g = set_params(m, identity(m), np.asarray(gpu_params[i][:nparams(m)], np.float64))
            ms_g.append((m, s_g))
            dst, msk = stack_remap(m, s_g, img, w, h, border)
            wt = np.where(msk > 0, float(gpu_weights[i]), 0.0)
            S_g += wt * dst
            W_g += wt
        if orc_status[i] != 0:
            continue
        s_o = orc_states[i]
        ms_o.append((m, s_o))
        if gpu_status[i] != 0:
            continue
        xa, ya = warp_grid(m, s_g, w, h)
        xb, yb = warp_grid(m, s_o, w, h)
        d2 = (xa - xb) ** 2 + (ya - yb) ** 2
        d_f = math.sqrt(float(d2.max()))
        warp_rms = max(warp_rms, math.sqrt(float(d2.mean())))
        disp_max = max(disp_max, d_f)
        dst_o, msk_o = stack_remap(m, s_o, img, w, h, border)
        w_o = laplacian_energy(pyrdown(smooth(img, input_sigma))) if laplacian_weights else 1.0
        dw_f = abs(float(gpu_weights[i]) / w_o - 1.0)
        dw_max = max(dw_max, dw_f)
        gx = np.zeros((h, w))
        gy = np.zeros((h, w))
        gx[:, :-1] = np.abs(np.diff(img, axis=1))
        gy[:-1, :] = np.abs(np.diff(img, axis=0))
        gs = maximum_filter(np.maximum(gx, gy), 5, mode="nearest")
        xi = np.clip(np.floor(xb), 0, w - 1).astype(np.int64)
        yi = np.clip(np.floor(yb), 0, h - 1).astype(np.int64)
        g = gs[yi, xi]
        wt = np.where(msk_o > 0, w_o, 0.0)
        G += wt * g * math.sqrt(2.0) * d_f
        T += wt * np.abs(dst_o - orc_avg) * dw_f
        Wb += wt
    keep_g = stack_compare_region(ms_g, w, h, w, h) & (W_g > 0)
    keep_o = stack_compare_region(ms_o, w, h, w, h) & (orc_W > 0) & (Wb > 0)
    arith = stack_rel_err(gpu_avg[keep_g], S_g[keep_g] / W_g[keep_g], floor_frac)
    e2e = stack_rel_err(gpu_avg[keep_o], orc_avg[keep_o], floor_frac)
    den = np.maximum(np.abs(orc_avg[keep_o]), floor_frac * float(np.abs(orc_avg[keep_o]).max()))
    bound = arith_tol * den + 2.0 * (G[keep_o] + T[keep_o]) / Wb[keep_o]
    frac = np.abs(gpu_avg[keep_o].astype(np.float64) - orc_avg[keep_o]) / bound
    return {"arith_max": float(arith.max()), "arith_median": float(np.median(arith)),
            "e2e_max": float(e2e.max()), "e2e_median": float(np.median(e2e)),
            "e2e_bound_frac": float(frac.max()), "warp_rms_max": warp_rms, "warp_disp_max": disp_max,
            "weight_rel_diff_max": dw_max, "region_frac": float(keep_o.mean())}


def pyrdown_border(img, border, dw=None, dh=None):
    """cv::pyrDown(src, dst, Size(), border): size ((w + 1) / 2, (h + 1) / 2)."""
    a = _f64(img)
    h, w = a.shape
    if dw is None:
        dw, dh = (w + 1) // 2, (h + 1) // 2
    out = np.empty((dh, dw))
    lib().orc_pyrdown_border(_ptr(a), w, h, _ptr(out), dw, dh, border)
    return out


def pyrup(img, dw, dh):
    a = _f64(img)
    out = np.empty((dh, dw))
    lib().orc_pyrup(_ptr(a), a.shape[1], a.shape[0], _ptr(out), dw, dh)
    return out


def mask_pyrdown_ge250(mask):
    m = _u8(mask)
    h, w = m.shape
    out = np.empty(((h + 1) // 2, (w + 1) // 2), np.uint8)
    lib().orc_mask_pyrdown_ge250(_ptr(m), w, h, _ptr(out), out.shape[1], out.shape[0])
    return out


def scale_image_size(w, h, scale):
    dw, dh = C.c_int(), C.c_int()
    lib().orc_scale_image_size(w, h, scale, C.byref(dw), C.byref(dh))
    return dw.value, dh.value


def scale_image(img, scale, mask=None):
    """scaleImage (c_frame_registration.cc:230-250) -> (image, mask or None)."""
    a = _f64(img)
    h, w = a.shape
    dw, dh = scale_image_size(w, h, scale)
    out = np.empty((dh, dw))
    mo = np.empty((dh, dw), np.uint8) if mask is not None else None
    lib().orc_scale_image(_ptr(a), _ptr(_u8(mask)), w, h, scale, _ptr(out), _ptr(mo))
    return out, mo


def ecc_normalize(img, lvl, mask=None):
    a = _f64(img)
    out = np.empty_like(a)
    lib().orc_ecc_normalize(_ptr(a), _ptr(_u8(mask)), a.shape[1], a.shape[0], lvl, _ptr(out))
    return out


def registration_opts(motion_type=AFFINE, method=LM, scale=0.5, eps=0.2, min_rho=0.8, input_smooth_sigma=1.0,
                      reference_smooth_sigma=1.0, update_step_scale=1.5, max_iterations=50, ecch_max_level=0,
                      ecch_minimum_image_size=16, normalization_scale=0, normalization_noise=0.01,
                      estimate_translation_first=1) -> RegistrationOpts:
    """Defaults of c_ecc_registration_options (c_frame_registration.h:47-63) and
    c_image_registration_options::motion_type (:121)."""
    return RegistrationOpts(motion_type, method, scale, eps, min_rho, input_smooth_sigma, reference_smooth_sigma,
                            update_step_scale, max_iterations, ecch_max_level, ecch_minimum_image_size,
                            normalization_scale, normalization_noise, estimate_translation_first)


def register_frame(o: RegistrationOpts, ref, cur, ref_mask=None):
    """setup_reference_frame + register_frame (ECC part) -> (status, state, rho, iterations)."""
    r, c = _f64(ref), _f64(cur)
    h, w = r.shape
    st = np.zeros(16)
    rho, it = C.c_double(), C.c_int()
    status = lib().orc_register_frame(C.byref(o), _ptr(r), _ptr(_u8(ref_mask)), w, h, _ptr(c), _ptr(st),
                                      C.byref(rho), C.byref(it))
    return status, st, rho.value, it.value


def refcpu_register_and_stack(o: PipelineOpts, ref, frames, frame_scale):
    """The FP32 reference-semantics CPU restatement (sst_refcpu.cc, the timed
    CPU baseline): register_frame with c_ecch over the motion passes, the
    correlation gate, base_remap and the FP32 running weighted mean, with the
    reference's sequence of full-image passes. Returns (states, status, rho,
    mean, weight sum)."""
    r = np.ascontiguousarray(ref, dtype=np.float32)
    fr = np.ascontiguousarray(frames, dtype=np.uint16)
    n = fr.shape[0]
    h, w = r.shape
    states = np.zeros((n, 16))
    status = np.zeros(n, np.int32)
    rho = np.zeros(n)
    acc = np.zeros((h, w), np.float32)
    accw = np.zeros((h, w), np.float32)
    lib().ref_register_and_stack(C.byref(o), _ptr(r), w, h, _ptr(fr), n, frame_scale, _ptr(states), _ptr(status),
                                 _ptr(rho), _ptr(acc), _ptr(accw))
    return states, status, rho, acc, accw


def lpg(img, k=2.0, p=2.0, dscale=2, uscale=6, mask=None):
    """lpg() (core/proc/lpg.cc:223-291) of an image already scaled like the
    reference's convertTo(1 / maxval): (map, metric); c_lpg_options defaults."""
    a = _f64(img)
    h, w = a.shape
    out = np.empty((h, w))
    met = C.c_double()
    r = lib().orc_lpg(_ptr(a), _ptr(_u8(mask)), w, h, k, p, dscale, uscale, _ptr(out), C.byref(met))
    if r != 0:
        raise ValueError("lpg: the map is smaller than 5 x 5")
    return out, met.value


def debayer_nn2(raw, colorid=8):
    """debayer NN2 (core/io/debayer.cc:828-1161): (h, w, 3) B, G, R of a u16 or f32 mosaic."""
    a = np.ascontiguousarray(raw)
    h, w = a.shape
    if a.dtype == np.uint16:
        out = np.empty((h, w, 3), np.uint16)
        r = lib().orc_debayer_nn2_u16(_ptr(a), w, h, colorid, _ptr(out))
    else:
        a = np.ascontiguousarray(a, np.float32)
        out = np.empty((h, w, 3), np.float32)
        r = lib().orc_debayer_nn2_f32(_ptr(a), w, h, colorid, _ptr(out))
    if r != 0:
        raise ValueError("debayer_nn2: odd size or not a Bayer pattern")
    return out


def optimal_dft_size(n):
    """cv::getOptimalDFTSize: the smallest 2^a 3^b 5^c >= n"""
    return lib().orc_optimal_dft_size(int(n))


def _hwc(frames):
    a = np.ascontiguousarray(frames, np.float64)
    if a.ndim == 3:
        a = a[..., None]
    return a


def fft_average(frames):
    """c_frame_accumulation_with_fft (c_frame_accumulation.cc:704-900) of n
    frames (n, h, w) or (n, h, w, cn) -> the average, same layout as a frame"""
    a = _hwc(frames)
    n, h, w, cn = a.shape
    out = np.empty((h, w, cn))
    if lib().orc_fft_average(_ptr(a), n, w, h, cn, _ptr(out)) != 0:
        raise ValueError("fft_average: invalid arguments")
    return out[..., 0] if np.ndim(frames) == 3 else out


def focus_stack(frames, masks=None, policy=0, inpaint=True, avgchannel=True, G=None):
    """c_laplacian_pyramid_focus_stacking (c_frame_accumulation.cc:464-688):
    policy 0 select_max_energy, 1 weighted_average; G the energy smoothing
    kernel (None: no smoothing) -> the fused image"""
    a = _hwc(frames)
    n, h, w, cn = a.shape
    m = None if masks is None else np.ascontiguousarray(masks, np.uint8)
    g = None if G is None else np.ascontiguousarray(G, np.float64)
    out = np.empty((h, w, cn))
    r = lib().orc_focus_stack(_ptr(a), _ptr(m), n, w, h, cn, policy, int(inpaint), int(avgchannel), _ptr(g),
                              0 if g is None else len(g), _ptr(out))
    if r < 0:
        raise ValueError("focus_stack: invalid arguments")
    return out[..., 0] if np.ndim(frames) == 3 else out


def canvas_average(frames, weights=None, boxes=None, rmaps=None, canvas=(0, 0)):
    """c_canvas_average (c_frame_accumulation.cc:264-450) over a sequence.
    weights: None, u8 masks or f64 weights (n, h, w); boxes (n, 4) x, y, w, h
    (w 0: no remap); rmaps: list of (bh, bw, 2) maps (None where no remap).
    Returns (acc (CH, CW[, cn]), W (CH, CW), status (n,), last bbox)."""
    a = _hwc(frames)
    n, h, w, cn = a.shape
    wk, wp = 0, None
    if weights is not None:
        if np.asarray(weights).dtype == np.uint8:
            wk, wp = 1, np.ascontiguousarray(weights, np.uint8)
        else:
            wk, wp = 2, np.ascontiguousarray(weights, np.float64)
    bx = np.zeros((n, 4), np.int32) if boxes is None else np.ascontiguousarray(boxes, np.int32)
    parts = [np.asarray(r, np.float64).reshape(-1) for r in (rmaps or []) if r is not None]
    rm = np.ascontiguousarray(np.concatenate(parts)) if parts else np.zeros(2)
    cv = np.array([canvas[0], canvas[1]], np.int32)
    CW, CH = max(canvas[0], 3 * w // 2), max(canvas[1], 3 * h // 2)
    acc = np.zeros((CH, CW, cn))
    W = np.zeros((CH, CW))
    st = np.zeros(n, np.int32)
    last = np.zeros(4, np.int32)
    lib().orc_canvas_average(_ptr(a), n, w, h, cn, wk, _ptr(wp), _ptr(bx), _ptr(rm), _ptr(cv), _ptr(acc), _ptr(W),
                             _ptr(st), _ptr(last))
    return (acc[..., 0] if np.ndim(frames) == 3 else acc), W, st, last


def linear_inpaint(image, mask):
    """linear_interpolation_inpaint (core/proc/inpaint/linear_interpolation_inpaint.cc)
    of (h, w) or (h, w, cn) with a u8 mask (0 = hole) -> the filled image"""
    a = _hwc(np.asarray(image)[None])[0].copy()
    h, w, cn = a.shape
    m = np.ascontiguousarray(mask, np.uint8)
    lib().orc_linear_inpaint(_ptr(a), _ptr(m), w, h, cn)
    return a[..., 0] if np.ndim(image) == 2 else a


def filter_bad_pixels(frame, colorid=0, threshold=3.0):
    """read_input_frame's bad-pixel filter (median_filter_bad_pixels,
    core/proc/bad_pixels.cc:14-70, or bayer_denoise, core/io/debayer.cc:
    1480-1612, for colorid 8..11) of one u16 or f32 frame"""
    a = np.ascontiguousarray(frame)
    h, w = a.shape
    out = np.empty_like(a)
    if a.dtype == np.uint16:
        r = lib().orc_filter_bad_pixels_u16(_ptr(a), w, h, colorid, threshold, _ptr(out))
    else:
        a = np.ascontiguousarray(a, np.float32)
        out = np.empty_like(a)
        r = lib().orc_filter_bad_pixels_f32(_ptr(a), w, h, colorid, threshold, _ptr(out))
    if r != 0:
        raise ValueError("filter_bad_pixels: odd size for a Bayer frame")
    return out
