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


def test_cpp_dropin_header_compiles_and_links(capi, tmp_path):
    """The C++ drop-in classes (include/serstacker_gb300.hpp) compile against the C ABI
    and run their host-only parts (option defaults, handle creation, the
    rejection of feature registration, scale_transfrom) without a GPU."""
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "t.cc"
    src.write_text(r'''
#include "serstacker_gb300.hpp"
#include <cstdio>
int main() {
  sst_gb300::c_ecch_options o;
  if( o.max_iterations != 50 || o.method != SST_ECC_INVERSE_COMPOSITIONAL_LM ) return 1;
  sst_gb300::c_ecch e(o);
  if( !e.handle() ) return 2;
  sst_gb300::image_transform t(SST_MOTION_HOMOGRAPHY);
  e.set_image_transform(&t);
  if( sst_gb300::c_ecch::nparams(t.model) != 8 ) return 3;
  sst_gb300::c_local_variance_map_options lo;
  if( lo.kradius != 2 || lo.dscale != 1 || lo.uscale != 3 ) return 4;
  sst_gb300::c_ser_reader ser(SER_PATH);
  if( !ser.is_open() || ser.image_width() != 6 || ser.image_height() != 4 || ser.num_frames() != 3 ) return 5;
  if( ser.bits_per_plane() != 12 || ser.depth() != SST_DEPTH_U16 || ser.frame_size() != 48 ) return 6;
  std::vector<uint8_t> f;
  if( !ser.seek(2) || !ser.read(f) || ser.curpos() != 3 ) return 7;
  const uint16_t * px = (const uint16_t *) f.data();
  for( int i = 0; i < 24; ++i ) if( px[i] != 2 * 1000 + i ) return 8;
  if( ser.read(f) ) return 9;          // past the last frame
  std::vector<uint64_t> ts = ser.timestamps();
  if( ts.size() != 3 || ts[1] != 11 ) return 10;
  sst_gb300::c_ser_writer wr;
  if( !wr.create(SER_OUT, 6, 4, 0, 12) || !wr.write(f.data(), 77) || !wr.close() ) return 11;
  sst_gb300::c_ser_reader back(SER_OUT);
  if( back.num_frames() != 1 || back.timestamps()[0] != 77 ) return 12;
  sst_gb300::c_image_registration_options ro;
  if( ro.ecc.scale != 0.5 || ro.ecc.eps != 0.2 || ro.ecc.ecc_method != SST_ECC_LM || ro.ecc.update_step_scale != 1.5 ||
      ro.ecc.ecch_max_level != 0 || !ro.ecc.ecch_estimate_translation_first || ro.eccflow.scale_factor != 0.75 ||
      ro.eccflow.support_scale != 4 || ro.motion_type != SST_MOTION_AFFINE || !ro.enable_feature_registration )
    return 13;
  sst_gb300::c_frame_registration fr(ro);
  std::vector<float> ref(64 * 48, 1.f);
  if( fr.setup_reference_frame(sst_gb300::image_view(ref.data(), 64, 48, SST_DEPTH_F32, 64 * 4)) ) return 14;
  if( sst_gb300::last_error().find("feature registration") == std::string::npos ) return 15;
  sst_gb300::image_transform ht(SST_MOTION_HOMOGRAPHY);
  ht.parameters = { 1.f, 0.f, 3.f, 0.f, 1.f, -2.f, 1e-5f, 0.f };
  if( !ht.scale_transfrom(2.0) || ht.parameters[2] != 6.f || ht.parameters[5] != -4.f || ht.parameters[6] != 5e-6f )
    return 16;
  if( sizeof(sst_image_registration_options) != 192 ) return 17;
  sst_gb300::c_bayer_average ba;
  ba.set_bayer_pattern(SST_COLORID_BAYER_GRBG);
  if( ba.bayer_pattern() != SST_COLORID_BAYER_GRBG ) return 18;
  sst_gb300::c_eccflow_options fo;
  if( fo.support_scale != 5 || fo.scale_factor != 0.5 ) return 19;
  sst_gb300::c_lpg_options lpo;
  if( lpo.k != 2 || lpo.p != 2 || lpo.dscale != 2 || lpo.uscale != 6 ) return 20;
  sst_gb300::c_lpg_sharpness_measure lpg(lpo);
  if( !lpg.handle() ) return 21;
  sst_gb300::c_laplacian_pyramid_focus_stacking::options fso;
  if( fso.fusing_policy != sst_gb300::c_laplacian_pyramid_focus_stacking::select_max_energy ||
      !fso.inpaint_mask_holes || !fso.avgchannel || fso.kradius != 0 || fso.ksigma != 0 ) return 22;
  sst_gb300::c_laplacian_pyramid_focus_stacking fs(fso);
  sst_gb300::c_frame_accumulation_with_fft fft;
  sst_gb300::c_canvas_average canvas;
  canvas.setCanvasSize(640, 480);
  if( fs.accumulated_frames() != 0 || fft.accumulated_frames() != 0 || canvas.accumulated_frames() != 0 ||
      !canvas.last_bbox().empty() ) return 23;
  std::vector<float> none;
  if( fft.compute(none, *new std::vector<uint8_t>()) ) return 24;      // nothing accumulated
  if( canvas.add(sst_gb300::image_view(), sst_gb300::image_view(), none, sst_gb300::rect()) ) return 25;
  std::printf("ok %s\n", sst_version());
  return 0;
}
'''.replace("SER_PATH", '"' + str(tmp_path / "t.ser") + '"').replace("SER_OUT", '"' + str(tmp_path / "o.ser") + '"'))
    import numpy as np
    from ser_files import write_ser
    frames = (np.arange(3)[:, None, None] * 1000 + np.arange(24).reshape(4, 6)).astype(np.uint16)
    write_ser(tmp_path / "t.ser", frames, bits=12, timestamps=[10, 11, 12])
    libdir = os.path.dirname(capi.LIB_PATH)
    exe = tmp_path / "t"
    subprocess.check_call([gxx, "-std=c++17", "-I", os.path.join(root, "include"), str(src), "-o", str(exe),
                           "-L", libdir, "-lsst_gb300", f"-Wl,-rpath,{libdir}"])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("ok")


def test_local_variance_host_checks(capi):
    """option defaults and argument checks of sst_local_variance_* (no GPU work)"""
    import ctypes as C
    o = capi.local_variance_options()
    assert (o.kradius, o.dscale, o.uscale) == (2, 1, 3)
    h = C.c_void_p()
    assert capi.lib().sst_local_variance_create(C.byref(h), C.byref(capi.local_variance_options(kradius=17))) == -3
    assert not h.value
    assert capi.lib().sst_local_variance_create(C.byref(h), C.byref(capi.local_variance_options(kradius=16))) == 0
    try:
        buf = (C.c_uint16 * 64)()
        lib = capi.lib()
        assert lib.sst_local_variance_compute(h, None, capi.DEPTH_U16, 1, 8, 8, 16, 128, 1.0, 0, None, None, None) == -1
        assert lib.sst_local_variance_compute(h, buf, capi.DEPTH_U16, 0, 8, 8, 16, 128, 1.0, 0, None, None, None) == -1
        assert lib.sst_local_variance_compute(h, buf, 3, 1, 8, 8, 16, 128, 1.0, 0, None, None, None) == -1
        assert lib.sst_local_variance_compute(h, buf, capi.DEPTH_U16, 2, 8, 8, 8, 128, 1.0, 0, None, None, None) == -1
    finally:
        capi.lib().sst_local_variance_destroy(h)


def test_inpaint_argument_checks(capi):
    """sst_average_pyramid_inpaint rejects bad arguments before any GPU work"""
    import ctypes as C
    lib = capi.lib()
    img = (C.c_float * 16)()
    msk = (C.c_uint8 * 16)()
    out = (C.c_float * 16)()
    om = (C.c_uint8 * 16)()
    assert lib.sst_average_pyramid_inpaint(None, 0, msk, 0, 4, 4, 100, out, 0, om, 0, 0, None) == -1
    assert lib.sst_average_pyramid_inpaint(img, 0, msk, 0, 0, 4, 100, out, 0, om, 0, 0, None) == -1
    assert lib.sst_average_pyramid_inpaint(img, 8, msk, 0, 4, 4, 100, out, 0, om, 0, 0, None) == -1   # stride < row
    assert lib.sst_average_pyramid_inpaint(img, 18, msk, 0, 4, 4, 100, out, 0, om, 0, 0, None) == -1  # unaligned


def test_calibration_argument_checks(capi):
    """sst_calibrate_frames rejects bad arguments before any GPU work"""
    lib = capi.lib()
    assert lib.sst_calibrate_frames(None, capi.DEPTH_U16, 1, 8, 8, 16, 128, 1.0, None, 0, None, 0, 1, 0, 0, None) == -1
    assert lib.sst_calibrate_frames(1, capi.DEPTH_U16, 0, 8, 8, 16, 128, 1.0, None, 0, None, 0, 1, 0, 0, None) == -1
    assert lib.sst_calibrate_frames(1, 3, 1, 8, 8, 16, 128, 1.0, None, 0, None, 0, 1, 0, 0, None) == -1
    assert lib.sst_calibrate_frames(1, capi.DEPTH_U16, 2, 8, 8, 16, 100, 1.0, None, 0, None, 0, 1, 0, 0, None) == -1
    assert lib.sst_calibrate_frames(1, capi.DEPTH_U16, 1, 8, 8, 15, 128, 1.0, None, 0, None, 0, 1, 0, 0, None) == -1


def test_registration_options_mirror_the_c_struct(capi):
    """The ctypes mirror of sst_image_registration_options has the C layout
    (192 bytes, checked in the compiled C++ test too) and the reference
    defaults of c_frame_registration.h:47-137."""
    import ctypes
    assert ctypes.sizeof(capi.ImageRegistrationOptions) == 192
    o = capi.ImageRegistrationOptions()
    capi.lib().sst_image_registration_options_default(ctypes.byref(o))
    assert (o.motion_type, o.ecc_registration_channel, o.interpolation, o.border_mode) == (3, 104, 1, 4)
    assert (o.ecc.scale, o.ecc.eps, o.ecc.min_rho, o.ecc.update_step_scale) == (0.5, 0.2, 0.8, 1.5)
    assert (o.ecc.ecc_method, o.ecc.max_iterations, o.ecc.ecch_max_level, o.ecc.ecch_minimum_image_size) == (2, 50, 0, 16)
    assert (o.ecc.normalization_scale, o.ecc.ecch_estimate_translation_first, o.ecc.se_radius) == (0, 1, 5)
    assert (o.eccflow.update_multiplier, o.eccflow.scale_factor, o.eccflow.max_iterations) == (1.5, 0.75, 3)
    assert (o.eccflow.support_scale, o.eccflow.min_image_size, o.eccflow.max_pyramid_level) == (4, -1, -1)
    assert (o.enable_feature_registration, o.enable_ecc_registration, o.enable_eccflow_registration) == (1, 0, 0)


def test_frame_registration_rejects_unsupported_options(capi):
    import ctypes
    h = ctypes.c_void_p()
    o = capi.ImageRegistrationOptions()
    capi.lib().sst_image_registration_options_default(ctypes.byref(o))
    assert capi.lib().sst_frame_registration_create(ctypes.byref(h), ctypes.byref(o)) == capi.ERR_UNSUPPORTED
    assert "feature registration" in capi.last_error()
    o.enable_feature_registration = 0
    assert capi.lib().sst_frame_registration_create(ctypes.byref(h), ctypes.byref(o)) == capi.ERR_INVALID_ARG
    o.enable_ecc_registration = 1
    o.ecc.replace_planetary_disk_with_mask = 1
    assert capi.lib().sst_frame_registration_create(ctypes.byref(h), ctypes.byref(o)) == capi.ERR_UNSUPPORTED
    o.ecc.replace_planetary_disk_with_mask = 0
    assert capi.lib().sst_frame_registration_create(ctypes.byref(h), ctypes.byref(o)) == 0
    assert capi.lib().sst_frame_registration_register_frames(h, ctypes.c_void_p(1), 2, 1, 64, 48, 128, 128 * 48, 1.0,
                                                             0, None, None, None, None, None, None) == capi.ERR_STATE
    capi.lib().sst_frame_registration_destroy(h)


def test_scale_transform_matches_oracle(capi, oracle):
    """sst_image_transform_scale (scale_transfrom) against the oracle's for
    every model."""
    import numpy as np
    O = oracle
    rng = np.random.default_rng(3)
    for t in (0, 1, 2, 3, 4, 5, 6):
        m = O.model(t)
        p = O.get_params(m, O.identity(m)) + rng.normal(0, 1e-3, O.nparams(m))
        want = O.get_params(m, O.scale(m, O.set_params(m, O.identity(m), p), 0.5))
        got = capi.scale_transform(t, p, 0.5)
        assert np.allclose(got, want, rtol=1e-6, atol=1e-6), t


def test_tuning_values_are_checked(capi):
    import ctypes
    C = capi
    reg = C.c_ecch(C.default_options())
    reg.set_tuning({"pass_ctas_per_sm": 2, "pass_tile_w": [64, 128, 0, 0]})
    assert reg.get_tuning()["pass_tile_w"] == [64, 128, 0, 0]
    for bad in ({"pass_tile_w": [32, 0, 0, 0]}, {"pass_ctas_per_sm": -1}, {"stack_max_chunks": 99}):
        t = C.Tuning.from_dict(bad)
        assert C.lib().sst_ecch_set_tuning(reg.handle, ctypes.byref(t)) == C.ERR_INVALID_ARG


def test_lpg_host_checks(capi):
    """c_lpg_options defaults and the argument checks of sst_lpg_* (no GPU work)"""
    import ctypes as C
    o = capi.lpg_options()
    assert (o.k, o.p, o.dscale, o.uscale) == (2.0, 2.0, 2, 6)
    lib = capi.lib()
    h = C.c_void_p()
    assert lib.sst_lpg_create(C.byref(h), C.byref(capi.lpg_options(dscale=-1))) == -1
    assert not h.value
    assert lib.sst_lpg_create(C.byref(h), None) == 0
    try:
        buf = (C.c_uint16 * 144)()
        assert lib.sst_lpg_compute(h, None, capi.DEPTH_U16, 1, 12, 12, 24, 288, None, 0, 0, 0, None, None, None) == -1
        assert lib.sst_lpg_compute(h, buf, 3, 1, 12, 12, 24, 288, None, 0, 0, 0, None, None, None) == -1
        assert lib.sst_lpg_compute(h, buf, capi.DEPTH_U16, 1, 12, 12, 12, 288, None, 0, 0, 0, None, None, None) == -1
        # two pyrDowns of 12 x 12 leave 3 x 3: too small for the 5 x 5 operators
        assert lib.sst_lpg_compute(h, buf, capi.DEPTH_U16, 1, 12, 12, 24, 288, None, 0, 0, 0, None, None, None) == -1
        assert "5 x 5" in capi.last_error()
    finally:
        lib.sst_lpg_destroy(h)


def test_debayer_nn2_argument_checks(capi):
    """sst_debayer_nn2 rejects bad arguments before any GPU work"""
    lib = capi.lib()
    assert lib.sst_debayer_nn2(None, capi.DEPTH_U16, 1, 8, 8, 16, 128, 8, 1, 0, 0, None) == -1
    assert lib.sst_debayer_nn2(1, capi.DEPTH_U16, 1, 8, 8, 16, 128, 7, 1, 0, 0, None) == -1    # not a Bayer pattern
    assert lib.sst_debayer_nn2(1, capi.DEPTH_U16, 1, 9, 8, 18, 144, 8, 1, 0, 0, None) == -1    # odd width
    assert lib.sst_debayer_nn2(1, capi.DEPTH_U16, 1, 8, 8, 14, 128, 8, 1, 0, 0, None) == -1    # short rows
    assert lib.sst_debayer_nn2(1, 6, 1, 8, 8, 64, 512, 8, 1, 0, 0, None) == -1                 # f64


def test_accumulator_host_checks(capi):
    """defaults and argument checks of the FFT, canvas and focus-stacking
    accumulators (no GPU work)"""
    import ctypes as C
    lib = capi.lib()
    assert [lib.sst_optimal_dft_size(n) for n in (1, 7, 29, 960, 1021)] == [1, 8, 30, 960, 1024]
    o = capi.focus_stack_options()
    assert (o.fusing_policy, o.inpaint_mask_holes, o.avgchannel, o.kradius, o.ksigma) == (0, 1, 1, 0, 0.0)
    h = C.c_void_p()
    assert lib.sst_focus_stack_create(C.byref(h), C.byref(capi.focus_stack_options(fusing_policy=7))) == -1
    assert lib.sst_focus_stack_create(C.byref(h), C.byref(capi.focus_stack_options(kradius=-1))) == -1
    assert not h.value
    buf = (C.c_float * 64)()
    f = C.c_void_p()
    assert lib.sst_fft_average_create(C.byref(f)) == 0
    try:
        assert lib.sst_fft_average_add(f, None, capi.DEPTH_F32, 1, 8, 8, 1, 32, 256, 1.0, 0, None) == -1
        assert lib.sst_fft_average_add(f, buf, capi.DEPTH_F32, 1, 8, 8, 5, 160, 1280, 1.0, 0, None) == -1
        assert lib.sst_fft_average_add(f, buf, capi.DEPTH_F32, 1, 8, 8, 1, 16, 256, 1.0, 0, None) == -1
        assert lib.sst_fft_average_compute(f, buf, 0, None, 0, 0, None) == -4      # empty: SST_ERR_STATE
    finally:
        lib.sst_fft_average_destroy(f)
    c = C.c_void_p()
    assert lib.sst_canvas_average_create(C.byref(c), 0, 0) == 0
    try:
        assert lib.sst_canvas_average_add(c, buf, capi.DEPTH_F32, 8, 8, 1, 16, 1.0, None, 0, 0, None, None, 0,
                                          None) == -1
        assert lib.sst_canvas_average_add(c, buf, capi.DEPTH_F32, 8, 8, 1, 32, 1.0, buf, 2, 32, None, None, 0,
                                          None) == -1    # u16 weights
        assert lib.sst_canvas_average_compute(c, buf, 0, None, 0, 1.0, None, None, 0, None) == -4
    finally:
        lib.sst_canvas_average_destroy(c)


def test_filter_bad_pixels_argument_checks(capi):
    """sst_filter_bad_pixels rejects bad arguments before any GPU work"""
    lib = capi.lib()
    assert lib.sst_filter_bad_pixels(None, capi.DEPTH_U16, 1, 8, 8, 16, 128, 0, 3.0, 1, 0, 0, None) == -1
    assert lib.sst_filter_bad_pixels(1, capi.DEPTH_U16, 1, 9, 8, 18, 144, 8, 3.0, 1, 0, 0, None) == -1   # odd Bayer
    assert lib.sst_filter_bad_pixels(1, 6, 1, 8, 8, 64, 512, 0, 3.0, 1, 0, 0, None) == -1               # f64
    assert lib.sst_filter_bad_pixels(1, capi.DEPTH_U16, 1, 8, 8, 14, 128, 0, 3.0, 1, 0, 0, None) == -1  # short rows
