/*
 * serstacker_gb300.hpp -- C++ drop-in classes for SerStacker's registration
 * and stacking hot path, over the C ABI of libsst_gb300.so.
 *
 * The class, option and method names follow the reference interfaces they
 * replace (paths relative to the SerStacker source tree):
 *   sst_gb300::c_ecch_options      core/proc/image_registration/ecc2.h:158-172
 *   sst_gb300::c_ecch              core/proc/image_registration/ecc2.h:193-308
 *   sst_gb300::image_transform     core/proc/image_registration/c_image_transform.h:42-117
 *                                  (parameters, scale_transfrom, create_remap)
 *   sst_gb300::c_eccflow           core/proc/image_registration/ecc2.h:548-662
 *   sst_gb300::c_ecc_registration_options, c_eccflow_registration_options,
 *   c_image_registration_options, c_frame_registration
 *                                  core/proc/image_registration/c_frame_registration.h:47-356
 *   sst_gb300::c_weigthed_average  core/average/c_frame_accumulation.h:39-63
 *   sst_gb300::c_bayer_average     core/average/c_frame_accumulation.h:222-262
 *   sst_gb300::c_local_variance_map_options, c_local_variance_sharpness_measure
 *                                  core/proc/sharpness_measure/c_local_variance_sharpness_measure.h:17-23
 *   sst_gb300::c_ser_reader        core/io/c_ser_file.h:136-174
 *   sst_gb300::c_ser_writer        core/io/c_ser_file.h:183-213
 *   sst_gb300::average_pyramid_inpaint  core/proc/inpaint/average_pyramid_inpaint.h:14-18
 *   sst_gb300::linear_interpolation_inpaint  core/proc/inpaint/linear_interpolation_inpaint.h
 *   sst_gb300::c_lpg_options, c_lpg_sharpness_measure
 *                                  core/proc/sharpness_measure/c_lpg_sharpness_measure.h:22-80
 *   sst_gb300::c_frame_accumulation_with_fft, c_canvas_average,
 *   c_laplacian_pyramid_focus_stacking
 *                                  core/average/c_frame_accumulation.h:65-199
 * (read_input_frame's NN2 debayer and bad-pixel filter work on device frames:
 * sst_debayer_nn2 / sst_filter_bad_pixels of the C ABI.)
 * Images are passed as `image_view` (pointer, size, OpenCV depth code,
 * stride) instead of cv::Mat, so this header needs no OpenCV; define
 * SST_GB300_WITH_OPENCV before including it to get cv::Mat overloads.
 * Errors follow the reference convention: methods return bool, and the
 * reason is available from last_error() (the reference logs it with CF_ERROR).
 */
#pragma once
#include "serstacker_gb300.h"

#include <cstdint>
#include <string>
#include <vector>

#ifdef SST_GB300_WITH_OPENCV
#include <opencv2/core.hpp>
#endif

namespace sst_gb300 {

inline std::string last_error() { return sst_last_error(); }

/* A host image: row-major pixels of OpenCV depth `depth` (CV_8U, CV_16U, CV_32F). */
struct image_view {
  const void * data = nullptr;
  int width = 0, height = 0;
  int depth = SST_DEPTH_F32;
  size_t stride = 0;        // bytes per row

  image_view() = default;
  image_view(const void * d, int w, int h, int dp, size_t s) : data(d), width(w), height(h), depth(dp), stride(s) {}
#ifdef SST_GB300_WITH_OPENCV
  image_view(const cv::Mat & m) : data(m.data), width(m.cols), height(m.rows), depth(m.depth()), stride(m.step) {}
#endif
  bool empty() const { return data == nullptr || width <= 0 || height <= 0; }
};

/* c_ecch_options (ecc2.h:158-172), same field names and defaults */
struct c_ecch_options {
  double epsx = 1e-5;
  double reference_smooth_sigma = 1;
  double input_smooth_sigma = 1;
  double update_step_scale = 1;
  int method = SST_ECC_INVERSE_COMPOSITIONAL_LM;
  int interpolation = 1;      // ECC_INTER_LINEAR
  int max_iterations = 50;
  int minimum_image_size = 8;
  int maxlevel = 0;
};

/* The motion model and its parameter vector: the c_image_transform object of
 * create_image_transform() (image_transform.cc:32-60) with its
 * parameters() / set_parameters(), scale_transfrom() and create_remap()
 * (c_image_transform.h:42-117). An empty parameter vector is the identity. */
struct image_transform {
  sst_motion_model model { SST_MOTION_AFFINE, 0, 0, 0 };
  std::vector<float> parameters;

  explicit image_transform(int motion_type = SST_MOTION_AFFINE)
  {
    model.type = motion_type;
    model.fix_scale = motion_type == SST_MOTION_EUCLIDEAN ? 1 : 0;
  }

  int num_parameters() const
  {
    switch ( model.type ) {
    case SST_MOTION_TRANSLATION: return 2;
    case SST_MOTION_EUCLIDEAN:
    case SST_MOTION_SCALED_EUCLIDEAN:
      return (model.fix_translation ? 0 : 2) + (model.fix_rotation ? 0 : 1) + (model.fix_scale ? 0 : 1);
    case SST_MOTION_AFFINE: return 6;
    case SST_MOTION_QUADRATIC: return 12;
    default: return 8;
    }
  }

  /* c_image_transform::set_parameters / parameters */
  void set_parameters(const std::vector<float> & p) { parameters = p; }
  std::vector<float> get_parameters() const
  {
    float p[12] = { 0 };
    fill(p);
    return std::vector<float>(p, p + num_parameters());
  }

  /* c_image_transform::scale_transfrom(factor) */
  bool scale_transfrom(double factor)
  {
    float p[12] = { 0 };
    fill(p);
    if( sst_image_transform_scale(&model, p, factor) != SST_OK ) return false;
    parameters.assign(p, p + num_parameters());
    return true;
  }

  /* c_image_transform::create_remap(size, map): width x height x 2 floats */
  bool create_remap(int width, int height, std::vector<float> & map) const
  {
    float p[12] = { 0 };
    fill(p);
    map.resize((size_t) width * height * 2);
    return sst_image_transform_create_remap(&model, p, width, height, map.data(), 0, nullptr) == SST_OK;
  }

  /* the parameter vector, the identity when none is set */
  void fill(float * p) const
  {
    if( !parameters.empty() ) {
      for( size_t i = 0; i < parameters.size() && i < 12; ++i ) p[i] = parameters[i];
      return;
    }
    switch ( model.type ) {
    case SST_MOTION_EUCLIDEAN:
    case SST_MOTION_SCALED_EUCLIDEAN:
      if( !model.fix_scale ) p[(model.fix_translation ? 0 : 2) + (model.fix_rotation ? 0 : 1)] = 1;
      break;
    case SST_MOTION_AFFINE:
    case SST_MOTION_HOMOGRAPHY:
    case SST_MOTION_EPIPOLAR_DEROTATION: p[0] = 1, p[4] = 1; break;
    case SST_MOTION_SEMI_QUADRATIC: p[0] = 1, p[5] = 1; break;
    case SST_MOTION_QUADRATIC: p[0] = 1, p[7] = 1; break;
    default: break;
    }
  }
};

/* c_ecch on the GPU. align() registers one frame (one launch per
 * Gauss-Newton step, like the reference's per-frame loop); align_batch()
 * registers a whole sequence in one graph replay. */
class c_ecch {
public:
  c_ecch() { create(); }
  explicit c_ecch(const c_ecch_options & opts) : _opts(opts) { create(); }
  ~c_ecch() { if( _h ) sst_ecch_destroy(_h); }
  c_ecch(const c_ecch &) = delete;
  c_ecch & operator=(const c_ecch &) = delete;

  const c_ecch_options & options() const { return _opts; }
  void set_options(const c_ecch_options & o) { _opts = o; create(); }
  void set_min_rho(double v) { _min_rho = v; create(); }

  void set_image_transform(image_transform * t) { _transform = t; }
  image_transform * image_transform_ptr() const { return _transform; }

  /* c_ecch::set_reference_image (ecc2.cc:984-1057) */
  bool set_reference_image(const image_view & img, const image_view & mask = image_view(), double scale = 1.0)
  {
    if( !_h ) return false;
    if( sst_ecch_set_reference_image(_h, img.data, img.depth, img.width, img.height, img.stride, scale,
            (const uint8_t *) mask.data, mask.stride, 0, nullptr) != SST_OK )
      return false;
    _ref_w = img.width, _ref_h = img.height;
    return true;
  }

  /* c_ecch::set_current_image(current_image) (ecc2.cc:1060-1120): the frame
   * the next align() registers (kept by reference, as a view) */
  bool set_current_image(const image_view & img, double scale = 1.0)
  {
    if( img.empty() ) return false;
    _current = img;
    _current_scale = scale;
    return true;
  }

  /* c_ecch::align() (ecc2.cc:1133-1176) of the current image */
  bool align() { return !_current.empty() && align(_current, _current_scale); }

  /* c_ecch::create_remap(map) (ecc2.h:300): the attached transform's remap at
   * the reference size, width x height x 2 floats */
  bool create_remap(std::vector<float> & map) const
  {
    return _transform && _ref_w > 0 && _transform->create_remap(_ref_w, _ref_h, map);
  }

  /* c_ecch::align(current_image, current_mask) (ecc2.cc:1123-1176): updates the
   * attached image_transform's parameters in place, as the reference does. */
  bool align(const image_view & img, double scale = 1.0)
  {
    if( !_h || !_transform ) return false;
    float params[12] = { 0 };
    for( size_t i = 0; i < _transform->parameters.size() && i < 12; ++i ) params[i] = _transform->parameters[i];
    int32_t status = 0, iters = 0;
    float eps = 0, rho = 0;
    const int rc = sst_ecch_align_plain(_h, img.data, img.depth, 1, img.width, img.height, img.stride,
        img.stride * img.height, scale, 0, 1, &_transform->model, _transform->parameters.empty() ? 0 : 1,
        params, &status, &iters, &eps, &rho, nullptr, nullptr);
    if( rc != SST_OK ) return false;
    const int M = nparams(_transform->model);
    _transform->parameters.assign(params, params + M);
    _eps = eps, _num_iterations = iters, _rho = rho;
    return status == SST_FRAME_OK;
  }

  /* n frames (host, consecutive with `frame_stride` bytes) through the batched engine. */
  bool align_batch(const void * frames, int depth, int n, int width, int height, size_t row_stride, size_t frame_stride,
      const std::vector<sst_motion_model> & passes, std::vector<float> & params /* n x 12 */,
      std::vector<int32_t> & status, double scale = 1.0)
  {
    if( !_h ) return false;
    params.assign((size_t) n * 12, 0.f);
    status.assign(n, 0);
    return sst_ecch_align_batch(_h, frames, depth, n, width, height, row_stride, frame_stride, scale, 0,
        (int) passes.size(), passes.data(), 0, params.data(), status.data(), nullptr, nullptr, nullptr, nullptr,
        nullptr) == SST_OK;
  }

  double eps() const { return _eps; }
  int num_iterations() const { return _num_iterations; }
  double rho() const { return _rho; }
  int num_levels() const { return _h ? sst_ecch_num_levels(_h) : 0; }
  /* pyramid level of the reference / of frame `frame` of the last batch into
   * out (host memory, lw x lh floats) */
  bool reference_image(int level, float * out) const { return _h && sst_ecch_reference_image(_h, level, out, 0) == SST_OK; }
  bool current_image(int frame, int level, float * out) const
  {
    return _h && sst_ecch_current_image(_h, frame, level, out, 0) == SST_OK;
  }
  sst_ecch * handle() const { return _h; }

  static int nparams(const sst_motion_model & m)
  {
    switch ( m.type ) {
    case SST_MOTION_TRANSLATION: return 2;
    case SST_MOTION_EUCLIDEAN:
    case SST_MOTION_SCALED_EUCLIDEAN:
      return (m.fix_translation ? 0 : 2) + (m.fix_rotation ? 0 : 1) + (m.fix_scale ? 0 : 1);
    case SST_MOTION_AFFINE: return 6;
    case SST_MOTION_QUADRATIC: return 12;
    default: return 8;
    }
  }

private:
  void create()
  {
    if( _h ) sst_ecch_destroy(_h), _h = nullptr;
    sst_ecch_options o;
    sst_ecch_options_default(&o);
    o.epsx = _opts.epsx;
    o.reference_smooth_sigma = _opts.reference_smooth_sigma;
    o.input_smooth_sigma = _opts.input_smooth_sigma;
    o.update_step_scale = _opts.update_step_scale;
    o.method = _opts.method;
    o.interpolation = _opts.interpolation;
    o.max_iterations = _opts.max_iterations;
    o.minimum_image_size = _opts.minimum_image_size;
    o.maxlevel = _opts.maxlevel;
    o.min_rho = _min_rho;
    if( sst_ecch_create(&_h, &o) != SST_OK ) _h = nullptr;
  }

  c_ecch_options _opts;
  double _min_rho = 0;
  sst_ecch * _h = nullptr;
  image_transform * _transform = nullptr;
  image_view _current;
  double _current_scale = 1.0;
  int _ref_w = 0, _ref_h = 0;
  double _eps = -1, _rho = -1;
  int _num_iterations = -1;
};

/* c_weigthed_average (c_frame_accumulation.h:39-63) on the GPU */
class c_weigthed_average {
public:
  c_weigthed_average() = default;
  ~c_weigthed_average() { if( _h ) sst_weighted_average_destroy(_h); }
  c_weigthed_average(const c_weigthed_average &) = delete;
  c_weigthed_average & operator=(const c_weigthed_average &) = delete;

  /* c_weigthed_average::add(src, weights) (c_frame_accumulation.cc:182-221) */
  bool add(const image_view & src, const image_view & weights = image_view(), double scale = 1.0)
  {
    if( !ensure(src.width, src.height) ) return false;
    return sst_weighted_average_add(_h, src.data, src.depth, src.stride, scale, weights.data, weights.depth,
        weights.stride, 0, nullptr) == SST_OK;
  }

  /* warp with the registered transform, weight and add (the stacking
   * pipeline's per-frame body, c_image_stacking_pipeline.cc:1644-1790) */
  bool add_warped(const image_view & src, const image_transform & t, float weight = 1.f, double scale = 1.0,
      int border = SST_BORDER_REFLECT101)
  {
    if( !ensure(src.width, src.height) ) return false;
    float p[12] = { 0 };
    for( size_t i = 0; i < t.parameters.size() && i < 12; ++i ) p[i] = t.parameters[i];
    int32_t st = SST_FRAME_OK;
    return sst_weighted_average_add_warped_batch(_h, src.data, src.depth, 1, src.width, src.height, src.stride,
        src.stride * src.height, scale, 0, &t.model, p, &st, &weight, border, nullptr) == SST_OK;
  }

  /* c_weigthed_average::compute (c_frame_accumulation.cc:223-248) */
  bool compute(std::vector<float> & avg, std::vector<uint8_t> & mask) const
  {
    if( !_h ) return false;
    avg.resize((size_t) _w * _hh);
    mask.resize((size_t) _w * _hh);
    return sst_weighted_average_compute(_h, avg.data(), mask.data(), 0, nullptr) == SST_OK;
  }

  bool get_acc_counters(std::vector<float> & accw) const
  {
    if( !_h ) return false;
    accw.resize((size_t) _w * _hh);
    return sst_weighted_average_get_acc_counters(_h, accw.data(), 0, nullptr) == SST_OK;
  }

  bool reinitialize(const std::vector<float> & avg, const std::vector<float> & accw, int width, int height)
  {
    if( !ensure(width, height) ) return false;
    return sst_weighted_average_reinitialize(_h, avg.data(), accw.data(), 0, nullptr) == SST_OK;
  }

  /* c_frame_accumulation_options::sharpness_measure: the map options of the
   * stacking pipeline's local-variance weights (sst_stack_frames weighting 3) */
  bool set_sharpness_measure(int kradius, int dscale, int uscale)
  {
    if( !_h ) return false;
    const sst_local_variance_options o = { kradius, dscale, uscale };
    return sst_weighted_average_set_local_variance(_h, &o) == SST_OK;
  }

  /* the accumulator must exist before its options can be set */
  bool create(int width, int height) { return ensure(width, height); }

  void clear() { if( _h ) sst_weighted_average_clear(_h, nullptr); }
  int accumulated_frames() const { return _h ? sst_weighted_average_accumulated_frames(_h) : 0; }
  int width() const { return _w; }
  int height() const { return _hh; }
  sst_weighted_average * handle() const { return _h; }

private:
  bool ensure(int w, int h)
  {
    if( _h && w == _w && h == _hh ) return true;
    if( _h ) return false;   // size mismatch: the reference rejects it (c_frame_accumulation.cc:195-200)
    if( sst_weighted_average_create(&_h, w, h) != SST_OK ) return false;
    _w = w, _hh = h;
    return true;
  }
  sst_weighted_average * _h = nullptr;
  int _w = 0, _hh = 0;
};

/* average_pyramid_inpaint (core/proc/inpaint/average_pyramid_inpaint.h:14-18)
 * on the GPU for a host image and mask of width x height (packed rows), in
 * place: the stacking pipeline's fill of the master frame's holes */
inline bool average_pyramid_inpaint(std::vector<float> & image, std::vector<uint8_t> & mask, int width, int height,
    int max_levels = 100)
{
  if( image.size() != (size_t) width * height || mask.size() != image.size() ) return false;
  std::vector<float> out(image.size());
  std::vector<uint8_t> om(mask.size());
  if( sst_average_pyramid_inpaint(image.data(), 0, mask.data(), 0, width, height, max_levels, out.data(), 0,
          om.data(), 0, 0, nullptr) != SST_OK )
    return false;
  image.swap(out);
  mask.swap(om);
  return true;
}

/* c_local_variance_map_options (c_local_variance_sharpness_measure.h:17-23) */
struct c_local_variance_map_options {
  int kradius = 2;
  int dscale = 1;
  int uscale = 3;
};

/* c_local_variance_sharpness_measure::create_map on the GPU: the map of a
 * host image converted to FP32 by `scale` (depthScale 20, the stacking
 * pipeline's CV_32F frames), returned at the image's size, and its quality Q */
class c_local_variance_sharpness_measure {
public:
  explicit c_local_variance_sharpness_measure(const c_local_variance_map_options & o = c_local_variance_map_options())
  {
    const sst_local_variance_options so = { o.kradius, o.dscale, o.uscale };
    if( sst_local_variance_create(&_h, &so) != SST_OK ) _h = nullptr;
  }
  ~c_local_variance_sharpness_measure() { if( _h ) sst_local_variance_destroy(_h); }
  c_local_variance_sharpness_measure(const c_local_variance_sharpness_measure &) = delete;
  c_local_variance_sharpness_measure & operator=(const c_local_variance_sharpness_measure &) = delete;

  bool create_map(const image_view & image, std::vector<float> & map, double * q = nullptr, double scale = 1.0)
  {
    if( !_h || image.empty() ) return false;
    map.resize((size_t) image.width * image.height);
    double qq = 0;
    const bool ok = sst_local_variance_compute(_h, image.data, image.depth, 1, image.width, image.height, image.stride,
        image.stride * image.height, scale, 0, map.data(), &qq, nullptr) == SST_OK;
    if( q ) *q = qq;
    return ok;
  }

  sst_local_variance * handle() const { return _h; }

private:
  sst_local_variance * _h = nullptr;
};

/* c_ser_reader (core/io/c_ser_file.h:136-174): header accessors, seek /
 * curpos and frame reads into a host buffer (pixel data byte-swapped to the
 * host's order). read() fills `frame` with one frame of frame_size() bytes. */
class c_ser_reader {
public:
  c_ser_reader() = default;
  explicit c_ser_reader(const std::string & filename) { open(filename); }
  ~c_ser_reader() { close(); }
  c_ser_reader(const c_ser_reader &) = delete;
  c_ser_reader & operator=(const c_ser_reader &) = delete;

  bool open(const std::string & filename)
  {
    close();
    if( sst_ser_open(&_h, filename.c_str()) != SST_OK ) return false;
    sst_ser_get_info(_h, &_info);
    return true;
  }
  void close()
  {
    if( _h ) sst_ser_close(_h);
    _h = nullptr;
  }
  bool is_open() const { return _h != nullptr; }

  int image_width() const { return _info.width; }
  int image_height() const { return _info.height; }
  int bits_per_plane() const { return _info.bits_per_plane; }
  int bytes_per_plane() const { return _info.bytes_per_plane; }
  int color_id() const { return _info.color_id; }
  int channels() const { return _info.channels; }
  int num_frames() const { return _info.frames; }
  int depth() const { return _info.depth; }
  const char * observer() const { return _info.observer; }
  const char * instrument() const { return _info.instrument; }
  const char * telescope() const { return _info.telescope; }
  size_t frame_size() const { return (size_t) _info.width * _info.height * _info.channels * _info.bytes_per_plane; }
  const sst_ser_info & info() const { return _info; }

  std::vector<uint64_t> timestamps() const
  {
    std::vector<uint64_t> ts;
    if( _h && _info.has_timestamps ) {
      ts.resize(_info.frames);
      sst_ser_timestamps(_h, ts.data(), _info.frames);
    }
    return ts;
  }

  int curpos() const { return _h ? sst_ser_curpos(_h) : -1; }
  bool seek(int frame_index) { return _h && sst_ser_seek(_h, frame_index) == SST_OK; }

  bool read(std::vector<uint8_t> & frame)
  {
    if( !_h ) return false;
    frame.resize(frame_size());
    int got = 0;
    return sst_ser_read(_h, 1, frame.data(), 0, &got) == SST_OK && got == 1;
  }
#ifdef SST_GB300_WITH_OPENCV
  bool read(cv::Mat & image)
  {
    if( !_h || _info.depth < 0 ) return false;
    image.create(_info.height, _info.width, CV_MAKETYPE(_info.depth, _info.channels));
    int got = 0;
    return sst_ser_read(_h, 1, image.data, 0, &got) == SST_OK && got == 1;
  }
#endif

  sst_ser_reader * handle() const { return _h; }

private:
  sst_ser_reader * _h = nullptr;
  sst_ser_info _info {};
};

/* c_ser_writer (core/io/c_ser_file.h:183-213): create, write frames of the
 * file's format with their timestamps, close (FrameCount and the trailer). */
class c_ser_writer {
public:
  ~c_ser_writer() { close(); }
  bool create(const std::string & filename, int image_width, int image_height, int color_id, int bits_per_plane)
  {
    close();
    return sst_ser_writer_create(&_h, filename.c_str(), image_width, image_height, color_id, bits_per_plane) == SST_OK;
  }
  bool is_open() const { return _h != nullptr; }
  bool write(const void * frame, uint64_t ts = UINT64_MAX) { return _h && sst_ser_write(_h, frame, 1, 0, &ts) == SST_OK; }
#ifdef SST_GB300_WITH_OPENCV
  bool write(const cv::Mat & image, uint64_t ts = UINT64_MAX) { return image.isContinuous() && write(image.data, ts); }
#endif
  bool close()
  {
    const bool ok = !_h || sst_ser_writer_close(_h) == SST_OK;
    _h = nullptr;
    return ok;
  }

private:
  sst_ser_writer * _h = nullptr;
};

/* c_eccflow_options (ecc2.h:515-527) */
struct c_eccflow_options {
  double update_multiplier = 1.5;
  double scale_factor = 0.5;
  double noise_level = -1;
  double input_smooth_sigma = 0;
  double reference_smooth_sigma = 0;
  int max_iterations = 1;
  int support_scale = 5;
  int min_image_size = 4;
  int max_pyramid_level = -1;
  int downscale_method = SST_ECCFLOW_DOWNSCALE_RECURSIVE_RESIZE;
};

/* c_eccflow (ecc2.h:548-662) on the GPU: set_reference_image(reference),
 * compute(current, rmap) refining rmap (width x height x 2 floats, the
 * identity when empty) in place. */
class c_eccflow {
public:
  c_eccflow() { create(); }
  explicit c_eccflow(const c_eccflow_options & o) : _opts(o) { create(); }
  ~c_eccflow() { if( _h ) sst_eccflow_destroy(_h); }
  c_eccflow(const c_eccflow &) = delete;
  c_eccflow & operator=(const c_eccflow &) = delete;

  const c_eccflow_options & options() const { return _opts; }
  void set_options(const c_eccflow_options & o) { _opts = o; create(); }

  /* c_eccflow::set_reference_image(reference, reference_mask) (ecc2.cc:2489-2672) */
  bool set_reference_image(const image_view & img, const image_view & mask = image_view(), double scale = 1.0)
  {
    if( !_h || img.empty() ) return false;
    if( sst_eccflow_set_reference_image_masked(_h, img.data, img.depth, img.width, img.height, img.stride, scale,
            (const uint8_t *) mask.data, mask.stride, 0, nullptr) != SST_OK )
      return false;
    _w = img.width, _hh = img.height;
    return true;
  }

  /* c_eccflow::compute(current, rmap, current_mask) (ecc2.cc:2856-2865) */
  bool compute(const image_view & current, std::vector<float> & rmap, const image_view & mask = image_view(),
      double scale = 1.0)
  {
    if( !_h || current.width != _w || current.height != _hh ) return false;
    const size_t n = (size_t) _w * _hh * 2;
    const bool have_init = rmap.size() == n;
    std::vector<float> out(n);
    if( sst_eccflow_compute_batch_masked(_h, current.data, current.depth, 1, current.stride,
            current.stride * current.height, scale, (const uint8_t *) mask.data, mask.stride,
            mask.stride * current.height, 0, have_init ? rmap.data() : nullptr, out.data(), nullptr) != SST_OK )
      return false;
    rmap.swap(out);
    return true;
  }

  int num_levels() const { return _h ? sst_eccflow_num_levels(_h) : 0; }
  sst_eccflow * handle() const { return _h; }

private:
  void create()
  {
    if( _h ) sst_eccflow_destroy(_h), _h = nullptr;
    sst_eccflow_options o;
    sst_eccflow_options_default(&o);
    o.update_multiplier = _opts.update_multiplier;
    o.scale_factor = _opts.scale_factor;
    o.noise_level = _opts.noise_level;
    o.input_smooth_sigma = _opts.input_smooth_sigma;
    o.reference_smooth_sigma = _opts.reference_smooth_sigma;
    o.max_iterations = _opts.max_iterations;
    o.support_scale = _opts.support_scale;
    o.min_image_size = _opts.min_image_size;
    o.max_pyramid_level = _opts.max_pyramid_level;
    o.downscale = _opts.downscale_method;
    if( sst_eccflow_create(&_h, &o) != SST_OK ) _h = nullptr;
  }
  c_eccflow_options _opts;
  sst_eccflow * _h = nullptr;
  int _w = 0, _hh = 0;
};

/* c_ecc_registration_options (c_frame_registration.h:47-63) */
struct c_ecc_registration_options {
  double scale = 0.5;
  double eps = 0.2;
  double min_rho = 0.8;
  double input_smooth_sigma = 1.0;
  double reference_smooth_sigma = 1.0;
  double update_step_scale = 1.5;
  int se_radius = 5;
  int ecc_method = SST_ECC_LM;
  int max_iterations = 50;
  int ecch_max_level = 0;
  int ecch_minimum_image_size = 16;
  double normalization_noise = 0.01;
  int normalization_scale = 0;
  bool ecch_estimate_translation_first = true;
  bool replace_planetary_disk_with_mask = false;
};

/* c_eccflow_registration_options (c_frame_registration.h:88-100) */
struct c_eccflow_registration_options {
  double update_multiplier = 1.5;
  double input_smooth_sigma = 0;
  double reference_smooth_sigma = 0;
  double noise_level = -1;
  double scale_factor = 0.75;
  int max_iterations = 3;
  int support_scale = 4;
  int min_image_size = -1;
  int max_pyramid_level = -1;
  int downscale_method = SST_ECCFLOW_DOWNSCALE_RECURSIVE_RESIZE;
};

/* c_image_registration_options (c_frame_registration.h:119-137). The
 * reference enables feature registration by default; this library has no
 * feature registration, so create() fails unless it is switched off. */
struct c_image_registration_options {
  int motion_type = SST_MOTION_AFFINE;
  int ecc_registration_channel = SST_COLOR_CHANNEL_GRAY;
  int interpolation = 1;                       // ECC_INTER_LINEAR
  int border_mode = SST_BORDER_REFLECT101;
  double border_value = 0;
  c_ecc_registration_options ecc;
  c_eccflow_registration_options eccflow;
  bool enable_feature_registration = true;
  bool enable_ecc_registration = false;
  bool enable_eccflow_registration = false;
  bool accumulate_and_compensate_turbulent_flow = false;
};

/* c_image_registration_status (c_frame_registration.h:185-207), the fields
 * the GPU path fills */
struct c_image_registration_status {
  double rho = -1;
  int num_iterations = 0;
  int frame_status = SST_FRAME_OK;
};

/* c_frame_registration (c_frame_registration.h:210-356) on the GPU for mono
 * frames: setup_reference_frame, register_frame (ECC with ecc.scale,
 * ecc_normalize and the translation estimate, then eccflow), remap /
 * custom_remap by the current remap, current_remap, image_transform, status.
 * register_frames registers a whole batch in one engine schedule. */
class c_frame_registration {
public:
  c_frame_registration() = default;
  explicit c_frame_registration(const c_image_registration_options & o) : _opts(o) {}
  ~c_frame_registration() { if( _h ) sst_frame_registration_destroy(_h); }
  c_frame_registration(const c_frame_registration &) = delete;
  c_frame_registration & operator=(const c_frame_registration &) = delete;

  const c_image_registration_options & options() const { return _opts; }
  c_image_registration_options & options() { return _opts; }

  /* setup_reference_frame(reference_image, reference_mask) (c_frame_registration.cc:565-719) */
  bool setup_reference_frame(const image_view & reference_image, const image_view & reference_mask = image_view(),
      double scale = 1.0)
  {
    if( !create() || reference_image.empty() ) return false;
    if( sst_frame_registration_setup_reference_frame(_h, reference_image.data, reference_image.depth,
            reference_image.width, reference_image.height, reference_image.stride, scale,
            (const uint8_t *) reference_mask.data, reference_mask.stride, 0, nullptr) != SST_OK )
      return false;
    _w = reference_image.width, _hh = reference_image.height;
    return true;
  }

  /* register_frame(current_image, current_mask, dst, dstmask)
   * (c_frame_registration.cc:721-964): false when registration fails (the
   * status says why); dst / dst_mask (optional, reference-size f32 / u8)
   * receive remap() of the frame */
  bool register_frame(const image_view & current_image, std::vector<float> * dst = nullptr,
      std::vector<uint8_t> * dst_mask = nullptr, double scale = 1.0)
  {
    if( !_h || current_image.width != _w || current_image.height != _hh ) return false;
    float params[12] = { 0 };
    int32_t status = 0, iters = 0;
    float rho = 0;
    _remap.resize((size_t) _w * _hh * 2);
    if( sst_frame_registration_register_frames(_h, current_image.data, current_image.depth, 1, _w, _hh,
            current_image.stride, current_image.stride * _hh, scale, 0, params, &status, &rho, &iters, _remap.data(),
            nullptr) != SST_OK )
      return false;
    _transform.parameters.assign(params, params + _transform.num_parameters());
    _status.rho = rho, _status.num_iterations = iters, _status.frame_status = status;
    if( status != SST_FRAME_OK ) return false;
    if( dst || dst_mask ) return remap(current_image, dst, image_view(), dst_mask, scale);
    return true;
  }

  /* register_frames: n frames (host, frame_stride bytes apart) in one batch;
   * params n x 12, status / rho per frame */
  bool register_frames(const void * frames, int depth, int n, size_t row_stride, size_t frame_stride,
      std::vector<float> & params, std::vector<int32_t> & status, std::vector<float> & rho, double scale = 1.0)
  {
    if( !_h ) return false;
    params.assign((size_t) n * 12, 0.f);
    status.assign(n, 0);
    rho.assign(n, 0.f);
    return sst_frame_registration_register_frames(_h, frames, depth, n, _w, _hh, row_stride, frame_stride, scale, 0,
        params.data(), status.data(), rho.data(), nullptr, nullptr, nullptr) == SST_OK;
  }

  /* remap(src, dst, src_mask, dst_mask) (c_frame_registration.cc:1386-1400):
   * base_remap with the current remap, the options' border */
  bool remap(const image_view & src, std::vector<float> * dst, const image_view & src_mask = image_view(),
      std::vector<uint8_t> * dst_mask = nullptr, double scale = 1.0) const
  {
    return custom_remap(_remap, src, dst, src_mask, dst_mask, scale);
  }

  /* custom_remap(rmap, src, dst, src_mask, dst_mask) (c_frame_registration.cc:1342-1384) */
  bool custom_remap(const std::vector<float> & rmap, const image_view & src, std::vector<float> * dst,
      const image_view & src_mask = image_view(), std::vector<uint8_t> * dst_mask = nullptr, double scale = 1.0) const
  {
    if( rmap.size() != (size_t) _w * _hh * 2 || src.empty() ) return false;
    if( dst ) dst->resize((size_t) _w * _hh);
    if( dst_mask ) dst_mask->resize((size_t) _w * _hh);
    return sst_remap_rmap(src.data, src.depth, src.width, src.height, src.stride, scale, rmap.data(), _w, _hh,
        _opts.border_mode, _opts.border_value, (const uint8_t *) src_mask.data, src_mask.stride,
        dst ? dst->data() : nullptr, dst_mask ? dst_mask->data() : nullptr, 0, nullptr) == SST_OK;
  }

  /* current_remap() (c_frame_registration.h:308): width x height x 2 floats */
  const std::vector<float> & current_remap() const { return _remap; }
  const image_transform & image_transform_ref() const { return _transform; }
  const c_image_registration_status & status() const { return _status; }
  sst_frame_registration * handle() const { return _h; }

private:
  bool create()
  {
    if( _h ) sst_frame_registration_destroy(_h), _h = nullptr;
    sst_image_registration_options o;
    sst_image_registration_options_default(&o);
    o.motion_type = _opts.motion_type;
    o.ecc_registration_channel = _opts.ecc_registration_channel;
    o.interpolation = _opts.interpolation;
    o.border_mode = _opts.border_mode;
    o.border_value = _opts.border_value;
    const c_ecc_registration_options & e = _opts.ecc;
    o.ecc.scale = e.scale, o.ecc.eps = e.eps, o.ecc.min_rho = e.min_rho;
    o.ecc.input_smooth_sigma = e.input_smooth_sigma, o.ecc.reference_smooth_sigma = e.reference_smooth_sigma;
    o.ecc.update_step_scale = e.update_step_scale, o.ecc.normalization_noise = e.normalization_noise;
    o.ecc.se_radius = e.se_radius, o.ecc.ecc_method = e.ecc_method, o.ecc.max_iterations = e.max_iterations;
    o.ecc.ecch_max_level = e.ecch_max_level, o.ecc.ecch_minimum_image_size = e.ecch_minimum_image_size;
    o.ecc.normalization_scale = e.normalization_scale;
    o.ecc.ecch_estimate_translation_first = e.ecch_estimate_translation_first;
    o.ecc.replace_planetary_disk_with_mask = e.replace_planetary_disk_with_mask;
    const c_eccflow_registration_options & f = _opts.eccflow;
    o.eccflow.update_multiplier = f.update_multiplier, o.eccflow.input_smooth_sigma = f.input_smooth_sigma;
    o.eccflow.reference_smooth_sigma = f.reference_smooth_sigma, o.eccflow.noise_level = f.noise_level;
    o.eccflow.scale_factor = f.scale_factor, o.eccflow.max_iterations = f.max_iterations;
    o.eccflow.support_scale = f.support_scale, o.eccflow.min_image_size = f.min_image_size;
    o.eccflow.max_pyramid_level = f.max_pyramid_level, o.eccflow.downscale_method = f.downscale_method;
    o.enable_feature_registration = _opts.enable_feature_registration;
    o.enable_ecc_registration = _opts.enable_ecc_registration;
    o.enable_eccflow_registration = _opts.enable_eccflow_registration;
    o.accumulate_and_compensate_turbulent_flow = _opts.accumulate_and_compensate_turbulent_flow;
    _transform = image_transform(_opts.motion_type);
    return sst_frame_registration_create(&_h, &o) == SST_OK;
  }

  c_image_registration_options _opts;
  sst_frame_registration * _h = nullptr;
  image_transform _transform;
  std::vector<float> _remap;
  c_image_registration_status _status;
  int _w = 0, _hh = 0;
};

/* c_bayer_average (c_frame_accumulation.h:222-262) on the GPU: the pattern
 * of set_bayer_pattern, the frame's transform in place of set_remap's map
 * (set_remap with a transform; clear_remap for no registration), add of raw
 * mosaic frames, compute of the B, G, R planes. */
class c_bayer_average {
public:
  c_bayer_average() = default;
  ~c_bayer_average() { if( _h ) sst_bayer_average_destroy(_h); }
  c_bayer_average(const c_bayer_average &) = delete;
  c_bayer_average & operator=(const c_bayer_average &) = delete;

  /* c_bayer_average::set_bayer_pattern (c_frame_accumulation.cc:1138-1144) */
  void set_bayer_pattern(int colorid) { _colorid = colorid; }
  int bayer_pattern() const { return _colorid; }

  /* c_bayer_average::set_remap (c_frame_accumulation.cc:1151-1159) */
  void set_remap(const image_transform & t) { _transform = t, _have_transform = true; }
  void clear_remap() { _have_transform = false; }

  /* c_bayer_average::add(src, weights) (c_frame_accumulation.cc:1175-1203)
   * for one raw frame (u16 or f32, values times `scale`) with a frame weight */
  bool add(const image_view & src, float weight = 1.f, double scale = 1.0)
  {
    if( !ensure(src.width, src.height) ) return false;
    float p[12] = { 0 };
    if( _have_transform ) _transform.fill(p);
    int32_t st = SST_FRAME_OK;
    return sst_bayer_average_add_batch(_h, src.data, src.depth, 1, src.stride, src.stride * src.height, scale, 0,
        _have_transform ? &_transform.model : nullptr, _have_transform ? p : nullptr, &st, &weight, nullptr) == SST_OK;
  }

  /* c_bayer_average::compute (c_frame_accumulation.cc:1205-1238): avg width x
   * height x 3 (B, G, R), mask u8 */
  bool compute(std::vector<float> & avg, std::vector<uint8_t> & mask) const
  {
    if( !_h ) return false;
    avg.resize((size_t) _w * _hh * 3);
    mask.resize((size_t) _w * _hh);
    return sst_bayer_average_compute(_h, avg.data(), mask.data(), nullptr, 0, nullptr) == SST_OK;
  }

  /* c_bayer_average::get_acc_counters (c_frame_accumulation.cc:1240-1250) */
  bool get_acc_counters(std::vector<float> & accw) const
  {
    if( !_h ) return false;
    accw.resize((size_t) _w * _hh * 3);
    return sst_bayer_average_compute(_h, nullptr, nullptr, accw.data(), 0, nullptr) == SST_OK;
  }

  void clear() { if( _h ) sst_bayer_average_clear(_h, nullptr); }
  int accumulated_frames() const { return _h ? sst_bayer_average_accumulated_frames(_h) : 0; }
  sst_bayer_average * handle() const { return _h; }

private:
  bool ensure(int w, int h)
  {
    if( _h && w == _w && h == _hh ) return true;
    if( _h ) return false;
    if( sst_bayer_average_create(&_h, w, h, _colorid) != SST_OK ) return false;
    _w = w, _hh = h;
    return true;
  }
  sst_bayer_average * _h = nullptr;
  int _colorid = SST_COLORID_BAYER_RGGB;
  image_transform _transform;
  bool _have_transform = false;
  int _w = 0, _hh = 0;
};

/* linear_interpolation_inpaint(image, mask) (core/proc/inpaint/
 * linear_interpolation_inpaint.cc) on the GPU: a host FP32 image of
 * `channels` interleaved channels (packed rows), in place */
inline bool linear_interpolation_inpaint(std::vector<float> & image, const std::vector<uint8_t> & mask, int width,
    int height, int channels = 1)
{
  if( image.size() != (size_t) width * height * channels || mask.size() != (size_t) width * height ) return false;
  return sst_linear_interpolation_inpaint(image.data(), 0, width, height, channels, mask.data(), 0, 0, nullptr) == SST_OK;
}

/* c_lpg_options (c_lpg_sharpness_measure.h:22-28) */
struct c_lpg_options {
  double k = 2;
  double p = 2;
  int dscale = 2;
  int uscale = 6;
};

/* c_lpg_sharpness_measure (c_lpg_sharpness_measure.h:44-80): lpg() maps and
 * the sharpness metric of a host image */
class c_lpg_sharpness_measure {
public:
  explicit c_lpg_sharpness_measure(const c_lpg_options & o = c_lpg_options())
  {
    const sst_lpg_options so = { o.k, o.p, o.dscale, o.uscale };
    if( sst_lpg_create(&_h, &so) != SST_OK ) _h = nullptr;
  }
  ~c_lpg_sharpness_measure() { if( _h ) sst_lpg_destroy(_h); }
  c_lpg_sharpness_measure(const c_lpg_sharpness_measure &) = delete;
  c_lpg_sharpness_measure & operator=(const c_lpg_sharpness_measure &) = delete;

  /* create_sharpness_map (the map at the image's size) and the metric, the
   * map's mean over the nonzero pixels of `mask` (empty view: all pixels) */
  bool compute(const image_view & image, std::vector<float> & map, double * metric = nullptr,
      const image_view & mask = image_view())
  {
    if( !_h || image.empty() ) return false;
    map.resize((size_t) image.width * image.height);
    double m = 0;
    const bool ok = sst_lpg_compute(_h, image.data, image.depth, 1, image.width, image.height, image.stride,
        image.stride * image.height, (const uint8_t *) mask.data, mask.stride, mask.stride * mask.height, 0,
        map.data(), &m, nullptr) == SST_OK;
    if( metric ) *metric = m;
    return ok;
  }

  sst_lpg * handle() const { return _h; }

private:
  sst_lpg * _h = nullptr;
};

/* c_frame_accumulation_with_fft (c_frame_accumulation.h:168-199) */
class c_frame_accumulation_with_fft {
public:
  c_frame_accumulation_with_fft() { if( sst_fft_average_create(&_h) != SST_OK ) _h = nullptr; }
  ~c_frame_accumulation_with_fft() { if( _h ) sst_fft_average_destroy(_h); }
  c_frame_accumulation_with_fft(const c_frame_accumulation_with_fft &) = delete;
  c_frame_accumulation_with_fft & operator=(const c_frame_accumulation_with_fft &) = delete;

  /* add(src) for one host frame of `channels` interleaved channels */
  bool add(const image_view & src, int channels = 1, double scale = 1.0)
  {
    if( !_h || src.empty() ) return false;
    if( sst_fft_average_add(_h, src.data, src.depth, 1, src.width, src.height, channels, src.stride,
            src.stride * src.height, scale, 0, nullptr) != SST_OK )
      return false;
    _w = src.width, _hh = src.height, _cn = channels;
    return true;
  }

  /* compute(avg, mask): avg width x height x channels FP32, mask all 255 */
  bool compute(std::vector<float> & avg, std::vector<uint8_t> & mask) const
  {
    if( !_h ) return false;
    avg.resize((size_t) _w * _hh * _cn);
    mask.resize((size_t) _w * _hh);
    return sst_fft_average_compute(_h, avg.data(), 0, mask.data(), 0, 0, nullptr) == SST_OK;
  }

  void clear() { if( _h ) sst_fft_average_clear(_h); }
  int accumulated_frames() const { return _h ? sst_fft_average_accumulated_frames(_h) : 0; }

private:
  sst_fft_average * _h = nullptr;
  int _w = 0, _hh = 0, _cn = 1;
};

/* a cv::Rect */
struct rect {
  int x = 0, y = 0, width = 0, height = 0;
  rect() = default;
  rect(int x_, int y_, int w_, int h_) : x(x_), y(y_), width(w_), height(h_) {}
  bool empty() const { return width <= 0 || height <= 0; }
};

/* c_canvas_average (c_frame_accumulation.h:65-146) */
class c_canvas_average {
public:
  c_canvas_average() { if( sst_canvas_average_create(&_h, 0, 0) != SST_OK ) _h = nullptr; }
  ~c_canvas_average() { if( _h ) sst_canvas_average_destroy(_h); }
  c_canvas_average(const c_canvas_average &) = delete;
  c_canvas_average & operator=(const c_canvas_average &) = delete;

  void setCanvasSize(int width, int height) { if( _h ) sst_canvas_average_set_canvas_size(_h, width, height); }

  /* add(current_image, current_weights_or_mask, rmap, new_canvas_bbox): rmap
   * holds bbox.width x bbox.height x 2 floats (empty with an empty box: no
   * remap); weights: an empty view, a u8 mask or f32 weights */
  bool add(const image_view & image, const image_view & weights, const std::vector<float> & rmap,
      const rect & new_canvas_bbox, int channels = 1, double scale = 1.0)
  {
    if( !_h || image.empty() ) return false;
    if( !rmap.empty() && rmap.size() != (size_t) new_canvas_bbox.width * new_canvas_bbox.height * 2 ) return false;
    const int32_t box[4] = { new_canvas_bbox.x, new_canvas_bbox.y, new_canvas_bbox.width, new_canvas_bbox.height };
    if( sst_canvas_average_add(_h, image.data, image.depth, image.width, image.height, channels, image.stride, scale,
            weights.data, weights.depth, weights.stride, rmap.empty() ? nullptr : rmap.data(),
            new_canvas_bbox.empty() ? nullptr : box, 0, nullptr) != SST_OK )
      return false;
    _cn = channels;
    return true;
  }

  /* compute(avg, mask, dscale, -1, rbbox): the canvas or its part in rbbox */
  bool compute(std::vector<float> & avg, std::vector<uint8_t> & mask, double dscale = 1.0, const rect & rbbox = rect(),
      rect * out_box = nullptr) const
  {
    int cw = 0, ch = 0;
    if( !_h || sst_canvas_average_state(_h, &cw, &ch, nullptr, nullptr) != SST_OK ) return false;
    const int bw = rbbox.empty() ? cw : rbbox.width, bh = rbbox.empty() ? ch : rbbox.height;
    avg.resize((size_t) bw * bh * _cn);
    mask.resize((size_t) bw * bh);
    const int32_t rb[4] = { rbbox.x, rbbox.y, rbbox.width, rbbox.height };
    int32_t ob[4] = { 0, 0, 0, 0 };
    if( sst_canvas_average_compute(_h, avg.data(), (size_t) bw * _cn * sizeof(float), mask.data(), (size_t) bw,
            dscale, rbbox.empty() ? nullptr : rb, ob, 0, nullptr) != SST_OK )
      return false;
    if( out_box ) *out_box = rect(ob[0], ob[1], ob[2], ob[3]);
    return true;
  }

  rect last_bbox() const
  {
    int32_t b[4] = { 0, 0, 0, 0 };
    if( _h ) sst_canvas_average_state(_h, nullptr, nullptr, b, nullptr);
    return rect(b[0], b[1], b[2], b[3]);
  }

  int accumulated_frames() const
  {
    int n = 0;
    if( _h ) sst_canvas_average_state(_h, nullptr, nullptr, nullptr, &n);
    return n;
  }

  void clear() { if( _h ) sst_canvas_average_clear(_h); }

private:
  sst_canvas_average * _h = nullptr;
  int _cn = 1;
};

/* c_laplacian_pyramid_focus_stacking::options (c_frame_accumulation.h:
 * 158-164); fusing_policy takes c_laplacian_pyramid_focus_stacking's enum */
struct c_laplacian_pyramid_focus_stacking_options {
  int fusing_policy = SST_FOCUS_SELECT_MAX_ENERGY;
  bool inpaint_mask_holes = true;
  bool avgchannel = true;
  int kradius = 0;
  double ksigma = 0;
};

/* c_laplacian_pyramid_focus_stacking (c_frame_accumulation.h:149-191) */
class c_laplacian_pyramid_focus_stacking {
public:
  enum fusing_policy { select_max_energy = SST_FOCUS_SELECT_MAX_ENERGY, weighted_average = SST_FOCUS_WEIGHTED_AVERAGE };
  typedef c_laplacian_pyramid_focus_stacking_options options;

  explicit c_laplacian_pyramid_focus_stacking(const options & o = options())
  {
    const sst_focus_stack_options so = { (int32_t) o.fusing_policy, o.inpaint_mask_holes ? 1 : 0,
        o.avgchannel ? 1 : 0, o.kradius, o.ksigma };
    if( sst_focus_stack_create(&_h, &so) != SST_OK ) _h = nullptr;
  }
  ~c_laplacian_pyramid_focus_stacking() { if( _h ) sst_focus_stack_destroy(_h); }
  c_laplacian_pyramid_focus_stacking(const c_laplacian_pyramid_focus_stacking &) = delete;
  c_laplacian_pyramid_focus_stacking & operator=(const c_laplacian_pyramid_focus_stacking &) = delete;

  /* add(src, mask): one host frame of `channels` interleaved channels; mask an
   * empty view or a u8 mask */
  bool add(const image_view & src, const image_view & mask = image_view(), int channels = 1, double scale = 1.0)
  {
    if( !_h || src.empty() ) return false;
    if( sst_focus_stack_add(_h, src.data, src.depth, 1, src.width, src.height, channels, src.stride,
            src.stride * src.height, scale, (const uint8_t *) mask.data, mask.stride, mask.stride * mask.height, 0,
            nullptr) != SST_OK )
      return false;
    _w = src.width, _hh = src.height, _cn = channels;
    return true;
  }

  /* compute(avg): width x height x channels FP32 */
  bool compute(std::vector<float> & avg) const
  {
    if( !_h ) return false;
    avg.resize((size_t) _w * _hh * _cn);
    return sst_focus_stack_compute(_h, avg.data(), 0, 0, nullptr) == SST_OK;
  }

  void clear() { if( _h ) sst_focus_stack_clear(_h); }
  int accumulated_frames() const { return _h ? sst_focus_stack_accumulated_frames(_h) : 0; }

private:
  sst_focus_stack * _h = nullptr;
  int _w = 0, _hh = 0, _cn = 1;
};

}  // namespace sst_gb300
