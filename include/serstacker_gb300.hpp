/*
 * serstacker_gb300.hpp -- C++ drop-in classes for SerStacker's registration
 * and stacking hot path, over the C ABI of libsst_gb300.so.
 *
 * The class, option and method names follow the reference interfaces they
 * replace (paths relative to the SerStacker source tree):
 *   sst_gb300::c_ecch_options      core/proc/image_registration/ecc2.h:158-172
 *   sst_gb300::c_ecch              core/proc/image_registration/ecc2.h:193-308
 *   sst_gb300::c_weigthed_average  core/average/c_frame_accumulation.h:39-63
 *   sst_gb300::c_local_variance_map_options, c_local_variance_sharpness_measure
 *                                  core/proc/sharpness_measure/c_local_variance_sharpness_measure.h:17-23
 *   sst_gb300::c_ser_reader        core/io/c_ser_file.h:136-174
 *   sst_gb300::c_ser_writer        core/io/c_ser_file.h:183-213
 *   sst_gb300::average_pyramid_inpaint  core/proc/inpaint/average_pyramid_inpaint.h:14-18
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

/* The motion model and its parameter vector (c_image_transform::parameters()). */
struct image_transform {
  sst_motion_model model { SST_MOTION_AFFINE, 0, 0, 0 };
  std::vector<float> parameters;

  explicit image_transform(int motion_type = SST_MOTION_AFFINE)
  {
    model.type = motion_type;
    model.fix_scale = motion_type == SST_MOTION_EUCLIDEAN ? 1 : 0;
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
    return sst_ecch_set_reference_image(_h, img.data, img.depth, img.width, img.height, img.stride, scale,
        (const uint8_t *) mask.data, mask.stride, 0, nullptr) == SST_OK;
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

}  // namespace sst_gb300
