/*
 * sst_registration.cu -- c_frame_registration's ECC glue on the GPU
 * (core/proc/image_registration/c_frame_registration.cc:230-250, 565-964,
 * 1265-1386; ecc2.cc:223-272, 385-397).
 *
 * sst_frame_registration owns a batched c_ecch engine (sst_ecch) and, when
 * eccflow registration is enabled, a c_eccflow engine (sst_eccflow). Per
 * batch of frames:
 *   1. create_ecc_image + scaleImage: one separable resampling pass per frame
 *      (k_resample_taps) from the raw frame (u8 / u16 / f32 times `scale`)
 *      to the f32 ECC image: pyrDown at ecc.scale 0.5, INTER_AREA otherwise;
 *   2. ecc_normalize (normalization_scale > 0 and normalization_noise > 0):
 *      pyrDown^lvl with BORDER_REPLICATE, the pyrUp chain back to the ECC
 *      size, subtraction (k_resample_taps passes, k_subtract_masked);
 *   3. the engine registers the batch: [translation, motion_type] with the
 *      0.75 min_rho gate after the translation estimate when
 *      ecch_estimate_translation_first applies, else [motion_type]; then the
 *      min_rho gate;
 *   4. scale_transfrom(1 / ecc.scale) of every frame's parameters;
 *   5. the current remap at the reference size (k_create_rmap) and, with
 *      eccflow registration, its c_eccflow refinement on the full-size frame.
 * base_remap by a dense remap is sst_remap_rmap (k_remap_rmap + erosion).
 *
 * The resampling passes gather their taps from global memory (the frame is
 * L2-resident while its CTA rows pass over it); they run once per frame and
 * are small next to the Gauss-Newton passes.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <new>
#include <string>
#include <vector>

#include "sst_engine.cuh"
#include "sst_host.h"
#include "sst_stack.cuh"
#include "sst_taps.h"
#include "sst_resample.cuh"

int sst_internal_error(int code, const char * msg);                                   // sst_capi.cu
void sst_internal_count_launches(int n);                                              // sst_capi.cu
int sst_internal_ecch_set_pass_gates(sst_ecch * h, int num, const double * gates);    // sst_capi.cu

namespace sst {

/* a = (mask && !mask[i]) ? 0 : a - b, per frame (grid.z) */
__global__ void k_subtract_masked(float * a, const float * b, size_t plane, const uint8_t * mask)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= plane ) return;
  const size_t k = (size_t) blockIdx.z * plane + i;
  a[k] = (mask && !mask[i]) ? 0.f : a[k] - b[k];
}

/* cv::pyrDown of a CV_8U mask (integer weights 1 4 6 4 1, (sum + 128) >> 8,
 * BORDER_REFLECT_101), then >= 250 -> 255 (scaleImage, c_frame_registration.cc:236-239) */
__global__ void k_mask_pyrdown_ge250(const uint8_t * src, int w, int h, size_t stride, uint8_t * dst, int dw, int dh)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= dw || y >= dh ) return;
  const int k[5] = { 1, 4, 6, 4, 1 };
  int s = 0;
  for( int j = 0; j < 5; ++j ) {
    const int yy = reflect101(2 * y + j - 2, h);
    int r = 0;
    for( int i = 0; i < 5; ++i ) r += k[i] * src[(size_t) yy * stride + reflect101(2 * x + i - 2, w)];
    s += k[j] * r;
  }
  dst[(size_t) y * dw + x] = ((s + 128) >> 8) >= 250 ? 255 : 0;
}

/* cvRound(v) >= 250 -> 255 (an INTER_AREA-resized CV_8U mask, then compare) */
__global__ void k_threshold_ge250(const float * v, size_t n, uint8_t * dst)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= n ) return;
  dst[i] = __float2int_rn(v[i]) >= 250 ? 255 : 0;
}

/* create_remap at the reference size: rmap(x, y) = W(x, y; p_f), grid.z = frame */
template<int FAM>
__global__ void k_create_rmap(const float * coeffs, int w, int h, float2 * rmap)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= w ) return;
  const float * c = coeffs + (size_t) blockIdx.z * SST_NCOEF;
  float dx, dy;
  warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
  rmap[(size_t) blockIdx.z * w * h + (size_t) y * w + x] =
      make_float2((float) (x + (int) c[12]) + dx, (float) (y + (int) c[13]) + dy);
}

template<typename T>
__device__ __forceinline__ float tap_border(const uint8_t * fb, size_t rs, int sw, int sh, int xi, int yi, int border,
    float bval)
{
  if( xi >= 0 && xi < sw && yi >= 0 && yi < sh ) return ldpx_rs<T>(fb, rs, xi, yi);
  switch ( border ) {
  case SST_BORDER_REPLICATE: return ldpx_rs<T>(fb, rs, clampi(xi, 0, sw - 1), clampi(yi, 0, sh - 1));
  case SST_BORDER_REFLECT101: return ldpx_rs<T>(fb, rs, reflect101(xi, sw), reflect101(yi, sh));
  case SST_BORDER_REFLECT: return ldpx_rs<T>(fb, rs, reflect(xi, sw), reflect(yi, sh));
  default: return bval;
  }
}

/* base_remap by a dense map (c_frame_registration.cc:1265-1340): the image
 * LINEAR with the border mode (bval for BORDER_CONSTANT, in output units),
 * the mask (src_mask, or all 255) LINEAR / BORDER_CONSTANT 0 compared
 * >= 255 into raw_mask (eroded afterwards) */
template<typename T>
__global__ void __launch_bounds__(256) k_remap_rmap(const uint8_t * src, int sw, int sh, size_t rs, float vscale,
    const float2 * rmap, int dw, int dh, int border, float bval, const uint8_t * smask, size_t mstride, float * dst,
    uint8_t * raw_mask)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= dw || y >= dh ) return;
  const size_t i = (size_t) y * dw + x;
  const float2 m = rmap[i];
  const float X = fminf(fmaxf(m.x, -1e8f), 1e8f), Y = fminf(fmaxf(m.y, -1e8f), 1e8f);
  const float fx0 = floorf(X), fy0 = floorf(Y);
  const int x0 = (int) fx0, y0 = (int) fy0;
  const float fx = X - fx0, fy = Y - fy0;
  if( dst ) {
    const float b = vscale != 0.f ? bval / vscale : 0.f;
    const float v00 = tap_border<T>(src, rs, sw, sh, x0, y0, border, b);
    const float v01 = tap_border<T>(src, rs, sw, sh, x0 + 1, y0, border, b);
    const float v10 = tap_border<T>(src, rs, sw, sh, x0, y0 + 1, border, b);
    const float v11 = tap_border<T>(src, rs, sw, sh, x0 + 1, y0 + 1, border, b);
    const float t0 = fmaf(fx, v01 - v00, v00), t1 = fmaf(fx, v11 - v10, v10);
    dst[i] = fmaf(fy, t1 - t0, t0) * vscale;
  }
  if( raw_mask ) {
    float v = 0.f;
    const float wts[4] = { (1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy };
    const int xs[4] = { x0, x0 + 1, x0, x0 + 1 }, ys[4] = { y0, y0, y0 + 1, y0 + 1 };
#pragma unroll
    for( int q = 0; q < 4; ++q ) {
      if( xs[q] >= 0 && xs[q] < sw && ys[q] >= 0 && ys[q] < sh ) {
        const float mv = smask ? (float) __ldg(smask + (size_t) ys[q] * mstride + xs[q]) : 255.f;
        v = fmaf(wts[q], mv, v);
      }
    }
    raw_mask[i] = v + 0.5f >= 255.f ? 255 : 0;
  }
}

}  // namespace sst

using namespace sst;

/* ------------------------------------------------------------- host side */

namespace {

#define SST_RCK(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if( e_ != cudaSuccess ) return fail(SST_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while ( 0 )

#define SST_RTRY(expr)                                                                \
  do {                                                                                \
    int r_ = (expr);                                                                  \
    if( r_ != SST_OK ) return r_;                                                     \
  } while ( 0 )

int fail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

bool is_half(double scale)
{
  return fabs(scale - 0.5) < 1e-2;
}

}  // namespace

extern "C" void sst_image_registration_options_default(sst_image_registration_options * o)
{
  if( !o ) return;
  memset(o, 0, sizeof(*o));
  o->motion_type = SST_MOTION_AFFINE;
  o->ecc_registration_channel = SST_COLOR_CHANNEL_GRAY;
  o->interpolation = 1;
  o->border_mode = SST_BORDER_REFLECT101;
  o->border_value = 0;
  sst_ecc_registration_options & e = o->ecc;
  e.scale = 0.5;
  e.eps = 0.2;
  e.min_rho = 0.8;
  e.input_smooth_sigma = 1.0;
  e.reference_smooth_sigma = 1.0;
  e.update_step_scale = 1.5;
  e.normalization_noise = 0.01;
  e.se_radius = 5;
  e.ecc_method = SST_ECC_LM;
  e.max_iterations = 50;
  e.ecch_max_level = 0;
  e.ecch_minimum_image_size = 16;
  e.normalization_scale = 0;
  e.ecch_estimate_translation_first = 1;
  e.replace_planetary_disk_with_mask = 0;
  sst_eccflow_registration_options & f = o->eccflow;
  f.update_multiplier = 1.5;
  f.input_smooth_sigma = 0;
  f.reference_smooth_sigma = 0;
  f.noise_level = -1;
  f.scale_factor = 0.75;
  f.max_iterations = 3;
  f.support_scale = 4;
  f.min_image_size = -1;
  f.max_pyramid_level = -1;
  f.downscale_method = SST_ECCFLOW_DOWNSCALE_RECURSIVE_RESIZE;
  o->enable_feature_registration = 1;
  o->enable_ecc_registration = 0;
  o->enable_eccflow_registration = 0;
  o->accumulate_and_compensate_turbulent_flow = 0;
}

struct sst_frame_registration {
  sst_image_registration_options o;
  sst_ecch * ecch = nullptr;
  sst_eccflow * flow = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_user = nullptr, ev_done = nullptr;
  int w = 0, h = 0;          // reference (frame) size
  int ew = 0, eh = 0;        // ECC image size
  bool scaled = false, normalized = false;
  int chunk = 256;
  std::vector<int> nw, nh;   // normalization pyramid sizes (level 0 = ECC size)
  Resampler scale_rs;                         // frame -> ECC image
  std::vector<Resampler> down_rs, up_rs;      // normalization: down l -> l + 1, up l + 1 -> l
  DevBuf ref_src, ref_ecc, ref_mask_in, ref_mask_ecc, mask_tmp;
  DevBuf stage, eframes, nbuf[2], up_buf;
  DevBuf d_params, d_status, d_rho, d_iters, coeffs, rmaps;
  std::vector<float> h_params;
  std::vector<int32_t> h_status, h_iters;
  std::vector<float> h_rho;
  int last_n = 0;
  sst_motion_model passes[2];
  int num_passes = 1;

  ~sst_frame_registration()
  {
    scale_rs.release();
    for( auto & r : down_rs ) r.release();
    for( auto & r : up_rs ) r.release();
    DevBuf * bufs[] = { &ref_src, &ref_ecc, &ref_mask_in, &ref_mask_ecc, &mask_tmp, &stage, &eframes, &nbuf[0], &nbuf[1],
        &up_buf, &d_params, &d_status, &d_rho, &d_iters, &coeffs, &rmaps };
    for( DevBuf * b : bufs ) b->release();
    if( ecch ) sst_ecch_destroy(ecch);
    if( flow ) sst_eccflow_destroy(flow);
    if( ev_user ) cudaEventDestroy(ev_user);
    if( ev_done ) cudaEventDestroy(ev_done);
    if( st ) cudaStreamDestroy(st);
  }
};

extern "C" int sst_frame_registration_create(sst_frame_registration ** out, const sst_image_registration_options * opts)
{
  if( !out ) return fail(SST_ERR_INVALID_ARG, "sst_frame_registration_create: out is NULL");
  *out = nullptr;
  sst_image_registration_options o;
  if( opts ) o = *opts;
  else sst_image_registration_options_default(&o);
  if( o.enable_feature_registration )
    return fail(SST_ERR_UNSUPPORTED, "feature registration is not on the GPU path: set enable_feature_registration = 0");
  if( o.accumulate_and_compensate_turbulent_flow )
    return fail(SST_ERR_UNSUPPORTED, "accumulate_and_compensate_turbulent_flow is not supported");
  if( o.ecc.replace_planetary_disk_with_mask )
    return fail(SST_ERR_UNSUPPORTED, "replace_planetary_disk_with_mask is not supported");
  if( o.interpolation != 1 ) return fail(SST_ERR_UNSUPPORTED, "only ECC_INTER_LINEAR interpolation is implemented");
  if( o.border_mode != SST_BORDER_CONSTANT && o.border_mode != SST_BORDER_REPLICATE &&
      o.border_mode != SST_BORDER_REFLECT && o.border_mode != SST_BORDER_REFLECT101 )
    return fail(SST_ERR_UNSUPPORTED, "unsupported border mode");
  if( o.motion_type < 0 || o.motion_type > 7 ) return fail(SST_ERR_INVALID_ARG, "invalid motion type");
  if( !o.enable_ecc_registration && !o.enable_eccflow_registration )
    return fail(SST_ERR_INVALID_ARG, "neither ECC nor eccflow registration is enabled");
  sst_frame_registration * h = new (std::nothrow) sst_frame_registration();
  if( !h ) return fail(SST_ERR_NOMEM, "out of host memory");
  h->o = o;
  if( o.enable_ecc_registration ) {
    sst_ecch_options eo;
    sst_ecch_options_default(&eo);
    eo.epsx = o.ecc.eps;
    eo.reference_smooth_sigma = o.ecc.reference_smooth_sigma;
    eo.input_smooth_sigma = o.ecc.input_smooth_sigma;
    eo.update_step_scale = o.ecc.update_step_scale;
    eo.method = o.ecc.ecc_method;
    eo.interpolation = 1;
    eo.max_iterations = o.ecc.max_iterations;
    eo.minimum_image_size = o.ecc.ecch_minimum_image_size;
    eo.maxlevel = o.ecc.ecch_max_level;
    eo.min_rho = o.ecc.min_rho;
    int r = sst_ecch_create(&h->ecch, &eo);
    if( r != SST_OK ) {
      delete h;
      return r;
    }
    sst_motion_model m = { o.motion_type, 0, 0, o.motion_type == SST_MOTION_EUCLIDEAN ? 1 : 0 };
    const bool tfirst = o.motion_type != SST_MOTION_TRANSLATION && o.ecc.ecch_estimate_translation_first &&
        o.ecc.ecch_max_level != 0;
    if( tfirst ) {
      h->passes[0] = { SST_MOTION_TRANSLATION, 0, 0, 0 };
      h->passes[1] = m;
      h->num_passes = 2;
      const double g[1] = { 0.75 * o.ecc.min_rho };
      r = sst_internal_ecch_set_pass_gates(h->ecch, 1, g);
    }
    else {
      h->passes[0] = m;
      h->num_passes = 1;
      r = sst_internal_ecch_set_pass_gates(h->ecch, 0, nullptr);
    }
    if( r != SST_OK ) {
      delete h;
      return r;
    }
  }
  if( o.enable_eccflow_registration ) {
    sst_eccflow_options fo;
    sst_eccflow_options_default(&fo);
    fo.update_multiplier = o.eccflow.update_multiplier;
    fo.scale_factor = o.eccflow.scale_factor;
    fo.noise_level = o.eccflow.noise_level;
    fo.input_smooth_sigma = o.eccflow.input_smooth_sigma;
    fo.reference_smooth_sigma = o.eccflow.reference_smooth_sigma;
    fo.max_iterations = o.eccflow.max_iterations;
    fo.support_scale = o.eccflow.support_scale;
    fo.min_image_size = o.eccflow.min_image_size;
    fo.max_pyramid_level = o.eccflow.max_pyramid_level;
    fo.downscale = o.eccflow.downscale_method;
    const int r = sst_eccflow_create(&h->flow, &fo);
    if( r != SST_OK ) {
      delete h;
      return r;
    }
  }
  *out = h;
  return SST_OK;
}

extern "C" int sst_frame_registration_destroy(sst_frame_registration * h)
{
  delete h;
  return SST_OK;
}

static int ensure_stream(sst_frame_registration * h)
{
  if( h->st ) return SST_OK;
  SST_RCK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  SST_RCK(cudaEventCreateWithFlags(&h->ev_user, cudaEventDisableTiming));
  SST_RCK(cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming));
  return SST_OK;
}

/* the ECC images of n frames into h->eframes (n x ew x eh f32): scaleImage,
 * then ecc_normalize; `mask` (ECC size) zeroes the normalized image */
static int make_ecc_images(sst_frame_registration * h, const void * d_frames, int depth, int n, size_t row_stride,
    size_t frame_stride, double scale, const uint8_t * mask)
{
  cudaStream_t st = h->st;
  const size_t eplane = (size_t) h->ew * h->eh;
  SST_RCK(h->eframes.ensure((size_t) n * eplane * sizeof(float)));
  float * e = h->eframes.as<float>();
  SST_RCK(h->scale_rs.run(d_frames, depth, row_stride, frame_stride, n, scale, e, eplane, st));
  if( !h->normalized ) return SST_OK;
  // ecc_downscale (pyrDown^lvl, REPLICATE) into nbuf ping-pong, then ecc_upscale
  const int L = (int) h->nw.size() - 1;
  size_t cap = 0;
  for( int l = 1; l <= L; ++l ) cap = std::max(cap, (size_t) h->nw[l] * h->nh[l]);
  SST_RCK(h->nbuf[0].ensure((size_t) n * cap * sizeof(float)));
  SST_RCK(h->nbuf[1].ensure((size_t) n * cap * sizeof(float)));
  SST_RCK(h->up_buf.ensure((size_t) n * eplane * sizeof(float)));
  const float * src = e;
  size_t src_row = (size_t) h->ew * sizeof(float), src_frame = eplane * sizeof(float);
  int cur = 0;
  for( int l = 0; l < L; ++l ) {
    float * d = h->nbuf[cur].as<float>();
    const size_t dplane = (size_t) h->nw[l + 1] * h->nh[l + 1];
    SST_RCK(h->down_rs[l].run(src, SST_DEPTH_F32, src_row, src_frame, n, 1.0, d, dplane, st));
    src = d;
    src_row = (size_t) h->nw[l + 1] * sizeof(float), src_frame = dplane * sizeof(float);
    cur ^= 1;
  }
  for( int l = L - 1; l >= 0; --l ) {
    float * d = l == 0 ? h->up_buf.as<float>() : h->nbuf[cur].as<float>();
    const size_t dplane = (size_t) h->nw[l] * h->nh[l];
    SST_RCK(h->up_rs[l].run(src, SST_DEPTH_F32, src_row, src_frame, n, 1.0, d, dplane, st));
    src = d;
    src_row = (size_t) h->nw[l] * sizeof(float), src_frame = dplane * sizeof(float);
    cur ^= 1;
  }
  dim3 grid((unsigned) ((eplane + 255) / 256), 1, n);
  k_subtract_masked<<<grid, 256, 0, st>>>(e, h->up_buf.as<float>(), eplane, mask);
  sst_internal_count_launches(1);
  SST_RCK(cudaGetLastError());
  return SST_OK;
}

extern "C" int sst_frame_registration_setup_reference_frame(sst_frame_registration * h, const void * image, int depth,
    int width, int height, size_t row_stride, double scale, const uint8_t * mask, size_t mask_stride, int on_device,
    void * stream)
{
  if( !h || !image ) return fail(SST_ERR_INVALID_ARG, "setup_reference_frame: NULL argument");
  if( depth_bytes(depth) == 0 ) return fail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( width < 8 || height < 8 ) return fail(SST_ERR_INVALID_ARG, "reference image too small");
  if( row_stride < (size_t) width * depth_bytes(depth) ) return fail(SST_ERR_INVALID_ARG, "row_stride too small");
  if( mask && mask_stride < (size_t) width ) return fail(SST_ERR_INVALID_ARG, "mask_stride too small");
  SST_RTRY(ensure_stream(h));
  SST_RCK(cudaEventRecord(h->ev_user, (cudaStream_t) stream));
  SST_RCK(cudaStreamWaitEvent(h->st, h->ev_user, 0));
  cudaStream_t st = h->st;
  h->w = width, h->h = height;
  const void * src = image;
  if( !on_device ) {
    SST_RCK(h->ref_src.ensure(row_stride * height));
    SST_RCK(cudaMemcpyAsync(h->ref_src.p, image, row_stride * height, cudaMemcpyHostToDevice, st));
    src = h->ref_src.p;
  }
  const uint8_t * dmask = mask;
  if( mask && !on_device ) {
    SST_RCK(h->ref_mask_in.ensure(mask_stride * height));
    SST_RCK(cudaMemcpyAsync(h->ref_mask_in.p, mask, mask_stride * height, cudaMemcpyHostToDevice, st));
    dmask = h->ref_mask_in.as<uint8_t>();
  }
  if( h->ecch ) {
    // scaleImage (c_frame_registration.cc:230-250) sizes and tables
    const double s = h->o.ecc.scale;
    h->scaled = s > 0 && s != 1;
    if( !h->scaled ) h->ew = width, h->eh = height;
    else if( is_half(s) ) h->ew = (width + 1) / 2, h->eh = (height + 1) / 2;
    else h->ew = (int) nearbyint(width * s), h->eh = (int) nearbyint(height * s);
    if( h->ew < 4 || h->eh < 4 ) return fail(SST_ERR_INVALID_ARG, "the scaled ECC image is smaller than 4 x 4");
    if( !h->scaled ) SST_RCK(h->scale_rs.upload(copy_taps(width), copy_taps(height), width, height, width, height, st));
    else if( is_half(s) ) {
      SST_RCK(h->scale_rs.upload(pyr_taps(width, h->ew), pyr_taps(height, h->eh), width, height, h->ew, h->eh, st));
    }
    else {
      SST_RCK(h->scale_rs.upload(area_taps(width, h->ew), area_taps(height, h->eh), width, height, h->ew, h->eh, st));
    }
    // ecc_normalize sizes and tables (ecc2.cc:223-272, 385-397)
    h->normalized = h->o.ecc.normalization_scale > 0 && h->o.ecc.normalization_noise > 0;
    h->nw.assign(1, h->ew), h->nh.assign(1, h->eh);
    for( auto & r : h->down_rs ) r.release();
    for( auto & r : h->up_rs ) r.release();
    h->down_rs.clear(), h->up_rs.clear();
    if( h->normalized ) {
      const int L = std::min(h->o.ecc.normalization_scale, 30);
      for( int l = 0; l < L; ++l ) h->nw.push_back((h->nw.back() + 1) / 2), h->nh.push_back((h->nh.back() + 1) / 2);
      h->down_rs.resize(L), h->up_rs.resize(L);
      for( int l = 0; l < L; ++l ) {
        SST_RCK(h->down_rs[l].upload(pyr_taps(h->nw[l], h->nw[l + 1], true), pyr_taps(h->nh[l], h->nh[l + 1], true),
            h->nw[l], h->nh[l], h->nw[l + 1], h->nh[l + 1], st));
        SST_RCK(h->up_rs[l].upload(pyrup_taps(h->nw[l + 1], h->nw[l]), pyrup_taps(h->nh[l + 1], h->nh[l]),
            h->nw[l + 1], h->nh[l + 1], h->nw[l], h->nh[l], st));
      }
    }
    // the reference ECC mask
    const uint8_t * emask = nullptr;
    if( dmask ) {
      SST_RCK(h->ref_mask_ecc.ensure((size_t) h->ew * h->eh));
      uint8_t * em = h->ref_mask_ecc.as<uint8_t>();
      if( !h->scaled ) {
        SST_RCK(cudaMemcpy2DAsync(em, width, dmask, mask_stride, width, height, cudaMemcpyDeviceToDevice, st));
      }
      else if( is_half(s) ) {
        k_mask_pyrdown_ge250<<<dim3((h->ew + 127) / 128, h->eh), 128, 0, st>>>(dmask, width, height, mask_stride, em,
            h->ew, h->eh);
        sst_internal_count_launches(1);
        SST_RCK(cudaGetLastError());
      }
      else {
        SST_RCK(h->mask_tmp.ensure((size_t) h->ew * h->eh * sizeof(float)));
        SST_RCK(h->scale_rs.run(dmask, SST_DEPTH_U8, mask_stride, mask_stride * height, 1, 1.0, h->mask_tmp.as<float>(),
            (size_t) h->ew * h->eh, st));
        const size_t np = (size_t) h->ew * h->eh;
        k_threshold_ge250<<<(unsigned) ((np + 255) / 256), 256, 0, st>>>(h->mask_tmp.as<float>(), np, em);
        sst_internal_count_launches(1);
        SST_RCK(cudaGetLastError());
      }
      emask = em;
    }
    SST_RTRY(make_ecc_images(h, src, depth, 1, row_stride, row_stride * height, scale, emask));
    SST_RCK(h->ref_ecc.ensure((size_t) h->ew * h->eh * sizeof(float)));
    SST_RCK(cudaMemcpyAsync(h->ref_ecc.p, h->eframes.p, (size_t) h->ew * h->eh * sizeof(float), cudaMemcpyDeviceToDevice,
        st));
    SST_RTRY(sst_ecch_set_reference_image(h->ecch, h->ref_ecc.p, SST_DEPTH_F32, h->ew, h->eh, (size_t) h->ew * sizeof(float),
        1.0, emask, emask ? (size_t) h->ew : 0, 1, h->st));
  }
  if( h->flow ) {
    // the eccflow reference: the full-size image and mask (c_frame_registration.cc:680-687)
    SST_RTRY(sst_eccflow_set_reference_image_masked(h->flow, src, depth, width, height, row_stride, scale, dmask,
        mask_stride, 1, h->st));
  }
  SST_RCK(cudaStreamSynchronize(st));
  SST_RCK(cudaEventRecord(h->ev_done, st));
  SST_RCK(cudaStreamWaitEvent((cudaStream_t) stream, h->ev_done, 0));
  return SST_OK;
}

extern "C" int sst_frame_registration_set_chunk_frames(sst_frame_registration * h, int frames)
{
  if( !h || frames < 1 ) return fail(SST_ERR_INVALID_ARG, "invalid chunk size");
  h->chunk = frames;
  return SST_OK;
}

static int copy_to(void * dst, const void * src, size_t bytes, int on_device, cudaStream_t st)
{
  if( !dst ) return SST_OK;
  SST_RCK(cudaMemcpyAsync(dst, src, bytes, on_device ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost, st));
  return SST_OK;
}

extern "C" int sst_frame_registration_register_frames(sst_frame_registration * h, const void * frames, int depth,
    int n, int width, int height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    float * params_out, int32_t * status_out, float * rho_out, int32_t * iterations_out, float * rmap_out, void * stream)
{
  if( !h || !frames ) return fail(SST_ERR_INVALID_ARG, "register_frames: NULL argument");
  if( h->w == 0 ) return fail(SST_ERR_STATE, "setup_reference_frame was not called");
  if( n < 1 || n > 65535 ) return fail(SST_ERR_INVALID_ARG, "n out of range 1..65535");
  if( width != h->w || height != h->h ) return fail(SST_ERR_INVALID_ARG, "frame size differs from the reference");
  if( depth_bytes(depth) == 0 ) return fail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( row_stride < (size_t) width * depth_bytes(depth) || frame_stride < row_stride * height )
    return fail(SST_ERR_INVALID_ARG, "invalid strides");
  SST_RTRY(ensure_stream(h));
  SST_RCK(cudaEventRecord(h->ev_user, (cudaStream_t) stream));
  SST_RCK(cudaStreamWaitEvent(h->st, h->ev_user, 0));
  cudaStream_t st = h->st;
  const sst_motion_model m = { h->o.motion_type, 0, 0, h->o.motion_type == SST_MOTION_EUCLIDEAN ? 1 : 0 };
  const int M = model_nparams(m);
  const size_t plane = (size_t) width * height;
  const int chunk = std::max(1, std::min(h->chunk, n));
  SST_RCK(h->d_params.ensure((size_t) chunk * 12 * sizeof(float)));
  SST_RCK(h->d_status.ensure((size_t) chunk * sizeof(int32_t)));
  SST_RCK(h->d_rho.ensure((size_t) chunk * sizeof(float)));
  SST_RCK(h->d_iters.ensure((size_t) chunk * sizeof(int32_t)));
  SST_RCK(h->coeffs.ensure((size_t) chunk * SST_NCOEF * sizeof(float)));
  const bool want_rmap = rmap_out || h->flow;
  if( want_rmap ) SST_RCK(h->rmaps.ensure((size_t) chunk * plane * 2 * sizeof(float)));
  h->h_params.assign((size_t) chunk * 12, 0.f);
  h->h_status.assign(chunk, 0);
  h->h_rho.assign(chunk, 0.f);
  h->h_iters.assign(chunk, 0);
  for( int f0 = 0; f0 < n; f0 += chunk ) {
    const int nc = std::min(chunk, n - f0);
    const uint8_t * fsrc = (const uint8_t *) frames + (size_t) f0 * frame_stride;
    const void * d_frames = fsrc;
    if( !on_device ) {
      SST_RCK(h->stage.ensure(frame_stride * nc));
      SST_RCK(cudaMemcpyAsync(h->stage.p, fsrc, frame_stride * nc, cudaMemcpyHostToDevice, st));
      d_frames = h->stage.p;
    }
    if( h->ecch ) {
      SST_RTRY(make_ecc_images(h, d_frames, depth, nc, row_stride, frame_stride, scale, nullptr));
      SST_RTRY(sst_ecch_align_batch(h->ecch, h->eframes.p, SST_DEPTH_F32, nc, h->ew, h->eh, (size_t) h->ew * sizeof(float),
          (size_t) h->ew * h->eh * sizeof(float), 1.0, 1, h->num_passes, h->passes, 0, h->d_params.as<float>(),
          h->d_status.as<int32_t>(), h->d_iters.as<int32_t>(), nullptr, h->d_rho.as<float>(), nullptr, st));
      SST_RCK(cudaMemcpyAsync(h->h_params.data(), h->d_params.p, (size_t) nc * 12 * sizeof(float), cudaMemcpyDeviceToHost, st));
      SST_RCK(cudaMemcpyAsync(h->h_status.data(), h->d_status.p, (size_t) nc * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      SST_RCK(cudaMemcpyAsync(h->h_rho.data(), h->d_rho.p, (size_t) nc * sizeof(float), cudaMemcpyDeviceToHost, st));
      SST_RCK(cudaMemcpyAsync(h->h_iters.data(), h->d_iters.p, (size_t) nc * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      SST_RCK(cudaStreamSynchronize(st));
      // scale_transfrom(1 / scale) (c_frame_registration.cc:877-879)
      for( int f = 0; f < nc; ++f ) {
        double s[16], p[12];
        model_identity(m, s);
        for( int j = 0; j < M; ++j ) p[j] = h->h_params[(size_t) f * 12 + j];
        model_set_params(m, s, p);
        if( h->scaled ) model_scale(m, s, 1.0 / h->o.ecc.scale);
        model_get_params(m, s, p);
        for( int j = 0; j < 12; ++j ) h->h_params[(size_t) f * 12 + j] = j < M ? (float) p[j] : 0.f;
      }
    }
    else {
      // eccflow alone starts from the identity transform (c_frame_registration.cc:745)
      for( int f = 0; f < nc; ++f ) {
        double s[16], p[12];
        model_identity(m, s);
        model_get_params(m, s, p);
        for( int j = 0; j < 12; ++j ) h->h_params[(size_t) f * 12 + j] = j < M ? (float) p[j] : 0.f;
        h->h_status[f] = SST_FRAME_OK, h->h_rho[f] = 0.f, h->h_iters[f] = 0;
      }
    }
    if( want_rmap ) {
      SST_RCK(cudaMemcpyAsync(h->d_params.p, h->h_params.data(), (size_t) nc * 12 * sizeof(float), cudaMemcpyHostToDevice, st));
      SST_RCK(launch_coeffs_from_params(m, h->d_params.as<float>(), nc, h->coeffs.as<float>(), st));
      dim3 grid((width + 127) / 128, height, nc);
      float2 * rm = h->rmaps.as<float2>();
      switch ( motion_family(m.type) ) {
      case FAM_HOMOG: k_create_rmap<FAM_HOMOG><<<grid, 128, 0, st>>>(h->coeffs.as<float>(), width, height, rm); break;
      case FAM_QUAD: k_create_rmap<FAM_QUAD><<<grid, 128, 0, st>>>(h->coeffs.as<float>(), width, height, rm); break;
      default: k_create_rmap<FAM_AFFINE><<<grid, 128, 0, st>>>(h->coeffs.as<float>(), width, height, rm); break;
      }
      sst_internal_count_launches(2);
      SST_RCK(cudaGetLastError());
      if( h->flow ) {
        // c_eccflow::compute(ecc_image, current_remap) (c_frame_registration.cc:915-920), in place
        SST_RTRY(sst_eccflow_compute_batch(h->flow, d_frames, depth, nc, row_stride, frame_stride, scale, 1,
            h->rmaps.as<float>(), h->rmaps.as<float>(), st));
      }
      if( rmap_out ) {
        SST_RCK(cudaMemcpyAsync(rmap_out + (size_t) f0 * plane * 2, h->rmaps.p, (size_t) nc * plane * 2 * sizeof(float),
            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
      }
    }
    SST_RTRY(copy_to(params_out ? params_out + (size_t) f0 * 12 : nullptr, h->h_params.data(), (size_t) nc * 12 * sizeof(float),
        on_device, st));
    SST_RTRY(copy_to(status_out ? status_out + f0 : nullptr, h->h_status.data(), (size_t) nc * sizeof(int32_t), on_device, st));
    SST_RTRY(copy_to(rho_out ? rho_out + f0 : nullptr, h->h_rho.data(), (size_t) nc * sizeof(float), on_device, st));
    SST_RTRY(copy_to(iterations_out ? iterations_out + f0 : nullptr, h->h_iters.data(), (size_t) nc * sizeof(int32_t),
        on_device, st));
    SST_RCK(cudaStreamSynchronize(st));   // host result buffers are reused by the next chunk
    h->last_n = nc;
  }
  SST_RCK(cudaEventRecord(h->ev_done, st));
  SST_RCK(cudaStreamWaitEvent((cudaStream_t) stream, h->ev_done, 0));
  return SST_OK;
}

extern "C" int sst_frame_registration_ecc_size(const sst_frame_registration * h, int * width, int * height)
{
  if( !h || !h->ecch || h->w == 0 ) return fail(SST_ERR_STATE, "no ECC reference");
  if( width ) *width = h->ew;
  if( height ) *height = h->eh;
  return SST_OK;
}

extern "C" int sst_frame_registration_ecc_image(sst_frame_registration * h, int frame, float * out, uint8_t * mask_out,
    int on_device)
{
  if( !h || !h->ecch || h->w == 0 ) return fail(SST_ERR_STATE, "no ECC reference");
  if( frame < -1 || frame >= h->last_n ) return fail(SST_ERR_INVALID_ARG, "frame out of range of the last chunk");
  const size_t eplane = (size_t) h->ew * h->eh;
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if( out ) {
    const float * src = frame < 0 ? h->ref_ecc.as<float>() : h->eframes.as<float>() + (size_t) frame * eplane;
    SST_RCK(cudaMemcpyAsync(out, src, eplane * sizeof(float), k, h->st));
  }
  if( mask_out ) {
    if( frame >= 0 || !h->ref_mask_ecc.p ) return fail(SST_ERR_INVALID_ARG, "only the reference has an ECC mask");
    SST_RCK(cudaMemcpyAsync(mask_out, h->ref_mask_ecc.p, eplane, k, h->st));
  }
  SST_RCK(cudaStreamSynchronize(h->st));
  return SST_OK;
}

extern "C" int sst_remap_rmap(const void * src, int depth, int src_width, int src_height, size_t row_stride, double scale,
    const float * rmap, int dst_width, int dst_height, int border, double border_value, const uint8_t * src_mask,
    size_t mask_stride, float * dst, uint8_t * dst_mask, int on_device, void * stream)
{
  if( !src || !rmap ) return fail(SST_ERR_INVALID_ARG, "sst_remap_rmap: NULL argument");
  if( depth_bytes(depth) == 0 ) return fail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( src_width < 1 || src_height < 1 || dst_width < 1 || dst_height < 1 ) return fail(SST_ERR_INVALID_ARG, "invalid size");
  if( row_stride < (size_t) src_width * depth_bytes(depth) ) return fail(SST_ERR_INVALID_ARG, "row_stride too small");
  if( src_mask && mask_stride < (size_t) src_width ) return fail(SST_ERR_INVALID_ARG, "mask_stride too small");
  if( border != SST_BORDER_CONSTANT && border != SST_BORDER_REPLICATE && border != SST_BORDER_REFLECT &&
      border != SST_BORDER_REFLECT101 )
    return fail(SST_ERR_UNSUPPORTED, "unsupported border mode");
  cudaStream_t st = (cudaStream_t) stream;
  const size_t dplane = (size_t) dst_width * dst_height;
  ScopedBuf raw, hs, hm, hmask, hdst, hdm;
  const void * d_src = src;
  const float * d_rmap = rmap;
  const uint8_t * d_smask = src_mask;
  float * d_dst = dst;
  uint8_t * d_dmask = dst_mask;
  if( !on_device ) {
    SST_RCK(hs.ensure(row_stride * src_height));
    SST_RCK(cudaMemcpyAsync(hs.p, src, row_stride * src_height, cudaMemcpyHostToDevice, st));
    d_src = hs.p;
    SST_RCK(hm.ensure(dplane * 2 * sizeof(float)));
    SST_RCK(cudaMemcpyAsync(hm.p, rmap, dplane * 2 * sizeof(float), cudaMemcpyHostToDevice, st));
    d_rmap = hm.as<float>();
    if( src_mask ) {
      SST_RCK(hmask.ensure(mask_stride * src_height));
      SST_RCK(cudaMemcpyAsync(hmask.p, src_mask, mask_stride * src_height, cudaMemcpyHostToDevice, st));
      d_smask = hmask.as<uint8_t>();
    }
    if( dst ) {
      SST_RCK(hdst.ensure(dplane * sizeof(float)));
      d_dst = hdst.as<float>();
    }
    if( dst_mask ) {
      SST_RCK(hdm.ensure(dplane));
      d_dmask = hdm.as<uint8_t>();
    }
  }
  if( dst_mask ) SST_RCK(raw.ensure(dplane));
  dim3 grid((dst_width + 31) / 32, (dst_height + 7) / 8);
  const uint8_t * s = (const uint8_t *) d_src;
  const float2 * m = (const float2 *) d_rmap;
  uint8_t * rm = dst_mask ? raw.as<uint8_t>() : nullptr;
#define SST_RR(T) k_remap_rmap<T><<<grid, 256, 0, st>>>(s, src_width, src_height, row_stride, (float) scale, m, \
    dst_width, dst_height, border, (float) border_value, d_smask, mask_stride, d_dst, rm)
  switch ( depth ) {
  case SST_DEPTH_U8: SST_RR(uint8_t); break;
  case SST_DEPTH_U16: SST_RR(uint16_t); break;
  default: SST_RR(float); break;
  }
#undef SST_RR
  sst_internal_count_launches(1);
  SST_RCK(cudaGetLastError());
  if( dst_mask ) {
    // cv::erode 5 x 5, BORDER_CONSTANT 255 (c_frame_registration.cc:1336-1337)
    SST_RCK(launch_erode5(rm, dst_width, dst_height, d_dmask, st));
    sst_internal_count_launches(1);
  }
  if( !on_device ) {
    if( dst ) SST_RCK(cudaMemcpyAsync(dst, d_dst, dplane * sizeof(float), cudaMemcpyDeviceToHost, st));
    if( dst_mask ) SST_RCK(cudaMemcpyAsync(dst_mask, d_dmask, dplane, cudaMemcpyDeviceToHost, st));
  }
  SST_RCK(cudaStreamSynchronize(st));   // the temporary buffers are released on return
  return SST_OK;
}

/* ------------------------------------------------ c_image_transform utilities */

extern "C" int sst_image_transform_scale(const sst_motion_model * model, float * params, double factor)
{
  if( !model || !params ) return fail(SST_ERR_INVALID_ARG, "NULL argument");
  if( model->type < 0 || model->type > 7 ) return fail(SST_ERR_INVALID_ARG, "invalid motion type");
  const int M = model_nparams(*model);
  double s[16], p[12];
  model_identity(*model, s);
  for( int j = 0; j < M; ++j ) p[j] = params[j];
  model_set_params(*model, s, p);
  model_scale(*model, s, factor);
  model_get_params(*model, s, p);
  for( int j = 0; j < M; ++j ) params[j] = (float) p[j];
  return SST_OK;
}

extern "C" int sst_image_transform_create_remap(const sst_motion_model * model, const float * params, int width,
    int height, float * rmap, int on_device, void * stream)
{
  if( !model || !params || !rmap ) return fail(SST_ERR_INVALID_ARG, "NULL argument");
  if( model->type < 0 || model->type > 7 ) return fail(SST_ERR_INVALID_ARG, "invalid motion type");
  if( width < 1 || height < 1 ) return fail(SST_ERR_INVALID_ARG, "invalid size");
  cudaStream_t st = (cudaStream_t) stream;
  ScopedBuf dp, dc, dm;
  SST_RCK(dp.ensure(12 * sizeof(float)));
  SST_RCK(dc.ensure(SST_NCOEF * sizeof(float)));
  SST_RCK(cudaMemcpyAsync(dp.p, params, model_nparams(*model) * sizeof(float),
      on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  SST_RCK(launch_coeffs_from_params(*model, dp.as<float>(), 1, dc.as<float>(), st));
  float2 * out = (float2 *) rmap;
  const size_t bytes = (size_t) width * height * sizeof(float2);
  if( !on_device ) {
    SST_RCK(dm.ensure(bytes));
    out = dm.as<float2>();
  }
  dim3 grid((width + 127) / 128, height, 1);
  switch ( motion_family(model->type) ) {
  case FAM_HOMOG: k_create_rmap<FAM_HOMOG><<<grid, 128, 0, st>>>(dc.as<float>(), width, height, out); break;
  case FAM_QUAD: k_create_rmap<FAM_QUAD><<<grid, 128, 0, st>>>(dc.as<float>(), width, height, out); break;
  default: k_create_rmap<FAM_AFFINE><<<grid, 128, 0, st>>>(dc.as<float>(), width, height, out); break;
  }
  sst_internal_count_launches(2);
  SST_RCK(cudaGetLastError());
  if( !on_device ) SST_RCK(cudaMemcpyAsync(rmap, out, bytes, cudaMemcpyDeviceToHost, st));
  SST_RCK(cudaStreamSynchronize(st));
  return SST_OK;
}
