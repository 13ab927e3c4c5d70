/*
 * sst_calib.cu -- the dark / flat calibration read_input_frame applies to
 * every raw frame before registration (read_input_frame,
 * c_image_stacking_pipeline_base.cc:142-183; the dark branch converts with
 * 1 / 2^bpp first, the flat branch converts if the dark branch did not):
 *   x = raw * scale                      convertTo(CV_32F, 1 / 2^bpp)
 *   x = x - dark                         cv::subtract(image, darkbayer)
 *   x = x * 5 / flat                     cv::divide(image, flatbayer, image, image.depth())
 * The reference passes the image depth (CV_32F = 5) as cv::divide's scale
 * argument, so a flat-fielded frame comes out 5 times brighter; that is kept.
 * One thread per pixel, FP32 with explicitly rounded operations (no
 * contraction), so the result is the sequence of FP32 operations above.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "sst_host.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

namespace sst {
namespace cal {

template<typename T>
__global__ void __launch_bounds__(256) k_calibrate(const uint8_t * frames, int w, int h, size_t rs, size_t fs, float scale,
    const float * dark, size_t dark_rs, const float * flat, size_t flat_rs, float * out, size_t out_rs, size_t out_fs)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const T * row = (const T *) (frames + (size_t) blockIdx.z * fs + (size_t) y * rs);
  float v = __fmul_rn((float) row[x], scale);
  if( dark ) v = __fsub_rn(v, *(const float *) ((const uint8_t *) dark + (size_t) y * dark_rs + (size_t) x * 4));
  if( flat ) v = __fdiv_rn(__fmul_rn(v, 5.f), *(const float *) ((const uint8_t *) flat + (size_t) y * flat_rs + (size_t) x * 4));
  *(float *) ((uint8_t *) out + (size_t) blockIdx.z * out_fs + (size_t) y * out_rs + (size_t) x * 4) = v;
}

}  // namespace cal
}  // namespace sst

namespace {

int cfail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_CCK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return cfail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

}  // namespace

extern "C" int sst_calibrate_frames(const void * frames, int depth, int n, int width, int height, size_t row_stride,
    size_t frame_stride, double scale, const float * dark, size_t dark_stride, const float * flat, size_t flat_stride,
    float * out, size_t out_row_stride, size_t out_frame_stride, void * stream)
{
  if( !frames || !out ) return cfail(SST_ERR_INVALID_ARG, "sst_calibrate_frames: NULL argument");
  if( n < 1 || width < 1 || height < 1 ) return cfail(SST_ERR_INVALID_ARG, "n, width and height must be >= 1");
  if( n > 65535 || height > 65535 * 8 ) return cfail(SST_ERR_INVALID_ARG, "too many frames or rows for one call");
  const int db = depth_bytes(depth);
  if( db == 0 ) return cfail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( dark_stride == 0 ) dark_stride = (size_t) width * 4;
  if( flat_stride == 0 ) flat_stride = (size_t) width * 4;
  if( out_row_stride == 0 ) out_row_stride = (size_t) width * 4;
  if( out_frame_stride == 0 ) out_frame_stride = out_row_stride * height;
  if( row_stride < (size_t) width * db || (n > 1 && frame_stride < row_stride * height) ||
      (dark && dark_stride < (size_t) width * 4) || (flat && flat_stride < (size_t) width * 4) ||
      out_row_stride < (size_t) width * 4 || (n > 1 && out_frame_stride < out_row_stride * height) ||
      (dark_stride & 3) || (flat_stride & 3) || (out_row_stride & 3) || (out_frame_stride & 3) ||
      (db > 1 && ((row_stride % db) || (frame_stride % db))) )
    return cfail(SST_ERR_INVALID_ARG, "invalid or misaligned strides");
  cudaStream_t st = (cudaStream_t) stream;
  const dim3 grid((width + 31) / 32, (height + 7) / 8, n);
  const uint8_t * f = (const uint8_t *) frames;
  const float s = (float) scale;
  switch ( depth ) {
  case SST_DEPTH_U8:
    sst::cal::k_calibrate<uint8_t><<<grid, 256, 0, st>>>(f, width, height, row_stride, frame_stride, s, dark, dark_stride,
        flat, flat_stride, out, out_row_stride, out_frame_stride);
    break;
  case SST_DEPTH_U16:
    sst::cal::k_calibrate<uint16_t><<<grid, 256, 0, st>>>(f, width, height, row_stride, frame_stride, s, dark, dark_stride,
        flat, flat_stride, out, out_row_stride, out_frame_stride);
    break;
  default:
    sst::cal::k_calibrate<float><<<grid, 256, 0, st>>>(f, width, height, row_stride, frame_stride, s, dark, dark_stride,
        flat, flat_stride, out, out_row_stride, out_frame_stride);
    break;
  }
  SST_CCK(cudaGetLastError());
  sst_internal_count_launches(1);
  return SST_OK;
}
