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
 *
 * Also read_input_frame's DEBAYER_NN2 demosaic of raw Bayer frames
 * (c_image_stacking_pipeline_base.cc:220-235, nninterpolation in
 * core/debayer.cc:828-1161) into BGR frames, one thread per pixel.
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

/* Bayer colour (0 B, 1 G, 2 R) at (x, y) of pattern colorid 8 RGGB, 9 GRBG,
 * 10 GBRG, 11 BGGR */
__device__ __forceinline__ int bayer_color(int colorid, int x, int y)
{
  const int i = (y & 1) * 2 + (x & 1);
  switch ( colorid ) {
  case 8: return i == 0 ? 2 : (i == 3 ? 0 : 1);
  case 9: return i == 1 ? 2 : (i == 2 ? 0 : 1);
  case 10: return i == 2 ? 2 : (i == 1 ? 0 : 1);
  default: return i == 3 ? 2 : (i == 0 ? 0 : 1);
  }
}

template<typename T, typename A>
__device__ __forceinline__ A nn2_at(const uint8_t * f, size_t rs, int w, int h, int x, int y)
{
  x = x < 0 ? -x : (x >= w ? 2 * (w - 1) - x : x);
  y = y < 0 ? -y : (y >= h ? 2 * (h - 1) - y : y);
  return (A) ((const T *) (f + (size_t) y * rs))[x];
}

template<typename T, typename A>
__device__ __forceinline__ T nn2_mean(A s, int n)
{
  if constexpr( sizeof(A) == 8 ) return (T) ((s + n / 2) / n);
  else return (T) __fdiv_rn(s, (float) n);
}

/* nninterpolation (core/debayer.cc:828-1161): one thread per pixel; sums in
 * A (int64 for integer frames, f32 for float ones) in the order N W E S /
 * NW NE SW SE / W E / N S */
template<typename T, typename A>
__global__ void __launch_bounds__(128) k_debayer_nn2(const uint8_t * frames, int w, int h, size_t rs, size_t fs,
    int colorid, uint8_t * dst, size_t drs, size_t dfs)
{
  const int x = blockIdx.x * 128 + threadIdx.x, y = blockIdx.y;
  if( x >= w ) return;
  const uint8_t * f = frames + (size_t) blockIdx.z * fs;
  const int own = bayer_color(colorid, x, y);
  T out[3];
#pragma unroll
  for( int ch = 0; ch < 3; ++ch ) {
    if( ch == own ) out[ch] = (T) nn2_at<T, A>(f, rs, w, h, x, y);
    else if( ch == 1 ) {
      A s = nn2_at<T, A>(f, rs, w, h, x, y - 1);
      s = s + nn2_at<T, A>(f, rs, w, h, x - 1, y);
      s = s + nn2_at<T, A>(f, rs, w, h, x + 1, y);
      s = s + nn2_at<T, A>(f, rs, w, h, x, y + 1);
      out[ch] = nn2_mean<T, A>(s, 4);
    }
    else if( own == 1 ) {
      if( bayer_color(colorid, x + 1, y) == ch )
        out[ch] = nn2_mean<T, A>(nn2_at<T, A>(f, rs, w, h, x - 1, y) + nn2_at<T, A>(f, rs, w, h, x + 1, y), 2);
      else out[ch] = nn2_mean<T, A>(nn2_at<T, A>(f, rs, w, h, x, y - 1) + nn2_at<T, A>(f, rs, w, h, x, y + 1), 2);
    }
    else {
      A s = nn2_at<T, A>(f, rs, w, h, x - 1, y - 1);
      s = s + nn2_at<T, A>(f, rs, w, h, x + 1, y - 1);
      s = s + nn2_at<T, A>(f, rs, w, h, x - 1, y + 1);
      s = s + nn2_at<T, A>(f, rs, w, h, x + 1, y + 1);
      out[ch] = nn2_mean<T, A>(s, 4);
    }
  }
  T * d = (T *) (dst + (size_t) blockIdx.z * dfs + (size_t) y * drs) + (size_t) x * 3;
  d[0] = out[0], d[1] = out[1], d[2] = out[2];
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

extern "C" int sst_debayer_nn2(const void * frames, int depth, int n, int width, int height, size_t row_stride,
    size_t frame_stride, int colorid, void * dst, size_t dst_row_stride, size_t dst_frame_stride, void * stream)
{
  if( !frames || !dst ) return cfail(SST_ERR_INVALID_ARG, "sst_debayer_nn2: NULL argument");
  if( colorid < 8 || colorid > 11 ) return cfail(SST_ERR_INVALID_ARG, "colorid must be 8 (RGGB) .. 11 (BGGR)");
  if( n < 1 || n > 65535 || width < 2 || height < 2 || height > 65535 || (width & 1) || (height & 1) )
    return cfail(SST_ERR_INVALID_ARG, "n in 1..65535, even width and height >= 2");
  const int db = depth_bytes(depth);
  if( db == 0 || depth == SST_DEPTH_S32 || depth == SST_DEPTH_F64 )
    return cfail(SST_ERR_INVALID_ARG, "depth must be u8, u16 or f32");
  if( dst_row_stride == 0 ) dst_row_stride = (size_t) width * 3 * db;
  if( dst_frame_stride == 0 ) dst_frame_stride = dst_row_stride * height;
  if( row_stride < (size_t) width * db || (n > 1 && frame_stride < row_stride * height) ||
      dst_row_stride < (size_t) width * 3 * db || (n > 1 && dst_frame_stride < dst_row_stride * height) ||
      (row_stride % db) || (frame_stride % db) || (dst_row_stride % db) || (dst_frame_stride % db) )
    return cfail(SST_ERR_INVALID_ARG, "invalid or misaligned strides");
  cudaStream_t st = (cudaStream_t) stream;
  const dim3 grid((width + 127) / 128, height, n);
  const uint8_t * f = (const uint8_t *) frames;
  uint8_t * d = (uint8_t *) dst;
  switch ( depth ) {
  case SST_DEPTH_U8:
    sst::cal::k_debayer_nn2<uint8_t, long long><<<grid, 128, 0, st>>>(f, width, height, row_stride, frame_stride,
        colorid, d, dst_row_stride, dst_frame_stride);
    break;
  case SST_DEPTH_U16:
    sst::cal::k_debayer_nn2<uint16_t, long long><<<grid, 128, 0, st>>>(f, width, height, row_stride, frame_stride,
        colorid, d, dst_row_stride, dst_frame_stride);
    break;
  default:
    sst::cal::k_debayer_nn2<float, float><<<grid, 128, 0, st>>>(f, width, height, row_stride, frame_stride, colorid, d,
        dst_row_stride, dst_frame_stride);
    break;
  }
  SST_CCK(cudaGetLastError());
  sst_internal_count_launches(1);
  return SST_OK;
}
