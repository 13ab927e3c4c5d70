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
 * core/debayer.cc:828-1161) into BGR frames, one thread per pixel, and its
 * bad-pixel filter (:200-216): per (Bayer plane) pixel a KS x KS median by a
 * register bitonic network and its absolute deviation, then the box mean of
 * the deviations decides whether the median replaces the pixel.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <type_traits>

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
__device__ __forceinline__ T nn2_mean(A s, int n)
{
  if constexpr( sizeof(A) == 4 && !std::is_floating_point<A>::value ) return (T) ((s + n / 2) / n);
  else return (T) __fdiv_rn(s, (float) n);
}

/* nninterpolation (core/debayer.cc:828-1161): one thread per 2 x 2 Bayer
 * cell, which holds the 4 x 4 raw block around it (rows and columns -1 .. +2,
 * BORDER_REFLECT_101) and writes its four BGR pixels. Sums in A (int for
 * integer frames: the rounded means (s + n / 2) / n are those of 64-bit sums;
 * f32 for float ones) in the order N W E S / NW NE SW SE / W E / N S. */
template<typename T, typename A>
__global__ void __launch_bounds__(128) k_debayer_nn2(const uint8_t * frames, int w, int h, size_t rs, size_t fs,
    int colorid, uint8_t * dst, size_t drs, size_t dfs)
{
  const int cx = blockIdx.x * 128 + threadIdx.x, cy = blockIdx.y;
  if( 2 * cx >= w ) return;
  const uint8_t * f = frames + (size_t) blockIdx.z * fs;
  int xs[4], ys[4];
#pragma unroll
  for( int k = 0; k < 4; ++k ) {
    const int x = 2 * cx - 1 + k, y = 2 * cy - 1 + k;
    xs[k] = x < 0 ? -x : (x >= w ? 2 * (w - 1) - x : x);
    ys[k] = y < 0 ? -y : (y >= h ? 2 * (h - 1) - y : y);
  }
  A v[4][4];
#pragma unroll
  for( int r = 0; r < 4; ++r ) {
    const T * row = (const T *) (f + (size_t) ys[r] * rs);
#pragma unroll
    for( int c = 0; c < 4; ++c ) v[r][c] = (A) row[xs[c]];
  }
#pragma unroll
  for( int dy = 0; dy < 2; ++dy ) {
    T out[6];
#pragma unroll
    for( int dx = 0; dx < 2; ++dx ) {
      const int r = 1 + dy, c = 1 + dx;
      const int own = bayer_color(colorid, 2 * cx + dx, 2 * cy + dy);
#pragma unroll
      for( int ch = 0; ch < 3; ++ch ) {
        T o;
        if( ch == own ) o = (T) v[r][c];
        else if( ch == 1 ) {
          A s = v[r - 1][c];
          s = s + v[r][c - 1];
          s = s + v[r][c + 1];
          s = s + v[r + 1][c];
          o = nn2_mean<T, A>(s, 4);
        }
        else if( own == 1 ) {
          // the colour of the horizontal neighbours takes their mean, the other the vertical one
          const bool horiz = bayer_color(colorid, 2 * cx + dx + 1, 2 * cy + dy) == ch;
          o = horiz ? nn2_mean<T, A>(v[r][c - 1] + v[r][c + 1], 2) : nn2_mean<T, A>(v[r - 1][c] + v[r + 1][c], 2);
        }
        else {
          A s = v[r - 1][c - 1];
          s = s + v[r - 1][c + 1];
          s = s + v[r + 1][c - 1];
          s = s + v[r + 1][c + 1];
          o = nn2_mean<T, A>(s, 4);
        }
        out[dx * 3 + ch] = o;
      }
    }
    T * d = (T *) (dst + (size_t) blockIdx.z * dfs + (size_t) (2 * cy + dy) * drs) + (size_t) 6 * cx;
#pragma unroll
    for( int k = 0; k < 6; ++k ) d[k] = out[k];
  }
}

/* --- bad pixels: median_filter_bad_pixels (core/proc/bad_pixels.cc:14-70) and
 * bayer_denoise (core/io/debayer.cc:1480-1612) --- */

/* ascending bitonic sort of N (a power of two) registers; the indices are
 * compile-time constants once unrolled */
template<int N>
__device__ __forceinline__ void bitonic_sort(float (&v)[N])
{
#pragma unroll
  for( int k = 2; k <= N; k <<= 1 ) {
#pragma unroll
    for( int j = k >> 1; j > 0; j >>= 1 ) {
#pragma unroll
      for( int i = 0; i < N; ++i ) {
        const int l = i ^ j;
        if( l > i ) {
          const float a = v[i], b = v[l];
          const bool up = (i & k) == 0;
          v[i] = up ? fminf(a, b) : fmaxf(a, b);
          v[l] = up ? fmaxf(a, b) : fminf(a, b);
        }
      }
    }
  }
}

template<typename T>
__device__ __forceinline__ float plane_px(const uint8_t * f, size_t rs, int step, int ox, int oy, int x, int y)
{
  return (float) ((const T *) (f + (size_t) (step * y + oy) * rs))[step * x + ox];
}

/* per plane pixel: the KS x KS median (cv::medianBlur, BORDER_REPLICATE) and
 * mad = |p - median|; plane z = frame * nplanes + p samples the frame at
 * (step x + (p & 1), step y + (p >> 1)) */
template<typename T, int KS>
__global__ void __launch_bounds__(256) k_bad_median(const uint8_t * src, size_t rs, size_t fs, int pw, int ph, int step,
    int nplanes, float * med, float * mad)
{
  constexpr int N = KS * KS <= 16 ? 16 : 32, R = KS / 2;
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= pw || y >= ph ) return;
  const int f = blockIdx.z / nplanes, p = blockIdx.z - f * nplanes;
  const int ox = step == 2 ? (p & 1) : 0, oy = step == 2 ? (p >> 1) : 0;
  const uint8_t * fb = src + (size_t) f * fs;
  float v[N];
#pragma unroll
  for( int j = 0; j < KS; ++j ) {
    const int yy = min(max(y + j - R, 0), ph - 1);
#pragma unroll
    for( int i = 0; i < KS; ++i ) v[j * KS + i] = plane_px<T>(fb, rs, step, ox, oy, min(max(x + i - R, 0), pw - 1), yy);
  }
  const float p0 = v[R * KS + R];
#pragma unroll
  for( int i = KS * KS; i < N; ++i ) v[i] = 3.0e38f;
  bitonic_sort<N>(v);
  const float m = v[KS * KS / 2];
  const size_t o = (size_t) blockIdx.z * pw * ph + (size_t) y * pw + x;
  med[o] = m;
  mad[o] = fabsf(p0 - m);
}

/* the normalized KS x KS box mean of mad (BORDER_REFLECT_101; rounded to the
 * nearest integer for integer frames), then p -> median where
 * |median - p| > k mad + minvar */
template<typename T, int KS>
__global__ void __launch_bounds__(256) k_bad_apply(const uint8_t * src, size_t rs, size_t fs, int pw, int ph, int step,
    int nplanes, const float * med, const float * mad, float k, float minvar, uint8_t * dst, size_t drs, size_t dfs)
{
  constexpr int R = KS / 2;
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= pw || y >= ph ) return;
  const int f = blockIdx.z / nplanes, p = blockIdx.z - f * nplanes;
  const int ox = step == 2 ? (p & 1) : 0, oy = step == 2 ? (p >> 1) : 0;
  const float * md = mad + (size_t) blockIdx.z * pw * ph;
  // integer frames: exact integer sums; f32 frames: FP64 sums, in the same order
  typedef typename std::conditional<(sizeof(T) < 4), int, double>::type Acc;
  Acc s = 0;
#pragma unroll
  for( int j = 0; j < KS; ++j ) {
    int yy = y + j - R;
    if( ph == 1 ) yy = 0;
    else while ( yy < 0 || yy >= ph ) yy = yy < 0 ? -yy : 2 * (ph - 1) - yy;
#pragma unroll
    for( int i = 0; i < KS; ++i ) {
      int xx = x + i - R;
      if( pw == 1 ) xx = 0;
      else while ( xx < 0 || xx >= pw ) xx = xx < 0 ? -xx : 2 * (pw - 1) - xx;
      s += (Acc) md[(size_t) yy * pw + xx];
    }
  }
  float q;
  if( sizeof(T) < 4 ) q = (float) (((int) s + KS * KS / 2) / (KS * KS));   // saturate_cast of sum / KS^2 (never a tie)
  else q = (float) ((double) s * (1.0 / (KS * KS)));
  const float p0 = plane_px<T>(src + (size_t) f * fs, rs, step, ox, oy, x, y);
  const float m = med[(size_t) blockIdx.z * pw * ph + (size_t) y * pw + x];
  const float out = fabsf(m - p0) > __fadd_rn(__fmul_rn(k, q), minvar) ? m : p0;
  ((T *) (dst + (size_t) f * dfs + (size_t) (step * y + oy) * drs))[step * x + ox] = (T) out;
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
  const dim3 grid((width / 2 + 127) / 128, height / 2, n);   // one thread per 2 x 2 cell
  const uint8_t * f = (const uint8_t *) frames;
  uint8_t * d = (uint8_t *) dst;
  switch ( depth ) {
  case SST_DEPTH_U8:
    sst::cal::k_debayer_nn2<uint8_t, int><<<grid, 128, 0, st>>>(f, width, height, row_stride, frame_stride,
        colorid, d, dst_row_stride, dst_frame_stride);
    break;
  case SST_DEPTH_U16:
    sst::cal::k_debayer_nn2<uint16_t, int><<<grid, 128, 0, st>>>(f, width, height, row_stride, frame_stride,
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

/* read_input_frame's bad-pixel filter (c_image_stacking_pipeline_base.cc:
 * 200-216): Bayer frames bayer_denoise (3 x 3 per Bayer plane), others
 * median_filter_bad_pixels (5 x 5) */
extern "C" int sst_filter_bad_pixels(const void * frames, int depth, int n, int width, int height, size_t row_stride,
    size_t frame_stride, int colorid, double variation_threshold, void * dst, size_t dst_row_stride,
    size_t dst_frame_stride, void * stream)
{
  if( !frames || !dst ) return cfail(SST_ERR_INVALID_ARG, "sst_filter_bad_pixels: NULL argument");
  const bool bayer = colorid >= SST_COLORID_BAYER_RGGB && colorid <= SST_COLORID_BAYER_BGGR;
  if( n < 1 || n > 16383 || width < 1 || height < 1 || (bayer && ((width & 1) || (height & 1))) )
    return cfail(SST_ERR_INVALID_ARG, "n in 1..16383, width, height >= 1 (even for Bayer frames)");
  const int db = depth_bytes(depth);
  if( db == 0 ) return cfail(SST_ERR_INVALID_ARG, "depth must be u8, u16 or f32");
  if( dst_row_stride == 0 ) dst_row_stride = (size_t) width * db;
  if( dst_frame_stride == 0 ) dst_frame_stride = dst_row_stride * height;
  if( row_stride < (size_t) width * db || (n > 1 && frame_stride < row_stride * height) ||
      dst_row_stride < (size_t) width * db || (n > 1 && dst_frame_stride < dst_row_stride * height) ||
      (row_stride % db) || (frame_stride % db) || (dst_row_stride % db) || (dst_frame_stride % db) )
    return cfail(SST_ERR_INVALID_ARG, "invalid or misaligned strides");
  cudaStream_t st = (cudaStream_t) stream;
  const int step = bayer ? 2 : 1, np = bayer ? 4 : 1;
  const int pw = width / step, ph = height / step;
  const size_t planes = (size_t) n * np * pw * ph;
  ScopedBuf med, mad;
  SST_CCK(med.ensure(planes * sizeof(float)));
  SST_CCK(mad.ensure(planes * sizeof(float)));
  const dim3 grid((pw + 31) / 32, (ph + 7) / 8, n * np);
  const uint8_t * f = (const uint8_t *) frames;
  uint8_t * d = (uint8_t *) dst;
  const float k = (float) variation_threshold, mv = depth == SST_DEPTH_F32 ? 1.f / 256.f : 1.f;
#define SST_BAD(TV, KSV)                                                                                         \
  sst::cal::k_bad_median<TV, KSV><<<grid, 256, 0, st>>>(f, row_stride, frame_stride, pw, ph, step, np,           \
      med.as<float>(), mad.as<float>());                                                                         \
  sst::cal::k_bad_apply<TV, KSV><<<grid, 256, 0, st>>>(f, row_stride, frame_stride, pw, ph, step, np,            \
      med.as<float>(), mad.as<float>(), k, mv, d, dst_row_stride, dst_frame_stride)
  switch ( depth ) {
  case SST_DEPTH_U8:
    if( bayer ) { SST_BAD(uint8_t, 3); } else { SST_BAD(uint8_t, 5); }
    break;
  case SST_DEPTH_U16:
    if( bayer ) { SST_BAD(uint16_t, 3); } else { SST_BAD(uint16_t, 5); }
    break;
  default:
    if( bayer ) { SST_BAD(float, 3); } else { SST_BAD(float, 5); }
    break;
  }
#undef SST_BAD
  SST_CCK(cudaGetLastError());
  sst_internal_count_launches(2);
  SST_CCK(cudaStreamSynchronize(st));   // the scratch planes are released on return
  return SST_OK;
}
