/*
 * sst_accum.cu -- the other frame accumulators of core/average/
 * c_frame_accumulation.cc on the GPU:
 *
 *   c_frame_accumulation_with_fft (:704-900)
 *     per batch of frames: k_fft_pad (BORDER_REFLECT padding to the optimal
 *     DFT size, fftGetOptimalSize core/proc/fft.cc:17-57), a batched cuFFT
 *     R2C transform, k_fft_accumulate (spectral weights max(s, (|F|^2 s)^3),
 *     s = 1 / area^2, fftPower :940-980, accumulated per bin in FP64 over the
 *     batch in frame order); compute(): k_fft_divide, C2R, k_fft_crop (the
 *     DFT_SCALE factor and the crop to the frame). A real frame's spectrum is
 *     conjugate-symmetric and so are its weights, so the half spectrum the
 *     R2C transform keeps carries the whole average.
 *
 *   c_canvas_average (:264-450)
 *     a canvas of max(requested, 3/2 frame) size, the first frame centred;
 *     maintainCanvasBoundaries (:273-318) as one shift copy; k_canvas_add
 *     remaps (image LINEAR / BORDER_REPLICATE, u8 masks NEAREST and f32
 *     weights LINEAR, BORDER_CONSTANT 0) and applies the reference's running
 *     mean (_weighted_average_update :20-129) in FP32 with explicitly rounded
 *     operations, one thread per box pixel.
 *
 * Planar FP32 planes in HBM (channel-major); frames and results cross the
 * C ABI interleaved, as cv::Mat holds them.
 */
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <math.h>
#include <string>
#include <map>
#include <new>

#include "sst_host.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

namespace sst {
namespace acc {

__device__ __forceinline__ int reflect_i(int p, int n)      // BORDER_REFLECT
{
  if( n == 1 ) return 0;
  while ( p < 0 || p >= n ) p = p < 0 ? -p - 1 : 2 * n - p - 1;
  return p;
}

template<typename T>
__device__ __forceinline__ float ldv(const uint8_t * base, size_t rs, int x, int y, int cn, int c)
{
  return (float) ((const T *) (base + (size_t) y * rs))[(size_t) x * cn + c];
}

/* padded real planes: plane z = f * cn + c of frame f0 + f */
template<typename T>
__global__ void __launch_bounds__(256) k_fft_pad(const uint8_t * src, size_t rs, size_t fs, float scale, int cn, int w,
    int h, int fw, int fh, int top, int left, float * dst)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= fw || y >= fh ) return;
  const int f = blockIdx.z / cn, c = blockIdx.z - f * cn;
  const float v = ldv<T>(src + (size_t) f * fs, rs, reflect_i(x - left, w), reflect_i(y - top, h), cn, c);
  dst[((size_t) blockIdx.z * fh + y) * fw + x] = v * scale;
}

/* acc[c][k] += F w, W[c][k] += w over the nb frames of the batch, in order */
__global__ void k_fft_accumulate(const float2 * spec, int nb, int cn, size_t bins, double s, double2 * acc, double * W)
{
  const size_t k = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( k >= bins ) return;
  const int c = blockIdx.y;
  double2 a = acc[(size_t) c * bins + k];
  double ws = W[(size_t) c * bins + k];
  for( int f = 0; f < nb; ++f ) {
    const float2 F = spec[((size_t) f * cn + c) * bins + k];
    const double re = F.x, im = F.y;
    const double q = (re * re + im * im) * s;
    const double wk = fmax(s, q * q * q);
    a.x += re * (double) (float) wk, a.y += im * (double) (float) wk;   // the reference keeps w as float
    ws += (double) (float) wk;
  }
  acc[(size_t) c * bins + k] = a;
  W[(size_t) c * bins + k] = ws;
}

__global__ void k_fft_divide(const double2 * acc, const double * W, size_t n, float2 * out)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= n ) return;
  const double w = W[i];
  out[i] = make_float2((float) (acc[i].x / w), (float) (acc[i].y / w));
}

/* crop of the inverse transform (DFT_SCALE) into interleaved channels */
__global__ void k_fft_crop(const float * real, int fw, int fh, int top, int left, int w, int h, int cn, float scale,
    float * dst, size_t drs)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const int c = blockIdx.z;
  ((float *) ((uint8_t *) dst + (size_t) y * drs))[(size_t) x * cn + c] =
      real[((size_t) c * fh + y + top) * fw + x + left] * scale;
}

/* ---------------------------------------------------------------- canvas */

/* one box pixel of c_canvas_average::add: the (remapped) value and weight,
 * then _weighted_average_update's running mean in FP32 */
template<typename T>
__global__ void __launch_bounds__(256) k_canvas_add(const uint8_t * src, size_t rs, int w, int h, int cn, float scale,
    const uint8_t * wts, size_t wrs, int wkind, const float * rmap, int bw, int bh, float * A, float * W, int cw,
    size_t plane, int rx, int ry)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= bw || y >= bh ) return;
  float wn = 1.f;
  float X = 0.f, Y = 0.f;
  int x0 = x, y0 = y;
  float fx = 0.f, fy = 0.f;
  if( rmap ) {
    X = rmap[((size_t) y * bw + x) * 2], Y = rmap[((size_t) y * bw + x) * 2 + 1];
    const float cx = fminf(fmaxf(X, -1e8f), 1e8f), cy = fminf(fmaxf(Y, -1e8f), 1e8f);
    x0 = __float2int_rd(cx), y0 = __float2int_rd(cy);
    fx = cx - (float) x0, fy = cy - (float) y0;
    if( wkind == 1 ) {
      const int xi = __float2int_rn(cx), yi = __float2int_rn(cy);
      wn = (xi >= 0 && xi < w && yi >= 0 && yi < h && wts[(size_t) yi * wrs + xi]) ? 1.f : 0.f;
    }
    else if( wkind == 2 ) {
      float v[4];
#pragma unroll
      for( int j = 0; j < 4; ++j ) {
        const int xi = x0 + (j & 1), yi = y0 + (j >> 1);
        v[j] = (xi >= 0 && xi < w && yi >= 0 && yi < h) ? ((const float *) (wts + (size_t) yi * wrs))[xi] : 0.f;
      }
      const float t0 = fmaf(fx, v[1] - v[0], v[0]), t1 = fmaf(fx, v[3] - v[2], v[2]);
      wn = fmaf(fy, t1 - t0, t0);
    }
  }
  else if( wkind == 1 ) wn = wts[(size_t) y * wrs + x] ? 1.f : 0.f;
  else if( wkind == 2 ) wn = ((const float *) (wts + (size_t) y * wrs))[x];
  if( !(wn > 0.f) ) return;
  const size_t o = (size_t) (ry + y) * cw + rx + x;
  const float Wn = __fadd_rn(W[o], wn);
  const float fac = wkind == 2 ? __fdiv_rn(wn, Wn) : __fdiv_rn(1.f, Wn);
  W[o] = Wn;
  const int xa = min(max(x0, 0), w - 1), xb = min(max(x0 + 1, 0), w - 1);
  const int ya = min(max(y0, 0), h - 1), yb = min(max(y0 + 1, 0), h - 1);
  for( int c = 0; c < cn; ++c ) {
    float I;
    if( rmap ) {   // BORDER_REPLICATE taps
      const float v00 = ldv<T>(src, rs, xa, ya, cn, c), v01 = ldv<T>(src, rs, xb, ya, cn, c);
      const float v10 = ldv<T>(src, rs, xa, yb, cn, c), v11 = ldv<T>(src, rs, xb, yb, cn, c);
      const float t0 = fmaf(fx, v01 - v00, v00), t1 = fmaf(fx, v11 - v10, v10);
      I = fmaf(fy, t1 - t0, t0) * scale;
    }
    else I = ldv<T>(src, rs, x, y, cn, c) * scale;
    float * a = A + (size_t) c * plane + o;
    const float Ao = *a;
    *a = __fadd_rn(Ao, __fmul_rn(__fsub_rn(I, Ao), fac));
  }
}

/* maintainCanvasBoundaries' copy: dst = zeros, dst(shifted box) = src(box) */
__global__ void k_canvas_shift(const float * src, float * dst, int cw, int ch, int planes, int sx, int sy)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= cw || y >= ch ) return;
  const int xs = x - sx, ys = y - sy;
  const bool in = xs >= 0 && xs < cw && ys >= 0 && ys < ch;
  const size_t plane = (size_t) cw * ch;
  for( int p = 0; p < planes; ++p )
    dst[(size_t) p * plane + (size_t) y * cw + x] = in ? src[(size_t) p * plane + (size_t) ys * cw + xs] : 0.f;
}

/* compute(): avg = A * dscale (interleaved), mask = 255 where W > 0 */
__global__ void k_canvas_compute(const float * A, const float * W, int cw, int ch, int cn, int bx, int by, int bw, int bh,
    float dscale, float * avg, size_t ars, uint8_t * mask, size_t mrs)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= bw || y >= bh ) return;
  const size_t plane = (size_t) cw * ch, o = (size_t) (by + y) * cw + bx + x;
  if( avg ) {
    float * d = (float *) ((uint8_t *) avg + (size_t) y * ars) + (size_t) x * cn;
    for( int c = 0; c < cn; ++c ) d[c] = dscale == 1.f ? A[(size_t) c * plane + o] : A[(size_t) c * plane + o] * dscale;
  }
  if( mask ) mask[(size_t) y * mrs + x] = W[o] > 0.f ? 255 : 0;
}

}  // namespace acc
}  // namespace sst

using namespace sst::acc;

namespace {

int afail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_ACK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return afail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

#define SST_FCK(call)                                                                          \
  do {                                                                                         \
    cufftResult r_ = (call);                                                                   \
    if( r_ != CUFFT_SUCCESS )                                                                  \
      return afail(SST_ERR_CUDA, std::string(#call) + " failed: cufft error " + std::to_string((int) r_)); \
  } while ( 0 )

bool is_235(int m)
{
  for( int f : { 2, 3, 5 } ) while ( m % f == 0 ) m /= f;
  return m == 1;
}

dim3 grid2(int w, int h, int z)
{
  return dim3((unsigned) ((w + 31) / 32), (unsigned) ((h + 7) / 8), (unsigned) z);
}

/* a host or device source brought to the device */
struct Staged {
  ScopedBuf buf;
  const void * p = nullptr;
  cudaError_t stage(const void * src, size_t bytes, int on_device, cudaStream_t st)
  {
    if( on_device || !src ) {
      p = src;
      return cudaSuccess;
    }
    cudaError_t e = buf.ensure(bytes);
    if( e != cudaSuccess ) return e;
    p = buf.p;
    return cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, st);
  }
};

}  // namespace

/* ---------------------------------------------------------- FFT average */

extern "C" int sst_optimal_dft_size(int n)
{
  if( n <= 1 ) return 1;
  int m = n;
  while ( !is_235(m) ) ++m;
  return m;
}

struct sst_fft_average {
  int w = 0, h = 0, cn = 0, fw = 0, fh = 0, top = 0, left = 0;
  size_t bins = 0;               // fh x (fw / 2 + 1)
  int frames = 0;
  DevBuf acc, W, pad, spec, real;
  std::map<int, cufftHandle> fwd;   // R2C plans by batch size
  cufftHandle inv = 0;
  bool has_inv = false;
  ~sst_fft_average() { reset(); }
  void reset()
  {
    for( auto & p : fwd ) cufftDestroy(p.second);
    fwd.clear();
    if( has_inv ) cufftDestroy(inv);
    has_inv = false;
    acc.release(), W.release(), pad.release(), spec.release(), real.release();
    w = h = cn = fw = fh = 0;
    bins = 0;
    frames = 0;
  }
};

extern "C" int sst_fft_average_create(sst_fft_average ** out)
{
  if( !out ) return afail(SST_ERR_INVALID_ARG, "sst_fft_average_create: out is NULL");
  *out = new (std::nothrow) sst_fft_average();
  return *out ? SST_OK : afail(SST_ERR_NOMEM, "out of host memory");
}

extern "C" int sst_fft_average_destroy(sst_fft_average * h)
{
  delete h;
  return SST_OK;
}

extern "C" int sst_fft_average_clear(sst_fft_average * h)
{
  if( !h ) return afail(SST_ERR_INVALID_ARG, "NULL accumulator");
  h->reset();
  return SST_OK;
}

extern "C" int sst_fft_average_accumulated_frames(const sst_fft_average * h)
{
  return h ? h->frames : 0;
}

extern "C" int sst_fft_average_size(const sst_fft_average * h, int * fft_width, int * fft_height)
{
  if( !h ) return afail(SST_ERR_INVALID_ARG, "NULL accumulator");
  if( fft_width ) *fft_width = h->fw;
  if( fft_height ) *fft_height = h->fh;
  return SST_OK;
}

static int fft_plan(sst_fft_average * a, int batch, cufftHandle * out)
{
  auto it = a->fwd.find(batch);
  if( it != a->fwd.end() ) {
    *out = it->second;
    return SST_OK;
  }
  cufftHandle p;
  int dims[2] = { a->fh, a->fw };
  SST_FCK(cufftPlanMany(&p, 2, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_R2C, batch));
  a->fwd[batch] = p;
  *out = p;
  return SST_OK;
}

extern "C" int sst_fft_average_add(sst_fft_average * a, const void * frames, int depth, int n, int width, int height,
    int channels, size_t row_stride, size_t frame_stride, double scale, int on_device, void * stream)
{
  if( !a || !frames ) return afail(SST_ERR_INVALID_ARG, "sst_fft_average_add: NULL argument");
  const int db = depth_bytes(depth);
  if( !db ) return afail(SST_ERR_INVALID_ARG, "depth must be u8, u16 or f32");
  if( n < 1 || width < 1 || height < 1 || channels < 1 || channels > 4 )
    return afail(SST_ERR_INVALID_ARG, "n, width, height >= 1 and 1..4 channels");
  if( row_stride < (size_t) width * channels * db || (n > 1 && frame_stride < row_stride * height) ||
      (row_stride % db) || (frame_stride % db) )
    return afail(SST_ERR_INVALID_ARG, "invalid or misaligned strides");
  if( a->cn && (a->w != width || a->h != height || a->cn != channels) )
    return afail(SST_ERR_INVALID_ARG, "frame size or channels differ from the accumulated frames");
  cudaStream_t st = (cudaStream_t) stream;
  if( !a->cn ) {
    a->w = width, a->h = height, a->cn = channels;
    a->fw = sst_optimal_dft_size(width), a->fh = sst_optimal_dft_size(height);
    a->top = (a->fh - height) / 2, a->left = (a->fw - width) / 2;
    a->bins = (size_t) a->fh * (a->fw / 2 + 1);
    SST_ACK(a->acc.ensure(a->bins * channels * sizeof(double2)));
    SST_ACK(a->W.ensure(a->bins * channels * sizeof(double)));
    SST_ACK(cudaMemsetAsync(a->acc.p, 0, a->bins * channels * sizeof(double2), st));
    SST_ACK(cudaMemsetAsync(a->W.p, 0, a->bins * channels * sizeof(double), st));
  }
  // frames per transform batch: about 64 planes
  const int cap = std::max(1, 64 / channels);
  const size_t fplane = (size_t) a->fw * a->fh;
  SST_ACK(a->pad.ensure((size_t) cap * channels * fplane * sizeof(float)));
  SST_ACK(a->spec.ensure((size_t) cap * channels * a->bins * sizeof(float2)));
  Staged src;
  SST_ACK(src.stage(frames, frame_stride * (n - 1) + row_stride * height, on_device, st));
  const double s = 1.0 / ((double) fplane * (double) fplane);
  for( int f0 = 0; f0 < n; f0 += cap ) {
    const int nb = std::min(cap, n - f0);
    const uint8_t * fb = (const uint8_t *) src.p + (size_t) f0 * frame_stride;
    const dim3 g = grid2(a->fw, a->fh, nb * channels);
    switch ( depth ) {
    case SST_DEPTH_U8:
      k_fft_pad<uint8_t><<<g, 256, 0, st>>>(fb, row_stride, frame_stride, (float) scale, channels, width, height, a->fw,
          a->fh, a->top, a->left, a->pad.as<float>());
      break;
    case SST_DEPTH_U16:
      k_fft_pad<uint16_t><<<g, 256, 0, st>>>(fb, row_stride, frame_stride, (float) scale, channels, width, height, a->fw,
          a->fh, a->top, a->left, a->pad.as<float>());
      break;
    default:
      k_fft_pad<float><<<g, 256, 0, st>>>(fb, row_stride, frame_stride, (float) scale, channels, width, height, a->fw,
          a->fh, a->top, a->left, a->pad.as<float>());
      break;
    }
    SST_ACK(cudaGetLastError());
    cufftHandle p;
    int r = fft_plan(a, nb * channels, &p);
    if( r != SST_OK ) return r;
    SST_FCK(cufftSetStream(p, st));
    SST_FCK(cufftExecR2C(p, a->pad.as<cufftReal>(), a->spec.as<cufftComplex>()));
    k_fft_accumulate<<<dim3((unsigned) ((a->bins + 255) / 256), channels), 256, 0, st>>>(a->spec.as<float2>(), nb,
        channels, a->bins, s, a->acc.as<double2>(), a->W.as<double>());
    SST_ACK(cudaGetLastError());
    sst_internal_count_launches(2);
  }
  if( !on_device ) SST_ACK(cudaStreamSynchronize(st));
  a->frames += n;
  return SST_OK;
}

extern "C" int sst_fft_average_compute(sst_fft_average * a, float * avg, size_t avg_row_stride, uint8_t * mask,
    size_t mask_row_stride, int on_device, void * stream)
{
  if( !a ) return afail(SST_ERR_INVALID_ARG, "NULL accumulator");
  if( a->frames < 1 ) return afail(SST_ERR_STATE, "c_frame_accumulation_with_fft: accumulator is empty");
  cudaStream_t st = (cudaStream_t) stream;
  const int w = a->w, h = a->h, cn = a->cn;
  if( avg_row_stride == 0 ) avg_row_stride = (size_t) w * cn * sizeof(float);
  if( mask_row_stride == 0 ) mask_row_stride = (size_t) w;
  if( avg_row_stride < (size_t) w * cn * sizeof(float) || (avg_row_stride & 3) || mask_row_stride < (size_t) w )
    return afail(SST_ERR_INVALID_ARG, "invalid strides");
  if( !a->has_inv ) {
    int dims[2] = { a->fh, a->fw };
    SST_FCK(cufftPlanMany(&a->inv, 2, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_C2R, cn));
    a->has_inv = true;
  }
  SST_ACK(a->spec.ensure((size_t) cn * a->bins * sizeof(float2)));
  SST_ACK(a->real.ensure((size_t) cn * a->fw * a->fh * sizeof(float)));
  const size_t nb = (size_t) cn * a->bins;
  k_fft_divide<<<(unsigned) ((nb + 255) / 256), 256, 0, st>>>(a->acc.as<double2>(), a->W.as<double>(), nb,
      a->spec.as<float2>());
  SST_ACK(cudaGetLastError());
  SST_FCK(cufftSetStream(a->inv, st));
  SST_FCK(cufftExecC2R(a->inv, a->spec.as<cufftComplex>(), a->real.as<cufftReal>()));
  ScopedBuf davg, dmask;
  float * out = avg;
  uint8_t * mout = mask;
  if( !on_device ) {
    if( avg ) {
      SST_ACK(davg.ensure(avg_row_stride * h));
      out = davg.as<float>();
    }
    if( mask ) {
      SST_ACK(dmask.ensure(mask_row_stride * h));
      mout = dmask.as<uint8_t>();
    }
  }
  if( out ) {
    k_fft_crop<<<grid2(w, h, cn), 256, 0, st>>>(a->real.as<float>(), a->fw, a->fh, a->top, a->left, w, h, cn,
        (float) (1.0 / ((double) a->fw * a->fh)), out, avg_row_stride);
    SST_ACK(cudaGetLastError());
  }
  if( mout ) SST_ACK(cudaMemset2DAsync(mout, mask_row_stride, 255, w, h, st));
  sst_internal_count_launches(out ? 2 : 1);
  if( !on_device ) {
    if( avg ) SST_ACK(cudaMemcpyAsync(avg, out, avg_row_stride * h, cudaMemcpyDeviceToHost, st));
    if( mask ) SST_ACK(cudaMemcpyAsync(mask, mout, mask_row_stride * h, cudaMemcpyDeviceToHost, st));
    SST_ACK(cudaStreamSynchronize(st));
  }
  return SST_OK;
}

/* ------------------------------------------------------- canvas average */

struct sst_canvas_average {
  int req_w = 0, req_h = 0;
  int cw = 0, ch = 0, cn = 0;
  int lx = 0, ly = 0, lw = 0, lh = 0;
  int frames = 0;
  DevBuf A, W, T;   // cn planes, the weight plane, shift scratch
  void reset()
  {
    A.release(), W.release(), T.release();
    cw = ch = cn = 0;
    lx = ly = lw = lh = 0;
    frames = 0;
  }
};

extern "C" int sst_canvas_average_create(sst_canvas_average ** out, int canvas_width, int canvas_height)
{
  if( !out ) return afail(SST_ERR_INVALID_ARG, "sst_canvas_average_create: out is NULL");
  sst_canvas_average * c = new (std::nothrow) sst_canvas_average();
  if( !c ) return afail(SST_ERR_NOMEM, "out of host memory");
  c->req_w = std::max(0, canvas_width), c->req_h = std::max(0, canvas_height);
  *out = c;
  return SST_OK;
}

extern "C" int sst_canvas_average_destroy(sst_canvas_average * c)
{
  if( c ) c->reset();
  delete c;
  return SST_OK;
}

extern "C" int sst_canvas_average_clear(sst_canvas_average * c)
{
  if( !c ) return afail(SST_ERR_INVALID_ARG, "NULL canvas");
  c->reset();
  return SST_OK;
}

extern "C" int sst_canvas_average_set_canvas_size(sst_canvas_average * c, int canvas_width, int canvas_height)
{
  if( !c ) return afail(SST_ERR_INVALID_ARG, "NULL canvas");
  c->reset();
  c->req_w = std::max(0, canvas_width), c->req_h = std::max(0, canvas_height);
  return SST_OK;
}

extern "C" int sst_canvas_average_state(const sst_canvas_average * c, int * canvas_width, int * canvas_height,
    int * last_bbox, int * accumulated_frames)
{
  if( !c ) return afail(SST_ERR_INVALID_ARG, "NULL canvas");
  if( canvas_width ) *canvas_width = c->cw;
  if( canvas_height ) *canvas_height = c->ch;
  if( last_bbox ) last_bbox[0] = c->lx, last_bbox[1] = c->ly, last_bbox[2] = c->lw, last_bbox[3] = c->lh;
  if( accumulated_frames ) *accumulated_frames = c->frames;
  return SST_OK;
}

static int canvas_launch(sst_canvas_average * c, const void * img, int depth, size_t rs, int w, int h, double scale,
    const void * wts, int wkind, size_t wrs, const float * rmap, int bw, int bh, int rx, int ry, cudaStream_t st)
{
  const dim3 g = grid2(bw, bh, 1);
  const size_t plane = (size_t) c->cw * c->ch;
  const uint8_t * s = (const uint8_t *) img;
  const uint8_t * wb = (const uint8_t *) wts;
  switch ( depth ) {
  case SST_DEPTH_U8:
    k_canvas_add<uint8_t><<<g, 256, 0, st>>>(s, rs, w, h, c->cn, (float) scale, wb, wrs, wkind, rmap, bw, bh,
        c->A.as<float>(), c->W.as<float>(), c->cw, plane, rx, ry);
    break;
  case SST_DEPTH_U16:
    k_canvas_add<uint16_t><<<g, 256, 0, st>>>(s, rs, w, h, c->cn, (float) scale, wb, wrs, wkind, rmap, bw, bh,
        c->A.as<float>(), c->W.as<float>(), c->cw, plane, rx, ry);
    break;
  default:
    k_canvas_add<float><<<g, 256, 0, st>>>(s, rs, w, h, c->cn, (float) scale, wb, wrs, wkind, rmap, bw, bh,
        c->A.as<float>(), c->W.as<float>(), c->cw, plane, rx, ry);
    break;
  }
  SST_ACK(cudaGetLastError());
  sst_internal_count_launches(1);
  return SST_OK;
}

extern "C" int sst_canvas_average_add(sst_canvas_average * c, const void * image, int depth, int width, int height,
    int channels, size_t row_stride, double scale, const void * weights, int weights_depth, size_t weights_stride,
    const float * rmap, const int32_t * bbox, int on_device, void * stream)
{
  if( !c || !image ) return afail(SST_ERR_INVALID_ARG, "sst_canvas_average_add: NULL argument");
  const int db = depth_bytes(depth);
  if( !db ) return afail(SST_ERR_INVALID_ARG, "depth must be u8, u16 or f32");
  if( width < 1 || height < 1 || channels < 1 || channels > 4 )
    return afail(SST_ERR_INVALID_ARG, "width, height >= 1 and 1..4 channels");
  if( row_stride < (size_t) width * channels * db || (row_stride % db) )
    return afail(SST_ERR_INVALID_ARG, "invalid or misaligned row stride");
  int wkind = 0;
  if( weights ) {
    if( weights_depth == SST_DEPTH_U8 ) wkind = 1;
    else if( weights_depth == SST_DEPTH_F32 ) wkind = 2;
    else return afail(SST_ERR_INVALID_ARG, "weights must be a u8 mask or f32 weights");
    if( weights_stride < (size_t) width * (wkind == 2 ? 4 : 1) || (wkind == 2 && (weights_stride & 3)) )
      return afail(SST_ERR_INVALID_ARG, "invalid weights stride");
  }
  if( c->cn && channels != c->cn ) return afail(SST_ERR_INVALID_ARG, "channels differ from the canvas");
  const int bx = bbox ? bbox[0] : 0, by = bbox ? bbox[1] : 0, bw = bbox ? bbox[2] : 0, bh = bbox ? bbox[3] : 0;
  const bool box_empty = bw <= 0 || bh <= 0;
  if( rmap && box_empty ) return afail(SST_ERR_INVALID_ARG, "ROI is empty");
  cudaStream_t st = (cudaStream_t) stream;
  Staged simg, swts, smap;
  SST_ACK(simg.stage(image, row_stride * height, on_device, st));
  SST_ACK(swts.stage(weights, weights_stride * height, on_device, st));
  if( rmap ) SST_ACK(smap.stage(rmap, (size_t) bw * bh * 2 * sizeof(float), on_device, st));
  int r = SST_OK;
  if( !c->frames ) {
    // the very first frame, centred on the canvas
    c->cw = std::max(c->req_w, 3 * width / 2), c->ch = std::max(c->req_h, 3 * height / 2), c->cn = channels;
    const size_t plane = (size_t) c->cw * c->ch;
    SST_ACK(c->A.ensure(plane * channels * sizeof(float)));
    SST_ACK(c->W.ensure(plane * sizeof(float)));
    SST_ACK(cudaMemsetAsync(c->A.p, 0, plane * channels * sizeof(float), st));
    SST_ACK(cudaMemsetAsync(c->W.p, 0, plane * sizeof(float), st));
    const int tx = c->cw / 2 - width / 2, ty = c->ch / 2 - height / 2;
    r = canvas_launch(c, simg.p, depth, row_stride, width, height, scale, swts.p, wkind, weights_stride, nullptr, width,
        height, tx, ty, st);
    c->lx = tx, c->ly = ty, c->lw = width, c->lh = height;
  }
  else if( box_empty && !rmap ) {
    // no remap: the frame on the last box, clipped to the canvas
    const int x0 = std::max(c->lx, 0), y0 = std::max(c->ly, 0);
    const int x1 = std::min(c->lx + width, c->cw), y1 = std::min(c->ly + height, c->ch);
    const int rw = std::max(0, x1 - x0), rh = std::max(0, y1 - y0);
    if( rw == width && rh == height )   // the reference's update rejects a clipped box
      r = canvas_launch(c, simg.p, depth, row_stride, width, height, scale, swts.p, wkind, weights_stride, nullptr,
          width, height, x0, y0, st);
    c->lx = x0, c->ly = y0, c->lw = rw, c->lh = rh;
  }
  else {
    int x0 = std::max(bx, 0), y0 = std::max(by, 0);
    const int rw = std::min(bx + bw, c->cw) - x0, rh = std::min(by + bh, c->ch) - y0;
    if( rw <= 0 || rh <= 0 ) return afail(SST_ERR_INVALID_ARG, "ROI is empty");
    // maintainCanvasBoundaries (c_frame_accumulation.cc:273-318)
    const int margin = 32;
    int sx = 0, sy = 0;
    if( x0 < margin ) sx = 2 * margin;
    else if( x0 + rw >= c->cw - margin ) sx = -2 * margin;
    if( y0 < margin ) sy = 2 * margin;
    else if( y0 + rh >= c->ch - margin ) sy = -2 * margin;
    if( (sx || sy) && c->cw - std::abs(sx) > 0 && c->ch - std::abs(sy) > 0 ) {
      const size_t plane = (size_t) c->cw * c->ch;
      SST_ACK(c->T.ensure(plane * (c->cn + 1) * sizeof(float)));
      // A and W are consecutive only through the scratch: shift each into it, then swap
      float * t = c->T.as<float>();
      k_canvas_shift<<<grid2(c->cw, c->ch, 1), 256, 0, st>>>(c->A.as<float>(), t, c->cw, c->ch, c->cn, sx, sy);
      k_canvas_shift<<<grid2(c->cw, c->ch, 1), 256, 0, st>>>(c->W.as<float>(), t + plane * c->cn, c->cw, c->ch, 1, sx,
          sy);
      SST_ACK(cudaGetLastError());
      sst_internal_count_launches(2);
      SST_ACK(cudaMemcpyAsync(c->A.p, t, plane * c->cn * sizeof(float), cudaMemcpyDeviceToDevice, st));
      SST_ACK(cudaMemcpyAsync(c->W.p, t + plane * c->cn, plane * sizeof(float), cudaMemcpyDeviceToDevice, st));
      x0 += sx, y0 += sy;
    }
    if( x0 < 0 || y0 < 0 || x0 + rw > c->cw || y0 + rh > c->ch )
      return afail(SST_ERR_INVALID_ARG, "the shifted box leaves the canvas");
    if( rmap && rw == bw && rh == bh )
      r = canvas_launch(c, simg.p, depth, row_stride, width, height, scale, swts.p, wkind, weights_stride,
          (const float *) smap.p, bw, bh, x0, y0, st);
    else if( !rmap && rw == width && rh == height )
      r = canvas_launch(c, simg.p, depth, row_stride, width, height, scale, swts.p, wkind, weights_stride, nullptr,
          width, height, x0, y0, st);
    c->lx = x0, c->ly = y0, c->lw = rw, c->lh = rh;
  }
  if( r != SST_OK ) return r;
  if( !on_device ) SST_ACK(cudaStreamSynchronize(st));
  ++c->frames;
  return SST_OK;
}

extern "C" int sst_canvas_average_compute(sst_canvas_average * c, float * avg, size_t avg_row_stride, uint8_t * mask,
    size_t mask_row_stride, double dscale, const int32_t * rbbox, int32_t * out_bbox, int on_device, void * stream)
{
  if( !c ) return afail(SST_ERR_INVALID_ARG, "NULL canvas");
  if( c->frames < 1 ) return afail(SST_ERR_STATE, "no frames accumulated");
  int bx = 0, by = 0, bw = c->cw, bh = c->ch;
  if( rbbox && rbbox[2] > 0 && rbbox[3] > 0 ) {
    bx = std::max(rbbox[0], 0), by = std::max(rbbox[1], 0);
    bw = std::min(rbbox[0] + rbbox[2], c->cw) - bx, bh = std::min(rbbox[1] + rbbox[3], c->ch) - by;
    if( bw <= 0 || bh <= 0 ) return afail(SST_ERR_INVALID_ARG, "the requested box misses the canvas");
  }
  if( out_bbox ) out_bbox[0] = bx, out_bbox[1] = by, out_bbox[2] = bw, out_bbox[3] = bh;
  if( avg_row_stride == 0 ) avg_row_stride = (size_t) bw * c->cn * sizeof(float);
  if( mask_row_stride == 0 ) mask_row_stride = (size_t) bw;
  if( avg_row_stride < (size_t) bw * c->cn * sizeof(float) || (avg_row_stride & 3) || mask_row_stride < (size_t) bw )
    return afail(SST_ERR_INVALID_ARG, "invalid strides");
  cudaStream_t st = (cudaStream_t) stream;
  ScopedBuf davg, dmask;
  float * out = avg;
  uint8_t * mout = mask;
  if( !on_device ) {
    if( avg ) {
      SST_ACK(davg.ensure(avg_row_stride * bh));
      out = davg.as<float>();
    }
    if( mask ) {
      SST_ACK(dmask.ensure(mask_row_stride * bh));
      mout = dmask.as<uint8_t>();
    }
  }
  if( out || mout ) {
    k_canvas_compute<<<grid2(bw, bh, 1), 256, 0, st>>>(c->A.as<float>(), c->W.as<float>(), c->cw, c->ch, c->cn, bx,
        by, bw, bh, (float) dscale, out, avg_row_stride, mout, mask_row_stride);
    SST_ACK(cudaGetLastError());
    sst_internal_count_launches(1);
  }
  if( !on_device ) {
    if( avg ) SST_ACK(cudaMemcpyAsync(avg, out, avg_row_stride * bh, cudaMemcpyDeviceToHost, st));
    if( mask ) SST_ACK(cudaMemcpyAsync(mask, mout, mask_row_stride * bh, cudaMemcpyDeviceToHost, st));
    SST_ACK(cudaStreamSynchronize(st));
  }
  return SST_OK;
}

/* the counter plane (c_canvas_average::counter()) */
extern "C" int sst_canvas_average_counter(sst_canvas_average * c, float * W, size_t row_stride, int on_device,
    void * stream)
{
  if( !c || !W ) return afail(SST_ERR_INVALID_ARG, "NULL argument");
  if( c->frames < 1 ) return afail(SST_ERR_STATE, "no frames accumulated");
  if( row_stride == 0 ) row_stride = (size_t) c->cw * sizeof(float);
  if( row_stride < (size_t) c->cw * sizeof(float) ) return afail(SST_ERR_INVALID_ARG, "invalid stride");
  cudaStream_t st = (cudaStream_t) stream;
  SST_ACK(cudaMemcpy2DAsync(W, row_stride, c->W.p, (size_t) c->cw * sizeof(float), (size_t) c->cw * sizeof(float), c->ch,
      on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
  if( !on_device ) SST_ACK(cudaStreamSynchronize(st));
  return SST_OK;
}
