/*
 * sst_focus.cu -- c_laplacian_pyramid_focus_stacking (core/average/
 * c_frame_accumulation.cc:464-688) and linear_interpolation_inpaint
 * (core/proc/inpaint/linear_interpolation_inpaint.cc) on the GPU.
 *
 * add() works on batches of frames: planar FP32 conversion, the optional
 * hole filling (row and column scans, one warp per row / column, iterated
 * until no hole gains a value), build_laplacian_pyramid (core/proc/
 * laplacian_pyramid.cc:45-96; tap-table pyrDown / pyrUp, minimum size 8) for
 * every frame of the batch at once, the u8 mask pyramid (cv::buildPyramid)
 * zeroing the Laplacian levels where it is below 255, then the fold into the
 * accumulator pyramid in frame order:
 *   - select_max_energy: per coefficient the frame's value replaces the
 *     accumulated one where |frame| > |acc| (one pass over the batch per
 *     level); with a smoothing kernel G, |.| is smoothed first, which makes
 *     each frame depend on the previous fold, so frames go one at a time;
 *   - weighted_average: acc += lap w, wwp += w with w = lap^2 (or the squared
 *     channel sum), G-smoothed + 1e-12 when G is set;
 *   - the top (Gaussian) level: blended frame by frame with the standard
 *     deviations of the accumulated and the new top level (one CTA).
 * compute(): reconstruct_laplacian_pyramid (:98-122) of acc (or acc / wwp).
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include <string>
#include <vector>
#include <new>

#include "sst_host.h"
#include "sst_taps.h"
#include "sst_resample.cuh"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu

namespace sst {
namespace fs {

/* interleaved u8 / u16 / f32 frames -> planar FP32 planes [f][c] */
template<typename T>
__global__ void __launch_bounds__(256) k_to_planar(const uint8_t * src, size_t rs, size_t fstride, int w, int h, int cn,
    float scale, float * dst)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const int f = blockIdx.z;
  const T * row = (const T *) (src + (size_t) f * fstride + (size_t) y * rs);
  const size_t plane = (size_t) w * h;
  for( int c = 0; c < cn; ++c ) dst[((size_t) f * cn + c) * plane + (size_t) y * w + x] = (float) row[(size_t) x * cn + c] * scale;
}

/* planar [c] -> interleaved FP32 output */
__global__ void k_to_interleaved(const float * src, int w, int h, int cn, float * dst, size_t drs)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const size_t plane = (size_t) w * h;
  float * d = (float *) ((uint8_t *) dst + (size_t) y * drs) + (size_t) x * cn;
  for( int c = 0; c < cn; ++c ) d[c] = src[(size_t) c * plane + (size_t) y * w + x];
}

/* --- linear_interpolation_inpaint: rows / columns of hole runs --- */

/* one warp per (frame, row) [rows] or (frame, column) [columns]: the values
 * and distances of _interpolate_holes_h2 / _v2 for every hole of the line.
 * Each lane takes a contiguous chunk of the line; the last valid position
 * before its chunk and the first one after it come from a prefix max / suffix
 * min over the lanes, so each hole run (which may span chunks) is filled from
 * the same end points s and e as the sequential scan, with the same FP32
 * operations. */
__global__ void __launch_bounds__(256) k_inpaint_scan(const float * img, const uint8_t * mask, int w, int h, int cn,
    int nf, int rows, float * out, float * dist)
{
  const int wid = (int) ((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  const int lines = rows ? h : w, len = rows ? w : h;
  if( wid >= lines * nf ) return;                       // the whole warp
  const int f = wid / lines, line = wid - f * lines;
  const size_t plane = (size_t) w * h;
  const size_t step = rows ? 1 : (size_t) w;
  const size_t base = rows ? (size_t) line * w : (size_t) line;
  const uint8_t * m = mask + (size_t) f * plane + base;
  const float * im = img + (size_t) f * cn * plane + base;
  float * o = out + (size_t) f * cn * plane + base;
  float * d = dist + (size_t) f * plane + base;
  const int chunk = (len + 31) / 32;
  const int c0 = min(lane * chunk, len), c1 = min(c0 + chunk, len);
  int lastv = -1, firstv = len;
  for( int x = c0; x < c1; ++x ) {
    if( m[(size_t) x * step] ) {
      if( firstv == len ) firstv = x;
      lastv = x;
    }
  }
  int pre = lastv, suf = firstv;
#pragma unroll
  for( int k = 1; k < 32; k <<= 1 ) {
    const int a = __shfl_up_sync(0xffffffffu, pre, k), b = __shfl_down_sync(0xffffffffu, suf, k);
    if( lane >= k ) pre = max(pre, a);
    if( lane + k < 32 ) suf = min(suf, b);
  }
  int before = __shfl_up_sync(0xffffffffu, pre, 1), after = __shfl_down_sync(0xffffffffu, suf, 1);
  if( lane == 0 ) before = -1;
  if( lane == 31 ) after = len;
  int s = before;                                       // the last valid position before x
  for( int x = c0; x < c1; ) {
    if( m[(size_t) x * step] ) {
      d[(size_t) x * step] = 0.f;
      s = x++;
      continue;
    }
    int pe = x + 1;
    while ( pe < c1 && !m[(size_t) pe * step] ) ++pe;
    const int e = pe < c1 ? pe : after;                 // the first valid position after the run
    if( s >= 0 && e < len ) {
      const float scale = __fdiv_rn(1.0f, (float) (e - s - 1));
      for( int q = x; q < pe; ++q ) {
        d[(size_t) q * step] = (float) max(q - s, e - q);
        for( int c = 0; c < cn; ++c ) {
          const float sv = im[c * plane + (size_t) s * step], ev = im[c * plane + (size_t) e * step];
          const float kk = __fmul_rn(__fsub_rn(ev, sv), scale);
          o[c * plane + (size_t) q * step] = __fadd_rn(sv, __fmul_rn((float) (q - s), kk));
        }
      }
    }
    else if( s >= 0 ) {
      for( int q = x; q < pe; ++q ) {
        d[(size_t) q * step] = (float) (q - s);
        for( int c = 0; c < cn; ++c ) o[c * plane + (size_t) q * step] = im[c * plane + (size_t) s * step];
      }
    }
    else if( e < len ) {
      for( int q = x; q < pe; ++q ) {
        d[(size_t) q * step] = (float) (e - q);
        for( int c = 0; c < cn; ++c ) o[c * plane + (size_t) q * step] = im[c * plane + (size_t) e * step];
      }
    }
    else {
      for( int q = x; q < pe; ++q ) d[(size_t) q * step] = 0.f;
    }
    x = pe;
  }
}

/* _fill_holes2: per hole, the row / column estimates weighted by the other
 * direction's distance; filled[f] counts the pixels filled in frame f */
__global__ void k_inpaint_fill(float * img, uint8_t * mask, const float * ih, const float * iv, const float * hd,
    const float * vd, int w, int h, int cn, int * filled)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int f = blockIdx.z;
  bool did = false;
  if( x < w && y < h ) {
    const size_t plane = (size_t) w * h, i = (size_t) y * w + x;
    uint8_t * m = mask + (size_t) f * plane + i;
    if( !*m ) {
      const float dh = hd[(size_t) f * plane + i], dv = vd[(size_t) f * plane + i];
      const size_t b = (size_t) f * cn * plane + i;
      if( dh > 0.f && dv > 0.f ) {
        const float dd = __fdiv_rn(1.0f, __fadd_rn(dh, dv));
        for( int c = 0; c < cn; ++c )
          img[b + c * plane] = __fmul_rn(dd, __fadd_rn(__fmul_rn(ih[b + c * plane], dv), __fmul_rn(iv[b + c * plane], dh)));
        did = true;
      }
      else if( dv > 0.f ) {
        for( int c = 0; c < cn; ++c ) img[b + c * plane] = iv[b + c * plane];
        did = true;
      }
      else if( dh > 0.f ) {
        for( int c = 0; c < cn; ++c ) img[b + c * plane] = ih[b + c * plane];
        did = true;
      }
      if( did ) *m = 255;
    }
  }
  const unsigned bal = __ballot_sync(0xffffffffu, did);
  if( (threadIdx.x & 31) == 0 && bal ) atomicAdd(filled + f, __popc(bal));
}

/* --- pyramids --- */

__global__ void k_sub(float * a, const float * b, size_t n)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i < n ) a[i] -= b[i];
}

__global__ void k_add(float * a, const float * b, size_t n)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i < n ) a[i] += b[i];
}

/* cv::pyrDown of u8 planes: [1 4 6 4 1]^2 / 256, REFLECT_101, rounded */
__global__ void k_pyrdown_u8(const uint8_t * src, int w, int h, uint8_t * dst, int dw, int dh)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= dw || y >= dh ) return;
  const uint8_t * s = src + (size_t) blockIdx.z * w * h;
  const int k[5] = { 1, 4, 6, 4, 1 };
  int acc = 0;
  for( int j = 0; j < 5; ++j ) {
    int yy = 2 * y - 2 + j;
    if( h == 1 ) yy = 0;
    else while ( yy < 0 || yy >= h ) yy = yy < 0 ? -yy : 2 * (h - 1) - yy;
    int r = 0;
    for( int i = 0; i < 5; ++i ) {
      int xx = 2 * x - 2 + i;
      if( w == 1 ) xx = 0;
      else while ( xx < 0 || xx >= w ) xx = xx < 0 ? -xx : 2 * (w - 1) - xx;
      r += k[i] * s[(size_t) yy * w + xx];
    }
    acc += k[j] * r;
  }
  dst[(size_t) blockIdx.z * dw * dh + (size_t) y * dw + x] = (uint8_t) ((acc + 128) >> 8);
}

/* lap[f][c] = 0 where the mask level of frame f is below 255 */
__global__ void k_apply_mask(float * lap, const uint8_t * m, size_t plane, int cn)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= plane ) return;
  const int f = blockIdx.y;
  if( m[(size_t) f * plane + i] < 255 )
    for( int c = 0; c < cn; ++c ) lap[((size_t) f * cn + c) * plane + i] = 0.f;
}

/* select_max_energy without smoothing: acc = frame where |frame| > |acc|, frames in order */
__global__ void k_fold_select(float * acc, const float * lap, size_t planes_per_frame, int nf)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= planes_per_frame ) return;
  float a = acc[i];
  for( int f = 0; f < nf; ++f ) {
    const float p = lap[(size_t) f * planes_per_frame + i];
    if( fabsf(p) > fabsf(a) ) a = p;
  }
  acc[i] = a;
}

/* select_max_energy with smoothed magnitudes: acc = frame where s1 > s0 */
__global__ void k_select_where(float * acc, const float * lap, const float * s0, const float * s1, size_t n)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i < n && s1[i] > s0[i] ) acc[i] = lap[i];
}

__global__ void k_abs(const float * a, float * b, size_t n)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i < n ) b[i] = fabsf(a[i]);
}

/* energy w of frame planes: lap^2 per channel (wcn == cn) or (sum_c lap)^2 (wcn == 1) */
__global__ void k_energy(const float * lap, float * w, size_t plane, int cn, int wcn)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= plane ) return;
  const int f = blockIdx.y;
  const float * l = lap + (size_t) f * cn * plane + i;
  float * o = w + (size_t) f * wcn * plane + i;
  if( wcn == cn ) {
    for( int c = 0; c < cn; ++c ) o[c * plane] = l[c * plane] * l[c * plane];
  }
  else {
    float s = 0.f;
    for( int c = 0; c < cn; ++c ) s += l[c * plane];
    o[0] = s * s;
  }
}

/* separable filter of planes with BORDER_REFLECT_101, + delta (rows pass then columns pass) */
__global__ void k_sep_rows(const float * src, float * dst, int w, int h, const float * g, int k)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const size_t b = (size_t) blockIdx.z * w * h + (size_t) y * w;
  const int r = k / 2;
  float s = 0.f;
  for( int i = 0; i < k; ++i ) {
    int xx = x - r + i;
    if( w == 1 ) xx = 0;
    else while ( xx < 0 || xx >= w ) xx = xx < 0 ? -xx : 2 * (w - 1) - xx;
    s = fmaf(g[i], src[b + xx], s);
  }
  dst[b + x] = s;
}

__global__ void k_sep_cols(const float * src, float * dst, int w, int h, const float * g, int k, float delta)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const size_t b = (size_t) blockIdx.z * w * h;
  const int r = k / 2;
  float s = 0.f;
  for( int j = 0; j < k; ++j ) {
    int yy = y - r + j;
    if( h == 1 ) yy = 0;
    else while ( yy < 0 || yy >= h ) yy = yy < 0 ? -yy : 2 * (h - 1) - yy;
    s = fmaf(g[j], src[b + (size_t) yy * w + x], s);
  }
  dst[b + (size_t) y * w + x] = s + delta;
}

/* weighted_average fold: lap *= w (broadcast when wcn == 1); acc += lap, wwp += w in frame order;
 * init: the first frame sets acc and wwp */
__global__ void k_fold_weighted(float * acc, float * wwp, const float * lap, const float * w, size_t plane, int cn,
    int wcn, int nf, int init)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= plane ) return;
  for( int c = 0; c < cn; ++c ) {
    float a = init ? 0.f : acc[(size_t) c * plane + i];
    for( int f = 0; f < nf; ++f ) {
      const float l = lap[((size_t) f * cn + c) * plane + i], ww = w[((size_t) f * wcn + (wcn == cn ? c : 0)) * plane + i];
      a = (init && f == 0) ? l * ww : a + l * ww;
    }
    acc[(size_t) c * plane + i] = a;
  }
  for( int c = 0; c < wcn; ++c ) {
    float s = init ? 0.f : wwp[(size_t) c * plane + i];
    for( int f = 0; f < nf; ++f ) {
      const float ww = w[((size_t) f * wcn + c) * plane + i];
      s = (init && f == 0) ? ww : s + ww;
    }
    wwp[(size_t) c * plane + i] = s;
  }
}

/* the sum over channels of population standard deviations of [cn][n] (FP64) */
__device__ double block_graystdev(const float * p, size_t n, int cn, double * red)
{
  double sv = 0;
  for( int c = 0; c < cn; ++c ) {
    const float * q = p + (size_t) c * n;
    double s = 0;
    for( size_t i = threadIdx.x; i < n; i += blockDim.x ) s += q[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for( int o = blockDim.x / 2; o > 0; o >>= 1 ) {
      if( (int) threadIdx.x < o ) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    const double mean = red[0] / (double) n;
    __syncthreads();
    double v = 0;
    for( size_t i = threadIdx.x; i < n; i += blockDim.x ) v += (q[i] - mean) * (q[i] - mean);
    red[threadIdx.x] = v;
    __syncthreads();
    for( int o = blockDim.x / 2; o > 0; o >>= 1 ) {
      if( (int) threadIdx.x < o ) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    sv += sqrt(red[0] / (double) n);
    __syncthreads();
  }
  return sv;
}

/* the top level: acc = acc a0 + frame a1 with a = stdev / (stdev0 + stdev1),
 * frames in order (one CTA of 256 threads); init: the first frame sets acc */
__global__ void __launch_bounds__(256) k_top_blend(float * acc, const float * top, size_t n, int cn, int nf, int init)
{
  __shared__ double red[256];
  const size_t pn = n * cn;
  int f0 = 0;
  if( init ) {
    for( size_t i = threadIdx.x; i < pn; i += blockDim.x ) acc[i] = top[i];
    __syncthreads();
    f0 = 1;
  }
  for( int f = f0; f < nf; ++f ) {
    const float * t = top + (size_t) f * pn;
    const double sv0 = block_graystdev(acc, n, cn, red), sv1 = block_graystdev(t, n, cn, red);
    const float a0 = (float) (sv0 / (sv0 + sv1)), a1 = (float) (sv1 / (sv0 + sv1));
    for( size_t i = threadIdx.x; i < pn; i += blockDim.x ) acc[i] = acc[i] * a0 + t[i] * a1;
    __syncthreads();
  }
}

/* lp = acc / wwp (broadcast when wcn == 1) */
__global__ void k_divide(const float * acc, const float * wwp, float * out, size_t plane, int cn, int wcn)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= plane ) return;
  for( int c = 0; c < cn; ++c )
    out[(size_t) c * plane + i] = acc[(size_t) c * plane + i] / wwp[(size_t) (wcn == cn ? c : 0) * plane + i];
}

}  // namespace fs
}  // namespace sst

using namespace sst::fs;

namespace {

int ffail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_FSCK(call)                                                                         \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return ffail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

dim3 g2(int w, int h, int z)
{
  return dim3((unsigned) ((w + 31) / 32), (unsigned) ((h + 7) / 8), (unsigned) z);
}

unsigned g1(size_t n)
{
  return (unsigned) ((n + 255) / 256);
}

/* linear_interpolation_inpaint of nf planar frames with their working masks,
 * in place; scratch holds 2 (cn + 1) planes per frame and nf counters */
int inpaint_batch(float * img, uint8_t * mask, int w, int h, int cn, int nf, float * scratch, int * counters,
    cudaStream_t st)
{
  const size_t plane = (size_t) w * h;
  float * ih = scratch, * iv = ih + (size_t) nf * cn * plane;
  float * hd = iv + (size_t) nf * cn * plane, * vd = hd + (size_t) nf * plane;
  std::vector<int> filled(nf);
  for( int it = 0; it < w * h + 1; ++it ) {
    SST_FSCK(cudaMemsetAsync(counters, 0, nf * sizeof(int), st));
    k_inpaint_scan<<<g1((size_t) h * nf * 32), 256, 0, st>>>(img, mask, w, h, cn, nf, 1, ih, hd);
    k_inpaint_scan<<<g1((size_t) w * nf * 32), 256, 0, st>>>(img, mask, w, h, cn, nf, 0, iv, vd);
    k_inpaint_fill<<<g2(w, h, nf), 256, 0, st>>>(img, mask, ih, iv, hd, vd, w, h, cn, counters);
    SST_FSCK(cudaGetLastError());
    sst_internal_count_launches(3);
    SST_FSCK(cudaMemcpyAsync(filled.data(), counters, nf * sizeof(int), cudaMemcpyDeviceToHost, st));
    SST_FSCK(cudaStreamSynchronize(st));
    int any = 0;
    for( int v : filled ) any += v;
    if( !any ) break;   // frames whose holes are all filled (or unreachable) stay unchanged
  }
  return SST_OK;
}

}  // namespace

extern "C" void sst_focus_stack_options_default(sst_focus_stack_options * o)
{
  if( !o ) return;
  o->fusing_policy = SST_FOCUS_SELECT_MAX_ENERGY;
  o->inpaint_mask_holes = 1;
  o->avgchannel = 1;
  o->kradius = 0;
  o->ksigma = 0;
}

struct sst_focus_stack {
  sst_focus_stack_options o;
  int w = 0, h = 0, cn = 0, L = 0, wcn = 1;
  int frames = 0;
  std::vector<int> lw, lh;
  std::vector<DevBuf> acc, wwp;
  std::vector<Resampler> down, up;   // level l -> l + 1, and l + 1 -> l
  DevBuf G;
  int gk = 0;
  DevBuf batch, lbuf, mbuf, wbuf, scratch, counters, tmp;
  void reset()
  {
    for( auto & b : acc ) b.release();
    for( auto & b : wwp ) b.release();
    for( auto & r : down ) r.release();
    for( auto & r : up ) r.release();
    acc.clear(), wwp.clear(), down.clear(), up.clear(), lw.clear(), lh.clear();
    batch.release(), lbuf.release(), mbuf.release(), wbuf.release(), scratch.release(), counters.release(), tmp.release();
    w = h = cn = L = 0;
    frames = 0;
  }
  ~sst_focus_stack()
  {
    reset();
    G.release();
  }
};

extern "C" int sst_focus_stack_create(sst_focus_stack ** out, const sst_focus_stack_options * opts)
{
  if( !out ) return ffail(SST_ERR_INVALID_ARG, "sst_focus_stack_create: out is NULL");
  sst_focus_stack_options o;
  if( opts ) o = *opts;
  else sst_focus_stack_options_default(&o);
  if( o.fusing_policy != SST_FOCUS_SELECT_MAX_ENERGY && o.fusing_policy != SST_FOCUS_WEIGHTED_AVERAGE )
    return ffail(SST_ERR_INVALID_ARG, "unknown fusing policy");
  if( o.kradius < 0 || o.kradius > 64 || !(o.ksigma >= 0) || o.ksigma > 100 )
    return ffail(SST_ERR_INVALID_ARG, "kradius in 0..64, ksigma in 0..100");
  sst_focus_stack * h = new (std::nothrow) sst_focus_stack();
  if( !h ) return ffail(SST_ERR_NOMEM, "out of host memory");
  h->o = o;
  // cv::getGaussianKernel(max(0, 2 kradius + 1), max(0, ksigma)); sigma <= 0 takes the
  // documented default 0.3 ((ksize - 1) / 2 - 1) + 0.8
  if( o.ksigma > 0 || o.kradius > 0 ) {
    const int k = 2 * o.kradius + 1;
    double sigma = o.ksigma > 0 ? o.ksigma : 0.3 * ((k - 1) * 0.5 - 1) + 0.8;
    std::vector<double> t(k);
    double sum = 0;
    for( int i = 0; i < k; ++i ) {
      const double x = i - (k - 1) * 0.5;
      t[i] = exp(-x * x / (2 * sigma * sigma));
      sum += t[i];
    }
    std::vector<float> g(k);
    for( int i = 0; i < k; ++i ) g[i] = (float) (t[i] / sum);
    if( h->G.ensure(k * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(h->G.p, g.data(), k * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ) {
      delete h;
      return ffail(SST_ERR_CUDA, "cannot upload the smoothing kernel");
    }
    h->gk = k;
  }
  *out = h;
  return SST_OK;
}

extern "C" int sst_focus_stack_destroy(sst_focus_stack * h)
{
  delete h;
  return SST_OK;
}

extern "C" int sst_focus_stack_clear(sst_focus_stack * h)
{
  if( !h ) return ffail(SST_ERR_INVALID_ARG, "NULL accumulator");
  h->reset();
  return SST_OK;
}

extern "C" int sst_focus_stack_accumulated_frames(const sst_focus_stack * h)
{
  return h ? h->frames : 0;
}

/* the smoothing kernel as created (n taps; k may be NULL to query n) */
extern "C" int sst_focus_stack_kernel(const sst_focus_stack * h, float * k, int * n)
{
  if( !h || !n ) return ffail(SST_ERR_INVALID_ARG, "NULL argument");
  *n = h->gk;
  if( k && h->gk ) SST_FSCK(cudaMemcpy(k, h->G.p, h->gk * sizeof(float), cudaMemcpyDeviceToHost));
  return SST_OK;
}

static int focus_plan(sst_focus_stack * a, int w, int h, int cn, cudaStream_t st)
{
  a->w = w, a->h = h, a->cn = cn;
  a->wcn = (a->o.avgchannel && cn > 1) ? 1 : cn;
  a->lw.assign(1, w), a->lh.assign(1, h);
  while ( true ) {   // build_laplacian_pyramid(image, lp, 8)
    const int nw = (a->lw.back() + 1) / 2, nh = (a->lh.back() + 1) / 2;
    if( std::min(nw, nh) <= 8 ) break;
    a->lw.push_back(nw), a->lh.push_back(nh);
  }
  a->L = (int) a->lw.size();
  a->acc.resize(a->L);
  a->wwp.resize(std::max(0, a->L - 1));
  a->down.resize(a->L - 1);
  a->up.resize(a->L - 1);
  for( int l = 0; l < a->L; ++l ) {
    SST_FSCK(a->acc[l].ensure((size_t) a->lw[l] * a->lh[l] * cn * sizeof(float)));
    if( l + 1 < a->L && a->o.fusing_policy == SST_FOCUS_WEIGHTED_AVERAGE )
      SST_FSCK(a->wwp[l].ensure((size_t) a->lw[l] * a->lh[l] * a->wcn * sizeof(float)));
  }
  for( int l = 0; l + 1 < a->L; ++l ) {
    SST_FSCK(a->down[l].upload(pyr_taps(a->lw[l], a->lw[l + 1]), pyr_taps(a->lh[l], a->lh[l + 1]), a->lw[l], a->lh[l],
        a->lw[l + 1], a->lh[l + 1], st));
    SST_FSCK(a->up[l].upload(pyrup_taps(a->lw[l + 1], a->lw[l]), pyrup_taps(a->lh[l + 1], a->lh[l]), a->lw[l + 1],
        a->lh[l + 1], a->lw[l], a->lh[l], st));
  }
  return SST_OK;
}

/* offsets of the levels of a batch pyramid of nb frames: level l holds nb x cn planes */
static size_t level_offset(const sst_focus_stack * a, int l, int nb, int planes_per_frame)
{
  size_t o = 0;
  for( int i = 0; i < l; ++i ) o += (size_t) a->lw[i] * a->lh[i] * nb * planes_per_frame;
  return o;
}

extern "C" int sst_focus_stack_add(sst_focus_stack * a, const void * frames, int depth, int n, int width, int height,
    int channels, size_t row_stride, size_t frame_stride, double scale, const uint8_t * masks, size_t mask_row_stride,
    size_t mask_frame_stride, int on_device, void * stream)
{
  if( !a || !frames ) return ffail(SST_ERR_INVALID_ARG, "sst_focus_stack_add: NULL argument");
  const int db = depth_bytes(depth);
  if( !db ) return ffail(SST_ERR_INVALID_ARG, "depth must be u8, u16 or f32");
  if( n < 1 || n > 65535 || width < 1 || height < 1 || channels < 1 || channels > 4 )
    return ffail(SST_ERR_INVALID_ARG, "n in 1..65535, width, height >= 1 and 1..4 channels");
  if( row_stride < (size_t) width * channels * db || (n > 1 && frame_stride < row_stride * height) ||
      (row_stride % db) || (frame_stride % db) )
    return ffail(SST_ERR_INVALID_ARG, "invalid or misaligned strides");
  if( masks && (mask_row_stride < (size_t) width || (n > 1 && mask_frame_stride < mask_row_stride * height)) )
    return ffail(SST_ERR_INVALID_ARG, "invalid mask strides");
  if( a->frames && (width != a->w || height != a->h) )
    return ffail(SST_ERR_INVALID_ARG, "input image size does not match the accumulated frames");
  if( a->frames && channels != a->cn ) return ffail(SST_ERR_INVALID_ARG, "number of channels does not match");
  cudaStream_t st = (cudaStream_t) stream;
  if( !a->frames ) {
    const int r = focus_plan(a, width, height, channels, st);
    if( r != SST_OK ) return r;
  }
  const int L = a->L, cn = channels, wcn = a->wcn;
  const size_t plane0 = (size_t) width * height;
  size_t pyr_px = 0;
  for( int l = 0; l < L; ++l ) pyr_px += (size_t) a->lw[l] * a->lh[l];
  // frames per batch: about 256 MB of pyramid
  const int cap = (int) std::max<size_t>(1, std::min<size_t>(64, ((size_t) 256 << 20) / (pyr_px * cn * 4 * 3)));
  const bool select = a->o.fusing_policy == SST_FOCUS_SELECT_MAX_ENERGY;
  const bool sequential_select = select && a->gk > 0;
  SST_FSCK(a->lbuf.ensure(pyr_px * cap * cn * sizeof(float)));   // Laplacian levels of the batch
  SST_FSCK(a->tmp.ensure(plane0 * cap * cn * sizeof(float)));     // pyrUp / filter scratch
  if( !select ) SST_FSCK(a->wbuf.ensure(pyr_px * cap * wcn * sizeof(float)));
  if( sequential_select ) SST_FSCK(a->wbuf.ensure(plane0 * cn * 4 * sizeof(float)));
  if( masks ) {
    SST_FSCK(a->mbuf.ensure(pyr_px * cap));
    SST_FSCK(a->counters.ensure(cap * sizeof(int)));
    if( a->o.inpaint_mask_holes ) SST_FSCK(a->scratch.ensure(plane0 * cap * 2 * (cn + 1) * sizeof(float)));
  }
  ScopedBuf hostf, hostm;
  for( int f0 = 0; f0 < n; f0 += cap ) {
    const int nb = std::min(cap, n - f0);
    // 1. planar FP32 level 0 (into the Laplacian buffer's level 0)
    const uint8_t * src = (const uint8_t *) frames + (size_t) f0 * frame_stride;
    if( !on_device ) {
      SST_FSCK(hostf.ensure(frame_stride * (nb - 1) + row_stride * height));
      SST_FSCK(cudaMemcpyAsync(hostf.p, src, frame_stride * (nb - 1) + row_stride * height, cudaMemcpyHostToDevice, st));
      src = hostf.as<uint8_t>();
    }
    float * lev0 = a->lbuf.as<float>();
    switch ( depth ) {
    case SST_DEPTH_U8:
      k_to_planar<uint8_t><<<g2(width, height, nb), 256, 0, st>>>(src, row_stride, frame_stride, width, height, cn,
          (float) scale, lev0);
      break;
    case SST_DEPTH_U16:
      k_to_planar<uint16_t><<<g2(width, height, nb), 256, 0, st>>>(src, row_stride, frame_stride, width, height, cn,
          (float) scale, lev0);
      break;
    default:
      k_to_planar<float><<<g2(width, height, nb), 256, 0, st>>>(src, row_stride, frame_stride, width, height, cn,
          (float) scale, lev0);
      break;
    }
    SST_FSCK(cudaGetLastError());
    sst_internal_count_launches(1);
    // masks: level 0 of the mask pyramid, packed
    uint8_t * m0 = nullptr;
    if( masks ) {
      m0 = a->mbuf.as<uint8_t>();
      for( int i = 0; i < nb; ++i ) {
        SST_FSCK(cudaMemcpy2DAsync(m0 + (size_t) i * plane0, width, masks + (size_t) (f0 + i) * mask_frame_stride,
            mask_row_stride, width, height, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
      }
      if( a->o.inpaint_mask_holes ) {
        // inpaint on a copy of the masks (the pyramid wants the original ones)
        SST_FSCK(hostm.ensure(plane0 * nb));
        SST_FSCK(cudaMemcpyAsync(hostm.p, m0, plane0 * nb, cudaMemcpyDeviceToDevice, st));
        const int r = inpaint_batch(lev0, hostm.as<uint8_t>(), width, height, cn, nb, a->scratch.as<float>(),
            a->counters.as<int>(), st);
        if( r != SST_OK ) return r;
      }
    }
    // 2. Laplacian pyramid of the batch: lbuf level l holds nb x cn planes
    for( int l = 0; l + 1 < L; ++l ) {
      float * cur = a->lbuf.as<float>() + level_offset(a, l, nb, cn);
      float * nxt = a->lbuf.as<float>() + level_offset(a, l + 1, nb, cn);
      const size_t pl = (size_t) a->lw[l] * a->lh[l], pn = (size_t) a->lw[l + 1] * a->lh[l + 1];
      SST_FSCK(a->down[l].run(cur, SST_DEPTH_F32, (size_t) a->lw[l] * 4, pl * 4, nb * cn, 1.0, nxt, pn, st));
      SST_FSCK(a->up[l].run(nxt, SST_DEPTH_F32, (size_t) a->lw[l + 1] * 4, pn * 4, nb * cn, 1.0, a->tmp.as<float>(), pl,
          st));
      k_sub<<<g1(pl * nb * cn), 256, 0, st>>>(cur, a->tmp.as<float>(), pl * nb * cn);
      SST_FSCK(cudaGetLastError());
      sst_internal_count_launches(1);
    }
    // 3. the mask pyramid zeroes the Laplacian levels below 255
    if( masks ) {
      size_t mo = 0;
      for( int l = 0; l + 1 < L; ++l ) {
        const size_t pl = (size_t) a->lw[l] * a->lh[l];
        uint8_t * ml = a->mbuf.as<uint8_t>() + mo;
        if( l > 0 ) {
          const uint8_t * mp = ml - (size_t) a->lw[l - 1] * a->lh[l - 1] * nb;
          k_pyrdown_u8<<<g2(a->lw[l], a->lh[l], nb), 256, 0, st>>>(mp, a->lw[l - 1], a->lh[l - 1], ml, a->lw[l],
              a->lh[l]);
          sst_internal_count_launches(1);
        }
        k_apply_mask<<<dim3(g1(pl), nb), 256, 0, st>>>(a->lbuf.as<float>() + level_offset(a, l, nb, cn), ml, pl, cn);
        SST_FSCK(cudaGetLastError());
        sst_internal_count_launches(1);
        mo += pl * nb;
      }
    }
    // 4. the fold, levels 0 .. L - 2
    const int init = a->frames == 0 && f0 == 0 ? 1 : 0;
    for( int l = 0; l + 1 < L; ++l ) {
      const size_t pl = (size_t) a->lw[l] * a->lh[l];
      float * lap = a->lbuf.as<float>() + level_offset(a, l, nb, cn);
      float * accl = a->acc[l].as<float>();
      if( select && !sequential_select ) {
        int fs = 0;
        if( init ) {
          SST_FSCK(cudaMemcpyAsync(accl, lap, pl * cn * sizeof(float), cudaMemcpyDeviceToDevice, st));
          fs = 1;
        }
        if( nb > fs ) {
          k_fold_select<<<g1(pl * cn), 256, 0, st>>>(accl, lap + (size_t) fs * pl * cn, pl * cn, nb - fs);
          sst_internal_count_launches(1);
        }
      }
      else if( select ) {
        float * s0 = a->wbuf.as<float>(), * s1 = s0 + pl * cn, * t = s1 + pl * cn, * u = t + pl * cn;
        for( int f = 0; f < nb; ++f ) {
          const float * lf = lap + (size_t) f * pl * cn;
          if( init && f == 0 ) {
            SST_FSCK(cudaMemcpyAsync(accl, lf, pl * cn * sizeof(float), cudaMemcpyDeviceToDevice, st));
            continue;
          }
          k_abs<<<g1(pl * cn), 256, 0, st>>>(accl, t, pl * cn);
          k_sep_rows<<<g2(a->lw[l], a->lh[l], cn), 256, 0, st>>>(t, u, a->lw[l], a->lh[l], a->G.as<float>(), a->gk);
          k_sep_cols<<<g2(a->lw[l], a->lh[l], cn), 256, 0, st>>>(u, s0, a->lw[l], a->lh[l], a->G.as<float>(), a->gk, 0.f);
          k_abs<<<g1(pl * cn), 256, 0, st>>>(lf, t, pl * cn);
          k_sep_rows<<<g2(a->lw[l], a->lh[l], cn), 256, 0, st>>>(t, u, a->lw[l], a->lh[l], a->G.as<float>(), a->gk);
          k_sep_cols<<<g2(a->lw[l], a->lh[l], cn), 256, 0, st>>>(u, s1, a->lw[l], a->lh[l], a->G.as<float>(), a->gk, 0.f);
          k_select_where<<<g1(pl * cn), 256, 0, st>>>(accl, lf, s0, s1, pl * cn);
          SST_FSCK(cudaGetLastError());
          sst_internal_count_launches(7);
        }
      }
      else {
        float * wl = a->wbuf.as<float>() + level_offset(a, l, nb, wcn);
        k_energy<<<dim3(g1(pl), nb), 256, 0, st>>>(lap, wl, pl, cn, wcn);
        sst_internal_count_launches(1);
        if( a->gk ) {
          k_sep_rows<<<g2(a->lw[l], a->lh[l], nb * wcn), 256, 0, st>>>(wl, a->tmp.as<float>(), a->lw[l], a->lh[l],
              a->G.as<float>(), a->gk);
          k_sep_cols<<<g2(a->lw[l], a->lh[l], nb * wcn), 256, 0, st>>>(a->tmp.as<float>(), wl, a->lw[l], a->lh[l],
              a->G.as<float>(), a->gk, 1e-12f);
          sst_internal_count_launches(2);
        }
        k_fold_weighted<<<g1(pl), 256, 0, st>>>(accl, a->wwp[l].as<float>(), lap, wl, pl, cn, wcn, nb, init);
        SST_FSCK(cudaGetLastError());
        sst_internal_count_launches(1);
      }
    }
    // 5. the top level, frame by frame
    {
      const size_t pt = (size_t) a->lw[L - 1] * a->lh[L - 1];
      k_top_blend<<<1, 256, 0, st>>>(a->acc[L - 1].as<float>(), a->lbuf.as<float>() + level_offset(a, L - 1, nb, cn),
          pt, cn, nb, init);
      SST_FSCK(cudaGetLastError());
      sst_internal_count_launches(1);
    }
    a->frames += nb;
  }
  if( !on_device ) SST_FSCK(cudaStreamSynchronize(st));
  return SST_OK;
}

extern "C" int sst_focus_stack_compute(sst_focus_stack * a, float * avg, size_t avg_row_stride, int on_device,
    void * stream)
{
  if( !a || !avg ) return ffail(SST_ERR_INVALID_ARG, "NULL argument");
  if( a->frames < 1 ) return ffail(SST_ERR_STATE, "no frames accumulated");
  const int L = a->L, cn = a->cn;
  if( avg_row_stride == 0 ) avg_row_stride = (size_t) a->w * cn * sizeof(float);
  if( avg_row_stride < (size_t) a->w * cn * sizeof(float) || (avg_row_stride & 3) )
    return ffail(SST_ERR_INVALID_ARG, "invalid stride");
  cudaStream_t st = (cudaStream_t) stream;
  // cur (level l, cn planes) in two ping-pong planes of the frame size
  ScopedBuf b0, b1, lev;
  const size_t plane0 = (size_t) a->w * a->h;
  SST_FSCK(b0.ensure(plane0 * cn * sizeof(float)));
  SST_FSCK(b1.ensure(plane0 * cn * sizeof(float)));
  SST_FSCK(lev.ensure(plane0 * cn * sizeof(float)));
  float * cur = b0.as<float>(), * nxt = b1.as<float>();
  const size_t pt = (size_t) a->lw[L - 1] * a->lh[L - 1];
  SST_FSCK(cudaMemcpyAsync(cur, a->acc[L - 1].p, pt * cn * sizeof(float), cudaMemcpyDeviceToDevice, st));
  for( int l = L - 2; l >= 0; --l ) {
    const size_t pl = (size_t) a->lw[l] * a->lh[l], pn = (size_t) a->lw[l + 1] * a->lh[l + 1];
    SST_FSCK(a->up[l].run(cur, SST_DEPTH_F32, (size_t) a->lw[l + 1] * 4, pn * 4, cn, 1.0, nxt, pl, st));
    const float * lp = a->acc[l].as<float>();
    if( a->o.fusing_policy == SST_FOCUS_WEIGHTED_AVERAGE ) {
      k_divide<<<g1(pl), 256, 0, st>>>(a->acc[l].as<float>(), a->wwp[l].as<float>(), lev.as<float>(), pl, cn, a->wcn);
      sst_internal_count_launches(1);
      lp = lev.as<float>();
    }
    k_add<<<g1(pl * cn), 256, 0, st>>>(nxt, lp, pl * cn);
    SST_FSCK(cudaGetLastError());
    sst_internal_count_launches(1);
    std::swap(cur, nxt);
  }
  ScopedBuf dout;
  float * out = avg;
  if( !on_device ) {
    SST_FSCK(dout.ensure(avg_row_stride * a->h));
    out = dout.as<float>();
  }
  k_to_interleaved<<<g2(a->w, a->h, 1), 256, 0, st>>>(cur, a->w, a->h, cn, out, avg_row_stride);
  SST_FSCK(cudaGetLastError());
  sst_internal_count_launches(1);
  if( !on_device ) {
    SST_FSCK(cudaMemcpyAsync(avg, out, avg_row_stride * a->h, cudaMemcpyDeviceToHost, st));
    SST_FSCK(cudaStreamSynchronize(st));
  }
  else SST_FSCK(cudaStreamSynchronize(st));   // the scratch planes are released on return
  return SST_OK;
}

/* linear_interpolation_inpaint(image, mask) of one interleaved FP32 image
 * (1..4 channels) in place */
extern "C" int sst_linear_interpolation_inpaint(float * image, size_t row_stride, int width, int height, int channels,
    const uint8_t * mask, size_t mask_stride, int on_device, void * stream)
{
  if( !image || !mask ) return ffail(SST_ERR_INVALID_ARG, "NULL argument");
  if( width < 1 || height < 1 || channels < 1 || channels > 4 ) return ffail(SST_ERR_INVALID_ARG, "invalid size");
  if( row_stride == 0 ) row_stride = (size_t) width * channels * 4;
  if( mask_stride == 0 ) mask_stride = (size_t) width;
  if( row_stride < (size_t) width * channels * 4 || (row_stride & 3) || mask_stride < (size_t) width )
    return ffail(SST_ERR_INVALID_ARG, "invalid strides");
  cudaStream_t st = (cudaStream_t) stream;
  const size_t plane = (size_t) width * height;
  ScopedBuf m, pl, scratch, cnt, dimg;
  const uint8_t * src = (const uint8_t *) image;
  if( !on_device ) {
    SST_FSCK(dimg.ensure(row_stride * height));
    SST_FSCK(cudaMemcpyAsync(dimg.p, image, row_stride * height, cudaMemcpyHostToDevice, st));
    src = dimg.as<uint8_t>();
  }
  SST_FSCK(pl.ensure(plane * channels * sizeof(float)));
  SST_FSCK(m.ensure(plane));
  SST_FSCK(scratch.ensure(plane * 2 * (channels + 1) * sizeof(float)));
  SST_FSCK(cnt.ensure(sizeof(int)));
  k_to_planar<float><<<g2(width, height, 1), 256, 0, st>>>(src, row_stride, 0, width, height, channels, 1.f,
      pl.as<float>());
  SST_FSCK(cudaMemcpy2DAsync(m.p, width, mask, mask_stride, width, height,
      on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  int r = inpaint_batch(pl.as<float>(), m.as<uint8_t>(), width, height, channels, 1, scratch.as<float>(), cnt.as<int>(),
      st);
  if( r != SST_OK ) return r;
  float * out = on_device ? image : dimg.as<float>();
  k_to_interleaved<<<g2(width, height, 1), 256, 0, st>>>(pl.as<float>(), width, height, channels, out, row_stride);
  SST_FSCK(cudaGetLastError());
  sst_internal_count_launches(2);
  if( !on_device ) SST_FSCK(cudaMemcpyAsync(image, out, row_stride * height, cudaMemcpyDeviceToHost, st));
  SST_FSCK(cudaStreamSynchronize(st));
  return SST_OK;
}
