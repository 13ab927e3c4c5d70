/*
 * sst_inpaint.cu -- the master frame's hole filling after stacking:
 * average_pyramid_inpaint (core/proc/inpaint/average_pyramid_inpaint.cc:
 * 18-126), which the stacking pipeline applies to the accumulated image and
 * its mask (c_image_stacking_pipeline.cc:763-767, max_levels 100).
 *
 * The reference recurses: at each level a 3 x 3 fill (box sums of image and
 * mask, REPLICATE; valid pixels keep their value, others with a non-zero mask
 * sum take the mean), a downstrike to the odd rows / columns (downstrike.cc:
 * 35-75), recursion while the smaller level still has holes, then an upject
 * of the filled smaller level to the odd positions (downstrike.cc:256-370)
 * and a second fill with the level's own pixels as the fallback.
 *
 * Here the recursion is unrolled into two passes over an explicit pyramid:
 *   down: per level, the fill evaluated only at the downstruck positions,
 *         with a flag per level "the new level's mask has a zero";
 *   the host reads the flags once and picks the level the recursion stops
 *         at (no holes left, a side of 1, or max_levels);
 *   up:   per level from there, the upject and the second fill in one kernel
 *         (the upjected mask marks every copied position, as upject_even's
 *         zmask does, whatever its value), the last one writing the output
 *         image and the output mask (x 255, rounded).
 * Every pixel is owned by one thread; the only atomics are the per-level
 * integer flags.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "sst_host.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

namespace sst {
namespace inp {

__device__ __forceinline__ int clampi(int v, int lo, int hi)
{
  return v < lo ? lo : (v > hi ? hi : v);
}

/* sets *flag when any in-range thread of the warp has `zero` */
__device__ __forceinline__ void flag_zero(bool zero, int * flag)
{
  const unsigned b = __ballot_sync(0xffffffffu, zero);
  if( (threadIdx.x & 31) == 0 && b ) atomicOr(flag, 1);
}

/* level 0: the image where the mask is set, else 0; the mask / 255 */
__global__ void __launch_bounds__(256) k_inp_init(const float * src, size_t src_stride, const uint8_t * mask,
    size_t mask_stride, int w, int h, float * I, float * M, int * flag)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const bool in = x < w && y < h;
  bool zero = false;
  if( in ) {
    const uint8_t m = mask[(size_t) y * mask_stride + x];
    const float v = *(const float *) ((const uint8_t *) src + (size_t) y * src_stride + (size_t) x * 4);
    I[(size_t) y * w + x] = m ? v : 0.f;
    M[(size_t) y * w + x] = (float) m / 255.f;
    zero = m == 0;
  }
  flag_zero(zero, flag);
}

/* the first fill of level (w x h) evaluated at the downstruck positions
 * (min(2x + 1, w - 1), min(2y + 1, h - 1)) of the next level (w2 x h2) */
__global__ void __launch_bounds__(256) k_inp_down(const float * I, const float * M, int w, int h, float * I2, float * M2,
    int w2, int h2, int * flag)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const bool in = x < w2 && y < h2;
  bool zero = false;
  if( in ) {
    const int sx = min(2 * x + 1, w - 1), sy = min(2 * y + 1, h - 1);
    const float m = M[(size_t) sy * w + sx];
    float vi, vm;
    if( m != 0.f ) {
      vi = I[(size_t) sy * w + sx], vm = 1.f;
    }
    else {
      float bi = 0.f, bm = 0.f;
      for( int j = -1; j <= 1; ++j ) {
        const size_t row = (size_t) clampi(sy + j, 0, h - 1) * w;
        for( int i = -1; i <= 1; ++i ) {
          const int xx = clampi(sx + i, 0, w - 1);
          bi += I[row + xx], bm += M[row + xx];
        }
      }
      if( bm != 0.f ) vi = bi / bm, vm = 1.f;
      else vi = bi, vm = bm;
    }
    I2[(size_t) y * w2 + x] = vi;
    M2[(size_t) y * w2 + x] = vm;
    zero = vm == 0.f;
  }
  flag_zero(zero, flag);
}

/* the upject of the filled next level (wn x hn) to this level's odd positions
 * and the second fill with this level's pixels (I, M) as the fallback; the
 * last level writes the output image and its mask (x 255, rounded) */
template<bool FINAL>
__global__ void __launch_bounds__(256) k_inp_up(const float * I, const float * M, int w, int h, const float * In, int wn,
    int hn, float * out, size_t out_stride, uint8_t * out_mask, size_t out_mask_stride)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const float m = M[(size_t) y * w + x];
  float v, vm;
  if( m != 0.f ) {
    v = I[(size_t) y * w + x], vm = 1.f;
  }
  else {
    float su = 0.f, sz = 0.f;
    for( int j = -1; j <= 1; ++j ) {
      const int yy = clampi(y + j, 0, h - 1);
      const int ny = (yy - 1) >> 1;
      const bool row_ok = (yy & 1) && ny < hn;
      for( int i = -1; i <= 1; ++i ) {
        const int xx = clampi(x + i, 0, w - 1);
        const int nx = (xx - 1) >> 1;
        if( row_ok && (xx & 1) && nx < wn ) su += In[(size_t) ny * wn + nx], sz += 1.f;
      }
    }
    if( sz != 0.f ) v = su / sz, vm = 1.f;
    else v = su, vm = 0.f;
  }
  if( FINAL ) {
    *(float *) ((uint8_t *) out + (size_t) y * out_stride + (size_t) x * 4) = v;
    out_mask[(size_t) y * out_mask_stride + x] = (uint8_t) fminf(fmaxf(rintf(vm * 255.f), 0.f), 255.f);
  }
  else {
    out[(size_t) y * w + x] = v;
  }
}

/* no recursion at all: the masked level-0 image and the mask (x 255, rounded) */
__global__ void __launch_bounds__(256) k_inp_level0(const float * I, const float * M, int w, int h, float * out,
    size_t out_stride, uint8_t * out_mask, size_t out_mask_stride)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  *(float *) ((uint8_t *) out + (size_t) y * out_stride + (size_t) x * 4) = I[(size_t) y * w + x];
  out_mask[(size_t) y * out_mask_stride + x] =
      (uint8_t) fminf(fmaxf(rintf(M[(size_t) y * w + x] * 255.f), 0.f), 255.f);
}

}  // namespace inp
}  // namespace sst

using namespace sst::inp;

namespace {

int ifail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_ICK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return ifail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

inline dim3 grid_of(int w, int h)
{
  return dim3((w + 31) / 32, (h + 7) / 8);
}

}  // namespace

extern "C" int sst_average_pyramid_inpaint(const float * src, size_t src_stride, const uint8_t * mask,
    size_t mask_stride, int width, int height, int max_levels, float * dst, size_t dst_stride, uint8_t * dst_mask,
    size_t dst_mask_stride, int on_device, void * stream)
{
  if( !src || !mask || !dst || !dst_mask ) return ifail(SST_ERR_INVALID_ARG, "sst_average_pyramid_inpaint: NULL argument");
  if( width < 1 || height < 1 ) return ifail(SST_ERR_INVALID_ARG, "width and height must be >= 1");
  if( width > 65535 * 32 || height > 65535 * 8 ) return ifail(SST_ERR_INVALID_ARG, "image too large");
  if( src_stride == 0 ) src_stride = (size_t) width * 4;
  if( mask_stride == 0 ) mask_stride = width;
  if( dst_stride == 0 ) dst_stride = (size_t) width * 4;
  if( dst_mask_stride == 0 ) dst_mask_stride = width;
  if( src_stride < (size_t) width * 4 || dst_stride < (size_t) width * 4 || mask_stride < (size_t) width ||
      dst_mask_stride < (size_t) width || (src_stride & 3) || (dst_stride & 3) )
    return ifail(SST_ERR_INVALID_ARG, "invalid strides");
  cudaStream_t st = (cudaStream_t) stream;
  // level sizes down to a side of 1
  std::vector<int> lw { width }, lh { height };
  while ( std::min(lw.back(), lh.back()) > 1 ) lw.push_back((lw.back() + 1) / 2), lh.push_back((lh.back() + 1) / 2);
  const int L = (int) lw.size();
  std::vector<size_t> off(L + 1, 0);
  for( int l = 0; l < L; ++l ) off[l + 1] = off[l] + (size_t) lw[l] * lh[l];
  ScopedBuf bI, bM, bO, bflag, bsrc, bmask, bdst, bdmask;
  SST_ICK(bI.ensure(off[L] * sizeof(float)));
  SST_ICK(bM.ensure(off[L] * sizeof(float)));
  SST_ICK(bO.ensure(off[L] * sizeof(float)));
  SST_ICK(bflag.ensure((size_t) L * sizeof(int)));
  const float * d_src = src;
  const uint8_t * d_mask = mask;
  float * d_dst = dst;
  uint8_t * d_dmask = dst_mask;
  size_t s_src = src_stride, s_mask = mask_stride, s_dst = dst_stride, s_dmask = dst_mask_stride;
  if( !on_device ) {
    SST_ICK(bsrc.ensure((size_t) width * height * 4));
    SST_ICK(bmask.ensure((size_t) width * height));
    SST_ICK(bdst.ensure((size_t) width * height * 4));
    SST_ICK(bdmask.ensure((size_t) width * height));
    SST_ICK(cudaMemcpy2DAsync(bsrc.p, (size_t) width * 4, src, src_stride, (size_t) width * 4, height,
        cudaMemcpyHostToDevice, st));
    SST_ICK(cudaMemcpy2DAsync(bmask.p, width, mask, mask_stride, width, height, cudaMemcpyHostToDevice, st));
    d_src = bsrc.as<float>(), d_mask = bmask.as<uint8_t>(), d_dst = bdst.as<float>(), d_dmask = bdmask.as<uint8_t>();
    s_src = (size_t) width * 4, s_mask = width, s_dst = (size_t) width * 4, s_dmask = width;
  }
  float * I = bI.as<float>();
  float * M = bM.as<float>();
  float * Ob = bO.as<float>();
  int * flag = bflag.as<int>();
  int launches = 0;
  SST_ICK(cudaMemsetAsync(flag, 0, (size_t) L * sizeof(int), st));
  k_inp_init<<<grid_of(width, height), 256, 0, st>>>(d_src, s_src, d_mask, s_mask, width, height, I, M, flag);
  SST_ICK(cudaGetLastError());
  ++launches;
  for( int l = 0; l + 1 < L; ++l ) {
    k_inp_down<<<grid_of(lw[l + 1], lh[l + 1]), 256, 0, st>>>(I + off[l], M + off[l], lw[l], lh[l], I + off[l + 1],
        M + off[l + 1], lw[l + 1], lh[l + 1], flag + l + 1);
    SST_ICK(cudaGetLastError());
    ++launches;
  }
  std::vector<int> hole(L);
  SST_ICK(cudaMemcpyAsync(hole.data(), flag, (size_t) L * sizeof(int), cudaMemcpyDeviceToHost, st));
  SST_ICK(cudaStreamSynchronize(st));
  if( !hole[0] ) {
    // no holes: the reference returns the image and the mask as they are
    SST_ICK(cudaMemcpy2DAsync(d_dst, s_dst, d_src, s_src, (size_t) width * 4, height, cudaMemcpyDeviceToDevice, st));
    SST_ICK(cudaMemcpy2DAsync(d_dmask, s_dmask, d_mask, s_mask, width, height, cudaMemcpyDeviceToDevice, st));
  }
  else {
    // the level the recursion stops at
    int leaf = 0, left = max_levels;
    while ( true ) {
      if( std::min(lw[leaf], lh[leaf]) <= 1 || left <= 0 ) break;
      ++leaf;
      if( !hole[leaf] ) break;
      --left;
    }
    if( leaf == 0 ) {
      k_inp_level0<<<grid_of(width, height), 256, 0, st>>>(I, M, width, height, d_dst, s_dst, d_dmask, s_dmask);
      SST_ICK(cudaGetLastError());
      ++launches;
    }
    for( int k = leaf - 1; k >= 0; --k ) {
      const float * In = (k + 1 == leaf) ? I + off[k + 1] : Ob + off[k + 1];
      if( k == 0 )
        k_inp_up<true><<<grid_of(lw[0], lh[0]), 256, 0, st>>>(I, M, lw[0], lh[0], In, lw[1], lh[1], d_dst, s_dst, d_dmask,
            s_dmask);
      else
        k_inp_up<false><<<grid_of(lw[k], lh[k]), 256, 0, st>>>(I + off[k], M + off[k], lw[k], lh[k], In, lw[k + 1],
            lh[k + 1], Ob + off[k], 0, nullptr, 0);
      SST_ICK(cudaGetLastError());
      ++launches;
    }
  }
  sst_internal_count_launches(launches);
  if( !on_device ) {
    SST_ICK(cudaMemcpy2DAsync(dst, dst_stride, d_dst, (size_t) width * 4, (size_t) width * 4, height,
        cudaMemcpyDeviceToHost, st));
    SST_ICK(cudaMemcpy2DAsync(dst_mask, dst_mask_stride, d_dmask, width, width, height, cudaMemcpyDeviceToHost, st));
  }
  SST_ICK(cudaStreamSynchronize(st));
  return SST_OK;
}
