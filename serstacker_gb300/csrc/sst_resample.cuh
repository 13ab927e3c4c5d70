/*
 * sst_resample.cuh -- separable resampling of batches of frames by host-built
 * tap tables (sst_taps.h): k_resample_taps reads u8 / u16 / f32 frames with
 * row and frame strides and writes packed f32 frames, one thread per output
 * pixel; Resampler owns one table pair on the device.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <utility>

#include "sst_host.h"
#include "sst_taps.h"

void sst_internal_count_launches(int n);   // sst_capi.cu

namespace sst {

template<typename T>
__device__ __forceinline__ float ldpx_rs(const uint8_t * base, size_t row_stride, int x, int y)
{
  return (float) __ldg((const T *) (base + (size_t) y * row_stride) + x);
}

/* dst(x, y) = vscale * sum_j wy_j sum_i wx_i src(ix_i, iy_j), one thread per
 * output pixel, grid.z = frame */
template<typename T>
__global__ void __launch_bounds__(256) k_resample_taps(const uint8_t * src, size_t src_row, size_t src_frame,
    float vscale, const int * __restrict__ ix, const float * __restrict__ wx, int KX, const int * __restrict__ iy,
    const float * __restrict__ wy, int KY, float * dst, int dw, int dh, size_t dst_frame)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= dw || y >= dh ) return;
  const uint8_t * s = src + (size_t) blockIdx.z * src_frame;
  float acc = 0.f;
  for( int j = 0; j < KY; ++j ) {
    const float b = __ldg(wy + (size_t) y * KY + j);
    if( b == 0.f ) continue;
    const int yy = __ldg(iy + (size_t) y * KY + j);
    float r = 0.f;
    for( int i = 0; i < KX; ++i ) {
      const float a = __ldg(wx + (size_t) x * KX + i);
      if( a != 0.f ) r = fmaf(a, ldpx_rs<T>(s, src_row, __ldg(ix + (size_t) x * KX + i), yy), r);
    }
    acc = fmaf(b, r, acc);
  }
  dst[(size_t) blockIdx.z * dst_frame + (size_t) y * dw + x] = acc * vscale;
}

}  // namespace sst

namespace {

/* one separable resampling: both axes' tables on the device */
struct Resampler {
  HostTaps hx, hy;
  DevBuf ix, wx, iy, wy;
  int sw = 0, sh = 0, dw = 0, dh = 0;

  cudaError_t upload(HostTaps tx, HostTaps ty, int sw_, int sh_, int dw_, int dh_, cudaStream_t st)
  {
    hx = std::move(tx), hy = std::move(ty);
    sw = sw_, sh = sh_, dw = dw_, dh = dh_;
    cudaError_t e;
    if( (e = ix.ensure(hx.idx.size() * sizeof(int))) != cudaSuccess ) return e;
    if( (e = wx.ensure(hx.w.size() * sizeof(float))) != cudaSuccess ) return e;
    if( (e = iy.ensure(hy.idx.size() * sizeof(int))) != cudaSuccess ) return e;
    if( (e = wy.ensure(hy.w.size() * sizeof(float))) != cudaSuccess ) return e;
    if( (e = cudaMemcpyAsync(ix.p, hx.idx.data(), hx.idx.size() * sizeof(int), cudaMemcpyHostToDevice, st)) ) return e;
    if( (e = cudaMemcpyAsync(wx.p, hx.w.data(), hx.w.size() * sizeof(float), cudaMemcpyHostToDevice, st)) ) return e;
    if( (e = cudaMemcpyAsync(iy.p, hy.idx.data(), hy.idx.size() * sizeof(int), cudaMemcpyHostToDevice, st)) ) return e;
    if( (e = cudaMemcpyAsync(wy.p, hy.w.data(), hy.w.size() * sizeof(float), cudaMemcpyHostToDevice, st)) ) return e;
    return cudaStreamSynchronize(st);   // the host tables may be released after this
  }

  cudaError_t run(const void * src, int depth, size_t src_row, size_t src_frame, int n, double vscale, float * dst,
      size_t dst_frame, cudaStream_t st) const
  {
    dim3 grid((dw + 31) / 32, (dh + 7) / 8, n);
    const uint8_t * s = (const uint8_t *) src;
#define SST_RS(T) sst::k_resample_taps<T><<<grid, 256, 0, st>>>(s, src_row, src_frame, (float) vscale, ix.as<int>(), \
    wx.as<float>(), hx.K, iy.as<int>(), wy.as<float>(), hy.K, dst, dw, dh, dst_frame)
    switch ( depth ) {
    case SST_DEPTH_U8: SST_RS(uint8_t); break;
    case SST_DEPTH_U16: SST_RS(uint16_t); break;
    case SST_DEPTH_F32: SST_RS(float); break;
    default: return cudaErrorInvalidValue;
    }
#undef SST_RS
    sst_internal_count_launches(1);
    return cudaGetLastError();
  }

  void release() { ix.release(), wx.release(), iy.release(), wy.release(); }
};

}  // namespace
