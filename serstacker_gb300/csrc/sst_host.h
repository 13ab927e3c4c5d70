/*
 * sst_host.h -- host-side helpers shared by the C ABI translation units:
 * device buffers, depth sizes, c_ecch's Gaussian kernel and level-count rules.
 */
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <algorithm>
#include "../../include/serstacker_gb300.h"

namespace {

/* a growable device allocation owned by an engine object */
struct DevBuf {
  void * p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t bytes)
  {
    if( bytes <= n && p ) return cudaSuccess;
    release();
    if( bytes == 0 ) bytes = 16;
    cudaError_t e = cudaMalloc(&p, bytes);
    if( e == cudaSuccess ) n = bytes;
    else p = nullptr;
    return e;
  }
  void release()
  {
    if( p ) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  template<class T> T * as() const { return (T *) p; }
};

/* a temporary device allocation released when it goes out of scope (cudaFree
 * waits for the work that may still use it) */
struct ScopedBuf : DevBuf {
  ScopedBuf() = default;
  ScopedBuf(const ScopedBuf &) = delete;
  ScopedBuf & operator=(const ScopedBuf &) = delete;
  ~ScopedBuf() { release(); }
};

inline int depth_bytes(int depth)
{
  switch ( depth ) {
  case SST_DEPTH_U8: return 1;
  case SST_DEPTH_U16: return 2;
  case SST_DEPTH_F32: return 4;
  }
  return 0;
}

/* getGaussianKernel(ksize, sigma > 0) with c_ecch's ksize rule (ecc2.cc:1001-1003) */
inline int gaussian_kernel(double sigma, float * k)
{
  const int n = std::max(3, 2 * ((int) (3 * sigma)) + 1);
  double t[64], sum = 0;
  for( int i = 0; i < n && i < 64; ++i ) {
    const double x = i - (n - 1) * 0.5;
    t[i] = exp(-0.5 * x * x / (sigma * sigma));
    sum += t[i];
  }
  for( int i = 0; i < n && i < 64; ++i ) k[i] = (float) (t[i] / sum);
  return n;
}

/* c_ecch::set_reference_image level-count rule (ecc2.cc:1009-1026) */
inline int ecch_num_levels(int w, int h, const sst_ecch_options & o)
{
  const int min_size = std::max(4, o.minimum_image_size);
  int tw = w, th = h, lv = 1;
  while ( lv < 32 ) {
    if( o.maxlevel >= 0 && lv >= std::max(0, o.maxlevel) ) break;
    const int nw = ((tw + 1) >> 1) & ~1, nh = ((th + 1) >> 1) & ~1;
    if( nw < min_size || nh < min_size ) break;
    tw = nw, th = nh, ++lv;
  }
  return lv;
}

}  // namespace
