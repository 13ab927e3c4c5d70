/*
 * sst_internal.cuh -- device-side building blocks shared by the sm_103a kernels.
 *
 * Warps are evaluated as displacements from the integer pixel position so
 * that FP32 keeps ~1e-6 px of sub-pixel precision on 4k-pixel frames:
 *   X = x + dX(x, y),  x0 = x + floor(dX),  fx = dX - floor(dX).
 *
 * Coefficient layout of one frame's warp (16 floats, see model_warp_coeffs()):
 * the translation is split into an integer part (c[12], c[13]) and the
 * remainder kept in the FP32 displacement, so the displacement stays below a
 * few pixels and keeps ~1e-7 px of precision.
 *   projective family (translation / euclidean / affine / homography):
 *     c = { a00-1, a01, a02-Ix, a10, a11-1, a12-Iy, a20, a21, 0,0,0,0, Ix, Iy }
 *     q = a20 x + a21 y,  w = 1 + q
 *     X = x + Ix + (c0 x + c1 y + c2 - q (x + Ix)) / w
 *     Y = y + Iy + (c3 x + c4 y + c5 - q (y + Iy)) / w
 *   quadratic family (semi-quadratic / quadratic):
 *     c = { a00-1, a01, a02-Ix, a03, a04, a05, a10, a11-1, a12-Iy, a13, a14, a15, Ix, Iy }
 *     X = x + Ix + c0 x + c1 y + c2 + c3 xy + c4 x^2 + c5 y^2  (same for Y)
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/serstacker_gb300.h"

#define SST_MAX_PARAMS 12
#define SST_STATE 16

namespace sst {

enum WarpFamily { FAM_AFFINE = 0, FAM_HOMOG = 1, FAM_QUAD = 2 };

__host__ __device__ inline int motion_family(int motion)
{
  switch ( motion ) {
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: return FAM_HOMOG;
  case SST_MOTION_SEMI_QUADRATIC:
  case SST_MOTION_QUADRATIC: return FAM_QUAD;
  default: return FAM_AFFINE;
  }
}

#define SST_NCOEF 16

/* displacement relative to (x + Ix, y + Iy) */
template<int FAM>
__device__ __forceinline__ void warp_disp(const float * __restrict__ c, float x, float y, float & dx, float & dy)
{
  if( FAM == FAM_AFFINE ) {
    dx = fmaf(c[0], x, fmaf(c[1], y, c[2]));
    dy = fmaf(c[3], x, fmaf(c[4], y, c[5]));
  }
  else if( FAM == FAM_HOMOG ) {
    const float q = fmaf(c[6], x, c[7] * y);       // a20 x + a21 y
    const float iw = __fdividef(1.0f, 1.0f + q);   // approximate reciprocal: w is near 1, <= 2 ulp
    const float nx = fmaf(c[0], x, fmaf(c[1], y, c[2])) - q * (x + c[12]);
    const float ny = fmaf(c[3], x, fmaf(c[4], y, c[5])) - q * (y + c[13]);
    dx = nx * iw;
    dy = ny * iw;
  }
  else {
    const float xy = x * y, xx = x * x, yy = y * y;
    dx = fmaf(c[0], x, fmaf(c[1], y, fmaf(c[3], xy, fmaf(c[4], xx, fmaf(c[5], yy, c[2])))));
    dy = fmaf(c[6], x, fmaf(c[7], y, fmaf(c[9], xy, fmaf(c[10], xx, fmaf(c[11], yy, c[8])))));
  }
}

/* sample position split into an integer base and a fraction */
struct spos {
  int x0, y0;
  float fx, fy;
};

__device__ __forceinline__ spos make_spos(int x, int y, float dx, float dy)
{
  const float ffx = floorf(fminf(fmaxf(dx, -1e8f), 1e8f)), ffy = floorf(fminf(fmaxf(dy, -1e8f), 1e8f));
  spos s;
  s.x0 = x + (int) ffx;
  s.y0 = y + (int) ffy;
  s.fx = dx - ffx;
  s.fy = dy - ffy;
  return s;
}

/* sample position of output pixel (x, y) under the frame's warp coefficients */
template<int FAM>
__device__ __forceinline__ spos warp_pos(const float * __restrict__ c, int x, int y)
{
  float dx, dy;
  warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
  return make_spos(x + (int) c[12], y + (int) c[13], dx, dy);
}

/* True when every bilinear tap of every output pixel of the rectangle
 * [x0, x1] x [y0, y1] lies inside a w x h source: the warp maps the
 * rectangle's corners to positions in [0, w-2] x [0, h-2] (with a small
 * margin). Exact for the projective family (the image of a rectangle is the
 * convex hull of its mapped corners when w > 0 on it); never used for the
 * quadratic family. Evaluated by lanes 0..3 and broadcast: warp-uniform, and
 * CTA-uniform when every warp tests the same rectangle. */
template<int FAM>
__device__ __forceinline__ bool rect_interior(const float * __restrict__ c, int x0, int y0, int x1, int y1, int w, int h)
{
  if( FAM == FAM_QUAD ) return false;
  const int lane = threadIdx.x & 31;
  bool ok = true;
  if( lane < 4 ) {
    const int x = (lane & 1) ? x1 : x0, y = (lane & 2) ? y1 : y0;
    float dx, dy;
    warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
    const float X = (float) (x + (int) c[12]) + dx, Y = (float) (y + (int) c[13]) + dy;
    ok = X >= 0.01f && X <= (float) (w - 2) - 0.01f && Y >= 0.01f && Y <= (float) (h - 2) - 0.01f;
    if( FAM == FAM_HOMOG ) ok = ok && (1.0f + fmaf(c[6], (float) x, c[7] * (float) y)) > 0.f;
  }
  return __all_sync(0xffffffffu, ok);
}

/* rect_interior's test for one output position (one thread): both bilinear
 * taps inside the w x h source with the 0.01 px margin, and w > 0 */
template<int FAM>
__device__ __forceinline__ bool point_interior(const float * __restrict__ c, int x, int y, int w, int h)
{
  if( FAM == FAM_QUAD ) return false;
  float dx, dy;
  warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
  const float X = (float) (x + (int) c[12]) + dx, Y = (float) (y + (int) c[13]) + dy;
  bool ok = X >= 0.01f && X <= (float) (w - 2) - 0.01f && Y >= 0.01f && Y <= (float) (h - 2) - 0.01f;
  if( FAM == FAM_HOMOG ) ok = ok && (1.0f + fmaf(c[6], (float) x, c[7] * (float) y)) > 0.f;
  return ok;
}

/* Source footprint of the rectangle [x0, x1] x [y0, y1]: whether every
 * bilinear tap is inside a w x h source (as rect_interior) and the integer
 * box [bx0, bx1] x [by0, by1] that holds every tap (0.01 px margin against
 * FP32 rounding of interior points). Warp-uniform results. */
template<int FAM>
__device__ __forceinline__ bool rect_footprint(const float * __restrict__ c, int x0, int y0, int x1, int y1, int w,
    int h, int & bx0, int & by0, int & bx1, int & by1)
{
  if( FAM == FAM_QUAD ) return false;
  const int lane = threadIdx.x & 31;
  float X = 0.f, Y = 0.f;
  bool ok = true;
  if( lane < 4 ) {
    const int x = (lane & 1) ? x1 : x0, y = (lane & 2) ? y1 : y0;
    float dx, dy;
    warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
    X = (float) (x + (int) c[12]) + dx, Y = (float) (y + (int) c[13]) + dy;
    ok = X >= 0.01f && X <= (float) (w - 2) - 0.01f && Y >= 0.01f && Y <= (float) (h - 2) - 0.01f;
    if( FAM == FAM_HOMOG ) ok = ok && (1.0f + fmaf(c[6], (float) x, c[7] * (float) y)) > 0.f;
  }
  ok = __all_sync(0xffffffffu, ok);
  float mnx = X, mxx = X, mny = Y, mxy = Y;
#pragma unroll
  for( int k = 1; k < 4; ++k ) {
    const float xs = __shfl_sync(0xffffffffu, X, k), ys = __shfl_sync(0xffffffffu, Y, k);
    mnx = fminf(mnx, xs), mxx = fmaxf(mxx, xs), mny = fminf(mny, ys), mxy = fmaxf(mxy, ys);
  }
  mnx = __shfl_sync(0xffffffffu, mnx, 0), mxx = __shfl_sync(0xffffffffu, mxx, 0);
  mny = __shfl_sync(0xffffffffu, mny, 0), mxy = __shfl_sync(0xffffffffu, mxy, 0);
  bx0 = (int) floorf(mnx - 0.01f), bx1 = (int) floorf(mxx + 0.01f) + 1;
  by0 = (int) floorf(mny - 0.01f), by1 = (int) floorf(mxy + 0.01f) + 1;
  return ok;
}

/* Bounding box of the mapped corners of [x0, x1] x [y0, y1] (0.01 px margin),
 * which holds every bilinear tap of the rectangle when the corners map to
 * finite positions with w > 0 (the return value), whether or not they lie
 * inside the w x h source; `inside` is rect_footprint's test (every tap
 * inside the source). Warp-uniform results. */
template<int FAM>
__device__ __forceinline__ bool rect_box(const float * __restrict__ c, int x0, int y0, int x1, int y1, int w, int h,
    int & bx0, int & by0, int & bx1, int & by1, bool & inside)
{
  inside = false;
  if( FAM == FAM_QUAD ) return false;
  const int lane = threadIdx.x & 31;
  float X = 0.f, Y = 0.f;
  bool ok = true, fin = true;
  if( lane < 4 ) {
    const int x = (lane & 1) ? x1 : x0, y = (lane & 2) ? y1 : y0;
    float dx, dy;
    warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
    X = (float) (x + (int) c[12]) + dx, Y = (float) (y + (int) c[13]) + dy;
    ok = X >= 0.01f && X <= (float) (w - 2) - 0.01f && Y >= 0.01f && Y <= (float) (h - 2) - 0.01f;
    fin = fabsf(X) < 1e6f && fabsf(Y) < 1e6f;
    if( FAM == FAM_HOMOG ) {
      const bool pos = (1.0f + fmaf(c[6], (float) x, c[7] * (float) y)) > 0.f;
      ok = ok && pos, fin = fin && pos;
    }
  }
  inside = __all_sync(0xffffffffu, ok);
  const bool boxable = __all_sync(0xffffffffu, fin);
  float mnx = X, mxx = X, mny = Y, mxy = Y;
#pragma unroll
  for( int k = 1; k < 4; ++k ) {
    const float xs = __shfl_sync(0xffffffffu, X, k), ys = __shfl_sync(0xffffffffu, Y, k);
    mnx = fminf(mnx, xs), mxx = fmaxf(mxx, xs), mny = fminf(mny, ys), mxy = fmaxf(mxy, ys);
  }
  mnx = __shfl_sync(0xffffffffu, mnx, 0), mxx = __shfl_sync(0xffffffffu, mxx, 0);
  mny = __shfl_sync(0xffffffffu, mny, 0), mxy = __shfl_sync(0xffffffffu, mxy, 0);
  if( boxable ) {
    bx0 = (int) floorf(mnx - 0.01f), bx1 = (int) floorf(mxx + 0.01f) + 1;
    by0 = (int) floorf(mny - 0.01f), by1 = (int) floorf(mxy + 0.01f) + 1;
  }
  else bx0 = by0 = bx1 = by1 = 0;
  return boxable;
}

/* nearest source pixel of output pixel (x, y) (cvRound of the map, INTER_NEAREST) */
template<int FAM>
__device__ __forceinline__ void warp_nearest(const float * __restrict__ c, int x, int y, int & rx, int & ry)
{
  float dx, dy;
  warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
  rx = x + (int) c[12] + __float2int_rn(dx);
  ry = y + (int) c[13] + __float2int_rn(dy);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi)
{
  return v < lo ? lo : (v > hi ? hi : v);
}

/* BORDER_REFLECT_101 index for any p (always inside [0, n)) */
__device__ __forceinline__ int reflect101(int p, int n)
{
  if( (unsigned) p < (unsigned) n ) return p;
  if( n == 1 ) return 0;
  const int period = 2 * (n - 1);
  p = clampi(p, -(1 << 29), 1 << 29);
  p = p < 0 ? -p : p;
  p = p % period;
  return p >= n ? period - p : p;
}

/* BORDER_REFLECT index for any p (always inside [0, n)) */
__device__ __forceinline__ int reflect(int p, int n)
{
  if( (unsigned) p < (unsigned) n ) return p;
  const int period = 2 * n;
  p = clampi(p, -(1 << 29), 1 << 29);
  p = p < 0 ? -p - 1 : p;
  p = p % period;
  return p >= n ? period - 1 - p : p;
}

/* bilinear sample of a f32 image, BORDER_REPLICATE (cv::remap semantics, exact weights) */
__device__ __forceinline__ float sample_replicate(const float * __restrict__ img, int w, int h, const spos & s)
{
  const int xa = clampi(s.x0, 0, w - 1), xb = clampi(s.x0 + 1, 0, w - 1);
  const int ya = clampi(s.y0, 0, h - 1), yb = clampi(s.y0 + 1, 0, h - 1);
  const float * ra = img + (size_t) ya * w;
  const float * rb = img + (size_t) yb * w;
  const float v00 = __ldg(ra + xa), v01 = __ldg(ra + xb);
  const float v10 = __ldg(rb + xa), v11 = __ldg(rb + xb);
  const float t0 = fmaf(s.fx, v01 - v00, v00);
  const float t1 = fmaf(s.fx, v11 - v10, v10);
  return fmaf(s.fy, t1 - t0, t0);
}

/* bilinear sample with BORDER_CONSTANT 0 */
__device__ __forceinline__ float sample_constant0(const float * __restrict__ img, int w, int h, const spos & s)
{
  const bool ix0 = s.x0 >= 0 && s.x0 < w, ix1 = s.x0 + 1 >= 0 && s.x0 + 1 < w;
  const bool iy0 = s.y0 >= 0 && s.y0 < h, iy1 = s.y0 + 1 >= 0 && s.y0 + 1 < h;
  const float v00 = (ix0 && iy0) ? __ldg(img + (size_t) s.y0 * w + s.x0) : 0.f;
  const float v01 = (ix1 && iy0) ? __ldg(img + (size_t) s.y0 * w + s.x0 + 1) : 0.f;
  const float v10 = (ix0 && iy1) ? __ldg(img + (size_t) (s.y0 + 1) * w + s.x0) : 0.f;
  const float v11 = (ix1 && iy1) ? __ldg(img + (size_t) (s.y0 + 1) * w + s.x0 + 1) : 0.f;
  const float t0 = fmaf(s.fx, v01 - v00, v00);
  const float t1 = fmaf(s.fx, v11 - v10, v10);
  return fmaf(s.fy, t1 - t0, t0);
}

/* LINEAR remap of an all-255 mask with BORDER_CONSTANT 0, divided by 255:
 * the bilinear weight that falls inside the image */
__device__ __forceinline__ float coverage(int w, int h, const spos & s)
{
  const bool ix0 = s.x0 >= 0 && s.x0 < w, ix1 = s.x0 + 1 >= 0 && s.x0 + 1 < w;
  const bool iy0 = s.y0 >= 0 && s.y0 < h, iy1 = s.y0 + 1 >= 0 && s.y0 + 1 < h;
  const float cx = (ix0 ? 1.0f - s.fx : 0.f) + (ix1 ? s.fx : 0.f);
  const float cy = (iy0 ? 1.0f - s.fy : 0.f) + (iy1 ? s.fy : 0.f);
  return cx * cy;
}

/* cv::compare(remapped_u8_mask, thr, CMP_GE) on round(255 * coverage) */
__device__ __forceinline__ bool mask_ok(float cov, int thr)
{
  return fmaf(255.0f, cov, 0.5f) >= (float) thr;
}

/* ---------------------------------------------------------------- reductions */

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
  for( int o = 16; o > 0; o >>= 1 ) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

/* Warp sums of NS values per lane, written to out[0 .. NS) by the lanes that
 * hold them. Each stage halves the vector: the lanes with the stage's lane bit
 * set keep the upper half and add their partner's upper half, the others the
 * lower half, so NS sums cost about NS + 5 shuffles instead of 5 NS. After
 * the halving stages lane L holds sum (L >> (5 - log2 N)) mod N (N = NS
 * rounded up to a power of two); the remaining lane bits are a plain butterfly. */
template<int NS>
__device__ __forceinline__ void warp_sums_to(const float (&v)[NS], float * out)
{
  constexpr int N = NS <= 1 ? 1 : NS <= 2 ? 2 : NS <= 4 ? 4 : NS <= 8 ? 8 : NS <= 16 ? 16 : 32;
  constexpr int LOGN = N == 1 ? 0 : N == 2 ? 1 : N == 4 ? 2 : N == 8 ? 3 : N == 16 ? 4 : 5;
  const int lane = threadIdx.x & 31;
  float w[N];
#pragma unroll
  for( int i = 0; i < N; ++i ) w[i] = i < NS ? v[i < NS ? i : 0] : 0.f;
#pragma unroll
  for( int t = 0; t < LOGN; ++t ) {
    const int H = N >> (t + 1), off = 16 >> t;
    const bool up = (lane & off) != 0;
#pragma unroll
    for( int i = 0; i < H; ++i ) {
      const float send = up ? w[i] : w[i + H];
      const float keep = up ? w[i + H] : w[i];
      w[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  float s = w[0];
#pragma unroll
  for( int off = 16 >> LOGN; off > 0; off >>= 1 ) s += __shfl_xor_sync(0xffffffffu, s, off);
  const int idx = (lane >> (5 - LOGN)) & (N - 1);
  if( (lane & ((32 >> LOGN) - 1)) == 0 && idx < NS ) out[idx] = s;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for( int o = 16; o > 0; o >>= 1 ) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

/* Block reduction of NS per-thread f32 sums into NS doubles (valid in out[] on
 * return for all threads). scratch: double[NWARPS * NS]. Fixed order: the
 * result does not depend on scheduling. */
template<int NS, int NT>
__device__ __forceinline__ void block_reduce(const float (&acc)[NS], double * scratch, double * out)
{
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for( int k = 0; k < NS; ++k ) {
    const float s = warp_sum(acc[k]);
    if( lane == 0 ) scratch[wid * NS + k] = (double) s;
  }
  __syncthreads();
  for( int k = threadIdx.x; k < NS; k += NT ) {
    double t = 0;
#pragma unroll
    for( int wv = 0; wv < NW; ++wv ) t += scratch[wv * NS + k];
    out[k] = t;
  }
  __syncthreads();
}

/* Kahan-Babuska (Neumaier) compensated add */
__device__ __forceinline__ void kahan_add(float & s, float & c, float v)
{
  const float t = s + v;
  if( fabsf(s) >= fabsf(v) ) c += (s - t) + v;
  else c += (v - t) + s;
  s = t;
}

}  // namespace sst
