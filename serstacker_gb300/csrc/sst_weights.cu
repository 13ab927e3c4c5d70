/*
 * sst_weights.cu -- local-variance sharpness maps as per-pixel stacking
 * weights, for batches of frames resident in HBM.
 *
 * compute_local_variance_map
 * (core/proc/sharpness_measure/c_local_variance_sharpness_measure.cc:193-249)
 * evaluated for n frames at once:
 *   1. pdownscale (:28-52): the frame, converted to scaled FP32, pyrDown'ed
 *      dscale times (5-tap, REFLECT_101), the first reduction straight from
 *      the raw frame;
 *   2. G = dilate - erode over the (2r+1)^2 square (cv::MORPH_GRADIENT,
 *      BORDER_REPLICATE) and P = ds^3 G^3 (_compute_sharpness_map,
 *      :131-165), with per-tile FP64 sums of G and G^4;
 *   3. per frame W = sum G, Q = ds^3 sum G^4 / W; W <= 0 means no map;
 *   4. INTER_AREA reduction of P by uscale halvings (dscaleSize, :15-25);
 *   5. + 0.05 Q and the INTER_LINEAR upscale to the frame's size
 *      (upscale_local_variance_map, :175-184).
 * Step 5 is never materialised for stacking: the stacking weight of an
 * output pixel is the map sampled bilinearly (BORDER_CONSTANT 0) at the
 * frame's warp of that pixel (c_image_stacking_pipeline.cc:1653-1658), and
 * each of its four taps evaluates the INTER_LINEAR upscale of the small map
 * on the fly.
 *
 * ds = 20, the CV_32F depth scale of the stacking pipeline's frames (which
 * it converts to scaled FP32 before weighting). The map is invariant under
 * value scale s with ds / s, so scale = 1 / maxval(depth) reproduces the
 * reference on an integer image up to its integer rounding of pyrDown.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "sst_engine.cuh"
#include "sst_host.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

namespace sst {
namespace lvm {

constexpr int LV_RMAX = 16;              // largest supported kernel radius
constexpr int DN_TX = 64, DN_TY = 16;    // reduction tile (output pixels)
constexpr int GR_TX = 64, GR_TY = 16;    // gradient tile

/* separable resampling taps along one axis: destination d reads the sources
 * idx[d K + k] with weights w[d K + k], k < K */
struct Taps {
  const int * idx;
  const float * w;
  int K;
};

/* INTER_LINEAR taps along one axis of the full-resolution grid: position p
 * reads small-map cells i0(p) and min(i0(p) + 1, m - 1) with weights
 * 1 - fr(p), fr(p). t[p + 1] = { i0(p), fr(p), i0(p + 1), fr(p + 1) } for
 * p = -1 ... full - 1 (a bilinear remap tap pair p, p + 1 in one load); the
 * entries outside the grid repeat the edge with zero fractions. */
struct LinTab {
  const float4 * t;
  int m;
};

template<typename T>
__device__ __forceinline__ float ld_raw(const uint8_t * fb, size_t rs, int x, int y)
{
  return (float) __ldg((const T *) (fb + (size_t) y * rs) + x);
}

/* first pyrDown straight from the raw frame: the frame converted to FP32
 * (x scale), 5-tap [1 4 6 4 1] / 16 rows first, REFLECT_101 */
template<typename T>
__global__ void __launch_bounds__(256) k_lv_down(const uint8_t * src, int sw, int sh, size_t rs, size_t fs, float scale,
    float * dst, int dw, int dh)
{
  constexpr int SW = 2 * DN_TX + 4, SH = 2 * DN_TY + 4;
  __shared__ float s_in[SH * SW];
  __shared__ float s_h[SH * DN_TX];
  const uint8_t * fb = src + (size_t) blockIdx.z * fs;
  float * out = dst + (size_t) blockIdx.z * dw * dh;
  const int tx0 = blockIdx.x * DN_TX, ty0 = blockIdx.y * DN_TY;
  const int sx0 = 2 * tx0 - 2, sy0 = 2 * ty0 - 2;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for( int yy = wid; yy < SH; yy += 8 ) {
    const int ry = reflect101(sy0 + yy, sh);
    for( int xx = lane; xx < SW; xx += 32 ) s_in[yy * SW + xx] = ld_raw<T>(fb, rs, reflect101(sx0 + xx, sw), ry) * scale;
  }
  __syncthreads();
  for( int yy = wid; yy < SH; yy += 8 ) {
#pragma unroll
    for( int k = 0; k < DN_TX / 32; ++k ) {
      const int xx = lane + 32 * k;
      const float * p = s_in + yy * SW + 2 * xx;
      s_h[yy * DN_TX + xx] = (p[0] + p[4]) * 0.0625f + (p[1] + p[3]) * 0.25f + p[2] * 0.375f;
    }
  }
  __syncthreads();
  for( int yy = wid; yy < DN_TY; yy += 8 ) {
    const int y = ty0 + yy;
    if( y >= dh ) break;
#pragma unroll
    for( int k = 0; k < DN_TX / 32; ++k ) {
      const int xx = lane + 32 * k, x = tx0 + xx;
      if( x < dw ) {
        const float * p = s_h + (2 * yy) * DN_TX + xx;
        out[(size_t) y * dw + x] = (p[0] + p[4 * DN_TX]) * 0.0625f + (p[DN_TX] + p[3 * DN_TX]) * 0.25f +
            p[2 * DN_TX] * 0.375f;
      }
    }
  }
}

/* tile sums of G and G^4 (FP64 across the warps) to part[2 tile] */
__device__ __forceinline__ void store_tile_sums(float sg, float sg4, double * part)
{
  __shared__ double s_red[2][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double a = sg, b = sg4;
#pragma unroll
  for( int o = 16; o > 0; o >>= 1 ) a += __shfl_xor_sync(0xffffffffu, a, o), b += __shfl_xor_sync(0xffffffffu, b, o);
  if( lane == 0 ) s_red[0][wid] = a, s_red[1][wid] = b;
  __syncthreads();
  if( threadIdx.x == 0 ) {
    double ta = 0, tb = 0;
    for( int i = 0; i < 8; ++i ) ta += s_red[0][i], tb += s_red[1][i];
    const size_t t = ((size_t) blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    part[2 * t] = ta, part[2 * t + 1] = tb;
  }
}

/* INTER_AREA reduction by whole fx x fy cells that tile a 64 x 16 tile
 * (fx | 64, fy | 16, the gradient's size a multiple of both): the tile
 * kernel writes the small map's cell means instead of P (fx = 0: P). */
struct AreaFuse {
  int fx, fy, mw, mh;
  float inv_area;
  float * small;
};

/* One 64 x 16 gradient tile with its radius-R halo (REPLICATE) for the
 * common radii, every staging load of a thread issued before its first use.
 * DOWN: the gradient's level is pyrDown of the raw frame (dscale 1): the raw
 * window under the clamped halo rows / columns (REFLECT_101 at the frame's
 * edges) is converted, reduced rows first, then columns, into the level
 * window. Otherwise the level window is read directly (the raw frame x scale
 * at dscale 0, or an FP32 pyramid level with scale 1). */
template<typename T, int R, bool DOWN>
__global__ void __launch_bounds__(256) k_lv_tile(const uint8_t * src, int sw, int sh, size_t rs, size_t fs, float scale,
    int gw, int gh, float ds3, float * p3, double * part, AreaFuse af)
{
  constexpr int LW = GR_TX + 2 * R, LH = GR_TY + 2 * R;                      // level window
  constexpr int RW = DOWN ? 2 * LW + 3 : LW, RH = DOWN ? 2 * LH + 3 : LH;    // staged source window
  constexpr int NS = RW * RH, PER = (NS + 255) / 256;
  constexpr int NH = DOWN ? RH * LW : 1, NL = DOWN ? LH * LW : 1, NM = DOWN ? 1 : 2 * LH * GR_TX;
  static_assert(!DOWN || NS >= 2 * LH * GR_TX, "the row extrema reuse the source window");
  static_assert((DOWN ? NH : NS) >= GR_TX * GR_TY, "the fused cells reuse a staging buffer");
  __shared__ __align__(16) float s_src[NS];
  __shared__ __align__(16) float s_h[NH];
  __shared__ __align__(16) float s_lvl[NL];
  __shared__ __align__(16) float s_m2[NM];
  const float * lvl = DOWN ? s_lvl : s_src;
  float * s_mx = DOWN ? s_src : s_m2;
  float * s_mn = s_mx + LH * GR_TX;
  float * s_p = DOWN ? s_h : s_src;          // the tile's P for the fused INTER_AREA cells (free by then)
  const uint8_t * fb = src + (size_t) blockIdx.z * fs;
  const int tx0 = blockIdx.x * GR_TX, ty0 = blockIdx.y * GR_TY;
  // first clamped level column / row of the window
  const int cx0 = max(tx0 - R, 0), cy0 = max(ty0 - R, 0);
  {
    // window origin in the source; a window inside the source needs no border rule
    const int ox = DOWN ? 2 * cx0 - 2 : tx0 - R, oy = DOWN ? 2 * cy0 - 2 : ty0 - R;
    const bool inside = ox >= 0 && oy >= 0 && ox + RW <= sw && oy + RH <= sh;
    const T * base = (const T *) (fb + (size_t) max(oy, 0) * rs) + max(ox, 0);
    float v[PER];
#pragma unroll
    for( int k = 0; k < PER; ++k ) {
      const int i = threadIdx.x + 256 * k;
      if( i < NS ) {
        const int yy = i / RW, xx = i - yy * RW;
        if( inside ) {
          v[k] = (float) __ldg((const T *) ((const uint8_t *) base + (size_t) yy * rs) + xx);
        }
        else {
          int sx, sy;
          if( DOWN ) sx = reflect101(ox + xx, sw), sy = reflect101(oy + yy, sh);
          else sx = clampi(ox + xx, 0, sw - 1), sy = clampi(oy + yy, 0, sh - 1);
          v[k] = (float) __ldg((const T *) (fb + (size_t) sy * rs) + sx);
        }
      }
    }
#pragma unroll
    for( int k = 0; k < PER; ++k ) {
      const int i = threadIdx.x + 256 * k;
      if( i < NS ) s_src[i] = v[k] * scale;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int NCL = (LW + 31) / 32;   // level-window columns per lane
  if( DOWN ) {
    // rows first: every staged row at the LW clamped level columns; the
    // lane's staged-column offsets are fixed over the rows
    int off[NCL];
#pragma unroll
    for( int k = 0; k < NCL; ++k ) off[k] = 2 * (clampi(tx0 - R + lane + 32 * k, 0, gw - 1) - cx0);
    for( int yy = wid; yy < RH; yy += 8 ) {
#pragma unroll
      for( int k = 0; k < NCL; ++k ) {
        const int c = lane + 32 * k;
        if( c < LW ) {
          const float * p = s_src + yy * RW + off[k];
          s_h[yy * LW + c] = (p[0] + p[4]) * 0.0625f + (p[1] + p[3]) * 0.25f + p[2] * 0.375f;
        }
      }
    }
    __syncthreads();
    for( int yy = wid; yy < LH; yy += 8 ) {
      const float * row = s_h + 2 * (clampi(ty0 - R + yy, 0, gh - 1) - cy0) * LW;
#pragma unroll
      for( int k = 0; k < NCL; ++k ) {
        const int c = lane + 32 * k;
        if( c < LW ) {
          const float * p = row + c;
          s_lvl[yy * LW + c] = (p[0] + p[4 * LW]) * 0.0625f + (p[LW] + p[3 * LW]) * 0.25f + p[2 * LW] * 0.375f;
        }
      }
    }
    __syncthreads();
  }
  // dilate / erode along rows over 2R + 1 columns
  for( int yy = wid; yy < LH; yy += 8 ) {
#pragma unroll
    for( int k = 0; k < GR_TX / 32; ++k ) {
      const int xx = lane + 32 * k;
      const float * p = lvl + yy * LW + xx;
      float mx = p[0], mn = p[0];
#pragma unroll
      for( int j = 1; j <= 2 * R; ++j ) mx = fmaxf(mx, p[j]), mn = fminf(mn, p[j]);
      s_mx[yy * GR_TX + xx] = mx, s_mn[yy * GR_TX + xx] = mn;
    }
  }
  __syncthreads();
  float sg = 0.f, sg4 = 0.f;
  float * out = p3 + (size_t) blockIdx.z * gw * gh;
#pragma unroll
  for( int r2 = 0; r2 < GR_TY / 8; ++r2 ) {
    const int yy = wid + 8 * r2, y = ty0 + yy;
#pragma unroll
    for( int k = 0; k < GR_TX / 32; ++k ) {
      const int xx = lane + 32 * k, x = tx0 + xx;
      if( y < gh && x < gw ) {
        float mx = s_mx[yy * GR_TX + xx], mn = s_mn[yy * GR_TX + xx];
#pragma unroll
        for( int j = 1; j <= 2 * R; ++j ) mx = fmaxf(mx, s_mx[(yy + j) * GR_TX + xx]), mn = fminf(mn, s_mn[(yy + j) * GR_TX + xx]);
        const float g = mx - mn;
        const float g3 = g * g * g;
        if( af.fx ) s_p[yy * GR_TX + xx] = g3 * ds3;
        else out[(size_t) y * gw + x] = g3 * ds3;
        sg += g;
        sg4 = fmaf(g3, g, sg4);
      }
    }
  }
  store_tile_sums(sg, sg4, part);   // ends with a barrier: s_p is complete
  if( af.fx ) {
    // cell sums along rows (into the free extrema buffer), then along columns
    const int ncx = GR_TX / af.fx, ncy = GR_TY / af.fy;
    float * s_q = s_mx;
    for( int i = threadIdx.x; i < GR_TY * ncx; i += 256 ) {
      const int yy = i / ncx, c = i - yy * ncx;
      const float * p = s_p + yy * GR_TX + c * af.fx;
      float a = 0.f;
      for( int j = 0; j < af.fx; ++j ) a += p[j];
      s_q[i] = a;
    }
    __syncthreads();
    for( int i = threadIdx.x; i < ncy * ncx; i += 256 ) {
      const int cy = i / ncx, c = i - cy * ncx;
      const int X = tx0 / af.fx + c, Y = ty0 / af.fy + cy;
      if( X < af.mw && Y < af.mh ) {
        float a = 0.f;
        for( int j = 0; j < af.fy; ++j ) a += s_q[(cy * af.fy + j) * ncx + c];
        af.small[(size_t) blockIdx.z * af.mw * af.mh + (size_t) Y * af.mw + X] = a * af.inv_area;
      }
    }
  }
}

/* Morphological gradient of one 64 x 16 tile: the window (tile + r on every
 * side, coordinates clamped) is staged in shared memory, row maxima / minima
 * over 2r + 1 columns, then column maxima / minima over 2r + 1 rows.
 * Writes P = ds^3 G^3 (G^3 then the scale, as the reference's float
 * expression) and the tile's FP64 sums of G and G^4 to part[2 tile]. */
__global__ void __launch_bounds__(256) k_lv_gradient(const float * src, int w, int h, int r, float ds3, float * p3,
    double * part)
{
  extern __shared__ float s_mem[];
  const int SW = GR_TX + 2 * r, SH = GR_TY + 2 * r;
  float * s_in = s_mem;
  float * s_mx = s_in + SH * SW;
  float * s_mn = s_mx + SH * GR_TX;
  const size_t plane = (size_t) w * h;
  const float * in = src + (size_t) blockIdx.z * plane;
  const int tx0 = blockIdx.x * GR_TX, ty0 = blockIdx.y * GR_TY;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for( int yy = wid; yy < SH; yy += 8 ) {
    const float * row = in + (size_t) clampi(ty0 - r + yy, 0, h - 1) * w;
    for( int xx = lane; xx < SW; xx += 32 ) s_in[yy * SW + xx] = __ldg(row + clampi(tx0 - r + xx, 0, w - 1));
  }
  __syncthreads();
  const int K = 2 * r + 1;
  for( int yy = wid; yy < SH; yy += 8 ) {
#pragma unroll
    for( int k = 0; k < GR_TX / 32; ++k ) {
      const int xx = lane + 32 * k;
      const float * p = s_in + yy * SW + xx;
      float mx = p[0], mn = p[0];
      for( int i = 1; i < K; ++i ) mx = fmaxf(mx, p[i]), mn = fminf(mn, p[i]);
      s_mx[yy * GR_TX + xx] = mx, s_mn[yy * GR_TX + xx] = mn;
    }
  }
  __syncthreads();
  float sg = 0.f, sg4 = 0.f;
  float * out = p3 + (size_t) blockIdx.z * plane;
  for( int yy = wid; yy < GR_TY; yy += 8 ) {
    const int y = ty0 + yy;
    if( y >= h ) break;
#pragma unroll
    for( int k = 0; k < GR_TX / 32; ++k ) {
      const int xx = lane + 32 * k, x = tx0 + xx;
      if( x < w ) {
        float mx = s_mx[yy * GR_TX + xx], mn = s_mn[yy * GR_TX + xx];
        for( int j = 1; j < K; ++j ) mx = fmaxf(mx, s_mx[(yy + j) * GR_TX + xx]), mn = fminf(mn, s_mn[(yy + j) * GR_TX + xx]);
        const float g = mx - mn;
        const float g3 = g * g * g;
        out[(size_t) y * w + x] = g3 * ds3;
        sg += g;
        sg4 = fmaf(g3, g, sg4);
      }
    }
  }
  store_tile_sums(sg, sg4, part);
}

/* per frame (one warp each, fixed summation order): W = sum G,
 * Q = ds^3 sum G^4 / W; frames with W <= 0 have no map */
__global__ void __launch_bounds__(256) k_lv_finish(const double * part, int tiles, int n, double ds3, double * q,
    float * addq, int * has)
{
  const int f = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if( f >= n ) return;
  const double * p = part + (size_t) f * tiles * 2;
  double a = 0, b = 0;
  for( int t = lane; t < tiles; t += 32 ) a += p[2 * t], b += p[2 * t + 1];
#pragma unroll
  for( int o = 16; o > 0; o >>= 1 ) a += __shfl_xor_sync(0xffffffffu, a, o), b += __shfl_xor_sync(0xffffffffu, b, o);
  if( lane == 0 ) {
    const bool ok = a > 0;
    const double Q = ok ? ds3 * b / a : 0.0;
    q[f] = Q;
    addq[f] = (float) (0.05 * Q);
    has[f] = ok ? 1 : 0;
  }
}

/* INTER_AREA reduction of every frame's map (separable taps); grid.z = frame */
__global__ void __launch_bounds__(256) k_lv_area(const float * src, int sw, int sh, float * dst, int dw, int dh,
    Taps tx, Taps ty)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= dw || y >= dh ) return;
  const float * s = src + (size_t) blockIdx.z * sw * sh;
  float acc = 0.f;
#pragma unroll 2
  for( int j = 0; j < ty.K; ++j ) {
    const float wy = __ldg(ty.w + y * ty.K + j);
    const float * row = s + (size_t) __ldg(ty.idx + y * ty.K + j) * sw;
    float r = 0.f;
#pragma unroll 4
    for( int i = 0; i < tx.K; ++i ) r = fmaf(__ldg(tx.w + x * tx.K + i), __ldg(row + __ldg(tx.idx + x * tx.K + i)), r);
    acc = fmaf(wy, r, acc);
  }
  dst[(size_t) blockIdx.z * dw * dh + (size_t) y * dw + x] = acc;
}

/* the full-resolution map at source pixel (px, py): the INTER_LINEAR upscale
 * of the small map plus 0.05 Q */
__device__ __forceinline__ float lv_at(const float * sm, LinTab ux, LinTab uy, float addq, int px, int py)
{
  const float4 ty = __ldg(uy.t + py + 1), tx = __ldg(ux.t + px + 1);
  const int y0 = (int) ty.x, y1 = min(y0 + 1, uy.m - 1), x0 = (int) tx.x, x1 = min(x0 + 1, ux.m - 1);
  const float * r0 = sm + (size_t) y0 * ux.m;
  const float * r1 = sm + (size_t) y1 * ux.m;
  const float t0 = (1.f - tx.y) * __ldg(r0 + x0) + tx.y * __ldg(r0 + x1);
  const float t1 = (1.f - tx.y) * __ldg(r1 + x0) + tx.y * __ldg(r1 + x1);
  return (1.f - ty.y) * t0 + ty.y * t1 + addq;
}

/* source-grid maps (w x h per frame); frames without a map are zero */
__global__ void __launch_bounds__(256) k_lv_expand(const float * small, LinTab ux, LinTab uy, const float * addq,
    const int * has, int w, int h, float * out)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const int f = blockIdx.z;
  const float * sm = small + (size_t) f * ux.m * uy.m;
  out[(size_t) f * w * h + (size_t) y * w + x] = __ldg(has + f) ? lv_at(sm, ux, uy, __ldg(addq + f), x, y) : 0.f;
}

/* Weights of the small-map cells c, c + 1, c + 2 (c = i0 of the first
 * position, cells clamped to the map) for the bilinear remap tap pair p, p + 1
 * with weights b0, b1 (zero outside the grid) composed with the INTER_LINEAR
 * upscale: tap p spreads over cells i0(p), i0(p) + 1, tap p + 1 over
 * i0(p + 1) = i0(p) + d (d = 0 or 1, the upscale never skips a cell). */
__device__ __forceinline__ void lin_pair(float4 t, float b0, float b1, float & w0, float & w1, float & w2)
{
  const bool same = t.z == t.x;
  const float a0 = b0 * (1.f - t.y), a1 = b0 * t.y, c0 = b1 * (1.f - t.w), c1 = b1 * t.w;
  w0 = same ? a0 + c0 : a0;
  w1 = same ? a1 + c1 : a1 + c0;
  w2 = same ? 0.f : c1;
}

/* output-grid stacking weights: the source-grid map sampled bilinearly at the
 * frame's warp of each output pixel, zero outside the frame
 * (BORDER_CONSTANT); a frame without a map weighs 1 everywhere. The
 * composition bilinear(remap) o bilinear(upscale) is separable: per axis the
 * two remap taps give weights over three consecutive small-map cells. */
constexpr int WP_ROWS = 4;   // output rows per thread of the warp-weight kernel (32 x 32 tiles)

template<int FAM>
__global__ void __launch_bounds__(256) k_lv_warp(const float * small, LinTab ux, LinTab uy, const float * addq,
    const int * has, const float * coeffs, int w, int h, int dw, int dh, float * out)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), yb = blockIdx.y * (8 * WP_ROWS) + (threadIdx.x >> 5);
  if( x >= dw || yb >= dh ) return;
  const int f = blockIdx.z;
  // the frame's flag, 0.05 Q and warp coefficients in one round of loads
  const int hf = __ldg(has + f);
  const float aq = __ldg(addq + f);
  float c[SST_NCOEF];
  const float4 * c4 = reinterpret_cast<const float4 *>(coeffs + (size_t) f * SST_NCOEF);
#pragma unroll
  for( int i = 0; i < SST_NCOEF / 4; ++i ) {
    const float4 v = __ldg(c4 + i);
    c[4 * i] = v.x, c[4 * i + 1] = v.y, c[4 * i + 2] = v.z, c[4 * i + 3] = v.w;
  }
  float * o = out + (size_t) f * dw * dh + x;
  const float * sm = small + (size_t) f * ux.m * uy.m;
  const int m = ux.m;
#pragma unroll
  for( int k = 0; k < WP_ROWS; ++k ) {
    const int y = min(yb + 8 * k, dh - 1);   // rows past the grid recompute the last one, unstored
    float res = 1.f;
    if( hf ) {
      res = 0.f;
      const spos s = warp_pos<FAM>(c, x, y);
      if( s.x0 >= -1 && s.x0 <= w - 1 && s.y0 >= -1 && s.y0 <= h - 1 ) {
        const float bx0 = s.x0 >= 0 ? 1.f - s.fx : 0.f, bx1 = s.x0 + 1 <= w - 1 ? s.fx : 0.f;
        const float by0 = s.y0 >= 0 ? 1.f - s.fy : 0.f, by1 = s.y0 + 1 <= h - 1 ? s.fy : 0.f;
        const float4 tx = __ldg(ux.t + s.x0 + 1), ty = __ldg(uy.t + s.y0 + 1);
        float wx0, wx1, wx2, wy0, wy1, wy2;
        lin_pair(tx, bx0, bx1, wx0, wx1, wx2);
        lin_pair(ty, by0, by1, wy0, wy1, wy2);
        const int cx = (int) tx.x, cx1 = min(cx + 1, m - 1), cx2 = min(cx + 2, m - 1);
        const int ry = (int) ty.x, ry1 = min(ry + 1, uy.m - 1), ry2 = min(ry + 2, uy.m - 1);
        auto row = [&](int r) {
          const float * p = sm + (size_t) r * m;
          float v = wx0 * __ldg(p + cx) + wx1 * __ldg(p + cx1);
          if( wx2 != 0.f ) v = fmaf(wx2, __ldg(p + cx2), v);
          return v;
        };
        float v = wy0 * row(ry) + wy1 * row(ry1);
        if( wy2 != 0.f ) v = fmaf(wy2, row(ry2), v);
        res = fmaf(aq, (bx0 + bx1) * (by0 + by1), v);
      }
    }
    if( yb + 8 * k < dh ) o[(size_t) y * dw] = res;
  }
}

}  // namespace lvm
}  // namespace sst

/* --------------------------------------------------------------- host side */

using namespace sst;
using namespace sst::lvm;

namespace {

/* INTER_AREA taps (OpenCV's area geometry): destination d averages source
 * [d s, (d + 1) s), s = ssize / dsize; partial cells below 1e-3 of a pixel at
 * either end are dropped */
void area_axis(int ssize, int dsize, std::vector<int> & idx, std::vector<float> & wt, int & K)
{
  std::vector<std::vector<std::pair<int, double>>> t(dsize);
  const double scale = (double) ssize / dsize;
  size_t k = 1;
  for( int d = 0; d < dsize; ++d ) {
    const double f1 = d * scale, f2 = f1 + scale;
    const double cell = std::min(scale, ssize - f1);
    const int s1 = (int) ceil(f1), s2 = std::min((int) floor(f2), ssize);
    if( s1 - f1 > 1e-3 && s1 - 1 >= 0 ) t[d].push_back({ s1 - 1, (s1 - f1) / cell });
    for( int s = s1; s < s2; ++s ) t[d].push_back({ s, 1.0 / cell });
    if( s2 < ssize && f2 - s2 > 1e-3 ) t[d].push_back({ s2, std::min(std::min(f2 - s2, 1.0), cell) / cell });
    k = std::max(k, t[d].size());
  }
  K = (int) k;
  idx.assign((size_t) dsize * K, 0);
  wt.assign((size_t) dsize * K, 0.f);
  for( int d = 0; d < dsize; ++d )
    for( size_t j = 0; j < t[d].size(); ++j ) idx[(size_t) d * K + j] = t[d][j].first, wt[(size_t) d * K + j] = (float) t[d][j].second;
}

/* INTER_LINEAR geometry: destination d samples f = (d + 0.5) ssize / dsize - 0.5,
 * clamped to the first / last source with a zero fraction; packed as the
 * LinTab pairs { i0(p), fr(p), i0(p + 1), fr(p + 1) }, p = -1 ... dsize - 1 */
std::vector<float4> linear_axis(int ssize, int dsize)
{
  std::vector<float> i0(dsize + 2), fr(dsize + 2, 0.f);
  const double s = (double) ssize / dsize;
  for( int d = 0; d < dsize; ++d ) {
    const double f = (d + 0.5) * s - 0.5;
    int si = (int) floor(f);
    double a = f - si;
    if( si < 0 ) si = 0, a = 0;
    if( si >= ssize - 1 ) si = ssize - 1, a = 0;
    i0[d + 1] = (float) si, fr[d + 1] = (float) a;
  }
  i0[0] = i0[1], i0[dsize + 1] = i0[dsize];   // outside the grid: the edge cell, zero fraction
  std::vector<float4> t(dsize + 1);
  for( int p = -1; p < dsize; ++p ) t[p + 1] = make_float4(i0[p + 1], fr[p + 1], i0[p + 2], fr[p + 2]);
  return t;
}

/* dscaleSize (c_local_variance_sharpness_measure.cc:15-25) */
void halved_size(int w, int h, int levels, int & ow, int & oh)
{
  for( int l = 0; l < levels; ++l ) {
    const int nw = (w + 1) / 2, nh = (h + 1) / 2;
    if( std::min(nw, nh) < 4 ) break;
    w = nw, h = nh;
  }
  ow = w, oh = h;
}

int lfail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_LCK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return lfail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

#define SST_TRY_L(expr)                                                                        \
  do {                                                                                         \
    int r_ = (expr);                                                                           \
    if( r_ != SST_OK ) return r_;                                                              \
  } while ( 0 )

#define SST_LLAUNCH(call)                                                                      \
  do {                                                                                         \
    SST_LCK(call);                                                                             \
    sst_internal_count_launches(1);                                                            \
  } while ( 0 )

template<class T>
cudaError_t upload(DevBuf & b, const std::vector<T> & v, cudaStream_t st)
{
  cudaError_t e = b.ensure(v.size() * sizeof(T));
  if( e != cudaSuccess ) return e;
  return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

}  // namespace

struct sst_local_variance {
  sst_local_variance_options o;
  // geometry of the last batch: frame, reduced level (gw x gh, after nlev
  // pyrDowns) and small map (mw x mh)
  int w = 0, h = 0, gw = 0, gh = 0, nlev = 0, mw = 0, mh = 0, tiles = 0;
  int n = 0;                              // frames of the last batch
  bool area_fused = false;                // the last batch's INTER_AREA cells came from the tile kernel
  DevBuf lv[2], p3, small, part, q, addq, has, stage, maps;
  DevBuf ax_i, ax_w, ay_i, ay_w;          // INTER_AREA taps (gradient grid -> small map)
  DevBuf ux, uy;                          // INTER_LINEAR tap pairs (small map -> frame grid)
  int ax_k = 0, ay_k = 0;
  int tab_key[6] = { -1, -1, -1, -1, -1, -1 };   // w, h, gw, gh, mw, mh of the uploaded tap tables
  ~sst_local_variance()
  {
    for( DevBuf * b : { &lv[0], &lv[1], &p3, &small, &part, &q, &addq, &has, &stage, &maps, &ax_i, &ax_w, &ay_i, &ay_w,
             &ux, &uy } )
      b->release();
  }
  const float * small_map() const { return (mw == gw && mh == gh) ? p3.as<float>() : small.as<float>(); }
  LinTab lx() const { return LinTab { ux.as<float4>(), mw }; }
  LinTab ly() const { return LinTab { uy.as<float4>(), mh }; }
};

namespace {

/* geometry of compute_local_variance_map for a w x h frame */
void lv_geometry(sst_local_variance * L, int w, int h)
{
  const int ds = std::max(0, L->o.dscale), us = std::max(0, L->o.uscale);
  int gw = w, gh = h, nlev = 0;
  if( ds > 0 && std::min(w, h) >= 4 ) {
    for( int l = 0; l < ds; ++l ) {
      gw = (gw + 1) / 2, gh = (gh + 1) / 2, ++nlev;
      if( std::min(gw, gh) < 4 ) break;
    }
  }
  int mw = gw, mh = gh;
  if( us > 0 ) halved_size(gw, gh, us, mw, mh);
  L->w = w, L->h = h, L->gw = gw, L->gh = gh, L->nlev = nlev, L->mw = mw, L->mh = mh;
  L->tiles = ((gw + GR_TX - 1) / GR_TX) * ((gh + GR_TY - 1) / GR_TY);
}

int lv_tables(sst_local_variance * L, cudaStream_t st)
{
  const int key[6] = { L->w, L->h, L->gw, L->gh, L->mw, L->mh };
  if( !memcmp(key, L->tab_key, sizeof(key)) ) return SST_OK;
  std::vector<int> i;
  std::vector<float> f;
  if( L->mw != L->gw || L->mh != L->gh ) {
    area_axis(L->gw, L->mw, i, f, L->ax_k);
    SST_LCK(upload(L->ax_i, i, st));
    SST_LCK(upload(L->ax_w, f, st));
    area_axis(L->gh, L->mh, i, f, L->ay_k);
    SST_LCK(upload(L->ay_i, i, st));
    SST_LCK(upload(L->ay_w, f, st));
  }
  const std::vector<float4> tx = linear_axis(L->mw, L->w), ty = linear_axis(L->mh, L->h);
  SST_LCK(upload(L->ux, tx, st));
  SST_LCK(upload(L->uy, ty, st));
  // pageable sources: the copies have read them when the stream reaches here
  SST_LCK(cudaStreamSynchronize(st));
  memcpy(L->tab_key, key, sizeof(key));
  return SST_OK;
}

}  // namespace

/* Steps 1-4 for n device frames: small maps, Q, and the has-map flags. */
int sst_internal_lv_build(sst_local_variance * L, const void * d_frames, int depth, int n, int w, int h,
    size_t row_stride, size_t frame_stride, double scale, cudaStream_t st)
{
  const int r = std::max(1, L->o.kradius);
  if( r > LV_RMAX ) return lfail(SST_ERR_UNSUPPORTED, "local variance map: kradius above 16 is not supported");
  if( n > 65535 ) return lfail(SST_ERR_INVALID_ARG, "local variance map: at most 65535 frames per batch");
  lv_geometry(L, w, h);
  L->n = n;
  SST_TRY_L(lv_tables(L, st));
  const size_t gplane = (size_t) L->gw * L->gh;
  SST_LCK(L->part.ensure((size_t) n * L->tiles * 2 * sizeof(double)));
  SST_LCK(L->q.ensure((size_t) n * sizeof(double)));
  SST_LCK(L->addq.ensure((size_t) n * sizeof(float)));
  SST_LCK(L->has.ensure((size_t) n * sizeof(int)));
  // steps 1-2: the gradient's level, P = ds^3 G^3 and the tile sums; radii up
  // to 3 (4 without a reduction) in one staged tile kernel straight from the
  // raw frames at dscale 0 and 1
  const double ds = 20.0, ds3 = ds * ds * ds;
  const dim3 ggrid((L->gw + GR_TX - 1) / GR_TX, (L->gh + GR_TY - 1) / GR_TY, n);
  const uint8_t * s = (const uint8_t *) d_frames;
  const float sc = (float) scale;
  float * p3 = nullptr;
  double * part = L->part.as<double>();
#define SST_LV_TILE(TV, RV, DV, SRC, SW, SH, RS, FS, SC)                                                       \
  k_lv_tile<TV, RV, DV><<<ggrid, 256, 0, st>>>(SRC, SW, SH, RS, FS, SC, L->gw, L->gh, (float) ds3, p3, part, af)
#define SST_LV_TILE_R(TV, DV, SRC, SW, SH, RS, FS, SC)                                                         \
  switch ( r ) {                                                                                               \
  case 1: SST_LV_TILE(TV, 1, DV, SRC, SW, SH, RS, FS, SC); break;                                              \
  case 2: SST_LV_TILE(TV, 2, DV, SRC, SW, SH, RS, FS, SC); break;                                              \
  case 3: SST_LV_TILE(TV, 3, DV, SRC, SW, SH, RS, FS, SC); break;                                              \
  default: SST_LV_TILE(TV, 4, false, SRC, SW, SH, RS, FS, SC); break;                                          \
  }
#define SST_LV_TILE_T(DV)                                                                                      \
  switch ( depth ) {                                                                                           \
  case SST_DEPTH_U8: SST_LV_TILE_R(uint8_t, DV, s, w, h, row_stride, frame_stride, sc); break;                \
  case SST_DEPTH_U16: SST_LV_TILE_R(uint16_t, DV, s, w, h, row_stride, frame_stride, sc); break;              \
  case SST_DEPTH_F32: SST_LV_TILE_R(float, DV, s, w, h, row_stride, frame_stride, sc); break;                 \
  default: return lfail(SST_ERR_INVALID_ARG, "unsupported depth");                                             \
  }
  const bool fused = (L->nlev == 0 && r <= 4) || (L->nlev == 1 && r <= 3);
  // INTER_AREA folded into the tile kernel when its cells tile the 64 x 16 tiles
  AreaFuse af = { 0, 0, L->mw, L->mh, 0.f, nullptr };
  const bool area = L->mw != L->gw || L->mh != L->gh;
  if( area && r <= 4 && L->gw % L->mw == 0 && L->gh % L->mh == 0 && GR_TX % (L->gw / L->mw) == 0 &&
      GR_TY % (L->gh / L->mh) == 0 ) {
    SST_LCK(L->small.ensure((size_t) n * L->mw * L->mh * sizeof(float)));
    af.fx = L->gw / L->mw, af.fy = L->gh / L->mh;
    af.inv_area = (float) (1.0 / ((double) af.fx * af.fy));
    af.small = L->small.as<float>();
  }
  L->area_fused = af.fx != 0;
  if( !L->area_fused ) {
    SST_LCK(L->p3.ensure((size_t) n * gplane * sizeof(float)));
    p3 = L->p3.as<float>();
  }
  if( fused ) {
    if( L->nlev == 0 ) {
      SST_LV_TILE_T(false)
    }
    else {
      SST_LV_TILE_T(true)
    }
    SST_LCK(cudaGetLastError());
    sst_internal_count_launches(1);
  }
  else {
    // step 1: scaled FP32 at the gradient's resolution
    const float * lvl = nullptr;
    if( L->nlev == 0 ) {
      SST_LCK(L->lv[0].ensure((size_t) n * w * h * sizeof(float)));
      SST_LLAUNCH(launch_convert_smooth(d_frames, depth, n, w, h, row_stride, frame_stride, scale, nullptr, 0,
          L->lv[0].as<float>(), (size_t) w * h, st));
      lvl = L->lv[0].as<float>();
    }
    else {
      int cw = (w + 1) / 2, ch = (h + 1) / 2;
      SST_LCK(L->lv[0].ensure((size_t) n * cw * ch * sizeof(float)));
      dim3 grid((cw + DN_TX - 1) / DN_TX, (ch + DN_TY - 1) / DN_TY, n);
      switch ( depth ) {
      case SST_DEPTH_U8: k_lv_down<uint8_t><<<grid, 256, 0, st>>>(s, w, h, row_stride, frame_stride, sc, L->lv[0].as<float>(), cw, ch); break;
      case SST_DEPTH_U16: k_lv_down<uint16_t><<<grid, 256, 0, st>>>(s, w, h, row_stride, frame_stride, sc, L->lv[0].as<float>(), cw, ch); break;
      case SST_DEPTH_F32: k_lv_down<float><<<grid, 256, 0, st>>>(s, w, h, row_stride, frame_stride, sc, L->lv[0].as<float>(), cw, ch); break;
      default: return lfail(SST_ERR_INVALID_ARG, "unsupported depth");
      }
      SST_LCK(cudaGetLastError());
      sst_internal_count_launches(1);
      int b = 0;
      for( int l = 1; l < L->nlev; ++l ) {
        const int nw = (cw + 1) / 2, nh = (ch + 1) / 2;
        SST_LCK(L->lv[b ^ 1].ensure((size_t) n * nw * nh * sizeof(float)));
        SST_LLAUNCH(launch_pyrdown(L->lv[b].as<float>(), cw, ch, (size_t) cw * ch, L->lv[b ^ 1].as<float>(), nw, nh,
            (size_t) nw * nh, n, st));
        b ^= 1, cw = nw, ch = nh;
      }
      lvl = L->lv[b].as<float>();
    }
    // step 2
    if( r <= 4 ) {
      const uint8_t * ls = (const uint8_t *) lvl;
      const size_t lrs = (size_t) L->gw * sizeof(float), lfs = (size_t) L->gw * L->gh * sizeof(float);
      SST_LV_TILE_R(float, false, ls, L->gw, L->gh, lrs, lfs, 1.f)
    }
    else {
      const size_t smem = ((size_t) (GR_TY + 2 * r) * (GR_TX + 2 * r) + 2 * (size_t) (GR_TY + 2 * r) * GR_TX) * sizeof(float);
      k_lv_gradient<<<ggrid, 256, smem, st>>>(lvl, L->gw, L->gh, r, (float) ds3, p3, part);
    }
    SST_LCK(cudaGetLastError());
    sst_internal_count_launches(1);
  }
#undef SST_LV_TILE_T
#undef SST_LV_TILE_R
#undef SST_LV_TILE
  // step 3: W and Q per frame
  k_lv_finish<<<(n + 7) / 8, 256, 0, st>>>(L->part.as<double>(), L->tiles, n, ds3, L->q.as<double>(),
      L->addq.as<float>(), L->has.as<int>());
  SST_LCK(cudaGetLastError());
  sst_internal_count_launches(1);
  // step 4: INTER_AREA reduction
  if( (L->mw != L->gw || L->mh != L->gh) && !L->area_fused ) {
    SST_LCK(L->small.ensure((size_t) n * L->mw * L->mh * sizeof(float)));
    dim3 grid((L->mw + 31) / 32, (L->mh + 7) / 8, n);
    k_lv_area<<<grid, 256, 0, st>>>(L->p3.as<float>(), L->gw, L->gh, L->small.as<float>(), L->mw, L->mh,
        Taps { L->ax_i.as<int>(), L->ax_w.as<float>(), L->ax_k }, Taps { L->ay_i.as<int>(), L->ay_w.as<float>(), L->ay_k });
    SST_LCK(cudaGetLastError());
    sst_internal_count_launches(1);
  }
  return SST_OK;
}

/* Output-grid stacking weights of the last built batch under the frames' warp
 * coefficients (n x SST_NCOEF floats on the device). */
int sst_internal_lv_warp(sst_local_variance * L, int motion, const float * coeffs, int dw, int dh, float * out,
    cudaStream_t st)
{
  dim3 grid((dw + 31) / 32, (dh + 8 * WP_ROWS - 1) / (8 * WP_ROWS), L->n);
  const int fam = motion_family(motion);
#define SST_LV_WARP(FAMV) k_lv_warp<FAMV><<<grid, 256, 0, st>>>(L->small_map(), L->lx(), L->ly(), L->addq.as<float>(), \
      L->has.as<int>(), coeffs, L->w, L->h, dw, dh, out)
  if( fam == FAM_AFFINE ) SST_LV_WARP(FAM_AFFINE);
  else if( fam == FAM_HOMOG ) SST_LV_WARP(FAM_HOMOG);
  else SST_LV_WARP(FAM_QUAD);
#undef SST_LV_WARP
  SST_LCK(cudaGetLastError());
  sst_internal_count_launches(1);
  return SST_OK;
}

int sst_internal_lv_create(sst_local_variance ** out, const sst_local_variance_options * o)
{
  if( o && o->kradius > LV_RMAX ) return lfail(SST_ERR_UNSUPPORTED, "local variance map: kradius above 16 is not supported");
  sst_local_variance * L = new (std::nothrow) sst_local_variance;
  if( !L ) return lfail(SST_ERR_NOMEM, "out of host memory");
  if( o ) L->o = *o;
  else sst_local_variance_options_default(&L->o);
  *out = L;
  return SST_OK;
}

/* ------------------------------------------------------------------ C ABI */

extern "C" void sst_local_variance_options_default(sst_local_variance_options * o)
{
  if( !o ) return;
  o->kradius = 2;
  o->dscale = 1;
  o->uscale = 3;
}

extern "C" int sst_local_variance_create(sst_local_variance ** out, const sst_local_variance_options * o)
{
  if( !out ) return lfail(SST_ERR_INVALID_ARG, "sst_local_variance_create: NULL argument");
  return sst_internal_lv_create(out, o);
}

extern "C" int sst_local_variance_destroy(sst_local_variance * h)
{
  delete h;
  return SST_OK;
}

extern "C" int sst_local_variance_compute(sst_local_variance * L, const void * frames, int depth, int n, int width,
    int height, size_t row_stride, size_t frame_stride, double scale, int on_device, float * maps, double * q,
    void * stream)
{
  if( !L || !frames ) return lfail(SST_ERR_INVALID_ARG, "sst_local_variance_compute: NULL argument");
  if( n < 1 || width < 1 || height < 1 ) return lfail(SST_ERR_INVALID_ARG, "n, width and height must be >= 1");
  if( depth_bytes(depth) == 0 ) return lfail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( row_stride < (size_t) width * depth_bytes(depth) || (n > 1 && frame_stride < row_stride * height) )
    return lfail(SST_ERR_INVALID_ARG, "invalid strides");
  cudaStream_t st = (cudaStream_t) stream;
  const void * d_frames = frames;
  if( !on_device ) {
    const size_t bytes = (size_t) (n - 1) * frame_stride + (size_t) (height - 1) * row_stride +
        (size_t) width * depth_bytes(depth);
    SST_LCK(L->stage.ensure(bytes));
    SST_LCK(cudaMemcpyAsync(L->stage.p, frames, bytes, cudaMemcpyHostToDevice, st));
    d_frames = L->stage.p;
  }
  SST_TRY_L(sst_internal_lv_build(L, d_frames, depth, n, width, height, row_stride, frame_stride, scale, st));
  const size_t plane = (size_t) width * height;
  if( maps ) {
    float * d_maps = maps;
    if( !on_device ) {
      SST_LCK(L->maps.ensure((size_t) n * plane * sizeof(float)));
      d_maps = L->maps.as<float>();
    }
    dim3 grid((width + 31) / 32, (height + 7) / 8, n);
    k_lv_expand<<<grid, 256, 0, st>>>(L->small_map(), L->lx(), L->ly(), L->addq.as<float>(), L->has.as<int>(), width,
        height, d_maps);
    SST_LCK(cudaGetLastError());
    sst_internal_count_launches(1);
    if( !on_device ) SST_LCK(cudaMemcpyAsync(maps, d_maps, (size_t) n * plane * sizeof(float), cudaMemcpyDeviceToHost, st));
  }
  if( q ) SST_LCK(cudaMemcpyAsync(q, L->q.p, (size_t) n * sizeof(double), on_device ? cudaMemcpyDeviceToDevice :
      cudaMemcpyDeviceToHost, st));
  if( !on_device ) SST_LCK(cudaStreamSynchronize(st));
  return SST_OK;
}
