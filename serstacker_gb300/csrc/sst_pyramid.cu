/*
 * sst_pyramid.cu -- c_ecch image pyramid and reference precompute kernels.
 *
 *   convert + Gaussian pre-smooth : ecc_convert_input_image (ecc2.cc:345-382) and
 *                                   sepFilter2D(G, G, BORDER_REPLICATE) (ecc2.cc:998-1006, 1079-1087)
 *   pyrDown                       : c_ecch::downscale_image (ecc2.cc:972-982), 5-tap
 *                                   [1 4 6 4 1]/16, BORDER_REFLECT_101
 *   reference gradients           : ecc_differentiate (ecc2.cc:142-169)
 *   IC Gauss-Newton matrix        : ecc_compute_hessian_matrix (ecc2.cc:295-321) of the
 *                                   steepest-descent images (c_image_transform.cc)
 *
 * All kernels are batched over frames; each input pixel is read from HBM
 * once per kernel (the fused level 0 + 1 pass re-reads only its strips'
 * nine-row halos, from L2 mostly).
 */
#include "sst_engine.cuh"

namespace sst {

/* ------------------------------------------------ convert + pre-smooth */

constexpr int CS_TX = 128, CS_TY = 32, CS_RMAX = 15;

template<typename T>
__device__ __forceinline__ float load_px(const uint8_t * base, size_t row_stride, int x, int y)
{
  return (float) __ldg((const T *) (base + (size_t) y * row_stride) + x);
}

/* One 128 x 32 output tile per CTA: the (128 + 2R) x (32 + 2R) input window
 * (REPLICATE) is converted and staged in shared memory row by row (coalesced),
 * filtered horizontally then vertically. */
template<typename T>
__global__ void __launch_bounds__(256) k_convert_smooth(const uint8_t * src, int w, int h, size_t row_stride,
    size_t frame_stride, float scale, const float * __restrict__ gk, int R, float * dst, size_t dst_stride,
    const RaggedImg * __restrict__ jobs)
{
  extern __shared__ float sm[];
  const uint8_t * fb = src + (size_t) blockIdx.z * frame_stride;
  float * out = dst + (size_t) blockIdx.z * dst_stride;
  if( jobs ) {
    // ragged batch: this image's size, rows and destination (uniform over the CTA)
    const RaggedImg j = jobs[blockIdx.z];
    w = j.sw, h = j.sh, row_stride = j.src_stride;
    fb = src + j.src_off;
    out = dst + j.dst_off;
    if( (int) blockIdx.x * CS_TX >= w || (int) blockIdx.y * CS_TY >= h ) return;
  }
  const int tx0 = blockIdx.x * CS_TX, ty0 = blockIdx.y * CS_TY;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if( R <= 0 ) {
    for( int yy = wid; yy < CS_TY; yy += 8 ) {
      const int y = ty0 + yy;
      if( y >= h ) break;
#pragma unroll
      for( int k = 0; k < CS_TX / 32; ++k ) {
        const int x = tx0 + lane + 32 * k;
        if( x < w ) out[(size_t) y * w + x] = load_px<T>(fb, row_stride, x, y) * scale;
      }
    }
    return;
  }
  const int SW = CS_TX + 2 * R, SH = CS_TY + 2 * R;
  float * s_in = sm;
  float * s_h = sm + SW * SH;
  float * g = s_h + CS_TX * SH;
  if( threadIdx.x <= 2 * R ) g[threadIdx.x] = gk[threadIdx.x];
  for( int yy = wid; yy < SH; yy += 8 ) {
    const int y = clampi(ty0 - R + yy, 0, h - 1);
    const uint8_t * rowp = fb + (size_t) y * row_stride;
#pragma unroll 4
    for( int xx = lane; xx < SW; xx += 32 ) {
      const int x = clampi(tx0 - R + xx, 0, w - 1);
      s_in[yy * SW + xx] = (float) __ldg((const T *) rowp + x) * scale;
    }
  }
  __syncthreads();
  for( int yy = wid; yy < SH; yy += 8 ) {
#pragma unroll
    for( int k = 0; k < CS_TX / 32; ++k ) {
      const int xx = lane + 32 * k;
      const float * p = s_in + yy * SW + xx;
      float a = 0.f;
      for( int i = 0; i <= 2 * R; ++i ) a = fmaf(g[i], p[i], a);
      s_h[yy * CS_TX + xx] = a;
    }
  }
  __syncthreads();
  for( int yy = wid; yy < CS_TY; yy += 8 ) {
    const int y = ty0 + yy;
    if( y >= h ) break;
#pragma unroll
    for( int k = 0; k < CS_TX / 32; ++k ) {
      const int xx = lane + 32 * k, x = tx0 + xx;
      if( x < w ) {
        float a = 0.f;
        for( int j = 0; j <= 2 * R; ++j ) a = fmaf(g[j], s_h[(yy + j) * CS_TX + xx], a);
        out[(size_t) y * w + x] = a;
      }
    }
  }
}

/* Fixed-radius form: the horizontal pass computes 4 outputs per thread from a
 * register window filled by 128-bit shared-memory loads, the vertical pass 4
 * rows per thread from a register column, so each output costs ~3 shared
 * loads instead of 2 (2R + 1). */
template<typename T, int R>
__global__ void __launch_bounds__(256) k_convert_smooth_r(const uint8_t * src, int w, int h, size_t row_stride,
    size_t frame_stride, float scale, const float * __restrict__ gk, float * dst, size_t dst_stride)
{
  constexpr int SW = (CS_TX + 2 * R + 3) & ~3, SH = CS_TY + 2 * R;   // row stride a multiple of 4 floats
  constexpr int NW = (4 + 2 * R + 3) / 4;                           // float4 loads per 4 outputs
  __shared__ __align__(16) float s_in[SH * SW];
  __shared__ __align__(16) float s_h[SH * CS_TX];
  __shared__ float g[2 * R + 1];
  const uint8_t * fb = src + (size_t) blockIdx.z * frame_stride;
  float * out = dst + (size_t) blockIdx.z * dst_stride;
  const int tx0 = blockIdx.x * CS_TX, ty0 = blockIdx.y * CS_TY;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if( threadIdx.x <= 2 * R ) g[threadIdx.x] = gk[threadIdx.x];
  for( int yy = wid; yy < SH; yy += 8 ) {
    const int y = clampi(ty0 - R + yy, 0, h - 1);
    const uint8_t * rowp = fb + (size_t) y * row_stride;
#pragma unroll 4
    for( int xx = lane; xx < SW; xx += 32 ) {
      const int x = clampi(tx0 - R + xx, 0, w - 1);
      s_in[yy * SW + xx] = (float) __ldg((const T *) rowp + x) * scale;
    }
  }
  __syncthreads();
  float gr[2 * R + 1];
#pragma unroll
  for( int i = 0; i <= 2 * R; ++i ) gr[i] = g[i];
  // horizontal: (row, 4-output group) items
  for( int q = threadIdx.x; q < SH * (CS_TX / 4); q += 256 ) {
    const int yy = q / (CS_TX / 4), x4 = (q % (CS_TX / 4)) * 4;
    float v[4 * NW];
#pragma unroll
    for( int k = 0; k < NW; ++k ) {
      const float4 t = *reinterpret_cast<const float4 *>(s_in + yy * SW + x4 + 4 * k);
      v[4 * k] = t.x, v[4 * k + 1] = t.y, v[4 * k + 2] = t.z, v[4 * k + 3] = t.w;
    }
    float o[4];
#pragma unroll
    for( int j = 0; j < 4; ++j ) {
      float a = 0.f;
#pragma unroll
      for( int i = 0; i <= 2 * R; ++i ) a = fmaf(gr[i], v[j + i], a);
      o[j] = a;
    }
    *reinterpret_cast<float4 *>(s_h + yy * CS_TX + x4) = make_float4(o[0], o[1], o[2], o[3]);
  }
  __syncthreads();
  // vertical: (4-row group, column) items
  for( int q = threadIdx.x; q < (CS_TY / 4) * CS_TX; q += 256 ) {
    const int xx = q % CS_TX, y4 = (q / CS_TX) * 4;
    const int x = tx0 + xx;
    float v[4 + 2 * R];
#pragma unroll
    for( int i = 0; i < 4 + 2 * R; ++i ) v[i] = s_h[(y4 + i) * CS_TX + xx];
    if( x >= w ) continue;
#pragma unroll
    for( int j = 0; j < 4; ++j ) {
      const int y = ty0 + y4 + j;
      if( y >= h ) break;
      float a = 0.f;
#pragma unroll
      for( int i = 0; i <= 2 * R; ++i ) a = fmaf(gr[i], v[j + i], a);
      out[(size_t) y * w + x] = a;
    }
  }
}

cudaError_t launch_convert_smooth(const void * src, int depth, int n, int w, int h, size_t row_stride,
    size_t frame_stride, double scale, const float * gk, int ksize, float * dst, size_t dst_stride, cudaStream_t st)
{
  // gk: device array of ksize weights (nullptr: no smoothing)
  const int R = gk ? ksize / 2 : 0;
  if( R > CS_RMAX ) return cudaErrorInvalidValue;
  const size_t smem = R > 0 ? ((size_t) (CS_TX + 2 * R) * (CS_TY + 2 * R) + (size_t) CS_TX * (CS_TY + 2 * R) + 32) * sizeof(float) : 0;
  dim3 grid((w + CS_TX - 1) / CS_TX, (h + CS_TY - 1) / CS_TY, n);
  const uint8_t * s = (const uint8_t *) src;
  static bool attr = false;
  if( !attr ) {
    const int mx = (int) (((CS_TX + 2 * CS_RMAX) * (CS_TY + 2 * CS_RMAX) + CS_TX * (CS_TY + 2 * CS_RMAX) + 32) * sizeof(float));
    cudaFuncSetAttribute(k_convert_smooth<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_convert_smooth<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_convert_smooth<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    attr = true;
  }
  if( R == 3 ) {   // sigma = 1 (the c_ecch default); 40 KB of static shared memory
#define SST_CS_R(RV)                                                                                                   \
    switch ( depth ) {                                                                                                 \
    case SST_DEPTH_U8: k_convert_smooth_r<uint8_t, RV><<<grid, 256, 0, st>>>(s, w, h, row_stride, frame_stride, (float) scale, gk, dst, dst_stride); break; \
    case SST_DEPTH_U16: k_convert_smooth_r<uint16_t, RV><<<grid, 256, 0, st>>>(s, w, h, row_stride, frame_stride, (float) scale, gk, dst, dst_stride); break; \
    case SST_DEPTH_F32: k_convert_smooth_r<float, RV><<<grid, 256, 0, st>>>(s, w, h, row_stride, frame_stride, (float) scale, gk, dst, dst_stride); break; \
    default: return cudaErrorInvalidValue;                                                                             \
    }
    SST_CS_R(3)
#undef SST_CS_R
    return cudaGetLastError();
  }
  switch ( depth ) {
  case SST_DEPTH_U8: k_convert_smooth<uint8_t><<<grid, 256, smem, st>>>(s, w, h, row_stride, frame_stride, (float) scale, gk, R, dst, dst_stride, nullptr); break;
  case SST_DEPTH_U16: k_convert_smooth<uint16_t><<<grid, 256, smem, st>>>(s, w, h, row_stride, frame_stride, (float) scale, gk, R, dst, dst_stride, nullptr); break;
  case SST_DEPTH_F32: k_convert_smooth<float><<<grid, 256, smem, st>>>(s, w, h, row_stride, frame_stride, (float) scale, gk, R, dst, dst_stride, nullptr); break;
  default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_convert_smooth_ragged(const void * src, int depth, const RaggedImg * jobs, int n, int max_w,
    int max_h, double scale, const float * gk, int ksize, float * dst, cudaStream_t st)
{
  const int R = gk ? ksize / 2 : 0;
  if( R > CS_RMAX || n > 65535 ) return cudaErrorInvalidValue;
  const size_t smem = R > 0 ? ((size_t) (CS_TX + 2 * R) * (CS_TY + 2 * R) + (size_t) CS_TX * (CS_TY + 2 * R) + 32) * sizeof(float) : 0;
  dim3 grid((max_w + CS_TX - 1) / CS_TX, (max_h + CS_TY - 1) / CS_TY, n);
  const uint8_t * s = (const uint8_t *) src;
  const int mx = (int) (((CS_TX + 2 * CS_RMAX) * (CS_TY + 2 * CS_RMAX) + CS_TX * (CS_TY + 2 * CS_RMAX) + 32) * sizeof(float));
  cudaFuncSetAttribute(k_convert_smooth<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_convert_smooth<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_convert_smooth<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  switch ( depth ) {
  case SST_DEPTH_U8: k_convert_smooth<uint8_t><<<grid, 256, smem, st>>>(s, 0, 0, 0, 0, (float) scale, gk, R, dst, 0, jobs); break;
  case SST_DEPTH_U16: k_convert_smooth<uint16_t><<<grid, 256, smem, st>>>(s, 0, 0, 0, 0, (float) scale, gk, R, dst, 0, jobs); break;
  case SST_DEPTH_F32: k_convert_smooth<float><<<grid, 256, smem, st>>>(s, 0, 0, 0, 0, (float) scale, gk, R, dst, 0, jobs); break;
  default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

/* ------------------------------------------------------------- pyrDown */

constexpr int PD_TX = 64, PD_TY = 16;

__global__ void __launch_bounds__(256) k_pyrdown(const float * src, int sw, int sh, size_t src_stride,
    float * dst, int dw, int dh, size_t dst_stride, const RaggedImg * __restrict__ jobs)
{
  constexpr int SW = 2 * PD_TX + 4, SH = 2 * PD_TY + 4;
  __shared__ float s_in[SH * SW];
  __shared__ float s_h[SH * PD_TX];
  const float * in = src + (size_t) blockIdx.z * src_stride;
  float * out = dst + (size_t) blockIdx.z * dst_stride;
  if( jobs ) {
    const RaggedImg j = jobs[blockIdx.z];
    sw = j.sw, sh = j.sh, dw = j.dw, dh = j.dh;
    in = src + j.src_off;
    out = dst + j.dst_off;
    if( (int) blockIdx.x * PD_TX >= dw || (int) blockIdx.y * PD_TY >= dh ) return;
  }
  const int tx0 = blockIdx.x * PD_TX, ty0 = blockIdx.y * PD_TY;
  const int sx0 = 2 * tx0 - 2, sy0 = 2 * ty0 - 2;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for( int yy = wid; yy < SH; yy += 8 ) {
    const float * rowp = in + (size_t) reflect101(sy0 + yy, sh) * sw;
#pragma unroll
    for( int xx = lane; xx < SW; xx += 32 ) s_in[yy * SW + xx] = __ldg(rowp + reflect101(sx0 + xx, sw));
  }
  __syncthreads();
  for( int yy = wid; yy < SH; yy += 8 ) {
#pragma unroll
    for( int k = 0; k < PD_TX / 32; ++k ) {
      const int xx = lane + 32 * k;
      const float * p = s_in + yy * SW + 2 * xx;
      s_h[yy * PD_TX + xx] = (p[0] + p[4]) * 0.0625f + (p[1] + p[3]) * 0.25f + p[2] * 0.375f;
    }
  }
  __syncthreads();
  for( int yy = wid; yy < PD_TY; yy += 8 ) {
    const int y = ty0 + yy;
    if( y >= dh ) break;
#pragma unroll
    for( int k = 0; k < PD_TX / 32; ++k ) {
      const int xx = lane + 32 * k, x = tx0 + xx;
      if( x < dw ) {
        const float * p = s_h + (2 * yy) * PD_TX + xx;
        out[(size_t) y * dw + x] = (p[0] + p[4 * PD_TX]) * 0.0625f + (p[PD_TX] + p[3 * PD_TX]) * 0.25f +
            p[2 * PD_TX] * 0.375f;
      }
    }
  }
}

cudaError_t launch_pyrdown(const float * src, int sw, int sh, size_t src_stride, float * dst, int dw, int dh,
    size_t dst_stride, int n, cudaStream_t st)
{
  dim3 grid((dw + PD_TX - 1) / PD_TX, (dh + PD_TY - 1) / PD_TY, n);
  k_pyrdown<<<grid, 256, 0, st>>>(src, sw, sh, src_stride, dst, dw, dh, dst_stride, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_pyrdown_ragged(const float * src, const RaggedImg * jobs, int n, int max_dw, int max_dh,
    float * dst, cudaStream_t st)
{
  if( n > 65535 ) return cudaErrorInvalidValue;
  dim3 grid((max_dw + PD_TX - 1) / PD_TX, (max_dh + PD_TY - 1) / PD_TY, n);
  k_pyrdown<<<grid, 256, 0, st>>>(src, 0, 0, 0, dst, 0, 0, 0, jobs);
  return cudaGetLastError();
}

/* ------------------------- fused convert + pre-smooth + first pyrDown */

/* One warp per strip of PS_TX = 120 level-0 columns by BH rows (and the strip's
 * 60 x BH/2 level-1 cells). Lane l owns the four smoothed columns
 * x0 = tx0 - 4 + 4l ... x0 + 3 and sweeps the strip's input rows top to bottom:
 *  - each input row (loaded PS_D rows ahead into registers) is converted and
 *    scaled; the 7-tap horizontal Gaussian reads the neighbouring lanes'
 *    cells through a per-warp row buffer in shared memory;
 *  - the vertical Gaussian adds each horizontal row into the seven smoothed
 *    rows it reaches (a ring of seven rows of accumulators, two column pairs
 *    each in paired FP32 FMAs, taps in order), so the smoothed row S of input
 *    row r is complete six rows later;
 *  - S is stored as level 0 where it lies in the strip, and its horizontal
 *    5-tap pyrDown (two level-1 columns per lane) enters a ring of five rows,
 *    from which every second S row gives one level-1 row (rows first, as
 *    pyrDown).
 * Lanes 0 and 31 compute halo columns only. Level 0 is written once and never
 * read back; no barrier, wait or shared-memory pass involves more than a warp.
 * Borders: input cells outside the image take the nearest in-image cell
 * (REPLICATE, as sepFilter2D); cells of S that pyrDown taps reach outside the
 * image take the reflected cell (REFLECT_101, as pyrDown): columns in the row
 * buffer, rows in the ring. */
constexpr int PS_TX = 120;        // level-0 columns per strip
constexpr int PS_D = 7;           // input rows in flight per lane
constexpr int PS_BUF = 136;       // row buffer: x = tx0 - 8 ... tx0 + 127
constexpr int PS_WARPS = 4;       // warps (strips) per CTA

template<typename T> struct ps_raw;                       // a lane's four input cells as loaded
template<> struct ps_raw<uint8_t> { typedef uint32_t type; };
template<> struct ps_raw<uint16_t> { typedef uint2 type; };
template<> struct ps_raw<float> { typedef float4 type; };

__device__ __forceinline__ uint32_t ps_load(const uint8_t * row, int x) { return __ldg((const uint32_t *) (row + x)); }
__device__ __forceinline__ uint2 ps_load(const uint16_t * row, int x) { return __ldg((const uint2 *) (row + x)); }
__device__ __forceinline__ float4 ps_load(const float * row, int x) { return __ldg((const float4 *) (row + x)); }

/* the four cells x ... x + 3 with each column clamped into the image */
__device__ __forceinline__ uint32_t ps_load_clamped(const uint8_t * row, int x, int w)
{
  uint32_t q = 0;
#pragma unroll
  for( int k = 0; k < 4; ++k ) q |= (uint32_t) __ldg(row + clampi(x + k, 0, w - 1)) << (8 * k);
  return q;
}

__device__ __forceinline__ uint2 ps_load_clamped(const uint16_t * row, int x, int w)
{
  uint32_t e[4];
#pragma unroll
  for( int k = 0; k < 4; ++k ) e[k] = __ldg(row + clampi(x + k, 0, w - 1));
  return make_uint2(e[0] | (e[1] << 16), e[2] | (e[3] << 16));
}

__device__ __forceinline__ float4 ps_load_clamped(const float * row, int x, int w)
{
  return make_float4(__ldg(row + clampi(x, 0, w - 1)), __ldg(row + clampi(x + 1, 0, w - 1)),
      __ldg(row + clampi(x + 2, 0, w - 1)), __ldg(row + clampi(x + 3, 0, w - 1)));
}

__device__ __forceinline__ float4 ps_convert(uint32_t q)
{
  return make_float4((float) (q & 0xffu), (float) ((q >> 8) & 0xffu), (float) ((q >> 16) & 0xffu), (float) (q >> 24));
}

__device__ __forceinline__ float4 ps_convert(uint2 q)
{
  return make_float4((float) (q.x & 0xffffu), (float) (q.x >> 16), (float) (q.y & 0xffffu), (float) (q.y >> 16));
}

__device__ __forceinline__ float4 ps_convert(float4 q)
{
  return q;
}

/* pyrDown's [1 4 6 4 1] / 16 of five taps */
__device__ __forceinline__ float pyr5f(float a, float b, float c, float d, float e)
{
  return fmaf(c, 0.375f, fmaf(a + e, 0.0625f, (b + d) * 0.25f));
}

/* The 7-tap horizontal Gaussian of four columns: v holds the cells from four
 * left of the lane's first column; column c takes v[c + 1] ... v[c + 7] in tap
 * order. Column pairs (0, 1) and (2, 3) run as paired FP32 FMAs (each lane an
 * ordinary fmaf, so the sums are those of the scalar loop). */
__device__ __forceinline__ float4 hgauss4(const float2 (&g)[7], const float (&v)[12])
{
  float2 a = make_float2(0.f, 0.f), b = a;
#pragma unroll
  for( int i = 0; i < 7; ++i ) {
    a = __ffma2_rn(g[i], make_float2(v[1 + i], v[2 + i]), a);
    b = __ffma2_rn(g[i], make_float2(v[3 + i], v[4 + i]), b);
  }
  return make_float4(a.x, a.y, b.x, b.y);
}

/* pyrDown's five-tap weights on two columns at once (pyr5f per lane) */
__device__ __forceinline__ float2 pyr5f2(float2 a, float2 b, float2 c, float2 d, float2 e)
{
  return __ffma2_rn(c, make_float2(0.375f, 0.375f), __ffma2_rn(__fadd2_rn(a, e), make_float2(0.0625f, 0.0625f),
      __fmul2_rn(__fadd2_rn(b, d), make_float2(0.25f, 0.25f))));
}

/* Strips of one launch: the interior strips (every lane's cells inside the
 * image: 8 <= tx0 and tx0 + 124 <= w), or the edge strips (the first one and
 * those from `first` on). Two launches keep each kernel's loop free of the
 * other's clamped loads. */
struct StripSet {
  int first, count;   // interior: strips first ... first + count - 1; edge: 0, then first ... first + count - 2
  int edge;
};

template<typename T, int BH, bool EDGE>
__global__ void __launch_bounds__(32 * PS_WARPS, 4) k_convert_pyr1(const T * __restrict__ src, size_t row_elems,
    size_t frame_elems, int w, int h, StripSet ss, int gy, int n, float scale, const float * __restrict__ gk,
    float * dst0, float * dst1, int dw, int dh, size_t dst_stride, int vec0, int vec1)
{
  static_assert(BH % 2 == 0, "level-1 rows pair level-0 rows");
  constexpr int NR = BH + 9;                                  // input rows of a strip
  static_assert(NR % 7 == 0, "whole periods of the seven-row ring");
  __shared__ __align__(16) float s_buf[PS_WARPS][2][PS_BUF];  // per warp: input row, S row
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long item = (long long) blockIdx.x * PS_WARPS + warp;
  const int per_frame = ss.count * gy;
  if( item >= (long long) per_frame * n ) return;             // uniform over the warp
  const int z = (int) (item / per_frame), rem = (int) (item - (long long) z * per_frame);
  const int by = rem / ss.count, k = rem - by * ss.count;
  const int bx = !EDGE ? ss.first + k : k == 0 ? 0 : ss.first + k - 1;
  const int tx0 = bx * PS_TX, ty0 = by * BH;
  const int x0 = tx0 - 4 + 4 * lane;
  const int xe = max(tx0 - 5, 0);                             // lane 0's extra input cell
  const T * frame = src + (size_t) z * frame_elems;
  float * rin = s_buf[warp][0];
  float * srow = s_buf[warp][1];
  for( int q = lane; q < 2 * PS_BUF; q += 32 ) rin[q] = 0.f;  // cells no lane writes are read as halo
  float2 g[7];                                                // each tap twice, for the paired FMAs
#pragma unroll
  for( int i = 0; i < 7; ++i ) g[i].x = g[i].y = __ldg(gk + i);
  const float2 sc = make_float2(scale, scale);

  // input rows ty0 - 5 + r, r = 0 ... NR - 1 (clamped into the image), PS_D in flight;
  // the row pointer of row r + PS_D moves on while that row is inside the image
  typename ps_raw<T>::type q[PS_D];
  T qe[PS_D];
  const T * rowp = frame;
#pragma unroll
  for( int i = 0; i < PS_D; ++i ) {
    rowp = frame + (size_t) clampi(ty0 - 5 + i, 0, h - 1) * row_elems;
    q[i] = EDGE ? ps_load_clamped(rowp, x0, w) : ps_load(rowp, x0);
    qe[i] = lane == 0 ? __ldg(rowp + xe) : (T) 0;
  }
  const int r_adv_end = h - 3 - ty0;                          // row r + PS_D = ty0 + 2 + r <= h - 1
  float2 A[7], B[7];                                          // columns (0, 1) and (2, 3) of the seven rows
#pragma unroll
  for( int i = 0; i < 7; ++i ) A[i] = B[i] = make_float2(0.f, 0.f);
  float2 p0 = make_float2(0.f, 0.f), p1 = p0, p2 = p0, p3 = p0;   // level-1 ring: S rows s - 4 ... s - 1
  // level 0: S rows s = 2 ... s_end0 - 1 (y = ty0 - 2 + s) of lanes 1 ... 30 inside the image
  const bool st0 = lane >= 1 && lane <= 30 && x0 < w;
  const bool st0v = st0 && vec0 && x0 + 3 < w;
  const unsigned n0 = (unsigned) max(0, min(BH, h - ty0));   // level-0 rows of the strip
  float * o0 = dst0 + (size_t) z * dst_stride + (size_t) ty0 * w + x0;   // row y = ty0 (s = 2)
  // level 1: rows i = 0 ... i_end - 1 (y1 = ty0 / 2 + i), columns x1, x1 + 1
  const int x1 = tx0 / 2 + 2 * lane - 2;
  const bool st1 = lane >= 1 && lane <= 30 && x1 < dw;
  const bool st1v = st1 && vec1 && x1 + 1 < dw;
  const int i_end = min(BH / 2, dh - ty0 / 2);
  const bool rfix = ty0 == 0 || ty0 + BH + 2 > h;             // pyrDown rows reach outside the image
  float * o1 = dst1 + (size_t) z * dst_stride + (size_t) (ty0 / 2) * dw + x1;
  __syncwarp();

#pragma unroll 1
  for( int r0 = 0; r0 < NR; r0 += 7 ) {
    const bool refill = r0 + 7 < NR;                          // rows r0 + 7 ... r0 + 13 exist
#pragma unroll
    for( int j = 0; j < 7; ++j ) {
      const int r = r0 + j;
      // convert this row's cells, then refill the slot with row r + PS_D
      const float4 fr = ps_convert(q[j]);
      const float2 f01 = __fmul2_rn(make_float2(fr.x, fr.y), sc), f23 = __fmul2_rn(make_float2(fr.z, fr.w), sc);
      const float4 f = make_float4(f01.x, f01.y, f23.x, f23.y);
      const float fe = (float) qe[j] * scale;
      if( refill ) {
        if( r <= r_adv_end ) rowp += row_elems;
        q[j] = EDGE ? ps_load_clamped(rowp, x0, w) : ps_load(rowp, x0);
        if( lane == 0 ) qe[j] = __ldg(rowp + xe);
      }
      // horizontal Gaussian through the row buffer
      *reinterpret_cast<float4 *>(rin + 4 * lane + 4) = f;
      if( lane == 0 ) rin[3] = fe;
      __syncwarp();
      const float4 lo = *reinterpret_cast<const float4 *>(rin + 4 * lane);
      const float4 hi = *reinterpret_cast<const float4 *>(rin + 4 * lane + 8);
      const float v[12] = { lo.x, lo.y, lo.z, lo.w, f.x, f.y, f.z, f.w, hi.x, hi.y, hi.z, hi.w };
      const float4 H = hgauss4(g, v);
      // vertical Gaussian: smoothed row r - i takes tap i in slot (j - i) mod 7;
      // tap 0 starts the row's sum; rows outside 0 ... NR - 7 are never read
#pragma unroll
      for( int i = 0; i < 7; ++i ) {
        const int sl = (j - i + 7) % 7;
        const float2 h01 = make_float2(H.x, H.y), h23 = make_float2(H.z, H.w);
        A[sl] = i == 0 ? __fmul2_rn(g[0], h01) : __ffma2_rn(g[i], h01, A[sl]);
        B[sl] = i == 0 ? __fmul2_rn(g[0], h23) : __ffma2_rn(g[i], h23, B[sl]);
      }
      if( r < 6 ) {
        __syncwarp();                                         // the row buffer is rewritten next row
        continue;
      }
      // smoothed row s complete (y = ty0 - 2 + s); the S-row barrier below also
      // orders this row's input-buffer reads before the next row's writes
      const int s = r - 6;
      const float4 S = make_float4(A[(j + 1) % 7].x, A[(j + 1) % 7].y, B[(j + 1) % 7].x, B[(j + 1) % 7].y);
      if( (unsigned) (s - 2) < n0 ) {
        if( !EDGE && vec0 ) {                                 // interior strips: lanes 1 ... 30 inside the image
          if( st0 ) *reinterpret_cast<float4 *>(o0) = S;
        }
        else if( st0v ) *reinterpret_cast<float4 *>(o0) = S;
        else if( st0 ) {
          o0[0] = S.x;
          if( x0 + 1 < w ) o0[1] = S.y;
          if( x0 + 2 < w ) o0[2] = S.z;
          if( x0 + 3 < w ) o0[3] = S.w;
        }
        o0 += w;
      }
      // horizontal pyrDown of S: level-1 columns x1 (taps x0 - 2 ... x0 + 2) and
      // x1 + 1 (taps x0 ... x0 + 4)
      *reinterpret_cast<float4 *>(srow + 4 * lane + 4) = S;
      __syncwarp();
      float4 c = S;
      if( EDGE ) {
        if( lane < 4 ) {
          const int x = lane < 2 ? lane - 2 : w + lane - 2, kk = x - tx0 + 8;
          if( kk >= 0 && kk < PS_BUF ) srow[kk] = srow[reflect101(x, w) - tx0 + 8];
        }
        __syncwarp();
        c = *reinterpret_cast<const float4 *>(srow + 4 * lane + 4);
      }
      const float2 l = *reinterpret_cast<const float2 *>(srow + 4 * lane + 2);
      const float rr = srow[4 * lane + 8];
      const float2 p = make_float2(pyr5f(l.x, l.y, c.x, c.y, c.z), pyr5f(c.x, c.y, c.z, c.w, rr));
      if( s & 1 ) {
        p3 = p;
        continue;
      }
      if( s >= 4 ) {
        // level-1 row i = (s - 4) / 2 at y = ty0 + 2i from S rows s - 4 ... s (REFLECT_101 rows)
        const int i = (s - 4) >> 1;
        float2 a = p0, b = p1, d = p3, e = p;
        if( rfix ) {
          const int yy = ty0 + 2 * i;
          if( yy == 0 ) a = e, b = d;
          if( yy + 2 == h ) e = p2;
          if( yy + 1 == h ) d = b, e = a;
        }
        if( i < i_end ) {
          const float2 o = pyr5f2(a, b, p2, d, e);
          if( !EDGE && vec1 ) {
            if( st1 ) *reinterpret_cast<float2 *>(o1) = o;
          }
          else if( st1v ) *reinterpret_cast<float2 *>(o1) = o;
          else if( st1 ) {
            o1[0] = o.x;
            if( x1 + 1 < dw ) o1[1] = o.y;
          }
          o1 += dw;
        }
      }
      p0 = p2, p1 = p3, p2 = p;
    }
  }
}

template<typename T>
static cudaError_t launch_fp(const void * src, size_t row_stride, size_t frame_stride, int n, int w, int h, float scale,
    const float * gk, float * dst0, float * dst1, int dw, int dh, size_t dst_stride, cudaStream_t st)
{
  constexpr int BH = 96;
  const int gx = (w + PS_TX - 1) / PS_TX, gy = (h + BH - 1) / BH;
  // interior strips: 1 ... bmin - 1 (bmin = the first strip with tx0 + 124 > w)
  // (and whose level-1 columns all lie inside dw; the interior launch stores without column tests)
  int bmin = w >= 124 ? std::min(gx, (w - 124) / PS_TX + 1) : 1;
  while ( bmin > 1 && (bmin - 1) * (PS_TX / 2) + PS_TX / 2 > dw ) --bmin;
  const StripSet in = { 1, std::max(0, bmin - 1), 0 };
  const StripSet ed = { bmin, 1 + (gx - bmin), 1 };
  const int vec0 = (w & 3) == 0 && (dst_stride & 3) == 0 && ((uintptr_t) dst0 & 15) == 0;
  const int vec1 = (dw & 1) == 0 && (dst_stride & 1) == 0 && ((uintptr_t) dst1 & 7) == 0;
  for( const StripSet & ss : { in, ed } ) {
    if( ss.count <= 0 ) continue;
    const long long items = (long long) ss.count * gy * n;
    const long long blocks = (items + PS_WARPS - 1) / PS_WARPS;
    if( blocks > (1ll << 30) ) return cudaErrorInvalidValue;
    if( ss.edge ) k_convert_pyr1<T, BH, true><<<(unsigned) blocks, 32 * PS_WARPS, 0, st>>>((const T *) src,
        row_stride / sizeof(T), frame_stride / sizeof(T), w, h, ss, gy, n, scale, gk, dst0, dst1, dw, dh, dst_stride,
        vec0, vec1);
    else k_convert_pyr1<T, BH, false><<<(unsigned) blocks, 32 * PS_WARPS, 0, st>>>((const T *) src,
        row_stride / sizeof(T), frame_stride / sizeof(T), w, h, ss, gy, n, scale, gk, dst0, dst1, dw, dh, dst_stride,
        vec0, vec1);
    const cudaError_t e = cudaGetLastError();
    if( e != cudaSuccess ) return e;
  }
  return cudaSuccess;
}

/* Level 0 and level 1 of n frames in one pass when the pre-smoothing is the
 * 7-tap Gaussian and the rows allow the lanes' vector loads (base and strides
 * multiples of four cells); *done = false (nothing launched) otherwise, and
 * the caller builds the levels separately. */
cudaError_t launch_convert_pyr1(const void * src, int depth, int n, int w, int h, size_t row_stride,
    size_t frame_stride, double scale, const float * gk, int ksize, float * dst0, float * dst1, int dw, int dh,
    size_t dst_stride, int * err, cudaStream_t st, bool * done)
{
  (void) err;                                   // the pass holds no waits
  *done = false;
  if( !gk || ksize != 7 || w < 8 || h < 8 || n < 1 || 2 * dw > w + 1 || 2 * dh > h + 1 ) return cudaSuccess;
  const size_t esz = depth == SST_DEPTH_U8 ? 1 : depth == SST_DEPTH_U16 ? 2 : depth == SST_DEPTH_F32 ? 4 : 0;
  if( !esz ) return cudaSuccess;
  const size_t al = 4 * esz;                    // a lane's four cells
  if( ((uintptr_t) src % al) || row_stride % al || (n > 1 && frame_stride % al) ) return cudaSuccess;
  if( n == 1 ) frame_stride = row_stride * h;
  cudaError_t e;
  switch ( depth ) {
  case SST_DEPTH_U8:
    e = launch_fp<uint8_t>(src, row_stride, frame_stride, n, w, h, (float) scale, gk, dst0, dst1, dw, dh, dst_stride, st);
    break;
  case SST_DEPTH_U16:
    e = launch_fp<uint16_t>(src, row_stride, frame_stride, n, w, h, (float) scale, gk, dst0, dst1, dw, dh, dst_stride, st);
    break;
  default:
    e = launch_fp<float>(src, row_stride, frame_stride, n, w, h, (float) scale, gk, dst0, dst1, dw, dh, dst_stride, st);
    break;
  }
  if( e == cudaSuccess ) *done = true;
  return e;
}

/* Sum of each image of a ragged job list (one CTA per image, fixed-order
 * FP64 reduction): sums[j] = sum of image j's sw x sh floats at src_off. */
__global__ void __launch_bounds__(256) k_roi_means(const float * pool, const RaggedImg * jobs, double * sums)
{
  __shared__ double s_w[8];
  const RaggedImg j = jobs[blockIdx.x];
  const float * p = pool + j.src_off;
  const size_t N = (size_t) j.sw * j.sh;
  double acc = 0;
  float part = 0.f;
  int k = 0;
  for( size_t i = threadIdx.x; i < N; i += 256 ) {
    part += __ldg(p + i);
    if( ++k == 64 ) acc += part, part = 0.f, k = 0;   // FP32 runs of 64 pixels, FP64 across runs
  }
  acc += part;
  acc = warp_sum(acc);
  if( (threadIdx.x & 31) == 0 ) s_w[threadIdx.x >> 5] = acc;
  __syncthreads();
  if( threadIdx.x == 0 ) {
    double t = 0;
    for( int w = 0; w < 8; ++w ) t += s_w[w];
    sums[blockIdx.x] = t;
  }
}

cudaError_t launch_roi_means(const float * pool, const RaggedImg * jobs, int n, double * sums, cudaStream_t st)
{
  k_roi_means<<<n, 256, 0, st>>>(pool, jobs, sums);
  return cudaGetLastError();
}

/* cv::resize(INTER_NEAREST) of a mask: sx = floor(dx * sw / dw) */
__global__ void k_resize_nearest_u8(const uint8_t * src, int sw, int sh, uint8_t * dst, int dw, int dh)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= dw || y >= dh ) return;
  const int sx = min((int) floor(x * ((double) sw / dw)), sw - 1);
  const int sy = min((int) floor(y * ((double) sh / dh)), sh - 1);
  dst[(size_t) y * dw + x] = src[(size_t) sy * sw + sx];
}

cudaError_t launch_resize_nearest_u8(const uint8_t * src, int sw, int sh, uint8_t * dst, int dw, int dh, cudaStream_t st)
{
  k_resize_nearest_u8<<<dim3((dw + 127) / 128, dh), 128, 0, st>>>(src, sw, sh, dst, dw, dh);
  return cudaGetLastError();
}

/* 5x5 erosion of a binary mask, window clipped to the image (every border
 * mode the path uses for erode reduces to this) */
__global__ void k_erode5(const uint8_t * src, int w, int h, uint8_t * dst)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= w || y >= h ) return;
  uint8_t m = 255;
  for( int j = max(0, y - 2); j <= min(h - 1, y + 2); ++j )
    for( int i = max(0, x - 2); i <= min(w - 1, x + 2); ++i ) m = min(m, src[(size_t) j * w + i]);
  dst[(size_t) y * w + x] = m;
}

cudaError_t launch_erode5(const uint8_t * src, int w, int h, uint8_t * dst, cudaStream_t st)
{
  k_erode5<<<dim3((w + 127) / 128, h), 128, 0, st>>>(src, w, h, dst);
  return cudaGetLastError();
}

/* ---------------------------------------------------- reference gradients */

constexpr int RG_TX = 32, RG_TY = 8;

__global__ void __launch_bounds__(256) k_ref_gradients(const float * img, const uint8_t * mask, int w, int h, float2 * grad)
{
  constexpr int SW = RG_TX + 4, SH = RG_TY + 4;
  __shared__ float s[SH * SW];
  const int tx0 = blockIdx.x * RG_TX, ty0 = blockIdx.y * RG_TY;
  for( int q = threadIdx.x; q < SW * SH; q += 256 ) {
    const int x = clampi(tx0 - 2 + q % SW, 0, w - 1), y = clampi(ty0 - 2 + q / SW, 0, h - 1);
    s[q] = __ldg(img + (size_t) y * w + x);
  }
  __syncthreads();
  const int lx = threadIdx.x % RG_TX, ly = threadIdx.x / RG_TX;
  const int x = tx0 + lx, y = ty0 + ly;
  if( x >= w || y >= h ) return;
  const float * p = s + (ly + 2) * SW + lx + 2;
  const float a = 1.f / 12.f, b = -2.f / 3.f;
  const float r0 = a * p[-SW - 2] + b * p[-SW - 1] - b * p[-SW + 1] - a * p[-SW + 2];
  const float r1 = a * p[-2] + b * p[-1] - b * p[1] - a * p[2];
  const float r2 = a * p[SW - 2] + b * p[SW - 1] - b * p[SW + 1] - a * p[SW + 2];
  const float c0 = a * p[-2 * SW - 1] + b * p[-SW - 1] - b * p[SW - 1] - a * p[2 * SW - 1];
  const float c1 = a * p[-2 * SW] + b * p[-SW] - b * p[SW] - a * p[2 * SW];
  const float c2 = a * p[-2 * SW + 1] + b * p[-SW + 1] - b * p[SW + 1] - a * p[2 * SW + 1];
  float2 g = make_float2(0.25f * r0 + 0.5f * r1 + 0.25f * r2, 0.25f * c0 + 0.5f * c1 + 0.25f * c2);
  if( mask && !mask[(size_t) y * w + x] ) g = make_float2(0.f, 0.f);
  grad[(size_t) y * w + x] = g;
}

cudaError_t launch_ref_gradients(const float * img, const uint8_t * mask, int w, int h, float2 * grad, cudaStream_t st)
{
  dim3 grid((w + RG_TX - 1) / RG_TX, (h + RG_TY - 1) / RG_TY);
  k_ref_gradients<<<grid, 256, 0, st>>>(img, mask, w, h, grad);
  return cudaGetLastError();
}

/* packed {T, gx, gy, 0} reference level for the pointwise passes */
__global__ void k_pack_reference(const float * img, const float2 * grad, size_t n, float4 * out)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= n ) return;
  const float2 g = grad[i];
  out[i] = make_float4(img[i], g.x, g.y, 0.f);
}

cudaError_t launch_pack_reference(const float * img, const float2 * grad, size_t n, float4 * out, cudaStream_t st)
{
  k_pack_reference<<<(unsigned) ((n + 255) / 256), 256, 0, st>>>(img, grad, n, out);
  return cudaGetLastError();
}

/* --------------------------------------------- IC Gauss-Newton matrix */

/* per-tile lower-triangle sums of J J^T with J at the identity warp */
template<int JK, int M>
__global__ void __launch_bounds__(256) k_ref_hessian(const float2 * grad, int w, int h, int tiles_x, const float * jc_in,
    double * partials)
{
  constexpr int NS = M * (M + 1) / 2;
  __shared__ double s_red[8 * NS];
  float jc[8];
  for( int i = 0; i < 8; ++i ) jc[i] = jc_in[i];
  const int t = blockIdx.x;
  const int tx0 = (t % tiles_x) * PW_TX, ty0 = (t / tiles_x) * PW_TY;
  const int x = tx0 + (threadIdx.x & (PW_TX - 1));
  float acc[NS];
  for( int k = 0; k < NS; ++k ) acc[k] = 0.f;
  if( x < w ) {
    for( int k = 0; k < PW_TY / 2; ++k ) {
      const int y = ty0 + (threadIdx.x >> 7) + 2 * k;
      if( y < h ) {
        const float2 g = grad[(size_t) y * w + x];
        float J[M];
        // same formulas as the pass kernels (sd_pixel), at the identity
        if( JK == J_TRANS ) { J[0] = g.x, J[1 < M ? 1 : 0] = g.y; }
        else if( JK == J_EUCL ) {
          const float xx = x - jc[3], yy = y - jc[4];
          J[0] = g.x, J[1] = g.y;
          const float u = jc[2] * xx - jc[1] * yy, v = jc[1] * xx + jc[2] * yy;
          J[2 < M ? 2 : 0] = jc[0] * (-g.x * v + g.y * u);
          if( M > 3 ) J[3 < M ? 3 : 0] = g.x * u + g.y * v;
        }
        else if( JK == J_AFFINE ) {
          J[0] = g.x * x, J[1] = g.x * y, J[2] = g.x;
          J[3 < M ? 3 : 0] = g.y * x, J[4 < M ? 4 : 0] = g.y * y, J[5 < M ? 5 : 0] = g.y;
        }
        else {
          const float den = 1.0f / fmaf((float) x, jc[6], fmaf((float) y, jc[7], 1.0f));
          const float hatX = -fmaf((float) x, jc[0], fmaf((float) y, jc[1], jc[2])) * den;
          const float hatY = -fmaf((float) x, jc[3], fmaf((float) y, jc[4], jc[5])) * den;
          const float ggx = g.x * den, ggy = g.y * den, gg = hatX * ggx + hatY * ggy;
          J[0] = ggx * x, J[1] = ggx * y, J[2] = ggx;
          J[3 < M ? 3 : 0] = ggy * x, J[4 < M ? 4 : 0] = ggy * y, J[5 < M ? 5 : 0] = ggy;
          J[6 < M ? 6 : 0] = gg * x, J[7 < M ? 7 : 0] = gg * y;
        }
        for( int u = 0, kk = 0; u < M; ++u )
          for( int v = 0; v <= u; ++v, ++kk ) acc[kk] = fmaf(J[u], J[v], acc[kk]);
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for( int k = 0; k < NS; ++k ) {
    const double s = warp_sum((double) acc[k]);
    if( lane == 0 ) s_red[wid * NS + k] = s;
  }
  __syncthreads();
  for( int k = threadIdx.x; k < NS; k += 256 ) {
    double s = 0;
    for( int wv = 0; wv < 8; ++wv ) s += s_red[wv * NS + k];
    partials[(size_t) t * NS + k] = s;
  }
}

cudaError_t launch_ref_hessian(const float2 * grad, int w, int h, int jkind, int M, const float * jc,
    double * partials, int * tiles_out, cudaStream_t st)
{
  int tx;
  const int tiles = tiles_of(w, h, PW_TX, PW_TY, &tx);
  *tiles_out = tiles;
  switch ( jkind ) {
  case J_TRANS: k_ref_hessian<J_TRANS, 2><<<tiles, 256, 0, st>>>(grad, w, h, tx, jc, partials); break;
  case J_EUCL:
    if( M == 3 ) k_ref_hessian<J_EUCL, 3><<<tiles, 256, 0, st>>>(grad, w, h, tx, jc, partials);
    else k_ref_hessian<J_EUCL, 4><<<tiles, 256, 0, st>>>(grad, w, h, tx, jc, partials);
    break;
  case J_AFFINE: k_ref_hessian<J_AFFINE, 6><<<tiles, 256, 0, st>>>(grad, w, h, tx, jc, partials); break;
  case J_HOMOG: k_ref_hessian<J_HOMOG, 8><<<tiles, 256, 0, st>>>(grad, w, h, tx, jc, partials); break;
  default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

/* per-tile {sum T, n(all), n(mask != 0)} of a reference level */
__global__ void __launch_bounds__(256) k_ref_stats(const float * img, const uint8_t * mask, int w, int h, int tiles_x,
    double * partials)
{
  __shared__ double s_red[8 * 3];
  const int t = blockIdx.x;
  const int tx0 = (t % tiles_x) * PW_TX, ty0 = (t / tiles_x) * PW_TY;
  const int x = tx0 + (threadIdx.x & (PW_TX - 1));
  float acc[3] = { 0, 0, 0 };
  if( x < w ) {
    for( int k = 0; k < PW_TY / 2; ++k ) {
      const int y = ty0 + (threadIdx.x >> 7) + 2 * k;
      if( y < h ) {
        acc[0] += img[(size_t) y * w + x];
        acc[1] += 1.f;
        acc[2] += (!mask || mask[(size_t) y * w + x]) ? 1.f : 0.f;
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for( int k = 0; k < 3; ++k ) {
    const double s = warp_sum((double) acc[k]);
    if( lane == 0 ) s_red[wid * 3 + k] = s;
  }
  __syncthreads();
  if( threadIdx.x < 3 ) {
    double s = 0;
    for( int wv = 0; wv < 8; ++wv ) s += s_red[wv * 3 + threadIdx.x];
    partials[(size_t) t * 3 + threadIdx.x] = s;
  }
}

cudaError_t launch_ref_stats(const float * img, const uint8_t * mask, int w, int h, double * partials,
    int * tiles_out, cudaStream_t st)
{
  int tx;
  const int tiles = tiles_of(w, h, PW_TX, PW_TY, &tx);
  *tiles_out = tiles;
  k_ref_stats<<<tiles, 256, 0, st>>>(img, mask, w, h, tx, partials);
  return cudaGetLastError();
}

/* -------------------------------------------------- frame sharpness weight */

/* mean over the interior of a pyramid level of the squared 5-point Laplacian:
 * per-tile {sum, count} partials, combined in order by k_finalize */
constexpr int LE_TX = 128, LE_TY = 32;   // 16 pixels per thread

int lap_tiles(int w, int h)
{
  return ((w + LE_TX - 1) / LE_TX) * ((h + LE_TY - 1) / LE_TY);
}

__global__ void __launch_bounds__(256) k_lap_energy(const float * pyr, size_t pyr_stride, size_t lvl_off, int w, int h,
    double * partials, int tiles)
{
  __shared__ float s_red[8 * 2];
  const int f = blockIdx.y, t = blockIdx.x;
  const float * img = pyr + (size_t) f * pyr_stride + lvl_off;
  const int tiles_x = (w + LE_TX - 1) / LE_TX;
  const int tx0 = (t % tiles_x) * LE_TX, ty0 = (t / tiles_x) * LE_TY;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // each thread walks 16 consecutive rows of one column with the rows above and
  // below in registers; the left and right neighbours come from the adjacent
  // lanes, and the warp's outer lanes load theirs. Cells are read clamped into the
  // image; only interior pixels count.
  const int x = tx0 + (threadIdx.x & (LE_TX - 1));
  const int ya = ty0 + (threadIdx.x >> 7) * (LE_TY / 2);
  const bool inx = x >= 1 && x < w - 1;
  const float * col = img + min(x, w - 1);
  const float * side = img + clampi(lane == 0 ? x - 1 : x + 1, 0, w - 1);   // lanes 0 and 31 only
  float s = 0.f, cnt = 0.f;
  float up = __ldg(col + (size_t) clampi(ya - 1, 0, h - 1) * w);
  float c = __ldg(col + (size_t) clampi(ya, 0, h - 1) * w);
#pragma unroll 4
  for( int k = 0; k < LE_TY / 2; ++k ) {
    const int y = ya + k;
    const size_t ro = (size_t) clampi(y, 0, h - 1) * w;
    const float dn = __ldg(col + (size_t) clampi(y + 1, 0, h - 1) * w);
    float l_ = __shfl_up_sync(0xffffffffu, c, 1), r_ = __shfl_down_sync(0xffffffffu, c, 1);
    if( lane == 0 ) l_ = __ldg(side + ro);
    if( lane == 31 ) r_ = __ldg(side + ro);
    if( inx && y >= 1 && y < h - 1 ) {
      const float l = (l_ + r_) + (up + dn) - 4.f * c;
      s = fmaf(l, l, s);
      cnt += 1.f;
    }
    up = c, c = dn;
  }
  // FP32 within warps (16 values per thread, 32 lanes), FP64 across the 8 warps
  s = warp_sum(s);
  cnt = warp_sum(cnt);
  if( lane == 0 ) s_red[wid * 2] = s, s_red[wid * 2 + 1] = cnt;
  __syncthreads();
  if( threadIdx.x < 2 ) {
    double a = 0;
    for( int wv = 0; wv < 8; ++wv ) a += (double) s_red[wv * 2 + threadIdx.x];
    partials[((size_t) f * tiles + t) * 2 + threadIdx.x] = a;
  }
}

cudaError_t launch_lap_energy(const float * pyr, size_t pyr_stride, size_t lvl_off, int w, int h, int n,
    double * partials, int tiles, cudaStream_t st)
{
  k_lap_energy<<<dim3(tiles, n), 256, 0, st>>>(pyr, pyr_stride, lvl_off, w, h, partials, tiles);
  return cudaGetLastError();
}

}  // namespace sst
