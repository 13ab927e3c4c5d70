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
 * All kernels are batched over frames (grid.z) and stage halo'd tiles in
 * shared memory; each input pixel is read from HBM once per kernel.
 */
#include "sst_engine.cuh"
#include "sst_tma.cuh"

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

/* One CTA per 128 x 32 level-0 tile (and its 64 x 16 level-1 tile). One TMA
 * copy stages the raw input window (tile + 2 + R rows above and below, and
 * enough columns for the smoothed window). The window is converted to scaled
 * FP32 once. The separable 7-tap Gaussian gives the smoothed window S: 36
 * rows (level-0 y = ty0 - 2 ... ty0 + 33) by 136 columns (x = tx0 - 4 ...
 * tx0 + 131, so the tile's own cells start on a 16-byte boundary). Its tile
 * part is stored as level 0; the 5-tap pyrDown of S (rows first, as pyrDown)
 * gives level 1. So level 0 is written once and never read back.
 * Borders: out-of-image input cells take the nearest in-image cell
 * (REPLICATE, as sepFilter2D). Out-of-image cells of S that pyrDown taps
 * reach take the reflected cell (REFLECT_101, as pyrDown). */
constexpr int FP_TX = 128, FP_TY = 32, FP_R = 3;
constexpr int FP_SW = FP_TX + 8, FP_SH = FP_TY + 4;       // smoothed window
constexpr int FP_IH = FP_SH + 2 * FP_R;                   // input rows

template<typename T>
struct fp_geom {
  static constexpr int VEC = 16 / (int) sizeof(T);                          // elements per 16 bytes
  static constexpr int XA = VEC >= 7 ? VEC : 8;                            // left margin: >= 4 + R, 16 B, 4 floats
  static constexpr int IW = (XA + FP_SW + VEC - 1) / VEC * VEC;            // input row (16-byte multiple)
  static constexpr size_t IN_BYTES = ((size_t) IW * FP_IH * sizeof(T) + 127) / 128 * 128;
  static constexpr size_t F_BYTES = ((size_t) IW * FP_IH * sizeof(float) + 127) / 128 * 128;
  static constexpr size_t H_BYTES = (size_t) FP_IH * FP_SW * sizeof(float);
  static constexpr size_t SMEM = 128 + 2 * IN_BYTES + F_BYTES + H_BYTES + 32;   // two input windows
  static_assert((size_t) FP_SH * FP_SW * sizeof(float) <= F_BYTES, "S aliases the converted window");
  static_assert(XA % 4 == 0 && XA >= 4 + FP_R, "left margin");
};

/* eight consecutive elements (16-byte aligned for u16 / f32, 8-byte for u8) as floats */
__device__ __forceinline__ void load8(const uint16_t * p, float (&v)[8])
{
  const uint4 q = *reinterpret_cast<const uint4 *>(p);
  const uint32_t u[4] = { q.x, q.y, q.z, q.w };
#pragma unroll
  for( int k = 0; k < 4; ++k ) v[2 * k] = (float) (u[k] & 0xffffu), v[2 * k + 1] = (float) (u[k] >> 16);
}

__device__ __forceinline__ void load8(const uint8_t * p, float (&v)[8])
{
  const uint2 q = *reinterpret_cast<const uint2 *>(p);
#pragma unroll
  for( int k = 0; k < 4; ++k ) v[k] = (float) ((q.x >> (8 * k)) & 0xffu), v[4 + k] = (float) ((q.y >> (8 * k)) & 0xffu);
}

__device__ __forceinline__ void load8(const float * p, float (&v)[8])
{
  const float4 a = *reinterpret_cast<const float4 *>(p), b = *reinterpret_cast<const float4 *>(p + 4);
  v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
}

__device__ __forceinline__ float4 pyr5(float4 a, float4 b, float4 c, float4 d, float4 e)
{
  float4 r;
  r.x = (a.x + e.x) * 0.0625f + (b.x + d.x) * 0.25f + c.x * 0.375f;
  r.y = (a.y + e.y) * 0.0625f + (b.y + d.y) * 0.25f + c.y * 0.375f;
  r.z = (a.z + e.z) * 0.0625f + (b.z + d.z) * 0.25f + c.z * 0.375f;
  r.w = (a.w + e.w) * 0.0625f + (b.w + d.w) * 0.25f + c.w * 0.375f;
  return r;
}

/* Persistent: each CTA walks (frame, tile) items frame-major, and the input
 * window of its next item is copied into the second buffer while the current
 * item computes. */
template<typename T>
__global__ void __launch_bounds__(256, 3) k_convert_pyr1(const __grid_constant__ CUtensorMap tmap, int w, int h,
    int gx, int gy, int n, float scale, const float * __restrict__ gk, float * dst0, float * dst1, int dw, int dh,
    size_t dst_stride, int * err)
{
  using G = fp_geom<T>;
  constexpr int IW = G::IW;
  constexpr int IN_ELEMS = (int) (G::IN_BYTES / sizeof(T));
  extern __shared__ unsigned char fp_smem[];
  unsigned char * base = (unsigned char *) (((uintptr_t) fp_smem + 127) & ~(uintptr_t) 127);
  T * s_in0 = (T *) base;                                         // two FP_IH x IW raw input windows
  float * s_f = (float *) (base + 2 * G::IN_BYTES);               // FP_IH x IW scaled FP32; then S: FP_SH x FP_SW
  float * s_h = (float *) (base + 2 * G::IN_BYTES + G::F_BYTES);  // FP_IH x FP_SW horizontal pass; then pyrDown rows
  float * s_S = s_f;
  uint64_t * bar = (uint64_t *) (base + 2 * G::IN_BYTES + G::F_BYTES + G::H_BYTES);
  uint32_t * s_infl = (uint32_t *) (bar + 2);                     // copies in flight, kept by thread 0
  int * s_gaveup = (int *) (s_infl + 1);                          // [2]: a wait gave up on this buffer

  const int per_frame = gx * gy, items = per_frame * n;
  if( (int) blockIdx.x >= items ) return;                         // uniform over the CTA
  if( threadIdx.x == 0 ) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    *s_infl = 0u;
    s_gaveup[0] = s_gaveup[1] = 0;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if( threadIdx.x == 0 ) {
    const int z = blockIdx.x / per_frame, rem = blockIdx.x - z * per_frame, by = rem / gx, bx = rem - by * gx;
    mbar_expect_tx(&bar[0], IW * FP_IH * sizeof(T));
    tma_load_3d(s_in0, &tmap, bx * FP_TX - G::XA, by * FP_TY - 2 - FP_R, z, &bar[0]);
    inflight_issued(s_infl, 0, 0u);
  }
  float g[2 * FP_R + 1];
#pragma unroll
  for( int i = 0; i <= 2 * FP_R; ++i ) g[i] = __ldg(gk + i);
  uint32_t phases = 0u;
  bool timed_out = false, stop = false;
  int b = 0;
  for( int item = blockIdx.x; item < items; item += gridDim.x, b ^= 1 ) {
    // the next item's window goes into the other buffer, last read by the
    // convert pass two items ago (every thread is past the barrier after it);
    // the previous item's wait flag was written before that item's barriers
    stop = stop || s_gaveup[b ^ 1];
    const int nitem = item + gridDim.x;
    if( threadIdx.x == 0 && nitem < items && !stop ) {
      const int z = nitem / per_frame, rem = nitem - z * per_frame, by = rem / gx, bx = rem - by * gx;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&bar[b ^ 1], IW * FP_IH * sizeof(T));
      tma_load_3d(s_in0 + (b ^ 1) * IN_ELEMS, &tmap, bx * FP_TX - G::XA, by * FP_TY - 2 - FP_R, z, &bar[b ^ 1]);
      inflight_issued(s_infl, b ^ 1, (phases >> (b ^ 1)) & 1u);
    }
    const int z = item / per_frame, rem = item - z * per_frame, by = rem / gx, bx = rem - by * gx;
    const int tx0 = bx * FP_TX, ty0 = by * FP_TY;
    const int wx0 = tx0 - G::XA, wy0 = ty0 - 2 - FP_R;            // input window origin
    const T * s_in = s_in0 + b * IN_ELEMS;
    if( !stop ) {
      if( !mbar_wait_bounded(&bar[b], (phases >> b) & 1u) ) timed_out = true, s_gaveup[b] = 1;
      else if( threadIdx.x == 0 ) inflight_landed(s_infl, b);
      phases ^= 1u << b;
    }

    // convert + scale; where the window leaves the image, each cell takes the
    // nearest in-image cell (REPLICATE)
    const bool edge_in = wx0 < 0 || wx0 + IW > w || wy0 < 0 || wy0 + FP_IH > h;
    if( !edge_in ) {
      for( int q = threadIdx.x; q < FP_IH * (IW / 8); q += 256 ) {
        const int r = q / (IW / 8), c = (q - r * (IW / 8)) * 8;
        float v[8];
        load8(s_in + r * IW + c, v);
        float * o = s_f + r * IW + c;
        *reinterpret_cast<float4 *>(o) = make_float4(v[0] * scale, v[1] * scale, v[2] * scale, v[3] * scale);
        *reinterpret_cast<float4 *>(o + 4) = make_float4(v[4] * scale, v[5] * scale, v[6] * scale, v[7] * scale);
      }
    }
    else {
      for( int q = threadIdx.x; q < FP_IH * IW; q += 256 ) {
        const int r = q / IW, c = q - r * IW;
        const int rs = clampi(wy0 + r, 0, h - 1) - wy0, cs = clampi(wx0 + c, 0, w - 1) - wx0;
        s_f[q] = (float) s_in[rs * IW + cs] * scale;
      }
    }
    __syncthreads();

    // horizontal Gaussian: S column c (x = tx0 - 4 + c) reads converted columns
    // c + XA - 7 ... c + XA - 1; four columns per item from three 16-byte loads
    for( int q = threadIdx.x; q < FP_IH * (FP_SW / 4); q += 256 ) {
      const int r = q / (FP_SW / 4), c0 = (q - r * (FP_SW / 4)) * 4;
      const float * p = s_f + r * IW + c0 + G::XA - 8;
      float v[12];
  #pragma unroll
      for( int k = 0; k < 3; ++k ) {
        const float4 t = *reinterpret_cast<const float4 *>(p + 4 * k);
        v[4 * k] = t.x, v[4 * k + 1] = t.y, v[4 * k + 2] = t.z, v[4 * k + 3] = t.w;
      }
      float o[4];
  #pragma unroll
      for( int j = 0; j < 4; ++j ) {
        float a = 0.f;
  #pragma unroll
        for( int i = 0; i <= 2 * FP_R; ++i ) a = fmaf(g[i], v[j + 1 + i], a);
        o[j] = a;
      }
      *reinterpret_cast<float4 *>(s_h + r * FP_SW + c0) = make_float4(o[0], o[1], o[2], o[3]);
    }
    __syncthreads();

    // vertical Gaussian: S row s (y = ty0 - 2 + s) reads rows s ... s + 2R of the
    // horizontal pass; 4 rows x 4 columns per item (S overwrites the converted window)
    for( int q = threadIdx.x; q < (FP_SH / 4) * (FP_SW / 4); q += 256 ) {
      const int rg = q / (FP_SW / 4), c0 = (q - rg * (FP_SW / 4)) * 4, s0 = rg * 4;
      float4 v[4 + 2 * FP_R];
  #pragma unroll
      for( int i = 0; i < 4 + 2 * FP_R; ++i ) v[i] = *reinterpret_cast<const float4 *>(s_h + (s0 + i) * FP_SW + c0);
  #pragma unroll
      for( int j = 0; j < 4; ++j ) {
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
  #pragma unroll
        for( int i = 0; i <= 2 * FP_R; ++i ) {
          a.x = fmaf(g[i], v[j + i].x, a.x), a.y = fmaf(g[i], v[j + i].y, a.y);
          a.z = fmaf(g[i], v[j + i].z, a.z), a.w = fmaf(g[i], v[j + i].w, a.w);
        }
        *reinterpret_cast<float4 *>(s_S + (s0 + j) * FP_SW + c0) = a;
      }
    }
    __syncthreads();

    // level 0: the tile's cells of S (rows 2 ... 33, columns 4 ... 131)
    float * out0 = dst0 + (size_t) z * dst_stride;
    const bool vec0 = (w & 3) == 0;
    for( int q = threadIdx.x; q < FP_TY * (FP_TX / 4); q += 256 ) {
      const int i = q / (FP_TX / 4), k = q - i * (FP_TX / 4);
      const int y = ty0 + i, x = tx0 + 4 * k;
      if( y >= h || x >= w ) continue;
      const float4 v = *reinterpret_cast<const float4 *>(s_S + (i + 2) * FP_SW + 4 + 4 * k);
      float * o = out0 + (size_t) y * w + x;
      if( vec0 && x + 3 < w ) *reinterpret_cast<float4 *>(o) = v;
      else {
        o[0] = v.x;
        if( x + 1 < w ) o[1] = v.y;
        if( x + 2 < w ) o[2] = v.z;
        if( x + 3 < w ) o[3] = v.w;
      }
    }

    // REFLECT_101 the cells of S that pyrDown taps reach outside the image
    // (x in {-2, -1, w, w + 1}, then y likewise), from in-image cells of S
    const bool edge_s = tx0 == 0 || ty0 == 0 || tx0 + FP_TX + 4 > w || ty0 + FP_TY + 2 > h;
    if( edge_s ) {
      for( int q = threadIdx.x; q < FP_SH * 4; q += 256 ) {
        const int s = q >> 2, k = q & 3;
        const int x = k < 2 ? k - 2 : w + k - 2, c = x - (tx0 - 4);
        if( c >= 0 && c < FP_SW ) s_S[s * FP_SW + c] = s_S[s * FP_SW + clampi(reflect101(x, w) - (tx0 - 4), 0, FP_SW - 1)];
      }
      __syncthreads();
      for( int q = threadIdx.x; q < 4 * FP_SW; q += 256 ) {
        const int k = q / FP_SW, c = q - k * FP_SW;
        const int y = k < 2 ? k - 2 : h + k - 2, s = y - (ty0 - 2);
        if( s >= 0 && s < FP_SH ) s_S[s * FP_SW + c] = s_S[clampi(reflect101(y, h) - (ty0 - 2), 0, FP_SH - 1) * FP_SW + c];
      }
    }
    __syncthreads();

    // pyrDown [1 4 6 4 1] / 16, rows first (as pyrDown): level-1 column j
    // (x = tx0 + 2j) reads S columns 2j + 2 ... 2j + 6; four columns per item
    constexpr int TX1 = FP_TX / 2, TY1 = FP_TY / 2;
    float * s_p = s_h;                                              // FP_SH x TX1
    for( int q = threadIdx.x; q < FP_SH * (TX1 / 4); q += 256 ) {
      const int s = q / (TX1 / 4), k = q - s * (TX1 / 4);
      const float * p = s_S + s * FP_SW + 8 * k;
      float v[16];
  #pragma unroll
      for( int m = 0; m < 4; ++m ) {
        const float4 t = *reinterpret_cast<const float4 *>(p + 4 * m);
        v[4 * m] = t.x, v[4 * m + 1] = t.y, v[4 * m + 2] = t.z, v[4 * m + 3] = t.w;
      }
      float o[4];
  #pragma unroll
      for( int m = 0; m < 4; ++m ) {
        const float * a = v + 2 * m + 2;
        o[m] = (a[0] + a[4]) * 0.0625f + (a[1] + a[3]) * 0.25f + a[2] * 0.375f;
      }
      *reinterpret_cast<float4 *>(s_p + s * TX1 + 4 * k) = make_float4(o[0], o[1], o[2], o[3]);
    }
    __syncthreads();
    // then columns: level-1 row i (y = ty0 + 2i) reads rows 2i ... 2i + 4
    float * out1 = dst1 + (size_t) z * dst_stride;
    const bool vec1 = (dw & 3) == 0;
    for( int q = threadIdx.x; q < TY1 * (TX1 / 4); q += 256 ) {
      const int i = q / (TX1 / 4), k = q - i * (TX1 / 4);
      const int y1 = ty0 / 2 + i, x1 = tx0 / 2 + 4 * k;
      if( y1 >= dh || x1 >= dw ) continue;
      const float * p = s_p + (2 * i) * TX1 + 4 * k;
      const float4 o = pyr5(*reinterpret_cast<const float4 *>(p), *reinterpret_cast<const float4 *>(p + TX1),
          *reinterpret_cast<const float4 *>(p + 2 * TX1), *reinterpret_cast<const float4 *>(p + 3 * TX1),
          *reinterpret_cast<const float4 *>(p + 4 * TX1));
      float * d = out1 + (size_t) y1 * dw + x1;
      if( vec1 && x1 + 3 < dw ) *reinterpret_cast<float4 *>(d) = o;
      else {
        d[0] = o.x;
        if( x1 + 1 < dw ) d[1] = o.y;
        if( x1 + 2 < dw ) d[2] = o.z;
        if( x1 + 3 < dw ) d[3] = o.w;
      }
    }
  }
  if( threadIdx.x == 0 ) inflight_drain(s_infl, bar);
  if( timed_out && err ) atomicExch(err, 1);
}

template<typename T>
static cudaError_t launch_fp(const CUtensorMap & map, int n, int w, int h, float scale, const float * gk, float * dst0,
    float * dst1, int dw, int dh, size_t dst_stride, int * err, cudaStream_t st)
{
  static int slots = 0;                       // resident CTAs on the device
  if( !slots ) {
    cudaError_t e = cudaFuncSetAttribute(k_convert_pyr1<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) fp_geom<T>::SMEM);
    if( e != cudaSuccess ) return e;
    int dev = 0, sms = 0, per_sm = 0;
    if( (e = cudaGetDevice(&dev)) != cudaSuccess ) return e;
    if( (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ) return e;
    if( (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_convert_pyr1<T>, 256, fp_geom<T>::SMEM)) != cudaSuccess )
      return e;
    slots = sms * (per_sm > 0 ? per_sm : 1);
  }
  const int gx = (w + FP_TX - 1) / FP_TX, gy = (h + FP_TY - 1) / FP_TY;
  const long long items = (long long) gx * gy * n;
  if( items > (1ll << 30) ) return cudaErrorInvalidValue;
  const int grid = (int) (items < slots ? items : slots);
  k_convert_pyr1<T><<<grid, 256, fp_geom<T>::SMEM, st>>>(map, w, h, gx, gy, n, scale, gk, dst0, dst1, dw, dh, dst_stride, err);
  return cudaGetLastError();
}

/* Level 0 and level 1 of n frames in one pass when the pre-smoothing is the
 * 7-tap Gaussian and the frames meet the TMA layout rules; *done = false
 * (nothing launched) otherwise, and the caller builds the levels separately. */
cudaError_t launch_convert_pyr1(const void * src, int depth, int n, int w, int h, size_t row_stride,
    size_t frame_stride, double scale, const float * gk, int ksize, float * dst0, float * dst1, int dw, int dh,
    size_t dst_stride, int * err, cudaStream_t st, bool * done)
{
  *done = false;
  if( !gk || ksize != 2 * FP_R + 1 || w < 8 || h < 8 || n < 1 || n > 65535 || 2 * dw > w + 1 || 2 * dh > h + 1 )
    return cudaSuccess;
  CUtensorMap map;
  const uint64_t dims[3] = { (uint64_t) w, (uint64_t) h, (uint64_t) n };
  const uint64_t strides[2] = { (uint64_t) row_stride, (uint64_t) (n > 1 ? frame_stride : row_stride * h) };
  cudaError_t e = cudaSuccess;
  switch ( depth ) {
  case SST_DEPTH_U8: {
    const uint32_t box[3] = { (uint32_t) fp_geom<uint8_t>::IW, (uint32_t) FP_IH, 1 };
    if( !encode_tensor_3d(&map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, src, dims, strides, box) ) return cudaSuccess;
    e = launch_fp<uint8_t>(map, n, w, h, (float) scale, gk, dst0, dst1, dw, dh, dst_stride, err, st);
    break;
  }
  case SST_DEPTH_U16: {
    const uint32_t box[3] = { (uint32_t) fp_geom<uint16_t>::IW, (uint32_t) FP_IH, 1 };
    if( !encode_tensor_3d(&map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, src, dims, strides, box) ) return cudaSuccess;
    e = launch_fp<uint16_t>(map, n, w, h, (float) scale, gk, dst0, dst1, dw, dh, dst_stride, err, st);
    break;
  }
  case SST_DEPTH_F32: {
    const uint32_t box[3] = { (uint32_t) fp_geom<float>::IW, (uint32_t) FP_IH, 1 };
    if( !encode_tensor_3d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src, dims, strides, box) ) return cudaSuccess;
    e = launch_fp<float>(map, n, w, h, (float) scale, gk, dst0, dst1, dw, dh, dst_stride, err, st);
    break;
  }
  default: return cudaSuccess;
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
  float s = 0.f, cnt = 0.f;
  const int x = tx0 + (threadIdx.x & (LE_TX - 1));
  if( x >= 1 && x < w - 1 ) {
#pragma unroll 4
    for( int k = 0; k < LE_TY / 2; ++k ) {
      const int y = ty0 + (threadIdx.x >> 7) + 2 * k;
      if( y >= 1 && y < h - 1 ) {
        const float * p = img + (size_t) y * w + x;
        const float l = (__ldg(p - 1) + __ldg(p + 1)) + (__ldg(p - w) + __ldg(p + w)) - 4.f * __ldg(p);
        s = fmaf(l, l, s);
        cnt += 1.f;
      }
    }
  }
  // FP32 within warps (16 values per thread, 32 lanes), FP64 across the 8 warps
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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
