/*
 * sst_stack.cu -- warp + weighted accumulation kernels (sm_103a).
 *
 *   batched warp + stack : c_frame_registration::base_remap
 *                          (c_frame_registration.cc:1265-1340) fused with
 *                          multiply_weights (c_image_stacking_pipeline.cc:1704-1714)
 *                          and c_weigthed_average::add (c_frame_accumulation.cc:182-221)
 *   plain add            : _weighted_average_update (c_frame_accumulation.cc:20-129)
 *   compute              : c_weigthed_average::compute (c_frame_accumulation.cc:223-248)
 *   remap                : base_remap for one frame (image + mask)
 *   Bayer planes         : extract_bayer_planes / average_bayer_planes (debayer.cc:96-147, 277-330)
 *
 * Accumulator layout in HBM: four planar FP32 planes of width x height:
 * S (sum of w*I), cS (its Kahan-Babuska compensation), W (sum of w), cW.
 * The batched kernel assigns each output pixel to one thread, which warps
 * and accumulates the frames of its chunk (partial sums in registers,
 * compensated sums in thread-private shared slots) and touches the
 * accumulator planes once per batch: no atomics, deterministic.
 */
#include <mutex>
#include "sst_engine.cuh"
#include "sst_stack.cuh"
#include "sst_tma.cuh"

namespace sst {

template<typename T>
__device__ __forceinline__ float ldpx(const uint8_t * base, size_t row_stride, int x, int y)
{
  return (float) __ldg((const T *) (base + (size_t) y * row_stride) + x);
}

/* per-frame FP32 displacement coefficients from API parameter vectors */
__global__ void k_coeffs_from_params(sst_motion_model m, const float * params, int n, float * coeffs)
{
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if( f >= n ) return;
  double s[16], p[12];
  model_identity(m, s);
  const int M = model_nparams(m);
  for( int j = 0; j < M; ++j ) p[j] = params[(size_t) f * 12 + j];
  model_set_params(m, s, p);
  model_warp_coeffs(m, s, coeffs + (size_t) f * SST_NCOEF);
}

cudaError_t launch_coeffs_from_params(const sst_motion_model & m, const float * params, int n, float * coeffs, cudaStream_t st)
{
  k_coeffs_from_params<<<(n + 127) / 128, 128, 0, st>>>(m, params, n, coeffs);
  return cudaGetLastError();
}

/* effective per-frame weight: weight (or 1) where status == OK, else 0 */
__global__ void k_effective_weights(const float * weights, const int32_t * status, int n, float * out)
{
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if( f >= n ) return;
  float w = weights ? weights[f] : 1.0f;
  if( status && status[f] != SST_FRAME_OK ) w = 0.f;
  out[f] = w > 0 ? w : 0.f;
}

cudaError_t launch_effective_weights(const float * weights, const int32_t * status, int n, float * out, cudaStream_t st)
{
  k_effective_weights<<<(n + 127) / 128, 128, 0, st>>>(weights, status, n, out);
  return cudaGetLastError();
}

/* one bilinear tap with the remap border mode (cv::remap, per-tap borderInterpolate) */
template<typename T>
__device__ __forceinline__ float tap(const uint8_t * fb, size_t rs, int sw, int sh, int xi, int yi, int border)
{
  if( xi >= 0 && xi < sw && yi >= 0 && yi < sh ) return ldpx<T>(fb, rs, xi, yi);
  switch ( border ) {
  case SST_BORDER_REPLICATE: return ldpx<T>(fb, rs, clampi(xi, 0, sw - 1), clampi(yi, 0, sh - 1));
  case SST_BORDER_REFLECT101: return ldpx<T>(fb, rs, reflect101(xi, sw), reflect101(yi, sh));
  case SST_BORDER_REFLECT: return ldpx<T>(fb, rs, reflect(xi, sw), reflect(yi, sh));
  default: return 0.f;
  }
}

constexpr int SK_TX = 32, SK_TY = 8;          // remap utility tile
constexpr int SA_TX = 64, SA_TY = 16;         // batched stack tile: 4 pixels per thread

/* frames accumulated in plain FP32 per pixel before each compensated merge */
constexpr int SA_FLUSH = 16;

/* L2 prefetch of the source footprint of frame f's tile (rows ty0 - 2 ..
 * ty0 + SA_TY + 1, both ends of each row): 40 threads, one line each */
template<typename T>
__device__ __forceinline__ void prefetch_footprint(const StackArgs & a, int f, int tx0, int ty0)
{
  if( threadIdx.x >= 2 * (SA_TY + 4) ) return;
  const float * c = a.coeffs + (size_t) f * SST_NCOEF;
  const int y = ty0 - 2 + (threadIdx.x >> 1), x = tx0 + (threadIdx.x & 1) * (SA_TX - 1);
  const float dx = fmaf(__ldg(c + 0), (float) x, fmaf(__ldg(c + 1), (float) y, __ldg(c + 2)));
  const float dy = fmaf(__ldg(c + 3), (float) x, fmaf(__ldg(c + 4), (float) y, __ldg(c + 5)));
  const int sx = clampi(x + (int) __ldg(c + 12) + (int) floorf(fminf(fmaxf(dx, -1e6f), 1e6f)), 0, a.sw - 1);
  const int sy = clampi(y + (int) __ldg(c + 13) + (int) floorf(fminf(fmaxf(dy, -1e6f), 1e6f)), 0, a.sh - 1);
  const uint8_t * p = a.frames + (size_t) f * a.frame_stride + (size_t) sy * a.row_stride + (size_t) sx * sizeof(T);
  asm volatile("prefetch.global.L2 [%0];" :: "l"(p));
}

template<int FAM, typename T>
__global__ void __launch_bounds__(256) k_stack_add_warped(StackArgs a)
{
  constexpr int VW = SA_TX + 4, VH = SA_TY + 4;
  constexpr int PPT = SA_TX * SA_TY / 256;
  __shared__ uint8_t s_v[VH * VW];
  __shared__ uint8_t s_h[VH * SA_TX];
  const int tx0 = blockIdx.x * SA_TX, ty0 = blockIdx.y * SA_TY;
  const int lx = threadIdx.x % SA_TX, ly0 = threadIdx.x / SA_TX;
  const int x = tx0 + lx;
  // window whose validity decides the tile's eroded mask (tile + 2 px halo, clipped)
  const int wx0 = max(tx0 - 2, 0), wy0 = max(ty0 - 2, 0);
  const int wx1 = min(tx0 + SA_TX + 1, a.dw - 1), wy1 = min(ty0 + SA_TY + 1, a.dh - 1);
  // compensated running sums, and plain FP32 partials of up to SA_FLUSH frames
  float S[PPT], cS[PPT], Wt[PPT], cW[PPT], pS[PPT], pW[PPT];
#pragma unroll
  for( int k = 0; k < PPT; ++k ) S[k] = cS[k] = Wt[k] = cW[k] = pS[k] = pW[k] = 0.f;
  int since = 0;                                // frames in the partials (uniform over the CTA)
  if( a.n > 0 ) prefetch_footprint<T>(a, 0, tx0, ty0);
  for( int f = 0; f < a.n; ++f ) {
    const float wf = __ldg(a.weights + f);
    if( !(wf > 0.f) ) continue;                 // uniform over the CTA
    if( f + 1 < a.n ) prefetch_footprint<T>(a, f + 1, tx0, ty0);
    float c[SST_NCOEF];
#pragma unroll
    for( int i = 0; i < SST_NCOEF; ++i ) c[i] = __ldg(a.coeffs + (size_t) f * SST_NCOEF + i);
    const uint8_t * fb = a.frames + (size_t) f * a.frame_stride;
    if( rect_interior<FAM>(c, wx0, wy0, wx1, wy1, a.sw, a.sh) ) {
      // every pixel of the window is valid and every tap is inside the frame:
      // issue the taps of all PPT pixels before using any (one memory round trip)
      if( x < a.dw ) {
        float v[PPT][4], fx[PPT], fy[PPT];
#pragma unroll
        for( int k = 0; k < PPT; ++k ) {
          const int y = min(ty0 + ly0 + 4 * k, a.dh - 1);
          const spos s = warp_pos<FAM>(c, x, y);
          const T * r0 = (const T *) (fb + (size_t) s.y0 * a.row_stride) + s.x0;
          const T * r1 = (const T *) ((const uint8_t *) r0 + a.row_stride);
          v[k][0] = (float) __ldg(r0), v[k][1] = (float) __ldg(r0 + 1);
          v[k][2] = (float) __ldg(r1), v[k][3] = (float) __ldg(r1 + 1);
          fx[k] = s.fx, fy[k] = s.fy;
        }
#pragma unroll
        for( int k = 0; k < PPT; ++k ) {
          const int y = ty0 + ly0 + 4 * k;
          if( y < a.dh ) {
            const float t0 = fmaf(fx[k], v[k][1] - v[k][0], v[k][0]), t1 = fmaf(fx[k], v[k][3] - v[k][2], v[k][2]);
            const float val = fmaf(fy[k], t1 - t0, t0) * a.scale;
            const float wp = a.wmap ? wf * __ldg(a.wmap + (size_t) f * a.plane + (size_t) y * a.dw + x) : wf;
            pS[k] = fmaf(wp, val, pS[k]);
            pW[k] += wp;
          }
        }
      }
    }
    else {
      // remap(255-mask, LINEAR, CONSTANT 0) >= 255 over the tile + 2 px halo;
      // positions outside the output count as 255 (erode border value)
      for( int q = threadIdx.x; q < VW * VH; q += 256 ) {
        const int qx = tx0 - 2 + q % VW, qy = ty0 - 2 + q / VW;
        uint8_t v = 1;
        if( qx >= 0 && qx < a.dw && qy >= 0 && qy < a.dh ) {
          v = mask_ok(coverage(a.sw, a.sh, warp_pos<FAM>(c, qx, qy)), 255) ? 1 : 0;
        }
        s_v[q] = v;
      }
      __syncthreads();
      for( int q = threadIdx.x; q < SA_TX * VH; q += 256 ) {
        const int xx = q % SA_TX, yy = q / SA_TX;
        const uint8_t * p = s_v + yy * VW + xx;
        s_h[yy * SA_TX + xx] = p[0] & p[1] & p[2] & p[3] & p[4];
      }
      __syncthreads();
      if( x < a.dw ) {
#pragma unroll
        for( int k = 0; k < PPT; ++k ) {
          const int ly = ly0 + 4 * k, y = ty0 + ly;
          if( y >= a.dh ) continue;
          const uint8_t * p = s_h + ly * SA_TX + lx;
          if( p[0] & p[SA_TX] & p[2 * SA_TX] & p[3 * SA_TX] & p[4 * SA_TX] ) {
            const spos s = warp_pos<FAM>(c, x, y);
            // the >= 255 test admits footprints with < 0.2 % of the weight outside the
            // frame: those taps take the image border mode (base_remap's cv::remap)
            const float v00 = tap<T>(fb, a.row_stride, a.sw, a.sh, s.x0, s.y0, a.border);
            const float v01 = tap<T>(fb, a.row_stride, a.sw, a.sh, s.x0 + 1, s.y0, a.border);
            const float v10 = tap<T>(fb, a.row_stride, a.sw, a.sh, s.x0, s.y0 + 1, a.border);
            const float v11 = tap<T>(fb, a.row_stride, a.sw, a.sh, s.x0 + 1, s.y0 + 1, a.border);
            const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
            const float val = fmaf(s.fy, t1 - t0, t0) * a.scale;
            const float wp = a.wmap ? wf * __ldg(a.wmap + (size_t) f * a.plane + (size_t) y * a.dw + x) : wf;
            pS[k] = fmaf(wp, val, pS[k]);
            pW[k] += wp;
          }
        }
      }
      __syncthreads();
    }
    if( ++since == SA_FLUSH ) {
#pragma unroll
      for( int k = 0; k < PPT; ++k ) {
        kahan_add(S[k], cS[k], pS[k]);
        kahan_add(Wt[k], cW[k], pW[k]);
        pS[k] = pW[k] = 0.f;
      }
      since = 0;
    }
  }
  if( x < a.dw ) {
#pragma unroll
    for( int k = 0; k < PPT; ++k ) {
      const int y = ty0 + ly0 + 4 * k;
      if( y >= a.dh ) continue;
      kahan_add(S[k], cS[k], pS[k]);
      kahan_add(Wt[k], cW[k], pW[k]);
      const size_t i = (size_t) y * a.dw + x;
      float gS = a.acc[i], gcS = a.acc[a.plane + i], gW = a.acc[2 * a.plane + i], gcW = a.acc[3 * a.plane + i];
      kahan_add(gS, gcS, S[k]);
      gcS += cS[k];
      kahan_add(gW, gcW, Wt[k]);
      gcW += cW[k];
      a.acc[i] = gS, a.acc[a.plane + i] = gcS, a.acc[2 * a.plane + i] = gW, a.acc[3 * a.plane + i] = gcW;
    }
  }
}

/* ------------------------------------------- TMA-staged batched stack */

/* Work item L of the batched stack grid: (tile, frame chunk). The tiles of
 * the outer ring come first (their frames often need the validity / border
 * path, so their CTAs run longest), then the inner tiles; the chunks of a tile
 * are consecutive items. */
__device__ __forceinline__ void stack_item(int L, int tx, int ty, int chunks, int & tile, int & chunk)
{
  const int ring = (tx > 2 && ty > 2) ? 2 * tx + 2 * (ty - 2) : 0;
  if( L < ring * chunks ) {
    const int r = L / chunks;
    chunk = L - r * chunks;
    if( r < tx ) tile = r;                                          // top row
    else if( r < 2 * tx ) tile = (ty - 1) * tx + (r - tx);          // bottom row
    else if( r < 2 * tx + ty - 2 ) tile = (1 + r - 2 * tx) * tx;    // left column
    else tile = (1 + r - 2 * tx - (ty - 2)) * tx + tx - 1;         // right column
    return;
  }
  const int q = (L - ring * chunks) / chunks;
  chunk = (L - ring * chunks) - q * chunks;
  if( !ring ) { tile = q; return; }
  tile = (1 + q / (tx - 2)) * tx + 1 + q % (tx - 2);
}

/* adds the partial sums of chunks 1 .. K - 1 into the accumulator, in chunk
 * order (the same compensated update the chunk-0 CTAs made) */
__global__ void k_stack_merge_chunks(float * acc, const float * part, size_t plane, int parts)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= plane ) return;
  float gS = acc[i], gcS = acc[plane + i], gW = acc[2 * plane + i], gcW = acc[3 * plane + i];
  for( int j = 0; j < parts; ++j ) {
    const float * P = part + (size_t) j * 4 * plane;
    kahan_add(gS, gcS, P[i]);
    gcS += P[plane + i];
    kahan_add(gW, gcW, P[2 * plane + i]);
    gcW += P[3 * plane + i];
  }
  acc[i] = gS, acc[plane + i] = gcS, acc[2 * plane + i] = gW, acc[3 * plane + i] = gcW;
}

/* Eroded validity of output pixel (x, y) for the projective family: the
 * reference's mask is remap(255, LINEAR, BORDER_CONSTANT 0) >= 255 eroded
 * 5 x 5 (window clipped to the output). The set of output positions whose
 * sample has full in-image coverage is convex (the coverage wx(X) wy(Y) is
 * log-concave in the source position, so its superlevel set is convex, and
 * its preimage under a projective map with w > 0 is convex), so the window
 * is valid exactly when its four corners are. */
template<int FAM>
__device__ __forceinline__ bool window_valid(const float * c, int x, int y, int dw, int dh, int sw, int sh)
{
  const int xa = max(x - 2, 0), xb = min(x + 2, dw - 1), ya = max(y - 2, 0), yb = min(y + 2, dh - 1);
  return mask_ok(coverage(sw, sh, warp_pos<FAM>(c, xa, ya)), 255) &&
      mask_ok(coverage(sw, sh, warp_pos<FAM>(c, xb, ya)), 255) &&
      mask_ok(coverage(sw, sh, warp_pos<FAM>(c, xa, yb)), 255) &&
      mask_ok(coverage(sw, sh, warp_pos<FAM>(c, xb, yb)), 255);
}

/* The batched stack for the affine and projective families, one output
 * pixel column of SA_PPT consecutive rows per thread, every warp on its own:
 * no shared memory and no barrier inside the frame loop. Each warp tests
 * its own 5 x 5 window region (the rect_interior test: every window pixel
 * valid, every tap inside the frame) for 8 frames at once, one corner and
 * frame per lane; inside, its pixels sample the frame
 * directly with positions stepped along the column and 32-bit element
 * offsets; otherwise each pixel tests its window by its four corners
 * (window_valid) and samples with the border mode. Partial sums of SA_FLUSH
 * frames go into compensated sums; chunk > 0 writes its sums to the scratch
 * planes for k_stack_merge_chunks. WMAP: per-pixel weight maps. */
constexpr int SA_PPT = 4, SA_GRP = 4;

template<int FAM, typename T, bool WMAP>
__global__ void __launch_bounds__(256, 4) k_stack_add_streamed(StackArgs a, int chunks)
{
  int tile, chunk;
  const int tiles_x = (a.dw + SA_TX - 1) / SA_TX;
  stack_item((int) blockIdx.x, tiles_x, (a.dh + SA_TY - 1) / SA_TY, chunks, tile, chunk);
  const int tx0 = (tile % tiles_x) * SA_TX, ty0 = (tile / tiles_x) * SA_TY;
  const int f0 = (int) ((long long) chunk * a.n / chunks), nf = (int) ((long long) (chunk + 1) * a.n / chunks) - f0;
  const int lx = threadIdx.x % SA_TX, yb = ty0 + (threadIdx.x / SA_TX) * SA_PPT;
  const int x = tx0 + lx;
  // this warp's pixels: 32 columns x SA_PPT rows; its 5 x 5 window region, clipped
  const int xw = tx0 + (lx & ~31);
  const int wx0 = max(xw - 2, 0), wx1 = min(xw + 33, a.dw - 1);
  const int wy0 = max(yb - 2, 0), wy1 = min(yb + SA_PPT + 1, a.dh - 1);
  const bool active = xw < a.dw && yb < a.dh;           // warp-uniform
  const bool xin = x < a.dw;
  const bool rows_in = yb + SA_PPT <= a.dh;             // warp-uniform: every row of the column exists
  const int rse = (int) (a.row_stride / sizeof(T));     // row stride in elements
  // compensated sums in thread-private shared slots [sum][pixel][thread]; partials in registers
  __shared__ float s_acc[4][SA_PPT][256];
  float pS[SA_PPT], pW[SA_PPT];
#pragma unroll
  for( int k = 0; k < SA_PPT; ++k ) {
    pS[k] = pW[k] = 0.f;
    s_acc[0][k][threadIdx.x] = s_acc[1][k][threadIdx.x] = s_acc[2][k][threadIdx.x] = s_acc[3][k][threadIdx.x] = 0.f;
  }
  int since = 0;
  const float fxc = (float) x, fyb = (float) yb;
  const float sc = a.scale;
  const int lane = threadIdx.x & 31;
  unsigned inner8 = 0u;                           // rect_interior of the window region, 8 frames at a time
  for( int j = 0; j < nf && active; ++j ) {
    const int f = f0 + j;
    if( (j & 7) == 0 ) {
      // lane l tests corner l & 3 of the window region for frame f + (l >> 2)
      const int fl = f + (lane >> 2);
      bool ok = false;
      if( fl < f0 + nf && FAM != FAM_QUAD ) {
        const float4 * cq = (const float4 *) (a.coeffs + (size_t) fl * SST_NCOEF);
        const float4 r0 = __ldg(cq), r1 = __ldg(cq + 1), r3 = __ldg(cq + 3);
        float cc[SST_NCOEF];
        cc[0] = r0.x, cc[1] = r0.y, cc[2] = r0.z, cc[3] = r0.w, cc[4] = r1.x, cc[5] = r1.y, cc[6] = r1.z, cc[7] = r1.w;
        cc[8] = cc[9] = cc[10] = cc[11] = 0.f;
        cc[12] = r3.x, cc[13] = r3.y, cc[14] = r3.z, cc[15] = r3.w;
        const int qx = (lane & 1) ? wx1 : wx0, qy = (lane & 2) ? wy1 : wy0;
        ok = point_interior<FAM>(cc, qx, qy, a.sw, a.sh);
      }
      inner8 = __ballot_sync(0xffffffffu, ok);
    }
    const bool inner = ((inner8 >> (4 * (j & 7))) & 0xFu) == 0xFu;
    const float wf = __ldg(a.weights + f);
    if( !(wf > 0.f) ) continue;                   // uniform over the CTA
    const float4 * cp = (const float4 *) (a.coeffs + (size_t) f * SST_NCOEF);
    const float4 q0 = __ldg(cp), q1 = __ldg(cp + 1), q3 = __ldg(cp + 3);
    float c[SST_NCOEF];
    c[0] = q0.x, c[1] = q0.y, c[2] = q0.z, c[3] = q0.w, c[4] = q1.x, c[5] = q1.y, c[6] = q1.z, c[7] = q1.w;
    c[8] = c[9] = c[10] = c[11] = 0.f;
    c[12] = q3.x, c[13] = q3.y, c[14] = q3.z, c[15] = q3.w;
    const T * fb = (const T *) (a.frames + (size_t) f * a.frame_stride);
    if( inner ) {
      if( xin ) {
        // displacements along the column as functions of t = y - yb (as warp_disp)
        const int Ix = (int) c[12], Iy = (int) c[13];
        float e0, e1, e2 = 0.f, e3 = 0.f, e4 = 0.f;
        if( FAM == FAM_AFFINE ) {
          e0 = fmaf(c[0], fxc, fmaf(c[1], fyb, c[2]));
          e1 = fmaf(c[3], fxc, fmaf(c[4], fyb, c[5]));
        }
        else {
          const float X1 = fxc + c[12], Y1 = fyb + c[13];
          const float qq = fmaf(c[6], fxc, c[7] * fyb);
          e0 = 1.0f + qq;
          e1 = fmaf(-qq, X1, fmaf(c[0], fxc, fmaf(c[1], fyb, c[2])));
          e2 = fmaf(-c[7], X1, c[1]);
          e3 = fmaf(-qq, Y1, fmaf(c[3], fxc, fmaf(c[4], fyb, c[5])));
          e4 = fmaf(-c[7], Y1, c[4] - qq);
        }
        // element offset of (x + Ix, yb + Iy); rows past the output's last one
        // sample its last row (inside the tested window)
        const int obase = (yb + Iy) * rse + x + Ix;
        const float wsc = wf * sc;
        // SA_GRP pixels' taps in flight at a time
#pragma unroll
        for( int g = 0; g < SA_PPT; g += SA_GRP ) {
          float v[SA_GRP][4], fx[SA_GRP], fy[SA_GRP];
#pragma unroll
          for( int q = 0; q < SA_GRP; ++q ) {
            const int k = g + q;
            const float t = (float) k;
            float dx, dy;
            if( FAM == FAM_AFFINE ) {
              dx = fmaf(c[1], t, e0);
              dy = fmaf(c[4], t, e1);
            }
            else {
              const float iw = __fdividef(1.0f, fmaf(c[7], t, e0));
              dx = fmaf(e2, t, e1) * iw;
              dy = fmaf(t, fmaf(-c[7], t, e4), e3) * iw;
            }
            const float ix = floorf(dx), iy = floorf(dy);
            fx[q] = dx - ix, fy[q] = dy - iy;
            const int kk = rows_in ? k : min(yb + k, a.dh - 1) - yb;
            const T * r0 = fb + (obase + (kk + (int) iy) * rse + (int) ix);
            v[q][0] = (float) __ldg(r0), v[q][1] = (float) __ldg(r0 + 1);
            v[q][2] = (float) __ldg(r0 + rse), v[q][3] = (float) __ldg(r0 + rse + 1);
          }
#pragma unroll
          for( int q = 0; q < SA_GRP; ++q ) {
            const int k = g + q;
            if( rows_in || yb + k < a.dh ) {
              const float t0 = fmaf(fx[q], v[q][1] - v[q][0], v[q][0]), t1 = fmaf(fx[q], v[q][3] - v[q][2], v[q][2]);
              const float val = fmaf(fy[q], t1 - t0, t0);
              if( WMAP ) {
                const float wp = wf * __ldg(a.wmap + (size_t) f * a.plane + (size_t) (yb + k) * a.dw + x);
                pS[k] = fmaf(wp, val * sc, pS[k]);
                pW[k] += wp;
              }
              else {
                pS[k] = fmaf(wsc, val, pS[k]);
                pW[k] += wf;
              }
            }
          }
        }
      }
    }
    else if( xin ) {
#pragma unroll
      for( int k = 0; k < SA_PPT; ++k ) {
        const int y = yb + k;
        if( y < a.dh && window_valid<FAM>(c, x, y, a.dw, a.dh, a.sw, a.sh) ) {
          const spos s = warp_pos<FAM>(c, x, y);
          float v00, v01, v10, v11;
          if( s.x0 >= 0 && s.x0 < a.sw - 1 && s.y0 >= 0 && s.y0 < a.sh - 1 ) {
            const T * r0 = fb + (s.y0 * rse + s.x0);
            v00 = (float) __ldg(r0), v01 = (float) __ldg(r0 + 1), v10 = (float) __ldg(r0 + rse), v11 = (float) __ldg(r0 + rse + 1);
          }
          else {
            // < 0.2 % of the weight may fall outside: those taps take the image border mode
            const uint8_t * fbb = (const uint8_t *) fb;
            v00 = tap<T>(fbb, a.row_stride, a.sw, a.sh, s.x0, s.y0, a.border);
            v01 = tap<T>(fbb, a.row_stride, a.sw, a.sh, s.x0 + 1, s.y0, a.border);
            v10 = tap<T>(fbb, a.row_stride, a.sw, a.sh, s.x0, s.y0 + 1, a.border);
            v11 = tap<T>(fbb, a.row_stride, a.sw, a.sh, s.x0 + 1, s.y0 + 1, a.border);
          }
          const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
          const float val = fmaf(s.fy, t1 - t0, t0) * sc;
          const float wp = WMAP ? wf * __ldg(a.wmap + (size_t) f * a.plane + (size_t) y * a.dw + x) : wf;
          pS[k] = fmaf(wp, val, pS[k]);
          pW[k] += wp;
        }
      }
    }
    if( ++since == SA_FLUSH ) {
#pragma unroll
      for( int k = 0; k < SA_PPT; ++k ) {
        float S = s_acc[0][k][threadIdx.x], cS = s_acc[1][k][threadIdx.x];
        float Wt = s_acc[2][k][threadIdx.x], cW = s_acc[3][k][threadIdx.x];
        kahan_add(S, cS, pS[k]);
        kahan_add(Wt, cW, pW[k]);
        s_acc[0][k][threadIdx.x] = S, s_acc[1][k][threadIdx.x] = cS;
        s_acc[2][k][threadIdx.x] = Wt, s_acc[3][k][threadIdx.x] = cW;
        pS[k] = pW[k] = 0.f;
      }
      since = 0;
    }
  }
  if( xin ) {
#pragma unroll
    for( int k = 0; k < SA_PPT; ++k ) {
      const int y = yb + k;
      if( y >= a.dh ) continue;
      float S = s_acc[0][k][threadIdx.x], cS = s_acc[1][k][threadIdx.x];
      float Wt = s_acc[2][k][threadIdx.x], cW = s_acc[3][k][threadIdx.x];
      kahan_add(S, cS, pS[k]);
      kahan_add(Wt, cW, pW[k]);
      const size_t i = (size_t) y * a.dw + x;
      if( chunk > 0 ) {
        float * P = a.part + (size_t) (chunk - 1) * 4 * a.plane;
        P[i] = S, P[a.plane + i] = cS, P[2 * a.plane + i] = Wt, P[3 * a.plane + i] = cW;
        continue;
      }
      float gS = a.acc[i], gcS = a.acc[a.plane + i], gW = a.acc[2 * a.plane + i], gcW = a.acc[3 * a.plane + i];
      kahan_add(gS, gcS, S);
      gcS += cS;
      kahan_add(gW, gcW, Wt);
      gcW += cW;
      a.acc[i] = gS, a.acc[a.plane + i] = gcS, a.acc[2 * a.plane + i] = gW, a.acc[3 * a.plane + i] = gcW;
    }
  }
}

/* cuTensorMapEncodeTiled through the runtime's driver entry point (no link to
 * the driver library); nullptr when unavailable */
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void * p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if( cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess )
      fn = (EncodeTiledFn) p;
    else cudaGetLastError();
  });
  return fn;
}

bool encode_tensor_3d(CUtensorMap * map, CUtensorMapDataType dt, int esz, const void * base, const uint64_t * dims,
    const uint64_t * strides, const uint32_t * box)
{
  EncodeTiledFn fn = encode_fn();
  if( !fn ) return false;
  if( ((uintptr_t) base & 15) || (strides[0] & 15) || (strides[1] & 15) || ((size_t) box[0] * esz) % 16 ) return false;
  const cuuint64_t d[3] = { dims[0], dims[1], dims[2] };
  const cuuint64_t st[2] = { strides[0], strides[1] };
  const cuuint32_t bx[3] = { box[0], box[1], box[2] };
  const cuuint32_t estr[3] = { 1, 1, 1 };
  return fn(map, dt, 3, (void *) base, d, st, bx, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_stack_add_warped(const StackArgs & a, int motion, int depth, cudaStream_t st)
{
  dim3 grid((a.dw + SA_TX - 1) / SA_TX, (a.dh + SA_TY - 1) / SA_TY);
  const int fam = motion_family(motion);
  const size_t esz = depth == SST_DEPTH_U8 ? 1 : depth == SST_DEPTH_U16 ? 2 : 4;
  if( fam != FAM_QUAD && a.n > 0 && a.row_stride % esz == 0 && a.row_stride / esz * (size_t) (a.sh + 1) < (1u << 31) ) {
    // frame chunks: enough (tile, chunk) CTAs for about items_per_slot per
    // resident slot, at least 32 frames per chunk, within the caller's scratch
    static int slots = 0;
    if( !slots ) {
      int dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      slots = 4 * (sms > 0 ? sms : 1);   // k_stack_add_streamed: 4 CTAs per SM
    }
    const int tiles = (int) (grid.x * grid.y);
    int chunks = 1;
    if( a.part && a.max_chunks > 1 ) {
      chunks = (a.items_per_slot * slots + tiles - 1) / tiles;
      chunks = chunks < a.max_chunks ? chunks : a.max_chunks;
      chunks = chunks < a.n / 32 ? chunks : a.n / 32;
      chunks = chunks > 1 ? chunks : 1;
    }
    const unsigned items = (unsigned) tiles * (unsigned) chunks;
#define SST_LAUNCH_TMA(FAMV, TV)                                                         \
    if( a.wmap ) k_stack_add_streamed<FAMV, TV, true><<<items, 256, 0, st>>>(a, chunks);  \
    else k_stack_add_streamed<FAMV, TV, false><<<items, 256, 0, st>>>(a, chunks)
    switch ( depth ) {
    case SST_DEPTH_U8:
      if( fam == FAM_AFFINE ) { SST_LAUNCH_TMA(FAM_AFFINE, uint8_t); } else { SST_LAUNCH_TMA(FAM_HOMOG, uint8_t); }
      break;
    case SST_DEPTH_U16:
      if( fam == FAM_AFFINE ) { SST_LAUNCH_TMA(FAM_AFFINE, uint16_t); } else { SST_LAUNCH_TMA(FAM_HOMOG, uint16_t); }
      break;
    default:
      if( fam == FAM_AFFINE ) { SST_LAUNCH_TMA(FAM_AFFINE, float); } else { SST_LAUNCH_TMA(FAM_HOMOG, float); }
      break;
    }
#undef SST_LAUNCH_TMA
    cudaError_t e = cudaGetLastError();
    if( e != cudaSuccess || chunks == 1 ) return e;
    k_stack_merge_chunks<<<(unsigned) ((a.plane + 255) / 256), 256, 0, st>>>(a.acc, a.part, a.plane, chunks - 1);
    return cudaGetLastError();
  }
#define SST_LAUNCH_STACK(FAMV, TV) k_stack_add_warped<FAMV, TV><<<grid, 256, 0, st>>>(a)
  switch ( depth ) {
  case SST_DEPTH_U8:
    if( fam == FAM_AFFINE ) SST_LAUNCH_STACK(FAM_AFFINE, uint8_t);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_STACK(FAM_HOMOG, uint8_t);
    else SST_LAUNCH_STACK(FAM_QUAD, uint8_t);
    break;
  case SST_DEPTH_U16:
    if( fam == FAM_AFFINE ) SST_LAUNCH_STACK(FAM_AFFINE, uint16_t);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_STACK(FAM_HOMOG, uint16_t);
    else SST_LAUNCH_STACK(FAM_QUAD, uint16_t);
    break;
  case SST_DEPTH_F32:
    if( fam == FAM_AFFINE ) SST_LAUNCH_STACK(FAM_AFFINE, float);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_STACK(FAM_HOMOG, float);
    else SST_LAUNCH_STACK(FAM_QUAD, float);
    break;
  default: return cudaErrorInvalidValue;
  }
#undef SST_LAUNCH_STACK
  return cudaGetLastError();
}

/* c_weigthed_average::add of one already-warped frame */
template<typename T>
__global__ void k_stack_add_plain(const uint8_t * src, size_t row_stride, float scale, const uint8_t * wts,
    int wdepth, size_t wstride, int w, int h, float * acc, size_t plane)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= w || y >= h ) return;
  float wt = 1.f;
  if( wts ) {
    if( wdepth == SST_DEPTH_U8 ) wt = wts[(size_t) y * wstride + x] ? 1.f : 0.f;
    else wt = *(const float *) (wts + (size_t) y * wstride + (size_t) x * 4);
  }
  if( !(wt > 0.f) ) return;
  const float v = (float) (*(const T *) (src + (size_t) y * row_stride + (size_t) x * sizeof(T))) * scale;
  const size_t i = (size_t) y * w + x;
  float gS = acc[i], gcS = acc[plane + i], gW = acc[2 * plane + i], gcW = acc[3 * plane + i];
  kahan_add(gS, gcS, wt * v);
  kahan_add(gW, gcW, wt);
  acc[i] = gS, acc[plane + i] = gcS, acc[2 * plane + i] = gW, acc[3 * plane + i] = gcW;
}

cudaError_t launch_stack_add_plain(const void * src, int depth, size_t row_stride, double scale, const void * wts,
    int wdepth, size_t wstride, int w, int h, float * acc, size_t plane, cudaStream_t st)
{
  dim3 grid((w + 127) / 128, h);
  const uint8_t * s = (const uint8_t *) src;
  const uint8_t * wp = (const uint8_t *) wts;
  switch ( depth ) {
  case SST_DEPTH_U8: k_stack_add_plain<uint8_t><<<grid, 128, 0, st>>>(s, row_stride, (float) scale, wp, wdepth, wstride, w, h, acc, plane); break;
  case SST_DEPTH_U16: k_stack_add_plain<uint16_t><<<grid, 128, 0, st>>>(s, row_stride, (float) scale, wp, wdepth, wstride, w, h, acc, plane); break;
  case SST_DEPTH_F32: k_stack_add_plain<float><<<grid, 128, 0, st>>>(s, row_stride, (float) scale, wp, wdepth, wstride, w, h, acc, plane); break;
  default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

__global__ void k_stack_compute(const float * acc, size_t plane, int n, float * avg, uint8_t * mask, float * accw)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= n ) return;
  const double S = (double) acc[i] + (double) acc[plane + i];
  const double W = (double) acc[2 * plane + i] + (double) acc[3 * plane + i];
  if( avg ) avg[i] = W > 0 ? (float) (S / W) : 0.f;
  if( mask ) mask[i] = W > 0 ? 255 : 0;
  if( accw ) accw[i] = (float) W;
}

cudaError_t launch_stack_compute(const float * acc, size_t plane, int n, float * avg, uint8_t * mask, float * accw, cudaStream_t st)
{
  k_stack_compute<<<(n + 255) / 256, 256, 0, st>>>(acc, plane, n, avg, mask, accw);
  return cudaGetLastError();
}

/* reinitialize(avg, accw): S = avg * accw, W = accw, compensations 0 */
__global__ void k_stack_reinit(float * acc, size_t plane, int n, const float * avg, const float * accw)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= n ) return;
  acc[i] = avg[i] * accw[i];
  acc[plane + i] = 0.f;
  acc[2 * plane + i] = accw[i];
  acc[3 * plane + i] = 0.f;
}

cudaError_t launch_stack_reinit(float * acc, size_t plane, int n, const float * avg, const float * accw, cudaStream_t st)
{
  k_stack_reinit<<<(n + 255) / 256, 256, 0, st>>>(acc, plane, n, avg, accw);
  return cudaGetLastError();
}

/* ------------------------------------------------------------- remap */

template<int FAM, typename T>
__global__ void __launch_bounds__(256) k_remap(const uint8_t * src, int sw, int sh, size_t rs, float scale,
    const float * coeffs, int border, float * dst, uint8_t * dst_mask, int dw, int dh)
{
  constexpr int VW = SK_TX + 4, VH = SK_TY + 4;
  __shared__ uint8_t s_v[VH * VW];
  __shared__ uint8_t s_h[VH * SK_TX];
  float c[SST_NCOEF];
#pragma unroll
  for( int i = 0; i < SST_NCOEF; ++i ) c[i] = __ldg(coeffs + i);
  const int tx0 = blockIdx.x * SK_TX, ty0 = blockIdx.y * SK_TY;
  const int lx = threadIdx.x % SK_TX, ly = threadIdx.x / SK_TX;
  const int x = tx0 + lx, y = ty0 + ly;
  if( dst_mask ) {
    for( int q = threadIdx.x; q < VW * VH; q += 256 ) {
      const int qx = tx0 - 2 + q % VW, qy = ty0 - 2 + q / VW;
      uint8_t v = 1;
      if( qx >= 0 && qx < dw && qy >= 0 && qy < dh ) {
        v = mask_ok(coverage(sw, sh, warp_pos<FAM>(c, qx, qy)), 255) ? 1 : 0;
      }
      s_v[q] = v;
    }
    __syncthreads();
    for( int q = threadIdx.x; q < SK_TX * VH; q += 256 ) {
      const int xx = q % SK_TX, yy = q / SK_TX;
      const uint8_t * p = s_v + yy * VW + xx;
      s_h[yy * SK_TX + xx] = p[0] & p[1] & p[2] & p[3] & p[4];
    }
    __syncthreads();
  }
  if( x >= dw || y >= dh ) return;
  const size_t i = (size_t) y * dw + x;
  if( dst_mask ) {
    const uint8_t * p = s_h + ly * SK_TX + lx;
    dst_mask[i] = (p[0] & p[SK_TX] & p[2 * SK_TX] & p[3 * SK_TX] & p[4 * SK_TX]) ? 255 : 0;
  }
  if( dst ) {
    const spos s = warp_pos<FAM>(c, x, y);
    const float v00 = tap<T>(src, rs, sw, sh, s.x0, s.y0, border), v01 = tap<T>(src, rs, sw, sh, s.x0 + 1, s.y0, border);
    const float v10 = tap<T>(src, rs, sw, sh, s.x0, s.y0 + 1, border), v11 = tap<T>(src, rs, sw, sh, s.x0 + 1, s.y0 + 1, border);
    const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
    dst[i] = fmaf(s.fy, t1 - t0, t0) * scale;
  }
}

cudaError_t launch_remap(const void * src, int depth, int sw, int sh, size_t rs, double scale, int motion,
    const float * coeffs, int border, float * dst, uint8_t * dst_mask, int dw, int dh, cudaStream_t st)
{
  dim3 grid((dw + SK_TX - 1) / SK_TX, (dh + SK_TY - 1) / SK_TY);
  const int fam = motion_family(motion);
  const uint8_t * s = (const uint8_t *) src;
  const float sc = (float) scale;
#define SST_LAUNCH_REMAP(FAMV, TV) k_remap<FAMV, TV><<<grid, 256, 0, st>>>(s, sw, sh, rs, sc, coeffs, border, dst, dst_mask, dw, dh)
  switch ( depth ) {
  case SST_DEPTH_U8:
    if( fam == FAM_AFFINE ) SST_LAUNCH_REMAP(FAM_AFFINE, uint8_t);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_REMAP(FAM_HOMOG, uint8_t);
    else SST_LAUNCH_REMAP(FAM_QUAD, uint8_t);
    break;
  case SST_DEPTH_U16:
    if( fam == FAM_AFFINE ) SST_LAUNCH_REMAP(FAM_AFFINE, uint16_t);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_REMAP(FAM_HOMOG, uint16_t);
    else SST_LAUNCH_REMAP(FAM_QUAD, uint16_t);
    break;
  case SST_DEPTH_F32:
    if( fam == FAM_AFFINE ) SST_LAUNCH_REMAP(FAM_AFFINE, float);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_REMAP(FAM_HOMOG, float);
    else SST_LAUNCH_REMAP(FAM_QUAD, float);
    break;
  default: return cudaErrorInvalidValue;
  }
#undef SST_LAUNCH_REMAP
  return cudaGetLastError();
}

/* ------------------------------------------------------- focus weights */

/* Focus-stacking weight of every output pixel of every frame (the README's
 * W(x, y) = (6 lap^2 + grad^2)^2 before its Gaussian blur): the frame warped to
 * the output grid (bilinear, BORDER_REPLICATE), its 5-point Laplacian and
 * central-difference gradient with the output grid replicated at its border. */
template<int FAM, typename T>
__global__ void __launch_bounds__(256) k_focus_energy(const uint8_t * frames, size_t rs, size_t fstride, int sw, int sh,
    float scale, const float * coeffs, int dw, int dh, float * out)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= dw || y >= dh ) return;
  const int f = blockIdx.z;
  float c[SST_NCOEF];
#pragma unroll
  for( int i = 0; i < SST_NCOEF; ++i ) c[i] = __ldg(coeffs + (size_t) f * SST_NCOEF + i);
  const uint8_t * fb = frames + (size_t) f * fstride;
  auto warped = [&](int xx, int yy) {
    const spos s = warp_pos<FAM>(c, clampi(xx, 0, dw - 1), clampi(yy, 0, dh - 1));
    const float v00 = tap<T>(fb, rs, sw, sh, s.x0, s.y0, SST_BORDER_REPLICATE);
    const float v01 = tap<T>(fb, rs, sw, sh, s.x0 + 1, s.y0, SST_BORDER_REPLICATE);
    const float v10 = tap<T>(fb, rs, sw, sh, s.x0, s.y0 + 1, SST_BORDER_REPLICATE);
    const float v11 = tap<T>(fb, rs, sw, sh, s.x0 + 1, s.y0 + 1, SST_BORDER_REPLICATE);
    const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
    return fmaf(s.fy, t1 - t0, t0) * scale;
  };
  const float c0 = warped(x, y), l = warped(x - 1, y), r = warped(x + 1, y), u = warped(x, y - 1), d = warped(x, y + 1);
  const float lap = (l + r + u + d) - 4.f * c0;
  const float gx = 0.5f * (r - l), gy = 0.5f * (d - u);
  const float e = fmaf(6.f * lap, lap, fmaf(gx, gx, gy * gy));
  out[(size_t) f * dw * dh + (size_t) y * dw + x] = e * e;
}

cudaError_t launch_focus_energy(const void * frames, int depth, size_t row_stride, size_t frame_stride, int sw, int sh,
    double scale, int motion, const float * coeffs, int n, int dw, int dh, float * out, cudaStream_t st)
{
  dim3 grid((dw + 31) / 32, (dh + 7) / 8, n);
  const uint8_t * fr = (const uint8_t *) frames;
  const int fam = motion_family(motion);
#define SST_LAUNCH_FOCUS(FAMV, TV) k_focus_energy<FAMV, TV><<<grid, 256, 0, st>>>(fr, row_stride, frame_stride, sw, sh, (float) scale, coeffs, dw, dh, out)
  switch ( depth ) {
  case SST_DEPTH_U8:
    if( fam == FAM_AFFINE ) SST_LAUNCH_FOCUS(FAM_AFFINE, uint8_t);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_FOCUS(FAM_HOMOG, uint8_t);
    else SST_LAUNCH_FOCUS(FAM_QUAD, uint8_t);
    break;
  case SST_DEPTH_U16:
    if( fam == FAM_AFFINE ) SST_LAUNCH_FOCUS(FAM_AFFINE, uint16_t);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_FOCUS(FAM_HOMOG, uint16_t);
    else SST_LAUNCH_FOCUS(FAM_QUAD, uint16_t);
    break;
  case SST_DEPTH_F32:
    if( fam == FAM_AFFINE ) SST_LAUNCH_FOCUS(FAM_AFFINE, float);
    else if( fam == FAM_HOMOG ) SST_LAUNCH_FOCUS(FAM_HOMOG, float);
    else SST_LAUNCH_FOCUS(FAM_QUAD, float);
    break;
  default: return cudaErrorInvalidValue;
  }
#undef SST_LAUNCH_FOCUS
  return cudaGetLastError();
}

/* ----------------------------------------------------------- Bayer planes */

/* extract_bayer_planes: dst[y][x][0..3] = src(2y,2x), src(2y,2x+1), src(2y+1,2x), src(2y+1,2x+1) */
__global__ void k_extract_bayer_planes_u16(const uint8_t * src, int w, int h, size_t rs, uint16_t * dst)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  const int c4 = w / 2;
  if( x >= c4 || y >= h / 2 ) return;
  const uint32_t r0 = __ldg((const uint32_t *) (src + (size_t) (2 * y) * rs) + x);
  const uint32_t r1 = __ldg((const uint32_t *) (src + (size_t) (2 * y + 1) * rs) + x);
  uint2 o;
  o.x = (r0 & 0xffffu) | (r0 & 0xffff0000u);
  o.y = (r1 & 0xffffu) | (r1 & 0xffff0000u);
  reinterpret_cast<uint2 *>(dst)[(size_t) y * c4 + x] = o;
}

/* average_bayer_planes of a raw mosaic: (2 + sum of the 2x2 block) / 4 */
__global__ void k_average_bayer_planes_u16(const uint8_t * src, int w, int h, size_t rs, uint16_t * dst)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  const int c4 = w / 2;
  if( x >= c4 || y >= h / 2 ) return;
  const uint32_t r0 = __ldg((const uint32_t *) (src + (size_t) (2 * y) * rs) + x);
  const uint32_t r1 = __ldg((const uint32_t *) (src + (size_t) (2 * y + 1) * rs) + x);
  const int s = 2 + (int) (r0 & 0xffffu) + (int) (r0 >> 16) + (int) (r1 & 0xffffu) + (int) (r1 >> 16);
  dst[(size_t) y * c4 + x] = (uint16_t) min(s / 4, 65535);
}

cudaError_t launch_bayer_planes(int op, const uint16_t * src, int w, int h, size_t rs, uint16_t * dst, cudaStream_t st)
{
  dim3 grid((w / 2 + 127) / 128, h / 2);
  if( op == 0 ) k_extract_bayer_planes_u16<<<grid, 128, 0, st>>>((const uint8_t *) src, w, h, rs, dst);
  else k_average_bayer_planes_u16<<<grid, 128, 0, st>>>((const uint8_t *) src, w, h, rs, dst);
  return cudaGetLastError();
}

/* average_bayer_planes of n mosaic frames: frame f at src + f * frame_stride,
 * binned frame f at dst + f * (w/2) * (h/2), rows of w/2 u16 */
__global__ void k_average_bayer_planes_batch(const uint8_t * src, int w, int h, size_t rs, size_t frame_stride,
    uint16_t * dst)
{
  const int f = blockIdx.z;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  const int c4 = w / 2;
  if( x >= c4 ) return;
  const uint8_t * fs = src + (size_t) f * frame_stride;
  const uint32_t r0 = __ldg((const uint32_t *) (fs + (size_t) (2 * y) * rs) + x);
  const uint32_t r1 = __ldg((const uint32_t *) (fs + (size_t) (2 * y + 1) * rs) + x);
  const int s = 2 + (int) (r0 & 0xffffu) + (int) (r0 >> 16) + (int) (r1 & 0xffffu) + (int) (r1 >> 16);
  dst[((size_t) f * (h / 2) + y) * c4 + x] = (uint16_t) min(s / 4, 65535);
}

cudaError_t launch_average_bayer_planes_batch(const void * src, int w, int h, size_t rs, size_t frame_stride, int n,
    uint16_t * dst, cudaStream_t st)
{
  dim3 grid((w / 2 + 127) / 128, h / 2, n);
  k_average_bayer_planes_batch<<<grid, 128, 0, st>>>((const uint8_t *) src, w, h, rs, frame_stride, dst);
  return cudaGetLastError();
}

/* ------------------------------------------------ Bayer planes, stacked */

/* Plane k (mosaic order: k = 0 (0,0), 1 (0,1), 2 (1,0), 3 (1,1) within each
 * 2x2 cell) of a raw mosaic is the pw x ph image plane_k(x, y) =
 * raw(2x + (k & 1), 2y + (k >> 1)), the channels extract_bayer_planes
 * produces (debayer.cc:96-147). The four planes of a frame share the plane
 * transform, so they share every sample position, the remapped mask and the
 * weight: one thread gathers the 4 x 4 raw block that holds all 16 taps of
 * its output pixel and updates four accumulators. */
__device__ __forceinline__ float raw_tap(const uint8_t * fb, size_t rs, int pw, int ph, int xi, int yi, int k,
    int border)
{
  if( xi < 0 || xi >= pw || yi < 0 || yi >= ph ) {
    switch ( border ) {
    case SST_BORDER_REPLICATE: xi = clampi(xi, 0, pw - 1), yi = clampi(yi, 0, ph - 1); break;
    case SST_BORDER_REFLECT101: xi = reflect101(xi, pw), yi = reflect101(yi, ph); break;
    case SST_BORDER_REFLECT: xi = reflect(xi, pw), yi = reflect(yi, ph); break;
    default: return 0.f;
    }
  }
  return (float) __ldg((const uint16_t *) (fb + (size_t) (2 * yi + (k >> 1)) * rs) + 2 * xi + (k & 1));
}

template<int FAM>
__global__ void __launch_bounds__(256) k_stack_bayer_planes(BayerPlanesArgs a)
{
  constexpr int VW = SA_TX + 4, VH = SA_TY + 4;
  constexpr int PPT = SA_TX * SA_TY / 256;
  __shared__ uint8_t s_v[VH * VW];
  __shared__ uint8_t s_h[VH * SA_TX];
  const int tx0 = blockIdx.x * SA_TX, ty0 = blockIdx.y * SA_TY;
  const int lx = threadIdx.x % SA_TX, ly0 = threadIdx.x / SA_TX;
  const int x = tx0 + lx;
  const int wx0 = max(tx0 - 2, 0), wy0 = max(ty0 - 2, 0);
  const int wx1 = min(tx0 + SA_TX + 1, a.pw - 1), wy1 = min(ty0 + SA_TY + 1, a.ph - 1);
  float S[PPT][4], cS[PPT][4], Wt[PPT], cW[PPT];
#pragma unroll
  for( int k = 0; k < PPT; ++k ) {
    Wt[k] = cW[k] = 0.f;
#pragma unroll
    for( int q = 0; q < 4; ++q ) S[k][q] = cS[k][q] = 0.f;
  }
  for( int f = 0; f < a.n; ++f ) {
    const float wf = __ldg(a.weights + f);
    if( !(wf > 0.f) ) continue;                 // uniform over the CTA
    float c[SST_NCOEF];
#pragma unroll
    for( int i = 0; i < SST_NCOEF; ++i ) c[i] = __ldg(a.coeffs + (size_t) f * SST_NCOEF + i);
    const uint8_t * fb = a.frames + (size_t) f * a.frame_stride;
    if( rect_interior<FAM>(c, wx0, wy0, wx1, wy1, a.pw, a.ph) ) {
      if( x < a.pw ) {
#pragma unroll
        for( int k = 0; k < PPT; ++k ) {
          const int y = ty0 + ly0 + 4 * k;
          if( y >= a.ph ) continue;
          const spos s = warp_pos<FAM>(c, x, y);
          const float wp = a.wmap ? wf * __ldg(a.wmap + (size_t) f * a.plane + (size_t) y * a.pw + x) : wf;
          // raw rows 2 y0 .. 2 y0 + 3, columns 2 x0 .. 2 x0 + 3 (two u32 per row)
          const uint8_t * r = fb + (size_t) (2 * s.y0) * a.row_stride + (size_t) s.x0 * 4;
          uint32_t q[4][2];
#pragma unroll
          for( int rr = 0; rr < 4; ++rr ) {
            q[rr][0] = __ldg((const uint32_t *) (r + (size_t) rr * a.row_stride));
            q[rr][1] = __ldg((const uint32_t *) (r + (size_t) rr * a.row_stride) + 1);
          }
#pragma unroll
          for( int p = 0; p < 4; ++p ) {
            const int dy = p >> 1, sh = (p & 1) * 16;
            const float v00 = (float) ((q[dy][0] >> sh) & 0xffffu), v01 = (float) ((q[dy][1] >> sh) & 0xffffu);
            const float v10 = (float) ((q[dy + 2][0] >> sh) & 0xffffu), v11 = (float) ((q[dy + 2][1] >> sh) & 0xffffu);
            const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
            kahan_add(S[k][p], cS[k][p], wp * (fmaf(s.fy, t1 - t0, t0) * a.scale));
          }
          kahan_add(Wt[k], cW[k], wp);
        }
      }
      continue;
    }
    for( int q = threadIdx.x; q < VW * VH; q += 256 ) {
      const int qx = tx0 - 2 + q % VW, qy = ty0 - 2 + q / VW;
      uint8_t v = 1;
      if( qx >= 0 && qx < a.pw && qy >= 0 && qy < a.ph ) {
        v = mask_ok(coverage(a.pw, a.ph, warp_pos<FAM>(c, qx, qy)), 255) ? 1 : 0;
      }
      s_v[q] = v;
    }
    __syncthreads();
    for( int q = threadIdx.x; q < SA_TX * VH; q += 256 ) {
      const int xx = q % SA_TX, yy = q / SA_TX;
      const uint8_t * p = s_v + yy * VW + xx;
      s_h[yy * SA_TX + xx] = p[0] & p[1] & p[2] & p[3] & p[4];
    }
    __syncthreads();
    if( x < a.pw ) {
#pragma unroll
      for( int k = 0; k < PPT; ++k ) {
        const int ly = ly0 + 4 * k, y = ty0 + ly;
        if( y >= a.ph ) continue;
        const uint8_t * pm = s_h + ly * SA_TX + lx;
        if( pm[0] & pm[SA_TX] & pm[2 * SA_TX] & pm[3 * SA_TX] & pm[4 * SA_TX] ) {
          const spos s = warp_pos<FAM>(c, x, y);
          const float wp = a.wmap ? wf * __ldg(a.wmap + (size_t) f * a.plane + (size_t) y * a.pw + x) : wf;
#pragma unroll
          for( int p = 0; p < 4; ++p ) {
            const float v00 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0, s.y0, p, a.border);
            const float v01 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0 + 1, s.y0, p, a.border);
            const float v10 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0, s.y0 + 1, p, a.border);
            const float v11 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0 + 1, s.y0 + 1, p, a.border);
            const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
            kahan_add(S[k][p], cS[k][p], wp * (fmaf(s.fy, t1 - t0, t0) * a.scale));
          }
          kahan_add(Wt[k], cW[k], wp);
        }
      }
    }
    __syncthreads();
  }
  if( x < a.pw ) {
#pragma unroll
    for( int k = 0; k < PPT; ++k ) {
      const int y = ty0 + ly0 + 4 * k;
      if( y >= a.ph ) continue;
      const size_t i = (size_t) y * a.pw + x;
#pragma unroll
      for( int p = 0; p < 4; ++p ) {
        float * P = a.acc[p];
        float gS = P[i], gcS = P[a.plane + i], gW = P[2 * a.plane + i], gcW = P[3 * a.plane + i];
        kahan_add(gS, gcS, S[k][p]);
        gcS += cS[k][p];
        kahan_add(gW, gcW, Wt[k]);
        gcW += cW[k];
        P[i] = gS, P[a.plane + i] = gcS, P[2 * a.plane + i] = gW, P[3 * a.plane + i] = gcW;
      }
    }
  }
}

/* The four-plane Bayer stack for the affine and projective families in the
 * form of k_stack_add_streamed: one output column of BP_PPT rows per thread,
 * warps on their own (interior tests 8 frames per ballot, four-corner window
 * validity at the border), FP32 partials of SA_FLUSH frames in registers and
 * the compensated sums of the four planes and the weight in thread-private
 * shared slots. */
constexpr int BP_PPT = 2, BP_TY = 2 * 256 / SA_TX;   // Bayer planes: 64 x 8 tiles, 2 rows per thread

template<int FAM, bool WMAP>
__global__ void __launch_bounds__(256, 3) k_stack_bayer_streamed(BayerPlanesArgs a)
{
  constexpr int NQ = 10;                              // S, cS of four planes; W, cW
  __shared__ float s_acc[NQ][BP_PPT][256];
  const int tx0 = blockIdx.x * SA_TX, ty0 = blockIdx.y * BP_TY;
  const int lx = threadIdx.x % SA_TX, yb = ty0 + (threadIdx.x / SA_TX) * BP_PPT;
  const int x = tx0 + lx;
  const int xw = tx0 + (lx & ~31);
  const int wx0 = max(xw - 2, 0), wx1 = min(xw + 33, a.pw - 1);
  const int wy0 = max(yb - 2, 0), wy1 = min(yb + BP_PPT + 1, a.ph - 1);
  const bool active = xw < a.pw && yb < a.ph;          // warp-uniform
  const bool xin = x < a.pw;
  const int lane = threadIdx.x & 31;
  float pS[BP_PPT][4], pW[BP_PPT];
#pragma unroll
  for( int k = 0; k < BP_PPT; ++k ) {
    pW[k] = 0.f;
#pragma unroll
    for( int q = 0; q < 4; ++q ) pS[k][q] = 0.f;
#pragma unroll
    for( int q = 0; q < NQ; ++q ) s_acc[q][k][threadIdx.x] = 0.f;
  }
  int since = 0;
  unsigned inner8 = 0u;
  for( int f = 0; f < a.n && active; ++f ) {
    if( (f & 7) == 0 ) {
      const int fl = f + (lane >> 2);
      bool ok = false;
      if( fl < a.n ) {
        const float4 * cq = (const float4 *) (a.coeffs + (size_t) fl * SST_NCOEF);
        const float4 r0 = __ldg(cq), r1 = __ldg(cq + 1), r3 = __ldg(cq + 3);
        float cc[SST_NCOEF];
        cc[0] = r0.x, cc[1] = r0.y, cc[2] = r0.z, cc[3] = r0.w, cc[4] = r1.x, cc[5] = r1.y, cc[6] = r1.z, cc[7] = r1.w;
        cc[8] = cc[9] = cc[10] = cc[11] = 0.f;
        cc[12] = r3.x, cc[13] = r3.y, cc[14] = r3.z, cc[15] = r3.w;
        ok = point_interior<FAM>(cc, (lane & 1) ? wx1 : wx0, (lane & 2) ? wy1 : wy0, a.pw, a.ph);
      }
      inner8 = __ballot_sync(0xffffffffu, ok);
    }
    const bool inner = ((inner8 >> (4 * (f & 7))) & 0xFu) == 0xFu;
    const float wf = __ldg(a.weights + f);
    if( !(wf > 0.f) ) continue;                       // uniform over the CTA
    const float4 * cp = (const float4 *) (a.coeffs + (size_t) f * SST_NCOEF);
    const float4 q0 = __ldg(cp), q1 = __ldg(cp + 1), q3 = __ldg(cp + 3);
    float c[SST_NCOEF];
    c[0] = q0.x, c[1] = q0.y, c[2] = q0.z, c[3] = q0.w, c[4] = q1.x, c[5] = q1.y, c[6] = q1.z, c[7] = q1.w;
    c[8] = c[9] = c[10] = c[11] = 0.f;
    c[12] = q3.x, c[13] = q3.y, c[14] = q3.z, c[15] = q3.w;
    const uint8_t * fb = a.frames + (size_t) f * a.frame_stride;
    if( xin ) {
#pragma unroll
      for( int k = 0; k < BP_PPT; ++k ) {
        const int y = yb + k;
        if( y >= a.ph ) continue;
        if( !inner && !window_valid<FAM>(c, x, y, a.pw, a.ph, a.pw, a.ph) ) continue;
        const spos s = warp_pos<FAM>(c, x, y);
        const float wp = WMAP ? wf * __ldg(a.wmap + (size_t) f * a.plane + (size_t) y * a.pw + x) : wf;
        const float wsc = wp * a.scale;
        if( inner || (s.x0 >= 0 && s.x0 < a.pw - 1 && s.y0 >= 0 && s.y0 < a.ph - 1) ) {
          // raw rows 2 y0 .. 2 y0 + 3, columns 2 x0 .. 2 x0 + 3 (two u32 per row)
          const uint8_t * r = fb + (size_t) (2 * s.y0) * a.row_stride + (size_t) s.x0 * 4;
          uint32_t q[4][2];
#pragma unroll
          for( int rr = 0; rr < 4; ++rr ) {
            q[rr][0] = __ldg((const uint32_t *) (r + (size_t) rr * a.row_stride));
            q[rr][1] = __ldg((const uint32_t *) (r + (size_t) rr * a.row_stride) + 1);
          }
#pragma unroll
          for( int p = 0; p < 4; ++p ) {
            const int dy = p >> 1, sh = (p & 1) * 16;
            const float v00 = (float) ((q[dy][0] >> sh) & 0xffffu), v01 = (float) ((q[dy][1] >> sh) & 0xffffu);
            const float v10 = (float) ((q[dy + 2][0] >> sh) & 0xffffu), v11 = (float) ((q[dy + 2][1] >> sh) & 0xffffu);
            const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
            pS[k][p] = fmaf(wsc, fmaf(s.fy, t1 - t0, t0), pS[k][p]);
          }
        }
        else {
#pragma unroll
          for( int p = 0; p < 4; ++p ) {
            const float v00 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0, s.y0, p, a.border);
            const float v01 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0 + 1, s.y0, p, a.border);
            const float v10 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0, s.y0 + 1, p, a.border);
            const float v11 = raw_tap(fb, a.row_stride, a.pw, a.ph, s.x0 + 1, s.y0 + 1, p, a.border);
            const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
            pS[k][p] = fmaf(wsc, fmaf(s.fy, t1 - t0, t0), pS[k][p]);
          }
        }
        pW[k] += wp;
      }
    }
    if( ++since == SA_FLUSH ) {
#pragma unroll
      for( int k = 0; k < BP_PPT; ++k ) {
#pragma unroll
        for( int p = 0; p < 4; ++p ) {
          float S = s_acc[2 * p][k][threadIdx.x], cS = s_acc[2 * p + 1][k][threadIdx.x];
          kahan_add(S, cS, pS[k][p]);
          s_acc[2 * p][k][threadIdx.x] = S, s_acc[2 * p + 1][k][threadIdx.x] = cS;
          pS[k][p] = 0.f;
        }
        float Wt = s_acc[8][k][threadIdx.x], cW = s_acc[9][k][threadIdx.x];
        kahan_add(Wt, cW, pW[k]);
        s_acc[8][k][threadIdx.x] = Wt, s_acc[9][k][threadIdx.x] = cW;
        pW[k] = 0.f;
      }
      since = 0;
    }
  }
  if( xin ) {
#pragma unroll
    for( int k = 0; k < BP_PPT; ++k ) {
      const int y = yb + k;
      if( y >= a.ph ) continue;
      const size_t i = (size_t) y * a.pw + x;
      float Wt = s_acc[8][k][threadIdx.x], cW = s_acc[9][k][threadIdx.x];
      kahan_add(Wt, cW, pW[k]);
#pragma unroll
      for( int p = 0; p < 4; ++p ) {
        float S = s_acc[2 * p][k][threadIdx.x], cS = s_acc[2 * p + 1][k][threadIdx.x];
        kahan_add(S, cS, pS[k][p]);
        float * P = a.acc[p];
        float gS = P[i], gcS = P[a.plane + i], gW = P[2 * a.plane + i], gcW = P[3 * a.plane + i];
        kahan_add(gS, gcS, S);
        gcS += cS;
        kahan_add(gW, gcW, Wt);
        gcW += cW;
        P[i] = gS, P[a.plane + i] = gcS, P[2 * a.plane + i] = gW, P[3 * a.plane + i] = gcW;
      }
    }
  }
}

cudaError_t launch_stack_bayer_planes(const BayerPlanesArgs & a, int motion, cudaStream_t st)
{
  const dim3 grid((a.pw + SA_TX - 1) / SA_TX, (a.ph + SA_TY - 1) / SA_TY);
  const dim3 sgrid((a.pw + SA_TX - 1) / SA_TX, (a.ph + BP_TY - 1) / BP_TY);
  switch ( motion_family(motion) ) {
  case FAM_AFFINE:
    if( a.wmap ) k_stack_bayer_streamed<FAM_AFFINE, true><<<sgrid, 256, 0, st>>>(a);
    else k_stack_bayer_streamed<FAM_AFFINE, false><<<sgrid, 256, 0, st>>>(a);
    break;
  case FAM_HOMOG:
    if( a.wmap ) k_stack_bayer_streamed<FAM_HOMOG, true><<<sgrid, 256, 0, st>>>(a);
    else k_stack_bayer_streamed<FAM_HOMOG, false><<<sgrid, 256, 0, st>>>(a);
    break;
  default: k_stack_bayer_planes<FAM_QUAD><<<grid, 256, 0, st>>>(a); break;
  }
  return cudaGetLastError();
}

}  // namespace sst
