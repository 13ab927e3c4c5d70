/*
 * sst_flow.cu -- c_eccflow on the GPU: the dense smooth optical flow of a
 * batch of frames against one reference (ecc2.h:509-662, ecc2.cc:2220-2865).
 *
 * Per reference level l (set_reference_image, ecc2.cc:2489-2672): the level
 * image (INTER_AREA or pyrDown of the previous level), its gradients
 * (ecc_differentiate), and D = (a00, a01, a11, mult / (|det| + reg)) from
 * the area-averaged structure tensor (avgdown: INTER_AREA by 2^support_scale
 * then a 3x3 Gaussian). Per frame and iteration (compute_uv, ecc2.cc:
 * 2237-2398, 2770-2835):
 *
 *   k_flow_area    remap the frame's level by uv (bilinear, REPLICATE),
 *                  It = T - I(x + uv), and the INTER_AREA average of
 *                  (It gx, It gy) over each low-resolution cell, fused: the
 *                  full-resolution products never reach HBM
 *   k_flow_solve   3x3 Gaussian of those averages and the 2x2 solve with D
 *   k_resample     Keys-cubic (a = -0.75) upsampling of the update, added
 *                  to uv in place
 *
 * Between levels uv is scaled by the size ratio and cubic-resampled to the
 * finer level. All frames of a batch advance level by level together
 * (grid.z = frame). Layout in HBM: per frame an f32 pyramid (levels back to
 * back) and two float2 flow planes of the level-0 size (ping-pong across
 * level changes); per level of the reference {T, gx, gy, 0} (float4) and D
 * (float4 at the low-resolution size); resampling tap tables per level.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <new>
#include <string>
#include <vector>

#include "sst_engine.cuh"
#include "sst_host.h"
#include "sst_taps.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

namespace sst {

/* One axis of a separable resampling: destination d reads the sources
 * idx[d * K + k] with weights w[d * K + k], k < K (zero weights pad). */
struct TapAxis {
  const int * idx;
  const float * w;
  int K;
};

/* dst(x, y)[c] = (add ? dst : 0) + mul[c] * sum_j wy_j sum_i wx_i src(ix_i, iy_j)[c]
 * for C interleaved channels; grid.z = frame */
template<int C>
__global__ void __launch_bounds__(256) k_resample(const float * src, int sw, size_t src_frame, float * dst, int dw,
    int dh, size_t dst_frame, TapAxis tx, TapAxis ty, float mul0, float mul1, int add)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= dw || y >= dh ) return;
  const float * s = src + (size_t) blockIdx.z * src_frame;
  float * d = dst + (size_t) blockIdx.z * dst_frame;
  float acc[C];
#pragma unroll
  for( int c = 0; c < C; ++c ) acc[c] = 0.f;
  for( int j = 0; j < ty.K; ++j ) {
    const float wy = __ldg(ty.w + y * ty.K + j);
    if( wy == 0.f ) continue;
    const float * row = s + (size_t) __ldg(ty.idx + y * ty.K + j) * sw * C;
    float r[C];
#pragma unroll
    for( int c = 0; c < C; ++c ) r[c] = 0.f;
    for( int i = 0; i < tx.K; ++i ) {
      const float wx = __ldg(tx.w + x * tx.K + i);
      const int ix = __ldg(tx.idx + x * tx.K + i);
#pragma unroll
      for( int c = 0; c < C; ++c ) r[c] = fmaf(wx, __ldg(row + (size_t) ix * C + c), r[c]);
    }
#pragma unroll
    for( int c = 0; c < C; ++c ) acc[c] = fmaf(wy, r[c], acc[c]);
  }
  const float mul[2] = { mul0, mul1 };
  float * o = d + ((size_t) y * dw + x) * C;
#pragma unroll
  for( int c = 0; c < C; ++c ) o[c] = (add ? o[c] : 0.f) + mul[c] * acc[c];
}

/* Area averages over the low-resolution cells of a level, one warp per cell:
 * MODE 0 (structure tensor of the reference): (gx^2, gx gy, gy^2);
 * MODE 1 (flow update): (It gx, It gy) with It = T - I(x + u, y + v). */
template<int MODE>
__global__ void __launch_bounds__(256) k_flow_area(const float4 * __restrict__ tg, const float * cur, size_t cur_frame,
    const float2 * uv, size_t uv_frame, int w, int h, TapAxis tx, TapAxis ty, int dw, int dh, float * out,
    size_t out_frame, const uint8_t * rmask = nullptr, const uint8_t * cmask = nullptr, size_t cmask_frame = 0)
{
  constexpr int NC = MODE == 0 ? 3 : 2;
  const int lane = threadIdx.x & 31;
  const int cell = blockIdx.x * 8 + (threadIdx.x >> 5);
  if( cell >= dw * dh ) return;
  const int X = cell % dw, Y = cell / dw;
  const float * img = MODE == 1 ? cur + (size_t) blockIdx.z * cur_frame : nullptr;
  const float2 * fl = MODE == 1 ? uv + (size_t) blockIdx.z * uv_frame : nullptr;
  const uint8_t * cm = MODE == 1 && cmask ? cmask + (size_t) blockIdx.z * cmask_frame : nullptr;
  float acc[NC];
#pragma unroll
  for( int c = 0; c < NC; ++c ) acc[c] = 0.f;
  const int n = tx.K * ty.K;
  for( int q = lane; q < n; q += 32 ) {
    const int i = q % tx.K, j = q / tx.K;
    const float wgt = __ldg(tx.w + X * tx.K + i) * __ldg(ty.w + Y * ty.K + j);
    if( wgt == 0.f ) continue;
    const int x = __ldg(tx.idx + X * tx.K + i), y = __ldg(ty.idx + Y * ty.K + j);
    const size_t p = (size_t) y * w + x;
    const float4 t = __ldg(tg + p);
    if( MODE == 0 ) {
      acc[0] = fmaf(wgt, t.y * t.y, acc[0]);
      acc[1] = fmaf(wgt, t.y * t.z, acc[1]);
      acc[2 % NC] = fmaf(wgt, t.z * t.z, acc[2 % NC]);
    }
    else {
      const float2 f = fl[p];
      const float sx = (float) x + f.x, sy = (float) y + f.y;
      // masks (compute_uv, ecc2.cc:2253-2281): the current mask remapped
      // INTER_NEAREST (cvRound) with BORDER_CONSTANT 0, ANDed with the
      // reference mask; It gx, It gy are zero where either is 0
      if( rmask && !__ldg(rmask + p) ) continue;
      if( cm ) {
        const int nx = __float2int_rn(fminf(fmaxf(sx, -1e8f), 1e8f)), ny = __float2int_rn(fminf(fmaxf(sy, -1e8f), 1e8f));
        if( nx < 0 || nx >= w || ny < 0 || ny >= h || !__ldg(cm + (size_t) ny * w + nx) ) continue;
      }
      // cv::remap INTER_LINEAR, BORDER_REPLICATE
      const float fx0 = floorf(fminf(fmaxf(sx, -1e8f), 1e8f)), fy0 = floorf(fminf(fmaxf(sy, -1e8f), 1e8f));
      const float ax = sx - fx0, ay = sy - fy0;
      const int x0 = (int) fx0, y0 = (int) fy0;
      const int xa = clampi(x0, 0, w - 1), xb = clampi(x0 + 1, 0, w - 1);
      const int ya = clampi(y0, 0, h - 1), yb = clampi(y0 + 1, 0, h - 1);
      const float v00 = __ldg(img + (size_t) ya * w + xa), v01 = __ldg(img + (size_t) ya * w + xb);
      const float v10 = __ldg(img + (size_t) yb * w + xa), v11 = __ldg(img + (size_t) yb * w + xb);
      const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
      const float It = t.x - fmaf(ay, t1 - t0, t0);
      acc[0] = fmaf(wgt, It * t.y, acc[0]);
      acc[1] = fmaf(wgt, It * t.z, acc[1]);
    }
  }
#pragma unroll
  for( int c = 0; c < NC; ++c ) acc[c] = warp_sum(acc[c]);
  if( lane == 0 ) {
    float * o = out + (size_t) blockIdx.z * out_frame + (size_t) cell * NC;
#pragma unroll
    for( int c = 0; c < NC; ++c ) o[c] = acc[c];
  }
}

__device__ __forceinline__ float gauss3_at(const float * a, int C, int c, int x, int y, int w, int h)
{
  float s = 0.f;
  const float k[3] = { 0.25f, 0.5f, 0.25f };
#pragma unroll
  for( int j = 0; j < 3; ++j ) {
    const int yy = clampi(y + j - 1, 0, h - 1);
    float r = 0.f;
#pragma unroll
    for( int i = 0; i < 3; ++i ) r = fmaf(k[i], a[((size_t) yy * w + clampi(x + i - 1, 0, w - 1)) * C + c], r);
    s = fmaf(k[j], r, s);
  }
  return s;
}

/* D of a reference level: 3x3 Gaussian of the tensor averages, then
 * (a00, a01, a11, mult / (|a00 a11 - a01^2| + reg)) */
__global__ void k_flow_tensor(const float * avg, int dw, int dh, float mult, float reg, float4 * D)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= dw * dh ) return;
  const int x = i % dw, y = i / dw;
  const float a00 = gauss3_at(avg, 3, 0, x, y, dw, dh), a01 = gauss3_at(avg, 3, 1, x, y, dw, dh);
  const float a11 = gauss3_at(avg, 3, 2, x, y, dw, dh);
  // the determinant cancels where the structure tensor is nearly rank one:
  // form it in FP64 (one evaluation per low-resolution cell and level)
  const double det = fabs((double) a00 * a11 - (double) a01 * a01);
  D[i] = make_float4(a00, a01, a11, (float) (mult / (det + reg)));
}

/* the 2x2 solve of one update (ecc2.cc:2373-2392), after the 3x3 Gaussian of (It gx, It gy) */
__global__ void k_flow_solve(const float * avg, size_t avg_frame, const float4 * D, int dw, int dh, float2 * duv,
    size_t duv_frame)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= dw * dh ) return;
  const float * a = avg + (size_t) blockIdx.z * avg_frame;
  const int x = i % dw, y = i / dw;
  const float b0 = gauss3_at(a, 2, 0, x, y, dw, dh), b1 = gauss3_at(a, 2, 1, x, y, dw, dh);
  const float4 d = D[i];
  // Cramer's rule; the differences cancel in the same cells as the determinant
  const double u = (double) d.w * ((double) d.z * b0 - (double) d.y * b1);
  const double v = (double) d.w * ((double) d.x * b1 - (double) d.y * b0);
  duv[(size_t) blockIdx.z * duv_frame + i] = make_float2((float) u, (float) v);
}

/* cv::resize INTER_NEAREST of u8 masks: source floor(d * ssize / dsize), grid.z = frame */
__global__ void k_resize_nearest_u8_batch(const uint8_t * src, int sw, int sh, size_t src_frame, uint8_t * dst, int dw,
    int dh, size_t dst_frame)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= dw ) return;
  const int sx = min((int) floor(x * ((double) sw / dw)), sw - 1), sy = min((int) floor(y * ((double) sh / dh)), sh - 1);
  dst[(size_t) blockIdx.z * dst_frame + (size_t) y * dw + x] = src[(size_t) blockIdx.z * src_frame + (size_t) sy * sw + sx];
}

/* rmap <-> flow (ecc_remap_to_optflow / ecc_flow_to_remap, ecc2.cc:400-500) */
__global__ void k_flow_grid(const float2 * src, float2 * dst, int w, int h, size_t frame, float sign)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= w ) return;
  const size_t i = (size_t) blockIdx.z * frame + (size_t) y * w + x;
  const float2 v = src[i];
  dst[i] = make_float2(v.x + sign * (float) x, v.y + sign * (float) y);
}

}  // namespace sst

using namespace sst;

/* --------------------------------------------------------------- host side */

struct sst_eccflow {
  sst_eccflow_options o;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_user = nullptr, ev_done = nullptr;
  int w = 0, h = 0, L = 0;
  std::vector<int> lw, lh, dw, dh, from0;   // level sizes, avgdown sizes, downscale source
  std::vector<size_t> loff, doff;         // level offsets (pixels), D offsets (cells)
  size_t pyr_px = 0, d_cells = 0, max_cells = 0;
  // tap tables: per level: down (from the source level), area (to the avgdown size),
  // up (cubic from the avgdown size), next (cubic from level l + 1)
  struct Tabs {
    HostTaps hx, hy;
    DevBuf ix, wx, iy, wy;
    TapAxis ax() const { return { ix.as<int>(), wx.as<float>(), hx.K }; }
    TapAxis ay() const { return { iy.as<int>(), wy.as<float>(), hy.K }; }
  };
  std::vector<Tabs> down, area, up, next;
  DevBuf ref, tg, Dm, tmp;              // reference pyramid, {T, gx, gy}, D, tensor averages
  DevBuf cur, uv[2], avg, duv, in;      // batch buffers
  DevBuf rmask, cmask, min_;            // reference mask pyramid; current mask pyramids; staged host masks
  bool has_rmask = false;
  size_t cap = 0;

  ~sst_eccflow()
  {
    for( auto * v : { &down, &area, &up, &next } )
      for( auto & t : *v ) t.ix.release(), t.wx.release(), t.iy.release(), t.wy.release();
    DevBuf * bufs[] = { &ref, &tg, &Dm, &tmp, &cur, &uv[0], &uv[1], &avg, &duv, &in, &rmask, &cmask, &min_ };
    for( DevBuf * b : bufs ) b->release();
    if( ev_user ) cudaEventDestroy(ev_user);
    if( ev_done ) cudaEventDestroy(ev_done);
    if( st ) cudaStreamDestroy(st);
  }
};

static int ffail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_FCK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return ffail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

#define SST_FLAUNCH(call)                                                                      \
  do {                                                                                         \
    SST_FCK(call);                                                                             \
    ++launches;                                                                                \
  } while ( 0 )

#define SST_TRYF(expr)                                                                         \
  do {                                                                                         \
    int r_ = (expr);                                                                           \
    if( r_ != SST_OK ) return r_;                                                              \
  } while ( 0 )

static int upload_tabs(sst_eccflow::Tabs & t, HostTaps hx, HostTaps hy, cudaStream_t st)
{
  t.hx = std::move(hx), t.hy = std::move(hy);
  SST_FCK(t.ix.ensure(t.hx.idx.size() * sizeof(int)));
  SST_FCK(t.wx.ensure(t.hx.w.size() * sizeof(float)));
  SST_FCK(t.iy.ensure(t.hy.idx.size() * sizeof(int)));
  SST_FCK(t.wy.ensure(t.hy.w.size() * sizeof(float)));
  SST_FCK(cudaMemcpyAsync(t.ix.p, t.hx.idx.data(), t.hx.idx.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  SST_FCK(cudaMemcpyAsync(t.wx.p, t.hx.w.data(), t.hx.w.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  SST_FCK(cudaMemcpyAsync(t.iy.p, t.hy.idx.data(), t.hy.idx.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  SST_FCK(cudaMemcpyAsync(t.wy.p, t.hy.w.data(), t.hy.w.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  return SST_OK;
}

extern "C" void sst_eccflow_options_default(sst_eccflow_options * o)
{
  if( !o ) return;
  memset(o, 0, sizeof(*o));
  o->update_multiplier = 1.5;
  o->scale_factor = 0.5;
  o->noise_level = -1;
  o->max_iterations = 1;
  o->support_scale = 5;
  o->min_image_size = 4;
  o->max_pyramid_level = -1;
  o->downscale = SST_ECCFLOW_DOWNSCALE_RECURSIVE_RESIZE;
}

extern "C" int sst_eccflow_create(sst_eccflow ** out, const sst_eccflow_options * o)
{
  if( !out || !o ) return ffail(SST_ERR_INVALID_ARG, "sst_eccflow_create: NULL argument");
  if( o->support_scale < 0 || o->support_scale > 12 || o->max_iterations < 0 || o->max_iterations > 100 ||
      !(o->scale_factor > 0 && o->scale_factor < 1) || o->downscale < 0 || o->downscale > 2 )
    return ffail(SST_ERR_INVALID_ARG, "sst_eccflow_create: invalid options");
  sst_eccflow * f = new (std::nothrow) sst_eccflow();
  if( !f ) return ffail(SST_ERR_NOMEM, "out of host memory");
  f->o = *o;
  cudaError_t e = cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking);
  if( e == cudaSuccess ) e = cudaEventCreateWithFlags(&f->ev_user, cudaEventDisableTiming);
  if( e == cudaSuccess ) e = cudaEventCreateWithFlags(&f->ev_done, cudaEventDisableTiming);
  if( e != cudaSuccess ) {
    delete f;
    return ffail(SST_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = f;
  return SST_OK;
}

extern "C" int sst_eccflow_destroy(sst_eccflow * f)
{
  delete f;
  return SST_OK;
}

extern "C" int sst_eccflow_num_levels(const sst_eccflow * f)
{
  return f ? f->L : 0;
}

/* level sizes of set_reference_image (ecc2.cc:2525-2600) */
static void flow_levels(sst_eccflow * f, int w, int h)
{
  const sst_eccflow_options & o = f->o;
  const int min_size = std::max(4, o.min_image_size);
  const bool big_aspect = std::max(w, h) / std::min(w, h) >= 2;
  f->lw.assign(1, w), f->lh.assign(1, h), f->from0.assign(1, 0);
  if( !(o.max_pyramid_level >= 0 && 0 >= o.max_pyramid_level) ) {
    while ( f->lw.size() < 64 ) {
      const int pw = f->lw.back(), ph = f->lh.back();
      int nw, nh;
      if( o.downscale == SST_ECCFLOW_DOWNSCALE_PYRAMID ) {
        nw = std::max(o.min_image_size, (pw + 1) / 2), nh = std::max(o.min_image_size, (ph + 1) / 2);
        if( (nw == pw && nh == ph) || std::min(nw, nh) <= min_size ) break;
      }
      else {
        nw = std::max(o.min_image_size, (int) ((pw + 1) * o.scale_factor));
        nh = std::max(o.min_image_size, (int) ((ph + 1) * o.scale_factor));
        if( (nw == pw && nh == ph) || std::max(nw, nh) <= min_size ) break;
      }
      f->lw.push_back(nw), f->lh.push_back(nh);
      f->from0.push_back(o.downscale == SST_ECCFLOW_DOWNSCALE_FULL_RESIZE ||
          (o.downscale == SST_ECCFLOW_DOWNSCALE_RECURSIVE_RESIZE && big_aspect && std::min(nw, nh) <= min_size + 1));
      if( o.max_pyramid_level >= 0 && (int) f->lw.size() - 1 >= o.max_pyramid_level ) break;
    }
  }
  f->L = (int) f->lw.size();
  f->dw.resize(f->L), f->dh.resize(f->L), f->loff.resize(f->L), f->doff.resize(f->L);
  f->pyr_px = 0, f->d_cells = 0, f->max_cells = 0;
  for( int l = 0; l < f->L; ++l ) {
    int sw = f->lw[l], sh = f->lh[l];
    for( int i = 0; i < o.support_scale; ++i ) sw = (sw + 1) / 2, sh = (sh + 1) / 2;
    f->dw[l] = sw, f->dh[l] = sh;
    f->loff[l] = f->pyr_px, f->pyr_px += (size_t) f->lw[l] * f->lh[l];
    f->doff[l] = f->d_cells, f->d_cells += (size_t) sw * sh;
    f->max_cells = std::max(f->max_cells, (size_t) sw * sh);
  }
}

/* the mask pyramid of `n` masks whose level 0 is in place: every coarser
 * level the INTER_NEAREST resize of its downscale source level */
static int mask_pyramid(sst_eccflow * f, uint8_t * m, int n, cudaStream_t st, int & launches)
{
  for( int l = 1; l < f->L; ++l ) {
    const int s = f->from0[l] ? 0 : l - 1;
    SST_FLAUNCH((k_resize_nearest_u8_batch<<<dim3((f->lw[l] + 127) / 128, f->lh[l], n), 128, 0, st>>>(m + f->loff[s],
        f->lw[s], f->lh[s], f->pyr_px, m + f->loff[l], f->lw[l], f->lh[l], f->pyr_px), cudaGetLastError()));
  }
  return SST_OK;
}

extern "C" int sst_eccflow_set_reference_image(sst_eccflow * f, const void * img, int depth, int width, int height,
    size_t row_stride, double scale, int on_device, void * stream)
{
  return sst_eccflow_set_reference_image_masked(f, img, depth, width, height, row_stride, scale, nullptr, 0, on_device,
      stream);
}

extern "C" int sst_eccflow_set_reference_image_masked(sst_eccflow * f, const void * img, int depth, int width,
    int height, size_t row_stride, double scale, const uint8_t * mask, size_t mask_stride, int on_device, void * stream)
{
  if( !f || !img ) return ffail(SST_ERR_INVALID_ARG, "sst_eccflow_set_reference_image: NULL argument");
  if( mask && mask_stride < (size_t) width ) return ffail(SST_ERR_INVALID_ARG, "mask_stride too small");
  const int bytes = depth_bytes(depth);
  if( !bytes || width < 4 || height < 4 || row_stride < (size_t) width * bytes )
    return ffail(SST_ERR_INVALID_ARG, "sst_eccflow_set_reference_image: invalid image");
  cudaStream_t st = f->st;
  int launches = 0;
  SST_FCK(cudaEventRecord(f->ev_user, (cudaStream_t) stream));
  SST_FCK(cudaStreamWaitEvent(st, f->ev_user, 0));
  flow_levels(f, width, height);
  f->w = width, f->h = height;
  f->cap = 0;                                    // batch buffers follow the new geometry
  const sst_eccflow_options & o = f->o;
  // tap tables
  f->down.clear(), f->area.clear(), f->up.clear(), f->next.clear();
  f->down.resize(f->L), f->area.resize(f->L), f->up.resize(f->L), f->next.resize(f->L);
  for( int l = 0; l < f->L; ++l ) {
    if( l > 0 ) {
      const int s = f->from0[l] ? 0 : l - 1;
      if( o.downscale == SST_ECCFLOW_DOWNSCALE_PYRAMID ) {
        if( upload_tabs(f->down[l], pyr_taps(f->lw[s], f->lw[l]), pyr_taps(f->lh[s], f->lh[l]), st) ) return SST_ERR_CUDA;
      }
      else if( upload_tabs(f->down[l], area_taps(f->lw[s], f->lw[l]), area_taps(f->lh[s], f->lh[l]), st) ) return SST_ERR_CUDA;
    }
    if( upload_tabs(f->area[l], area_taps(f->lw[l], f->dw[l]), area_taps(f->lh[l], f->dh[l]), st) ) return SST_ERR_CUDA;
    HostTaps ux = f->dw[l] == f->lw[l] ? copy_taps(f->lw[l]) : cubic_taps(f->dw[l], f->lw[l]);
    HostTaps uy = f->dh[l] == f->lh[l] ? copy_taps(f->lh[l]) : cubic_taps(f->dh[l], f->lh[l]);
    if( upload_tabs(f->up[l], std::move(ux), std::move(uy), st) ) return SST_ERR_CUDA;
    if( l + 1 < f->L ) {
      HostTaps nx = f->lw[l + 1] == f->lw[l] ? copy_taps(f->lw[l]) : cubic_taps(f->lw[l + 1], f->lw[l]);
      HostTaps ny = f->lh[l + 1] == f->lh[l] ? copy_taps(f->lh[l]) : cubic_taps(f->lh[l + 1], f->lh[l]);
      if( upload_tabs(f->next[l], std::move(nx), std::move(ny), st) ) return SST_ERR_CUDA;
    }
  }
  // reference pyramid, {T, gx, gy}, D
  SST_FCK(f->ref.ensure(f->pyr_px * sizeof(float)));
  SST_FCK(f->tg.ensure(f->pyr_px * sizeof(float4)));
  SST_FCK(f->Dm.ensure(f->d_cells * sizeof(float4)));
  SST_FCK(f->tmp.ensure(std::max(f->max_cells * 3 * sizeof(float), f->pyr_px * sizeof(float2))));
  const void * src = img;
  if( !on_device ) {
    SST_FCK(f->in.ensure(row_stride * height));
    SST_FCK(cudaMemcpyAsync(f->in.p, img, row_stride * height, cudaMemcpyHostToDevice, st));
    src = f->in.p;
  }
  float * ref = f->ref.as<float>();
  SST_FLAUNCH(launch_convert_smooth(src, depth, 1, width, height, row_stride, row_stride * height, scale, nullptr, 0,
      ref, f->pyr_px, st));
  const float noise = (float) (o.noise_level >= 0 ? o.noise_level : 1e-3);
  for( int l = 0; l < f->L; ++l ) {
    if( l > 0 ) {
      const int s = f->from0[l] ? 0 : l - 1;
      SST_FLAUNCH((k_resample<1><<<dim3((f->lw[l] + 31) / 32, (f->lh[l] + 7) / 8, 1), 256, 0, st>>>(
          ref + f->loff[s], f->lw[s], 0, ref + f->loff[l], f->lw[l], f->lh[l], 0, f->down[l].ax(), f->down[l].ay(),
          1.f, 1.f, 0), cudaGetLastError()));
    }
    float2 * grad = f->tmp.as<float2>();
    SST_FLAUNCH(launch_ref_gradients(ref + f->loff[l], nullptr, f->lw[l], f->lh[l], grad, st));
    SST_FLAUNCH(launch_pack_reference(ref + f->loff[l], grad, (size_t) f->lw[l] * f->lh[l],
        f->tg.as<float4>() + f->loff[l], st));
    const int cells = f->dw[l] * f->dh[l];
    float * avg = f->tmp.as<float>();
    SST_FLAUNCH((k_flow_area<0><<<dim3((cells + 7) / 8, 1, 1), 256, 0, st>>>(f->tg.as<float4>() + f->loff[l], nullptr, 0,
        nullptr, 0, f->lw[l], f->lh[l], f->area[l].ax(), f->area[l].ay(), f->dw[l], f->dh[l], avg, 0), cudaGetLastError()));
    const float reg = noise > 0 ? (float) pow(1e-5 * noise / (double) (1 << std::min(l, 30)), 4) : 0.f;
    SST_FLAUNCH((k_flow_tensor<<<(cells + 127) / 128, 128, 0, st>>>(avg, f->dw[l], f->dh[l], (float) o.update_multiplier,
        reg, f->Dm.as<float4>() + f->doff[l]), cudaGetLastError()));
  }
  f->has_rmask = mask != nullptr;
  if( mask ) {
    SST_FCK(f->rmask.ensure(f->pyr_px));
    SST_FCK(cudaMemcpy2DAsync(f->rmask.p, width, mask, mask_stride, width, height,
        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    SST_TRYF(mask_pyramid(f, f->rmask.as<uint8_t>(), 1, st, launches));
  }
  SST_FCK(cudaEventRecord(f->ev_done, st));
  SST_FCK(cudaStreamWaitEvent((cudaStream_t) stream, f->ev_done, 0));
  if( !on_device ) SST_FCK(cudaStreamSynchronize(st));
  sst_internal_count_launches(launches);
  return SST_OK;
}

extern "C" int sst_eccflow_compute_batch(sst_eccflow * f, const void * frames, int depth, int n, size_t row_stride,
    size_t frame_stride, double scale, int on_device, const float * init_rmap, float * rmap_out, void * stream)
{
  return sst_eccflow_compute_batch_masked(f, frames, depth, n, row_stride, frame_stride, scale, nullptr, 0, 0,
      on_device, init_rmap, rmap_out, stream);
}

extern "C" int sst_eccflow_compute_batch_masked(sst_eccflow * f, const void * frames, int depth, int n,
    size_t row_stride, size_t frame_stride, double scale, const uint8_t * masks, size_t mask_row_stride,
    size_t mask_frame_stride, int on_device, const float * init_rmap, float * rmap_out, void * stream)
{
  if( !f || !frames || !rmap_out ) return ffail(SST_ERR_INVALID_ARG, "sst_eccflow_compute_batch: NULL argument");
  if( masks && (mask_row_stride < (size_t) f->w || mask_frame_stride < mask_row_stride * f->h) )
    return ffail(SST_ERR_INVALID_ARG, "invalid mask strides");
  if( f->L == 0 ) return ffail(SST_ERR_STATE, "c_eccflow: no reference image was set");
  if( n < 1 || n > 65535 ) return ffail(SST_ERR_INVALID_ARG, "n must be 1..65535");
  const int bytes = depth_bytes(depth);
  if( !bytes || row_stride < (size_t) f->w * bytes || frame_stride < row_stride * f->h )
    return ffail(SST_ERR_INVALID_ARG, "invalid depth or strides");
  cudaStream_t st = f->st;
  int launches = 0;
  SST_FCK(cudaEventRecord(f->ev_user, (cudaStream_t) stream));
  SST_FCK(cudaStreamWaitEvent(st, f->ev_user, 0));
  const size_t plane = (size_t) f->w * f->h;
  if( (size_t) n > f->cap ) {
    SST_FCK(f->cur.ensure((size_t) n * f->pyr_px * sizeof(float)));
    SST_FCK(f->uv[0].ensure((size_t) n * plane * sizeof(float2)));
    SST_FCK(f->uv[1].ensure((size_t) n * plane * sizeof(float2)));
    SST_FCK(f->avg.ensure((size_t) n * f->max_cells * 2 * sizeof(float)));
    SST_FCK(f->duv.ensure((size_t) n * f->max_cells * sizeof(float2)));
    f->cap = n;
  }
  const void * src = frames;
  const float * init = init_rmap;
  float2 * out = (float2 *) rmap_out;
  if( !on_device ) {
    SST_FCK(f->in.ensure(frame_stride * n + (init_rmap ? (size_t) n * plane * sizeof(float2) : 0)));
    SST_FCK(cudaMemcpyAsync(f->in.p, frames, frame_stride * n, cudaMemcpyHostToDevice, st));
    src = f->in.p;
    if( init_rmap ) {
      float * d_init = (float *) (f->in.as<uint8_t>() + frame_stride * n);
      SST_FCK(cudaMemcpyAsync(d_init, init_rmap, (size_t) n * plane * sizeof(float2), cudaMemcpyHostToDevice, st));
      init = d_init;
    }
  }
  // current pyramids of the batch (setup_input_image)
  float * cur = f->cur.as<float>();
  SST_FLAUNCH(launch_convert_smooth(src, depth, n, f->w, f->h, row_stride, frame_stride, scale, nullptr, 0, cur,
      f->pyr_px, st));
  for( int l = 1; l < f->L; ++l ) {
    const int s = f->from0[l] ? 0 : l - 1;
    SST_FLAUNCH((k_resample<1><<<dim3((f->lw[l] + 31) / 32, (f->lh[l] + 7) / 8, n), 256, 0, st>>>(cur + f->loff[s],
        f->lw[s], f->pyr_px, cur + f->loff[l], f->lw[l], f->lh[l], f->pyr_px, f->down[l].ax(), f->down[l].ay(), 1.f,
        1.f, 0), cudaGetLastError()));
  }
  // current mask pyramids (setup_input_image: INTER_NEAREST per level)
  uint8_t * cmask = nullptr;
  if( masks ) {
    SST_FCK(f->cmask.ensure((size_t) n * f->pyr_px));
    cmask = f->cmask.as<uint8_t>();
    const uint8_t * msrc = masks;
    if( !on_device ) {
      SST_FCK(f->min_.ensure(mask_frame_stride * n));
      SST_FCK(cudaMemcpyAsync(f->min_.p, masks, mask_frame_stride * n, cudaMemcpyHostToDevice, st));
      msrc = f->min_.as<uint8_t>();
    }
    for( int i = 0; i < n; ++i ) {
      SST_FCK(cudaMemcpy2DAsync(cmask + (size_t) i * f->pyr_px, f->w, msrc + (size_t) i * mask_frame_stride,
          mask_row_stride, f->w, f->h, cudaMemcpyDeviceToDevice, st));
    }
    SST_TRYF(mask_pyramid(f, cmask, n, st, launches));
  }
  // initial flow at the coarsest level
  const int Lc = f->L - 1;
  int a = 0;                                     // uv[a] holds the flow of the current level
  float2 * uv0 = f->uv[0].as<float2>(), * uv1 = f->uv[1].as<float2>();
  if( !init ) {
    SST_FCK(cudaMemsetAsync(uv0, 0, (size_t) n * plane * sizeof(float2), st));
  }
  else {
    SST_FLAUNCH((k_flow_grid<<<dim3((f->w + 127) / 128, f->h, n), 128, 0, st>>>((const float2 *) init, uv1, f->w, f->h,
        plane, -1.f), cudaGetLastError()));
    if( Lc == 0 ) {
      a = 1;
    }
    else {
      HostTaps cx = cubic_taps(f->w, f->lw[Lc]), cy = cubic_taps(f->h, f->lh[Lc]);
      sst_eccflow::Tabs t0;
      if( upload_tabs(t0, std::move(cx), std::move(cy), st) ) return SST_ERR_CUDA;
      SST_FLAUNCH((k_resample<2><<<dim3((f->lw[Lc] + 31) / 32, (f->lh[Lc] + 7) / 8, n), 256, 0, st>>>(
          (const float *) uv1, f->w, plane * 2, (float *) uv0, f->lw[Lc], f->lh[Lc], plane * 2, t0.ax(), t0.ay(),
          (float) ((double) f->lw[Lc] / f->w), (float) ((double) f->lh[Lc] / f->h), 0), cudaGetLastError()));
      SST_FCK(cudaStreamSynchronize(st));
      t0.ix.release(), t0.wx.release(), t0.iy.release(), t0.wy.release();
    }
  }
  const sst_eccflow_options & o = f->o;
  for( int l = Lc; l >= 0; --l ) {
    if( l < Lc ) {
      // uv *= size ratio, cubic to this level (compute_uv level loop)
      const float rx = (float) ((double) f->lw[l] / f->lw[l + 1]), ry = (float) ((double) f->lh[l] / f->lh[l + 1]);
      float2 * s = a ? uv1 : uv0, * d = a ? uv0 : uv1;
      SST_FLAUNCH((k_resample<2><<<dim3((f->lw[l] + 31) / 32, (f->lh[l] + 7) / 8, n), 256, 0, st>>>((const float *) s,
          f->lw[l + 1], plane * 2, (float *) d, f->lw[l], f->lh[l], plane * 2, f->next[l].ax(), f->next[l].ay(), rx, ry,
          0), cudaGetLastError()));
      a ^= 1;
    }
    float2 * u = a ? uv1 : uv0;
    const int cells = f->dw[l] * f->dh[l];
    for( int it = 0; it < o.max_iterations; ++it ) {
      SST_FLAUNCH((k_flow_area<1><<<dim3((cells + 7) / 8, 1, n), 256, 0, st>>>(f->tg.as<float4>() + f->loff[l],
          cur + f->loff[l], f->pyr_px, u, plane, f->lw[l], f->lh[l], f->area[l].ax(), f->area[l].ay(), f->dw[l],
          f->dh[l], f->avg.as<float>(), f->max_cells * 2, f->has_rmask ? f->rmask.as<uint8_t>() + f->loff[l] : nullptr,
          cmask ? cmask + f->loff[l] : nullptr, f->pyr_px), cudaGetLastError()));
      SST_FLAUNCH((k_flow_solve<<<dim3((cells + 127) / 128, 1, n), 128, 0, st>>>(f->avg.as<float>(), f->max_cells * 2,
          f->Dm.as<float4>() + f->doff[l], f->dw[l], f->dh[l], f->duv.as<float2>(), f->max_cells), cudaGetLastError()));
      SST_FLAUNCH((k_resample<2><<<dim3((f->lw[l] + 31) / 32, (f->lh[l] + 7) / 8, n), 256, 0, st>>>(
          (const float *) f->duv.as<float2>(), f->dw[l], f->max_cells * 2, (float *) u, f->lw[l], f->lh[l], plane * 2,
          f->up[l].ax(), f->up[l].ay(), 1.f, 1.f, 1), cudaGetLastError()));
    }
  }
  // rmap = uv + (x, y) at level 0
  float2 * u = a ? uv1 : uv0;
  if( on_device ) {
    SST_FLAUNCH((k_flow_grid<<<dim3((f->w + 127) / 128, f->h, n), 128, 0, st>>>(u, out, f->w, f->h, plane, 1.f),
        cudaGetLastError()));
  }
  else {
    SST_FLAUNCH((k_flow_grid<<<dim3((f->w + 127) / 128, f->h, n), 128, 0, st>>>(u, u, f->w, f->h, plane, 1.f),
        cudaGetLastError()));
    SST_FCK(cudaMemcpyAsync(rmap_out, u, (size_t) n * plane * sizeof(float2), cudaMemcpyDeviceToHost, st));
    SST_FCK(cudaStreamSynchronize(st));
  }
  SST_FCK(cudaEventRecord(f->ev_done, st));
  SST_FCK(cudaStreamWaitEvent((cudaStream_t) stream, f->ev_done, 0));
  sst_internal_count_launches(launches);
  return SST_OK;
}
