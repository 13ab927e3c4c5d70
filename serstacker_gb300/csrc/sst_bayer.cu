/*
 * sst_bayer.cu -- c_bayer_average on the GPU: the mosaic-aware accumulator of
 * raw Bayer frames (core/average/c_frame_accumulation.cc:988-1334).
 *
 * For every output pixel the reference takes the remap position p of the
 * frame, truncates it to integers (sx, sy) = ((int) p.x, (int) p.y), and when
 * the 2x2 neighbourhood is inside the frame adds each of the four raw mosaic
 * samples, with its bilinear weight times the frame weight, to the colour
 * channel of that sample's position in the Bayer pattern (_bayer_accumulate,
 * c_frame_accumulation.cc:1043-1122). compute() divides the channel sums by
 * the channel weight sums (:1205-1238).
 *
 * In the stacking pipeline the per-pixel weight is the frame's remapped
 * mask times its weight (c_image_stacking_pipeline.cc:1704-1714, 1730-1749).
 * Here the remap is the registered transform evaluated on the fly (no map in
 * HBM), each output pixel is owned by one thread that accumulates a whole
 * batch of frames in registers with compensated (Kahan-Babuska) FP32 sums,
 * and the accumulator planes are touched once per batch. Layout in HBM: 12
 * planar f32 planes of width x height: for channel c = B, G, R the sum of
 * w*I, its compensation, the sum of w, its compensation.
 *
 * The reference fills its pattern mask only over whole 2x2 cells and leaves
 * the last row / column of an odd-sized frame uninitialised (cv::Mat::create);
 * here the pattern continues by parity there.
 */
#include <new>
#include "sst_engine.cuh"
#include "sst_stack.cuh"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

namespace sst {

/* colour channel (BAYER_B = 0, BAYER_G = 1, BAYER_R = 2) of mosaic position
 * (x, y) for each COLORID pattern (generate_bayer_pattern_mask,
 * c_frame_accumulation.cc:1262-1334) */
__host__ __device__ inline int bayer_channel(int colorid, int x, int y)
{
  const int q = ((y & 1) << 1) | (x & 1);
  switch ( colorid ) {
  case SST_COLORID_BAYER_RGGB: return q == 0 ? 2 : (q == 3 ? 0 : 1);
  case SST_COLORID_BAYER_GRBG: return q == 1 ? 2 : (q == 2 ? 0 : 1);
  case SST_COLORID_BAYER_GBRG: return q == 2 ? 2 : (q == 1 ? 0 : 1);
  case SST_COLORID_BAYER_BGGR: return q == 3 ? 2 : (q == 0 ? 0 : 1);
  }
  return 1;
}

struct BayerArgs {
  const uint8_t * frames;
  size_t row_stride, frame_stride;
  int w, h, n;
  float scale;
  const float * coeffs;     // n x SST_NCOEF, or nullptr: no remap (direct accumulation)
  const float * weights;    // n effective weights
  int colorid;
  float * acc;              // 12 planes
  size_t plane;
};

/* the mosaic gather of one output pixel: (int) p truncates toward zero, so a
 * position in (-1, 0) starts at 0 with a negative right-hand weight, as in
 * the reference's interpolate lambda */
template<typename T>
__device__ __forceinline__ void bayer_gather(const uint8_t * fb, size_t rs, int w, int h, int colorid, float scale,
    spos s, float wt, float * S, float * cS, float * Wt, float * cW)
{
  int sx = s.x0, sy = s.y0;
  float bx = s.fx, by = s.fy;
  if( sx == -1 && bx > 0.f ) sx = 0, bx -= 1.f;
  if( sy == -1 && by > 0.f ) sy = 0, by -= 1.f;
  if( sx < 0 || sx >= w - 1 || sy < 0 || sy >= h - 1 ) return;
  const float ax = 1.f - bx, ay = 1.f - by;
  const float s4[4] = { ax * ay * wt, bx * ay * wt, ax * by * wt, bx * by * wt };
  const T * r0 = (const T *) (fb + (size_t) sy * rs) + sx;
  const T * r1 = (const T *) ((const uint8_t *) r0 + rs);
  const float v4[4] = { (float) __ldg(r0) * scale, (float) __ldg(r0 + 1) * scale,
                        (float) __ldg(r1) * scale, (float) __ldg(r1 + 1) * scale };
#pragma unroll
  for( int q = 0; q < 4; ++q ) {
    const int ch = bayer_channel(colorid, sx + (q & 1), sy + (q >> 1));
#pragma unroll
    for( int cc = 0; cc < 3; ++cc ) {
      if( cc == ch ) {
        kahan_add(S[cc], cS[cc], v4[q] * s4[q]);
        kahan_add(Wt[cc], cW[cc], s4[q]);
      }
    }
  }
}

constexpr int BA_TX = 64, BA_TY = 16;     // 4 output pixels per thread

/* One CTA owns a 64 x 16 tile of the accumulator and walks the frames of the
 * batch. Per output pixel the weight is the frame weight times the remapped
 * frame mask (remap of 255 LINEAR/CONSTANT 0, >= 255, 5x5 erode), the
 * current_mask the stacking pipeline hands to c_bayer_average::add. */
template<int FAM, typename T>
__global__ void __launch_bounds__(256) k_bayer_accumulate(BayerArgs a)
{
  constexpr int VW = BA_TX + 4, VH = BA_TY + 4, PPT = BA_TX * BA_TY / 256;
  __shared__ uint8_t s_v[VH * VW];
  __shared__ uint8_t s_h[VH * BA_TX];
  const int tx0 = blockIdx.x * BA_TX, ty0 = blockIdx.y * BA_TY;
  const int lx = threadIdx.x % BA_TX, ly0 = threadIdx.x / BA_TX;
  const int x = tx0 + lx;
  const int wx0 = max(tx0 - 2, 0), wy0 = max(ty0 - 2, 0);
  const int wx1 = min(tx0 + BA_TX + 1, a.w - 1), wy1 = min(ty0 + BA_TY + 1, a.h - 1);
  float S[PPT][3], cS[PPT][3], Wt[PPT][3], cW[PPT][3];
#pragma unroll
  for( int k = 0; k < PPT; ++k )
#pragma unroll
    for( int ch = 0; ch < 3; ++ch ) S[k][ch] = cS[k][ch] = Wt[k][ch] = cW[k][ch] = 0.f;
  for( int f = 0; f < a.n; ++f ) {
    const float wf = __ldg(a.weights + f);
    if( !(wf > 0.f) ) continue;                 // uniform over the CTA
    const uint8_t * fb = a.frames + (size_t) f * a.frame_stride;
    if( !a.coeffs ) {
      // no remap: acc[y][x][pattern(x, y)] += src(x, y) * w (c_frame_accumulation.cc:996-1041)
      if( x < a.w ) {
#pragma unroll
        for( int k = 0; k < PPT; ++k ) {
          const int y = ty0 + ly0 + 4 * k;
          if( y >= a.h ) continue;
          const int ch = bayer_channel(a.colorid, x, y);
          const float v = (float) __ldg((const T *) (fb + (size_t) y * a.row_stride) + x) * a.scale;
#pragma unroll
          for( int cc = 0; cc < 3; ++cc ) {
            if( cc == ch ) {
              kahan_add(S[k][cc], cS[k][cc], v * wf);
              kahan_add(Wt[k][cc], cW[k][cc], wf);
            }
          }
        }
      }
      continue;
    }
    float c[SST_NCOEF];
#pragma unroll
    for( int i = 0; i < SST_NCOEF; ++i ) c[i] = __ldg(a.coeffs + (size_t) f * SST_NCOEF + i);
    if( rect_interior<FAM>(c, wx0, wy0, wx1, wy1, a.w, a.h) ) {
      if( x < a.w ) {
#pragma unroll
        for( int k = 0; k < PPT; ++k ) {
          const int y = ty0 + ly0 + 4 * k;
          if( y < a.h )
            bayer_gather<T>(fb, a.row_stride, a.w, a.h, a.colorid, a.scale, warp_pos<FAM>(c, x, y), wf, S[k], cS[k],
                Wt[k], cW[k]);
        }
      }
      continue;
    }
    for( int q = threadIdx.x; q < VW * VH; q += 256 ) {
      const int qx = tx0 - 2 + q % VW, qy = ty0 - 2 + q / VW;
      uint8_t v = 1;
      if( qx >= 0 && qx < a.w && qy >= 0 && qy < a.h ) {
        v = mask_ok(coverage(a.w, a.h, warp_pos<FAM>(c, qx, qy)), 255) ? 1 : 0;
      }
      s_v[q] = v;
    }
    __syncthreads();
    for( int q = threadIdx.x; q < BA_TX * VH; q += 256 ) {
      const int xx = q % BA_TX, yy = q / BA_TX;
      const uint8_t * p = s_v + yy * VW + xx;
      s_h[yy * BA_TX + xx] = p[0] & p[1] & p[2] & p[3] & p[4];
    }
    __syncthreads();
    if( x < a.w ) {
#pragma unroll
      for( int k = 0; k < PPT; ++k ) {
        const int ly = ly0 + 4 * k, y = ty0 + ly;
        if( y >= a.h ) continue;
        const uint8_t * p = s_h + ly * BA_TX + lx;
        if( p[0] & p[BA_TX] & p[2 * BA_TX] & p[3 * BA_TX] & p[4 * BA_TX] )
          bayer_gather<T>(fb, a.row_stride, a.w, a.h, a.colorid, a.scale, warp_pos<FAM>(c, x, y), wf, S[k], cS[k],
              Wt[k], cW[k]);
      }
    }
    __syncthreads();
  }
  if( x < a.w ) {
#pragma unroll
    for( int k = 0; k < PPT; ++k ) {
      const int y = ty0 + ly0 + 4 * k;
      if( y >= a.h ) continue;
      const size_t i = (size_t) y * a.w + x;
#pragma unroll
      for( int ch = 0; ch < 3; ++ch ) {
        float * P = a.acc + (size_t) ch * 4 * a.plane;
        float gS = P[i], gcS = P[a.plane + i], gW = P[2 * a.plane + i], gcW = P[3 * a.plane + i];
        kahan_add(gS, gcS, S[k][ch]);
        gcS += cS[k][ch];
        kahan_add(gW, gcW, Wt[k][ch]);
        gcW += cW[k][ch];
        P[i] = gS, P[a.plane + i] = gcS, P[2 * a.plane + i] = gW, P[3 * a.plane + i] = gcW;
      }
    }
  }
}

/* compute(): channel sums / channel weights, 0 where no weight; mask = any channel weighted */
__global__ void k_bayer_compute(const float * acc, size_t plane, int n, float * avg, uint8_t * mask, float * accw)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= n ) return;
  bool any = false;
  for( int ch = 0; ch < 3; ++ch ) {
    const float * P = acc + (size_t) ch * 4 * plane;
    const double S = (double) P[i] + (double) P[plane + i];
    const double W = (double) P[2 * plane + i] + (double) P[3 * plane + i];
    if( avg ) avg[(size_t) i * 3 + ch] = W > 0 ? (float) (S / W) : 0.f;
    // get_acc_counters scales the green counter by 0.5 (c_frame_accumulation.cc:1240-1250)
    if( accw ) accw[(size_t) i * 3 + ch] = (float) (ch == 1 ? 0.5 * W : W);
    any = any || W > 0;
  }
  if( mask ) mask[i] = any ? 255 : 0;
}

template<typename T>
static cudaError_t launch_bayer_t(const BayerArgs & a, int motion, cudaStream_t st)
{
  dim3 grid((a.w + BA_TX - 1) / BA_TX, (a.h + BA_TY - 1) / BA_TY);
  switch ( motion_family(motion) ) {
  case FAM_AFFINE: k_bayer_accumulate<FAM_AFFINE, T><<<grid, 256, 0, st>>>(a); break;
  case FAM_HOMOG: k_bayer_accumulate<FAM_HOMOG, T><<<grid, 256, 0, st>>>(a); break;
  default: k_bayer_accumulate<FAM_QUAD, T><<<grid, 256, 0, st>>>(a); break;
  }
  return cudaGetLastError();
}

static cudaError_t launch_bayer(const BayerArgs & a, int motion, int depth, cudaStream_t st)
{
  switch ( depth ) {
  case SST_DEPTH_U8: return launch_bayer_t<uint8_t>(a, motion, st);
  case SST_DEPTH_U16: return launch_bayer_t<uint16_t>(a, motion, st);
  case SST_DEPTH_F32: return launch_bayer_t<float>(a, motion, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace sst

using namespace sst;

struct sst_bayer_average {
  int w = 0, h = 0, colorid = 0, frames = 0;
  float * acc = nullptr;
  float * coeffs = nullptr;
  float * weff = nullptr;
  int cap = 0;
  size_t plane() const { return (size_t) w * h; }
};

static int bfail(int code, const char * msg)
{
  return sst_internal_error(code, msg);
}

#define SST_BCK(call)                                                               \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if( e_ != cudaSuccess ) return bfail(SST_ERR_CUDA, cudaGetErrorString(e_));      \
  } while ( 0 )

static int ensure_batch(sst_bayer_average * b, int n)
{
  if( n <= b->cap ) return SST_OK;
  if( b->coeffs ) cudaFree(b->coeffs), b->coeffs = nullptr;
  if( b->weff ) cudaFree(b->weff), b->weff = nullptr;
  b->cap = 0;
  SST_BCK(cudaMalloc((void **) &b->coeffs, (size_t) n * SST_NCOEF * sizeof(float)));
  SST_BCK(cudaMalloc((void **) &b->weff, (size_t) n * sizeof(float)));
  b->cap = n;
  return SST_OK;
}

extern "C" int sst_bayer_average_create(sst_bayer_average ** out, int width, int height, int colorid)
{
  if( !out || width < 2 || height < 2 ) return bfail(SST_ERR_INVALID_ARG, "sst_bayer_average_create: invalid arguments");
  if( colorid < SST_COLORID_BAYER_RGGB || colorid > SST_COLORID_BAYER_BGGR )
    return bfail(SST_ERR_UNSUPPORTED, "only the RGGB / GRBG / GBRG / BGGR patterns are supported");
  sst_bayer_average * b = new (std::nothrow) sst_bayer_average();
  if( !b ) return bfail(SST_ERR_NOMEM, "out of host memory");
  b->w = width, b->h = height, b->colorid = colorid;
  cudaError_t e = cudaMalloc((void **) &b->acc, 12 * b->plane() * sizeof(float));
  if( e == cudaSuccess ) e = cudaMemset(b->acc, 0, 12 * b->plane() * sizeof(float));
  if( e != cudaSuccess ) {
    if( b->acc ) cudaFree(b->acc);
    delete b;
    return bfail(SST_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = b;
  return SST_OK;
}

extern "C" int sst_bayer_average_destroy(sst_bayer_average * b)
{
  if( !b ) return SST_OK;
  if( b->acc ) cudaFree(b->acc);
  if( b->coeffs ) cudaFree(b->coeffs);
  if( b->weff ) cudaFree(b->weff);
  delete b;
  return SST_OK;
}

extern "C" int sst_bayer_average_clear(sst_bayer_average * b, void * stream)
{
  if( !b ) return bfail(SST_ERR_INVALID_ARG, "NULL accumulator");
  SST_BCK(cudaMemsetAsync(b->acc, 0, 12 * b->plane() * sizeof(float), (cudaStream_t) stream));
  b->frames = 0;
  return SST_OK;
}

extern "C" int sst_bayer_average_accumulated_frames(const sst_bayer_average * b)
{
  return b ? b->frames : 0;
}

/* device scratch owned by one call */
struct TmpBuf {
  void * p = nullptr;
  ~TmpBuf() { if( p ) cudaFree(p); }
};

/* stages a host buffer on the device (on_device == 0), else returns it */
static int stage(const void * src, size_t bytes, int on_device, TmpBuf & t, cudaStream_t st, const void ** out)
{
  *out = src;
  if( on_device || !src ) return SST_OK;
  SST_BCK(cudaMalloc(&t.p, bytes));
  SST_BCK(cudaMemcpyAsync(t.p, src, bytes, cudaMemcpyHostToDevice, st));
  *out = t.p;
  return SST_OK;
}

#define SST_BTRY(expr)                   \
  do {                                   \
    const int r_ = (expr);               \
    if( r_ != SST_OK ) return r_;        \
  } while ( 0 )

extern "C" int sst_bayer_average_add_batch(sst_bayer_average * b, const void * frames, int depth, int n,
    size_t row_stride, size_t frame_stride, double scale, int on_device, const sst_motion_model * model,
    const float * params, const int32_t * status, const float * weights, void * stream)
{
  if( !b || !frames ) return bfail(SST_ERR_INVALID_ARG, "sst_bayer_average_add_batch: NULL argument");
  if( n < 1 ) return bfail(SST_ERR_INVALID_ARG, "n must be >= 1");
  const int bytes = depth == SST_DEPTH_U8 ? 1 : depth == SST_DEPTH_U16 ? 2 : depth == SST_DEPTH_F32 ? 4 : 0;
  if( !bytes ) return bfail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( row_stride < (size_t) b->w * bytes || frame_stride < row_stride * b->h || row_stride % bytes )
    return bfail(SST_ERR_INVALID_ARG, "invalid strides");
  if( model && (model->type < 0 || model->type > 7) ) return bfail(SST_ERR_INVALID_ARG, "invalid motion type");
  if( model && !params ) return bfail(SST_ERR_INVALID_ARG, "params are required with a motion model");
  cudaStream_t st = (cudaStream_t) stream;
  SST_BTRY(ensure_batch(b, n));
  TmpBuf tf, tp, ts, tw;
  const void * dframes, * dparams, * dstatus, * dweights;
  SST_BTRY(stage(frames, frame_stride * n, on_device, tf, st, &dframes));
  SST_BTRY(stage(model ? params : nullptr, (size_t) n * 12 * sizeof(float), on_device, tp, st, &dparams));
  SST_BTRY(stage(status, (size_t) n * sizeof(int32_t), on_device, ts, st, &dstatus));
  SST_BTRY(stage(weights, (size_t) n * sizeof(float), on_device, tw, st, &dweights));
  cudaError_t e = cudaSuccess;
  int launches = 0;
  if( model ) e = launch_coeffs_from_params(*model, (const float *) dparams, n, b->coeffs, st), ++launches;
  if( e == cudaSuccess ) e = launch_effective_weights((const float *) dweights, (const int32_t *) dstatus, n, b->weff, st), ++launches;
  BayerArgs a;
  a.frames = (const uint8_t *) dframes;
  a.row_stride = row_stride, a.frame_stride = frame_stride;
  a.w = b->w, a.h = b->h, a.n = n;
  a.scale = (float) scale;
  a.coeffs = model ? b->coeffs : nullptr;
  a.weights = b->weff;
  a.colorid = b->colorid;
  a.acc = b->acc;
  a.plane = b->plane();
  if( e == cudaSuccess ) e = launch_bayer(a, model ? model->type : SST_MOTION_TRANSLATION, depth, st), ++launches;
  if( e == cudaSuccess ) sst_internal_count_launches(launches);
  // staged host buffers are freed on return: wait for the kernels that read them
  if( !on_device && e == cudaSuccess ) e = cudaStreamSynchronize(st);
  if( e != cudaSuccess ) return bfail(SST_ERR_CUDA, cudaGetErrorString(e));
  b->frames += n;
  return SST_OK;
}

extern "C" int sst_bayer_average_compute(sst_bayer_average * b, float * avg, uint8_t * mask, float * accw,
    int on_device, void * stream)
{
  if( !b ) return bfail(SST_ERR_INVALID_ARG, "NULL accumulator");
  if( b->frames < 1 ) return bfail(SST_ERR_STATE, "no frames accumulated");
  cudaStream_t st = (cudaStream_t) stream;
  const size_t N = b->plane();
  float * da = avg, * dw = accw;
  uint8_t * dm = mask;
  TmpBuf ta, tm, tw;
  if( !on_device ) {
    if( avg ) {
      SST_BCK(cudaMalloc(&ta.p, N * 3 * sizeof(float)));
      da = (float *) ta.p;
    }
    if( mask ) {
      SST_BCK(cudaMalloc(&tm.p, N));
      dm = (uint8_t *) tm.p;
    }
    if( accw ) {
      SST_BCK(cudaMalloc(&tw.p, N * 3 * sizeof(float)));
      dw = (float *) tw.p;
    }
  }
  k_bayer_compute<<<(unsigned) ((N + 255) / 256), 256, 0, st>>>(b->acc, N, (int) N, da, dm, dw);
  cudaError_t e = cudaGetLastError();
  if( e == cudaSuccess ) sst_internal_count_launches(1);
  if( !on_device ) {
    if( e == cudaSuccess && avg ) e = cudaMemcpyAsync(avg, da, N * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if( e == cudaSuccess && mask ) e = cudaMemcpyAsync(mask, dm, N, cudaMemcpyDeviceToHost, st);
    if( e == cudaSuccess && accw ) e = cudaMemcpyAsync(accw, dw, N * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if( e == cudaSuccess ) e = cudaStreamSynchronize(st);
  }
  if( e != cudaSuccess ) return bfail(SST_ERR_CUDA, cudaGetErrorString(e));
  return SST_OK;
}

/* checkpoint / merge of the 12 compensated planes (host buffer of 12 x width x height f32) */
extern "C" int sst_bayer_average_save_state(sst_bayer_average * b, float * state12, int32_t * frames, void * stream)
{
  if( !b || !state12 ) return bfail(SST_ERR_INVALID_ARG, "sst_bayer_average_save_state: NULL argument");
  cudaStream_t st = (cudaStream_t) stream;
  SST_BCK(cudaMemcpyAsync(state12, b->acc, 12 * b->plane() * sizeof(float), cudaMemcpyDeviceToHost, st));
  SST_BCK(cudaStreamSynchronize(st));
  if( frames ) *frames = b->frames;
  return SST_OK;
}

extern "C" int sst_bayer_average_load_state(sst_bayer_average * b, const float * state12, int32_t frames, void * stream)
{
  if( !b || !state12 || frames < 0 ) return bfail(SST_ERR_INVALID_ARG, "sst_bayer_average_load_state: invalid arguments");
  cudaStream_t st = (cudaStream_t) stream;
  SST_BCK(cudaMemcpyAsync(b->acc, state12, 12 * b->plane() * sizeof(float), cudaMemcpyHostToDevice, st));
  SST_BCK(cudaStreamSynchronize(st));
  b->frames = frames;
  return SST_OK;
}
