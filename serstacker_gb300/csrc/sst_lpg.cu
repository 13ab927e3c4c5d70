/*
 * sst_lpg.cu -- the LPG sharpness map on the GPU (lpg(), core/proc/lpg.cc:
 * 223-291; c_lpg_sharpness_measure, core/proc/sharpness_measure/
 * c_lpg_sharpness_measure.h:22-28, 44-80) for batches of mono frames.
 *
 * Per batch (grid.z = frame):
 *   1. convert (1 / maxval of the depth) and the dscale pyrDowns
 *      (BORDER_REFLECT_101, lpg.cc downscale :134-155), the 1 / (1 + dscale)
 *      factor folded into the first pass (k_resample_taps);
 *   2. k_lpg5x5: alpha lap^2 + beta |grad|^2 + eps with the 5 x 5 noise-robust
 *      Laplacian and extended Sobel gradient (lpg.cc:60-131); the two outer
 *      rows and columns take their inner neighbours' values;
 *   3. the (uscale - dscale) further pyrDowns, then k_scale_pow: times
 *      (uscale - dscale), raised to p (cv::pow);
 *   4. the pyrUp chain back to the frame size (lpg.cc upscale :157-185);
 *   5. the metric mean(map) (masked): FP64 partial sums per (frame, block),
 *      added on the host in a fixed order.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <new>
#include <string>
#include <vector>

#include "sst_host.h"
#include "sst_taps.h"
#include "sst_resample.cuh"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu

namespace sst {

/* compute_lpg_5x5_parallel (lpg.cc:60-131) over a batch; edge rows / columns
 * evaluate at the nearest inner position (the reference copies them) */
__global__ void __launch_bounds__(256) k_lpg5x5(const float * s, int w, int h, size_t frame, float alpha, float beta,
    float eps, float * m)
{
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if( x >= w || y >= h ) return;
  const float * b = s + (size_t) blockIdx.z * frame;
  const int c = min(max(x, 2), w - 3), yc = min(max(y, 2), h - 3);
  const float * r0 = b + (size_t) (yc - 2) * w, * r1 = r0 + w, * r2 = r1 + w, * r3 = r2 + w, * r4 = r3 + w;
  const float gx = (r0[c + 2] + 2 * r1[c + 2] + 4 * r2[c + 2] + 2 * r3[c + 2] + r4[c + 2]) -
      (r0[c - 2] + 2 * r1[c - 2] + 4 * r2[c - 2] + 2 * r3[c - 2] + r4[c - 2]) +
      2.0f * ((r1[c + 1] + 2 * r2[c + 1] + r3[c + 1]) - (r1[c - 1] + 2 * r2[c - 1] + r3[c - 1]));
  const float gy = (r4[c - 2] + 2 * r4[c - 1] + 4 * r4[c] + 2 * r4[c + 1] + r4[c + 2]) -
      (r0[c - 2] + 2 * r0[c - 1] + 4 * r0[c] + 2 * r0[c + 1] + r0[c + 2]) +
      2.0f * ((r3[c - 1] + 2 * r3[c] + r3[c + 1]) - (r1[c - 1] + 2 * r1[c] + r1[c + 1]));
  const float lv = 16.0f * r2[c] - 2.0f * (r1[c] + r3[c] + r2[c - 1] + r2[c + 1]) -
      (r1[c - 1] + r1[c + 1] + r3[c - 1] + r3[c + 1]) - (r0[c] + r4[c] + r2[c - 2] + r2[c + 2]);
  m[(size_t) blockIdx.z * frame + (size_t) y * w + x] = alpha * (lv * lv) + beta * (gx * gx + gy * gy) + eps;
}

/* m = pow(m * mul, p) (p == 1: no power), grid.z = frame */
__global__ void k_scale_pow(float * m, size_t plane, float mul, float p)
{
  const size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if( i >= plane ) return;
  float * v = m + (size_t) blockIdx.z * plane + i;
  const float a = *v * mul;
  *v = p == 1.f ? a : (p == 2.f ? a * a : powf(a, p));
}

/* FP64 partial sums of each frame's map (masked) and of its pixel count:
 * block b of frame z writes part[(z * nb + b) * 2 + {0, 1}] */
__global__ void __launch_bounds__(256) k_map_sums(const float * m, size_t plane, const uint8_t * masks,
    size_t mask_frame, int nb, double * part)
{
  __shared__ double ss[256], sn[256];
  const float * mz = m + (size_t) blockIdx.z * plane;
  const uint8_t * mk = masks ? masks + (size_t) blockIdx.z * mask_frame : nullptr;
  double s = 0, c = 0;
  for( size_t i = (size_t) blockIdx.x * 256 + threadIdx.x; i < plane; i += (size_t) nb * 256 ) {
    if( mk && !mk[i] ) continue;
    s += mz[i], c += 1;
  }
  ss[threadIdx.x] = s, sn[threadIdx.x] = c;
  __syncthreads();
  for( int o = 128; o > 0; o >>= 1 ) {
    if( threadIdx.x < o ) ss[threadIdx.x] += ss[threadIdx.x + o], sn[threadIdx.x] += sn[threadIdx.x + o];
    __syncthreads();
  }
  if( threadIdx.x == 0 ) {
    part[((size_t) blockIdx.z * nb + blockIdx.x) * 2] = ss[0];
    part[((size_t) blockIdx.z * nb + blockIdx.x) * 2 + 1] = sn[0];
  }
}

}  // namespace sst

using namespace sst;

namespace {

int lfail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_LCK(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if( e_ != cudaSuccess ) return lfail(SST_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while ( 0 )

}  // namespace

extern "C" void sst_lpg_options_default(sst_lpg_options * o)
{
  if( !o ) return;
  o->k = 2, o->p = 2, o->dscale = 2, o->uscale = 6;
}

struct sst_lpg {
  sst_lpg_options o;
  int w = 0, h = 0, depth = -1;
  std::vector<int> dw, dh;        // sizes after each dscale pyrDown (index 0: the frame)
  std::vector<int> uw, uh;        // sizes after each further pyrDown of the map
  std::vector<int> pw, ph;        // pyrUp chain: the frame's size halved down to just above the map's
  std::vector<Resampler> down, mdown, up;
  DevBuf buf[2], part, mk;
  ~sst_lpg()
  {
    for( auto * v : { &down, &mdown, &up } )
      for( auto & r : *v ) r.release();
    buf[0].release(), buf[1].release(), part.release(), mk.release();
  }
};

extern "C" int sst_lpg_create(sst_lpg ** out, const sst_lpg_options * opts)
{
  if( !out ) return lfail(SST_ERR_INVALID_ARG, "sst_lpg_create: out is NULL");
  sst_lpg_options o;
  if( opts ) o = *opts;
  else sst_lpg_options_default(&o);
  if( !(o.k >= 0) || o.dscale < 0 || o.dscale > 16 || o.uscale < 0 || o.uscale > 16 )
    return lfail(SST_ERR_INVALID_ARG, "invalid LPG options");
  sst_lpg * h = new (std::nothrow) sst_lpg();
  if( !h ) return lfail(SST_ERR_NOMEM, "out of host memory");
  h->o = o;
  *out = h;
  return SST_OK;
}

extern "C" int sst_lpg_destroy(sst_lpg * h)
{
  delete h;
  return SST_OK;
}

/* lpg.cc downscale(): sizes of `level` pyrDowns from (w, h), stopping once the
 * smaller side is below 4 (none at all when the source is already) */
static void downscale_sizes(int w, int h, int level, std::vector<int> & ws, std::vector<int> & hs)
{
  ws.assign(1, w), hs.assign(1, h);
  if( std::min(w, h) < 4 ) return;
  for( int l = 0; l < level; ++l ) {
    ws.push_back((ws.back() + 1) / 2), hs.push_back((hs.back() + 1) / 2);
    if( std::min(ws.back(), hs.back()) < 4 ) break;
  }
}

static int plan(sst_lpg * L, int w, int h, int depth, cudaStream_t st)
{
  if( L->w == w && L->h == h && L->depth == depth ) return SST_OK;
  for( auto * v : { &L->down, &L->mdown, &L->up } ) {
    for( auto & r : *v ) r.release();
    v->clear();
  }
  L->w = L->h = 0;
  const sst_lpg_options & o = L->o;
  downscale_sizes(w, h, o.dscale > 0 ? o.dscale : 0, L->dw, L->dh);
  const int sw = L->dw.back(), sh = L->dh.back();
  if( sw < 5 || sh < 5 ) return lfail(SST_ERR_INVALID_ARG, "the LPG map is smaller than 5 x 5 after dscale");
  if( o.uscale > 0 && o.uscale > o.dscale ) downscale_sizes(sw, sh, o.uscale - o.dscale, L->uw, L->uh);
  else L->uw.assign(1, sw), L->uh.assign(1, sh);
  const int mw = L->uw.back(), mh = L->uh.back();
  // the pyrUp chain (lpg.cc:157-185): sizes halved from the frame's until the map's
  L->pw.assign(1, w), L->ph.assign(1, h);
  if( mw != w || mh != h ) {
    while ( true ) {
      const int nw = (L->pw.back() + 1) / 2, nh = (L->ph.back() + 1) / 2;
      if( nw == mw && nh == mh ) break;
      if( nw < mw || nh < mh ) return lfail(SST_ERR_INVALID_ARG, "LPG upscale: sizes do not chain");
      L->pw.push_back(nw), L->ph.push_back(nh);
    }
  }
  // tables: the first dscale pass also converts (identity taps when there is none)
  const int nd = (int) L->dw.size() - 1;
  if( nd == 0 ) {
    L->down.resize(1);
    SST_LCK(L->down[0].upload(copy_taps(w), copy_taps(h), w, h, w, h, st));
  }
  else {
    L->down.resize(nd);
    for( int l = 0; l < nd; ++l ) {
      SST_LCK(L->down[l].upload(pyr_taps(L->dw[l], L->dw[l + 1]), pyr_taps(L->dh[l], L->dh[l + 1]), L->dw[l], L->dh[l],
          L->dw[l + 1], L->dh[l + 1], st));
    }
  }
  const int nu = (int) L->uw.size() - 1;
  L->mdown.resize(nu);
  for( int l = 0; l < nu; ++l ) {
    SST_LCK(L->mdown[l].upload(pyr_taps(L->uw[l], L->uw[l + 1]), pyr_taps(L->uh[l], L->uh[l + 1]), L->uw[l], L->uh[l],
        L->uw[l + 1], L->uh[l + 1], st));
  }
  const int np = mw != w || mh != h ? (int) L->pw.size() : 0;
  L->up.resize(np);
  for( int i = 0; i < np; ++i ) {
    // step i: to pw[np - 1 - i] from the next smaller size (the map for i = 0)
    const int k = np - 1 - i;
    const int fw = k + 1 < (int) L->pw.size() ? L->pw[k + 1] : mw, fh = k + 1 < (int) L->ph.size() ? L->ph[k + 1] : mh;
    SST_LCK(L->up[i].upload(pyrup_taps(fw, L->pw[k]), pyrup_taps(fh, L->ph[k]), fw, fh, L->pw[k], L->ph[k], st));
  }
  L->w = w, L->h = h, L->depth = depth;
  return SST_OK;
}

extern "C" int sst_lpg_compute(sst_lpg * L, const void * frames, int depth, int n, int width, int height,
    size_t row_stride, size_t frame_stride, const uint8_t * masks, size_t mask_row_stride, size_t mask_frame_stride,
    int on_device, float * maps, double * metrics, void * stream)
{
  if( !L || !frames ) return lfail(SST_ERR_INVALID_ARG, "sst_lpg_compute: NULL argument");
  const int bytes = depth_bytes(depth);
  if( !bytes ) return lfail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( n < 1 || n > 65535 || width < 5 || height < 5 ) return lfail(SST_ERR_INVALID_ARG, "invalid batch or size");
  if( row_stride < (size_t) width * bytes || frame_stride < row_stride * height )
    return lfail(SST_ERR_INVALID_ARG, "invalid strides");
  if( masks && (mask_row_stride < (size_t) width || mask_frame_stride < mask_row_stride * height) )
    return lfail(SST_ERR_INVALID_ARG, "invalid mask strides");
  cudaStream_t st = (cudaStream_t) stream;
  int r = plan(L, width, height, depth, st);
  if( r != SST_OK ) return r;
  const sst_lpg_options & o = L->o;
  const size_t plane = (size_t) width * height;
  SST_LCK(L->buf[0].ensure((size_t) n * plane * sizeof(float)));
  SST_LCK(L->buf[1].ensure((size_t) n * plane * sizeof(float)));
  ScopedBuf tf;
  const void * src = frames;
  if( !on_device ) {
    SST_LCK(tf.ensure(frame_stride * n));
    SST_LCK(cudaMemcpyAsync(tf.p, frames, frame_stride * n, cudaMemcpyHostToDevice, st));
    src = tf.p;
  }
  // 1. convert (1 / maxval) and dscale, with 1 / (1 + dscale)
  const double maxval = depth == SST_DEPTH_U8 ? 255.0 : depth == SST_DEPTH_U16 ? 65535.0 : 1.0;
  const double conv = (1.0 / maxval) * (o.dscale > 0 ? 1.0 / (1 + o.dscale) : 1.0);
  float * cur = L->buf[0].as<float>(), * oth = L->buf[1].as<float>();
  const void * s = src;
  int sd = depth;
  size_t srow = row_stride, sframe = frame_stride;
  for( size_t l = 0; l < L->down.size(); ++l ) {
    const Resampler & R = L->down[l];
    SST_LCK(R.run(s, sd, srow, sframe, n, l == 0 ? conv : 1.0, cur, (size_t) R.dw * R.dh, st));
    s = cur, sd = SST_DEPTH_F32, srow = (size_t) R.dw * sizeof(float), sframe = (size_t) R.dw * R.dh * sizeof(float);
    std::swap(cur, oth);
  }
  // 2. the 5 x 5 map
  const int sw = L->dw.back(), sh = L->dh.back();
  const double l_norm = 100.0 / 4.0, g_norm = 100.0 / 36.0;
  const float alpha = (float) (o.k / (o.k + 1) * l_norm * l_norm), beta = (float) (1.0 / (o.k + 1) * g_norm * g_norm);
  {
    dim3 grid((sw + 31) / 32, (sh + 7) / 8, n);
    k_lpg5x5<<<grid, 256, 0, st>>>((const float *) s, sw, sh, (size_t) sw * sh, alpha, beta, 1e-9f, cur);
    sst_internal_count_launches(1);
    SST_LCK(cudaGetLastError());
    s = cur, srow = (size_t) sw * sizeof(float), sframe = (size_t) sw * sh * sizeof(float);
    std::swap(cur, oth);
  }
  // 3. uscale pyrDowns, then times (uscale - dscale) and the power p
  for( const Resampler & R : L->mdown ) {
    SST_LCK(R.run(s, SST_DEPTH_F32, srow, sframe, n, 1.0, cur, (size_t) R.dw * R.dh, st));
    s = cur, srow = (size_t) R.dw * sizeof(float), sframe = (size_t) R.dw * R.dh * sizeof(float);
    std::swap(cur, oth);
  }
  const int mw = L->uw.back(), mh = L->uh.back();
  const float mul = o.uscale > 0 && o.uscale > o.dscale ? (float) (o.uscale - o.dscale) : 1.f;
  const float p = (o.p != 0 && o.p != 1) ? (float) o.p : 1.f;
  if( mul != 1.f || p != 1.f ) {
    const size_t mp = (size_t) mw * mh;
    k_scale_pow<<<dim3((unsigned) ((mp + 255) / 256), 1, n), 256, 0, st>>>((float *) s, mp, mul, p);
    sst_internal_count_launches(1);
    SST_LCK(cudaGetLastError());
  }
  // 4. the pyrUp chain to the frame size
  for( const Resampler & R : L->up ) {
    SST_LCK(R.run(s, SST_DEPTH_F32, srow, sframe, n, 1.0, cur, (size_t) R.dw * R.dh, st));
    s = cur, srow = (size_t) R.dw * sizeof(float), sframe = (size_t) R.dw * R.dh * sizeof(float);
    std::swap(cur, oth);
  }
  const float * mapd = (const float *) s;   // n x width x height, packed
  // 5. the metric
  if( metrics ) {
    const uint8_t * mk = nullptr;
    if( masks ) {
      SST_LCK(L->mk.ensure((size_t) n * plane));
      for( int i = 0; i < n; ++i ) {
        SST_LCK(cudaMemcpy2DAsync(L->mk.as<uint8_t>() + (size_t) i * plane, width, masks + (size_t) i * mask_frame_stride,
            mask_row_stride, width, height, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
      }
      mk = L->mk.as<uint8_t>();
    }
    const int nb = 64;
    SST_LCK(L->part.ensure((size_t) n * nb * 2 * sizeof(double)));
    k_map_sums<<<dim3(nb, 1, n), 256, 0, st>>>(mapd, plane, mk, plane, nb, L->part.as<double>());
    sst_internal_count_launches(1);
    SST_LCK(cudaGetLastError());
    std::vector<double> hp((size_t) n * nb * 2);
    SST_LCK(cudaMemcpyAsync(hp.data(), L->part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    SST_LCK(cudaStreamSynchronize(st));
    for( int i = 0; i < n; ++i ) {
      double a = 0, c = 0;
      for( int b = 0; b < nb; ++b ) a += hp[((size_t) i * nb + b) * 2], c += hp[((size_t) i * nb + b) * 2 + 1];
      metrics[i] = c > 0 ? a / c : 0;
    }
  }
  if( maps ) {
    SST_LCK(cudaMemcpyAsync(maps, mapd, (size_t) n * plane * sizeof(float),
        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
  }
  SST_LCK(cudaStreamSynchronize(st));
  return SST_OK;
}
