/*
 * sst_adjoint.cu -- the warp residual objective of a batch of frames and its
 * hand-written adjoint (no counterpart in the reference, whose registration
 * is not differentiable; this is the differentiable form of the ECC residual
 * that c_ecc_forward_additive / c_ecclm minimise, ecc2.cc:1247-1365,
 * 1444-1650).
 *
 * For frame f with motion parameters p_f and an optional dense flow u_f:
 *
 *   r_f(x) = I_f(W(x; p_f) + u_f(x)) - T(x)     bilinear, BORDER_REPLICATE
 *   L_f    = 1/2 sum_x r_f(x)^2
 *
 *   dL_f/dp_f = sum_x r_f(x) J(x)     J = grad I at the sample (the exact
 *                                       derivative of the bilinear interpolant)
 *                                       times dW/dp (the steepest-descent row)
 *   dL_f/dT   = -r_f                   dL_f/du_f(x) = r_f(x) grad I
 *
 * The backward pass recomputes the warp (nothing of the forward pass is
 * stored). One kernel forms per pixel V = [J (M), r] and accumulates the
 * tile's Gram matrix V^T V on the tensor cores: its blocks are the
 * Gauss-Newton matrix J^T J, the gradient J^T r and 2 L. The template
 * gradient sums -r over the frames per pixel in a fixed order (one thread
 * per pixel, no atomics).
 */
#include <cuda_runtime.h>
#include <string.h>
#include <string>

#include "sst_engine.cuh"
#include "sst_kernels.cuh"
#include "sst_host.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

namespace sst {

constexpr int AJ_TX = 64, AJ_TY = 16;

struct ResidArgs {
  const float * frames;       // n x h x w
  size_t frame_stride;        // floats
  const float * tmpl;         // h x w
  const float2 * flow;        // n x h x w or nullptr
  const float * coeffs;       // n x 16 warp coefficients
  const float * jcs;          // n x 8 steepest-descent coefficients
  int w, h, n, tiles_x, tiles;
  double * partials;          // n x tiles x NS
  float2 * grad_flow;         // n x h x w or nullptr (scaled by grad_loss)
  const double * grad_loss;   // n or nullptr (1)
};

/* bilinear value and exact gradient at (sx, sy), BORDER_REPLICATE */
__device__ __forceinline__ float bilinear_grad(const float * img, int w, int h, float sx, float sy, float & gX, float & gY)
{
  const float fx0 = floorf(fminf(fmaxf(sx, -1e8f), 1e8f)), fy0 = floorf(fminf(fmaxf(sy, -1e8f), 1e8f));
  const float ax = sx - fx0, ay = sy - fy0;
  const int x0 = (int) fx0, y0 = (int) fy0;
  const int xa = clampi(x0, 0, w - 1), xb = clampi(x0 + 1, 0, w - 1);
  const int ya = clampi(y0, 0, h - 1), yb = clampi(y0 + 1, 0, h - 1);
  const float v00 = __ldg(img + (size_t) ya * w + xa), v01 = __ldg(img + (size_t) ya * w + xb);
  const float v10 = __ldg(img + (size_t) yb * w + xa), v11 = __ldg(img + (size_t) yb * w + xb);
  gX = fmaf(ay, (v11 - v10) - (v01 - v00), v01 - v00);
  gY = fmaf(ax, (v11 - v01) - (v10 - v00), v10 - v00);
  const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
  return fmaf(ay, t1 - t0, t0);
}

/* sample position of pixel (x, y): W(x; p) + u(x) */
template<int FAM>
__device__ __forceinline__ void sample_pos(const float * c, const float2 * flow, int x, int y, int w, float & sx, float & sy)
{
  float dx, dy;
  warp_disp<FAM>(c, (float) x, (float) y, dx, dy);
  sx = (float) (x + (int) c[12]) + dx;
  sy = (float) (y + (int) c[13]) + dy;
  if( flow ) {
    const float2 u = flow[(size_t) y * w + x];
    sx += u.x, sy += u.y;
  }
}

/* per tile: Gram matrix of V = [J (M), r] -> sums H (packed lower), J^T r, r^2 */
template<int FAM, int JK, int M>
__global__ void __launch_bounds__(256) k_residual_tiles(ResidArgs a)
{
  constexpr int nH = M * (M + 1) / 2, NS = nH + M + 1;
  static_assert(M + 1 <= 16, "V must fit 16 components");
  __shared__ __align__(16) float s_v[8][32 * GV_LD];
  __shared__ float s_c[24];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int f = blockIdx.y;
  const float * img = a.frames + (size_t) f * a.frame_stride;
  const float2 * flow = a.flow ? a.flow + (size_t) f * a.w * a.h : nullptr;
  if( threadIdx.x < 16 ) s_c[threadIdx.x] = a.coeffs[(size_t) f * SST_NCOEF + threadIdx.x];
  else if( threadIdx.x < 24 ) s_c[threadIdx.x] = a.jcs[(size_t) f * 8 + threadIdx.x - 16];
  __syncthreads();
  float c[16], jc[8];
#pragma unroll
  for( int i = 0; i < 16; ++i ) c[i] = s_c[i];
#pragma unroll
  for( int i = 0; i < 8; ++i ) jc[i] = s_c[16 + i];
  const float gl = a.grad_loss ? (float) a.grad_loss[f] : 1.f;
  for( int t = blockIdx.x; t < a.tiles; t += gridDim.x ) {
    const int tx0 = (t % a.tiles_x) * AJ_TX, ty0 = (t / a.tiles_x) * AJ_TY;
    const int x = tx0 + (threadIdx.x & (AJ_TX - 1));
    float g0[4] = { 0.f, 0.f, 0.f, 0.f }, g1[4] = { 0.f, 0.f, 0.f, 0.f };
    float * sv = s_v[wid];
#pragma unroll 1
    for( int k = 0; k < AJ_TY / 4; ++k ) {
      const int y = ty0 + (threadIdx.x >> 6) + 4 * k;
      float v[16];
#pragma unroll
      for( int q = 0; q < 16; ++q ) v[q] = 0.f;
      if( x < a.w && y < a.h ) {
        float sx, sy, gX, gY;
        sample_pos<FAM>(c, flow, x, y, a.w, sx, sy);
        const float I = bilinear_grad(img, a.w, a.h, sx, sy, gX, gY);
        const float r = I - __ldg(a.tmpl + (size_t) y * a.w + x);
        float J[M];
        sd_pixel<JK, M>(jc, (float) x, (float) y, gX, gY, J);
#pragma unroll
        for( int q = 0; q < M; ++q ) v[q] = J[q];
        v[M] = r;
        if( a.grad_flow ) a.grad_flow[(size_t) f * a.w * a.h + (size_t) y * a.w + x] = make_float2(gl * r * gX, gl * r * gY);
      }
      __syncwarp();
      float4 * dst = reinterpret_cast<float4 *>(sv + lane * GV_LD);
#pragma unroll
      for( int q = 0; q < 4; ++q ) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      __syncwarp();
      gram_accumulate(sv, g0, g1);
    }
    __syncwarp();
    {
      const int gq = lane >> 2, tq = lane & 3;
      sv[gq * 16 + 2 * tq] = g0[0], sv[gq * 16 + 2 * tq + 1] = g0[1];
      sv[(gq + 8) * 16 + 2 * tq] = g0[2], sv[(gq + 8) * 16 + 2 * tq + 1] = g0[3];
      sv[gq * 16 + 8 + 2 * tq] = g1[0], sv[gq * 16 + 8 + 2 * tq + 1] = g1[1];
      sv[(gq + 8) * 16 + 8 + 2 * tq] = g1[2], sv[(gq + 8) * 16 + 8 + 2 * tq + 1] = g1[3];
    }
    __syncthreads();
    if( threadIdx.x < NS ) {
      int gi, gj;
      const int k = threadIdx.x;
      if( k < nH ) {
        int r = 0;
        while ( (r + 1) * (r + 2) / 2 <= k ) ++r;
        gi = r, gj = k - r * (r + 1) / 2;
      }
      else if( k < nH + M ) gi = k - nH, gj = M;
      else gi = gj = M;
      double s = 0;
#pragma unroll
      for( int wv = 0; wv < 8; ++wv ) s += (double) s_v[wv][gi * 16 + gj];
      a.partials[((size_t) f * a.tiles + t) * NS + k] = s;
    }
    __syncthreads();
  }
}

/* per frame: combine the tiles in a fixed order (one warp per frame):
 * loss, gradient (scaled by grad_loss) and Gauss-Newton matrix */
__global__ void k_residual_combine(const double * partials, int n, int tiles, int M, const double * grad_loss,
    double * loss, float * grad_p, double * hess)
{
  const int lane = threadIdx.x & 31;
  const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if( f >= n ) return;
  const int nH = M * (M + 1) / 2, NS = nH + M + 1;
  const double * P = partials + (size_t) f * tiles * NS;
  const double gl = grad_loss ? grad_loss[f] : 1.0;
  for( int k = 0; k < NS; ++k ) {
    double v = 0;
    for( int t = lane; t < tiles; t += 32 ) v += P[(size_t) t * NS + k];
    v = warp_sum(v);
    if( lane != 0 ) continue;
    if( k < nH ) {
      if( hess ) {
        int r = 0;
        while ( (r + 1) * (r + 2) / 2 <= k ) ++r;
        const int c = k - r * (r + 1) / 2;
        hess[(size_t) f * 144 + r * M + c] = hess[(size_t) f * 144 + c * M + r] = v;
      }
    }
    else if( k < nH + M ) {
      if( grad_p ) grad_p[(size_t) f * 12 + (k - nH)] = (float) (gl * v);
    }
    else if( loss ) loss[f] = 0.5 * v;
  }
}

/* dL/dT(x) = -sum_f grad_loss_f r_f(x), frames summed in order per pixel */
template<int FAM>
__global__ void k_grad_template(ResidArgs a, float * grad_t)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if( x >= a.w ) return;
  const float T = __ldg(a.tmpl + (size_t) y * a.w + x);
  double s = 0;
  for( int f = 0; f < a.n; ++f ) {
    float c[16];
#pragma unroll
    for( int i = 0; i < 16; ++i ) c[i] = __ldg(a.coeffs + (size_t) f * SST_NCOEF + i);
    float sx, sy, gX, gY;
    sample_pos<FAM>(c, a.flow ? a.flow + (size_t) f * a.w * a.h : nullptr, x, y, a.w, sx, sy);
    const float r = bilinear_grad(a.frames + (size_t) f * a.frame_stride, a.w, a.h, sx, sy, gX, gY) - T;
    s += (a.grad_loss ? a.grad_loss[f] : 1.0) * (double) r;
  }
  grad_t[(size_t) y * a.w + x] = (float) -s;
}

/* per-frame warp and steepest-descent coefficients from parameter vectors */
__global__ void k_adjoint_coeffs(sst_motion_model m, const float * params, int n, float * coeffs, float * jcs)
{
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if( f >= n ) return;
  double s[16], p[12];
  model_identity(m, s);
  const int M = model_nparams(m);
  for( int j = 0; j < M; ++j ) p[j] = params[(size_t) f * 12 + j];
  model_set_params(m, s, p);
  model_warp_coeffs(m, s, coeffs + (size_t) f * SST_NCOEF);
  model_sd_coeffs(m, s, jcs + (size_t) f * 8);
}

template<int FAM, int JK, int M>
static cudaError_t launch_tiles(const ResidArgs & a, cudaStream_t st)
{
  dim3 grid(std::min(a.tiles, 1024), a.n);
  k_residual_tiles<FAM, JK, M><<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

static cudaError_t launch_tiles_m(int type, int M, const ResidArgs & a, cudaStream_t st)
{
  switch ( type ) {
  case SST_MOTION_TRANSLATION: return launch_tiles<FAM_AFFINE, J_TRANS, 2>(a, st);
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN:
    return M == 3 ? launch_tiles<FAM_AFFINE, J_EUCL, 3>(a, st) : launch_tiles<FAM_AFFINE, J_EUCL, 4>(a, st);
  case SST_MOTION_AFFINE: return launch_tiles<FAM_AFFINE, J_AFFINE, 6>(a, st);
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: return launch_tiles<FAM_HOMOG, J_HOMOG, 8>(a, st);
  case SST_MOTION_SEMI_QUADRATIC: return launch_tiles<FAM_QUAD, J_SEMIQ, 8>(a, st);
  case SST_MOTION_QUADRATIC: return launch_tiles<FAM_QUAD, J_QUAD, 12>(a, st);
  }
  return cudaErrorInvalidValue;
}

static cudaError_t launch_grad_t(int type, const ResidArgs & a, float * gt, cudaStream_t st)
{
  dim3 grid((a.w + 127) / 128, a.h);
  switch ( motion_family(type) ) {
  case FAM_AFFINE: k_grad_template<FAM_AFFINE><<<grid, 128, 0, st>>>(a, gt); break;
  case FAM_HOMOG: k_grad_template<FAM_HOMOG><<<grid, 128, 0, st>>>(a, gt); break;
  default: k_grad_template<FAM_QUAD><<<grid, 128, 0, st>>>(a, gt); break;
  }
  return cudaGetLastError();
}

}  // namespace sst

using namespace sst;

namespace {

/* scratch of the adjoint calls (per device, grown on demand; calls on one
 * device are serialised by the caller's stream order) */
struct AdjointScratch {
  DevBuf coeffs, jcs, partials;
};
AdjointScratch g_adj;

int afail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

}  // namespace

#define SST_ACK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return afail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

/* device buffers; grad outputs may be NULL (forward: only loss) */
extern "C" int sst_warp_residual(const float * frames, int n, int width, int height, size_t frame_stride,
    const float * tmpl, const sst_motion_model * model, const float * params, const float * flow,
    const double * grad_loss, double * loss, float * grad_params, float * grad_template, float * grad_flow,
    double * hessian, void * stream)
{
  if( !frames || !tmpl || !model || !params ) return afail(SST_ERR_INVALID_ARG, "sst_warp_residual: NULL argument");
  if( n < 1 || n > 65535 || width < 2 || height < 2 || frame_stride < (size_t) width * height )
    return afail(SST_ERR_INVALID_ARG, "sst_warp_residual: invalid sizes");
  if( model->type < 0 || model->type > 7 ) return afail(SST_ERR_INVALID_ARG, "invalid motion type");
  cudaStream_t st = (cudaStream_t) stream;
  const int M = model_nparams(*model);
  int tiles_x = 0;
  const int tiles = tiles_of(width, height, AJ_TX, AJ_TY, &tiles_x);
  const int NS = M * (M + 1) / 2 + M + 1;
  SST_ACK(g_adj.coeffs.ensure((size_t) n * SST_NCOEF * sizeof(float)));
  SST_ACK(g_adj.jcs.ensure((size_t) n * 8 * sizeof(float)));
  SST_ACK(g_adj.partials.ensure((size_t) n * tiles * NS * sizeof(double)));
  int launches = 0;
  k_adjoint_coeffs<<<(n + 127) / 128, 128, 0, st>>>(*model, params, n, g_adj.coeffs.as<float>(), g_adj.jcs.as<float>());
  SST_ACK(cudaGetLastError());
  ++launches;
  ResidArgs a;
  memset(&a, 0, sizeof(a));
  a.frames = frames, a.frame_stride = frame_stride, a.tmpl = tmpl, a.flow = (const float2 *) flow;
  a.coeffs = g_adj.coeffs.as<float>(), a.jcs = g_adj.jcs.as<float>();
  a.w = width, a.h = height, a.n = n, a.tiles_x = tiles_x, a.tiles = tiles;
  a.partials = g_adj.partials.as<double>();
  a.grad_flow = (float2 *) grad_flow;
  a.grad_loss = grad_loss;
  if( hessian ) SST_ACK(cudaMemsetAsync(hessian, 0, (size_t) n * 144 * sizeof(double), st));
  if( grad_params ) SST_ACK(cudaMemsetAsync(grad_params, 0, (size_t) n * 12 * sizeof(float), st));
  SST_ACK(launch_tiles_m(model->type, M, a, st));
  ++launches;
  k_residual_combine<<<(n + 7) / 8, 256, 0, st>>>(a.partials, n, tiles, M, grad_loss, loss, grad_params, hessian);
  SST_ACK(cudaGetLastError());
  ++launches;
  if( grad_template ) {
    SST_ACK(launch_grad_t(model->type, a, grad_template, st));
    ++launches;
  }
  sst_internal_count_launches(launches);
  return SST_OK;
}
