/*
 * sst_capi.cu -- the C ABI of libsst_gb300.so: engine objects, memory layout,
 * scheduling of the batched registration (CUDA graphs) and the streamed
 * register + stack pipeline.
 *
 * Memory layout in HBM (one engine):
 *   reference : f32 pyramid (levels back to back), float2 gradient pyramid,
 *               optional u8 mask pyramid and its 5x5 erosion, per-model IC
 *               Gauss-Newton matrices (levels x 12 x 12 doubles)
 *   batch     : per frame slot an f32 pyramid (sum of level areas), a
 *               FrameState, tile partials (tiles x sums doubles) and a tile
 *               ticket; one active-frame list per Gauss-Newton step
 *   staging   : two chunks of input frames for the streamed pipeline
 * The reference pyramid (~17 MB at 1280x960) stays L2-resident while the
 * batch streams through.
 */
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <math.h>
#include <string>
#include <vector>
#include <map>
#include <atomic>
#include <algorithm>

#include "sst_engine.cuh"
#include "sst_stack.cuh"
#include "sst_host.h"

using namespace sst;

/* ------------------------------------------------------------ errors */

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches(0);

static int set_error(int code, const char * fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define SST_CK(call)                                                                  \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if( e_ != cudaSuccess ) {                                                         \
      return set_error(SST_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
          __FILE__, __LINE__);                                                        \
    }                                                                                 \
  } while ( 0 )

#define SST_CK_LAUNCH(call)                                                           \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if( e_ != cudaSuccess ) {                                                         \
      return set_error(SST_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
          __FILE__, __LINE__);                                                        \
    }                                                                                 \
    g_launches.fetch_add(1);                                                          \
  } while ( 0 )

#define SST_TRY(expr)                                                                 \
  do {                                                                                \
    int r_ = (expr);                                                                  \
    if( r_ != SST_OK ) return r_;                                                     \
  } while ( 0 )

/* error reporting for entry points defined in other translation units */
int sst_internal_error(int code, const char * msg)
{
  return set_error(code, "%s", msg);
}

/* kernel launches made by entry points defined in other translation units */
void sst_internal_count_launches(int n)
{
  g_launches.fetch_add(n);
}

extern "C" const char * sst_last_error(void)
{
  return g_last_error.c_str();
}

extern "C" const char * sst_version(void)
{
  return "serstacker_gb300 0.1 (sm_103a)";
}

extern "C" int sst_device_count(void)
{
  int n = 0;
  if( cudaGetDeviceCount(&n) != cudaSuccess ) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

extern "C" long long sst_kernel_launch_count(int reset)
{
  // host launches plus the iterations of the graph level loops (counted on the device)
  const long long loops = sst::loop_launches(reset != 0);
  return (reset ? g_launches.exchange(0) : g_launches.load()) + loops;
}

extern "C" void sst_ecch_options_default(sst_ecch_options * o)
{
  if( !o ) return;
  memset(o, 0, sizeof(*o));
  o->epsx = 1e-5;
  o->reference_smooth_sigma = 1;
  o->input_smooth_sigma = 1;
  o->update_step_scale = 1;
  o->method = SST_ECC_INVERSE_COMPOSITIONAL_LM;
  o->interpolation = 1;
  o->max_iterations = 50;
  o->minimum_image_size = 8;
  o->maxlevel = 0;
  o->min_rho = 0;
  o->ic_jacobian_at_identity = 1;
}

/* ------------------------------------------------------- device buffers */

namespace {

struct GraphEntry {
  std::vector<long long> key;
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
};

}  // namespace

/* ============================================================ sst_ecch */

struct sst_ecch {
  sst_ecch_options o;
  cudaStream_t st = nullptr, st_copy = nullptr;
  cudaStream_t st_body = nullptr;   // captures the bodies of the level loops
  cudaEvent_t ev_user = nullptr, ev_done = nullptr, ev_copy[2] = { nullptr, nullptr }, ev_free[2] = { nullptr, nullptr };
  int num_sms = 0;

  // reference
  int w = 0, h = 0, L = 0;
  int lw[32], lh[32];
  size_t loff[32];
  size_t pyr_px = 0;
  DevBuf ref, grad, refTG, mask, mask_e, refsrc, jc_id, hpart, gk_in, gk_ref;
  bool has_mask = false;
  double RMA[32];
  float tshift[32];
  int ks_in = 0;
  std::map<int, DevBuf> H;           // per model: levels x 144 matrices, then levels x 144 inverses
  std::map<int, std::vector<int>> Hinv_ok;

  // batch
  int cap = 0;
  int chunk = 512;
  DevBuf stage[2];
  DevBuf pyr, fs, part, cnt, lists, counts, lap, init;
  DevBuf out_params, out_status, out_iters, out_eps, out_rho, out_weight, weff, coeffs;
  DevBuf res_params, res_status, res_rho, res_weight;   // whole-sequence results of sst_stack_frames
  DevBuf binned;                     // 2x2-binned luminance of a chunk of raw Bayer frames
  DevBuf err;                        // device flag: a bounded wait for a staged tile gave up
  DevBuf loopst;                     // per pass and level: loop cursor and the two list counts
  int loops_ok = 1;                  // graph WHILE loops usable (cleared when building one fails)
  bool loops_enabled = true;         // sst_ecch_set_level_loops
  size_t part_stride = 0;
  int steps_cap = 0;
  int lap_t = 0;
  std::vector<GraphEntry> graphs;
  cudaEvent_t prof[3][32][2];
  bool prof_ready = false;
  int last_steps[3][32];
  int last_method = 0;
  int last_n = 0;                 // frames whose pyramids the batch buffer holds
  double gate[3] = { 0, 0, 0 };   // correlation gate after pass k < last (0: none)
  sst_tuning tune {};             // launch shapes (zero fields: the defaults)

  ~sst_ecch()
  {
    if( prof_ready ) for( auto & a : prof ) for( auto & b : a ) for( auto & e : b ) cudaEventDestroy(e);
    for( auto & g : graphs ) if( g.exec ) cudaGraphExecDestroy(g.exec);
    graphs.clear();
    DevBuf * bufs[] = { &ref, &grad, &refTG, &mask, &mask_e, &refsrc, &jc_id, &hpart, &gk_in, &gk_ref, &stage[0], &stage[1],
        &pyr, &fs, &part, &cnt, &lists, &counts, &lap, &init, &out_params, &out_status, &out_iters, &out_eps,
        &out_rho, &out_weight, &weff, &coeffs, &res_params, &res_status, &res_rho, &res_weight, &binned, &err, &loopst };
    for( DevBuf * b : bufs ) b->release();
    for( auto & kv : H ) kv.second.release();
    if( ev_user ) cudaEventDestroy(ev_user);
    if( ev_done ) cudaEventDestroy(ev_done);
    for( int i = 0; i < 2; ++i ) {
      if( ev_copy[i] ) cudaEventDestroy(ev_copy[i]);
      if( ev_free[i] ) cudaEventDestroy(ev_free[i]);
    }
    if( st ) cudaStreamDestroy(st);
    if( st_copy ) cudaStreamDestroy(st_copy);
    if( st_body ) cudaStreamDestroy(st_body);
  }

  void drop_graphs()
  {
    for( auto & g : graphs ) if( g.exec ) cudaGraphExecDestroy(g.exec);
    graphs.clear();
  }
};

static int ensure_streams(sst_ecch * h)
{
  if( h->st ) return SST_OK;
  SST_CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  SST_CK(cudaStreamCreateWithFlags(&h->st_copy, cudaStreamNonBlocking));
  SST_CK(cudaStreamCreateWithFlags(&h->st_body, cudaStreamNonBlocking));
  SST_CK(cudaEventCreateWithFlags(&h->ev_user, cudaEventDisableTiming));
  SST_CK(cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming));
  for( int i = 0; i < 2; ++i ) {
    SST_CK(cudaEventCreateWithFlags(&h->ev_copy[i], cudaEventDisableTiming));
    SST_CK(cudaEventCreateWithFlags(&h->ev_free[i], cudaEventDisableTiming));
  }
  for( auto & a : h->prof ) for( auto & b : a ) for( auto & e : b ) SST_CK(cudaEventCreate(&e));
  h->prof_ready = true;
  int dev = 0;
  SST_CK(cudaGetDevice(&dev));
  SST_CK(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev));
  return SST_OK;
}

/* the internal stream starts after the work the caller queued on its stream */
static int join_user(sst_ecch * h, void * stream)
{
  SST_CK(cudaEventRecord(h->ev_user, (cudaStream_t) stream));
  SST_CK(cudaStreamWaitEvent(h->st, h->ev_user, 0));
  return SST_OK;
}

static int release_to_user(sst_ecch * h, void * stream)
{
  SST_CK(cudaEventRecord(h->ev_done, h->st));
  SST_CK(cudaStreamWaitEvent((cudaStream_t) stream, h->ev_done, 0));
  return SST_OK;
}

extern "C" int sst_ecch_create(sst_ecch ** out, const sst_ecch_options * opts)
{
  if( !out ) return set_error(SST_ERR_INVALID_ARG, "sst_ecch_create: out is NULL");
  sst_ecch_options o;
  if( opts ) o = *opts;
  else sst_ecch_options_default(&o);
  if( o.interpolation != 1 ) return set_error(SST_ERR_UNSUPPORTED, "only ECC_INTER_LINEAR interpolation is implemented");
  if( o.method < 0 || o.method > 3 ) return set_error(SST_ERR_INVALID_ARG, "invalid ECC method %d", o.method);
  if( o.max_iterations < 0 || o.max_iterations > 1000 ) return set_error(SST_ERR_INVALID_ARG, "max_iterations out of range");
  if( o.input_smooth_sigma > 5 || o.reference_smooth_sigma > 5 )
    return set_error(SST_ERR_UNSUPPORTED, "smoothing sigma > 5 is not supported");
  if( !o.ic_jacobian_at_identity )
    return set_error(SST_ERR_UNSUPPORTED, "only identity-warp IC steepest-descent images are implemented");
  sst_ecch * h = new (std::nothrow) sst_ecch();
  if( !h ) return set_error(SST_ERR_NOMEM, "out of host memory");
  h->o = o;
  *out = h;
  return SST_OK;
}

extern "C" int sst_ecch_destroy(sst_ecch * h)
{
  delete h;
  return SST_OK;
}

extern "C" int sst_ecch_num_levels(const sst_ecch * h)
{
  return h ? h->L : 0;
}

extern "C" int sst_set_chunk_frames(sst_ecch * h, int frames)
{
  if( !h || frames < 1 ) return set_error(SST_ERR_INVALID_ARG, "invalid chunk size");
  h->chunk = frames;
  return SST_OK;
}

/* correlation gates after passes 0 .. num - 1 of the following registrations
 * (0: none); used by the frame-registration glue (sst_registration.cu) */
int sst_internal_ecch_set_pass_gates(sst_ecch * h, int num, const double * gates)
{
  if( !h || num < 0 || num > 3 ) return set_error(SST_ERR_INVALID_ARG, "invalid pass gates");
  for( int k = 0; k < 3; ++k ) h->gate[k] = k < num && gates ? gates[k] : 0.0;
  return SST_OK;
}

static int check_tuning(const sst_tuning * t)
{
  if( !t ) return set_error(SST_ERR_INVALID_ARG, "NULL tuning");
  if( t->pass_ctas_per_sm < 0 || t->pass_ctas_per_sm > 16 || t->corr_ctas_per_sm < 0 || t->corr_ctas_per_sm > 16 )
    return set_error(SST_ERR_INVALID_ARG, "CTAs per SM out of range 0..16");
  for( int c = 0; c < 4; ++c ) {
    if( t->pass_tile_w[c] != 0 && t->pass_tile_w[c] != 64 && t->pass_tile_w[c] != PW_TX )
      return set_error(SST_ERR_INVALID_ARG, "pass tile width must be 0, 64 or %d", PW_TX);
  }
  if( t->stack_max_chunks < 0 || t->stack_max_chunks > 16 || t->stack_items_per_slot < 0 || t->stack_items_per_slot > 64 )
    return set_error(SST_ERR_INVALID_ARG, "stack chunk settings out of range");
  return SST_OK;
}

extern "C" int sst_ecch_set_tuning(sst_ecch * h, const sst_tuning * t)
{
  if( !h ) return set_error(SST_ERR_INVALID_ARG, "NULL engine");
  SST_TRY(check_tuning(t));
  h->tune = *t;
  h->drop_graphs();
  return SST_OK;
}

extern "C" int sst_ecch_get_tuning(const sst_ecch * h, sst_tuning * t)
{
  if( !h || !t ) return set_error(SST_ERR_INVALID_ARG, "NULL argument");
  *t = h->tune;
  return SST_OK;
}

extern "C" int sst_ecch_set_level_loops(sst_ecch * h, int enable)
{
  if( !h ) return set_error(SST_ERR_INVALID_ARG, "NULL engine");
  h->loops_enabled = enable != 0;
  return SST_OK;
}

/* the device word that TMA-staged kernels set when a bounded wait gives up */
static int ensure_err(sst_ecch * h)
{
  if( !h->err.p ) {
    SST_CK(h->err.ensure(sizeof(int)));
    SST_CK(cudaMemsetAsync(h->err.p, 0, sizeof(int), h->st));
  }
  return SST_OK;
}

/* reports (and clears) a staged-tile wait that gave up during the last work */
static int check_wait_flag(sst_ecch * h)
{
  if( !h->err.p ) return SST_OK;
  int e = 0;
  SST_CK(cudaMemcpyAsync(&e, h->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  SST_CK(cudaStreamSynchronize(h->st));
  if( !e ) return SST_OK;
  SST_CK(cudaMemsetAsync(h->err.p, 0, sizeof(int), h->st));
  return set_error(SST_ERR_TIMEOUT, "a bounded wait for a staged tile copy gave up; results are invalid");
}

/* Pyramid of n frames (levels at loff[], frame stride dst_stride floats):
 * convert + pre-smooth, then pyrDown per level. Levels 0 and 1 come from one
 * fused pass when it applies (7-tap Gaussian, TMA-compatible layout). */
static int build_pyramid(sst_ecch * h, const void * src, int depth, int n, size_t row_stride, size_t frame_stride,
    double scale, const float * gk, int ks, float * pyr, size_t dst_stride, cudaStream_t st)
{
  int l0 = 1;
  bool fused = false;
  if( h->L > 1 ) {
    SST_CK_LAUNCH(launch_convert_pyr1(src, depth, n, h->lw[0], h->lh[0], row_stride, frame_stride, scale, gk, ks, pyr,
        pyr + h->loff[1], h->lw[1], h->lh[1], dst_stride, h->err.as<int>(), st, &fused));
  }
  if( fused ) l0 = 2;
  else {
    SST_CK_LAUNCH(launch_convert_smooth(src, depth, n, h->lw[0], h->lh[0], row_stride, frame_stride, scale, gk, ks, pyr,
        dst_stride, st));
  }
  for( int l = l0; l < h->L; ++l ) {
    SST_CK_LAUNCH(launch_pyrdown(pyr + h->loff[l - 1], h->lw[l - 1], h->lh[l - 1], dst_stride, pyr + h->loff[l], h->lw[l],
        h->lh[l], dst_stride, n, st));
  }
  return SST_OK;
}

static int upload_image(DevBuf & dst, const void * src, size_t row_stride, int rows, int on_device, const void ** dptr,
    cudaStream_t st)
{
  if( on_device ) {
    *dptr = src;
    return SST_OK;
  }
  SST_CK(dst.ensure(row_stride * rows));
  SST_CK(cudaMemcpyAsync(dst.p, src, row_stride * rows, cudaMemcpyHostToDevice, st));
  *dptr = dst.p;
  return SST_OK;
}

extern "C" int sst_ecch_set_reference_image(sst_ecch * h, const void * image, int depth, int width, int height,
    size_t row_stride, double scale, const uint8_t * mask, size_t mask_stride, int on_device, void * stream)
{
  if( !h || !image ) return set_error(SST_ERR_INVALID_ARG, "sst_ecch_set_reference_image: NULL argument");
  if( depth_bytes(depth) == 0 ) return set_error(SST_ERR_INVALID_ARG, "unsupported depth %d", depth);
  if( width < 4 || height < 4 ) return set_error(SST_ERR_INVALID_ARG, "image too small: %dx%d", width, height);
  if( row_stride < (size_t) width * depth_bytes(depth) ) return set_error(SST_ERR_INVALID_ARG, "row_stride too small");
  if( mask && mask_stride < (size_t) width ) return set_error(SST_ERR_INVALID_ARG, "mask_stride too small");
  SST_TRY(ensure_streams(h));
  SST_TRY(join_user(h, stream));
  cudaStream_t st = h->st;
  h->drop_graphs();
  for( auto & kv : h->H ) kv.second.release();
  h->H.clear();
  h->Hinv_ok.clear();

  const int L = ecch_num_levels(width, height, h->o);
  h->w = width, h->h = height, h->L = L;
  size_t off = 0;
  for( int l = 0; l < L; ++l ) {
    if( l == 0 ) h->lw[0] = width, h->lh[0] = height;
    else h->lw[l] = ((h->lw[l - 1] + 1) >> 1) & ~1, h->lh[l] = ((h->lh[l - 1] + 1) >> 1) & ~1;
    h->loff[l] = off;
    off += (size_t) h->lw[l] * h->lh[l];
  }
  h->pyr_px = off;
  SST_CK(h->ref.ensure(off * sizeof(float)));
  SST_CK(h->grad.ensure(off * sizeof(float2)));

  // Gaussian kernels of the reference and the input pre-smooth
  float gk[64];
  int ks_ref = 0;
  if( h->o.reference_smooth_sigma > 0 ) {
    ks_ref = gaussian_kernel(h->o.reference_smooth_sigma, gk);
    SST_CK(h->gk_ref.ensure(64 * sizeof(float)));
    SST_CK(cudaMemcpyAsync(h->gk_ref.p, gk, ks_ref * sizeof(float), cudaMemcpyHostToDevice, st));
    SST_CK(cudaStreamSynchronize(st));
  }
  if( h->o.input_smooth_sigma > 0 ) {
    h->ks_in = gaussian_kernel(h->o.input_smooth_sigma, gk);
    SST_CK(h->gk_in.ensure(64 * sizeof(float)));
    SST_CK(cudaMemcpyAsync(h->gk_in.p, gk, h->ks_in * sizeof(float), cudaMemcpyHostToDevice, st));
    SST_CK(cudaStreamSynchronize(st));
  }
  else h->ks_in = 0;

  const void * src = nullptr;
  SST_TRY(upload_image(h->refsrc, image, row_stride, height, on_device, &src, st));
  float * ref = h->ref.as<float>();
  SST_TRY(ensure_err(h));
  SST_TRY(build_pyramid(h, src, depth, 1, row_stride, row_stride * height, scale,
      ks_ref ? h->gk_ref.as<float>() : nullptr, ks_ref, ref, 0, st));

  // masks: level 0 copy, nearest resize per level (c_ecch::downscale_image), 5x5 erosion
  h->has_mask = mask != nullptr;
  if( mask ) {
    SST_CK(h->mask.ensure(off));
    SST_CK(h->mask_e.ensure(off));
    uint8_t * m = h->mask.as<uint8_t>();
    SST_CK(cudaMemcpy2DAsync(m, width, mask, mask_stride, width, height,
        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    for( int l = 1; l < L; ++l ) {
      SST_CK_LAUNCH(launch_resize_nearest_u8(m + h->loff[l - 1], h->lw[l - 1], h->lh[l - 1], m + h->loff[l], h->lw[l],
          h->lh[l], st));
    }
    for( int l = 0; l < L; ++l ) {
      SST_CK_LAUNCH(launch_erode5(m + h->loff[l], h->lw[l], h->lh[l], h->mask_e.as<uint8_t>() + h->loff[l], st));
    }
  }
  for( int l = 0; l < L; ++l ) {
    SST_CK_LAUNCH(launch_ref_gradients(ref + h->loff[l], mask ? h->mask.as<uint8_t>() + h->loff[l] : nullptr,
        h->lw[l], h->lh[l], h->grad.as<float2>() + h->loff[l], st));
  }
  SST_CK(h->refTG.ensure(off * sizeof(float4)));
  SST_CK_LAUNCH(launch_pack_reference(ref, h->grad.as<float2>(), off, h->refTG.as<float4>(), st));
  // per-level statistics: mean (numerical shift) and RMA (valid reference pixels)
  int tx;
  const int tmax = tiles_of(width, height, PW_TX, PW_TY, &tx);
  SST_CK(h->hpart.ensure((size_t) tmax * 78 * sizeof(double)));
  std::vector<double> hp((size_t) tmax * 3);
  for( int l = 0; l < L; ++l ) {
    int tiles = 0;
    SST_CK_LAUNCH(launch_ref_stats(ref + h->loff[l], mask ? h->mask.as<uint8_t>() + h->loff[l] : nullptr, h->lw[l],
        h->lh[l], h->hpart.as<double>(), &tiles, st));
    SST_CK(cudaMemcpyAsync(hp.data(), h->hpart.p, (size_t) tiles * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SST_CK(cudaStreamSynchronize(st));
    double s = 0, n = 0, m = 0;
    for( int t = 0; t < tiles; ++t ) s += hp[t * 3], n += hp[t * 3 + 1], m += hp[t * 3 + 2];
    h->tshift[l] = (float) (n > 0 ? s / n : 0);
    h->RMA[l] = m;
  }
  SST_CK(cudaStreamSynchronize(st));
  SST_TRY(check_wait_flag(h));
  SST_TRY(release_to_user(h, stream));
  return SST_OK;
}

static bool model_cholesky_solve_host(const double * A, const double * b, int n, double * x)
{
  return cholesky_solve(A, b, n, x);
}

/* IC Gauss-Newton matrix per level for one model (identity warp) */
static int ensure_H(sst_ecch * h, const sst_motion_model & m, const double ** out)
{
  const int M = model_nparams(m);
  const int key = m.type * 16 + M;
  auto it = h->H.find(key);
  if( it != h->H.end() ) {
    *out = it->second.as<double>();
    return SST_OK;
  }
  DevBuf & buf = h->H[key];
  SST_CK(buf.ensure((size_t) h->L * 2 * 144 * sizeof(double)));
  double s[16];
  float jc[8];
  model_identity(m, s);
  model_sd_coeffs(m, s, jc);
  SST_CK(h->jc_id.ensure(8 * sizeof(float)));
  SST_CK(cudaMemcpy(h->jc_id.p, jc, sizeof(jc), cudaMemcpyHostToDevice));
  const int NS = M * (M + 1) / 2;
  std::vector<double> hp, Hm((size_t) h->L * 2 * 144, 0.0);
  std::vector<int> & okv = h->Hinv_ok[key];
  okv.assign(h->L, 0);
  for( int l = 0; l < h->L; ++l ) {
    int tiles = 0;
    SST_CK_LAUNCH(launch_ref_hessian(h->grad.as<float2>() + h->loff[l], h->lw[l], h->lh[l], jac_kind(m.type), M,
        h->jc_id.as<float>(), h->hpart.as<double>(), &tiles, h->st));
    hp.resize((size_t) tiles * NS);
    SST_CK(cudaMemcpyAsync(hp.data(), h->hpart.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    SST_CK(cudaStreamSynchronize(h->st));
    double * Hl = Hm.data() + (size_t) l * 144;
    for( int t = 0; t < tiles; ++t ) {
      for( int u = 0, k = 0; u < M; ++u )
        for( int v = 0; v <= u; ++v, ++k ) Hl[u * M + v] += hp[(size_t) t * NS + k];
    }
    for( int u = 0; u < M; ++u ) for( int v = u + 1; v < M; ++v ) Hl[u * M + v] = Hl[v * M + u];
    // inverse by FP64 Cholesky solves of the unit vectors (the matrix is constant per level)
    double * Hi = Hm.data() + (size_t) (h->L + l) * 144;
    bool ok = true;
    for( int j = 0; j < M && ok; ++j ) {
      double e[12] = { 0 }, col[12];
      e[j] = 1;
      ok = model_cholesky_solve_host(Hl, e, M, col);
      for( int i = 0; i < M; ++i ) Hi[i * M + j] = col[i];
    }
    okv[l] = ok ? 1 : 0;
  }
  SST_CK(cudaMemcpy(buf.p, Hm.data(), Hm.size() * sizeof(double), cudaMemcpyHostToDevice));
  *out = buf.as<double>();
  return SST_OK;
}

/* timing event: a graph event node while capturing, a plain record otherwise */
static cudaError_t record_prof(cudaEvent_t e, cudaStream_t st, bool host_driven)
{
  return host_driven ? cudaEventRecord(e, st) : cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
}

/* the level-width class of the tuning tables: <= 192, <= 384, <= 768, wider */
static int width_class(int w)
{
  return w <= 192 ? 0 : w <= 384 ? 1 : w <= 768 ? 2 : 3;
}

/* tile width of the staged IC / IC-LM pass at a level: the tuned width of the
 * level's width class, else 64 on levels at most 384 px wide (fewer idle
 * columns in the last tile) and PW_TX on wider ones */
static int pointwise_tile_w(const sst_ecch * h, int l)
{
  const int t = h->tune.pass_tile_w[width_class(h->lw[l])];
  if( t == 64 || t == PW_TX ) return t;
  return h->lw[l] <= 384 ? 64 : PW_TX;
}

/* grid of the Gauss-Newton pass launches: tuned CTAs per SM, else the
 * kernel's occupancy (-1) */
static int pass_grid(const sst_ecch * h)
{
  return h->tune.pass_ctas_per_sm > 0 ? std::max(1, h->num_sms) * h->tune.pass_ctas_per_sm : -1;
}

/* tiles of a level's pass; for IC / IC-LM the staged pass's tiling, which has at
 * least as many tiles as the PW_TX-wide one of the unstaged pass */
static int level_tiles(const sst_ecch * h, int l, int method, int * tiles_x)
{
  if( method == M_FA || method == M_LM ) return tiles_of(h->lw[l], h->lh[l], ST_TX, ST_TY, tiles_x);
  return tiles_of(h->lw[l], h->lh[l], pointwise_tile_w(h, l), PW_TY, tiles_x);
}

static int ensure_capacity(sst_ecch * h, int n, int method, int num_passes, const sst_motion_model * passes)
{
  size_t pstride = 0;
  for( int k = 0; k < num_passes; ++k ) {
    const int NS = pass_num_sums(method, model_nparams(passes[k]));
    for( int l = 0; l < h->L; ++l ) {
      int tx;
      pstride = std::max(pstride, (size_t) level_tiles(h, l, method, &tx) * NS);
    }
  }
  int tx;
  pstride = std::max(pstride, (size_t) tiles_of(h->w, h->h, PW_TX, PW_TY, &tx) * 6);
  const int steps = 1 + num_passes * h->L * (h->o.max_iterations + 2);
  const int lap_level = h->L > 1 ? 1 : 0;
  const int lt = lap_tiles(h->lw[lap_level], h->lh[lap_level]);
  const bool grow = n > h->cap || pstride > h->part_stride || steps > h->steps_cap || lt != h->lap_t ||
      (size_t) std::max(n, h->cap) * h->pyr_px * sizeof(float) > h->pyr.n;   // a larger reference needs larger pyramids
  if( !grow ) return SST_OK;
  h->drop_graphs();
  const int cap = std::max(n, h->cap);
  h->part_stride = std::max(pstride, h->part_stride);
  h->steps_cap = std::max(steps, h->steps_cap);
  h->lap_t = lt;
  SST_CK(h->pyr.ensure((size_t) cap * h->pyr_px * sizeof(float)));
  SST_CK(h->fs.ensure((size_t) cap * sizeof(FrameState)));
  SST_CK(h->part.ensure((size_t) cap * h->part_stride * sizeof(double)));
  SST_CK(h->cnt.ensure((size_t) cap * sizeof(unsigned)));
  SST_CK(cudaMemsetAsync(h->cnt.p, 0, (size_t) cap * sizeof(unsigned), h->st));
  SST_CK(h->lists.ensure((size_t) h->steps_cap * cap * sizeof(int)));
  SST_CK(h->counts.ensure((size_t) h->steps_cap * sizeof(int)));
  SST_CK(h->lap.ensure((size_t) cap * lt * 2 * sizeof(double)));
  SST_CK(h->init.ensure((size_t) cap * 16 * sizeof(double)));
  SST_CK(h->out_params.ensure((size_t) cap * 12 * sizeof(float)));
  SST_CK(h->out_status.ensure((size_t) cap * sizeof(int32_t)));
  SST_CK(h->out_iters.ensure((size_t) cap * sizeof(int32_t)));
  SST_CK(h->out_eps.ensure((size_t) cap * sizeof(float)));
  SST_CK(h->out_rho.ensure((size_t) cap * sizeof(float)));
  SST_CK(h->out_weight.ensure((size_t) cap * sizeof(float)));
  SST_CK(h->weff.ensure((size_t) cap * sizeof(float)));
  SST_CK(h->coeffs.ensure((size_t) cap * SST_NCOEF * sizeof(float)));
  SST_TRY(ensure_err(h));
  h->cap = cap;
  return SST_OK;
}

/* Adds a WHILE node after the work captured so far on st (a capture must be
 * active) and captures its body on the engine's body stream: body(stream,
 * handle) enqueues one iteration; the loop runs while the handle, 1 at each
 * graph launch, stays non-zero. The capture on st continues after the node. */
template<typename Body>
static int add_level_loop(sst_ecch * h, cudaStream_t st, Body body)
{
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t * deps = nullptr;
  size_t nd = 0;
  SST_CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
  if( cs != cudaStreamCaptureStatusActive ) return set_error(SST_ERR_STATE, "level loop outside a graph capture");
  cudaGraphConditionalHandle hc;
  SST_CK(cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams p = { cudaGraphNodeTypeConditional };   // the rest zero-initialised
  p.conditional.handle = hc;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  SST_CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
  SST_CK(cudaStreamBeginCaptureToGraph(h->st_body, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
      cudaStreamCaptureModeThreadLocal));
  const int r = body(h->st_body, hc);
  cudaGraph_t out = nullptr;
  const cudaError_t e = cudaStreamEndCapture(h->st_body, &out);
  if( r != SST_OK ) return r;
  SST_CK(e);
  SST_CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return SST_OK;
}

/* compute_correlation of every frame still registering against the level-0
 * reference under the model's current state, and the gate rho >= min_rho
 * (min_rho <= 0: rho only) */
static int enqueue_correlation(sst_ecch * h, int n, const sst_motion_model & model, double min_rho, cudaStream_t st)
{
  const int grid = std::max(1, h->num_sms) * (h->tune.corr_ctas_per_sm > 0 ? h->tune.corr_ctas_per_sm : 4);
  CorrArgs c;
  memset(&c, 0, sizeof(c));
  c.pyr = h->pyr.as<float>();
  c.pyr_stride = h->pyr_px;
  c.w = h->w, c.h = h->h;
  c.tiles = tiles_of(h->w, h->h, PW_TX, PW_TY, &c.tiles_x);
  c.refT = h->ref.as<float>();
  c.refM = h->has_mask ? h->mask.as<uint8_t>() : nullptr;
  c.tshift = h->tshift[0];
  c.fs = h->fs.as<FrameState>();
  c.n = n;
  c.partials = h->part.as<double>();
  c.part_stride = h->part_stride;
  c.counters = h->cnt.as<unsigned>();
  c.model = model;
  c.min_rho = min_rho;
  c.err = h->err.as<int>();
  CUtensorMap cmap;
  const bool cstaged = encode_pass_level(h->pyr.as<float>(), h->w, h->h, h->pyr_px, h->cap, &cmap);
  SST_CK_LAUNCH(launch_correlation(c, grid, st, cstaged ? &cmap : nullptr));
  return SST_OK;
}

/* The Gauss-Newton schedule of one batch: pass begin, per level a level
 * begin and max_iterations + 1 pass launches, then the correlation. In
 * host-driven mode every step is followed by a synchronisation and an early
 * exit when no frame is left (the plain one-frame-per-launch form). */
static int enqueue_schedule(sst_ecch * h, int n, int method, int num_passes, const sst_motion_model * passes,
    bool have_init, bool host_driven, long long * kernels, bool loops = false)
{
  cudaStream_t st = h->st;
  const int L = h->L;
  const int max_it = h->o.max_iterations;
  const int pgrid = pass_grid(h);
  const int solve_grid = std::max(1, std::min((n + 7) / 8, std::max(1, h->num_sms) * 8));
  long long k = 0;
  SST_CK(cudaMemsetAsync(h->counts.p, 0, (size_t) h->steps_cap * sizeof(int), st));
  int step = 0;
  int * lists = h->lists.as<int>();
  int * counts = h->counts.as<int>();
  FrameState * fs = h->fs.as<FrameState>();
  for( int k_pass = 0; k_pass < num_passes; ++k_pass ) {
    const sst_motion_model & m = passes[k_pass];
    PassBeginArgs pb;
    memset(&pb, 0, sizeof(pb));
    pb.fs = fs, pb.n = n, pb.pass = k_pass, pb.model = m, pb.prev_model = k_pass ? passes[k_pass - 1] : m;
    pb.init_states = (k_pass == 0 && have_init) ? h->init.as<double>() : nullptr;
    pb.scale_to_coarsest = L > 1 ? (double) h->lw[L - 1] / (double) h->lw[0] : 0.0;
    SST_CK_LAUNCH(launch_pass_begin(pb, st));
    ++k;
    const double * H = nullptr;
    if( method == M_IC || method == M_ICLM ) SST_TRY(ensure_H(h, m, &H));
    for( int l = L - 1; l >= 0; --l ) {
      SST_CK(record_prof(h->prof[k_pass][l][0], st, host_driven));
      h->last_steps[k_pass][l] = step;
      // graph loops: [cursor, count A, count B] of this pass and level; list A is the
      // level's first list slot, list B the second, the step counts the history
      int * lp = loops ? h->loopst.as<int>() + 4 * (k_pass * 32 + l) : nullptr;
      if( loops ) SST_CK(cudaMemsetAsync(lp, 0, 4 * sizeof(int), st));
      LevelBeginArgs lb;
      memset(&lb, 0, sizeof(lb));
      lb.fs = fs, lb.n = n, lb.model = m, lb.method = method;
      lb.list_out = lists + (size_t) step * h->cap;
      lb.count_out = loops ? lp + 1 : counts + step;
      lb.level_is_first = l == L - 1;
      SST_CK_LAUNCH(launch_level_begin(lb, st));
      ++k;
      PassArgs a;
      memset(&a, 0, sizeof(a));
      a.pyr = h->pyr.as<float>();
      a.pyr_stride = h->pyr_px;
      a.lvl_off = h->loff[l];
      a.w = h->lw[l], a.h = h->lh[l];
      a.tiles = level_tiles(h, l, method, &a.tiles_x);
      a.refT = h->ref.as<float>() + h->loff[l];
      a.refG = h->grad.as<float2>() + h->loff[l];
      a.refTG = h->refTG.as<float4>() + h->loff[l];
      a.refM = h->has_mask ? h->mask.as<uint8_t>() + h->loff[l] : nullptr;
      a.refMe = h->has_mask ? h->mask_e.as<uint8_t>() + h->loff[l] : nullptr;
      a.H = H ? H + (size_t) l * 144 : nullptr;
      {
        const int key = m.type * 16 + model_nparams(m);
        const bool inv_ok = H && h->Hinv_ok.count(key) && h->Hinv_ok[key][l];
        a.Hinv = (method == M_IC && inv_ok) ? H + (size_t) (L + l) * 144 : nullptr;
      }
      a.RMA = h->RMA[l];
      a.tshift = h->tshift[l];
      {
        double s[16];
        model_identity(m, s);
        model_sd_coeffs(m, s, a.jc_id);
      }
      a.fs = fs;
      a.partials = h->part.as<double>();
      a.part_stride = h->part_stride;
      a.counters = h->cnt.as<unsigned>();
      a.model = m;
      a.M = model_nparams(m);
      a.max_eps = h->o.epsx * pow(2.0, l);
      a.step = h->o.update_step_scale;
      a.max_it = max_it;
      a.scale_next = l > 0 ? (double) h->lw[l - 1] / (double) h->lw[l] : 0.0;
      a.err = h->err.as<int>();
      // IC / IC-LM: the level of every frame slot as a TMA tensor (footprints staged in shared
      // memory); the unstaged pass keeps PW_TX-wide tiles
      CUtensorMap map;
      const int tw = pointwise_tile_w(h, l);
      const bool staged = (method == M_IC || method == M_ICLM) &&
          encode_pass_level(h->pyr.as<float>() + h->loff[l], h->lw[l], h->lh[l], h->pyr_px, h->cap, &map, tw);
      if( method == M_IC || method == M_ICLM ) {
        a.tile_w = staged ? tw : PW_TX;
        a.tiles = tiles_of(h->lw[l], h->lh[l], a.tile_w, PW_TY, &a.tiles_x);
      }
      if( loops ) {
        a.list_in = lists + (size_t) step * h->cap;
        a.count_in = lp + 1;
        a.list_out = lists + (size_t) (step + 1) * h->cap;
        a.count_out = lp + 2;
        LevelLoopArgs la;
        la.cursor = lp, la.list_a = lists + (size_t) step * h->cap, la.count_a = lp + 1;
        la.list_b = lists + (size_t) (step + 1) * h->cap, la.count_b = lp + 2;
        la.hist = counts + step, la.max_it = max_it;
        SST_TRY(add_level_loop(h, st, [&](cudaStream_t sb, cudaGraphConditionalHandle hc) -> int {
          la.handle = hc;
          SST_CK(launch_pass(method, a, pgrid, sb, staged ? &map : nullptr));
          SST_CK(launch_solve(method, a, solve_grid, sb));
          SST_CK(launch_level_advance(la, sb));
          return SST_OK;
        }));
      }
      for( int it = 0; !loops && it <= max_it; ++it ) {
        a.list_in = lists + (size_t) (step + it) * h->cap;
        a.count_in = counts + step + it;
        a.list_out = lists + (size_t) (step + it + 1) * h->cap;
        a.count_out = counts + step + it + 1;
        SST_CK_LAUNCH(launch_pass(method, a, pgrid, st, staged ? &map : nullptr));
        SST_CK_LAUNCH(launch_solve(method, a, solve_grid, st));
        k += 2;
        if( host_driven ) {
          int c = 0;
          SST_CK(cudaMemcpyAsync(&c, counts + step + it + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
          SST_CK(cudaStreamSynchronize(st));
          if( c == 0 ) break;
        }
      }
      SST_CK(record_prof(h->prof[k_pass][l][1], st, host_driven));
      step += max_it + 2;
    }
    // an intermediate correlation gate (register_frame's translation estimate,
    // c_frame_registration.cc:825-834): frames below it stop registering
    if( k_pass + 1 < num_passes && h->gate[k_pass] > 0 ) {
      SST_TRY(enqueue_correlation(h, n, m, h->gate[k_pass], st));
      k += 2;
    }
  }
  SST_TRY(enqueue_correlation(h, n, passes[num_passes - 1], h->o.min_rho, st));
  k += 2;
  if( kernels ) *kernels = k;
  return SST_OK;
}

/* per-level timing of the last registration call (CUDA events around each
 * level's Gauss-Newton launches) and the frame-iterations it executed */
extern "C" int sst_ecch_level_stats(sst_ecch * h, int pass, int level, float * ms, double * frame_iterations,
    double * algorithmic_bytes)
{
  if( !h || pass < 0 || pass > 2 || level < 0 || level >= h->L || !h->prof_ready )
    return set_error(SST_ERR_INVALID_ARG, "sst_ecch_level_stats: invalid arguments");
  SST_CK(cudaStreamSynchronize(h->st));
  float t = 0;
  SST_CK(cudaEventElapsedTime(&t, h->prof[pass][level][0], h->prof[pass][level][1]));
  std::vector<int> c(h->o.max_iterations + 1);
  SST_CK(cudaMemcpy(c.data(), h->counts.as<int>() + h->last_steps[pass][level], c.size() * sizeof(int),
      cudaMemcpyDeviceToHost));
  double fi = 0;
  for( int v : c ) fi += v;
  // algorithmic bytes per pixel and frame-iteration: IC / IC-LM read the warped
  // source (4 B), the template (4 B) and its gradients (8 B); FA / LM read the
  // warped source and the template and recompute gradients on chip (8 B)
  const double bpp = (h->last_method == M_IC || h->last_method == M_ICLM) ? 16.0 : 8.0;
  if( ms ) *ms = t;
  if( frame_iterations ) *frame_iterations = fi;
  if( algorithmic_bytes ) *algorithmic_bytes = fi * bpp * (double) h->lw[level] * h->lh[level];
  return SST_OK;
}

/* one pyramid level (lw x lh floats, rows packed) to host or device memory */
static int copy_level(sst_ecch * h, const float * level_base, int level, float * out, int on_device)
{
  const size_t bytes = (size_t) h->lw[level] * h->lh[level] * sizeof(float);
  SST_CK(cudaMemcpyAsync(out, level_base, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->st));
  SST_CK(cudaStreamSynchronize(h->st));
  return SST_OK;
}

extern "C" int sst_ecch_reference_image(sst_ecch * h, int level, float * out, int on_device)
{
  if( !h || !out || level < 0 || level >= h->L || !h->ref.p )
    return set_error(SST_ERR_INVALID_ARG, "sst_ecch_reference_image: invalid arguments");
  return copy_level(h, h->ref.as<float>() + h->loff[level], level, out, on_device);
}

extern "C" int sst_ecch_current_image(sst_ecch * h, int frame, int level, float * out, int on_device)
{
  if( !h || !out || level < 0 || level >= h->L || frame < 0 || frame >= h->last_n || !h->pyr.p )
    return set_error(SST_ERR_INVALID_ARG, "sst_ecch_current_image: invalid arguments");
  return copy_level(h, h->pyr.as<float>() + (size_t) frame * h->pyr_px + h->loff[level], level, out, on_device);
}

static int validate_passes(const sst_ecch * h, int num_passes, const sst_motion_model * passes)
{
  if( num_passes < 1 || num_passes > 3 || !passes ) return set_error(SST_ERR_INVALID_ARG, "1..3 motion passes are required");
  for( int k = 0; k < num_passes; ++k ) {
    const sst_motion_model & m = passes[k];
    if( m.type < 0 || m.type > 7 ) return set_error(SST_ERR_INVALID_ARG, "invalid motion type %d", m.type);
    if( is_euclid(m.type) && (m.fix_translation || m.fix_rotation) )
      return set_error(SST_ERR_UNSUPPORTED, "euclidean with fixed translation or rotation is not implemented");
    if( m.type == SST_MOTION_EUCLIDEAN && !m.fix_scale )
      return set_error(SST_ERR_INVALID_ARG, "EUCLIDEAN motion requires fix_scale = 1 (image_transform.cc:35-39)");
    if( m.type == SST_MOTION_SCALED_EUCLIDEAN && m.fix_scale )
      return set_error(SST_ERR_INVALID_ARG, "SCALED_EUCLIDEAN motion requires fix_scale = 0");
  }
  return SST_OK;
}

/* Register n device-resident frames; results stay in the engine's device
 * output arrays. */
static int register_device(sst_ecch * h, const void * d_frames, int depth, int n, size_t row_stride,
    size_t frame_stride, double scale, int num_passes, const sst_motion_model * passes,
    const double * init_states_host, bool plain)
{
  cudaStream_t st = h->st;
  const int method = h->o.method;
  h->last_method = method;
  SST_TRY(ensure_capacity(h, n, method, num_passes, passes));
  if( init_states_host ) {
    SST_CK(cudaMemcpyAsync(h->init.p, init_states_host, (size_t) n * 16 * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  // pyramid of every frame: convert + pre-smooth, pyrDown
  float * pyr = h->pyr.as<float>();
  SST_TRY(build_pyramid(h, d_frames, depth, n, row_stride, frame_stride, scale,
      h->ks_in ? h->gk_in.as<float>() : nullptr, h->ks_in, pyr, h->pyr_px, st));
  h->last_n = n;
  const int lap_level = h->L > 1 ? 1 : 0;
  SST_CK_LAUNCH(launch_lap_energy(pyr, h->pyr_px, h->loff[lap_level], h->lw[lap_level], h->lh[lap_level], n,
      h->lap.as<double>(), h->lap_t, st));

  // IC / IC-LM: the per-level matrices must exist before graph capture
  if( method == M_IC || method == M_ICLM ) {
    for( int k = 0; k < num_passes; ++k ) {
      const double * Hd;
      SST_TRY(ensure_H(h, passes[k], &Hd));
    }
  }
  if( plain ) {
    long long kk = 0;
    SST_TRY(enqueue_schedule(h, n, method, num_passes, passes, init_states_host != nullptr, true, &kk));
  }
  else {
    const bool want_loops = h->loops_ok && h->loops_enabled;
    std::vector<long long> key = { n, method, num_passes, init_states_host ? 1 : 0, h->o.max_iterations, want_loops };
    for( int k = 0; k < num_passes; ++k ) {
      key.push_back(passes[k].type);
      key.push_back(passes[k].fix_scale);
      long long g;
      memcpy(&g, &h->gate[k], sizeof(g));
      key.push_back(g);
    }
    key.push_back(h->tune.pass_ctas_per_sm);
    key.push_back(h->tune.corr_ctas_per_sm);
    for( int c = 0; c < 4; ++c ) key.push_back(h->tune.pass_tile_w[c]);
    GraphEntry * ge = nullptr;
    for( auto & g : h->graphs ) if( g.key == key ) ge = &g;
    if( !ge ) {
      // levels as graph WHILE loops (no launches for iterations no frame needs);
      // the unrolled schedule when such a graph cannot be built
      if( want_loops ) SST_CK(h->loopst.ensure((size_t) 3 * 32 * 4 * sizeof(int)));
      GraphEntry g;
      g.key = key;
      for( int attempt = want_loops ? 0 : 1; attempt < 2; ++attempt ) {
        const bool loops = attempt == 0;
        cudaGraph_t graph = nullptr;
        SST_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        long long kk = 0;
        const long long before = g_launches.load();
        const int r = enqueue_schedule(h, n, method, num_passes, passes, init_states_host != nullptr, false, &kk, loops);
        g_launches.store(before);
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        if( r == SST_OK && e == cudaSuccess ) e = cudaGraphInstantiate(&g.exec, graph, 0);
        if( graph ) cudaGraphDestroy(graph);
        if( r == SST_OK && e == cudaSuccess ) {
          g.kernels = kk;
          break;
        }
        cudaGetLastError();
        if( loops ) {
          h->loops_ok = 0;
          continue;
        }
        if( r != SST_OK ) return r;
        return set_error(SST_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
      }
      h->graphs.push_back(g);
      ge = &h->graphs.back();
    }
    SST_CK(cudaGraphLaunch(ge->exec, st));
    g_launches.fetch_add(ge->kernels);
  }
  FinalizeArgs fa;
  fa.fs = h->fs.as<FrameState>();
  fa.n = n;
  fa.model = passes[num_passes - 1];
  fa.lap_partials = h->lap.as<double>();
  fa.lap_tiles = h->lap_t;
  fa.params_out = h->out_params.as<float>();
  fa.status_out = h->out_status.as<int32_t>();
  fa.iters_out = h->out_iters.as<int32_t>();
  fa.eps_out = h->out_eps.as<float>();
  fa.rho_out = h->out_rho.as<float>();
  fa.weight_out = h->out_weight.as<float>();
  SST_CK_LAUNCH(launch_finalize(fa, st));
  return SST_OK;
}

static int copy_out(void * dst, const void * src, size_t bytes, int on_device, cudaStream_t st)
{
  if( !dst ) return SST_OK;
  SST_CK(cudaMemcpyAsync(dst, src, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
  return SST_OK;
}

static int init_states_from_params(const sst_motion_model & m, const float * params, int n, int on_device,
    std::vector<double> & states)
{
  std::vector<float> hp((size_t) n * 12);
  if( on_device ) SST_CK(cudaMemcpy(hp.data(), params, hp.size() * sizeof(float), cudaMemcpyDeviceToHost));
  else memcpy(hp.data(), params, hp.size() * sizeof(float));
  states.assign((size_t) n * 16, 0.0);
  const int M = model_nparams(m);
  for( int f = 0; f < n; ++f ) {
    double p[12];
    for( int j = 0; j < M; ++j ) p[j] = hp[(size_t) f * 12 + j];
    model_identity(m, &states[(size_t) f * 16]);
    model_set_params(m, &states[(size_t) f * 16], p);
  }
  return SST_OK;
}

static int align_common(sst_ecch * h, const void * frames, int depth, int n, int width, int height,
    size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int use_initial_params,
    float * params_inout, int32_t * status_out, int32_t * iterations_out, float * eps_out,
    float * rho_out, float * weight_out, void * stream, bool plain)
{
  if( !h || !frames ) return set_error(SST_ERR_INVALID_ARG, "align: NULL argument");
  if( h->L == 0 ) return set_error(SST_ERR_STATE, "c_ecch: no reference image was set");
  if( n < 1 || n > 65535 ) return set_error(SST_ERR_INVALID_ARG, "n = %d out of range 1..65535", n);
  if( width != h->w || height != h->h )
    return set_error(SST_ERR_INVALID_ARG, "frame size %dx%d differs from the reference %dx%d", width, height, h->w, h->h);
  if( depth_bytes(depth) == 0 ) return set_error(SST_ERR_INVALID_ARG, "unsupported depth %d", depth);
  if( row_stride < (size_t) width * depth_bytes(depth) || frame_stride < row_stride * height )
    return set_error(SST_ERR_INVALID_ARG, "invalid strides");
  if( use_initial_params && !params_inout ) return set_error(SST_ERR_INVALID_ARG, "initial parameters are NULL");
  SST_TRY(validate_passes(h, num_passes, passes));
  const int method = h->o.method;
  if( method == M_IC || method == M_ICLM ) {
    for( int k = 0; k < num_passes; ++k ) {
      if( !model_invertible(passes[k]) ) {
        // c_ecc_inverse_compositional::align refuses non-invertible transforms (ecc2.cc:1702-1705)
        return set_error(SST_ERR_UNSUPPORTED, "inverse compositional ECC requires an invertible motion model");
      }
    }
  }
  SST_TRY(ensure_streams(h));
  SST_TRY(join_user(h, stream));
  cudaStream_t st = h->st;
  std::vector<double> init;
  if( use_initial_params ) SST_TRY(init_states_from_params(passes[0], params_inout, n, on_device, init));

  const int chunk = plain ? 1 : n;
  for( int f0 = 0; f0 < n; f0 += chunk ) {
    const int nc = std::min(chunk, n - f0);
    const void * d_frames = nullptr;
    const uint8_t * fsrc = (const uint8_t *) frames + (size_t) f0 * frame_stride;
    if( on_device ) d_frames = fsrc;
    else {
      SST_CK(h->stage[0].ensure(frame_stride * nc));
      SST_CK(cudaMemcpyAsync(h->stage[0].p, fsrc, frame_stride * nc, cudaMemcpyHostToDevice, st));
      d_frames = h->stage[0].p;
    }
    SST_TRY(register_device(h, d_frames, depth, nc, row_stride, frame_stride, scale, num_passes, passes,
        use_initial_params ? init.data() + (size_t) f0 * 16 : nullptr, plain));
    SST_TRY(copy_out(params_inout ? params_inout + (size_t) f0 * 12 : nullptr, h->out_params.p, (size_t) nc * 12 * sizeof(float), on_device, st));
    SST_TRY(copy_out(status_out ? status_out + f0 : nullptr, h->out_status.p, (size_t) nc * sizeof(int32_t), on_device, st));
    SST_TRY(copy_out(iterations_out ? iterations_out + f0 : nullptr, h->out_iters.p, (size_t) nc * sizeof(int32_t), on_device, st));
    SST_TRY(copy_out(eps_out ? eps_out + f0 : nullptr, h->out_eps.p, (size_t) nc * sizeof(float), on_device, st));
    SST_TRY(copy_out(rho_out ? rho_out + f0 : nullptr, h->out_rho.p, (size_t) nc * sizeof(float), on_device, st));
    SST_TRY(copy_out(weight_out ? weight_out + f0 : nullptr, h->out_weight.p, (size_t) nc * sizeof(float), on_device, st));
    if( plain || !on_device ) SST_CK(cudaStreamSynchronize(st));
  }
  if( !on_device ) {
    SST_CK(cudaStreamSynchronize(st));
    SST_TRY(check_wait_flag(h));
  }
  SST_TRY(release_to_user(h, stream));
  return SST_OK;
}

extern "C" int sst_ecch_align_batch(sst_ecch * h, const void * frames, int depth, int n, int width, int height,
    size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int use_initial_params,
    float * params_inout, int32_t * status_out, int32_t * iterations_out, float * eps_out,
    float * rho_out, float * weight_out, void * stream)
{
  return align_common(h, frames, depth, n, width, height, row_stride, frame_stride, scale, on_device, num_passes,
      passes, use_initial_params, params_inout, status_out, iterations_out, eps_out, rho_out, weight_out, stream, false);
}

extern "C" int sst_ecch_align_plain(sst_ecch * h, const void * frames, int depth, int n, int width, int height,
    size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int use_initial_params,
    float * params_inout, int32_t * status_out, int32_t * iterations_out, float * eps_out,
    float * rho_out, float * weight_out, void * stream)
{
  return align_common(h, frames, depth, n, width, height, row_stride, frame_stride, scale, on_device, num_passes,
      passes, use_initial_params, params_inout, status_out, iterations_out, eps_out, rho_out, weight_out, stream, true);
}

/* ================================================ sst_weighted_average */

struct sst_weighted_average {
  int w = 0, h = 0;
  DevBuf acc, coeffs, weff, src, wsrc;
  DevBuf part;                         // partial sums of the frame chunks of one batch
  DevBuf err;                          // the stacking kernels' error flag (StackArgs::err)
  DevBuf focus_e, focus_w, gk_focus;   // focus weighting: energy maps, blurred maps, Gaussian taps
  DevBuf out_avg, out_mask;            // device staging of compute() results bound for host memory
  int gk_n = 0;
  sst_local_variance * lv = nullptr;   // local-variance weighting (created on first use)
  sst_local_variance_options lvo = { 2, 1, 3 };
  int frames = 0;
  int max_chunks = 4;                  // a tile's frames split over at most this many CTAs
  int items_per_slot = 4;              // (tile, chunk) CTAs aimed at per resident CTA slot
  size_t plane() const { return (size_t) w * h; }
  ~sst_weighted_average()
  {
    acc.release(), coeffs.release(), weff.release(), src.release(), wsrc.release(), part.release(), err.release();
    focus_e.release(), focus_w.release(), gk_focus.release(), out_avg.release(), out_mask.release();
    sst_local_variance_destroy(lv);
  }
};

/* focus weighting: per-pixel W = (6 lap^2 + grad^2)^2 of each warped frame,
 * blurred by a Gaussian of sigma 3 (ksize 19, BORDER_REPLICATE); returns the
 * n maps on the accumulator's grid */
static int focus_maps(sst_weighted_average * a, const void * d_frames, int depth, int n, int sw, int sh,
    size_t row_stride, size_t frame_stride, double scale, int motion, const float * coeffs, const float ** maps,
    cudaStream_t st)
{
  const size_t plane = a->plane();
  SST_CK(a->focus_e.ensure((size_t) n * plane * sizeof(float)));
  SST_CK(a->focus_w.ensure((size_t) n * plane * sizeof(float)));
  if( !a->gk_n ) {
    float gk[64];
    a->gk_n = gaussian_kernel(3.0, gk);
    SST_CK(a->gk_focus.ensure(64 * sizeof(float)));
    SST_CK(cudaMemcpy(a->gk_focus.p, gk, a->gk_n * sizeof(float), cudaMemcpyHostToDevice));
  }
  SST_CK_LAUNCH(launch_focus_energy(d_frames, depth, row_stride, frame_stride, sw, sh, scale, motion, coeffs, n, a->w,
      a->h, a->focus_e.as<float>(), st));
  SST_CK_LAUNCH(launch_convert_smooth(a->focus_e.p, SST_DEPTH_F32, n, a->w, a->h, (size_t) a->w * sizeof(float),
      plane * sizeof(float), 1.0, a->gk_focus.as<float>(), a->gk_n, a->focus_w.as<float>(), plane, st));
  *maps = a->focus_w.as<float>();
  return SST_OK;
}

int sst_internal_lv_create(sst_local_variance ** out, const sst_local_variance_options * o);   // sst_weights.cu
int sst_internal_lv_build(sst_local_variance * L, const void * d_frames, int depth, int n, int w, int h,
    size_t row_stride, size_t frame_stride, double scale, cudaStream_t st);
int sst_internal_lv_warp(sst_local_variance * L, int motion, const float * coeffs, int dw, int dh, float * out,
    cudaStream_t st);

/* local-variance weighting: each frame's compute_local_variance_map warped
 * to the accumulator's grid (bilinear, BORDER_CONSTANT 0); no maps (weight 1)
 * when kradius <= 0, as weights_required (c_image_stacking_pipeline.cc:
 * 2005-2011) */
static int lv_maps(sst_weighted_average * a, const void * d_frames, int depth, int n, int sw, int sh,
    size_t row_stride, size_t frame_stride, double scale, int motion, const float * coeffs, const float ** maps,
    cudaStream_t st)
{
  *maps = nullptr;
  if( a->lvo.kradius <= 0 ) return SST_OK;
  if( !a->lv ) SST_TRY(sst_internal_lv_create(&a->lv, &a->lvo));
  SST_CK(a->focus_w.ensure((size_t) n * a->plane() * sizeof(float)));
  SST_TRY(sst_internal_lv_build(a->lv, d_frames, depth, n, sw, sh, row_stride, frame_stride, scale, st));
  SST_TRY(sst_internal_lv_warp(a->lv, motion, coeffs, a->w, a->h, a->focus_w.as<float>(), st));
  *maps = a->focus_w.as<float>();
  return SST_OK;
}

extern "C" int sst_weighted_average_set_local_variance(sst_weighted_average * h, const sst_local_variance_options * o)
{
  if( !h || !o ) return set_error(SST_ERR_INVALID_ARG, "sst_weighted_average_set_local_variance: NULL argument");
  if( o->kradius > 16 ) return set_error(SST_ERR_UNSUPPORTED, "local variance map: kradius above 16 is not supported");
  h->lvo = *o;
  sst_local_variance_destroy(h->lv);   // re-created with the new options on first use
  h->lv = nullptr;
  return SST_OK;
}

extern "C" int sst_weighted_average_create(sst_weighted_average ** out, int width, int height)
{
  if( !out || width < 1 || height < 1 ) return set_error(SST_ERR_INVALID_ARG, "sst_weighted_average_create: invalid arguments");
  sst_weighted_average * a = new (std::nothrow) sst_weighted_average();
  if( !a ) return set_error(SST_ERR_NOMEM, "out of host memory");
  a->w = width, a->h = height;
  cudaError_t e = a->acc.ensure(4 * a->plane() * sizeof(float));
  if( e == cudaSuccess ) e = cudaMemset(a->acc.p, 0, 4 * a->plane() * sizeof(float));
  if( e != cudaSuccess ) {
    delete a;
    return set_error(SST_ERR_CUDA, "accumulator allocation failed: %s", cudaGetErrorString(e));
  }
  *out = a;
  return SST_OK;
}

extern "C" int sst_weighted_average_set_tuning(sst_weighted_average * a, const sst_tuning * t)
{
  if( !a ) return set_error(SST_ERR_INVALID_ARG, "NULL accumulator");
  SST_TRY(check_tuning(t));
  a->max_chunks = t->stack_max_chunks > 0 ? t->stack_max_chunks : 4;
  a->items_per_slot = t->stack_items_per_slot > 0 ? t->stack_items_per_slot : 4;
  return SST_OK;
}

extern "C" int sst_weighted_average_destroy(sst_weighted_average * a)
{
  delete a;
  return SST_OK;
}

extern "C" int sst_weighted_average_clear(sst_weighted_average * a, void * stream)
{
  if( !a ) return set_error(SST_ERR_INVALID_ARG, "NULL accumulator");
  SST_CK(cudaMemsetAsync(a->acc.p, 0, 4 * a->plane() * sizeof(float), (cudaStream_t) stream));
  a->frames = 0;
  return SST_OK;
}

extern "C" int sst_weighted_average_accumulated_frames(const sst_weighted_average * a)
{
  return a ? a->frames : 0;
}

extern "C" int sst_weighted_average_add(sst_weighted_average * a, const void * src, int depth, size_t row_stride,
    double scale, const void * weights, int weights_depth, size_t weights_stride, int on_device, void * stream)
{
  if( !a || !src ) return set_error(SST_ERR_INVALID_ARG, "sst_weighted_average_add: NULL argument");
  if( depth_bytes(depth) == 0 ) return set_error(SST_ERR_INVALID_ARG, "unsupported depth %d", depth);
  if( weights && weights_depth != SST_DEPTH_U8 && weights_depth != SST_DEPTH_F32 )
    return set_error(SST_ERR_INVALID_ARG, "weights must be CV_8UC1 or CV_32FC1");
  cudaStream_t st = (cudaStream_t) stream;
  const void * dsrc = src, * dw = weights;
  if( !on_device ) {
    SST_CK(a->src.ensure(row_stride * a->h));
    SST_CK(cudaMemcpyAsync(a->src.p, src, row_stride * a->h, cudaMemcpyHostToDevice, st));
    dsrc = a->src.p;
    if( weights ) {
      SST_CK(a->wsrc.ensure(weights_stride * a->h));
      SST_CK(cudaMemcpyAsync(a->wsrc.p, weights, weights_stride * a->h, cudaMemcpyHostToDevice, st));
      dw = a->wsrc.p;
    }
  }
  SST_CK_LAUNCH(launch_stack_add_plain(dsrc, depth, row_stride, scale, dw, weights_depth, weights_stride, a->w, a->h,
      a->acc.as<float>(), a->plane(), st));
  if( !on_device ) SST_CK(cudaStreamSynchronize(st));
  ++a->frames;
  return SST_OK;
}

static int add_warped_device(sst_weighted_average * a, const void * d_frames, int depth, int n, int sw, int sh,
    size_t row_stride, size_t frame_stride, double scale, const sst_motion_model & m, const float * d_params,
    const int32_t * d_status, const float * d_weights, int border, cudaStream_t st, int wmode = 0)
{
  SST_CK(a->coeffs.ensure((size_t) n * SST_NCOEF * sizeof(float)));
  SST_CK(a->weff.ensure((size_t) n * sizeof(float)));
  SST_CK_LAUNCH(launch_coeffs_from_params(m, d_params, n, a->coeffs.as<float>(), st));
  SST_CK_LAUNCH(launch_effective_weights(d_weights, d_status, n, a->weff.as<float>(), st));
  const float * maps = nullptr;
  if( wmode == 2 ) SST_TRY(focus_maps(a, d_frames, depth, n, sw, sh, row_stride, frame_stride, scale, m.type,
      a->coeffs.as<float>(), &maps, st));
  if( wmode == 3 ) SST_TRY(lv_maps(a, d_frames, depth, n, sw, sh, row_stride, frame_stride, scale, m.type,
      a->coeffs.as<float>(), &maps, st));
  StackArgs s;
  s.wmap = maps;
  s.frames = (const uint8_t *) d_frames;
  s.row_stride = row_stride, s.frame_stride = frame_stride;
  s.sw = sw, s.sh = sh, s.n = n;
  s.scale = (float) scale;
  s.coeffs = a->coeffs.as<float>();
  s.weights = a->weff.as<float>();
  s.dw = a->w, s.dh = a->h;
  s.acc = a->acc.as<float>();
  s.plane = a->plane();
  s.border = border;
  // a tile's frames may be split over up to four CTAs (partial sums merged in order)
  const int kChunks = a->max_chunks;
  if( kChunks > 1 ) SST_CK(a->part.ensure((size_t) (kChunks - 1) * 4 * a->plane() * sizeof(float)));
  s.part = kChunks > 1 ? a->part.as<float>() : nullptr, s.max_chunks = kChunks;
  s.items_per_slot = a->items_per_slot;
  if( !a->err.p ) {
    SST_CK(a->err.ensure(sizeof(int)));
    SST_CK(cudaMemsetAsync(a->err.p, 0, sizeof(int), st));
  }
  s.err = a->err.as<int>();
  SST_CK_LAUNCH(launch_stack_add_warped(s, m.type, depth, st));
  return SST_OK;
}

/* reports (and clears) the stacking kernels' error flag */
static int check_acc_wait_flag(sst_weighted_average * a, cudaStream_t st)
{
  if( !a->err.p ) return SST_OK;
  int e = 0;
  SST_CK(cudaMemcpyAsync(&e, a->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  SST_CK(cudaStreamSynchronize(st));
  if( !e ) return SST_OK;
  SST_CK(cudaMemsetAsync(a->err.p, 0, sizeof(int), st));
  return set_error(SST_ERR_TIMEOUT, "a stacking kernel raised its error flag; the accumulator is invalid");
}

extern "C" int sst_weighted_average_add_warped_batch(sst_weighted_average * a, const void * frames, int depth, int n,
    int src_width, int src_height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    const sst_motion_model * model, const float * params, const int32_t * status, const float * weights,
    int border, void * stream)
{
  if( !a || !frames || !model || !params ) return set_error(SST_ERR_INVALID_ARG, "add_warped_batch: NULL argument");
  if( n < 1 ) return set_error(SST_ERR_INVALID_ARG, "n must be >= 1");
  if( depth_bytes(depth) == 0 ) return set_error(SST_ERR_INVALID_ARG, "unsupported depth %d", depth);
  if( row_stride < (size_t) src_width * depth_bytes(depth) || frame_stride < row_stride * src_height )
    return set_error(SST_ERR_INVALID_ARG, "invalid strides");
  if( model->type < 0 || model->type > 7 ) return set_error(SST_ERR_INVALID_ARG, "invalid motion type");
  if( border != SST_BORDER_CONSTANT && border != SST_BORDER_REPLICATE && border != SST_BORDER_REFLECT &&
      border != SST_BORDER_REFLECT101 )
    return set_error(SST_ERR_UNSUPPORTED, "unsupported border mode %d", border);
  cudaStream_t st = (cudaStream_t) stream;
  const void * dframes = frames;
  const float * dparams = params;
  const int32_t * dstatus = status;
  const float * dweights = weights;
  ScopedBuf tf, tp, ts, tw;
  if( !on_device ) {
    SST_CK(tf.ensure(frame_stride * n));
    SST_CK(cudaMemcpyAsync(tf.p, frames, frame_stride * n, cudaMemcpyHostToDevice, st));
    dframes = tf.p;
    SST_CK(tp.ensure((size_t) n * 12 * sizeof(float)));
    SST_CK(cudaMemcpyAsync(tp.p, params, (size_t) n * 12 * sizeof(float), cudaMemcpyHostToDevice, st));
    dparams = tp.as<float>();
    if( status ) {
      SST_CK(ts.ensure((size_t) n * sizeof(int32_t)));
      SST_CK(cudaMemcpyAsync(ts.p, status, (size_t) n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
      dstatus = ts.as<int32_t>();
    }
    if( weights ) {
      SST_CK(tw.ensure((size_t) n * sizeof(float)));
      SST_CK(cudaMemcpyAsync(tw.p, weights, (size_t) n * sizeof(float), cudaMemcpyHostToDevice, st));
      dweights = tw.as<float>();
    }
  }
  const int r = add_warped_device(a, dframes, depth, n, src_width, src_height, row_stride, frame_stride, scale, *model,
      dparams, dstatus, dweights, border, st);
  if( !on_device ) {
    cudaStreamSynchronize(st);
    tf.release(), tp.release(), ts.release(), tw.release();
  }
  if( r != SST_OK ) return r;
  a->frames += n;
  return SST_OK;
}

extern "C" int sst_weighted_average_compute(sst_weighted_average * a, float * avg, uint8_t * mask, int on_device, void * stream)
{
  if( !a ) return set_error(SST_ERR_INVALID_ARG, "NULL accumulator");
  if( a->frames < 1 ) return set_error(SST_ERR_STATE, "no frames accumulated");
  cudaStream_t st = (cudaStream_t) stream;
  const size_t N = a->plane();
  SST_TRY(check_acc_wait_flag(a, st));
  if( on_device ) {
    SST_CK_LAUNCH(launch_stack_compute(a->acc.as<float>(), N, (int) N, avg, mask, nullptr, st));
    return SST_OK;
  }
  // staged in buffers kept with the accumulator: no allocation per call
  if( avg ) SST_CK(a->out_avg.ensure(N * sizeof(float)));
  if( mask ) SST_CK(a->out_mask.ensure(N));
  SST_CK_LAUNCH(launch_stack_compute(a->acc.as<float>(), N, (int) N, avg ? a->out_avg.as<float>() : nullptr,
      mask ? a->out_mask.as<uint8_t>() : nullptr, nullptr, st));
  if( avg ) SST_CK(cudaMemcpyAsync(avg, a->out_avg.p, N * sizeof(float), cudaMemcpyDeviceToHost, st));
  if( mask ) SST_CK(cudaMemcpyAsync(mask, a->out_mask.p, N, cudaMemcpyDeviceToHost, st));
  SST_CK(cudaStreamSynchronize(st));
  return SST_OK;
}

extern "C" int sst_weighted_average_get_acc_counters(sst_weighted_average * a, float * accw, int on_device, void * stream)
{
  if( !a || !accw ) return set_error(SST_ERR_INVALID_ARG, "NULL argument");
  cudaStream_t st = (cudaStream_t) stream;
  const size_t N = a->plane();
  if( on_device ) {
    SST_CK_LAUNCH(launch_stack_compute(a->acc.as<float>(), N, (int) N, nullptr, nullptr, accw, st));
    return SST_OK;
  }
  ScopedBuf d;
  SST_CK(d.ensure(N * sizeof(float)));
  SST_CK_LAUNCH(launch_stack_compute(a->acc.as<float>(), N, (int) N, nullptr, nullptr, d.as<float>(), st));
  SST_CK(cudaMemcpyAsync(accw, d.p, N * sizeof(float), cudaMemcpyDeviceToHost, st));
  SST_CK(cudaStreamSynchronize(st));
  return SST_OK;
}

extern "C" int sst_weighted_average_reinitialize(sst_weighted_average * a, const float * avg, const float * accw,
    int on_device, void * stream)
{
  if( !a || !avg || !accw ) return set_error(SST_ERR_INVALID_ARG, "NULL argument");
  cudaStream_t st = (cudaStream_t) stream;
  const size_t N = a->plane();
  const float * da = avg, * dw = accw;
  ScopedBuf ta, tw;
  if( !on_device ) {
    SST_CK(ta.ensure(N * sizeof(float)));
    SST_CK(tw.ensure(N * sizeof(float)));
    SST_CK(cudaMemcpyAsync(ta.p, avg, N * sizeof(float), cudaMemcpyHostToDevice, st));
    SST_CK(cudaMemcpyAsync(tw.p, accw, N * sizeof(float), cudaMemcpyHostToDevice, st));
    da = ta.as<float>(), dw = tw.as<float>();
  }
  SST_CK_LAUNCH(launch_stack_reinit(a->acc.as<float>(), N, (int) N, da, dw, st));
  if( !on_device ) SST_CK(cudaStreamSynchronize(st));
  a->frames = 1;   // c_weigthed_average::reinitialize sets _accumulated_frames = 1
  return SST_OK;
}

extern "C" int sst_weighted_average_save_state(sst_weighted_average * a, float * state4, int32_t * frames, void * stream)
{
  if( !a || !state4 ) return set_error(SST_ERR_INVALID_ARG, "NULL argument");
  cudaStream_t st = (cudaStream_t) stream;
  SST_CK(cudaMemcpyAsync(state4, a->acc.p, 4 * a->plane() * sizeof(float), cudaMemcpyDeviceToHost, st));
  SST_CK(cudaStreamSynchronize(st));
  SST_TRY(check_acc_wait_flag(a, st));
  if( frames ) *frames = a->frames;
  return SST_OK;
}

extern "C" int sst_weighted_average_load_state(sst_weighted_average * a, const float * state4, int32_t frames, void * stream)
{
  if( !a || !state4 ) return set_error(SST_ERR_INVALID_ARG, "NULL argument");
  cudaStream_t st = (cudaStream_t) stream;
  SST_CK(cudaMemcpyAsync(a->acc.p, state4, 4 * a->plane() * sizeof(float), cudaMemcpyHostToDevice, st));
  SST_CK(cudaStreamSynchronize(st));
  a->frames = frames;
  return SST_OK;
}

/* ================================================ streamed pipeline */

/* Frames per chunk of a streamed sequence (sst_stack_frames and its Bayer
 * form). Device frames: chunks of `chunk` frames. Host frames: the copy of
 * the first chunk cannot overlap anything, and every chunk pays the
 * registration's convergence tail once, so the chunks grow geometrically
 * (x 2.5, a frame's registration takes about 2.5 times its copy) from a
 * quarter of `chunk` up to `chunk`; a remainder is absorbed into the chunk
 * before it when that stays within `chunk`. */
static std::vector<int> chunk_plan(int n, int chunk, bool host)
{
  std::vector<int> sizes;
  if( !host ) {
    for( int f0 = 0; f0 < n; f0 += chunk ) sizes.push_back(std::min(chunk, n - f0));
    return sizes;
  }
  int first = std::min(chunk, std::max(64, chunk / 4));
  if( n <= first ) return { n };
  sizes.push_back(first);
  int rem = n - first;
  while ( rem > 0 ) {
    const int nxt = (int) std::min<long long>(chunk, ((long long) sizes.back() * 5 + 1) / 2);
    int take;
    if( rem <= nxt ) take = rem;
    else if( rem <= chunk && rem - nxt < sizes.back() / 2 ) take = rem;
    else take = nxt;
    sizes.push_back(take);
    rem -= take;
  }
  return sizes;
}

extern "C" int sst_stack_frames(sst_ecch * h, sst_weighted_average * acc, const void * frames, int depth, int n,
    int width, int height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int border, int weighting,
    float * params_out, int32_t * status_out, float * rho_out, float * weight_out, void * stream)
{
  if( !h || !acc || !frames ) return set_error(SST_ERR_INVALID_ARG, "sst_stack_frames: NULL argument");
  if( border != SST_BORDER_CONSTANT && border != SST_BORDER_REPLICATE && border != SST_BORDER_REFLECT &&
      border != SST_BORDER_REFLECT101 )
    return set_error(SST_ERR_UNSUPPORTED, "unsupported border mode %d", border);
  if( h->L == 0 ) return set_error(SST_ERR_STATE, "c_ecch: no reference image was set");
  if( n < 1 ) return set_error(SST_ERR_INVALID_ARG, "n must be >= 1");
  if( weighting < 0 || weighting > 3 ) return set_error(SST_ERR_INVALID_ARG, "weighting must be 0, 1, 2 or 3");
  if( width != h->w || height != h->h || acc->w != h->w || acc->h != h->h )
    return set_error(SST_ERR_INVALID_ARG, "frame, reference and accumulator sizes must match");
  if( depth_bytes(depth) == 0 ) return set_error(SST_ERR_INVALID_ARG, "unsupported depth %d", depth);
  if( row_stride < (size_t) width * depth_bytes(depth) || frame_stride < row_stride * height )
    return set_error(SST_ERR_INVALID_ARG, "invalid strides");
  SST_TRY(validate_passes(h, num_passes, passes));
  if( h->o.method == M_IC || h->o.method == M_ICLM ) {
    for( int k = 0; k < num_passes; ++k )
      if( !model_invertible(passes[k]) )
        return set_error(SST_ERR_UNSUPPORTED, "inverse compositional ECC requires an invertible motion model");
  }
  SST_TRY(ensure_streams(h));
  SST_TRY(join_user(h, stream));
  cudaStream_t st = h->st, cp = h->st_copy;
  const int chunk = std::max(1, std::min(h->chunk, n));
  const sst_motion_model & last = passes[num_passes - 1];
  if( !on_device ) {
    SST_CK(h->stage[0].ensure(frame_stride * chunk));
    SST_CK(h->stage[1].ensure(frame_stride * chunk));
    SST_CK(cudaEventRecord(h->ev_free[0], st));
    SST_CK(cudaEventRecord(h->ev_free[1], st));
  }
  SST_CK(h->res_params.ensure((size_t) n * 12 * sizeof(float)));
  SST_CK(h->res_status.ensure((size_t) n * sizeof(int32_t)));
  SST_CK(h->res_rho.ensure((size_t) n * sizeof(float)));
  SST_CK(h->res_weight.ensure((size_t) n * sizeof(float)));
  int buf = 0, f0 = 0;
  for( const int nc : chunk_plan(n, chunk, !on_device) ) {
    const uint8_t * fsrc = (const uint8_t *) frames + (size_t) f0 * frame_stride;
    const void * d_frames = fsrc;
    if( !on_device ) {
      // copy engine: wait until this staging buffer's previous chunk is consumed
      SST_CK(cudaStreamWaitEvent(cp, h->ev_free[buf], 0));
      SST_CK(cudaMemcpyAsync(h->stage[buf].p, fsrc, frame_stride * nc, cudaMemcpyHostToDevice, cp));
      SST_CK(cudaEventRecord(h->ev_copy[buf], cp));
      SST_CK(cudaStreamWaitEvent(st, h->ev_copy[buf], 0));
      d_frames = h->stage[buf].p;
    }
    SST_TRY(register_device(h, d_frames, depth, nc, row_stride, frame_stride, scale, num_passes, passes, nullptr, false));
    SST_TRY(add_warped_device(acc, d_frames, depth, nc, width, height, row_stride, frame_stride, scale, last,
        h->out_params.as<float>(), h->out_status.as<int32_t>(), weighting == 1 ? h->out_weight.as<float>() : nullptr,
        border, st, weighting));
    if( !on_device ) SST_CK(cudaEventRecord(h->ev_free[buf], st));
    SST_TRY(copy_out(h->res_params.as<float>() + (size_t) f0 * 12, h->out_params.p, (size_t) nc * 12 * sizeof(float), 1, st));
    SST_TRY(copy_out(h->res_status.as<int32_t>() + f0, h->out_status.p, (size_t) nc * sizeof(int32_t), 1, st));
    SST_TRY(copy_out(h->res_rho.as<float>() + f0, h->out_rho.p, (size_t) nc * sizeof(float), 1, st));
    SST_TRY(copy_out(h->res_weight.as<float>() + f0, h->out_weight.p, (size_t) nc * sizeof(float), 1, st));
    f0 += nc, buf ^= 1;
  }
  SST_TRY(copy_out(params_out, h->res_params.p, (size_t) n * 12 * sizeof(float), on_device, st));
  SST_TRY(copy_out(status_out, h->res_status.p, (size_t) n * sizeof(int32_t), on_device, st));
  SST_TRY(copy_out(rho_out, h->res_rho.p, (size_t) n * sizeof(float), on_device, st));
  SST_TRY(copy_out(weight_out, h->res_weight.p, (size_t) n * sizeof(float), on_device, st));
  // c_frame_accumulation::_accumulated_frames counts the frames actually added
  std::vector<int32_t> stv(n);
  SST_CK(cudaMemcpyAsync(stv.data(), h->res_status.p, (size_t) n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  SST_CK(cudaStreamSynchronize(st));
  for( int f = 0; f < n; ++f ) acc->frames += stv[f] == SST_FRAME_OK ? 1 : 0;
  SST_TRY(check_wait_flag(h));
  SST_TRY(release_to_user(h, stream));
  return SST_OK;
}

/* The Bayer form of the stacking loop body: register the 2x2-binned
 * luminance of each raw frame (average_bayer_planes, debayer.cc:277-330)
 * against the binned reference of `h`, then warp the four Bayer planes of
 * the raw frame (extract_bayer_planes order, debayer.cc:96-147) with the
 * registered transform and add them to the four plane accumulators. */
extern "C" int sst_stack_bayer_frames(sst_ecch * h, sst_weighted_average * const * acc, const void * frames, int n,
    int width, int height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int border, int weighting,
    float * params_out, int32_t * status_out, float * rho_out, float * weight_out, void * stream)
{
  if( !h || !acc || !frames ) return set_error(SST_ERR_INVALID_ARG, "sst_stack_bayer_frames: NULL argument");
  for( int k = 0; k < 4; ++k )
    if( !acc[k] ) return set_error(SST_ERR_INVALID_ARG, "sst_stack_bayer_frames: NULL plane accumulator");
  if( border != SST_BORDER_CONSTANT && border != SST_BORDER_REPLICATE && border != SST_BORDER_REFLECT &&
      border != SST_BORDER_REFLECT101 )
    return set_error(SST_ERR_UNSUPPORTED, "unsupported border mode %d", border);
  if( h->L == 0 ) return set_error(SST_ERR_STATE, "c_ecch: no reference image was set");
  if( n < 1 ) return set_error(SST_ERR_INVALID_ARG, "n must be >= 1");
  if( (width & 1) || (height & 1) )
    return set_error(SST_ERR_INVALID_ARG, "Can not average raw bayer planes for uneven image size %dx%d", width, height);
  if( weighting < 0 || weighting > 3 ) return set_error(SST_ERR_INVALID_ARG, "weighting must be 0, 1, 2 or 3");
  const int pw = width / 2, ph = height / 2;
  if( pw != h->w || ph != h->h )
    return set_error(SST_ERR_INVALID_ARG, "the reference must be the binned size (width/2 x height/2)");
  for( int k = 0; k < 4; ++k )
    if( acc[k]->w != pw || acc[k]->h != ph ) return set_error(SST_ERR_INVALID_ARG, "plane accumulators must be width/2 x height/2");
  if( row_stride < (size_t) width * 2 || frame_stride < row_stride * height || (row_stride & 3) || (frame_stride & 3) ||
      ((uintptr_t) frames & 3) )
    return set_error(SST_ERR_INVALID_ARG, "invalid or misaligned strides");
  SST_TRY(validate_passes(h, num_passes, passes));
  if( h->o.method == M_IC || h->o.method == M_ICLM ) {
    for( int k = 0; k < num_passes; ++k )
      if( !model_invertible(passes[k]) )
        return set_error(SST_ERR_UNSUPPORTED, "inverse compositional ECC requires an invertible motion model");
  }
  SST_TRY(ensure_streams(h));
  SST_TRY(join_user(h, stream));
  cudaStream_t st = h->st, cp = h->st_copy;
  const int chunk = std::max(1, std::min(std::min(h->chunk, n), 65535));
  const sst_motion_model & last = passes[num_passes - 1];
  const size_t bin_frame = (size_t) pw * ph * 2;
  if( !on_device ) {
    SST_CK(h->stage[0].ensure(frame_stride * chunk));
    SST_CK(h->stage[1].ensure(frame_stride * chunk));
    SST_CK(cudaEventRecord(h->ev_free[0], st));
    SST_CK(cudaEventRecord(h->ev_free[1], st));
  }
  SST_CK(h->binned.ensure(bin_frame * chunk));
  SST_CK(h->res_params.ensure((size_t) n * 12 * sizeof(float)));
  SST_CK(h->res_status.ensure((size_t) n * sizeof(int32_t)));
  SST_CK(h->res_rho.ensure((size_t) n * sizeof(float)));
  SST_CK(h->res_weight.ensure((size_t) n * sizeof(float)));
  sst_weighted_average * a0 = acc[0];
  SST_CK(a0->coeffs.ensure((size_t) chunk * SST_NCOEF * sizeof(float)));
  SST_CK(a0->weff.ensure((size_t) chunk * sizeof(float)));
  int buf = 0, f0 = 0;
  for( const int nc : chunk_plan(n, chunk, !on_device) ) {
    const uint8_t * fsrc = (const uint8_t *) frames + (size_t) f0 * frame_stride;
    const void * d_frames = fsrc;
    if( !on_device ) {
      SST_CK(cudaStreamWaitEvent(cp, h->ev_free[buf], 0));
      SST_CK(cudaMemcpyAsync(h->stage[buf].p, fsrc, frame_stride * nc, cudaMemcpyHostToDevice, cp));
      SST_CK(cudaEventRecord(h->ev_copy[buf], cp));
      SST_CK(cudaStreamWaitEvent(st, h->ev_copy[buf], 0));
      d_frames = h->stage[buf].p;
    }
    SST_CK_LAUNCH(launch_average_bayer_planes_batch(d_frames, width, height, row_stride, frame_stride, nc,
        h->binned.as<uint16_t>(), st));
    SST_TRY(register_device(h, h->binned.p, SST_DEPTH_U16, nc, (size_t) pw * 2, bin_frame, scale, num_passes, passes,
        nullptr, false));
    SST_CK_LAUNCH(launch_coeffs_from_params(last, h->out_params.as<float>(), nc, a0->coeffs.as<float>(), st));
    SST_CK_LAUNCH(launch_effective_weights(weighting == 1 ? h->out_weight.as<float>() : nullptr,
        h->out_status.as<int32_t>(), nc, a0->weff.as<float>(), st));
    const float * maps = nullptr;
    if( weighting == 2 ) {
      // focus weights of the warped binned luminance, shared by the four planes
      SST_TRY(focus_maps(a0, h->binned.p, SST_DEPTH_U16, nc, pw, ph, (size_t) pw * 2, bin_frame, scale, last.type,
          a0->coeffs.as<float>(), &maps, st));
    }
    if( weighting == 3 ) {
      // local-variance maps of the binned luminance, shared by the four planes
      SST_TRY(lv_maps(a0, h->binned.p, SST_DEPTH_U16, nc, pw, ph, (size_t) pw * 2, bin_frame, scale, last.type,
          a0->coeffs.as<float>(), &maps, st));
    }
    BayerPlanesArgs b;
    b.wmap = maps;
    b.frames = (const uint8_t *) d_frames;
    b.row_stride = row_stride, b.frame_stride = frame_stride;
    b.pw = pw, b.ph = ph, b.n = nc;
    b.scale = (float) scale;
    b.coeffs = a0->coeffs.as<float>();
    b.weights = a0->weff.as<float>();
    for( int k = 0; k < 4; ++k ) b.acc[k] = acc[k]->acc.as<float>();
    b.plane = a0->plane();
    b.border = border;
    SST_CK_LAUNCH(launch_stack_bayer_planes(b, last.type, st));
    if( !on_device ) SST_CK(cudaEventRecord(h->ev_free[buf], st));
    SST_TRY(copy_out(h->res_params.as<float>() + (size_t) f0 * 12, h->out_params.p, (size_t) nc * 12 * sizeof(float), 1, st));
    SST_TRY(copy_out(h->res_status.as<int32_t>() + f0, h->out_status.p, (size_t) nc * sizeof(int32_t), 1, st));
    SST_TRY(copy_out(h->res_rho.as<float>() + f0, h->out_rho.p, (size_t) nc * sizeof(float), 1, st));
    SST_TRY(copy_out(h->res_weight.as<float>() + f0, h->out_weight.p, (size_t) nc * sizeof(float), 1, st));
    f0 += nc, buf ^= 1;
  }
  SST_TRY(copy_out(params_out, h->res_params.p, (size_t) n * 12 * sizeof(float), on_device, st));
  SST_TRY(copy_out(status_out, h->res_status.p, (size_t) n * sizeof(int32_t), on_device, st));
  SST_TRY(copy_out(rho_out, h->res_rho.p, (size_t) n * sizeof(float), on_device, st));
  SST_TRY(copy_out(weight_out, h->res_weight.p, (size_t) n * sizeof(float), on_device, st));
  std::vector<int32_t> stv(n);
  SST_CK(cudaMemcpyAsync(stv.data(), h->res_status.p, (size_t) n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  SST_CK(cudaStreamSynchronize(st));
  int added = 0;
  for( int f = 0; f < n; ++f ) added += stv[f] == SST_FRAME_OK ? 1 : 0;
  for( int k = 0; k < 4; ++k ) acc[k]->frames += added;
  SST_TRY(check_wait_flag(h));
  SST_TRY(release_to_user(h, stream));
  return SST_OK;
}

/* ================================================ utilities */

extern "C" int sst_remap(const void * src, int depth, int src_width, int src_height, size_t row_stride, double scale,
    const sst_motion_model * model, const float * params, int border,
    float * dst, uint8_t * dst_mask, int dst_width, int dst_height, void * stream)
{
  if( !src || !model || !params ) return set_error(SST_ERR_INVALID_ARG, "sst_remap: NULL argument");
  if( depth_bytes(depth) == 0 ) return set_error(SST_ERR_INVALID_ARG, "unsupported depth %d", depth);
  if( border != SST_BORDER_CONSTANT && border != SST_BORDER_REPLICATE && border != SST_BORDER_REFLECT &&
      border != SST_BORDER_REFLECT101 )
    return set_error(SST_ERR_UNSUPPORTED, "unsupported border mode %d", border);
  cudaStream_t st = (cudaStream_t) stream;
  double s[16], p[12];
  model_identity(*model, s);
  const int M = model_nparams(*model);
  for( int j = 0; j < M; ++j ) p[j] = params[j];
  model_set_params(*model, s, p);
  float c[SST_NCOEF];
  model_warp_coeffs(*model, s, c);
  ScopedBuf dc;
  SST_CK(dc.ensure(sizeof(c)));
  SST_CK(cudaMemcpyAsync(dc.p, c, sizeof(c), cudaMemcpyHostToDevice, st));
  SST_CK_LAUNCH(launch_remap(src, depth, src_width, src_height, row_stride, scale, model->type, dc.as<float>(), border,
      dst, dst_mask, dst_width, dst_height, st));
  SST_CK(cudaStreamSynchronize(st));
  return SST_OK;
}

extern "C" int sst_extract_bayer_planes_u16(const uint16_t * src, int width, int height, size_t row_stride,
    uint16_t * dst, void * stream)
{
  if( !src || !dst ) return set_error(SST_ERR_INVALID_ARG, "NULL argument");
  if( (width & 1) || (height & 1) ) return set_error(SST_ERR_INVALID_ARG, "Can not make debayer for uneven image size %dx%d", width, height);
  if( (row_stride & 3) || ((uintptr_t) src & 3) || ((uintptr_t) dst & 7) )
    return set_error(SST_ERR_INVALID_ARG, "misaligned bayer buffers");
  SST_CK_LAUNCH(launch_bayer_planes(0, src, width, height, row_stride, dst, (cudaStream_t) stream));
  return SST_OK;
}

extern "C" int sst_average_bayer_planes_u16(const uint16_t * src, int width, int height, size_t row_stride,
    uint16_t * dst, void * stream)
{
  if( !src || !dst ) return set_error(SST_ERR_INVALID_ARG, "NULL argument");
  if( (width & 1) || (height & 1) ) return set_error(SST_ERR_INVALID_ARG, "Can not average raw bayer planes for uneven image size %dx%d", width, height);
  if( (row_stride & 3) || ((uintptr_t) src & 3) ) return set_error(SST_ERR_INVALID_ARG, "misaligned bayer buffers");
  SST_CK_LAUNCH(launch_bayer_planes(1, src, width, height, row_stride, dst, (cudaStream_t) stream));
  return SST_OK;
}
