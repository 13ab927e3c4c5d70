/*
 * sst_roi.cu -- ROI batches: many crops of different sizes, each registered
 * against its own reference crop, in one level-synchronous schedule.
 *
 * In the reference every crop is one c_ecch: set_reference_image(ref crop)
 * builds that crop's reference pyramid (ecc2.cc:984-1057), align(cur crop)
 * builds the current pyramid and runs coarse-to-fine (ecc2.cc:1060-1176).
 * Here the pyramids of all crops are packed side by side in two f32 pools
 * (reference, current) built by ragged batched kernels (grid.z = crop), and
 * the Gauss-Newton steps of every crop still iterating at a level run as one
 * pass launch + one solve launch, with per-crop level geometry (RoiLevel).
 * Crops with fewer pyramid levels join at their own coarsest level.
 *
 * Methods: forward-additive and LM (the stencil passes). IC and IC-LM need
 * per-crop reference Gauss-Newton matrices and are not offered for ROI
 * batches; the quadratic models of these batches cannot use them anyway
 * (c_image_transform.h:154-157: not invertible).
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <new>
#include <string>
#include <vector>

#include "sst_engine.cuh"
#include "sst_host.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu
void sst_internal_count_launches(int n);              // sst_capi.cu

using namespace sst;

static int rfail(int code, const std::string & msg)
{
  return sst_internal_error(code, msg.c_str());
}

#define SST_RCK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if( e_ != cudaSuccess )                                                                    \
      return rfail(SST_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while ( 0 )

#define SST_RLAUNCH(call)                                                                      \
  do {                                                                                         \
    SST_RCK(call);                                                                             \
    ++launches;                                                                                \
  } while ( 0 )

struct sst_roi_batch {
  sst_ecch_options o;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_user = nullptr, ev_done = nullptr;
  int num_sms = 0;
  DevBuf cur_in, ref_in;                 // staged host pools
  DevBuf cur, ref;                       // packed f32 pyramids
  DevBuf roi, jobs, sums, gk_in, gk_ref;
  DevBuf fs, part, lists, counts, prefix, total, ctp, init;
  DevBuf out_params, out_status, out_iters, out_eps, out_rho;
  // geometry and schedule of the last call (level statistics)
  std::vector<RoiLevel> h_roi;
  int n = 0, lmax = 0, num_passes = 0, max_it = 0, method = 0;
  int level_step[3][32];
  cudaEvent_t prof[3][32][2];
  bool prof_ready = false;

  ~sst_roi_batch()
  {
    if( prof_ready ) for( auto & a : prof ) for( auto & b : a ) for( auto & e : b ) cudaEventDestroy(e);
    DevBuf * bufs[] = { &cur_in, &ref_in, &cur, &ref, &roi, &jobs, &sums, &gk_in, &gk_ref, &fs, &part, &lists,
        &counts, &prefix, &total, &ctp, &init, &out_params, &out_status, &out_iters, &out_eps, &out_rho };
    for( DevBuf * b : bufs ) b->release();
    if( ev_user ) cudaEventDestroy(ev_user);
    if( ev_done ) cudaEventDestroy(ev_done);
    if( st ) cudaStreamDestroy(st);
  }
};

extern "C" int sst_roi_batch_create(sst_roi_batch ** out, const sst_ecch_options * o)
{
  if( !out || !o ) return rfail(SST_ERR_INVALID_ARG, "sst_roi_batch_create: NULL argument");
  if( o->method != SST_ECC_FORWARD_ADDITIVE && o->method != SST_ECC_LM )
    return rfail(SST_ERR_UNSUPPORTED, "ROI batches run the forward-additive or LM method");
  if( o->max_iterations < 1 || o->max_iterations > 1000 ) return rfail(SST_ERR_INVALID_ARG, "max_iterations must be 1..1000");
  if( o->reference_smooth_sigma > 4.5 || o->input_smooth_sigma > 4.5 )
    return rfail(SST_ERR_UNSUPPORTED, "smoothing sigma above 4.5 is not supported");
  sst_roi_batch * h = new (std::nothrow) sst_roi_batch();
  if( !h ) return rfail(SST_ERR_NOMEM, "out of host memory");
  h->o = *o;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if( e == cudaSuccess ) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if( e == cudaSuccess ) e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if( e == cudaSuccess ) e = cudaEventCreateWithFlags(&h->ev_user, cudaEventDisableTiming);
  if( e == cudaSuccess ) e = cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming);
  if( e != cudaSuccess ) {
    delete h;
    return rfail(SST_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = h;
  return SST_OK;
}

extern "C" int sst_roi_batch_destroy(sst_roi_batch * h)
{
  delete h;
  return SST_OK;
}

static int check_models(int num_passes, const sst_motion_model * passes)
{
  if( num_passes < 1 || num_passes > 3 || !passes ) return rfail(SST_ERR_INVALID_ARG, "1..3 motion passes are required");
  for( int k = 0; k < num_passes; ++k ) {
    const sst_motion_model & m = passes[k];
    if( m.type < 0 || m.type > 7 ) return rfail(SST_ERR_INVALID_ARG, "invalid motion type");
    if( (m.type == SST_MOTION_EUCLIDEAN || m.type == SST_MOTION_SCALED_EUCLIDEAN) && (m.fix_translation || m.fix_rotation) )
      return rfail(SST_ERR_UNSUPPORTED, "euclidean with fixed translation or rotation is not implemented");
    if( m.type == SST_MOTION_EUCLIDEAN && !m.fix_scale )
      return rfail(SST_ERR_INVALID_ARG, "EUCLIDEAN motion requires fix_scale = 1 (image_transform.cc:35-39)");
    if( m.type == SST_MOTION_SCALED_EUCLIDEAN && m.fix_scale )
      return rfail(SST_ERR_INVALID_ARG, "SCALED_EUCLIDEAN motion requires fix_scale = 0");
  }
  return SST_OK;
}

/* byte extent of a pool that holds every crop */
static size_t pool_extent(const sst_roi * rois, int n, bool ref, int bytes)
{
  size_t e = 0;
  for( int i = 0; i < n; ++i ) {
    const sst_roi & r = rois[i];
    const size_t off = (size_t) (ref ? r.ref_offset : r.cur_offset);
    const size_t rs = (size_t) (ref ? r.ref_row_stride : r.cur_row_stride);
    e = std::max(e, off + (size_t) (r.height - 1) * rs + (size_t) r.width * bytes);
  }
  return e;
}

extern "C" int sst_roi_batch_align(sst_roi_batch * h, int n, const sst_roi * rois, const void * ref_pool,
    const void * cur_pool, int depth, double scale, int on_device, int num_passes, const sst_motion_model * passes,
    const float * init_params, float * params_out, int32_t * status_out, int32_t * iters_out, float * eps_out,
    float * rho_out, void * stream)
{
  if( !h || !rois || !ref_pool || !cur_pool ) return rfail(SST_ERR_INVALID_ARG, "sst_roi_batch_align: NULL argument");
  if( n < 1 || n > 65535 ) return rfail(SST_ERR_INVALID_ARG, "n must be 1..65535");
  const int bytes = depth_bytes(depth);
  if( !bytes ) return rfail(SST_ERR_INVALID_ARG, "unsupported depth");
  {
    const int r = check_models(num_passes, passes);
    if( r != SST_OK ) return r;
  }
  const sst_ecch_options & o = h->o;
  const int min_side = std::max(4, o.minimum_image_size);
  for( int i = 0; i < n; ++i ) {
    const sst_roi & r = rois[i];
    if( r.width < min_side || r.height < min_side || r.ref_offset < 0 || r.cur_offset < 0 ||
        r.ref_row_stride < (int64_t) r.width * bytes || r.cur_row_stride < (int64_t) r.width * bytes )
      return rfail(SST_ERR_INVALID_ARG, "invalid ROI " + std::to_string(i));
  }
  cudaStream_t st = h->st;
  int launches = 0;
  SST_RCK(cudaEventRecord(h->ev_user, (cudaStream_t) stream));
  SST_RCK(cudaStreamWaitEvent(st, h->ev_user, 0));

  // ---- per-crop pyramid geometry
  const int method = o.method;
  int NSmax = 0;
  for( int k = 0; k < num_passes; ++k ) NSmax = std::max(NSmax, pass_num_sums(method, model_nparams(passes[k])));
  std::vector<int> L(n);
  int lmax = 1;
  for( int i = 0; i < n; ++i ) lmax = std::max(lmax, L[i] = ecch_num_levels(rois[i].width, rois[i].height, o));
  std::vector<RoiLevel> R((size_t) n * lmax);
  memset(R.data(), 0, R.size() * sizeof(RoiLevel));
  std::vector<int> ctp(n + 1, 0);
  size_t cur_total = 0, part_total = 0;
  int max_w = 0, max_h = 0;
  for( int i = 0; i < n; ++i ) {
    int lw = rois[i].width, lh = rois[i].height;
    max_w = std::max(max_w, lw), max_h = std::max(max_h, lh);
    for( int l = 0; l < L[i]; ++l ) {
      if( l > 0 ) lw = ((lw + 1) >> 1) & ~1, lh = ((lh + 1) >> 1) & ~1;
      RoiLevel & E = R[(size_t) i * lmax + l];
      E.w = lw, E.h = lh;
      E.cur_off = E.ref_off = cur_total;     // the two pools share one layout
      cur_total += (size_t) lw * lh;
      E.tiles = tiles_of(lw, lh, ST_TX, ST_TY, &E.tiles_x);
      E.scale_next = l > 0 ? (double) R[(size_t) i * lmax + l - 1].w / (double) lw : 0.0;
    }
    RoiLevel & E0 = R[(size_t) i * lmax];
    E0.ctiles = tiles_of(E0.w, E0.h, PW_TX, PW_TY, &E0.ctiles_x);
    E0.scale_first = L[i] > 1 ? (double) R[(size_t) i * lmax + L[i] - 1].w / (double) E0.w : 0.0;
    const size_t psz = std::max((size_t) E0.tiles * NSmax, (size_t) E0.ctiles * 6);
    for( int l = 0; l < L[i]; ++l ) R[(size_t) i * lmax + l].part_off = part_total;
    part_total += psz;
    ctp[i + 1] = ctp[i] + E0.ctiles;
  }

  // ---- buffers
  const int max_it = o.max_iterations;
  const int steps = num_passes * lmax * (max_it + 2);
  SST_RCK(h->cur.ensure(cur_total * sizeof(float)));
  SST_RCK(h->ref.ensure(cur_total * sizeof(float)));
  SST_RCK(h->roi.ensure(R.size() * sizeof(RoiLevel)));
  SST_RCK(h->fs.ensure((size_t) n * sizeof(FrameState)));
  SST_RCK(h->part.ensure(part_total * sizeof(double)));
  SST_RCK(h->lists.ensure((size_t) steps * n * sizeof(int)));
  SST_RCK(h->counts.ensure((size_t) steps * sizeof(int)));
  SST_RCK(h->prefix.ensure((size_t) n * sizeof(int)));
  SST_RCK(h->total.ensure(sizeof(int)));
  SST_RCK(h->ctp.ensure((size_t) (n + 1) * sizeof(int)));
  SST_RCK(h->init.ensure((size_t) n * 16 * sizeof(double)));
  SST_RCK(h->out_params.ensure((size_t) n * 12 * sizeof(float)));
  SST_RCK(h->out_status.ensure((size_t) n * sizeof(int32_t)));
  SST_RCK(h->out_iters.ensure((size_t) n * sizeof(int32_t)));
  SST_RCK(h->out_eps.ensure((size_t) n * sizeof(float)));
  SST_RCK(h->out_rho.ensure((size_t) n * sizeof(float)));

  // ---- inputs
  const uint8_t * d_ref = (const uint8_t *) ref_pool, * d_cur = (const uint8_t *) cur_pool;
  if( !on_device ) {
    const size_t er = pool_extent(rois, n, true, bytes), ec = pool_extent(rois, n, false, bytes);
    SST_RCK(h->ref_in.ensure(er));
    SST_RCK(h->cur_in.ensure(ec));
    SST_RCK(cudaMemcpyAsync(h->ref_in.p, ref_pool, er, cudaMemcpyHostToDevice, st));
    SST_RCK(cudaMemcpyAsync(h->cur_in.p, cur_pool, ec, cudaMemcpyHostToDevice, st));
    d_ref = h->ref_in.as<uint8_t>(), d_cur = h->cur_in.as<uint8_t>();
  }

  // ---- pyramids: jobs [ref convert n][cur convert n] then per level [ref pyrDown][cur pyrDown], then means
  std::vector<RaggedImg> jobs;
  for( int pool = 0; pool < 2; ++pool ) {
    for( int i = 0; i < n; ++i ) {
      const sst_roi & r = rois[i];
      RaggedImg j;
      j.src_off = (size_t) (pool == 0 ? r.ref_offset : r.cur_offset);
      j.src_stride = (size_t) (pool == 0 ? r.ref_row_stride : r.cur_row_stride);
      j.sw = j.dw = r.width, j.sh = j.dh = r.height;
      j.dst_off = R[(size_t) i * lmax].cur_off;
      jobs.push_back(j);
    }
  }
  std::vector<size_t> lvl_job0(lmax, 0);
  std::vector<int> lvl_jobs(lmax, 0), lvl_mw(lmax, 0), lvl_mh(lmax, 0);
  for( int l = 1; l < lmax; ++l ) {
    lvl_job0[l] = jobs.size();
    for( int i = 0; i < n; ++i ) {
      if( l >= L[i] ) continue;
      const RoiLevel & S = R[(size_t) i * lmax + l - 1], & D = R[(size_t) i * lmax + l];
      RaggedImg j;
      j.src_off = S.cur_off, j.src_stride = 0, j.sw = S.w, j.sh = S.h;
      j.dst_off = D.cur_off, j.dw = D.w, j.dh = D.h;
      jobs.push_back(j);
      lvl_mw[l] = std::max(lvl_mw[l], D.w), lvl_mh[l] = std::max(lvl_mh[l], D.h);
    }
    lvl_jobs[l] = (int) (jobs.size() - lvl_job0[l]);
  }
  const size_t mean_job0 = jobs.size();
  std::vector<size_t> mean_idx;                  // (i, l) of each mean job
  for( int i = 0; i < n; ++i ) {
    for( int l = 0; l < L[i]; ++l ) {
      const RoiLevel & E = R[(size_t) i * lmax + l];
      RaggedImg j;
      j.src_off = E.ref_off, j.src_stride = 0, j.sw = E.w, j.sh = E.h, j.dst_off = 0, j.dw = j.dh = 0;
      jobs.push_back(j);
      mean_idx.push_back((size_t) i * lmax + l);
    }
  }
  SST_RCK(h->jobs.ensure(jobs.size() * sizeof(RaggedImg)));
  SST_RCK(cudaMemcpyAsync(h->jobs.p, jobs.data(), jobs.size() * sizeof(RaggedImg), cudaMemcpyHostToDevice, st));
  const RaggedImg * dj = h->jobs.as<RaggedImg>();
  float gk[64];
  int ks_ref = 0, ks_in = 0;
  if( o.reference_smooth_sigma > 0 ) {
    ks_ref = gaussian_kernel(o.reference_smooth_sigma, gk);
    SST_RCK(h->gk_ref.ensure(64 * sizeof(float)));
    SST_RCK(cudaMemcpyAsync(h->gk_ref.p, gk, ks_ref * sizeof(float), cudaMemcpyHostToDevice, st));
    SST_RCK(cudaStreamSynchronize(st));          // gk is reused below
  }
  if( o.input_smooth_sigma > 0 ) {
    ks_in = gaussian_kernel(o.input_smooth_sigma, gk);
    SST_RCK(h->gk_in.ensure(64 * sizeof(float)));
    SST_RCK(cudaMemcpyAsync(h->gk_in.p, gk, ks_in * sizeof(float), cudaMemcpyHostToDevice, st));
  }
  float * d_refp = h->ref.as<float>(), * d_curp = h->cur.as<float>();
  SST_RLAUNCH(launch_convert_smooth_ragged(d_ref, depth, dj, n, max_w, max_h, scale,
      ks_ref ? h->gk_ref.as<float>() : nullptr, ks_ref, d_refp, st));
  SST_RLAUNCH(launch_convert_smooth_ragged(d_cur, depth, dj + n, n, max_w, max_h, scale,
      ks_in ? h->gk_in.as<float>() : nullptr, ks_in, d_curp, st));
  for( int l = 1; l < lmax; ++l ) {
    if( !lvl_jobs[l] ) continue;
    SST_RLAUNCH(launch_pyrdown_ragged(d_refp, dj + lvl_job0[l], lvl_jobs[l], lvl_mw[l], lvl_mh[l], d_refp, st));
    SST_RLAUNCH(launch_pyrdown_ragged(d_curp, dj + lvl_job0[l], lvl_jobs[l], lvl_mw[l], lvl_mh[l], d_curp, st));
  }
  // reference level means: the numerical shift of the FA sums
  const int nmean = (int) mean_idx.size();
  SST_RCK(h->sums.ensure((size_t) nmean * sizeof(double)));
  SST_RLAUNCH(launch_roi_means(d_refp, dj + mean_job0, nmean, h->sums.as<double>(), st));
  std::vector<double> sums(nmean);
  SST_RCK(cudaMemcpyAsync(sums.data(), h->sums.p, (size_t) nmean * sizeof(double), cudaMemcpyDeviceToHost, st));
  SST_RCK(cudaStreamSynchronize(st));
  for( int k = 0; k < nmean; ++k ) {
    RoiLevel & E = R[mean_idx[k]];
    E.tshift = (float) (sums[k] / ((double) E.w * E.h));
  }
  SST_RCK(cudaMemcpyAsync(h->roi.p, R.data(), R.size() * sizeof(RoiLevel), cudaMemcpyHostToDevice, st));
  SST_RCK(cudaMemcpyAsync(h->ctp.p, ctp.data(), (size_t) (n + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  std::vector<double> init;
  if( init_params ) {
    init.assign((size_t) n * 16, 0.0);
    for( int i = 0; i < n; ++i ) {
      double s[16], p[12];
      model_identity(passes[0], s);
      const int M = model_nparams(passes[0]);
      for( int j = 0; j < M; ++j ) p[j] = init_params[(size_t) i * 12 + j];
      model_set_params(passes[0], s, p);
      for( int j = 0; j < 16; ++j ) init[(size_t) i * 16 + j] = s[j];
    }
    SST_RCK(cudaMemcpyAsync(h->init.p, init.data(), init.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  }

  // ---- the level-synchronous schedule
  if( !h->prof_ready ) {
    for( auto & a : h->prof ) for( auto & b : a ) for( auto & e : b ) SST_RCK(cudaEventCreate(&e));
    h->prof_ready = true;
  }
  const RoiLevel * d_roi = h->roi.as<RoiLevel>();
  FrameState * fs = h->fs.as<FrameState>();
  int * lists = h->lists.as<int>(), * counts = h->counts.as<int>();
  SST_RCK(cudaMemsetAsync(counts, 0, (size_t) steps * sizeof(int), st));
  const int solve_grid = std::max(1, std::min((n + 7) / 8, std::max(1, h->num_sms) * 8));
  int step = 0;
  for( int k_pass = 0; k_pass < num_passes; ++k_pass ) {
    const sst_motion_model & m = passes[k_pass];
    PassBeginArgs pb;
    memset(&pb, 0, sizeof(pb));
    pb.fs = fs, pb.n = n, pb.pass = k_pass, pb.model = m, pb.prev_model = k_pass ? passes[k_pass - 1] : m;
    pb.init_states = (k_pass == 0 && init_params) ? h->init.as<double>() : nullptr;
    pb.roi = d_roi, pb.lmax = lmax;
    SST_RLAUNCH(launch_pass_begin(pb, st));
    for( int l = lmax - 1; l >= 0; --l ) {
      SST_RCK(cudaEventRecord(h->prof[k_pass][l][0], st));
      h->level_step[k_pass][l] = step;
      LevelBeginArgs lb;
      memset(&lb, 0, sizeof(lb));
      lb.fs = fs, lb.n = n, lb.model = m, lb.method = method;
      lb.list_out = lists + (size_t) step * n;
      lb.count_out = counts + step;
      lb.level_is_first = l == lmax - 1;
      lb.roi = d_roi, lb.lmax = lmax, lb.level = l;
      SST_RLAUNCH(launch_level_begin(lb, st));
      PassArgs a;
      memset(&a, 0, sizeof(a));
      a.pyr = d_curp;
      a.refT = d_refp;
      a.fs = fs;
      a.partials = h->part.as<double>();
      a.model = m;
      a.M = model_nparams(m);
      a.max_eps = o.epsx * pow(2.0, l);
      a.step = o.update_step_scale;
      a.max_it = max_it;
      a.roi = d_roi, a.lmax = lmax, a.level = l;
      a.tile_prefix = h->prefix.as<int>();
      a.tile_total = h->total.as<int>();
      for( int it = 0; it <= max_it; ++it ) {
        a.list_in = lists + (size_t) (step + it) * n;
        a.count_in = counts + step + it;
        a.list_out = lists + (size_t) (step + it + 1) * n;
        a.count_out = counts + step + it + 1;
        SST_RLAUNCH(launch_roi_scan(a.list_in, a.count_in, d_roi, lmax, l, h->prefix.as<int>(), h->total.as<int>(), st));
        SST_RLAUNCH(launch_pass(method, a, -1, st));
        SST_RLAUNCH(launch_solve(method, a, solve_grid, st));
      }
      SST_RCK(cudaEventRecord(h->prof[k_pass][l][1], st));
      step += max_it + 2;
    }
  }
  CorrArgs c;
  memset(&c, 0, sizeof(c));
  c.pyr = d_curp;
  c.refT = d_refp;
  c.fs = fs;
  c.n = n;
  c.partials = h->part.as<double>();
  c.model = passes[num_passes - 1];
  c.min_rho = o.min_rho;
  c.roi = d_roi, c.lmax = lmax;
  c.tile_prefix = h->ctp.as<int>();
  SST_RLAUNCH(launch_correlation(c, std::max(1, h->num_sms) * 4, st));
  ++launches;                                    // the correlation finish kernel
  FinalizeArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.fs = fs, fa.n = n, fa.model = passes[num_passes - 1];
  fa.params_out = h->out_params.as<float>();
  fa.status_out = h->out_status.as<int32_t>();
  fa.iters_out = h->out_iters.as<int32_t>();
  fa.eps_out = h->out_eps.as<float>();
  fa.rho_out = h->out_rho.as<float>();
  SST_RLAUNCH(launch_finalize(fa, st));

  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  struct { void * dst; const void * src; size_t bytes; } outs[] = {
    { params_out, h->out_params.p, (size_t) n * 12 * sizeof(float) },
    { status_out, h->out_status.p, (size_t) n * sizeof(int32_t) },
    { iters_out, h->out_iters.p, (size_t) n * sizeof(int32_t) },
    { eps_out, h->out_eps.p, (size_t) n * sizeof(float) },
    { rho_out, h->out_rho.p, (size_t) n * sizeof(float) } };
  for( auto & q : outs ) if( q.dst ) SST_RCK(cudaMemcpyAsync(q.dst, q.src, q.bytes, kind, st));
  if( !on_device ) SST_RCK(cudaStreamSynchronize(st));
  SST_RCK(cudaEventRecord(h->ev_done, st));
  SST_RCK(cudaStreamWaitEvent((cudaStream_t) stream, h->ev_done, 0));
  sst_internal_count_launches(launches);
  h->h_roi.swap(R);
  h->n = n, h->lmax = lmax, h->num_passes = num_passes, h->max_it = max_it, h->method = method;
  return SST_OK;
}

/* Per-level timing of the last call, the frame-iterations it executed and
 * their algorithmic bytes (8 B per pixel and frame-iteration: the warped
 * source and the template; gradients are recomputed on chip). */
extern "C" int sst_roi_batch_level_stats(sst_roi_batch * h, int pass, int level, float * ms,
    double * frame_iterations, double * pixel_iterations, double * algorithmic_bytes)
{
  if( !h || !h->prof_ready || pass < 0 || pass >= h->num_passes || level < 0 || level >= h->lmax )
    return rfail(SST_ERR_INVALID_ARG, "sst_roi_batch_level_stats: invalid arguments");
  SST_RCK(cudaStreamSynchronize(h->st));
  float t = 0;
  SST_RCK(cudaEventElapsedTime(&t, h->prof[pass][level][0], h->prof[pass][level][1]));
  const int s0 = h->level_step[pass][level], ns = h->max_it + 1;
  std::vector<int> c(ns);
  SST_RCK(cudaMemcpy(c.data(), h->counts.as<int>() + s0, (size_t) ns * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> list((size_t) h->n);
  double fi = 0, px = 0;
  for( int k = 0; k < ns; ++k ) {
    if( !c[k] ) continue;
    SST_RCK(cudaMemcpy(list.data(), h->lists.as<int>() + (size_t) (s0 + k) * h->n, (size_t) c[k] * sizeof(int),
        cudaMemcpyDeviceToHost));
    fi += c[k];
    for( int q = 0; q < c[k]; ++q ) {
      const RoiLevel & E = h->h_roi[(size_t) list[q] * h->lmax + level];
      px += (double) E.w * E.h;
    }
  }
  if( ms ) *ms = t;
  if( frame_iterations ) *frame_iterations = fi;
  if( pixel_iterations ) *pixel_iterations = px;
  if( algorithmic_bytes ) *algorithmic_bytes = 8.0 * px;
  return SST_OK;
}
