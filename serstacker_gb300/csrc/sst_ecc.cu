/*
 * sst_ecc.cu -- batched ECC Gauss-Newton passes for sm_103a.
 *
 * One launch = one Gauss-Newton step of every frame still iterating at the
 * current level. Per pixel the kernels evaluate W(x;p), sample the frame's
 * pyramid level bilinearly, form the residual and accumulate the
 * steepest-descent projections in FP32 registers; CTAs reduce in FP64 and the
 * last CTA of a frame runs the reference's per-iteration logic in FP64:
 *
 *   IC    c_ecc_inverse_compositional::align   ecc2.cc:1693-1788
 *   IC-LM c_ecclm_inverse_compositional::align ecc2.cc:1926-2086
 *   FA    c_ecc_forward_additive::align        ecc2.cc:1247-1365
 *   LM    c_ecclm::align                       ecc2.cc:1528-1650
 *
 * followed, when a frame leaves a level, by c_ecch::align's rescale to the
 * next finer level (ecc2.cc:1159-1171: only after a successful level).
 *
 * Fusions relative to the reference: the remap, the mask remap + threshold,
 * the residual, the steepest-descent images and the Hessian / projection dot
 * products of one iteration are one pass over the level (the reference makes
 * M(M+1)/2 + M full-image passes); an LM / IC-LM trial evaluation also
 * produces the Jacobian products at the trial point, which the reference
 * recomputes after accepting it (identical values).
 */
#include "sst_engine.cuh"
#include "sst_kernels.cuh"
#include "sst_tma.cuh"
#include <float.h>

namespace sst {

/* ------------------------------------------------------- tile bookkeeping */

/* Deterministic combine of a frame's tile partials: thread group g sums tiles
 * g, g+G, ... of sum k; the G group results are added in order. */
__device__ void combine_partials(const double * P, int tiles, int NS, double * tmp, double * out)
{
  const int G = (256 / NS) > 0 ? (256 / NS) : 1;
  const int tid = threadIdx.x;
  if( tid < NS * G ) {
    const int k = tid % NS, g = tid / NS;
    double s = 0;
    for( int t = g; t < tiles; t += G ) s += __ldcg(P + (size_t) t * NS + k);
    tmp[tid] = s;
  }
  __syncthreads();
  if( tid < NS ) {
    double s = 0;
    for( int g = 0; g < G; ++g ) s += tmp[g * NS + tid];
    out[tid] = s;
  }
  __syncthreads();
}

/* Tile reduction: FP32 warp shuffles (32 lanes x a few pixels each), then
 * the 8 warp sums added in FP64 in a fixed order (GB300's FP64 rate is a
 * small fraction of FP32: keep it off the per-thread path). */
template<int NS>
__device__ __forceinline__ void block_reduce_d(const float (&acc)[NS], float * scratch, double * out)
{
  warp_sums_to<NS>(acc, scratch + (threadIdx.x >> 5) * NS);
  __syncthreads();
  for( int k = threadIdx.x; k < NS; k += 256 ) {
    double t = 0;
#pragma unroll
    for( int wv = 0; wv < 8; ++wv ) t += (double) scratch[wv * NS + k];
    out[k] = t;
  }
  __syncthreads();
}

/* Store one tile's sums; the frame's solve kernel combines them after the
 * launch (the kernel boundary orders the stores before the loads). */
template<int NS>
__device__ __forceinline__ void write_tile(const PassArgs & a, int f, int t, const double * tile_sums)
{
  if( threadIdx.x < NS ) a.partials[(size_t) f * a.part_stride + (size_t) t * NS + threadIdx.x] = tile_sums[threadIdx.x];
}

template<int NS>
__device__ __forceinline__ void write_tile_at(double * base, int t, const double * tile_sums)
{
  if( threadIdx.x < NS ) base[(size_t) t * NS + threadIdx.x] = tile_sums[threadIdx.x];
}

/* ROI batches: entry k of the active list that owns work index `item`
 * (largest k with prefix[k] <= item; prefix is strictly increasing) */
__device__ __forceinline__ int roi_entry(const int * prefix, int count, int item)
{
  int lo = 0, hi = count - 1;
  while ( lo < hi ) {
    const int mid = (lo + hi + 1) >> 1;
    if( __ldcg(prefix + mid) <= item ) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

/* ------------------------------------------------------ per-frame control */

__device__ void set_eval(FrameState * F, const sst_motion_model & m, const double * s)
{
  for( int i = 0; i < 16; ++i ) F->eval[i] = s[i];
  model_warp_coeffs(m, s, F->wc);
  model_sd_coeffs(m, s, F->jc);
}

__device__ bool state_finite(const double * s, int n)
{
  for( int i = 0; i < n; ++i ) if( !isfinite(s[i]) ) return false;
  return true;
}

/* c_ecch::align per-level epilogue (ecc2.cc:1159-1173) */
__device__ void level_finish(FrameState * F, const PassArgs & a, bool ok)
{
  F->level_ok = ok;
  F->total_iters += F->n;
  if( !state_finite(F->state, 16) ) {
    F->status = SST_FRAME_NAN;
    ok = false;
  }
  if( ok && a.scale_next > 0 ) model_scale(a.model, F->state, a.scale_next);
  set_eval(F, a.model, F->state);
}

__device__ void append(const PassArgs & a, int f)
{
  const int k = atomicAdd(a.count_out, 1);
  a.list_out[k] = f;
}

/* IC: ecc2.cc:1740-1785 */
__device__ void solve_ic(FrameState * F, const double * S, const PassArgs & a, int f)
{
  const int M = a.M;
  F->n += 1;
  const double cnt = S[M + 1];
  if( !(cnt > 0) ) {
    F->status = SST_FRAME_EMPTY_MASK;
    level_finish(F, a, false);
    return;
  }
  const double q = a.RMA / cnt;
  const double rmsnew = S[M] * q * q;
  double b[12], x[12];
  for( int j = 0; j < M; ++j ) b[j] = S[j] * q;
  if( a.Hinv ) {
    // the IC matrix is constant per level: its inverse (FP64 Cholesky on the host) replaces the solve
    for( int i = 0; i < M; ++i ) {
      double t = 0;
      for( int j = 0; j < M; ++j ) t += a.Hinv[i * M + j] * b[j];
      x[i] = t;
    }
  }
  else if( !cholesky_solve(a.H, b, M, x) ) for( int j = 0; j < M; ++j ) x[j] = 0;
  if( rmsnew >= F->rmsold ) {
    level_finish(F, a, true);
    return;
  }
  double sdp[12], ns[16];
  for( int j = 0; j < M; ++j ) sdp[j] = a.step * x[j];
  model_invert_and_compose(a.model, F->state, sdp, ns);
  for( int i = 0; i < 16; ++i ) F->state[i] = ns[i];
  F->rmsold = rmsnew;
  F->eps = model_eps(a.model, F->state, x, a.w, a.h);
  if( F->eps < a.max_eps ) {
    level_finish(F, a, true);
    return;
  }
  if( F->n >= a.max_it ) {
    F->n += 1;   // the failing `_num_iterations++ < _max_iterations` test
    level_finish(F, a, true);
    return;
  }
  set_eval(F, a.model, F->state);
  append(a, f);
}

/* IC-LM: ecc2.cc:1983-2083 as a state machine over pass results */
__device__ void solve_iclm(FrameState * F, const double * S, const PassArgs & a, int f)
{
  const int M = a.M;
  const double cnt = S[M + 1];
  if( !(cnt > 0) ) {
    F->status = SST_FRAME_EMPTY_MASK;
    level_finish(F, a, false);
    return;
  }
  const double q = a.RMA / cnt;
  const double rms = S[M] * q * q;
  double vv[12];
  for( int j = 0; j < M; ++j ) vv[j] = S[j] * q;

  bool go_after = false;
  double newerr = 0;
  if( F->phase == PH_START ) {
    F->err = rms;
    for( int j = 0; j < M; ++j ) F->v[j] = vv[j];
  }
  else {
    newerr = rms;
    F->dpe = model_eps(a.model, F->state, F->dpv, a.w, a.h);
    if( F->dpe < a.max_eps ) go_after = true;
    else {
      double dS = 0;
      for( int i = 0; i < M; ++i ) {
        double t = 2 * F->v[i];
        for( int j = 0; j < M; ++j ) t -= a.H[i * M + j] * F->dpv[j];
        dS += F->dpv[i] * t;
      }
      const double rho = (F->err - newerr) / (fabs(dS) > DBL_EPSILON ? dS : 1.0);
      if( rho > 0.25 ) {
        if( F->lambda > 1e-6 ) F->lambda = fmax(1e-6, F->lambda / 5);
      }
      else if( rho > 0.1 ) {
      }
      else if( F->lambda < 1 ) F->lambda = 1;
      else F->lambda *= 10;
      if( newerr < F->err ) go_after = true;
      else if( !(F->n < a.max_it) ) go_after = true;
    }
    if( go_after ) {
      if( newerr < F->err ) {
        F->err = newerr;
        for( int i = 0; i < 16; ++i ) F->state[i] = F->eval[i];
        for( int j = 0; j < M; ++j ) F->v[j] = vv[j];
      }
      if( F->dpe < a.max_eps || !(F->n < a.max_it) ) {
        F->eps = F->dpe;
        level_finish(F, a, true);
        return;
      }
    }
  }
  // do { ... } body: damped solve and the next trial point
  F->n += 1;
  double H[144], x[12];
  for( int i = 0; i < M * M; ++i ) H[i] = a.H[i];
  for( int i = 0; i < M; ++i ) H[i * M + i] = (1 + F->lambda) * a.H[i * M + i];
  if( !cholesky_solve(H, F->v, M, x) ) for( int j = 0; j < M; ++j ) x[j] = 0;
  for( int j = 0; j < M; ++j ) F->dpv[j] = x[j];
  double sdp[12], ns[16];
  for( int j = 0; j < M; ++j ) sdp[j] = a.step * x[j];
  model_invert_and_compose(a.model, F->state, sdp, ns);
  F->phase = PH_TRIAL;
  set_eval(F, a.model, ns);
  append(a, f);
}

/* FA: ecc2.cc:1295-1360. Sum layout: H (packed lower), SJg, SJf, SJ, Sf, Sf2, Sg, Sg2, n */
__device__ void solve_fa(FrameState * F, const double * S, const PassArgs & a, int f)
{
  const int M = a.M, nH = M * (M + 1) / 2;
  F->n += 1;
  const double * SJg = S + nH, * SJf = S + nH + M, * SJ = S + nH + 2 * M;
  const double Sf = S[nH + 3 * M], Sf2 = S[nH + 3 * M + 1], Sg = S[nH + 3 * M + 2], Sg2 = S[nH + 3 * M + 3];
  const double cnt = S[nH + 3 * M + 4];
  if( !(cnt > 0) ) {
    F->status = SST_FRAME_EMPTY_MASK;
    level_finish(F, a, false);
    return;
  }
  const double fm = Sf / cnt, gm = Sg / cnt;
  const double fs = sqrt(fmax(Sf2 / cnt - fm * fm, 0.0)), gs = sqrt(fmax(Sg2 / cnt - gm * gm, 0.0));
  const double r = gs / fs;
  double H[144], ep[12], x[12];
  for( int i = 0, k = 0; i < M; ++i ) {
    for( int j = 0; j <= i; ++j, ++k ) H[i * M + j] = H[j * M + i] = S[k];
  }
  for( int j = 0; j < M; ++j ) ep[j] = SJg[j] - r * SJf[j] - (gm - r * fm) * SJ[j];
  if( !cholesky_solve(H, ep, M, x) ) {
    level_finish(F, a, false);   // _failed = true: align() returns false, no rescale
    return;
  }
  double p[12], dp[12];
  model_get_params(a.model, F->state, p);
  for( int j = 0; j < M; ++j ) {
    dp[j] = -a.step * x[j];
    p[j] += dp[j];
  }
  model_set_params(a.model, F->state, p);
  F->eps = model_eps(a.model, F->state, dp, a.w, a.h);
  const double max_eps = a.max_eps > 0 ? a.max_eps : 1e-3;
  if( F->eps < max_eps ) {
    level_finish(F, a, true);
    return;
  }
  if( F->n >= a.max_it ) {
    F->n += 1;
    level_finish(F, a, true);
    return;
  }
  set_eval(F, a.model, F->state);
  append(a, f);
}

/* LM: ecc2.cc:1564-1646. Sum layout: H (packed lower), v, ssq, n */
__device__ void solve_lm(FrameState * F, const double * S, const PassArgs & a, int f)
{
  const int M = a.M, nH = M * (M + 1) / 2;
  const double ssq = S[nH + M];
  enum { OUTER, INNER } next;
  if( F->phase == PH_START ) {
    F->err = ssq;
    for( int i = 0, k = 0; i < M; ++i ) for( int j = 0; j <= i; ++j, ++k ) F->Hs[i * M + j] = F->Hs[j * M + i] = S[k];
    for( int j = 0; j < M; ++j ) F->v[j] = S[nH + j];
    next = OUTER;
  }
  else {
    const double newerr = ssq;
    if( newerr > F->err ) {
      if( F->lambda > 1e6 ) next = OUTER;     // no convergence at this lambda: back to the outer loop
      else {
        F->lambda *= 10.0;
        next = INNER;
      }
    }
    else {
      // accept: the trial point becomes the state; its Jacobian products are the new H, v
      for( int i = 0; i < 16; ++i ) F->state[i] = F->eval[i];
      const double diff = F->err - newerr;
      double dS = 0;
      for( int i = 0; i < M; ++i ) {
        double t = 2 * F->v[i];
        for( int j = 0; j < M; ++j ) t -= F->Hs[i * M + j] * F->dpv[j];
        dS += F->dpv[i] * t;
      }
      const double err_old = F->err;
      F->err = newerr;
      for( int i = 0, k = 0; i < M; ++i ) for( int j = 0; j <= i; ++j, ++k ) F->Hs[i * M + j] = F->Hs[j * M + i] = S[k];
      for( int j = 0; j < M; ++j ) F->v[j] = S[nH + j];
      if( diff < err_old * 1e-4 ) {
        F->converged = 1;
        level_finish(F, a, true);
        return;
      }
      const double rho = fabs(dS) > 1e-9 ? diff / fabs(dS) : diff;
      if( rho > 0.25 ) F->lambda = fmax(1e-8, 0.2 * F->lambda);
      else if( rho < 0.1 ) F->lambda = F->lambda < 1.0 ? 1.0 : F->lambda * 10.0;
      next = OUTER;
    }
  }
  if( next == OUTER ) {
    if( !(F->n < a.max_it) ) {
      level_finish(F, a, F->converged != 0);
      return;
    }
    if( F->err < 1 ) {
      F->converged = 1;
      level_finish(F, a, true);
      return;
    }
  }
  // inner loop head: while (iteration++ < max_iterations)
  if( !(F->n < a.max_it) ) {
    F->n += 1;
    level_finish(F, a, F->converged != 0);
    return;
  }
  F->n += 1;
  double H[144], x[12], p[12];
  for( int i = 0; i < M * M; ++i ) H[i] = F->Hs[i];
  for( int i = 0; i < M; ++i ) H[i * M + i] = (1 + F->lambda) * F->Hs[i * M + i];
  if( !cholesky_solve(H, F->v, M, x) ) for( int j = 0; j < M; ++j ) x[j] = 0;
  for( int j = 0; j < M; ++j ) F->dpv[j] = x[j];
  model_get_params(a.model, F->state, p);
  for( int j = 0; j < M; ++j ) p[j] -= a.step * x[j];
  F->eps = model_eps(a.model, F->state, x, a.w, a.h);
  double ns[16];
  for( int i = 0; i < 16; ++i ) ns[i] = F->state[i];
  model_set_params(a.model, ns, p);
  if( F->eps <= a.max_eps ) {
    for( int i = 0; i < 16; ++i ) F->state[i] = ns[i];
    F->converged = 1;
    level_finish(F, a, true);
    return;
  }
  F->phase = PH_TRIAL;
  set_eval(F, a.model, ns);
  append(a, f);
}

/* ------------------------------------------------------ pointwise passes */

/* IC / IC-LM pass: sums {J^T r (M), |r|^2, count}, J from the reference gradients */
/* Number of per-thread column partials the identity-warp steepest-descent
 * projection needs. Each thread owns one column x, so with u = gx r and
 * w = gy r the projections factor into x-free sums:
 *   translation  U, W
 *   euclidean    U, W, Uy            (+ Wy when the scale is free)
 *   affine       U, W, Uy, Wy
 *   homography   U, W, Uy, Wy, Wyy
 * where Uy = sum y u, Wy = sum y w, Wyy = sum y^2 w. */
template<int JK, int M>
struct column_sums {
  static constexpr int N = JK == J_TRANS ? 2 : JK == J_EUCL ? (M > 3 ? 4 : 3) : JK == J_AFFINE ? 4 : 5;
};

/* J^T r at the identity warp from the column partials (c_image_transform.cc SD formulas
 * with the identity parameters): P = {U, W, Uy, Wy, Wyy} */
template<int JK, int M>
__device__ __forceinline__ void column_project(const float * P, float x, float * acc)
{
  const float U = P[0], W = P[1];
  if( JK == J_TRANS ) {
    acc[0] = U, acc[1 < M ? 1 : 0] = W;
  }
  else if( JK == J_EUCL ) {
    const float Uy = P[2];
    acc[0] = U, acc[1] = W;
    acc[2 < M ? 2 : 0] = fmaf(x, W, -Uy);                 // -gx y + gy x
    if( M > 3 ) acc[3 < M ? 3 : 0] = fmaf(x, U, P[3 < column_sums<JK, M>::N ? 3 : 0]);   // gx x + gy y
  }
  else if( JK == J_AFFINE ) {
    const float Uy = P[2], Wy = P[3];
    acc[0] = x * U, acc[1] = Uy, acc[2] = U;
    acc[3 < M ? 3 : 0] = x * W, acc[4 < M ? 4 : 0] = Wy, acc[5 < M ? 5 : 0] = W;
  }
  else {
    const float Uy = P[2], Wy = P[3], Wyy = P[4 < column_sums<JK, M>::N ? 4 : 0];
    acc[0] = x * U, acc[1] = Uy, acc[2] = U;
    acc[3 < M ? 3 : 0] = x * W, acc[4 < M ? 4 : 0] = Wy, acc[5 < M ? 5 : 0] = W;
    acc[6 < M ? 6 : 0] = -x * fmaf(x, U, Wy);             // -x (x u + y w)
    acc[7 < M ? 7 : 0] = -fmaf(x, Uy, Wyy);               // -y (x u + y w)
  }
}

/* IC / IC-LM pass: sums {J^T r (M), |r|^2, count}, J = steepest-descent images of
 * the reference at the identity warp */
/* IC / IC-LM pass: sums {J^T r (M), |r|^2, count}, J = steepest-descent images of
 * the reference at the identity warp. When every tap of a tile is inside the
 * level (warp-uniform corner test) the taps are gathered without the
 * coverage / mask / border logic. */
template<int METHOD, int FAM, int JK, int M>
__global__ void __launch_bounds__(256, 5) k_pass_pointwise(PassArgs a)
{
  constexpr int NS = M + 2;
  constexpr int NP = column_sums<JK, M>::N;
  __shared__ float s_red[8 * NS];
  __shared__ double s_tile[NS];
  __shared__ float s_c[16];

  const int nitems = __ldcg(a.count_in) * a.tiles;
  for( int item = blockIdx.x; item < nitems; item += gridDim.x ) {
    const int fi = item / a.tiles;
    const int t = item - fi * a.tiles;
    const int f = __ldcg(a.list_in + fi);
    const FrameState * F = a.fs + f;
    if( threadIdx.x < 16 ) s_c[threadIdx.x] = F->wc[threadIdx.x];
    __syncthreads();
    float c[16];
#pragma unroll
    for( int i = 0; i < 16; ++i ) c[i] = s_c[i];
    const float * img = a.pyr + (size_t) f * a.pyr_stride + a.lvl_off;
    const int tx0 = (t % a.tiles_x) * PW_TX, ty0 = (t / a.tiles_x) * PW_TY;
    const int x = tx0 + (threadIdx.x & (PW_TX - 1));
    const int yend = min(ty0 + PW_TY, a.h);
    // warm L2 with the source footprint of this CTA's next item (its taps otherwise come from DRAM)
    if( item + (int) gridDim.x < nitems ) {
      const int nitem = item + gridDim.x;
      const int nfi = nitem / a.tiles, nt = nitem - nfi * a.tiles;
      const int nf = __ldcg(a.list_in + nfi);
      const float * nw = a.fs[nf].wc;
      const int nx0 = (nt % a.tiles_x) * PW_TX, ny0 = (nt / a.tiles_x) * PW_TY;
      const int row = threadIdx.x >> 2;                 // 64 rows, 4 lines of 32 floats per row
      if( row < PW_TY ) {
        const int y = min(ny0 + row, a.h - 1);
        const int x = min(nx0 + (threadIdx.x & 3) * 32, a.w - 1);
        const float dx = fmaf(__ldg(nw + 0), (float) x, fmaf(__ldg(nw + 1), (float) y, __ldg(nw + 2)));
        const float dy = fmaf(__ldg(nw + 3), (float) x, fmaf(__ldg(nw + 4), (float) y, __ldg(nw + 5)));
        const int sx = clampi(x + (int) __ldg(nw + 12) + (int) floorf(dx), 0, a.w - 1);
        const int sy = clampi(y + (int) __ldg(nw + 13) + (int) floorf(dy), 0, a.h - 1);
        const float * p = a.pyr + (size_t) nf * a.pyr_stride + a.lvl_off + (size_t) sy * a.w + sx;
        asm volatile("prefetch.global.L2 [%0];" :: "l"(p));
      }
    }
    float P[NP], rr = 0.f, cnt = 0.f;
#pragma unroll
    for( int k = 0; k < NP; ++k ) P[k] = 0.f;
    // each warp owns a 32-column strip (one row parity); the interior test runs per
    // 16-row chunk of the strip, so only chunks near the level border take the
    // coverage / mask / border path
    const int xs0 = tx0 + (threadIdx.x & (PW_TX - 1) & ~31);
    const int xs1 = min(xs0 + 31, a.w - 1);
    const float fx = (float) x;
    for( int yc = ty0; yc < yend; yc += 16 ) {
      const int yc1 = min(yc + 15, yend - 1);
      const bool interior = (METHOD == M_IC || !a.refM) && xs0 < a.w &&
          rect_interior<FAM>(c, xs0, yc, xs1, yc1, a.w, a.h);
      if( x >= a.w ) continue;
      if( interior ) {
        // every tap is inside the level: no clamps, 32-bit offsets, the pixel
        // count known in advance, the row coordinate carried in FP32
        const int y0r = yc + (threadIdx.x >> 7);
        if( y0r <= yc1 ) cnt += (float) ((yc1 - y0r) / 2 + 1);
        const int xI = x + (int) c[12], yI = (int) c[13];
        const float fx = (float) x;
        const float4 * tgp = a.refTG + (size_t) y0r * a.w + x;
        float fy = (float) y0r;
#pragma unroll 4
        for( int y = y0r; y <= yc1; y += 2, fy += 2.f, tgp += 2 * a.w ) {
          float dx, dy;
          warp_disp<FAM>(c, fx, fy, dx, dy);
          const float flx = floorf(dx), fly = floorf(dy);
          const float ax = dx - flx, ay = dy - fly;
          const float * r0 = img + ((y + yI + (int) fly) * a.w + xI + (int) flx);
          const float v00 = __ldg(r0), v01 = __ldg(r0 + 1), v10 = __ldg(r0 + a.w), v11 = __ldg(r0 + a.w + 1);
          const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
          const float4 tg = __ldg(tgp);
          const float r = fmaf(ay, t1 - t0, t0) - tg.x;
          const float u = tg.y * r, w = tg.z * r;
          rr = fmaf(r, r, rr);
          P[0] += u, P[1] += w;
          if( NP > 2 ) P[2 < NP ? 2 : 0] = fmaf(fy, u, P[2 < NP ? 2 : 0]);
          if( NP > 3 ) P[3 < NP ? 3 : 0] = fmaf(fy, w, P[3 < NP ? 3 : 0]);
          if( NP > 4 ) P[4 < NP ? 4 : 0] = fmaf(fy * fy, w, P[4 < NP ? 4 : 0]);
        }
      }
      else {
#pragma unroll 2
        for( int y = yc + (threadIdx.x >> 7); y <= yc1; y += 2 ) {
          const spos s = warp_pos<FAM>(c, x, y);
          const size_t i = (size_t) y * a.w + x;
          bool ok;
          if( METHOD == M_IC ) {
            ok = mask_ok(coverage(a.w, a.h, s), 250);
          }
          else {
            int rx, ry;
            warp_nearest<FAM>(c, x, y, rx, ry);
            ok = rx >= 0 && rx < a.w && ry >= 0 && ry < a.h;
            if( a.refM ) ok = ok && __ldg(a.refM + i) != 0;
          }
          const float v = sample_replicate(img, a.w, a.h, s);
          const float4 tg = __ldg(a.refTG + i);
          const float r = ok ? v - tg.x : 0.f;
          const float fy = (float) y;
          const float u = tg.y * r, w = tg.z * r;
          rr = fmaf(r, r, rr);
          cnt += ok ? 1.f : 0.f;
          P[0] += u, P[1] += w;
          if( NP > 2 ) P[2 < NP ? 2 : 0] = fmaf(fy, u, P[2 < NP ? 2 : 0]);
          if( NP > 3 ) P[3 < NP ? 3 : 0] = fmaf(fy, w, P[3 < NP ? 3 : 0]);
          if( NP > 4 ) P[4 < NP ? 4 : 0] = fmaf(fy * fy, w, P[4 < NP ? 4 : 0]);
        }
      }
    }
    (void) fx;
    float acc[NS];
#pragma unroll
    for( int k = 0; k < NS; ++k ) acc[k] = 0.f;
    if( x < a.w ) column_project<JK, M>(P, (float) x, acc);
    acc[M] = rr;
    acc[M + 1] = cnt;
    block_reduce_d<NS>(acc, s_red, s_tile);
    write_tile<NS>(a, f, t, s_tile);
  }
}

/* ------------------------------------------- TMA-staged pointwise pass */

/* source footprint box of one 128 x 32 tile (floats): x origin a multiple of 4 */
constexpr int PB_W = 144, PB_H = 40;

struct ItemPlan {
  int f, t;         // frame and tile of the item
  int use;          // 1: the footprint box is staged (every tap of the tile lies in it)
  int inside;       // 1: every tap inside the level as well (no per-pixel border test)
  int bx0, by0;     // box origin in the level
};

/* Plans one work item (warp 0) from values loaded an item earlier, so that
 * the plan waits on no memory: the item's frame f and, in lane l, coefficient
 * l & 15 of that frame. Writes the coefficients (s_c) and whether the item's
 * footprint is staged. */
template<int METHOD, int FAM, int TXS>
__device__ __forceinline__ void plan_item(const PassArgs & a, int item, int f, float cl, float * s_c, ItemPlan * plan)
{
  constexpr int BW = TXS + 16;
  const int lane = threadIdx.x & 31;
  const int t = item - (item / a.tiles) * a.tiles;
  float c[16];
#pragma unroll
  for( int i = 0; i < 16; ++i ) c[i] = __shfl_sync(0xffffffffu, cl, i);
  if( lane < 16 ) s_c[lane] = cl;
  const int tx0 = (t % a.tiles_x) * TXS, ty0 = (t / a.tiles_x) * PW_TY;
  const int tx1 = min(tx0 + TXS, a.w) - 1, ty1 = min(ty0 + PW_TY, a.h) - 1;
  int bx0, by0, bx1, by1;
  bool inside;
  bool use = rect_box<FAM>(c, tx0, ty0, tx1, ty1, a.w, a.h, bx0, by0, bx1, by1, inside);
  use = use && (METHOD == M_IC || !a.refM);
  if( use ) {
    bx0 = bx0 >= 0 ? bx0 & ~3 : -((-bx0 + 3) & ~3);
    use = bx1 < bx0 + BW && by1 < by0 + PB_H;
  }
  if( lane == 0 ) {
    plan->f = f, plan->t = t;
    plan->use = use ? 1 : 0;
    plan->inside = inside ? 1 : 0;
    plan->bx0 = bx0, plan->by0 = by0;
  }
}

/* frame of work item `item` (active-list entry item / tiles), or 0 past the end */
__device__ __forceinline__ int item_frame(const PassArgs & a, int item, int nitems)
{
  return item < nitems ? __ldcg(a.list_in + item / a.tiles) : 0;
}

/* FP64 sum, in warp order, of the 8 warp sums of an item (lanes < NS of
 * one warp) stored as that item's tile partials */
template<int NS, int NW = 8>
__device__ __forceinline__ void store_item_sums(const PassArgs & a, int f, int t, const float * scratch)
{
  const int lane = threadIdx.x & 31;
  if( lane < NS ) {
    double s = 0;
#pragma unroll
    for( int wv = 0; wv < NW; ++wv ) s += (double) scratch[wv * NS + lane];
    a.partials[(size_t) f * a.part_stride + (size_t) t * NS + lane] = s;
  }
}

/* The IC / IC-LM pass with each item's source footprint staged in shared
 * memory by one TMA copy, double-buffered across the CTA's consecutive items:
 * the gathers become shared-memory loads with no address arithmetic in
 * 64 bits, and the next item's copy is in flight while this one computes.
 * Items whose taps leave the level or the box take the global path. */
// The projective pass runs 128 threads per CTA (four CTAs per SM, shared memory
// bound): each thread takes twice the samples per item, so the per-item plan,
// barrier and reduction weigh half as much, and the registers the projective
// positions need fit without spills. The affine pass keeps 256 (its occupancy
// matters more).
template<int FAM>
__host__ __device__ constexpr int pw_threads() { return FAM == FAM_HOMOG ? 128 : 256; }

template<int METHOD, int FAM, int JK, int M, int TXS>
__global__ void __launch_bounds__(pw_threads<FAM>(), 4) k_pass_pointwise_tma(PassArgs a, const __grid_constant__ CUtensorMap tmap)
{
  constexpr int NS = M + 2;
  constexpr int NP = column_sums<JK, M>::N;
  constexpr int NT = pw_threads<FAM>(), NW = NT / 32;
  constexpr int PB_W = TXS + 16;                    // footprint box width (tile + 16 px)
  constexpr int RS = NT / TXS;                      // rows between a thread's samples
  constexpr int RSH = TXS == 128 ? 7 : 6;           // log2 TXS
  __shared__ __align__(128) float s_box[2][PB_H * PB_W];
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ float s_red[2][NW * NS];    // warp sums of the current and the previous item
  __shared__ float s_c[3][16];
  __shared__ ItemPlan s_plan[3];
  __shared__ uint32_t s_infl;             // copies in flight, kept by thread 0
  __shared__ int s_gaveup[2];             // a wait gave up during an item of this buffer parity

  const int count = __ldcg(a.count_in);
  const int nitems = count * a.tiles;
  if( (int) blockIdx.x >= nitems ) return;          // uniform over the CTA
  if( threadIdx.x == 0 ) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    s_infl = 0u;
    s_gaveup[0] = s_gaveup[1] = 0;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  // warp 0 keeps the frame of the item after next (f2) and the frame and lane
  // coefficient of the next item (f1, c1) in flight one item ahead of their use
  int f1 = 0, f2 = 0;
  float c1 = 0.f;
  if( threadIdx.x < 32 ) {
    const int lane = threadIdx.x & 31;
    const int f0 = item_frame(a, blockIdx.x, nitems);
    plan_item<METHOD, FAM, TXS>(a, blockIdx.x, f0, __ldcg(a.fs[f0].wc + (lane & 15)), s_c[0], &s_plan[0]);
    f1 = item_frame(a, blockIdx.x + gridDim.x, nitems);
    c1 = __ldcg(a.fs[f1].wc + (lane & 15));
    f2 = item_frame(a, blockIdx.x + 2 * gridDim.x, nitems);
  }
  __syncthreads();
  if( threadIdx.x == 0 && s_plan[0].use ) {
    mbar_expect_tx(&s_bar[0], PB_W * PB_H * sizeof(float));
    tma_load_3d(s_box[0], &tmap, s_plan[0].bx0, s_plan[0].by0, s_plan[0].f, &s_bar[0]);
    inflight_issued(&s_infl, 0, 0u);
  }
  uint32_t phases = 0u;
  bool timed_out = false, stop = false;
  int slot = 0, b = 0;
  int pf = -1, pt = 0;                              // previous item (its sums wait in s_red[b ^ 1])
  for( int item = blockIdx.x; item < nitems; item += gridDim.x, b ^= 1 ) {
    const int nitem = item + gridDim.x;
    const int nslot = slot == 2 ? 0 : slot + 1;
    if( threadIdx.x < 32 && nitem < nitems ) {
      plan_item<METHOD, FAM, TXS>(a, nitem, f1, c1, s_c[nslot], &s_plan[nslot]);
      if( nitem + gridDim.x < nitems ) c1 = __ldcg(a.fs[f2].wc + (threadIdx.x & 15));
      f1 = f2;
      f2 = item_frame(a, nitem + 2 * gridDim.x, nitems);
    }
    // orders: the next plan; the previous item's warp sums; the previous item's
    // reads of the box buffer that the next copy overwrites
    __syncthreads();
    // once a wait gave up no further copy is issued or consumed; the previous item's
    // flag is read after the barrier and written again no earlier than the next item,
    // so every thread sees the same value
    stop = stop || s_gaveup[b ^ 1];
    if( threadIdx.x == 0 && nitem < nitems && s_plan[nslot].use && !stop ) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&s_bar[b ^ 1], PB_W * PB_H * sizeof(float));
      tma_load_3d(s_box[b ^ 1], &tmap, s_plan[nslot].bx0, s_plan[nslot].by0, s_plan[nslot].f, &s_bar[b ^ 1]);
      inflight_issued(&s_infl, b ^ 1, (phases >> (b ^ 1)) & 1u);
    }
    if( pf >= 0 && (threadIdx.x >> 5) == 1 ) store_item_sums<NS, NW>(a, pf, pt, s_red[b ^ 1]);
    const ItemPlan pl = s_plan[slot];
    pf = pl.f, pt = pl.t;
    float c[16];
#pragma unroll
    for( int i = 0; i < 16; ++i ) c[i] = s_c[slot][i];
    slot = nslot;
    const int f = pl.f, t = pl.t;
    const float * img = a.pyr + (size_t) f * a.pyr_stride + a.lvl_off;
    const int tx0 = (t % a.tiles_x) * TXS, ty0 = (t / a.tiles_x) * PW_TY;
    const int x = tx0 + (threadIdx.x & (TXS - 1));
    const int yend = min(ty0 + PW_TY, a.h);
    float P[NP], rr = 0.f, cnt = 0.f;
#pragma unroll
    for( int k = 0; k < NP; ++k ) P[k] = 0.f;
    if( pl.use && !stop ) {
      if( !mbar_wait_bounded(&s_bar[b], (phases >> b) & 1u) ) timed_out = true, s_gaveup[b] = 1;
      else if( threadIdx.x == 0 ) inflight_landed(&s_infl, b);
      phases ^= 1u << b;
      if( x < a.w ) {
        const float * box = s_box[b];
        const int y0r = ty0 + (threadIdx.x >> RSH);
        // The column's sample positions as functions of the tile-local row tr = y - ty0,
        // in box coordinates: (Kx, Ky) is the integer offset of (x + Ix, ty0 + Iy) from
        // the box origin, the warp's displacement is added to it. Box coordinates are
        // positive (footprint test), so truncation is the floor.
        const float fx = (float) x, fty0 = (float) ty0;
        const float Kx = (float) (x + (int) c[12] - pl.bx0), Ky = (float) (ty0 + (int) c[13] - pl.by0);
        float e0, e1, e2, e3, e4, e5, e6;
        if( FAM == FAM_AFFINE ) {
          e0 = Kx + fmaf(c[0], fx, fmaf(c[1], fty0, c[2]));      // X = e0 + c1 tr
          e1 = Ky + fmaf(c[3], fx, fmaf(c[4], fty0, c[5]));      // Y = e1 + (1 + c4) tr
          e2 = 1.0f + c[4];
          e3 = e4 = e5 = e6 = 0.f;
        }
        else {
          // denominator 1 + q0 + c7 tr; x numerator nx0 + nxs tr; y numerator
          // ny0 + tr (nys - c7 tr) (the displacement form of warp_disp, expanded in tr)
          const float X1 = fx + c[12], Y1 = fty0 + c[13];
          const float q0 = fmaf(c[6], fx, c[7] * fty0);
          e0 = 1.0f + q0;
          e1 = fmaf(-q0, X1, fmaf(c[0], fx, fmaf(c[1], fty0, c[2])));
          e2 = fmaf(-c[7], X1, c[1]);
          e3 = fmaf(-q0, Y1, fmaf(c[3], fx, fmaf(c[4], fty0, c[5])));
          e4 = fmaf(-c[7], Y1, c[4] - q0);
          e5 = c[7], e6 = -c[7];
        }
        const float4 * tgp = a.refTG + (size_t) y0r * a.w + x;
        float tr = (float) (threadIdx.x >> RSH);
        if( pl.inside ) {
          if( y0r < yend ) cnt = (float) ((yend - 1 - y0r) / RS + 1);
#pragma unroll 4
        for( int y = y0r; y < yend; y += RS, tr += (float) RS, tgp += RS * a.w ) {
          float X, Y;
          if( FAM == FAM_AFFINE ) {
            X = fmaf(c[1], tr, e0);
            Y = fmaf(e2, tr, e1);
          }
          else {
            const float iw = __fdividef(1.0f, fmaf(e5, tr, e0));
            X = fmaf(fmaf(e2, tr, e1), iw, Kx);
            Y = fmaf(fmaf(tr, fmaf(e6, tr, e4), e3), iw, Ky + tr);
          }
          const int ix = __float2int_rz(X), iy = __float2int_rz(Y);
          const float ax = X - (float) ix, ay = Y - (float) iy;
          // inside the box by construction (footprint test); the clamp only guards the array
          const int o = (int) min((unsigned) (iy * PB_W + ix), (unsigned) (PB_W * PB_H - PB_W - 2));
          const float v00 = box[o], v01 = box[o + 1], v10 = box[o + PB_W], v11 = box[o + PB_W + 1];
          const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
          const float4 tg = __ldg(tgp);
          const float r = fmaf(ay, t1 - t0, t0) - tg.x;
          const float u = tg.y * r, w = tg.z * r;
          rr = fmaf(r, r, rr);
          P[0] += u, P[1] += w;
          if( NP > 2 ) P[2 < NP ? 2 : 0] = fmaf(tr, u, P[2 < NP ? 2 : 0]);
          if( NP > 3 ) P[3 < NP ? 3 : 0] = fmaf(tr, w, P[3 < NP ? 3 : 0]);
          if( NP > 4 ) P[4 < NP ? 4 : 0] = fmaf(tr * tr, w, P[4 < NP ? 4 : 0]);
        }
        }
        else {
          // tile at the level's border: samples whose four taps lie inside the level
          // read the box (full coverage, the same value as the global path); the
          // others take the global path's validity test and border mode
#pragma unroll 2
          for( int y = y0r; y < yend; y += RS, tr += (float) RS, tgp += RS * a.w ) {
            float X, Y;
            if( FAM == FAM_AFFINE ) {
              X = fmaf(c[1], tr, e0);
              Y = fmaf(e2, tr, e1);
            }
            else {
              const float iw = __fdividef(1.0f, fmaf(e5, tr, e0));
              X = fmaf(fmaf(e2, tr, e1), iw, Kx);
              Y = fmaf(fmaf(tr, fmaf(e6, tr, e4), e3), iw, Ky + tr);
            }
            const int ix = __float2int_rz(X), iy = __float2int_rz(Y);
            float v;
            bool ok;
            if( (unsigned) (ix + pl.bx0) <= (unsigned) (a.w - 2) && (unsigned) (iy + pl.by0) <= (unsigned) (a.h - 2) ) {
              const float ax = X - (float) ix, ay = Y - (float) iy;
              const int o = (int) min((unsigned) (iy * PB_W + ix), (unsigned) (PB_W * PB_H - PB_W - 2));
              const float v00 = box[o], v01 = box[o + 1], v10 = box[o + PB_W], v11 = box[o + PB_W + 1];
              const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
              v = fmaf(ay, t1 - t0, t0);
              ok = true;
            }
            else {
              const spos sp = warp_pos<FAM>(c, x, y);
              if( METHOD == M_IC ) ok = mask_ok(coverage(a.w, a.h, sp), 250);
              else {
                int rx, ry;
                warp_nearest<FAM>(c, x, y, rx, ry);
                ok = rx >= 0 && rx < a.w && ry >= 0 && ry < a.h;
              }
              v = sample_replicate(img, a.w, a.h, sp);
            }
            const float4 tg = __ldg(tgp);
            const float r = ok ? v - tg.x : 0.f;
            const float u = tg.y * r, w = tg.z * r;
            rr = fmaf(r, r, rr);
            cnt += ok ? 1.f : 0.f;
            P[0] += u, P[1] += w;
            if( NP > 2 ) P[2 < NP ? 2 : 0] = fmaf(tr, u, P[2 < NP ? 2 : 0]);
            if( NP > 3 ) P[3 < NP ? 3 : 0] = fmaf(tr, w, P[3 < NP ? 3 : 0]);
            if( NP > 4 ) P[4 < NP ? 4 : 0] = fmaf(tr * tr, w, P[4 < NP ? 4 : 0]);
          }
        }
        // row moments about y = 0 from the moments about y = ty0
        if( NP > 4 ) P[4 < NP ? 4 : 0] = fmaf(fty0, fmaf(fty0, P[1], 2.0f * P[3 < NP ? 3 : 0]), P[4 < NP ? 4 : 0]);
        if( NP > 3 ) P[3 < NP ? 3 : 0] = fmaf(fty0, P[1], P[3 < NP ? 3 : 0]);
        if( NP > 2 ) P[2 < NP ? 2 : 0] = fmaf(fty0, P[0], P[2 < NP ? 2 : 0]);
      }
    }
    else {
      const int xs0 = tx0 + (threadIdx.x & (TXS - 1) & ~31);
      const int xs1 = min(xs0 + 31, a.w - 1);
      for( int yc = ty0; yc < yend; yc += 16 ) {
        const int yc1 = min(yc + 15, yend - 1);
        const bool interior = (METHOD == M_IC || !a.refM) && xs0 < a.w &&
            rect_interior<FAM>(c, xs0, yc, xs1, yc1, a.w, a.h);
        if( x >= a.w ) continue;
        if( interior ) {
          const int y0r = yc + (threadIdx.x >> RSH);
          if( y0r <= yc1 ) cnt += (float) ((yc1 - y0r) / RS + 1);
          const int xI = x + (int) c[12], yI = (int) c[13];
          const float fx = (float) x;
          const float4 * tgp = a.refTG + (size_t) y0r * a.w + x;
          float fy = (float) y0r;
#pragma unroll 4
          for( int y = y0r; y <= yc1; y += RS, fy += (float) RS, tgp += RS * a.w ) {
            float dx, dy;
            warp_disp<FAM>(c, fx, fy, dx, dy);
            const float flx = floorf(dx), fly = floorf(dy);
            const float ax = dx - flx, ay = dy - fly;
            const float * r0 = img + ((y + yI + (int) fly) * a.w + xI + (int) flx);
            const float v00 = __ldg(r0), v01 = __ldg(r0 + 1), v10 = __ldg(r0 + a.w), v11 = __ldg(r0 + a.w + 1);
            const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
            const float4 tg = __ldg(tgp);
            const float r = fmaf(ay, t1 - t0, t0) - tg.x;
            const float u = tg.y * r, w = tg.z * r;
            rr = fmaf(r, r, rr);
            P[0] += u, P[1] += w;
            if( NP > 2 ) P[2 < NP ? 2 : 0] = fmaf(fy, u, P[2 < NP ? 2 : 0]);
            if( NP > 3 ) P[3 < NP ? 3 : 0] = fmaf(fy, w, P[3 < NP ? 3 : 0]);
            if( NP > 4 ) P[4 < NP ? 4 : 0] = fmaf(fy * fy, w, P[4 < NP ? 4 : 0]);
          }
        }
        else {
#pragma unroll 2
          for( int y = yc + (threadIdx.x >> RSH); y <= yc1; y += RS ) {
            const spos s = warp_pos<FAM>(c, x, y);
            const size_t i = (size_t) y * a.w + x;
            bool ok;
            if( METHOD == M_IC ) {
              ok = mask_ok(coverage(a.w, a.h, s), 250);
            }
            else {
              int rx, ry;
              warp_nearest<FAM>(c, x, y, rx, ry);
              ok = rx >= 0 && rx < a.w && ry >= 0 && ry < a.h;
              if( a.refM ) ok = ok && __ldg(a.refM + i) != 0;
            }
            const float v = sample_replicate(img, a.w, a.h, s);
            const float4 tg = __ldg(a.refTG + i);
            const float r = ok ? v - tg.x : 0.f;
            const float fy = (float) y;
            const float u = tg.y * r, w = tg.z * r;
            rr = fmaf(r, r, rr);
            cnt += ok ? 1.f : 0.f;
            P[0] += u, P[1] += w;
            if( NP > 2 ) P[2 < NP ? 2 : 0] = fmaf(fy, u, P[2 < NP ? 2 : 0]);
            if( NP > 3 ) P[3 < NP ? 3 : 0] = fmaf(fy, w, P[3 < NP ? 3 : 0]);
            if( NP > 4 ) P[4 < NP ? 4 : 0] = fmaf(fy * fy, w, P[4 < NP ? 4 : 0]);
          }
        }
      }
    }
    float acc[NS];
#pragma unroll
    for( int k = 0; k < NS; ++k ) acc[k] = 0.f;
    if( x < a.w ) column_project<JK, M>(P, (float) x, acc);
    acc[M] = rr;
    acc[M + 1] = cnt;
    warp_sums_to<NS>(acc, &s_red[b][(threadIdx.x >> 5) * NS]);
  }
  __syncthreads();
  if( pf >= 0 && (threadIdx.x >> 5) == 1 ) store_item_sums<NS, NW>(a, pf, pt, s_red[b ^ 1]);
  if( threadIdx.x == 0 ) inflight_drain(&s_infl, s_bar);
  if( timed_out && a.err ) atomicExch(a.err, 1);
}

/* -------------------------------------------------------- stencil passes */

/* Gram-matrix entry (i, j) that holds pass sum k. FA: V = [J (M), g - s, f - s, 1],
 * sums H (packed lower), SJg, SJf, SJ, Sf, Sf2, Sg, Sg2, n. LM: V = [J (M), r, 1],
 * sums H (packed lower), J^T r, |r|^2, n. */
template<int METHOD, int M>
__device__ __forceinline__ void sum_entry(int k, int & i, int & j)
{
  constexpr int nH = M * (M + 1) / 2;
  if( k < nH ) {
    int r = 0;
    while ( (r + 1) * (r + 2) / 2 <= k ) ++r;
    i = r, j = k - r * (r + 1) / 2;
    return;
  }
  k -= nH;
  if( METHOD == M_FA ) {
    if( k < 3 * M ) {
      i = k % M, j = M + k / M;                  // SJg: col M, SJf: col M + 1, SJ: col M + 2
      return;
    }
    switch ( k - 3 * M ) {
    case 0: i = M + 1, j = M + 2; return;        // Sf
    case 1: i = M + 1, j = M + 1; return;        // Sf2
    case 2: i = M, j = M + 2; return;            // Sg
    case 3: i = M, j = M; return;                // Sg2
    default: i = M + 2, j = M + 2; return;       // n
    }
  }
  else {
    if( k < M ) {
      i = k, j = M;
      return;
    }
    if( k == M ) i = j = M;
    else i = j = M + 1;
  }
}

/* FA / LM pass: the warped tile (+2 px halo, REPLICATE at the level border)
 * is staged in shared memory and differentiated there (ecc_differentiate),
 * so the warped image and its gradients never touch HBM. Each pixel forms
 * V = [steepest-descent row, residual terms, 1]; the tile's sums are the
 * entries of the Gram matrix sum V^T V, accumulated on the tensor cores
 * (32 pixels per warp per mma batch), then reduced over the 8 warps in FP64. */
template<int METHOD, int FAM, int JK, int M, bool ROI>
__global__ void __launch_bounds__(256) k_pass_stencil(PassArgs a)
{
  constexpr int nH = M * (M + 1) / 2;
  constexpr int NS = (METHOD == M_FA) ? nH + 3 * M + 5 : nH + M + 2;
  constexpr int SW = ST_TX + 4, SH = ST_TY + 4;
  static_assert(M + 3 <= 16, "V must fit 16 components");
  __shared__ float s_img[SH * SW];
  __shared__ __align__(16) float s_v[8][32 * GV_LD];      // per warp: V of 32 pixels, then its Gram matrix
  __shared__ double s_tile[NS];
  __shared__ float s_c[16];
  __shared__ float s_j[8];

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int count = __ldcg(a.count_in);
  const int nitems = ROI ? (count > 0 ? __ldcg(a.tile_total) : 0) : count * a.tiles;
  for( int item = blockIdx.x; item < nitems; item += gridDim.x ) {
    int fi, t, f, lw, lh, tiles_x;
    const float * img, * refT;
    const uint8_t * refMe;
    float tshift;
    double * part;
    if constexpr( ROI ) {
      fi = roi_entry(a.tile_prefix, count, item);
      t = item - __ldcg(a.tile_prefix + fi);
      f = __ldcg(a.list_in + fi);
      const RoiLevel & R = a.roi[(size_t) f * a.lmax + a.level];
      lw = R.w, lh = R.h, tiles_x = R.tiles_x;
      img = a.pyr + R.cur_off;
      refT = a.refT + R.ref_off;
      refMe = nullptr;
      tshift = R.tshift;
      part = a.partials + R.part_off;
    }
    else {
      fi = item / a.tiles;
      t = item - fi * a.tiles;
      f = __ldcg(a.list_in + fi);
      lw = a.w, lh = a.h, tiles_x = a.tiles_x;
      img = a.pyr + (size_t) f * a.pyr_stride + a.lvl_off;
      refT = a.refT;
      refMe = a.refMe;
      tshift = a.tshift;
      part = a.partials + (size_t) f * a.part_stride;
    }
    const FrameState * F = a.fs + f;
    if( threadIdx.x < 16 ) s_c[threadIdx.x] = F->wc[threadIdx.x];
    if( threadIdx.x < 8 ) s_j[threadIdx.x] = F->jc[threadIdx.x];
    __syncthreads();
    float c[16], jc[8];
#pragma unroll
    for( int i = 0; i < 16; ++i ) c[i] = s_c[i];
#pragma unroll
    for( int i = 0; i < 8; ++i ) jc[i] = s_j[i];
    const int tx0 = (t % tiles_x) * ST_TX, ty0 = (t / tiles_x) * ST_TY;

    // stage the warped image gw over the tile + halo (positions clamped: BORDER_REPLICATE)
    for( int q = threadIdx.x; q < SW * SH; q += 256 ) {
      const int xx = clampi(tx0 - 2 + q % SW, 0, lw - 1);
      const int yy = clampi(ty0 - 2 + q / SW, 0, lh - 1);
      s_img[q] = sample_replicate(img, lw, lh, warp_pos<FAM>(c, xx, yy));
    }
    __syncthreads();

    float g0[4] = { 0.f, 0.f, 0.f, 0.f }, g1[4] = { 0.f, 0.f, 0.f, 0.f };
    float * sv = s_v[wid];
    const int lx = threadIdx.x & (ST_TX - 1);
    const int x = tx0 + lx;
#pragma unroll 1
    for( int k = 0; k < ST_TY / 4; ++k ) {
      const int ly = (threadIdx.x >> 6) + 4 * k;
      const int y = ty0 + ly;
      float v[16];
#pragma unroll
      for( int u = 0; u < 16; ++u ) v[u] = 0.f;
      if( x < lw && y < lh ) {
        const float fx = (float) x, fy = (float) y;
        const spos s = warp_pos<FAM>(c, x, y);
        const size_t i = (size_t) y * lw + x;
        const float cov = coverage(lw, lh, s);
        bool ok = mask_ok(cov, METHOD == M_FA ? 255 : 250);
        if( refMe ) ok = ok && __ldg(refMe + i) != 0;
        // gx = d5 (x) (*) s3 (y), gy = s3 (x) (*) d5 (y)
        const float * p = s_img + (ly + 2) * SW + (lx + 2);
        const float d5a = 1.f / 12.f, d5b = -2.f / 3.f;
        float gxw, gyw;
        {
          const float r0 = d5a * p[-SW - 2] + d5b * p[-SW - 1] - d5b * p[-SW + 1] - d5a * p[-SW + 2];
          const float r1 = d5a * p[-2] + d5b * p[-1] - d5b * p[1] - d5a * p[2];
          const float r2 = d5a * p[SW - 2] + d5b * p[SW - 1] - d5b * p[SW + 1] - d5a * p[SW + 2];
          gxw = 0.25f * r0 + 0.5f * r1 + 0.25f * r2;
          const float c0 = d5a * p[-2 * SW - 1] + d5b * p[-SW - 1] - d5b * p[SW - 1] - d5a * p[2 * SW - 1];
          const float c1 = d5a * p[-2 * SW] + d5b * p[-SW] - d5b * p[SW] - d5a * p[2 * SW];
          const float c2 = d5a * p[-2 * SW + 1] + d5b * p[-SW + 1] - d5b * p[SW + 1] - d5a * p[2 * SW + 1];
          gyw = 0.25f * c0 + 0.5f * c1 + 0.25f * c2;
        }
        if( !ok ) gxw = gyw = 0.f;
        const float gw = p[0];
        const float T = __ldg(refT + i);
        float J[M];
        sd_pixel<JK, M>(jc, fx, fy, gxw, gyw, J);
#pragma unroll
        for( int u = 0; u < M; ++u ) v[u] = J[u];
        if( ok ) {
          if( METHOD == M_FA ) {
            v[M] = gw - tshift;
            v[M + 1] = T - tshift;
            v[M + 2] = 1.f;
          }
          else {
            v[M] = gw - T;
            v[M + 1] = 1.f;
          }
        }
      }
      __syncwarp();
      float4 * dst = reinterpret_cast<float4 *>(sv + lane * GV_LD);
#pragma unroll
      for( int q = 0; q < 4; ++q ) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      __syncwarp();
      gram_accumulate(sv, g0, g1);
    }
    // this warp's Gram matrix into its staging area (16 x 16, row stride 16)
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
      sum_entry<METHOD, M>(threadIdx.x, gi, gj);
      double tsum = 0;
#pragma unroll
      for( int wv = 0; wv < 8; ++wv ) tsum += (double) s_v[wv][gi * 16 + gj];
      s_tile[threadIdx.x] = tsum;
    }
    __syncthreads();
    write_tile_at<NS>(part, t, s_tile);
  }
}

/* ------------------------------------------------------------- dispatch */

__host__ __device__ int pass_num_sums(int method, int M)
{
  const int nH = M * (M + 1) / 2;
  switch ( method ) {
  case M_FA: return nH + 3 * M + 5;
  case M_LM: return nH + M + 2;
  default: return M + 2;
  }
}

/* The per-frame Gauss-Newton logic of one step: one warp per active frame
 * combines the frame's tile partials in a fixed order (lane-strided sums, then
 * a fixed butterfly) and lane 0 runs the reference's per-iteration update in
 * FP64. */
__global__ void __launch_bounds__(256) k_solve(PassArgs a, int method)
{
  __shared__ double s_sum[8][160];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int warp = blockIdx.x * 8 + wid, nwarps = gridDim.x * 8;
  const int NS = pass_num_sums(method, a.M);
  const int count = __ldcg(a.count_in);
  for( int fi = warp; fi < count; fi += nwarps ) {
    const int f = __ldcg(a.list_in + fi);
    const RoiLevel * R = a.roi ? a.roi + (size_t) f * a.lmax + a.level : nullptr;
    const double * P = R ? a.partials + R->part_off : a.partials + (size_t) f * a.part_stride;
    const int tiles = R ? R->tiles : a.tiles;
    for( int k = 0; k < NS; ++k ) {
      double v = 0;
      for( int t = lane; t < tiles; t += 32 ) v += __ldcg(P + (size_t) t * NS + k);
      v = warp_sum(v);
      if( lane == 0 ) s_sum[wid][k] = v;
    }
    __syncwarp();
    if( lane == 0 ) {
      FrameState * F = a.fs + f;
      if( R ) {
        // ROI batch: this frame's level size and rescale factor
        PassArgs b = a;
        b.w = R->w, b.h = R->h, b.scale_next = R->scale_next, b.tiles = R->tiles;
        if( method == M_FA ) solve_fa(F, s_sum[wid], b, f);
        else solve_lm(F, s_sum[wid], b, f);
      }
      else {
        switch ( method ) {
        case M_IC: solve_ic(F, s_sum[wid], a, f); break;
        case M_ICLM: solve_iclm(F, s_sum[wid], a, f); break;
        case M_FA: solve_fa(F, s_sum[wid], a, f); break;
        default: solve_lm(F, s_sum[wid], a, f); break;
        }
      }
    }
    __syncwarp();
  }
}

cudaError_t launch_solve(int method, const PassArgs & a, int grid, cudaStream_t st)
{
  k_solve<<<grid, 256, 0, st>>>(a, method);
  return cudaGetLastError();
}

/* persistent grid: every SM filled to the kernel's occupancy */
template<typename K>
static int persistent_grid(K kernel, int nt = 256)
{
  static int sms = 0;
  if( !sms ) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if( sms <= 0 ) sms = 1;
  }
  int per_sm = 0;
  if( cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nt, 0) != cudaSuccess || per_sm < 1 ) {
    cudaGetLastError();
    per_sm = 1;
  }
  return sms * per_sm;
}

template<int METHOD, int FAM, int JK, int M>
static cudaError_t launch_t(const PassArgs & a, int grid, cudaStream_t st, const CUtensorMap * map)
{
  if constexpr( METHOD == M_IC || METHOD == M_ICLM ) {
    if( map && FAM != FAM_QUAD ) {
      // a tuned grid counts CTAs of 256 threads
      constexpr int NT = pw_threads<FAM>();
      if( a.tile_w == 64 ) {
        static int g = 0;
        if( !g ) g = persistent_grid(k_pass_pointwise_tma<METHOD, FAM, JK, M, 64>, NT);
        k_pass_pointwise_tma<METHOD, FAM, JK, M, 64><<<grid > 0 ? grid * (256 / NT) : g, NT, 0, st>>>(a, *map);
      }
      else {
        static int g = 0;
        if( !g ) g = persistent_grid(k_pass_pointwise_tma<METHOD, FAM, JK, M, PW_TX>, NT);
        k_pass_pointwise_tma<METHOD, FAM, JK, M, PW_TX><<<grid > 0 ? grid * (256 / NT) : g, NT, 0, st>>>(a, *map);
      }
      return cudaGetLastError();
    }
    static int g = 0;
    if( !g ) {
      g = persistent_grid(k_pass_pointwise<METHOD, FAM, JK, M>);
    }
    k_pass_pointwise<METHOD, FAM, JK, M><<<grid > 0 ? grid : g, 256, 0, st>>>(a);
  }
  else if( a.roi ) {
    static int g = 0;
    if( !g ) g = persistent_grid(k_pass_stencil<METHOD, FAM, JK, M, true>);
    k_pass_stencil<METHOD, FAM, JK, M, true><<<grid > 0 ? grid : g, 256, 0, st>>>(a);
  }
  else {
    static int g = 0;
    if( !g ) g = persistent_grid(k_pass_stencil<METHOD, FAM, JK, M, false>);
    k_pass_stencil<METHOD, FAM, JK, M, false><<<grid > 0 ? grid : g, 256, 0, st>>>(a);
  }
  return cudaGetLastError();
}

template<int METHOD>
static cudaError_t launch_m(const PassArgs & a, int grid, cudaStream_t st, const CUtensorMap * map)
{
  switch ( a.model.type ) {
  case SST_MOTION_TRANSLATION: return launch_t<METHOD, FAM_AFFINE, J_TRANS, 2>(a, grid, st, map);
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN:
    if( a.M == 3 ) return launch_t<METHOD, FAM_AFFINE, J_EUCL, 3>(a, grid, st, map);
    return launch_t<METHOD, FAM_AFFINE, J_EUCL, 4>(a, grid, st, map);
  case SST_MOTION_AFFINE: return launch_t<METHOD, FAM_AFFINE, J_AFFINE, 6>(a, grid, st, map);
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: return launch_t<METHOD, FAM_HOMOG, J_HOMOG, 8>(a, grid, st, map);
  case SST_MOTION_SEMI_QUADRATIC:
    if( METHOD == M_FA || METHOD == M_LM ) return launch_t<(METHOD == M_FA ? M_FA : M_LM), FAM_QUAD, J_SEMIQ, 8>(a, grid, st, map);
    return cudaErrorInvalidValue;
  case SST_MOTION_QUADRATIC:
    if( METHOD == M_FA || METHOD == M_LM ) return launch_t<(METHOD == M_FA ? M_FA : M_LM), FAM_QUAD, J_QUAD, 12>(a, grid, st, map);
    return cudaErrorInvalidValue;
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_pass(int method, const PassArgs & a, int grid, cudaStream_t st, const CUtensorMap * map)
{
  if( a.roi && method != M_FA && method != M_LM ) return cudaErrorInvalidValue;
  switch ( method ) {
  case M_IC: return launch_m<M_IC>(a, grid, st, map);
  case M_ICLM: return launch_m<M_ICLM>(a, grid, st, map);
  case M_FA: return launch_m<M_FA>(a, grid, st, nullptr);
  case M_LM: return launch_m<M_LM>(a, grid, st, nullptr);
  }
  return cudaErrorInvalidValue;
}

/* the pyramid level of every frame slot as a 3-D tensor (x, y, frame) with
 * the pointwise footprint box; false when the level's layout breaks the TMA
 * rules (row and frame strides multiples of 16 bytes, aligned base) */
bool encode_pass_level(const float * level0_of_slot0, int w, int h, size_t pyr_stride, int frames, CUtensorMap * map,
    int tile_w)
{
  const uint64_t dims[3] = { (uint64_t) w, (uint64_t) h, (uint64_t) frames };
  const uint64_t strides[2] = { (uint64_t) w * sizeof(float), (uint64_t) pyr_stride * sizeof(float) };
  const uint32_t box[3] = { (uint32_t) (tile_w + 16), (uint32_t) PB_H, 1 };
  return encode_tensor_3d(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, level0_of_slot0, dims, strides, box);
}

/* ------------------------------------------------------ level / pass glue */

/* c_ecch per-level align() prologue: reset the per-level solver state and
 * list every frame still registering. One thread per frame over the whole
 * grid (the FP64 state work spreads over the SMs); frames are appended with
 * one atomic per warp, in no particular order (nothing depends on the order
 * of an active list). *count_out is zero before the launch. */
__global__ void __launch_bounds__(128) k_level_begin(LevelBeginArgs a)
{
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  bool alive = false;
  if( f < a.n ) {
    FrameState * F = a.fs + f;
    alive = F->status == SST_FRAME_OK;
    if( a.roi && a.roi[(size_t) f * a.lmax + a.level].w == 0 ) alive = false;   // no such level
    F->n = 0;
    F->phase = PH_START;
    F->converged = 0;
    F->level_ok = 0;
    F->err = 0;
    F->rmsold = FLT_MAX;
    F->eps = FLT_MAX;
    F->dpe = 0;
    F->lambda = a.method == M_LM ? 0.1 : 0.001;
    set_eval(F, a.model, F->state);
  }
  const unsigned b = __ballot_sync(0xffffffffu, alive);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if( lane == 0 && b ) base = atomicAdd(a.count_out, __popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  if( alive ) a.list_out[base + __popc(b & ((1u << lane) - 1u))] = f;
}

cudaError_t launch_level_begin(const LevelBeginArgs & a, cudaStream_t st)
{
  k_level_begin<<<(unsigned) (a.n > 0 ? (a.n + 127) / 128 : 1), 128, 0, st>>>(a);
  return cudaGetLastError();
}

/* launches of the level loops' kernels (pass, solve, advance), counted on the device */
__device__ unsigned long long g_loop_launches = 0;

/* End of one iteration of a level run as a graph WHILE loop: records the
 * active count the next iteration starts with, moves list B (the solve's
 * output) to list A (the next pass's input), clears B and keeps the loop
 * going while frames remain and iterations are left (the unrolled schedule's
 * max_iterations + 1 passes). */
__global__ void __launch_bounds__(1024) k_level_advance(LevelLoopArgs a)
{
  const int it = *a.cursor;
  const int cb = *a.count_b;
  for( int i = threadIdx.x; i < cb; i += blockDim.x ) a.list_a[i] = a.list_b[i];
  __syncthreads();                                   // every thread has read the counts
  if( threadIdx.x == 0 ) {
    if( it == 0 ) a.hist[0] = *a.count_a;
    a.hist[it + 1] = cb;
    *a.count_a = cb;
    *a.count_b = 0;
    *a.cursor = it + 1;
    g_loop_launches += 3;
    cudaGraphSetConditional(a.handle, (cb > 0 && it + 1 <= a.max_it) ? 1u : 0u);
  }
}

cudaError_t launch_level_advance(const LevelLoopArgs & a, cudaStream_t st)
{
  k_level_advance<<<1, 1024, 0, st>>>(a);
  return cudaGetLastError();
}

long long loop_launches(bool reset)
{
  unsigned long long v = 0;
  if( cudaDeviceSynchronize() != cudaSuccess ) {
    cudaGetLastError();
    return 0;
  }
  if( cudaMemcpyFromSymbol(&v, g_loop_launches, sizeof(v)) != cudaSuccess ) return 0;
  if( reset ) {
    const unsigned long long z = 0;
    cudaMemcpyToSymbol(g_loop_launches, &z, sizeof(z));
  }
  return (long long) v;
}

/* c_ecch::align prologue (ecc2.cc:1133-1151): start state of the pass, then
 * scale_transfrom to the coarsest level. */
__global__ void k_pass_begin(PassBeginArgs a)
{
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if( f >= a.n ) return;
  FrameState * F = a.fs + f;
  if( a.pass == 0 ) {
    F->status = SST_FRAME_OK;
    F->total_iters = 0;
    F->rho = 0;
    F->weight = 0;
    F->eps = FLT_MAX;
    if( a.init_states ) for( int i = 0; i < 16; ++i ) F->state[i] = a.init_states[(size_t) f * 16 + i];
    else model_identity(a.model, F->state);
  }
  else {
    double s[16];
    model_convert(a.prev_model, F->state, a.model, s);
    for( int i = 0; i < 16; ++i ) F->state[i] = s[i];
  }
  const double sc = a.roi ? a.roi[(size_t) f * a.lmax].scale_first : a.scale_to_coarsest;
  if( sc > 0 ) model_scale(a.model, F->state, sc);
  set_eval(F, a.model, F->state);
}

cudaError_t launch_pass_begin(const PassBeginArgs & a, cudaStream_t st)
{
  k_pass_begin<<<(a.n + 127) / 128, 128, 0, st>>>(a);
  return cudaGetLastError();
}

/* --------------------------------------------------------- correlation */

/* compute_correlation(current, mask, reference, mask, rmap) (ecc2.cc:100-137)
 * on level 0 at the final state: LINEAR / BORDER_CONSTANT remap, mask >= 254.
 * Sums of the values shifted by the reference mean. */
template<int FAM>
__global__ void __launch_bounds__(256) k_correlation(CorrArgs a)
{
  constexpr int NS = 6;
  __shared__ float s_red[8 * NS];
  __shared__ double s_tile[NS];
  __shared__ float s_c[16];
  const int nitems = a.roi ? __ldg(a.tile_prefix + a.n) : a.n * a.tiles;
  for( int item = blockIdx.x; item < nitems; item += gridDim.x ) {
    int f, t, lw, lh, tiles_x;
    const float * img, * refT;
    float tshift;
    double * part;
    if( a.roi ) {
      f = roi_entry(a.tile_prefix, a.n, item);
      t = item - __ldg(a.tile_prefix + f);
      const RoiLevel & R = a.roi[(size_t) f * a.lmax];
      lw = R.w, lh = R.h, tiles_x = R.ctiles_x;
      img = a.pyr + R.cur_off;
      refT = a.refT + R.ref_off;
      tshift = R.tshift;
      part = a.partials + R.part_off;
    }
    else {
      f = item / a.tiles;
      t = item - f * a.tiles;
      lw = a.w, lh = a.h, tiles_x = a.tiles_x;
      img = a.pyr + (size_t) f * a.pyr_stride;
      refT = a.refT;
      tshift = a.tshift;
      part = a.partials + (size_t) f * a.part_stride;
    }
    const FrameState * F = a.fs + f;
    if( F->status != SST_FRAME_OK ) continue;   // uniform per CTA: no barrier skipped unevenly
    if( threadIdx.x < 16 ) s_c[threadIdx.x] = F->wc[threadIdx.x];
    __syncthreads();
    float c[16];
#pragma unroll
    for( int i = 0; i < 16; ++i ) c[i] = s_c[i];
    const int tx0 = (t % tiles_x) * PW_TX, ty0 = (t / tiles_x) * PW_TY;
    const int x = tx0 + (threadIdx.x & (PW_TX - 1));
    const int yend = min(ty0 + PW_TY, lh);
    // warm L2 with the source footprint of this CTA's next item (uniform tiles)
    if( !a.roi && item + (int) gridDim.x < nitems ) {
      const int nitem = item + gridDim.x;
      const int nf = nitem / a.tiles, nt = nitem - nf * a.tiles;
      const float * nw = a.fs[nf].wc;
      const int nx0 = (nt % a.tiles_x) * PW_TX, ny0 = (nt / a.tiles_x) * PW_TY;
      const int row = threadIdx.x >> 2;
      if( row < PW_TY ) {
        const int yy = min(ny0 + row, a.h - 1);
        const int xx = min(nx0 + (threadIdx.x & 3) * 32, a.w - 1);
        const float dx = fmaf(__ldg(nw + 0), (float) xx, fmaf(__ldg(nw + 1), (float) yy, __ldg(nw + 2)));
        const float dy = fmaf(__ldg(nw + 3), (float) xx, fmaf(__ldg(nw + 4), (float) yy, __ldg(nw + 5)));
        const int sx = clampi(xx + (int) __ldg(nw + 12) + (int) floorf(dx), 0, a.w - 1);
        const int sy = clampi(yy + (int) __ldg(nw + 13) + (int) floorf(dy), 0, a.h - 1);
        const float * pp = a.pyr + (size_t) nf * a.pyr_stride + (size_t) sy * a.w + sx;
        asm volatile("prefetch.global.L2 [%0];" :: "l"(pp));
      }
    }
    float acc[NS] = { 0, 0, 0, 0, 0, 0 };
    // per 32-column warp strip and 16-row chunk: chunks whose every tap is inside
    // the level gather directly (no coverage, no border logic)
    const int xs0 = tx0 + (threadIdx.x & (PW_TX - 1) & ~31);
    const int xs1 = min(xs0 + 31, lw - 1);
    for( int yc = ty0; yc < yend; yc += 16 ) {
      const int yc1 = min(yc + 15, yend - 1);
      const bool interior = !a.refM && xs0 < lw && rect_interior<FAM>(c, xs0, yc, xs1, yc1, lw, lh);
      if( x >= lw ) continue;
      if( interior ) {
#pragma unroll 4
        for( int y = yc + (threadIdx.x >> 7); y <= yc1; y += 2 ) {
          const spos s = warp_pos<FAM>(c, x, y);
          const float * r0 = img + (size_t) s.y0 * lw + s.x0;
          const float v00 = __ldg(r0), v01 = __ldg(r0 + 1), v10 = __ldg(r0 + lw), v11 = __ldg(r0 + lw + 1);
          const float t0 = fmaf(s.fx, v01 - v00, v00), t1 = fmaf(s.fx, v11 - v10, v10);
          const float av = __ldg(refT + (size_t) y * lw + x) - tshift;
          const float bv = fmaf(s.fy, t1 - t0, t0) - tshift;
          acc[0] += av, acc[1] += bv;
          acc[2] = fmaf(av, av, acc[2]);
          acc[3] = fmaf(bv, bv, acc[3]);
          acc[4] = fmaf(av, bv, acc[4]);
          acc[5] += 1.f;
        }
      }
      else {
#pragma unroll 2
        for( int y = yc + (threadIdx.x >> 7); y <= yc1; y += 2 ) {
          const spos s = warp_pos<FAM>(c, x, y);
          const size_t i = (size_t) y * lw + x;
          bool ok = mask_ok(coverage(lw, lh, s), 254);
          if( a.refM ) ok = ok && __ldg(a.refM + i) != 0;
          if( ok ) {
            const float av = __ldg(refT + i) - tshift;
            const float bv = sample_constant0(img, lw, lh, s) - tshift;
            acc[0] += av, acc[1] += bv;
            acc[2] = fmaf(av, av, acc[2]);
            acc[3] = fmaf(bv, bv, acc[3]);
            acc[4] = fmaf(av, bv, acc[4]);
            acc[5] += 1.f;
          }
        }
      }
    }
    block_reduce_d<NS>(acc, s_red, s_tile);
    write_tile_at<NS>(part, t, s_tile);
  }
}

/* rho = cov / (sigma1 sigma2) per frame and the min_rho gate */
__global__ void __launch_bounds__(256) k_correlation_finish(CorrArgs a)
{
  __shared__ double s_tmp[256];
  __shared__ double s_sum[8];
  for( int f = blockIdx.x; f < a.n; f += gridDim.x ) {
    FrameState * F = a.fs + f;
    if( F->status != SST_FRAME_OK ) continue;
    const RoiLevel * R = a.roi ? a.roi + (size_t) f * a.lmax : nullptr;
    combine_partials(R ? a.partials + R->part_off : a.partials + (size_t) f * a.part_stride, R ? R->ctiles : a.tiles,
        6, s_tmp, s_sum);
    if( threadIdx.x == 0 ) {
      const double n = s_sum[5];
      double rho = 0;
      if( n > 0 ) {
        const double ma = s_sum[0] / n, mb = s_sum[1] / n;
        const double va = s_sum[2] / n - ma * ma, vb = s_sum[3] / n - mb * mb;
        const double cv = s_sum[4] / n - ma * mb;
        rho = cv / (sqrt(fmax(va, 0.0)) * sqrt(fmax(vb, 0.0)));
      }
      F->rho = (float) rho;
      if( a.min_rho > 0 && !(rho >= a.min_rho) ) F->status = SST_FRAME_LOW_RHO;
    }
    __syncthreads();
  }
}

/* Correlation with each (frame, tile) footprint staged by TMA (uniform
 * batches): same structure as the staged IC pass; items whose taps leave
 * the level or the box, or with a reference mask, take the global path. */
template<int FAM>
__device__ __forceinline__ void plan_corr_item(const CorrArgs & a, int item, int status, float cl, float * s_c,
    ItemPlan * plan)
{
  // values loaded an item earlier: the frame's status and, in lane l, its coefficient l & 15
  const int lane = threadIdx.x & 31;
  const int f = item / a.tiles, t = item - f * a.tiles;
  const bool live = status == SST_FRAME_OK;
  float c[16];
#pragma unroll
  for( int i = 0; i < 16; ++i ) c[i] = __shfl_sync(0xffffffffu, cl, i);
  if( lane < 16 ) s_c[lane] = cl;
  const int tx0 = (t % a.tiles_x) * PW_TX, ty0 = (t / a.tiles_x) * PW_TY;
  const int tx1 = min(tx0 + PW_TX, a.w) - 1, ty1 = min(ty0 + PW_TY, a.h) - 1;
  int bx0, by0, bx1, by1;
  bool inside;
  bool use = rect_box<FAM>(c, tx0, ty0, tx1, ty1, a.w, a.h, bx0, by0, bx1, by1, inside);
  use = use && live && !a.refM;
  if( use ) {
    bx0 = bx0 >= 0 ? bx0 & ~3 : -((-bx0 + 3) & ~3);
    use = bx1 < bx0 + PB_W && by1 < by0 + PB_H;
  }
  if( lane == 0 ) {
    plan->f = live ? f : -1, plan->t = t;
    plan->use = use ? 1 : 0;
    plan->inside = inside ? 1 : 0;
    plan->bx0 = bx0, plan->by0 = by0;
  }
}

template<int FAM>
__global__ void __launch_bounds__(256, 4) k_correlation_tma(CorrArgs a, const __grid_constant__ CUtensorMap tmap)
{
  constexpr int NS = 6;
  __shared__ __align__(128) float s_box[2][PB_H * PB_W];
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ float s_red[2][8 * NS];     // warp sums of the current and the previous item
  __shared__ float s_c[3][16];
  __shared__ ItemPlan s_plan[3];
  __shared__ uint32_t s_infl;             // copies in flight, kept by thread 0
  __shared__ int s_gaveup[2];             // a wait gave up during an item of this buffer parity
  const int nitems = a.n * a.tiles;
  if( (int) blockIdx.x >= nitems ) return;          // uniform over the CTA
  if( threadIdx.x == 0 ) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    s_infl = 0u;
    s_gaveup[0] = s_gaveup[1] = 0;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  // warp 0 keeps the next item's frame status and lane coefficient in flight
  int st1 = 0;
  float c1 = 0.f;
  if( threadIdx.x < 32 ) {
    const int lane = threadIdx.x & 31;
    const FrameState * F0 = a.fs + blockIdx.x / a.tiles;
    plan_corr_item<FAM>(a, blockIdx.x, __ldcg(&F0->status), __ldcg(F0->wc + (lane & 15)), s_c[0], &s_plan[0]);
    const int it1 = blockIdx.x + gridDim.x;
    if( it1 < nitems ) {
      const FrameState * F1 = a.fs + it1 / a.tiles;
      st1 = __ldcg(&F1->status), c1 = __ldcg(F1->wc + (lane & 15));
    }
  }
  __syncthreads();
  if( threadIdx.x == 0 && s_plan[0].use ) {
    mbar_expect_tx(&s_bar[0], PB_W * PB_H * sizeof(float));
    tma_load_3d(s_box[0], &tmap, s_plan[0].bx0, s_plan[0].by0, s_plan[0].f, &s_bar[0]);
    inflight_issued(&s_infl, 0, 0u);
  }
  uint32_t phases = 0u;
  bool timed_out = false, stop = false;
  int slot = 0, b = 0;
  int pf = -1, pt = 0;                              // previous item (its sums wait in s_red[b ^ 1])
  for( int item = blockIdx.x; item < nitems; item += gridDim.x, b ^= 1 ) {
    const int nitem = item + gridDim.x;
    const int nslot = slot == 2 ? 0 : slot + 1;
    if( threadIdx.x < 32 && nitem < nitems ) {
      plan_corr_item<FAM>(a, nitem, st1, c1, s_c[nslot], &s_plan[nslot]);
      const int it2 = nitem + gridDim.x;
      if( it2 < nitems ) {
        const FrameState * F2 = a.fs + it2 / a.tiles;
        st1 = __ldcg(&F2->status), c1 = __ldcg(F2->wc + (threadIdx.x & 15));
      }
    }
    // orders: the next plan; the previous item's warp sums; the previous item's
    // reads of the box buffer that the next copy overwrites
    __syncthreads();
    // once a wait gave up no further copy is issued or consumed; the previous item's
    // flag is read after the barrier and written again no earlier than the next item,
    // so every thread sees the same value
    stop = stop || s_gaveup[b ^ 1];
    if( threadIdx.x == 0 && nitem < nitems && s_plan[nslot].use && !stop ) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&s_bar[b ^ 1], PB_W * PB_H * sizeof(float));
      tma_load_3d(s_box[b ^ 1], &tmap, s_plan[nslot].bx0, s_plan[nslot].by0, s_plan[nslot].f, &s_bar[b ^ 1]);
      inflight_issued(&s_infl, b ^ 1, (phases >> (b ^ 1)) & 1u);
    }
    if( pf >= 0 && (threadIdx.x >> 5) == 1 ) {
      // FP64 sum, in warp order, of the previous item's 8 warp sums: its tile partials
      const int lane = threadIdx.x & 31;
      if( lane < NS ) {
        double sum = 0;
#pragma unroll
        for( int wv = 0; wv < 8; ++wv ) sum += (double) s_red[b ^ 1][wv * NS + lane];
        a.partials[(size_t) pf * a.part_stride + (size_t) pt * NS + lane] = sum;
      }
    }
    const ItemPlan pl = s_plan[slot];
    pf = pl.f, pt = pl.t;
    float c[16];
#pragma unroll
    for( int i = 0; i < 16; ++i ) c[i] = s_c[slot][i];
    slot = nslot;
    if( pl.f < 0 ) continue;                        // frame already rejected: uniform over the CTA
    const int f = pl.f, t = pl.t;
    const float * img = a.pyr + (size_t) f * a.pyr_stride;
    const int tx0 = (t % a.tiles_x) * PW_TX, ty0 = (t / a.tiles_x) * PW_TY;
    const int x = tx0 + (threadIdx.x & (PW_TX - 1));
    const int yend = min(ty0 + PW_TY, a.h);
    float acc[NS] = { 0, 0, 0, 0, 0, 0 };
    if( pl.use && !stop ) {
      if( !mbar_wait_bounded(&s_bar[b], (phases >> b) & 1u) ) timed_out = true, s_gaveup[b] = 1;
      else if( threadIdx.x == 0 ) inflight_landed(&s_infl, b);
      phases ^= 1u << b;
      if( x < a.w ) {
        const float * box = s_box[b];
        const int y0r = ty0 + (threadIdx.x >> 7);
        // sample positions in box coordinates as functions of the tile-local row
        // (as in the IC pass): positive by the footprint test, so truncation floors
        const float fx = (float) x, fty0 = (float) ty0;
        const float Kx = (float) (x + (int) c[12] - pl.bx0), Ky = (float) (ty0 + (int) c[13] - pl.by0);
        float e0, e1, e2, e3 = 0.f, e4 = 0.f, e5 = 0.f, e6 = 0.f;
        if( FAM == FAM_AFFINE ) {
          e0 = Kx + fmaf(c[0], fx, fmaf(c[1], fty0, c[2]));
          e1 = Ky + fmaf(c[3], fx, fmaf(c[4], fty0, c[5]));
          e2 = 1.0f + c[4];
        }
        else {
          const float X1 = fx + c[12], Y1 = fty0 + c[13];
          const float q0 = fmaf(c[6], fx, c[7] * fty0);
          e0 = 1.0f + q0;
          e1 = fmaf(-q0, X1, fmaf(c[0], fx, fmaf(c[1], fty0, c[2])));
          e2 = fmaf(-c[7], X1, c[1]);
          e3 = fmaf(-q0, Y1, fmaf(c[3], fx, fmaf(c[4], fty0, c[5])));
          e4 = fmaf(-c[7], Y1, c[4] - q0);
          e5 = c[7], e6 = -c[7];
        }
        float tr = (float) (threadIdx.x >> 7);
        if( pl.inside ) {
          // every sample counts (full coverage): the count is known in advance
          if( y0r < yend ) acc[5] = (float) ((yend - 1 - y0r) / 2 + 1);
          const float * rp = a.refT + (size_t) y0r * a.w + x;
#pragma unroll 4
        for( int y = y0r; y < yend; y += 2, tr += 2.f, rp += 2 * a.w ) {
          float X, Y;
          if( FAM == FAM_AFFINE ) {
            X = fmaf(c[1], tr, e0);
            Y = fmaf(e2, tr, e1);
          }
          else {
            const float iw = __fdividef(1.0f, fmaf(e5, tr, e0));
            X = fmaf(fmaf(e2, tr, e1), iw, Kx);
            Y = fmaf(fmaf(tr, fmaf(e6, tr, e4), e3), iw, Ky + tr);
          }
          const int ix = __float2int_rz(X), iy = __float2int_rz(Y);
          const float ax = X - (float) ix, ay = Y - (float) iy;
          const int o = (int) min((unsigned) (iy * PB_W + ix), (unsigned) (PB_W * PB_H - PB_W - 2));
          const float v00 = box[o], v01 = box[o + 1], v10 = box[o + PB_W], v11 = box[o + PB_W + 1];
          const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
          const float av = __ldg(rp) - a.tshift;
          const float bv = fmaf(ay, t1 - t0, t0) - a.tshift;
          acc[0] += av, acc[1] += bv;
          acc[2] = fmaf(av, av, acc[2]);
          acc[3] = fmaf(bv, bv, acc[3]);
          acc[4] = fmaf(av, bv, acc[4]);
        }
        }
        else {
          // tile at the level's border: samples whose four taps lie inside the level
          // read the box (full coverage, the same value as the global path); the
          // others take the global path's coverage test and constant border
#pragma unroll 2
          for( int y = y0r; y < yend; y += 2, tr += 2.f ) {
            float X, Y;
            if( FAM == FAM_AFFINE ) {
              X = fmaf(c[1], tr, e0);
              Y = fmaf(e2, tr, e1);
            }
            else {
              const float iw = __fdividef(1.0f, fmaf(e5, tr, e0));
              X = fmaf(fmaf(e2, tr, e1), iw, Kx);
              Y = fmaf(fmaf(tr, fmaf(e6, tr, e4), e3), iw, Ky + tr);
            }
            const int ix = __float2int_rz(X), iy = __float2int_rz(Y);
            float v;
            bool ok;
            if( (unsigned) (ix + pl.bx0) <= (unsigned) (a.w - 2) && (unsigned) (iy + pl.by0) <= (unsigned) (a.h - 2) ) {
              const float ax = X - (float) ix, ay = Y - (float) iy;
              const int o = (int) min((unsigned) (iy * PB_W + ix), (unsigned) (PB_W * PB_H - PB_W - 2));
              const float v00 = box[o], v01 = box[o + 1], v10 = box[o + PB_W], v11 = box[o + PB_W + 1];
              const float t0 = fmaf(ax, v01 - v00, v00), t1 = fmaf(ax, v11 - v10, v10);
              v = fmaf(ay, t1 - t0, t0);
              ok = true;
            }
            else {
              const spos sp = warp_pos<FAM>(c, x, y);
              ok = mask_ok(coverage(a.w, a.h, sp), 254);
              v = ok ? sample_constant0(img, a.w, a.h, sp) : 0.f;
            }
            if( ok ) {
              const float av = __ldg(a.refT + (size_t) y * a.w + x) - a.tshift;
              const float bv = v - a.tshift;
              acc[0] += av, acc[1] += bv;
              acc[2] = fmaf(av, av, acc[2]);
              acc[3] = fmaf(bv, bv, acc[3]);
              acc[4] = fmaf(av, bv, acc[4]);
              acc[5] += 1.f;
            }
          }
        }
      }
    }
    else {
      for( int y = ty0 + (threadIdx.x >> 7); y < yend && x < a.w; y += 2 ) {
        const spos s = warp_pos<FAM>(c, x, y);
        const size_t i = (size_t) y * a.w + x;
        bool ok = mask_ok(coverage(a.w, a.h, s), 254);
        if( a.refM ) ok = ok && __ldg(a.refM + i) != 0;
        if( ok ) {
          const float av = __ldg(a.refT + i) - a.tshift;
          const float bv = sample_constant0(img, a.w, a.h, s) - a.tshift;
          acc[0] += av, acc[1] += bv;
          acc[2] = fmaf(av, av, acc[2]);
          acc[3] = fmaf(bv, bv, acc[3]);
          acc[4] = fmaf(av, bv, acc[4]);
          acc[5] += 1.f;
        }
      }
    }
    warp_sums_to<NS>(acc, &s_red[b][(threadIdx.x >> 5) * NS]);
  }
  __syncthreads();
  if( pf >= 0 && (threadIdx.x >> 5) == 1 ) {
    const int lane = threadIdx.x & 31;
    if( lane < NS ) {
      double sum = 0;
#pragma unroll
      for( int wv = 0; wv < 8; ++wv ) sum += (double) s_red[b ^ 1][wv * NS + lane];
      a.partials[(size_t) pf * a.part_stride + (size_t) pt * NS + lane] = sum;
    }
  }
  if( threadIdx.x == 0 ) inflight_drain(&s_infl, s_bar);
  if( timed_out && a.err ) atomicExch(a.err, 1);
}

cudaError_t launch_correlation(const CorrArgs & a, int grid, cudaStream_t st, const CUtensorMap * map)
{
  const int fam = motion_family(a.model.type);
  if( map && !a.roi && fam != FAM_QUAD ) {
    if( fam == FAM_AFFINE ) k_correlation_tma<FAM_AFFINE><<<grid, 256, 0, st>>>(a, *map);
    else k_correlation_tma<FAM_HOMOG><<<grid, 256, 0, st>>>(a, *map);
  }
  else switch ( fam ) {
  case FAM_AFFINE: k_correlation<FAM_AFFINE><<<grid, 256, 0, st>>>(a); break;
  case FAM_HOMOG: k_correlation<FAM_HOMOG><<<grid, 256, 0, st>>>(a); break;
  default: k_correlation<FAM_QUAD><<<grid, 256, 0, st>>>(a); break;
  }
  cudaError_t e = cudaGetLastError();
  if( e != cudaSuccess ) return e;
  k_correlation_finish<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

/* ---------------------------------------------------------- ROI scan */

/* Exclusive prefix sums of the tile counts of the active list's frames at
 * `level` (one CTA; a list of up to a few thousand frames) and their total. */
__global__ void __launch_bounds__(1024) k_roi_scan(const int * list, const int * count, const RoiLevel * roi,
    int lmax, int level, int * prefix, int * total)
{
  __shared__ int s_w[32];
  __shared__ int s_base;
  const int n = __ldcg(count);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if( threadIdx.x == 0 ) s_base = 0;
  __syncthreads();
  for( int k0 = 0; k0 < n; k0 += 1024 ) {
    const int k = k0 + threadIdx.x;
    const int v = k < n ? roi[(size_t) __ldcg(list + k) * lmax + level].tiles : 0;
    int incl = v;
#pragma unroll
    for( int o = 1; o < 32; o <<= 1 ) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if( lane >= o ) incl += u;
    }
    if( lane == 31 ) s_w[wid] = incl;
    __syncthreads();
    if( wid == 0 ) {
      int x = s_w[lane];
#pragma unroll
      for( int o = 1; o < 32; o <<= 1 ) {
        const int u = __shfl_up_sync(0xffffffffu, x, o);
        if( lane >= o ) x += u;
      }
      s_w[lane] = x;
    }
    __syncthreads();
    const int base = s_base + (wid > 0 ? s_w[wid - 1] : 0);
    if( k < n ) prefix[k] = base + incl - v;
    __syncthreads();
    if( threadIdx.x == 0 ) s_base += s_w[31];
    __syncthreads();
  }
  if( threadIdx.x == 0 ) *total = s_base;
}

cudaError_t launch_roi_scan(const int * list, const int * count, const RoiLevel * roi, int lmax, int level,
    int * prefix, int * total, cudaStream_t st)
{
  k_roi_scan<<<1, 1024, 0, st>>>(list, count, roi, lmax, level, prefix, total);
  return cudaGetLastError();
}

/* ----------------------------------------------------------- finalize */

__global__ void k_finalize(FinalizeArgs a)
{
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if( f >= a.n ) return;
  FrameState * F = a.fs + f;
  double p[12] = { 0 };
  model_get_params(a.model, F->state, p);
  const int M = model_nparams(a.model);
  for( int j = 0; j < 12; ++j ) a.params_out[(size_t) f * 12 + j] = j < M ? (float) p[j] : 0.f;
  if( F->status == SST_FRAME_OK && !state_finite(F->state, 16) ) F->status = SST_FRAME_NAN;
  double w = 0;
  if( a.lap_partials ) {
    double s = 0, n = 0;
    const double * P = a.lap_partials + (size_t) f * a.lap_tiles * 2;
    for( int t = 0; t < a.lap_tiles; ++t ) s += P[2 * t], n += P[2 * t + 1];
    w = n > 0 ? s / n : 0;
  }
  F->weight = (float) w;
  if( a.status_out ) a.status_out[f] = F->status;
  if( a.iters_out ) a.iters_out[f] = F->total_iters;
  if( a.eps_out ) a.eps_out[f] = (float) F->eps;
  if( a.rho_out ) a.rho_out[f] = F->rho;
  if( a.weight_out ) a.weight_out[f] = F->weight;
}

cudaError_t launch_finalize(const FinalizeArgs & a, cudaStream_t st)
{
  k_finalize<<<(a.n + 127) / 128, 128, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace sst
