/*
 * sst_refcpu.cc -- FP32 CPU restatement of the reference's headline stacking
 * path, with the reference's data flow: the timed CPU baseline.
 *
 * TEST / BASELINE INFRASTRUCTURE ONLY: bench.py's cpu_baseline leg and
 * --impl reference arm time it; tests/ check it against the FP64 oracle. The
 * product never links or calls it.
 *
 * The reference itself cannot be built here (its CMake requires OpenCV, TBB
 * and libconfig). This restates, per frame, the sequence of full-image
 * operations the reference performs for register_frame with c_ecch (IC) and
 * the stacking pipeline's remap + weighted-average body, each one an
 * OpenMP loop over rows with a static partition, as the reference's
 * parallel_for with tbb::static_partitioner (core/proc/run-loop.h:13-20)
 * distributes cv:: row ranges. Images are FP32 (cv::Mat1f); dot products
 * accumulate in FP64 as cv::Mat::dot does; the accumulator is the reference's
 * FP32 running mean. Per frame (core/proc/image_registration/ecc2.cc and
 * c_frame_registration.cc unless stated):
 *
 *   set_current_image  ecc2.cc:1060-1120  convert (x scale), GaussianBlur
 *                      (sepFilter2D, REPLICATE), pyrDown per level
 *   align per pass     ecc2.cc:1133-1176  scale_transfrom to the coarsest
 *                      level, then per level c_ecc_inverse_compositional::
 *                      align (ecc2.cc:1693-1788), per iteration:
 *                        create_remap (Mat2f)     ecc2.cc:181-188
 *                        remap image (REPLICATE)  ecc2.cc:188
 *                        remap 255-mask, >= 250   ecc2.cc:190-216
 *                        subtract, setTo(~mask)   ecc2.cc:1750-1753
 *                        countNonZero, norm L2SQR ecc2.cc:1755-1762
 *                        M dot products, solve    ecc2.cc:295-338, 1763-1765
 *                        invert_and_compose, eps  ecc2.cc:1771-1784
 *   compute_correlation  ecc2.cc:100-137 (remap, >= 254 mask, means, dots)
 *   base_remap           c_frame_registration.cc:1265-1340 (create_remap,
 *                        remap REFLECT101, mask remap >= 255, erode 5 x 5)
 *   weights x mask, _weighted_average_update  c_frame_accumulation.cc:20-129
 *
 * The steepest-descent images and Gauss-Newton matrix of each reference
 * level are computed once per model, as the reference caches them
 * (ecc2.cc:1731-1738). Scalar per-iteration work (eps, composition, the
 * M x M Cholesky) reuses the oracle's model functions.
 */
#include "sst_oracle.h"
#include <cmath>
#include <cfloat>
#include <cstring>
#include <vector>
#include <algorithm>
#include <map>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Img {
  int w = 0, h = 0;
  std::vector<float> d;
  void create(int ww, int hh) { w = ww, h = hh, d.resize((size_t) ww * hh); }
  float * row(int y) { return d.data() + (size_t) y * w; }
  const float * row(int y) const { return d.data() + (size_t) y * w; }
};

struct Msk {
  int w = 0, h = 0;
  std::vector<uint8_t> d;
  void create(int ww, int hh) { w = ww, h = hh, d.resize((size_t) ww * hh); }
};

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

inline int reflect101(int p, int n)
{
  if( n == 1 ) return 0;
  while ( p < 0 || p >= n ) p = p < 0 ? -p : 2 * (n - 1) - p;
  return p;
}

/* cv::sepFilter2D(src, dst, CV_32F, kx, ky), BORDER_REPLICATE */
void sep_filter(const Img & s, const float * kx, int nx, const float * ky, int ny, Img & d)
{
  Img t;
  t.create(s.w, s.h);
  d.create(s.w, s.h);
  const int rx = nx / 2, ry = ny / 2;
#pragma omp parallel for schedule(static)
  for( int y = 0; y < s.h; ++y ) {
    const float * sr = s.row(y);
    float * tr = t.row(y);
    for( int x = 0; x < s.w; ++x ) {
      float a = 0;
      for( int i = 0; i < nx; ++i ) a += kx[i] * sr[clampi(x + i - rx, 0, s.w - 1)];
      tr[x] = a;
    }
  }
#pragma omp parallel for schedule(static)
  for( int y = 0; y < s.h; ++y ) {
    float * dr = d.row(y);
    for( int x = 0; x < s.w; ++x ) dr[x] = 0;
    for( int j = 0; j < ny; ++j ) {
      const float * tr = t.row(clampi(y + j - ry, 0, s.h - 1));
      for( int x = 0; x < s.w; ++x ) dr[x] += ky[j] * tr[x];
    }
  }
}

void gaussian(const Img & s, double sigma, Img & d)
{
  double k[256];
  const int n = orc_gaussian_kernel(sigma, k);
  float kf[256];
  for( int i = 0; i < n; ++i ) kf[i] = (float) k[i];
  sep_filter(s, kf, n, kf, n, d);
}

/* cv::pyrDown to (dw, dh), BORDER_REFLECT_101 */
void pyrdown(const Img & s, int dw, int dh, Img & d)
{
  static const float k[5] = { 1 / 16.f, 4 / 16.f, 6 / 16.f, 4 / 16.f, 1 / 16.f };
  Img t;
  t.create(dw, s.h);
  d.create(dw, dh);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < s.h; ++y ) {
    const float * sr = s.row(y);
    float * tr = t.row(y);
    for( int x = 0; x < dw; ++x ) {
      float a = 0;
      for( int i = 0; i < 5; ++i ) a += k[i] * sr[reflect101(2 * x + i - 2, s.w)];
      tr[x] = a;
    }
  }
#pragma omp parallel for schedule(static)
  for( int y = 0; y < dh; ++y ) {
    float * dr = d.row(y);
    for( int x = 0; x < dw; ++x ) dr[x] = 0;
    for( int j = 0; j < 5; ++j ) {
      const float * tr = t.row(reflect101(2 * y + j - 2, s.h));
      for( int x = 0; x < dw; ++x ) dr[x] += k[j] * tr[x];
    }
  }
}

/* the warp as a 3 x 3 matrix (projective family) */
void warp_matrix(const orc_model * m, const double * s, double * M)
{
  if( m->type == ORC_MOTION_HOMOGRAPHY || m->type == ORC_MOTION_EPIPOLAR_DEROTATION ) {
    for( int i = 0; i < 8; ++i ) M[i] = s[i];
    M[8] = 1;
    return;
  }
  double x0, y0, x1, y1, x2, y2;
  orc_model_warp(m, s, 0, 0, &x0, &y0);
  orc_model_warp(m, s, 1, 0, &x1, &y1);
  orc_model_warp(m, s, 0, 1, &x2, &y2);
  M[0] = x1 - x0, M[1] = x2 - x0, M[2] = x0;
  M[3] = y1 - y0, M[4] = y2 - y0, M[5] = y0;
  M[6] = 0, M[7] = 0, M[8] = 1;
}

/* c_image_transform::create_remap: Mat2f of W(x, y) */
void create_remap(const orc_model * m, const double * s, int w, int h, std::vector<float> & map)
{
  double M[9];
  warp_matrix(m, s, M);
  const float a0 = (float) M[0], a1 = (float) M[1], a2 = (float) M[2], a3 = (float) M[3], a4 = (float) M[4],
      a5 = (float) M[5], a6 = (float) M[6], a7 = (float) M[7];
  map.resize((size_t) w * h * 2);
  const bool proj = a6 != 0 || a7 != 0;
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    float * mp = map.data() + (size_t) y * w * 2;
    for( int x = 0; x < w; ++x ) {
      const float X = a0 * x + a1 * y + a2, Y = a3 * x + a4 * y + a5;
      if( proj ) {
        const float iw = 1.f / (a6 * x + a7 * y + 1.f);
        mp[2 * x] = X * iw, mp[2 * x + 1] = Y * iw;
      }
      else mp[2 * x] = X, mp[2 * x + 1] = Y;
    }
  }
}

enum { B_CONST = 0, B_REPL = 1, B_R101 = 4 };

/* cv::remap INTER_LINEAR of an f32 image */
void remap_img(const Img & s, const std::vector<float> & map, int w, int h, int border, Img & d)
{
  d.create(w, h);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    const float * mp = map.data() + (size_t) y * w * 2;
    float * dr = d.row(y);
    for( int x = 0; x < w; ++x ) {
      const float X = mp[2 * x], Y = mp[2 * x + 1];
      const float fx0 = std::floor(X), fy0 = std::floor(Y);
      const int x0 = (int) fx0, y0 = (int) fy0;
      const float fx = X - fx0, fy = Y - fy0;
      float v[4];
      for( int q = 0; q < 4; ++q ) {
        int xi = x0 + (q & 1), yi = y0 + (q >> 1);
        if( xi < 0 || xi >= s.w || yi < 0 || yi >= s.h ) {
          if( border == B_CONST ) {
            v[q] = 0;
            continue;
          }
          if( border == B_REPL ) xi = clampi(xi, 0, s.w - 1), yi = clampi(yi, 0, s.h - 1);
          else xi = reflect101(xi, s.w), yi = reflect101(yi, s.h);
        }
        v[q] = s.d[(size_t) yi * s.w + xi];
      }
      dr[x] = (1 - fy) * ((1 - fx) * v[0] + fx * v[1]) + fy * ((1 - fx) * v[2] + fx * v[3]);
    }
  }
}

/* cv::remap INTER_LINEAR, BORDER_CONSTANT 0 of an all-255 u8 image, rounded */
void remap_full_mask(int sw, int sh, const std::vector<float> & map, int w, int h, Msk & d)
{
  d.create(w, h);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    const float * mp = map.data() + (size_t) y * w * 2;
    uint8_t * dr = d.d.data() + (size_t) y * w;
    for( int x = 0; x < w; ++x ) {
      const float X = mp[2 * x], Y = mp[2 * x + 1];
      const float fx0 = std::floor(X), fy0 = std::floor(Y);
      const int x0 = (int) fx0, y0 = (int) fy0;
      const float fx = X - fx0, fy = Y - fy0;
      const float cx = (x0 >= 0 && x0 < sw ? 1 - fx : 0) + (x0 + 1 >= 0 && x0 + 1 < sw ? fx : 0);
      const float cy = (y0 >= 0 && y0 < sh ? 1 - fy : 0) + (y0 + 1 >= 0 && y0 + 1 < sh ? fy : 0);
      dr[x] = (uint8_t) std::lround(255.f * cx * cy);
    }
  }
}

/* cv::compare(m, thr, CMP_GE) */
void compare_ge(Msk & m, int thr)
{
#pragma omp parallel for schedule(static)
  for( int y = 0; y < m.h; ++y ) {
    uint8_t * r = m.d.data() + (size_t) y * m.w;
    for( int x = 0; x < m.w; ++x ) r[x] = r[x] >= thr ? 255 : 0;
  }
}

/* cv::erode 5 x 5, BORDER_CONSTANT 255 (the window clipped to the image) */
void erode5(Msk & m)
{
  Msk t;
  t.create(m.w, m.h);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < m.h; ++y ) {
    const uint8_t * r = m.d.data() + (size_t) y * m.w;
    uint8_t * tr = t.d.data() + (size_t) y * m.w;
    for( int x = 0; x < m.w; ++x ) {
      uint8_t v = 255;
      for( int i = std::max(0, x - 2); i <= std::min(m.w - 1, x + 2); ++i ) v = std::min(v, r[i]);
      tr[x] = v;
    }
  }
#pragma omp parallel for schedule(static)
  for( int y = 0; y < m.h; ++y ) {
    uint8_t * r = m.d.data() + (size_t) y * m.w;
    for( int x = 0; x < m.w; ++x ) {
      uint8_t v = 255;
      for( int j = std::max(0, y - 2); j <= std::min(m.h - 1, y + 2); ++j ) v = std::min(v, t.d[(size_t) j * m.w + x]);
      r[x] = v;
    }
  }
}

double dot(const float * a, const float * b, size_t n)
{
  double s = 0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for( long i = 0; i < (long) n; ++i ) s += (double) a[i] * b[i];
  return s;
}

bool cholesky_solve(const float * A, const float * b, int n, float * x)
{
  double L[144] = { 0 };
  for( int i = 0; i < n; ++i ) {
    for( int j = 0; j <= i; ++j ) {
      double s = A[i * n + j];
      for( int k = 0; k < j; ++k ) s -= L[i * 12 + k] * L[j * 12 + k];
      if( i == j ) {
        if( s <= 0 ) return false;
        L[i * 12 + i] = std::sqrt(s);
      }
      else L[i * 12 + j] = s / L[j * 12 + j];
    }
  }
  double y[12];
  for( int i = 0; i < n; ++i ) {
    double s = b[i];
    for( int k = 0; k < i; ++k ) s -= L[i * 12 + k] * y[k];
    y[i] = s / L[i * 12 + i];
  }
  for( int i = n - 1; i >= 0; --i ) {
    double s = y[i];
    for( int k = i + 1; k < n; ++k ) s -= L[k * 12 + i] * x[k];
    x[i] = (float) (s / L[i * 12 + i]);
  }
  return true;
}

struct RefLevel {
  Img img, gx, gy;
  std::map<int, std::vector<Img>> J;     // per model: M steepest-descent images
  std::map<int, std::vector<float>> H;   // per model: M x M
};

/* ecc_differentiate (ecc2.cc:142-169) */
void differentiate(const Img & s, Img & gx, Img & gy)
{
  static const float d5[5] = { 1.f / 12, -2.f / 3, 0.f, 2.f / 3, -1.f / 12 };
  static const float s3[3] = { 0.25f, 0.5f, 0.25f };
  sep_filter(s, d5, 5, s3, 3, gx);
  sep_filter(s, s3, 3, d5, 5, gy);
}

/* create_steepest_descent_images + ecc_compute_hessian_matrix at the identity */
void ensure_jacobian(RefLevel & L, const orc_model * m)
{
  const int key = m->type * 16 + orc_model_nparams(m);
  if( L.J.count(key) ) return;
  const int M = orc_model_nparams(m), w = L.img.w, h = L.img.h;
  double id[16];
  orc_model_identity(m, id);
  std::vector<Img> & J = L.J[key];
  J.resize(M);
  for( Img & j : J ) j.create(w, h);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    double jr[12];
    for( int x = 0; x < w; ++x ) {
      const size_t i = (size_t) y * w + x;
      orc_model_sd(m, id, x, y, L.gx.d[i], L.gy.d[i], jr);
      for( int a = 0; a < M; ++a ) J[a].d[i] = (float) jr[a];
    }
  }
  std::vector<float> & H = L.H[key];
  H.assign((size_t) M * M, 0.f);
  const size_t N = (size_t) w * h;
  for( int a = 0; a < M; ++a )
    for( int b = 0; b <= a; ++b ) H[a * M + b] = H[b * M + a] = (float) dot(J[a].d.data(), J[b].d.data(), N);
}

/* c_ecc_inverse_compositional::align (ecc2.cc:1693-1788) at one level */
void align_ic(RefLevel & R, const Img & cur, const orc_model * m, double * state, int max_it, double max_eps,
    double step)
{
  ensure_jacobian(R, m);
  const int key = m->type * 16 + orc_model_nparams(m);
  const std::vector<Img> & J = R.J[key];
  const std::vector<float> & H = R.H[key];
  const int M = orc_model_nparams(m), w = R.img.w, h = R.img.h;
  const size_t N = (size_t) w * h;
  const double RMA = (double) N;
  std::vector<float> map;
  Img rem, rhs;
  Msk rmask, inv;
  double rmsold = FLT_MAX;
  int n = 0;
  while ( n++ < max_it ) {
    create_remap(m, state, w, h, map);
    remap_img(cur, map, w, h, B_REPL, rem);
    remap_full_mask(cur.w, cur.h, map, w, h, rmask);
    compare_ge(rmask, 250);
    rhs.create(w, h);
#pragma omp parallel for schedule(static)
    for( long i = 0; i < (long) N; ++i ) rhs.d[i] = rem.d[i] - R.img.d[i];
    inv.create(w, h);
#pragma omp parallel for schedule(static)
    for( long i = 0; i < (long) N; ++i ) inv.d[i] = (uint8_t) ~rmask.d[i];
#pragma omp parallel for schedule(static)
    for( long i = 0; i < (long) N; ++i ) if( inv.d[i] ) rhs.d[i] = 0;
    long cnt = 0;
#pragma omp parallel for schedule(static) reduction(+ : cnt)
    for( long i = 0; i < (long) N; ++i ) cnt += rmask.d[i] != 0;
    const double CMA = (double) cnt;
    const double rmsnew = dot(rhs.d.data(), rhs.d.data(), N) * (RMA * RMA) / (CMA * CMA);
    float v[12], dp[12];
    for( int a = 0; a < M; ++a ) v[a] = (float) (dot(J[a].d.data(), rhs.d.data(), N) * (RMA / CMA));
    if( !cholesky_solve(H.data(), v, M, dp) ) for( int a = 0; a < M; ++a ) dp[a] = 0;
    if( rmsnew >= rmsold ) break;
    double sdp[16] = { 0 }, dpd[16] = { 0 }, ns[16];
    for( int a = 0; a < M; ++a ) sdp[a] = step * dp[a], dpd[a] = dp[a];
    orc_model_invert_and_compose(m, state, sdp, ns);
    rmsold = rmsnew;
    memcpy(state, ns, sizeof(ns));
    if( orc_model_eps(m, state, dpd, w, h) < max_eps ) break;
  }
}

/* affine-family state conversion between passes (set_parameters of the next model) */
void convert(const orc_model * from, const double * s, const orc_model * to, double * out)
{
  orc_model_identity(to, out);
  if( from->type == to->type ) {
    memcpy(out, s, 16 * sizeof(double));
    return;
  }
  double M[9];
  warp_matrix(from, s, M);
  switch ( to->type ) {
  case ORC_MOTION_TRANSLATION: out[0] = M[2], out[1] = M[5]; break;
  case ORC_MOTION_AFFINE: for( int i = 0; i < 6; ++i ) out[i] = M[i]; break;
  case ORC_MOTION_HOMOGRAPHY: for( int i = 0; i < 8; ++i ) out[i] = M[i]; break;
  default: break;
  }
}

void build_pyramid(Img & l0, int levels, std::vector<Img> & P)
{
  P.resize(levels);
  P[0] = std::move(l0);
  for( int l = 1; l < levels; ++l ) {
    const int nw = ((P[l - 1].w + 1) >> 1) & ~1, nh = ((P[l - 1].h + 1) >> 1) & ~1;
    pyrdown(P[l - 1], nw, nh, P[l]);
  }
}

}  // namespace

/* register_frame with c_ecch (IC) over the pipeline's motion passes, the
 * correlation gate, base_remap and the FP32 running weighted mean, for n
 * u16 frames (reference: f32, already scaled). acc / accw: the running mean
 * and its weight sum (w x h f32, zero before the first call). */
extern "C" int ref_register_and_stack(const orc_pipeline_opts * o, const float * ref, int w, int h,
    const uint16_t * frames, int n, double frame_scale, double * out_states, int * out_status, double * out_rho,
    float * acc, float * accw)
{
  const int L = orc_ecch_num_levels(w, h, &o->ecch);
  // set_reference_image (ecc2.cc:984-1057): smooth, pyramid, gradients
  std::vector<RefLevel> R(L);
  {
    Img r0, s0;
    r0.create(w, h);
    memcpy(r0.d.data(), ref, (size_t) w * h * sizeof(float));
    if( o->ecch.reference_smooth_sigma > 0 ) gaussian(r0, o->ecch.reference_smooth_sigma, s0);
    else s0 = r0;
    std::vector<Img> P;
    build_pyramid(s0, L, P);
    for( int l = 0; l < L; ++l ) {
      R[l].img = std::move(P[l]);
      differentiate(R[l].img, R[l].gx, R[l].gy);
    }
  }
  const size_t N = (size_t) w * h;
  Img raw, sm;
  std::vector<Img> C;
  std::vector<float> map;
  Img warped, wts;
  Msk wmask;
  for( int f = 0; f < n; ++f ) {
    // set_current_image: ecc_convert_input_image, GaussianBlur, pyramid
    raw.create(w, h);
    const uint16_t * fr = frames + (size_t) f * N;
#pragma omp parallel for schedule(static)
    for( long i = 0; i < (long) N; ++i ) raw.d[i] = (float) (fr[i] * frame_scale);
    if( o->ecch.input_smooth_sigma > 0 ) gaussian(raw, o->ecch.input_smooth_sigma, sm);
    else sm = raw;
    build_pyramid(sm, L, C);
    double state[16], prev[16];
    orc_model pm = { 0, 0, 0, 0 };
    for( int k = 0; k < o->num_passes; ++k ) {
      orc_model m = { o->pass_motion[k], 0, 0, o->pass_motion[k] == ORC_MOTION_EUCLIDEAN ? 1 : 0 };
      if( k == 0 ) orc_model_identity(&m, state);
      else convert(&pm, prev, &m, state);
      // c_ecch::align (ecc2.cc:1133-1176)
      int lvl = L - 1;
      if( lvl > 0 ) orc_model_scale(&m, state, (double) R[lvl].img.w / R[0].img.w);
      for( ; lvl >= 0; --lvl ) {
        align_ic(R[lvl], C[lvl], &m, state, o->ecch.max_iterations, o->ecch.epsx * std::pow(2.0, lvl),
            o->ecch.update_step_scale);
        if( lvl > 0 ) orc_model_scale(&m, state, (double) R[lvl - 1].img.w / R[lvl].img.w);
      }
      memcpy(prev, state, sizeof(state));
      pm = m;
    }
    // compute_correlation (ecc2.cc:100-137)
    create_remap(&pm, state, w, h, map);
    Img cw;
    Msk cm;
    remap_img(C[0], map, w, h, B_CONST, cw);
    remap_full_mask(w, h, map, w, h, cm);
    compare_ge(cm, 254);
    double s1 = 0, s2 = 0, cnt = 0;
#pragma omp parallel for schedule(static) reduction(+ : s1, s2, cnt)
    for( long i = 0; i < (long) N; ++i ) {
      if( cm.d[i] ) s1 += R[0].img.d[i], s2 += cw.d[i], cnt += 1;
    }
    double rho = 0;
    if( cnt > 0 ) {
      const double m1 = s1 / cnt, m2 = s2 / cnt;
      double v1 = 0, v2 = 0, cv = 0;
#pragma omp parallel for schedule(static) reduction(+ : v1, v2, cv)
      for( long i = 0; i < (long) N; ++i ) {
        if( cm.d[i] ) {
          const double a = R[0].img.d[i] - m1, c = cw.d[i] - m2;
          v1 += a * a, v2 += c * c, cv += a * c;
        }
      }
      rho = (cv / cnt) / (std::sqrt(v1 / cnt) * std::sqrt(v2 / cnt));
    }
    memcpy(out_states + (size_t) f * 16, state, sizeof(state));
    out_rho[f] = rho;
    if( !(rho >= o->min_rho) ) {
      out_status[f] = 3;
      continue;
    }
    out_status[f] = 0;
    // base_remap of the frame and its mask (the map is the registered transform's)
    remap_img(raw, map, w, h, o->border_mode == ORC_BORDER_REPLICATE ? B_REPL : B_R101, warped);
    remap_full_mask(w, h, map, w, h, wmask);
    compare_ge(wmask, 255);
    erode5(wmask);
    // frame weight (Laplacian energy of pyramid level 1) times the mask
    double lap = 1.0;
    if( o->use_laplacian_weights && L > 1 ) {
      const Img & l1 = C[1];
      double s = 0;
#pragma omp parallel for schedule(static) reduction(+ : s)
      for( int y = 1; y < l1.h - 1; ++y ) {
        const float * r = l1.row(y);
        for( int x = 1; x < l1.w - 1; ++x ) {
          const float v = r[x - 1] + r[x + 1] + r[x - l1.w] + r[x + l1.w] - 4 * r[x];
          s += (double) v * v;
        }
      }
      lap = s / ((double) (l1.w - 2) * (l1.h - 2));
    }
    wts.create(w, h);
#pragma omp parallel for schedule(static)
    for( long i = 0; i < (long) N; ++i ) wts.d[i] = wmask.d[i] ? (float) lap : 0.f;
    // _weighted_average_update (c_frame_accumulation.cc:83-124): FP32 running mean
#pragma omp parallel for schedule(static)
    for( long i = 0; i < (long) N; ++i ) {
      const float wn = wts.d[i];
      if( wn > 0 ) {
        const float Wn = accw[i] + wn;
        accw[i] = Wn;
        acc[i] += (warped.d[i] - acc[i]) * (wn / Wn);
      }
    }
  }
  return 0;
}
