/*
 * sst_oracle.cc -- FP64 restatement of the ECC / c_ecch / stacking hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of the parity tests and the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it.
 *
 * Reference anchors (core/proc/image_registration/ecc2.cc unless stated):
 *   compute_correlation        65-137
 *   ecc_differentiate          142-169, 1838-1863
 *   ecc_remap                  172-219, 1865-1892
 *   ecc_compute_hessian_matrix 295-321
 *   c_ecch set_reference/set_current/align  984-1176
 *   c_ecc_forward_additive     1187-1365
 *   c_ecclm                    1376-1650
 *   c_ecc_inverse_compositional 1660-1788
 *   c_ecclm_inverse_compositional 1792-2086
 *   c_frame_registration::base_remap   c_frame_registration.cc:1265-1386
 *   _weighted_average_update    core/average/c_frame_accumulation.cc:20-129
 *   _bayer_accumulate           core/average/c_frame_accumulation.cc:988-1126
 *   generate_bayer_pattern_mask core/average/c_frame_accumulation.cc:1262-1334
 *   _extract_bayer_planes       core/io/debayer.cc:96-134
 *   _average_bayer_planes       core/io/debayer.cc:277-330
 */
#include "sst_oracle.h"
#include <cmath>
#include <cstring>
#include <cfloat>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline double sq(double x) { return x * x; }

extern "C" void orc_set_num_threads(int n)
{
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void) n;
#endif
}

extern "C" int orc_get_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static inline int border_index(int p, int n, int border)
{
  if( p >= 0 && p < n ) return p;
  switch ( border ) {
  case ORC_BORDER_REPLICATE: return p < 0 ? 0 : n - 1;
  case ORC_BORDER_REFLECT101:
    if( n == 1 ) return 0;
    while ( p < 0 || p >= n ) {
      if( p < 0 ) p = -p;
      if( p >= n ) p = 2 * (n - 1) - p;
    }
    return p;
  case ORC_BORDER_REFLECT:
    while ( p < 0 || p >= n ) {
      if( p < 0 ) p = -p - 1;
      if( p >= n ) p = 2 * n - 1 - p;
    }
    return p;
  }
  return -1;   // constant
}

/* cv::getGaussianKernel(ksize, sigma > 0), ksize = max(3, 2*int(3 sigma)+1)
 * as chosen by c_ecch (ecc2.cc:1001-1003) */
extern "C" int orc_gaussian_kernel(double sigma, double * k)
{
  const int n = std::max(3, 2 * ((int) (3 * sigma)) + 1);
  const double s2 = -0.5 / (sigma * sigma);
  double sum = 0;
  for( int i = 0; i < n; ++i ) {
    const double x = i - (n - 1) * 0.5;
    k[i] = std::exp(s2 * x * x);
    sum += k[i];
  }
  for( int i = 0; i < n; ++i ) k[i] /= sum;
  return n;
}

/* cv::sepFilter2D(src, dst, kx, ky, anchor=center, delta=0, border) */
static void sep_filter(const double * src, int w, int h, const double * kx, int nx, const double * ky, int ny,
    int border, double * dst)
{
  std::vector<double> tmp((size_t) w * h);
  const int rx = nx / 2, ry = ny / 2;
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    const double * s = src + (size_t) y * w;
    double * t = tmp.data() + (size_t) y * w;
    for( int x = 0; x < w; ++x ) {
      double a = 0;
      for( int i = 0; i < nx; ++i ) a += kx[i] * s[border_index(x + i - rx, w, border)];
      t[x] = a;
    }
  }
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    double * d = dst + (size_t) y * w;
    for( int x = 0; x < w; ++x ) {
      double a = 0;
      for( int j = 0; j < ny; ++j ) a += ky[j] * tmp[(size_t) border_index(y + j - ry, h, border) * w + x];
      d[x] = a;
    }
  }
}

extern "C" void orc_smooth(const double * src, int w, int h, double sigma, double * dst)
{
  double k[256];
  const int n = orc_gaussian_kernel(sigma, k);
  sep_filter(src, w, h, k, n, k, n, ORC_BORDER_REPLICATE, dst);
}

/* cv::pyrDown: 5x5 [1 4 6 4 1]/16 separable, BORDER_REFLECT_101, dst(x,y) at src(2x,2y) */
extern "C" void orc_pyrdown(const double * src, int w, int h, double * dst, int dw, int dh)
{
  static const double k[5] = { 1 / 16., 4 / 16., 6 / 16., 4 / 16., 1 / 16. };
  std::vector<double> tmp((size_t) dw * h);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( int i = 0; i < 5; ++i ) a += k[i] * src[(size_t) y * w + border_index(2 * x + i - 2, w, ORC_BORDER_REFLECT101)];
      tmp[(size_t) y * dw + x] = a;
    }
  }
#pragma omp parallel for schedule(static)
  for( int y = 0; y < dh; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( int j = 0; j < 5; ++j ) a += k[j] * tmp[(size_t) border_index(2 * y + j - 2, h, ORC_BORDER_REFLECT101) * dw + x];
      dst[(size_t) y * dw + x] = a;
    }
  }
}

/* cv::resize(..., INTER_NEAREST): sx = floor(dx * sw/dw) */
extern "C" void orc_resize_nearest_u8(const uint8_t * src, int w, int h, uint8_t * dst, int dw, int dh)
{
  const double fx = (double) w / dw, fy = (double) h / dh;
  for( int y = 0; y < dh; ++y ) {
    const int sy = std::min((int) std::floor(y * fy), h - 1);
    for( int x = 0; x < dw; ++x ) {
      const int sx = std::min((int) std::floor(x * fx), w - 1);
      dst[(size_t) y * dw + x] = src[(size_t) sy * w + sx];
    }
  }
}

/* ecc_differentiate (ecc2.cc:142-169): gx = sepFilter2D(d5 along x, s3 along y),
 * gy = sepFilter2D(s3 along x, d5 along y), BORDER_REPLICATE, zero outside valid */
extern "C" void orc_differentiate(const double * src, int w, int h, const uint8_t * valid, double * gx, double * gy)
{
  static const double d5[5] = { 1. / 12., -2. / 3., 0., 2. / 3., -1. / 12. };
  static const double s3[3] = { 0.25, 0.5, 0.25 };
  sep_filter(src, w, h, d5, 5, s3, 3, ORC_BORDER_REPLICATE, gx);
  sep_filter(src, w, h, s3, 3, d5, 5, ORC_BORDER_REPLICATE, gy);
  if( valid ) {
    for( size_t i = 0, n = (size_t) w * h; i < n; ++i ) {
      if( !valid[i] ) gx[i] = gy[i] = 0;
    }
  }
}

/* bilinear sample with per-tap border handling (cv::remap INTER_LINEAR) */
extern "C" double orc_sample_bilinear(const double * src, int w, int h, double sx, double sy, int border, double bval)
{
  const double fx0 = std::floor(sx), fy0 = std::floor(sy);
  const double fx = sx - fx0, fy = sy - fy0;
  const int x0 = (int) fx0, y0 = (int) fy0;
  double v[4];
  const int xs[2] = { x0, x0 + 1 }, ys[2] = { y0, y0 + 1 };
  for( int j = 0; j < 2; ++j ) {
    for( int i = 0; i < 2; ++i ) {
      const int xi = border_index(xs[i], w, border), yi = border_index(ys[j], h, border);
      v[j * 2 + i] = (xi < 0 || yi < 0) ? bval : src[(size_t) yi * w + xi];
    }
  }
  return (1 - fy) * ((1 - fx) * v[0] + fx * v[1]) + fy * ((1 - fx) * v[2] + fx * v[3]);
}

/* LINEAR remap of a u8 mask (NULL = all 255) with BORDER_CONSTANT 0, divided by 255 */
extern "C" double orc_mask_coverage(const uint8_t * mask, int w, int h, double sx, double sy)
{
  const double fx0 = std::floor(sx), fy0 = std::floor(sy);
  const double fx = sx - fx0, fy = sy - fy0;
  const int x0 = (int) fx0, y0 = (int) fy0;
  const double wt[4] = { (1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy };
  double s = 0;
  for( int j = 0; j < 2; ++j ) {
    for( int i = 0; i < 2; ++i ) {
      const int xi = x0 + i, yi = y0 + j;
      if( xi >= 0 && xi < w && yi >= 0 && yi < h ) {
        const double m = mask ? mask[(size_t) yi * w + xi] / 255.0 : 1.0;
        s += wt[j * 2 + i] * m;
      }
    }
  }
  return s;
}

/* remap(mask) >= thr on a u8 result: round(255 * coverage) >= thr */
static inline bool mask_ok(double coverage, int thr)
{
  return 255.0 * coverage + 0.5 >= (double) thr;
}

/* cv::erode 5x5 of a binary mask. Every border mode used on the path
 * (REPLICATE, CONSTANT 255, morphologyDefaultBorderValue) reduces to the
 * minimum over the window clipped to the image. */
extern "C" void orc_erode5(const uint8_t * src, int w, int h, int /*border_is_max*/, uint8_t * dst)
{
  std::vector<uint8_t> tmp((size_t) w * h);
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      uint8_t m = 255;
      for( int i = std::max(0, x - 2); i <= std::min(w - 1, x + 2); ++i ) m = std::min(m, src[(size_t) y * w + i]);
      tmp[(size_t) y * w + x] = m;
    }
  }
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      uint8_t m = 255;
      for( int j = std::max(0, y - 2); j <= std::min(h - 1, y + 2); ++j ) m = std::min(m, tmp[(size_t) j * w + x]);
      dst[(size_t) y * w + x] = m;
    }
  }
}

extern "C" void orc_remap_model(const orc_model * m, const double * state, const double * src, int sw, int sh,
    int dw, int dh, int border, double bval, double * dst)
{
#pragma omp parallel for schedule(static)
  for( int y = 0; y < dh; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      double X, Y;
      orc_model_warp(m, state, x, y, &X, &Y);
      dst[(size_t) y * dw + x] = orc_sample_bilinear(src, sw, sh, X, Y, border, bval);
    }
  }
}

/* create_remap of a transform: W(x; p) at every pixel of a w x h grid */
extern "C" void orc_warp_grid(const orc_model * m, const double * state, int w, int h, double * mapx, double * mapy)
{
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      orc_model_warp(m, state, x, y, mapx + (size_t) y * w + x, mapy + (size_t) y * w + x);
    }
  }
}

/* FP64 Cholesky: solves A x = b (A n x n SPD). Returns 0 if not positive definite. */
static bool cholesky_solve(const double * A, const double * b, int n, double * x)
{
  double L[16 * 16];
  for( int i = 0; i < n; ++i ) {
    for( int j = 0; j <= i; ++j ) {
      double s = A[i * n + j];
      for( int k = 0; k < j; ++k ) s -= L[i * 16 + k] * L[j * 16 + k];
      if( i == j ) {
        if( !(s > 0) ) return false;
        L[i * 16 + i] = std::sqrt(s);
      }
      else {
        L[i * 16 + j] = s / L[j * 16 + j];
      }
    }
  }
  double yv[16];
  for( int i = 0; i < n; ++i ) {
    double s = b[i];
    for( int k = 0; k < i; ++k ) s -= L[i * 16 + k] * yv[k];
    yv[i] = s / L[i * 16 + i];
  }
  for( int i = n - 1; i >= 0; --i ) {
    double s = yv[i];
    for( int k = i + 1; k < n; ++k ) s -= L[k * 16 + i] * x[k];
    x[i] = s / L[i * 16 + i];
  }
  return true;
}

static bool all_nonzero(const uint8_t * m, size_t n)
{
  for( size_t i = 0; i < n; ++i ) if( !m[i] ) return false;
  return true;
}

namespace {

struct level_ctx {
  const orc_model * m;
  int w, h, cw, ch;
  const double * ref, * cur;
  const uint8_t * ref_mask, * cur_mask;
};

/* per-pixel warped sample + coverage of the current mask */
inline void warp_pixel(const level_ctx & c, const double * s, int x, int y, double * val, double * cov, double * X, double * Y)
{
  orc_model_warp(c.m, s, x, y, X, Y);
  *val = orc_sample_bilinear(c.cur, c.cw, c.ch, *X, *Y, ORC_BORDER_REPLICATE, 0);
  *cov = orc_mask_coverage(c.cur_mask, c.cw, c.ch, *X, *Y);
}

/* reduction helper: sums over rows in a fixed order */
struct sums {
  double v[16 + 136 + 8];
};

}  // namespace

/* ------------------------------------------------------------------------ */
/* c_ecc_forward_additive::align (ecc2.cc:1247-1365) */
static int align_fa(const level_ctx & c0, double * state, const orc_align_opts * o, int * iters, double * eps_out)
{
  level_ctx c = c0;
  const int w = c.w, h = c.h, M = orc_model_nparams(c.m);
  const size_t N = (size_t) w * h;
  // set_reference_image: release an all-nonzero mask, erode a partial one (ecc2.cc:1187-1212)
  std::vector<uint8_t> rmask, cmask;
  if( c.ref_mask ) {
    if( all_nonzero(c.ref_mask, N) ) c.ref_mask = nullptr;
    else {
      rmask.resize(N);
      orc_erode5(c.ref_mask, w, h, 0, rmask.data());
      c.ref_mask = rmask.data();
    }
  }
  // set_current_image: create an all-255 mask or erode a partial one (ecc2.cc:1215-1234)
  if( c.cur_mask && !all_nonzero(c.cur_mask, (size_t) c.cw * c.ch) ) {
    cmask.resize((size_t) c.cw * c.ch);
    orc_erode5(c.cur_mask, c.cw, c.ch, 0, cmask.data());
    c.cur_mask = cmask.data();
  }
  double max_eps = o->max_eps <= 0 ? 1e-3 : o->max_eps;

  std::vector<double> gw(N), gxw(N), gyw(N);
  std::vector<uint8_t> wmask(N);
  bool failed = false;
  int n = 0;
  double eps = FLT_MAX;
  while ( n++ < o->max_iterations ) {
#pragma omp parallel for schedule(static)
    for( int y = 0; y < h; ++y ) {
      for( int x = 0; x < w; ++x ) {
        double v, cov, X, Y;
        warp_pixel(c, state, x, y, &v, &cov, &X, &Y);
        const size_t i = (size_t) y * w + x;
        gw[i] = v;
        bool ok = mask_ok(cov, 255);
        if( c.ref_mask && !c.ref_mask[i] ) ok = false;
        wmask[i] = ok ? 255 : 0;
      }
    }
    orc_differentiate(gw.data(), w, h, wmask.data(), gxw.data(), gyw.data());
    // meanStdDev of f (ref) and g (warped) over wmask
    double nf = 0, sf = 0, sf2 = 0, sg = 0, sg2 = 0;
    for( size_t i = 0; i < N; ++i ) {
      if( wmask[i] ) {
        nf += 1, sf += c.ref[i], sg += gw[i];
      }
    }
    const double fMean = nf > 0 ? sf / nf : 0, gMean = nf > 0 ? sg / nf : 0;
    for( size_t i = 0; i < N; ++i ) {
      if( wmask[i] ) sf2 += sq(c.ref[i] - fMean), sg2 += sq(gw[i] - gMean);
    }
    const double fStd = nf > 0 ? std::sqrt(sf2 / nf) : 0, gStd = nf > 0 ? std::sqrt(sg2 / nf) : 0;
    const double ratio = gStd / fStd;
    // H and ep
    double H[144] = { 0 }, ep[12] = { 0 };
    std::vector<double> rowH((size_t) h * 144, 0.0), rowE((size_t) h * 12, 0.0);
#pragma omp parallel for schedule(static)
    for( int y = 0; y < h; ++y ) {
      double * hh = &rowH[(size_t) y * 144];
      double * ee = &rowE[(size_t) y * 12];
      for( int x = 0; x < w; ++x ) {
        const size_t i = (size_t) y * w + x;
        double J[12];
        orc_model_sd(c.m, state, x, y, gxw[i], gyw[i], J);
        const double rhs = wmask[i] ? (gw[i] - ratio * c.ref[i]) - (gMean - ratio * fMean) : 0.0;
        for( int a = 0; a < M; ++a ) {
          ee[a] += J[a] * rhs;
          for( int b = 0; b <= a; ++b ) hh[a * 12 + b] += J[a] * J[b];
        }
      }
    }
    for( int y = 0; y < h; ++y ) {
      for( int a = 0; a < M; ++a ) {
        ep[a] += rowE[(size_t) y * 12 + a];
        for( int b = 0; b <= a; ++b ) H[a * M + b] += rowH[(size_t) y * 144 + a * 12 + b];
      }
    }
    for( int a = 0; a < M; ++a ) for( int b = a + 1; b < M; ++b ) H[a * M + b] = H[b * M + a];
    double x[12];
    if( !cholesky_solve(H, ep, M, x) ) {
      failed = true;
      break;
    }
    double dp[12], p[12];
    for( int a = 0; a < M; ++a ) dp[a] = -o->update_step_scale * x[a];
    orc_model_get_params(c.m, state, p);
    for( int a = 0; a < M; ++a ) p[a] += dp[a];
    orc_model_set_params(c.m, state, p);
    eps = orc_model_eps(c.m, state, dp, w, h);
    if( eps < max_eps ) break;
  }
  *iters = n;
  *eps_out = eps;
  return !failed;
}

/* r = I(W) - T, coverage, count: shared by IC / LM / IC-LM */
namespace {
struct resid_img {
  std::vector<double> img;    // remapped current
  std::vector<uint8_t> ok;    // valid pixels
  std::vector<double> rhs;
  double count = 0, ssq = 0;
};
}

/* ecc_remap free function (ecc2.cc:176-219): LINEAR image / REPLICATE, mask LINEAR
 * CONSTANT 0 >= 250; IC-LM variant (ecc2.cc:1865-1892): inverse mask NEAREST with
 * border 255. */
static void compute_resid(const level_ctx & c, const double * state, bool nearest_inv_mask, bool apply_ref_mask,
    resid_img & r)
{
  const int w = c.w, h = c.h;
  const size_t N = (size_t) w * h;
  r.img.resize(N), r.ok.resize(N), r.rhs.resize(N);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      const size_t i = (size_t) y * w + x;
      double X, Y;
      orc_model_warp(c.m, state, x, y, &X, &Y);
      const double v = orc_sample_bilinear(c.cur, c.cw, c.ch, X, Y, ORC_BORDER_REPLICATE, 0);
      bool ok;
      if( nearest_inv_mask ) {
        const double rx = std::nearbyint(X), ry = std::nearbyint(Y);
        if( rx < 0 || ry < 0 || rx >= c.cw || ry >= c.ch ) ok = false;
        else ok = !c.cur_mask || c.cur_mask[(size_t) ry * c.cw + (size_t) rx] != 0;
      }
      else {
        ok = mask_ok(orc_mask_coverage(c.cur_mask, c.cw, c.ch, X, Y), 250);
      }
      if( apply_ref_mask && c.ref_mask && !c.ref_mask[i] ) ok = false;
      r.img[i] = v;
      r.ok[i] = ok;
      r.rhs[i] = ok ? v - c.ref[i] : 0.0;
    }
  }
  double cnt = 0, ssq = 0;
  for( size_t i = 0; i < N; ++i ) {
    cnt += r.ok[i] ? 1 : 0;
    ssq += r.rhs[i] * r.rhs[i];
  }
  r.count = cnt, r.ssq = ssq;
}

/* v_i = sum J_i rhs, H = sum J J over the level, J from gradients gx, gy
 * evaluated with the given state */
static void project(const level_ctx & c, const double * jstate, const double * gx, const double * gy,
    const double * rhs, double * v, double * H)
{
  const int w = c.w, h = c.h, M = orc_model_nparams(c.m);
  std::vector<double> rowH(H ? (size_t) h * 144 : 0, 0.0), rowV((size_t) h * 12, 0.0);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < h; ++y ) {
    double * vv = &rowV[(size_t) y * 12];
    double * hh = H ? &rowH[(size_t) y * 144] : nullptr;
    for( int x = 0; x < w; ++x ) {
      const size_t i = (size_t) y * w + x;
      double J[12];
      orc_model_sd(c.m, jstate, x, y, gx[i], gy[i], J);
      if( rhs ) for( int a = 0; a < M; ++a ) vv[a] += J[a] * rhs[i];
      if( hh ) for( int a = 0; a < M; ++a ) for( int b = 0; b <= a; ++b ) hh[a * 12 + b] += J[a] * J[b];
    }
  }
  if( v ) {
    for( int a = 0; a < M; ++a ) v[a] = 0;
    for( int y = 0; y < h; ++y ) for( int a = 0; a < M; ++a ) v[a] += rowV[(size_t) y * 12 + a];
  }
  if( H ) {
    for( int a = 0; a < M * M; ++a ) H[a] = 0;
    for( int y = 0; y < h; ++y )
      for( int a = 0; a < M; ++a ) for( int b = 0; b <= a; ++b ) H[a * M + b] += rowH[(size_t) y * 144 + a * 12 + b];
    for( int a = 0; a < M; ++a ) for( int b = a + 1; b < M; ++b ) H[a * M + b] = H[b * M + a];
  }
}

/* c_ecc_inverse_compositional::align (ecc2.cc:1693-1788) */
static int align_ic(const level_ctx & c, double * state, const orc_align_opts * o, int * iters, double * eps_out)
{
  const orc_model * m = c.m;
  if( !orc_model_invertible(m) ) {
    *iters = 0, *eps_out = FLT_MAX;
    return 0;
  }
  const int w = c.w, h = c.h, M = orc_model_nparams(m);
  const size_t N = (size_t) w * h;
  double RMA = 0;
  if( c.ref_mask ) { for( size_t i = 0; i < N; ++i ) RMA += c.ref_mask[i] ? 1 : 0; }
  else RMA = (double) N;

  std::vector<double> gx(N), gy(N);
  orc_differentiate(c.ref, w, h, c.ref_mask, gx.data(), gy.data());
  double jstate[16];
  if( o->ic_jacobian_at_identity ) {
    orc_model_identity(m, jstate);
    if( m->type == ORC_MOTION_EUCLIDEAN || m->type == ORC_MOTION_SCALED_EUCLIDEAN ) {
      jstate[4] = state[4], jstate[5] = state[5];  // keep the centre
    }
  }
  else memcpy(jstate, state, sizeof(jstate));
  double H[144];
  project(c, jstate, gx.data(), gy.data(), nullptr, nullptr, H);

  int n = 0;
  double eps = FLT_MAX, rmsold = FLT_MAX;
  const double lambda = o->update_step_scale;
  resid_img r;
  while ( n++ < o->max_iterations ) {
    compute_resid(c, state, false, false, r);
    const double CMA = r.count;
    const double rmsnew = r.ssq * (RMA * RMA) / (CMA * CMA);
    double v[12], dpv[12];
    project(c, jstate, gx.data(), gy.data(), r.rhs.data(), v, nullptr);
    for( int a = 0; a < M; ++a ) v[a] *= RMA / CMA;
    if( !cholesky_solve(H, v, M, dpv) ) for( int a = 0; a < M; ++a ) dpv[a] = 0;
    if( rmsnew >= rmsold ) break;
    double sdp[12], ns[16];
    for( int a = 0; a < M; ++a ) sdp[a] = lambda * dpv[a];
    orc_model_invert_and_compose(m, state, sdp, ns);
    rmsold = rmsnew;
    memcpy(state, ns, sizeof(ns));
    if( (eps = orc_model_eps(m, state, dpv, w, h)) < o->max_eps ) break;
  }
  *iters = n;
  *eps_out = eps;
  return 1;
}

/* c_ecclm::align (ecc2.cc:1528-1650) */
static int align_lm(const level_ctx & c0, double * state, const orc_align_opts * o, int * iters, double * eps_out)
{
  level_ctx c = c0;
  const int w = c.w, h = c.h, M = orc_model_nparams(c.m);
  const size_t N = (size_t) w * h;
  std::vector<uint8_t> rmask;
  if( c.ref_mask ) {   // set_reference_image erodes 5x5 (ecc2.cc:1387-1391)
    rmask.resize(N);
    orc_erode5(c.ref_mask, w, h, 1, rmask.data());
    c.ref_mask = rmask.data();
  }
  const double epsx = o->max_eps, epse = 1e-4;
  double lambda = 0.1;
  int iteration = 0;
  bool converged = false;
  double eps = FLT_MAX;
  std::vector<double> gx(N), gy(N);
  resid_img r;
  double p[12], newp[12], H[144], Hp[144], v[12], dpv[12];
  orc_model_get_params(c.m, state, p);
  while ( iteration < o->max_iterations ) {
    // compute_jac(params): remap, rhs, rms, gradients of the remapped image, SD, v, H
    compute_resid(c, state, false, true, r);
    const double err = r.ssq;
    orc_differentiate(r.img.data(), w, h, r.ok.data(), gx.data(), gy.data());
    project(c, state, gx.data(), gy.data(), r.rhs.data(), v, H);
    if( err < 1 ) {
      converged = true;
      break;
    }
    memcpy(Hp, H, sizeof(H));
    while ( iteration++ < o->max_iterations ) {
      for( int i = 0; i < M; ++i ) H[i * M + i] = (1 + lambda) * Hp[i * M + i];
      if( !cholesky_solve(H, v, M, dpv) ) for( int a = 0; a < M; ++a ) dpv[a] = 0;
      for( int a = 0; a < M; ++a ) newp[a] = p[a] - o->update_step_scale * dpv[a];
      if( (eps = orc_model_eps(c.m, state, dpv, w, h)) <= epsx ) {
        orc_model_set_params(c.m, state, newp);
        memcpy(p, newp, sizeof(p));
        converged = true;
        break;
      }
      double tstate[16];
      memcpy(tstate, state, sizeof(tstate));
      orc_model_set_params(c.m, tstate, newp);
      resid_img rt;
      compute_resid(c, tstate, false, true, rt);
      const double newerr = rt.ssq;
      if( newerr > err ) {
        if( lambda > 1e6 ) break;
        lambda *= 10.0;
        continue;
      }
      orc_model_set_params(c.m, state, newp);
      memcpy(p, newp, sizeof(p));
      const double diff = err - newerr;
      if( diff < err * epse ) {
        converged = true;
        break;
      }
      double dS = 0;
      for( int a = 0; a < M; ++a ) {
        double t = 2 * v[a];
        for( int b = 0; b < M; ++b ) t -= Hp[a * M + b] * dpv[b];
        dS += dpv[a] * t;
      }
      const double rho = std::fabs(dS) > 1e-9 ? diff / std::fabs(dS) : diff;
      if( rho > 0.25 ) lambda = std::max(1e-8, 0.2 * lambda);
      else if( rho < 0.1 ) lambda = lambda < 1.0 ? 1.0 : lambda * 10.0;
      break;
    }
    if( converged ) break;
  }
  *iters = iteration;
  *eps_out = eps;
  return converged;
}

/* c_ecclm_inverse_compositional::align (ecc2.cc:1926-2086) */
static int align_iclm(const level_ctx & c, double * state, const orc_align_opts * o, int * iters, double * eps_out)
{
  const orc_model * m = c.m;
  if( !orc_model_invertible(m) ) {
    *iters = 0, *eps_out = FLT_MAX;
    return 0;
  }
  const int w = c.w, h = c.h, M = orc_model_nparams(m);
  const size_t N = (size_t) w * h;
  double RMA = 0;
  if( c.ref_mask ) { for( size_t i = 0; i < N; ++i ) RMA += c.ref_mask[i] ? 1 : 0; }
  else RMA = (double) N;
  std::vector<double> gx(N), gy(N);
  orc_differentiate(c.ref, w, h, c.ref_mask, gx.data(), gy.data());
  double jstate[16];
  if( o->ic_jacobian_at_identity ) {
    orc_model_identity(m, jstate);
    if( m->type == ORC_MOTION_EUCLIDEAN || m->type == ORC_MOTION_SCALED_EUCLIDEAN ) {
      jstate[4] = state[4], jstate[5] = state[5];
    }
  }
  else memcpy(jstate, state, sizeof(jstate));
  double Hp[144], H[144];
  project(c, jstate, gx.data(), gy.data(), nullptr, nullptr, Hp);

  double lambda = 0.001, dp = 0, err = 0, newerr = 0;
  bool recompute = true;
  int n = 0;
  resid_img r;
  double v[12], dpv[12] = { 0 }, newstate[16];
  double CMA = (double) N;
  auto compute_rhs = [&](const double * s, resid_img & rr, double & cma) -> double {
    compute_resid(c, s, true, true, rr);
    cma = rr.count;
    return rr.ssq * (RMA * RMA) / (cma * cma);
  };
  double last_rms = 0;
  while ( n < o->max_iterations ) {
    if( recompute ) last_rms = compute_rhs(state, r, CMA);
    project(c, jstate, gx.data(), gy.data(), r.rhs.data(), v, nullptr);
    for( int a = 0; a < M; ++a ) v[a] *= RMA / CMA;
    memcpy(H, Hp, sizeof(H));
    err = last_rms;
    do {
      ++n;
      recompute = true;
      for( int i = 0; i < M; ++i ) H[i * M + i] = (1 + lambda) * Hp[i * M + i];
      if( !cholesky_solve(H, v, M, dpv) ) for( int a = 0; a < M; ++a ) dpv[a] = 0;
      double sdp[12];
      for( int a = 0; a < M; ++a ) sdp[a] = o->update_step_scale * dpv[a];
      orc_model_invert_and_compose(m, state, sdp, newstate);
      resid_img rt;
      double cmat;
      newerr = compute_rhs(newstate, rt, cmat);
      // the trial residual becomes the object's _rhs / CMA (ecc2.cc:1894-1916)
      r = std::move(rt);
      CMA = cmat;
      last_rms = newerr;
      if( (dp = orc_model_eps(m, state, dpv, w, h)) < o->max_eps ) break;
      double dS = 0;
      for( int a = 0; a < M; ++a ) {
        double t = 2 * v[a];
        for( int b = 0; b < M; ++b ) t -= Hp[a * M + b] * dpv[b];
        dS += dpv[a] * t;
      }
      const double rho = (err - newerr) / (std::fabs(dS) > DBL_EPSILON ? dS : 1);
      if( rho > 0.25 ) {
        if( lambda > 1e-6 ) lambda = std::max(1e-6, lambda / 5);
      }
      else if( rho > 0.1 ) {
      }
      else if( lambda < 1 ) lambda = 1;
      else lambda *= 10;
      if( newerr < err ) break;
    } while ( n < o->max_iterations );
    if( newerr < err ) {
      err = newerr;
      recompute = false;
      memcpy(state, newstate, sizeof(newstate));
    }
    if( dp < o->max_eps ) break;
  }
  *iters = n;
  *eps_out = dp;
  return 1;
}

extern "C" int orc_ecc_align(const orc_model * m, double * state, const orc_level * l, const orc_align_opts * o,
    int * iters, double * eps)
{
  level_ctx c;
  c.m = m;
  c.w = l->w, c.h = l->h, c.cw = l->cw, c.ch = l->ch;
  c.ref = l->ref, c.cur = l->cur, c.ref_mask = l->ref_mask, c.cur_mask = l->cur_mask;
  switch ( o->method ) {
  case ORC_ECC_FORWARD_ADDITIVE: return align_fa(c, state, o, iters, eps);
  case ORC_ECC_INVERSE_COMPOSITIONAL: return align_ic(c, state, o, iters, eps);
  case ORC_ECC_INVERSE_COMPOSITIONAL_LM: return align_iclm(c, state, o, iters, eps);
  default: return align_lm(c, state, o, iters, eps);
  }
}

/* ------------------------------------------------------------------------ */
/* c_ecch (ecc2.cc:984-1176) */

static inline void next_size(int w, int h, int * nw, int * nh)
{
  *nw = ((w + 1) >> 1) & ~1;
  *nh = ((h + 1) >> 1) & ~1;
}

extern "C" int orc_ecch_num_levels(int w, int h, const orc_ecch_opts * o)
{
  const int min_size = std::max(4, o->minimum_image_size);
  int tw = w, th = h, lv = 1;
  while ( true ) {
    if( o->maxlevel >= 0 && lv >= std::max(0, o->maxlevel) ) break;
    int nw, nh;
    next_size(tw, th, &nw, &nh);
    if( nw < min_size || nh < min_size ) break;
    tw = nw, th = nh, ++lv;
  }
  return lv;
}

namespace {
struct pyr_level {
  int w = 0, h = 0;
  std::vector<double> img;
  std::vector<uint8_t> mask;
};
}

static void build_pyramid(const double * src, const uint8_t * mask, int w, int h, double sigma, int levels,
    bool stop_below_4, std::vector<pyr_level> & pyr)
{
  pyr.clear();
  pyr.resize(levels);
  pyr_level & l0 = pyr[0];
  l0.w = w, l0.h = h;
  l0.img.resize((size_t) w * h);
  if( sigma > 0 ) orc_smooth(src, w, h, sigma, l0.img.data());
  else memcpy(l0.img.data(), src, (size_t) w * h * sizeof(double));
  if( mask ) l0.mask.assign(mask, mask + (size_t) w * h);
  for( int l = 1; l < levels; ++l ) {
    int nw, nh;
    next_size(pyr[l - 1].w, pyr[l - 1].h, &nw, &nh);
    if( stop_below_4 && (nw < 4 || nh < 4) ) {
      pyr.resize(l);
      break;
    }
    pyr_level & d = pyr[l];
    d.w = nw, d.h = nh;
    d.img.resize((size_t) nw * nh);
    orc_pyrdown(pyr[l - 1].img.data(), pyr[l - 1].w, pyr[l - 1].h, d.img.data(), nw, nh);
    if( mask ) {
      d.mask.resize((size_t) nw * nh);
      orc_resize_nearest_u8(pyr[l - 1].mask.data(), pyr[l - 1].w, pyr[l - 1].h, d.mask.data(), nw, nh);
    }
  }
}

static int ecch_align_pyr(const orc_model * m, double * state, const orc_ecch_opts * o,
    const std::vector<pyr_level> & R, const std::vector<pyr_level> & C, int * iters, double * eps)
{
  const int lvls = (int) R.size();
  int lvl = std::min(lvls, (int) C.size()) - 1;
  if( lvl > 0 ) orc_model_scale(m, state, (double) R[lvl].w / (double) R[0].w);
  int total = 0;
  double e0 = FLT_MAX;
  for( ; lvl >= 0; --lvl ) {
    orc_align_opts ao;
    ao.method = o->method;
    ao.max_iterations = o->max_iterations;
    ao.max_eps = o->epsx * std::pow(2.0, lvl);
    ao.update_step_scale = o->update_step_scale;
    ao.ic_jacobian_at_identity = o->ic_jacobian_at_identity;
    orc_level L;
    L.w = R[lvl].w, L.h = R[lvl].h;
    L.ref = R[lvl].img.data(), L.ref_mask = R[lvl].mask.empty() ? nullptr : R[lvl].mask.data();
    L.cw = C[lvl].w, L.ch = C[lvl].h;
    L.cur = C[lvl].img.data(), L.cur_mask = C[lvl].mask.empty() ? nullptr : C[lvl].mask.data();
    int it = 0;
    double e = 0;
    const int ok = orc_ecc_align(m, state, &L, &ao, &it, &e);
    if( ok && lvl > 0 ) orc_model_scale(m, state, (double) R[lvl - 1].w / (double) R[lvl].w);
    total += it;
    if( lvl == 0 ) e0 = e;
  }
  *iters = total;
  *eps = e0;
  return 1;
}

extern "C" int orc_ecch_align(const orc_model * m, double * state, const orc_ecch_opts * o,
    const double * ref, const uint8_t * ref_mask, int w, int h,
    const double * cur, const uint8_t * cur_mask, int cw, int ch, int * iters, double * eps)
{
  const int lv = orc_ecch_num_levels(w, h, o);
  std::vector<pyr_level> R, C;
  build_pyramid(ref, ref_mask, w, h, o->reference_smooth_sigma, lv, false, R);
  build_pyramid(cur, cur_mask, cw, ch, o->input_smooth_sigma, lv, true, C);
  return ecch_align_pyr(m, state, o, R, C, iters, eps);
}

/* c_ecch::align(current) after set_reference_image(reference, reference_mask)
 * (ecc2.cc:984-1176) on w x h images, then compute_correlation of the
 * result against the level-0 reference and its mask
 * (c_frame_registration.cc:837-839); rho may be NULL */
extern "C" int orc_ecch_align_pyramids(const orc_model * m, double * state, const orc_ecch_opts * o,
    const double * ref, const uint8_t * ref_mask, const double * cur, int w, int h, int * iters, double * eps,
    double * rho)
{
  const int lv = orc_ecch_num_levels(w, h, o);
  std::vector<pyr_level> R, C;
  build_pyramid(ref, ref_mask, w, h, o->reference_smooth_sigma, lv, false, R);
  build_pyramid(cur, nullptr, w, h, o->input_smooth_sigma, lv, true, C);
  int it = 0;
  double e = 0;
  ecch_align_pyr(m, state, o, R, C, &it, &e);
  if( iters ) *iters = it;
  if( eps ) *eps = e;
  if( rho ) {
    *rho = orc_correlation(C[0].img.data(), nullptr, w, h, R[0].img.data(), R[0].mask.empty() ? nullptr : R[0].mask.data(),
        w, h, m, state);
  }
  return 1;
}

/* compute_correlation(current, current_mask, reference, reference_mask, rmap)
 * (ecc2.cc:65-137): remap LINEAR / BORDER_CONSTANT, mask >= 254 */
extern "C" double orc_correlation(const double * cur, const uint8_t * cur_mask, int cw, int ch,
    const double * ref, const uint8_t * ref_mask, int w, int h, const orc_model * m, const double * state)
{
  double n = 0, s1 = 0, s2 = 0;
  std::vector<double> b((size_t) w * h);
  std::vector<uint8_t> ok((size_t) w * h);
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      const size_t i = (size_t) y * w + x;
      double X, Y;
      orc_model_warp(m, state, x, y, &X, &Y);
      b[i] = orc_sample_bilinear(cur, cw, ch, X, Y, ORC_BORDER_CONSTANT, 0);
      bool k = mask_ok(orc_mask_coverage(cur_mask, cw, ch, X, Y), 254);
      if( ref_mask && !ref_mask[i] ) k = false;
      ok[i] = k;
      if( k ) n += 1, s1 += ref[i], s2 += b[i];
    }
  }
  if( n <= 0 ) return 0;
  const double m1 = s1 / n, m2 = s2 / n;
  double v1 = 0, v2 = 0, cv = 0;
  for( size_t i = 0; i < (size_t) w * h; ++i ) {
    if( ok[i] ) {
      const double a = ref[i] - m1, c = b[i] - m2;
      v1 += a * a, v2 += c * c, cv += a * c;
    }
  }
  return (cv / n) / (std::sqrt(v1 / n) * std::sqrt(v2 / n));
}

/* c_frame_registration::base_remap (c_frame_registration.cc:1265-1340) */
extern "C" void orc_stack_remap(const orc_model * m, const double * state, const double * src, int sw, int sh,
    int dw, int dh, int border, double * dst, uint8_t * dst_mask)
{
  std::vector<uint8_t> raw((size_t) dw * dh);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < dh; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      double X, Y;
      orc_model_warp(m, state, x, y, &X, &Y);
      const size_t i = (size_t) y * dw + x;
      dst[i] = orc_sample_bilinear(src, sw, sh, X, Y, border, 0);
      raw[i] = mask_ok(orc_mask_coverage(nullptr, sw, sh, X, Y), 255) ? 255 : 0;
    }
  }
  orc_erode5(raw.data(), dw, dh, 1, dst_mask);
}

/* exact weighted sums: acc += w * I, accw += w (the reference's running mean
 * A += (I - A) w / W equals acc / accw in exact arithmetic) */
extern "C" void orc_weighted_average_add(double * acc, double * accw, int w, int h, const double * src, const double * weights)
{
  const size_t N = (size_t) w * h;
  for( size_t i = 0; i < N; ++i ) {
    const double wt = weights ? weights[i] : 1.0;
    if( wt > 0 ) {
      acc[i] += wt * src[i];
      accw[i] += wt;
    }
  }
}

/* _weighted_average_update with CV_32FC1 weights, in the reference's own float
 * running-mean form (c_frame_accumulation.cc:104-122) */
extern "C" void orc_running_mean_add_f32(float * acc, float * accw, int w, int h, const float * src, const float * weights)
{
  const size_t N = (size_t) w * h;
  for( size_t i = 0; i < N; ++i ) {
    const float wn = weights ? weights[i] : 1.0f;
    if( wn > 0 ) {
      const float Wn = accw[i] + wn;
      const float f = wn / Wn;
      accw[i] = Wn;
      acc[i] = acc[i] + (src[i] - acc[i]) * f;
    }
  }
}

extern "C" void orc_extract_bayer_planes_u16(const uint16_t * src, int w, int h, uint16_t * dst)
{
  const int r4 = h / 2, c4 = w / 2;
  for( int y = 0; y < r4; ++y ) {
    const uint16_t * s0 = src + (size_t) (2 * y) * w;
    const uint16_t * s1 = src + (size_t) (2 * y + 1) * w;
    uint16_t * d = dst + (size_t) y * c4 * 4;
    for( int x = 0; x < c4; ++x ) {
      d[4 * x + 0] = s0[2 * x], d[4 * x + 1] = s0[2 * x + 1];
      d[4 * x + 2] = s1[2 * x], d[4 * x + 3] = s1[2 * x + 1];
    }
  }
}

extern "C" void orc_average_bayer_planes_u16(const uint16_t * src, int w, int h, uint16_t * dst)
{
  const int r4 = h / 2, c4 = w / 2;
  for( int y = 0; y < r4; ++y ) {
    const uint16_t * s0 = src + (size_t) (2 * y) * w;
    const uint16_t * s1 = src + (size_t) (2 * y + 1) * w;
    for( int x = 0; x < c4; ++x ) {
      const int sum = (2 + s0[2 * x] + s0[2 * x + 1] + s1[2 * x] + s1[2 * x + 1]) / 4;
      dst[(size_t) y * c4 + x] = (uint16_t) std::min(65535, sum);
    }
  }
}

/* generate_bayer_pattern_mask: BAYER_B = 0, BAYER_G = 1, BAYER_R = 2 */
extern "C" void orc_bayer_pattern_mask(int colorid, int w, int h, uint8_t * dst)
{
  uint8_t q[4];
  switch ( colorid ) {
  case 8:  q[0] = 2, q[1] = 1, q[2] = 1, q[3] = 0; break;  // RGGB
  case 9:  q[0] = 1, q[1] = 2, q[2] = 0, q[3] = 1; break;  // GRBG
  case 10: q[0] = 1, q[1] = 0, q[2] = 2, q[3] = 1; break;  // GBRG
  case 11: q[0] = 0, q[1] = 1, q[2] = 1, q[3] = 2; break;  // BGGR
  default: memset(dst, 0, (size_t) w * h); return;
  }
  // whole 2x2 cells as generate_bayer_pattern_mask; the reference leaves the
  // last row / column of an odd-sized frame uninitialised, here the pattern
  // continues by parity there
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      dst[(size_t) y * w + x] = q[((y & 1) << 1) | (x & 1)];
    }
  }
}

/* _bayer_accumulate with an rmap and float weights (c_frame_accumulation.cc:1043-1122) */
extern "C" void orc_bayer_accumulate(const double * src, int w, int h, const double * mapx, const double * mapy,
    const uint8_t * pat, const double * weights, double * acc, double * cntr)
{
  if( !mapx || !mapy ) {
    // empty rmap: each raw sample to its own channel (c_frame_accumulation.cc:996-1041)
    for( size_t i = 0; i < (size_t) w * h; ++i ) {
      const double wt = weights ? weights[i] : 1.0;
      acc[i * 3 + pat[i]] += src[i] * wt;
      cntr[i * 3 + pat[i]] += wt;
    }
    return;
  }
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      const size_t i = (size_t) y * w + x;
      const double px = mapx[i], py = mapy[i];
      const double wt = weights ? weights[i] : 1.0;
      const int sx = (int) px, sy = (int) py;   // truncation toward zero
      if( sx >= 0 && sx < w - 1 && sy >= 0 && sy < h - 1 ) {
        const double ax = sx + 1 - px, ay = sy + 1 - py, bx = px - sx, by = py - sy;
        const double s[4] = { ax * ay * wt, bx * ay * wt, ax * by * wt, bx * by * wt };
        const int xs[4] = { sx, sx + 1, sx, sx + 1 }, ys[4] = { sy, sy, sy + 1, sy + 1 };
        for( int k = 0; k < 4; ++k ) {
          const size_t j = (size_t) ys[k] * w + xs[k];
          const int cc = pat[j];
          acc[i * 3 + cc] += src[j] * s[k];
          cntr[i * 3 + cc] += s[k];
        }
      }
    }
  }
}

extern "C" double orc_laplacian_energy(const double * img, int w, int h)
{
  double s = 0;
  long n = 0;
  for( int y = 1; y < h - 1; ++y ) {
    for( int x = 1; x < w - 1; ++x ) {
      const size_t i = (size_t) y * w + x;
      const double l = img[i - 1] + img[i + 1] + img[i - w] + img[i + w] - 4 * img[i];
      s += l * l;
      ++n;
    }
  }
  return n > 0 ? s / n : 0;
}

/* ------------------------------------------------------------------------ */
/* register_frame (c_frame_registration.cc:721-964) with ecc.scale = 1,
 * no feature registration, followed by the stacking pipeline's per-frame body
 * (c_image_stacking_pipeline.cc:1539-1790): remap frame + mask, weights, add. */

static void convert_state(const orc_model * from, const double * s, const orc_model * to, double * out)
{
  orc_model_identity(to, out);
  // affine-like 2x3 view of the source state
  double a[6] = { 1, 0, 0, 0, 1, 0 };
  switch ( from->type ) {
  case ORC_MOTION_TRANSLATION: a[2] = s[0], a[5] = s[1]; break;
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN: {
    const double sa = std::sin(s[2]), ca = std::cos(s[2]), sc = s[3];
    a[0] = sc * ca, a[1] = -sc * sa, a[2] = s[0] - sc * ca * s[4] + sc * sa * s[5];
    a[3] = sc * sa, a[4] = sc * ca, a[5] = s[1] - sc * sa * s[4] - sc * ca * s[5];
    break;
  }
  case ORC_MOTION_SEMI_QUADRATIC:
    a[0] = s[0], a[1] = s[1], a[2] = s[2], a[3] = s[4], a[4] = s[5], a[5] = s[6];
    break;
  case ORC_MOTION_QUADRATIC:
    a[0] = s[0], a[1] = s[1], a[2] = s[2], a[3] = s[6], a[4] = s[7], a[5] = s[8];
    break;
  default: memcpy(a, s, sizeof(a));
  }
  switch ( to->type ) {
  case ORC_MOTION_TRANSLATION: out[0] = a[2], out[1] = a[5]; break;
  case ORC_MOTION_AFFINE: memcpy(out, a, sizeof(a)); break;
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION:
    if( from->type == ORC_MOTION_HOMOGRAPHY || from->type == ORC_MOTION_EPIPOLAR_DEROTATION ) memcpy(out, s, 8 * sizeof(double));
    else memcpy(out, a, sizeof(a));
    break;
  case ORC_MOTION_SEMI_QUADRATIC:
    out[0] = a[0], out[1] = a[1], out[2] = a[2], out[4] = a[3], out[5] = a[4], out[6] = a[5];
    if( from->type == ORC_MOTION_SEMI_QUADRATIC ) memcpy(out, s, 8 * sizeof(double));
    break;
  case ORC_MOTION_QUADRATIC:
    out[0] = a[0], out[1] = a[1], out[2] = a[2], out[6] = a[3], out[7] = a[4], out[8] = a[5];
    if( from->type == ORC_MOTION_SEMI_QUADRATIC ) out[3] = s[3], out[9] = s[7];
    if( from->type == ORC_MOTION_QUADRATIC ) memcpy(out, s, 12 * sizeof(double));
    break;
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN:
    out[0] = a[2], out[1] = a[5];
    out[2] = std::atan2(a[3], a[0]);
    if( to->type == ORC_MOTION_SCALED_EUCLIDEAN ) out[3] = std::sqrt(a[0] * a[0] + a[3] * a[3]);
    break;
  default: break;
  }
}

extern "C" int orc_register_and_stack(const orc_pipeline_opts * o,
    const double * ref, int w, int h,
    const uint16_t * frames, int n, double frame_scale,
    double * out_states, int * out_status, double * out_rho,
    double * acc, double * accw)
{
  const int lv = orc_ecch_num_levels(w, h, &o->ecch);
  std::vector<pyr_level> R;
  build_pyramid(ref, nullptr, w, h, o->ecch.reference_smooth_sigma, lv, false, R);
  const size_t N = (size_t) w * h;
  std::vector<double> img(N), warped(N), wts(N);
  std::vector<uint8_t> msk(N);
  for( int f = 0; f < n; ++f ) {
    const uint16_t * fr = frames + (size_t) f * N;
    for( size_t i = 0; i < N; ++i ) img[i] = fr[i] * frame_scale;
    std::vector<pyr_level> C;
    build_pyramid(img.data(), nullptr, w, h, o->ecch.input_smooth_sigma, lv, true, C);
    double state[16], prev[16];
    orc_model pm = { 0, 0, 0, 0 };
    for( int k = 0; k < o->num_passes; ++k ) {
      orc_model m = { o->pass_motion[k], 0, 0, o->pass_motion[k] == ORC_MOTION_EUCLIDEAN ? 1 : 0 };
      if( k == 0 ) orc_model_identity(&m, state);
      else convert_state(&pm, prev, &m, state);
      int it;
      double e;
      ecch_align_pyr(&m, state, &o->ecch, R, C, &it, &e);
      memcpy(prev, state, sizeof(state));
      pm = m;
    }
    const double rho = orc_correlation(C[0].img.data(), nullptr, w, h, R[0].img.data(), nullptr, w, h, &pm, state);
    memcpy(out_states + (size_t) f * 16, state, sizeof(state));
    out_rho[f] = rho;
    if( !(rho >= o->min_rho) ) {
      out_status[f] = 3;  // low correlation: frame skipped
      continue;
    }
    out_status[f] = 0;
    orc_stack_remap(&pm, state, img.data(), w, h, w, h, o->border_mode, warped.data(), msk.data());
    const double fw = o->use_laplacian_weights && C.size() > 1 ? orc_laplacian_energy(C[1].img.data(), C[1].w, C[1].h) : 1.0;
    for( size_t i = 0; i < N; ++i ) wts[i] = msk[i] ? fw : 0.0;
    orc_weighted_average_add(acc, accw, w, h, warped.data(), wts.data());
  }
  return 0;
}
