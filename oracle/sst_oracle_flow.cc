/*
 * sst_oracle_flow.cc -- FP64 restatement of c_eccflow and of the warp
 * residual objective used by the adjoint.
 *
 * TEST INFRASTRUCTURE ONLY (see sst_oracle.h).
 *
 *   c_eccflow::set_reference_image   ecc2.cc:2489-2672
 *   c_eccflow::setup_input_image     ecc2.cc:2674-2768
 *   c_eccflow::compute_uv            ecc2.cc:2770-2835 (level loop), 2237-2398 (one update)
 *   c_eccflow::avgdown / downscale   ecc2.cc:2400-2450
 *   ecc_flow_to_remap / ecc_remap_to_optflow  ecc2.cc:400-500
 *
 * OpenCV primitives restated from their documented semantics:
 *   cv::resize INTER_AREA  : each destination pixel averages the source area
 *                            it covers (pixel-area relation; partial cells
 *                            below 1e-3 of a pixel are dropped)
 *   cv::resize INTER_CUBIC : Keys cubic convolution, a = -0.75, pixel centres
 *                            at (x + 0.5) * scale - 0.5, taps clamped to the image
 *   getGaussianKernel(3, 0): [1/4, 1/2, 1/4]
 */
#include "sst_oracle.h"

#include <math.h>
#include <string.h>
#include <algorithm>
#include <vector>

namespace {

struct tap {
  int i;
  double w;
};

/* INTER_AREA weights of one axis: destination d covers source [d s, (d + 1) s) */
std::vector<std::vector<tap>> area_taps(int ssize, int dsize)
{
  std::vector<std::vector<tap>> t(dsize);
  const double scale = (double) ssize / dsize;
  for( int d = 0; d < dsize; ++d ) {
    const double f1 = d * scale, f2 = f1 + scale;
    const double cell = std::min(scale, ssize - f1);
    const int s1 = (int) ceil(f1), s2 = std::min((int) floor(f2), ssize);
    if( s1 - f1 > 1e-3 && s1 - 1 >= 0 ) t[d].push_back({ s1 - 1, (s1 - f1) / cell });
    for( int s = s1; s < s2; ++s ) t[d].push_back({ s, 1.0 / cell });
    if( s2 < ssize && f2 - s2 > 1e-3 ) t[d].push_back({ s2, std::min(std::min(f2 - s2, 1.0), cell) / cell });
  }
  return t;
}

/* Keys cubic weights (a = -0.75) of one axis with clamped taps */
std::vector<std::vector<tap>> cubic_taps(int ssize, int dsize)
{
  std::vector<std::vector<tap>> t(dsize);
  const double scale = (double) ssize / dsize, A = -0.75;
  for( int d = 0; d < dsize; ++d ) {
    const double fx = (d + 0.5) * scale - 0.5;
    const int sx = (int) floor(fx);
    const double u = fx - sx;
    double w[4];
    w[0] = ((A * (u + 1) - 5 * A) * (u + 1) + 8 * A) * (u + 1) - 4 * A;
    w[1] = ((A + 2) * u - (A + 3)) * u * u + 1;
    w[2] = ((A + 2) * (1 - u) - (A + 3)) * (1 - u) * (1 - u) + 1;
    w[3] = 1 - w[0] - w[1] - w[2];
    for( int k = 0; k < 4; ++k ) t[d].push_back({ std::min(std::max(sx - 1 + k, 0), ssize - 1), w[k] });
  }
  return t;
}

void separable(const double * src, int sw, int sh, double * dst, int dw, int dh,
    const std::vector<std::vector<tap>> & tx, const std::vector<std::vector<tap>> & ty)
{
  std::vector<double> tmp((size_t) dw * sh);
#pragma omp parallel for schedule(static)
  for( int y = 0; y < sh; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( const tap & k : tx[x] ) a += k.w * src[(size_t) y * sw + k.i];
      tmp[(size_t) y * dw + x] = a;
    }
  }
#pragma omp parallel for schedule(static)
  for( int y = 0; y < dh; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( const tap & k : ty[y] ) a += k.w * tmp[(size_t) k.i * dw + x];
      dst[(size_t) y * dw + x] = a;
    }
  }
}

/* 3x3 Gaussian [1/4 1/2 1/4] separable, BORDER_REPLICATE, in place */
void gauss3(double * img, int w, int h)
{
  std::vector<double> tmp((size_t) w * h);
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      const double * r = img + (size_t) y * w;
      tmp[(size_t) y * w + x] = 0.25 * r[std::max(x - 1, 0)] + 0.5 * r[x] + 0.25 * r[std::min(x + 1, w - 1)];
    }
  }
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      img[(size_t) y * w + x] = 0.25 * tmp[(size_t) std::max(y - 1, 0) * w + x] + 0.5 * tmp[(size_t) y * w + x] +
          0.25 * tmp[(size_t) std::min(y + 1, h - 1) * w + x];
    }
  }
}

/* avgdown (ecc2.cc:2400-2418): INTER_AREA to the size halved support_scale
 * times, then the 3x3 Gaussian */
void avgdown(const double * src, int w, int h, int support_scale, std::vector<double> & dst, int * dw, int * dh)
{
  int sw = w, sh = h;
  for( int i = 0; i < support_scale; ++i ) sw = (sw + 1) / 2, sh = (sh + 1) / 2;
  dst.assign((size_t) sw * sh, 0.0);
  orc_resize_area(src, w, h, dst.data(), sw, sh);
  gauss3(dst.data(), sw, sh);
  *dw = sw, *dh = sh;
}

struct level {
  int w, h;
  std::vector<double> ref, cur, Ix, Iy;
  std::vector<uint8_t> rmask, cmask;
  int dw, dh;
  std::vector<double> D;   // dw x dh x 4: a00, a01, a11, mult / (|det| + reg)
};

void downscale(const orc_flow_opts * o, const double * src, int sw, int sh, double * dst, int dw, int dh)
{
  if( o->downscale == 2 ) orc_pyrdown(src, sw, sh, dst, dw, dh);
  else orc_resize_area(src, sw, sh, dst, dw, dh);
}

}  // namespace

extern "C" void orc_resize_area(const double * src, int sw, int sh, double * dst, int dw, int dh)
{
  separable(src, sw, sh, dst, dw, dh, area_taps(sw, dw), area_taps(sh, dh));
}

extern "C" void orc_resize_cubic(const double * src, int sw, int sh, double * dst, int dw, int dh)
{
  if( sw == dw && sh == dh ) {
    memcpy(dst, src, sizeof(double) * (size_t) sw * sh);
    return;
  }
  separable(src, sw, sh, dst, dw, dh, cubic_taps(sw, dw), cubic_taps(sh, dh));
}

/* level sizes of set_reference_image (ecc2.cc:2525-2600) */
extern "C" int orc_eccflow_levels(int w, int h, const orc_flow_opts * o, int * ws, int * hs, int max_levels)
{
  const int min_size = std::max(4, o->min_image_size);
  int n = 0;
  ws[n] = w, hs[n] = h, ++n;
  if( o->max_pyramid_level >= 0 && 0 >= o->max_pyramid_level ) return n;
  while ( n < max_levels ) {
    const int pw = ws[n - 1], ph = hs[n - 1];
    int nw, nh;
    if( o->downscale == 2 ) {
      nw = std::max(o->min_image_size, (pw + 1) / 2), nh = std::max(o->min_image_size, (ph + 1) / 2);
      if( (nw == pw && nh == ph) || std::min(nw, nh) <= min_size ) break;
    }
    else {
      nw = std::max(o->min_image_size, (int) ((pw + 1) * o->scale_factor));
      nh = std::max(o->min_image_size, (int) ((ph + 1) * o->scale_factor));
      if( (nw == pw && nh == ph) || std::max(nw, nh) <= min_size ) break;
    }
    ws[n] = nw, hs[n] = nh, ++n;
    if( o->max_pyramid_level >= 0 && n - 1 >= o->max_pyramid_level ) break;
  }
  return n;
}

extern "C" int orc_eccflow(const orc_flow_opts * o, const double * ref, const double * cur, int w, int h,
    const double * init_flow, double * flow)
{
  return orc_eccflow_masked(o, ref, nullptr, cur, nullptr, w, h, init_flow, flow);
}

/* c_eccflow with masks: each level's reference and current masks are the
 * INTER_NEAREST resizes of the masks of the level the image comes from
 * (downscale, ecc2.cc:2431-2456); in an update, the current mask is
 * remapped INTER_NEAREST (cvRound, BORDER_CONSTANT 0) by the flow and ANDed
 * with the reference mask, and It gx, It gy are zero where that fails
 * (compute_uv, ecc2.cc:2253-2335). The reference gradients and D ignore the
 * masks, as in the reference (ecc2.cc:2604-2605). */
extern "C" int orc_eccflow_masked(const orc_flow_opts * o, const double * ref, const uint8_t * ref_mask,
    const double * cur, const uint8_t * cur_mask, int w, int h, const double * init_flow, double * flow)
{
  int ws[64], hs[64];
  const int L = orc_eccflow_levels(w, h, o, ws, hs, 64);
  const int min_size = std::max(4, o->min_image_size);
  const bool big_aspect = std::max(w, h) / std::min(w, h) >= 2;
  const double noise = o->noise_level >= 0 ? o->noise_level : 1e-3;
  std::vector<level> P(L);
  // reference pyramid and per-level D (set_reference_image)
  for( int l = 0; l < L; ++l ) {
    level & e = P[l];
    e.w = ws[l], e.h = hs[l];
    e.ref.resize((size_t) e.w * e.h);
    e.cur.resize((size_t) e.w * e.h);
    if( ref_mask ) e.rmask.resize(e.ref.size());
    if( cur_mask ) e.cmask.resize(e.ref.size());
    if( l == 0 ) {
      memcpy(e.ref.data(), ref, sizeof(double) * e.ref.size());
      memcpy(e.cur.data(), cur, sizeof(double) * e.cur.size());
      if( ref_mask ) memcpy(e.rmask.data(), ref_mask, e.rmask.size());
      if( cur_mask ) memcpy(e.cmask.data(), cur_mask, e.cmask.size());
    }
    else {
      const bool from0 = o->downscale == 1 ||
          (o->downscale == 0 && big_aspect && std::min(e.w, e.h) <= min_size + 1);
      const level & s = from0 ? P[0] : P[l - 1];
      downscale(o, s.ref.data(), s.w, s.h, e.ref.data(), e.w, e.h);
      downscale(o, s.cur.data(), s.w, s.h, e.cur.data(), e.w, e.h);
      if( ref_mask ) orc_resize_nearest_u8(s.rmask.data(), s.w, s.h, e.rmask.data(), e.w, e.h);
      if( cur_mask ) orc_resize_nearest_u8(s.cmask.data(), s.w, s.h, e.cmask.data(), e.w, e.h);
    }
    e.Ix.resize(e.ref.size());
    e.Iy.resize(e.ref.size());
    orc_differentiate(e.ref.data(), e.w, e.h, nullptr, e.Ix.data(), e.Iy.data());
    std::vector<double> pxx(e.ref.size()), pxy(e.ref.size()), pyy(e.ref.size());
    for( size_t i = 0; i < e.ref.size(); ++i ) {
      pxx[i] = e.Ix[i] * e.Ix[i], pxy[i] = e.Ix[i] * e.Iy[i], pyy[i] = e.Iy[i] * e.Iy[i];
    }
    std::vector<double> axx, axy, ayy;
    avgdown(pxx.data(), e.w, e.h, o->support_scale, axx, &e.dw, &e.dh);
    avgdown(pxy.data(), e.w, e.h, o->support_scale, axy, &e.dw, &e.dh);
    avgdown(pyy.data(), e.w, e.h, o->support_scale, ayy, &e.dw, &e.dh);
    const double reg = noise > 0 ? pow(1e-5 * noise / (1 << l), 4) : 0;
    e.D.resize((size_t) e.dw * e.dh * 4);
    for( size_t i = 0; i < axx.size(); ++i ) {
      const double det = fabs(axx[i] * ayy[i] - axy[i] * axy[i]);
      e.D[4 * i] = axx[i], e.D[4 * i + 1] = axy[i], e.D[4 * i + 2] = ayy[i];
      e.D[4 * i + 3] = o->update_multiplier / (det + reg);
    }
  }
  // initial flow at the coarsest level (compute_uv, ecc2.cc:2780-2805)
  std::vector<double> u, v;
  {
    const level & c = P[L - 1];
    u.assign((size_t) c.w * c.h, 0.0), v.assign(u.size(), 0.0);
    if( init_flow ) {
      std::vector<double> u0((size_t) w * h), v0((size_t) w * h);
      for( size_t i = 0; i < u0.size(); ++i ) u0[i] = init_flow[2 * i], v0[i] = init_flow[2 * i + 1];
      orc_resize_cubic(u0.data(), w, h, u.data(), c.w, c.h);
      orc_resize_cubic(v0.data(), w, h, v.data(), c.w, c.h);
      const double rx = (double) c.w / w, ry = (double) c.h / h;
      for( size_t i = 0; i < u.size(); ++i ) u[i] *= rx, v[i] *= ry;
    }
  }
  for( int l = L - 1; l >= 0; --l ) {
    level & e = P[l];
    if( l < L - 1 ) {
      const level & p = P[l + 1];
      const double rx = (double) e.w / p.w, ry = (double) e.h / p.h;
      for( size_t i = 0; i < u.size(); ++i ) u[i] *= rx, v[i] *= ry;
      std::vector<double> nu((size_t) e.w * e.h), nv((size_t) e.w * e.h);
      orc_resize_cubic(u.data(), p.w, p.h, nu.data(), e.w, e.h);
      orc_resize_cubic(v.data(), p.w, p.h, nv.data(), e.w, e.h);
      u.swap(nu), v.swap(nv);
    }
    for( int it = 0; it < o->max_iterations; ++it ) {
      // one update (ecc2.cc:2237-2398): remap current by uv, It (Ix, Iy), avgdown, 2x2 solve, cubic up
      std::vector<double> bx((size_t) e.w * e.h), by((size_t) e.w * e.h);
#pragma omp parallel for schedule(static)
      for( int y = 0; y < e.h; ++y ) {
        for( int x = 0; x < e.w; ++x ) {
          const size_t i = (size_t) y * e.w + x;
          bool ok = e.rmask.empty() || e.rmask[i] != 0;
          if( ok && !e.cmask.empty() ) {
            const double X = nearbyint(x + u[i]), Y = nearbyint(y + v[i]);
            ok = X >= 0 && X < e.w && Y >= 0 && Y < e.h && e.cmask[(size_t) Y * e.w + (size_t) X] != 0;
          }
          if( !ok ) {
            bx[i] = by[i] = 0;
            continue;
          }
          const double W = orc_sample_bilinear(e.cur.data(), e.w, e.h, x + u[i], y + v[i], ORC_BORDER_REPLICATE, 0);
          const double It = e.ref[i] - W;
          bx[i] = It * e.Ix[i], by[i] = It * e.Iy[i];
        }
      }
      std::vector<double> ax, ay;
      int dw, dh;
      avgdown(bx.data(), e.w, e.h, o->support_scale, ax, &dw, &dh);
      avgdown(by.data(), e.w, e.h, o->support_scale, ay, &dw, &dh);
      std::vector<double> du((size_t) dw * dh), dv((size_t) dw * dh);
      for( size_t i = 0; i < du.size(); ++i ) {
        const double * D = e.D.data() + 4 * i;
        du[i] = D[3] * (D[2] * ax[i] - D[1] * ay[i]);
        dv[i] = D[3] * (D[0] * ay[i] - D[1] * ax[i]);
      }
      std::vector<double> uu((size_t) e.w * e.h), vv((size_t) e.w * e.h);
      orc_resize_cubic(du.data(), dw, dh, uu.data(), e.w, e.h);
      orc_resize_cubic(dv.data(), dw, dh, vv.data(), e.w, e.h);
      for( size_t i = 0; i < u.size(); ++i ) u[i] += uu[i], v[i] += vv[i];
    }
  }
  for( size_t i = 0; i < u.size(); ++i ) flow[2 * i] = u[i], flow[2 * i + 1] = v[i];
  return L;
}

/* ------------------------------------------------------- adjoint objective */

extern "C" double orc_warp_residual(const orc_model * m, const double * state, const double * img, const double * tmpl,
    const double * flow, int w, int h, double * grad_p, double * grad_t, double * grad_u)
{
  const int M = orc_model_nparams(m);
  double L = 0, gp[16] = { 0 };
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      const size_t i = (size_t) y * w + x;
      double X, Y;
      orc_model_warp(m, state, x, y, &X, &Y);
      if( flow ) X += flow[2 * i], Y += flow[2 * i + 1];
      const double fx0 = floor(X), fy0 = floor(Y);
      const int x0 = (int) fx0, y0 = (int) fy0;
      const double ax = X - fx0, ay = Y - fy0;
      auto at = [&](int xx, int yy) {
        return img[(size_t) std::min(std::max(yy, 0), h - 1) * w + std::min(std::max(xx, 0), w - 1)];
      };
      const double v00 = at(x0, y0), v01 = at(x0 + 1, y0), v10 = at(x0, y0 + 1), v11 = at(x0 + 1, y0 + 1);
      const double I = (1 - ay) * ((1 - ax) * v00 + ax * v01) + ay * ((1 - ax) * v10 + ax * v11);
      const double gX = (1 - ay) * (v01 - v00) + ay * (v11 - v10);
      const double gY = (1 - ax) * (v10 - v00) + ax * (v11 - v01);
      const double r = I - tmpl[i];
      L += 0.5 * r * r;
      if( grad_t ) grad_t[i] = -r;
      if( grad_u ) grad_u[2 * i] = r * gX, grad_u[2 * i + 1] = r * gY;
      if( grad_p ) {
        double J[16];
        orc_model_sd(m, state, x, y, gX, gY, J);
        for( int k = 0; k < M; ++k ) gp[k] += r * J[k];
      }
    }
  }
  if( grad_p ) for( int k = 0; k < M; ++k ) grad_p[k] = gp[k];
  return L;
}

/* ------------------------------------------------------- focus weights */

/* W = (6 lap^2 + |grad|^2)^2 of the frame warped to the dw x dh grid
 * (bilinear, BORDER_REPLICATE), 5-point Laplacian and central differences
 * with the output grid replicated at its border, then a Gaussian of sigma 3
 * (getGaussianKernel(19, 3), BORDER_REPLICATE) */
extern "C" void orc_focus_weights(const orc_model * m, const double * state, const double * src, int sw, int sh,
    int dw, int dh, double * out)
{
  std::vector<double> wv((size_t) dw * dh), e((size_t) dw * dh);
  orc_remap_model(m, state, src, sw, sh, dw, dh, ORC_BORDER_REPLICATE, 0, wv.data());
  auto at = [&](int x, int y) {
    return wv[(size_t) std::min(std::max(y, 0), dh - 1) * dw + std::min(std::max(x, 0), dw - 1)];
  };
  for( int y = 0; y < dh; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      const double c = at(x, y), l = at(x - 1, y), r = at(x + 1, y), u = at(x, y - 1), d = at(x, y + 1);
      const double lap = l + r + u + d - 4 * c, gx = 0.5 * (r - l), gy = 0.5 * (d - u);
      const double v = 6 * lap * lap + gx * gx + gy * gy;
      e[(size_t) y * dw + x] = v * v;
    }
  }
  orc_smooth(e.data(), dw, dh, 3.0, out);
}
