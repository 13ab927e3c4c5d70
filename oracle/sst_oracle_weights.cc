/*
 * sst_oracle_weights.cc -- FP64 restatement of the local-variance sharpness
 * map used as per-pixel stacking weights. Test infrastructure only: this is
 * the oracle of the CUDA weight maps, never the thing measured or shipped.
 *
 * Follows compute_local_variance_map
 * (core/proc/sharpness_measure/c_local_variance_sharpness_measure.cc:193-249)
 * and its helpers dscaleSize (:15-25), pdownscale (:28-52),
 * _compute_sharpness_map (:131-165) and upscale_local_variance_map
 * (:175-184), with OpenCV's morphological gradient (dilate - erode over a
 * square, BORDER_REPLICATE), INTER_AREA and INTER_LINEAR resize geometry.
 */
#include <math.h>
#include <string.h>
#include <algorithm>
#include <vector>

#include "sst_oracle.h"

namespace {

/* dscaleSize: halve (s + 1) / 2 up to `levels` times, stopping before the
 * smaller side would drop below 4 */
void halved_size(int w, int h, int levels, int * ow, int * oh)
{
  for( int l = 0; l < levels; ++l ) {
    const int nw = (w + 1) / 2, nh = (h + 1) / 2;
    if( std::min(nw, nh) < 4 ) break;
    w = nw, h = nh;
  }
  *ow = w, *oh = h;
}

/* INTER_LINEAR geometry along one axis: destination d samples
 * f = (d + 0.5) * ssize / dsize - 0.5; left of the first source or at / past
 * the last one the tap clamps to the edge with a zero fraction */
void linear_axis(int ssize, int dsize, std::vector<int> & i0, std::vector<double> & fr)
{
  i0.resize(dsize), fr.resize(dsize);
  const double s = (double) ssize / dsize;
  for( int d = 0; d < dsize; ++d ) {
    const double f = (d + 0.5) * s - 0.5;
    int si = (int) floor(f);
    double a = f - si;
    if( si < 0 ) si = 0, a = 0;
    if( si >= ssize - 1 ) si = ssize - 1, a = 0;
    i0[d] = si, fr[d] = a;
  }
}

/* morphological gradient max - min over the (2r+1)^2 square around every
 * pixel, coordinates clamped to the image (BORDER_REPLICATE) */
void morph_gradient(const double * src, int w, int h, int r, double * g)
{
  std::vector<double> hmax((size_t) w * h), hmin((size_t) w * h);
  for( int y = 0; y < h; ++y ) {
    const double * row = src + (size_t) y * w;
    for( int x = 0; x < w; ++x ) {
      double mx = -INFINITY, mn = INFINITY;
      for( int k = -r; k <= r; ++k ) {
        const double v = row[std::min(std::max(x + k, 0), w - 1)];
        mx = std::max(mx, v), mn = std::min(mn, v);
      }
      hmax[(size_t) y * w + x] = mx, hmin[(size_t) y * w + x] = mn;
    }
  }
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      double mx = -INFINITY, mn = INFINITY;
      for( int k = -r; k <= r; ++k ) {
        const size_t i = (size_t) std::min(std::max(y + k, 0), h - 1) * w + x;
        mx = std::max(mx, hmax[i]), mn = std::min(mn, hmin[i]);
      }
      g[(size_t) y * w + x] = mx - mn;
    }
  }
}

}  // namespace

extern "C" void orc_resize_linear(const double * src, int sw, int sh, double * dst, int dw, int dh)
{
  if( sw == dw && sh == dh ) {
    memcpy(dst, src, sizeof(double) * (size_t) sw * sh);
    return;
  }
  std::vector<int> ix, iy;
  std::vector<double> fx, fy;
  linear_axis(sw, dw, ix, fx);
  linear_axis(sh, dh, iy, fy);
  for( int y = 0; y < dh; ++y ) {
    const double * r0 = src + (size_t) iy[y] * sw;
    const double * r1 = src + (size_t) std::min(iy[y] + 1, sh - 1) * sw;
    for( int x = 0; x < dw; ++x ) {
      const int x0 = ix[x], x1 = std::min(x0 + 1, sw - 1);
      const double t0 = r0[x0] * (1 - fx[x]) + r0[x1] * fx[x];
      const double t1 = r1[x0] * (1 - fx[x]) + r1[x1] * fx[x];
      dst[(size_t) y * dw + x] = t0 * (1 - fy[y]) + t1 * fy[y];
    }
  }
}

extern "C" int orc_local_variance_size(int w, int h, int dscale, int uscale, int * mw, int * mh)
{
  // pdownscale: pyrDown while levels remain, stopping after a level whose
  // smaller side is below 4 (an input already below 4 is kept as it is)
  int gw = w, gh = h;
  if( dscale > 0 && std::min(w, h) >= 4 ) {
    for( int l = 0; l < dscale; ++l ) {
      gw = (gw + 1) / 2, gh = (gh + 1) / 2;
      if( std::min(gw, gh) < 4 ) break;
    }
  }
  int ow = gw, oh = gh;
  if( uscale > 0 ) halved_size(gw, gh, uscale, &ow, &oh);
  // the full-resolution upscale runs only when the gradient's size differs
  // from the image's (a reduced map is returned as it is otherwise)
  if( gw != w || gh != h ) ow = w, oh = h;
  *mw = ow, *mh = oh;
  return (gw != w || gh != h) ? 1 : 0;
}

extern "C" int orc_local_variance_map(const double * img, int w, int h, int kradius, int dscale, int uscale,
    double depth_scale, double * map, int * mw, int * mh, double * q)
{
  std::vector<double> M(img, img + (size_t) w * h), T;
  int gw = w, gh = h;
  if( dscale > 0 && std::min(w, h) >= 4 ) {
    for( int l = 0; l < dscale; ++l ) {
      const int nw = (gw + 1) / 2, nh = (gh + 1) / 2;
      T.resize((size_t) nw * nh);
      orc_pyrdown(M.data(), gw, gh, T.data(), nw, nh);
      M.swap(T);
      gw = nw, gh = nh;
      if( std::min(gw, gh) < 4 ) break;
    }
  }
  const int r = std::max(1, kradius);
  std::vector<double> G((size_t) gw * gh);
  morph_gradient(M.data(), gw, gh, r, G.data());
  double W = 0, S4 = 0;
  for( double g : G ) W += fabs(g), S4 += g * g * g * g;
  *q = 0;
  *mw = *mh = 0;
  if( !(W > 0) ) return 0;   // a flat image has no map
  const double ds3 = depth_scale * depth_scale * depth_scale;
  const double Q = ds3 * S4 / W;
  std::vector<double> P((size_t) gw * gh);
  for( size_t i = 0; i < P.size(); ++i ) P[i] = G[i] * G[i] * G[i] * ds3;
  int pw = gw, ph = gh;
  if( uscale > 0 ) {
    int uw, uh;
    halved_size(gw, gh, uscale, &uw, &uh);
    T.resize((size_t) uw * uh);
    orc_resize_area(P.data(), gw, gh, T.data(), uw, uh);
    P.swap(T);
    pw = uw, ph = uh;
  }
  for( double & v : P ) v += 0.05 * Q;
  if( gw != w || gh != h ) {
    orc_resize_linear(P.data(), pw, ph, map, w, h);
    pw = w, ph = h;
  }
  else {
    memcpy(map, P.data(), sizeof(double) * (size_t) pw * ph);
  }
  *mw = pw, *mh = ph;
  *q = Q;
  return 1;
}
