/*
 * sst_oracle_lpg.cc -- FP64 restatement of the LPG sharpness map
 * (lpg(), core/proc/lpg.cc:223-291, with compute_lpg_5x5_parallel :60-131,
 * downscale :134-155 and upscale :157-185; c_lpg_options defaults in
 * core/proc/sharpness_measure/c_lpg_sharpness_measure.h:22-28).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of the GPU LPG maps.
 *
 * cv::pyrDown (BORDER_DEFAULT = REFLECT_101) and cv::pyrUp follow their
 * documented semantics as in sst_oracle_reg.cc (orc_pyrdown_border,
 * orc_pyrup).
 */
#include "sst_oracle.h"
#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

struct Im {
  int w = 0, h = 0;
  std::vector<double> d;
};

/* lpg.cc downscale(): one pyrDown when the source is at least 4 px on its
 * smaller side, then up to level - 1 more while the result stays >= 4 */
void downscale(Im & m, int level)
{
  if( std::min(m.w, m.h) < 4 ) return;
  for( int l = 0; l < level; ++l ) {
    Im d;
    d.w = (m.w + 1) / 2, d.h = (m.h + 1) / 2;
    d.d.resize((size_t) d.w * d.h);
    orc_pyrdown_border(m.d.data(), m.w, m.h, d.d.data(), d.w, d.h, ORC_BORDER_REFLECT101);
    m = std::move(d);
    if( std::min(m.w, m.h) < 4 ) break;
  }
}

}  // namespace

/* lpg(image, mask, map, k, p, dscale, uscale, &metric) of a mono image of
 * `maxval`-scaled values (1 for float input): map (w x h, the image's size)
 * and the sharpness metric mean(map) (masked by the nearest-resized mask
 * when given). Returns 0, or -1 when the reference would read rows it never
 * wrote (a map smaller than 5 x 5 after dscale). */
extern "C" int orc_lpg(const double * img, const uint8_t * mask, int w, int h, double k, double p, int dscale,
    int uscale, double * map, double * metric)
{
  Im s;
  s.w = w, s.h = h;
  s.d.assign(img, img + (size_t) w * h);
  if( dscale > 0 ) {
    downscale(s, dscale);
    for( double & v : s.d ) v *= 1.0 / (1 + dscale);
  }
  if( s.w < 5 || s.h < 5 ) return -1;
  // compute_lpg_5x5_parallel (lpg.cc:60-131)
  const double l_norm = 100.0 / 4.0, g_norm = 100.0 / 36.0;
  const double alpha = k / (k + 1) * l_norm * l_norm, beta = 1.0 / (k + 1) * g_norm * g_norm, eps = 1e-9;
  Im m;
  m.w = s.w, m.h = s.h;
  m.d.resize(s.d.size());
  for( int y = 0; y < s.h; ++y ) {
    const int yc = std::min(std::max(y, 2), s.h - 3);
    const double * r0 = s.d.data() + (size_t) (yc - 2) * s.w;
    const double * r1 = r0 + s.w, * r2 = r1 + s.w, * r3 = r2 + s.w, * r4 = r3 + s.w;
    for( int x = 0; x < s.w; ++x ) {
      const int c = std::min(std::max(x, 2), s.w - 3);
      const double gx = (r0[c + 2] + 2 * r1[c + 2] + 4 * r2[c + 2] + 2 * r3[c + 2] + r4[c + 2]) -
          (r0[c - 2] + 2 * r1[c - 2] + 4 * r2[c - 2] + 2 * r3[c - 2] + r4[c - 2]) +
          2.0 * ((r1[c + 1] + 2 * r2[c + 1] + r3[c + 1]) - (r1[c - 1] + 2 * r2[c - 1] + r3[c - 1]));
      const double gy = (r4[c - 2] + 2 * r4[c - 1] + 4 * r4[c] + 2 * r4[c + 1] + r4[c + 2]) -
          (r0[c - 2] + 2 * r0[c - 1] + 4 * r0[c] + 2 * r0[c + 1] + r0[c + 2]) +
          2.0 * ((r3[c - 1] + 2 * r3[c] + r3[c + 1]) - (r1[c - 1] + 2 * r1[c] + r1[c + 1]));
      const double lv = 16.0 * r2[c] - 2.0 * (r1[c] + r3[c] + r2[c - 1] + r2[c + 1]) -
          (r1[c - 1] + r1[c + 1] + r3[c - 1] + r3[c + 1]) - (r0[c] + r4[c] + r2[c - 2] + r2[c + 2]);
      m.d[(size_t) y * m.w + x] = alpha * lv * lv + beta * (gx * gx + gy * gy) + eps;
    }
  }
  if( uscale > 0 && uscale > dscale ) {
    downscale(m, uscale - dscale);
    for( double & v : m.d ) v *= (uscale - dscale);
  }
  if( p != 0 && p != 1 ) {
    for( double & v : m.d ) v = std::pow(v, p);
  }
  // upscale (lpg.cc:157-185): pyrUp through the sizes halved from the image size
  if( m.w != w || m.h != h ) {
    std::vector<int> ws(1, w), hs(1, h);
    while ( true ) {
      const int nw = (ws.back() + 1) / 2, nh = (hs.back() + 1) / 2;
      if( nw == m.w && nh == m.h ) break;
      if( nw < m.w || nh < m.h ) return -1;
      ws.push_back(nw), hs.push_back(nh);
    }
    for( int i = (int) ws.size() - 1; i >= 0; --i ) {
      Im u;
      u.w = ws[i], u.h = hs[i];
      u.d.resize((size_t) u.w * u.h);
      orc_pyrup(m.d.data(), m.w, m.h, u.d.data(), u.w, u.h);
      m = std::move(u);
    }
  }
  double s_ = 0, n_ = 0;
  for( size_t i = 0; i < m.d.size(); ++i ) {
    if( mask && !mask[i] ) continue;
    s_ += m.d[i], n_ += 1;
  }
  if( metric ) *metric = n_ > 0 ? s_ / n_ : 0;
  if( map ) memcpy(map, m.d.data(), m.d.size() * sizeof(double));
  return 0;
}
