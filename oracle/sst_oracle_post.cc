/*
 * sst_oracle_post.cc -- FP64 restatement of the stacking pipeline's
 * post-stack hole filling (test infrastructure only: the oracle for a GPU
 * implementation, never shipped).
 *
 * average_pyramid_inpaint (core/proc/inpaint/average_pyramid_inpaint.cc:
 * 18-126), called on the master frame after compute()
 * (c_image_stacking_pipeline.cc:763-767, max_levels 100), with its helpers
 * downstrike_even (core/proc/downstrike.cc:35-75: keeps rows / columns
 * 1, 3, 5 ... clamped to the last one) and upject_even (downstrike.cc:256-370:
 * source pixel (y, x) to (2y + 1, 2x + 1), zeros elsewhere, and a mask of the
 * copied positions).
 */
#include <math.h>
#include <string.h>
#include <algorithm>
#include <vector>

#include "sst_oracle.h"

namespace {

struct plane {
  int w = 0, h = 0;
  std::vector<double> v;
  plane() = default;
  plane(int w_, int h_) : w(w_), h(h_), v((size_t) w_ * h_, 0.0) {}
  double & at(int x, int y) { return v[(size_t) y * w + x]; }
  double at(int x, int y) const { return v[(size_t) y * w + x]; }
};

/* 3 x 3 box sum (not normalised), BORDER_REPLICATE */
plane box3(const plane & s)
{
  plane d(s.w, s.h);
  for( int y = 0; y < s.h; ++y )
    for( int x = 0; x < s.w; ++x ) {
      double a = 0;
      for( int j = -1; j <= 1; ++j )
        for( int i = -1; i <= 1; ++i )
          a += s.at(std::min(std::max(x + i, 0), s.w - 1), std::min(std::max(y + j, 0), s.h - 1));
      d.at(x, y) = a;
    }
  return d;
}

/* _average_pyramid_filter2 (average_pyramid_inpaint.cc:18-58): box sums of
 * the image and the mask; a pixel valid in the fallback takes the fallback's
 * value, else one with a non-zero mask sum takes the mean; both get mask 1 */
void filter2(const plane & src, const plane & srcmask, plane & dst, plane & dstmask, const plane & fb,
    const plane & fbmask)
{
  plane d = box3(src), m = box3(srcmask);
  for( size_t i = 0; i < d.v.size(); ++i ) {
    if( fbmask.v[i] != 0 ) {
      m.v[i] = 1;
      d.v[i] = fb.v[i];
    }
    else if( m.v[i] != 0 ) {
      d.v[i] = d.v[i] / m.v[i];
      m.v[i] = 1;
    }
  }
  dst = std::move(d);
  dstmask = std::move(m);
}

plane downstrike(const plane & s)
{
  plane d((s.w + 1) / 2, (s.h + 1) / 2);
  for( int y = 0; y < d.h; ++y )
    for( int x = 0; x < d.w; ++x ) d.at(x, y) = s.at(std::min(2 * x + 1, s.w - 1), std::min(2 * y + 1, s.h - 1));
  return d;
}

/* upject to w x h: (y, x) -> (2y + 1, 2x + 1) where that fits; zmask marks
 * the copied positions */
plane upject(const plane & s, int w, int h, plane * zmask)
{
  plane d(w, h), z(w, h);
  for( int y = 0; y < s.h; ++y ) {
    if( 2 * y + 1 >= h ) break;
    for( int x = 0; x < s.w; ++x ) {
      if( 2 * x + 1 >= w ) break;
      d.at(2 * x + 1, 2 * y + 1) = s.at(x, y);
      z.at(2 * x + 1, 2 * y + 1) = 1;
    }
  }
  *zmask = std::move(z);
  return d;
}

/* average_pyramid_recurse (average_pyramid_inpaint.cc:69-94) */
void recurse(plane & image, plane & mask, int max_levels)
{
  if( std::min(image.w, image.h) <= 1 || max_levels <= 0 ) return;
  plane fi, fm;
  filter2(image, mask, fi, fm, image, mask);
  fi = downstrike(fi);
  fm = downstrike(fm);
  size_t nz = 0;
  for( double v : fm.v ) nz += v != 0;
  if( nz < fm.v.size() ) recurse(fi, fm, max_levels - 1);
  plane zm;
  plane up = upject(fi, image.w, image.h, &zm);
  filter2(up, zm, fi, fm, image, mask);
  image = std::move(fi);
  mask = std::move(fm);
}

}  // namespace

extern "C" void orc_average_pyramid_inpaint(const double * src, const uint8_t * mask, int w, int h, int max_levels,
    double * dst, uint8_t * dstmask)
{
  const size_t n = (size_t) w * h;
  size_t nz = 0;
  for( size_t i = 0; i < n; ++i ) nz += mask[i] != 0;
  if( nz == n ) {
    memcpy(dst, src, n * sizeof(double));
    memcpy(dstmask, mask, n);
    return;
  }
  plane img(w, h), msk(w, h);
  for( size_t i = 0; i < n; ++i ) {
    img.v[i] = mask[i] ? src[i] : 0.0;
    msk.v[i] = mask[i] / 255.0;
  }
  recurse(img, msk, max_levels);
  for( size_t i = 0; i < n; ++i ) {
    dst[i] = img.v[i];
    const double m = std::min(std::max(msk.v[i] * 255.0, 0.0), 255.0);
    dstmask[i] = (uint8_t) lrint(m);
  }
}
