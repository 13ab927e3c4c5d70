/*
 * sst_oracle_reg.cc -- FP64 restatement of c_frame_registration's ECC glue.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of the parity tests. Only tests/,
 * __graft_entry__.smoke() and bench.py's checker legs use it.
 *
 * Reference anchors (core/proc/image_registration/ unless stated):
 *   scaleImage                        c_frame_registration.cc:230-250
 *   setup_reference_frame (ECC part)  c_frame_registration.cc:565-636
 *   register_frame (ECC part)         c_frame_registration.cc:788-896
 *   ecc_downscale / ecc_upscale       ecc2.cc:223-272
 *   ecc_normalize                     ecc2.cc:385-397
 *   translation() / set_translation() c_image_transform.cc:91-116, 425-434, 864-873, 1124-1139
 *
 * OpenCV primitives, from their documented semantics:
 *   cv::pyrDown(src, dst, Size(), border): dst size ((w + 1) / 2, (h + 1) / 2),
 *     5 x 5 [1 4 6 4 1] / 16 separable, dst(x, y) centred on src(2x, 2y);
 *     on CV_8U the weights are the integers 1 4 6 4 1 and the result is
 *     (sum + 128) >> 8.
 *   cv::pyrUp(src, dst, dsize): the source with zero rows / columns inserted
 *     (src at even positions of a 2w x 2h grid), convolved with the same
 *     kernel times 4, BORDER_REFLECT_101 on that 2w x 2h grid; a dsize of
 *     2w - 1 (2h - 1) keeps its first 2w - 1 (2h - 1) samples.
 *   cv::resize(src, dst, Size(0, 0), s, s, INTER_AREA): dst size
 *     (cvRound(w s), cvRound(h s)), pixel-area averages (orc_resize_area);
 *     on CV_8U the average is rounded to the nearest integer.
 */
#include "sst_oracle.h"
#include <cmath>
#include <cfloat>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

int border_index(int p, int n, int border)
{
  if( p >= 0 && p < n ) return p;
  if( border == ORC_BORDER_REPLICATE ) return p < 0 ? 0 : n - 1;
  if( n == 1 ) return 0;
  while ( p < 0 || p >= n ) {   // REFLECT_101
    if( p < 0 ) p = -p;
    if( p >= n ) p = 2 * (n - 1) - p;
  }
  return p;
}

const double K5[5] = { 1 / 16., 4 / 16., 6 / 16., 4 / 16., 1 / 16. };

/* pyrUp along one axis: dst d of the zero-inserted 2s grid (REFLECT_101 on it) */
void pyrup_axis(int s, int d, std::vector<std::vector<std::pair<int, double>>> & t)
{
  t.assign(d, {});
  for( int k = 0; k < d; ++k ) {
    for( int i = -2; i <= 2; ++i ) {
      const int u = border_index(k + i, 2 * s, ORC_BORDER_REFLECT101);
      if( u & 1 ) continue;
      const int si = u / 2;
      const double wt = 2 * K5[i + 2];
      bool found = false;
      for( auto & pr : t[k] ) if( pr.first == si ) pr.second += wt, found = true;
      if( !found ) t[k].push_back({ si, wt });
    }
  }
}

std::vector<double> pyrdown_b(const std::vector<double> & src, int w, int h, int dw, int dh, int border)
{
  std::vector<double> tmp((size_t) dw * h), dst((size_t) dw * dh);
  for( int y = 0; y < h; ++y )
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( int i = 0; i < 5; ++i ) a += K5[i] * src[(size_t) y * w + border_index(2 * x + i - 2, w, border)];
      tmp[(size_t) y * dw + x] = a;
    }
  for( int y = 0; y < dh; ++y )
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( int j = 0; j < 5; ++j ) a += K5[j] * tmp[(size_t) border_index(2 * y + j - 2, h, border) * dw + x];
      dst[(size_t) y * dw + x] = a;
    }
  return dst;
}

/* cv::saturate_cast<int>(double): round half to even */
int cv_round(double v)
{
  return (int) std::nearbyint(v);
}

}  // namespace

extern "C" void orc_pyrdown_border(const double * src, int w, int h, double * dst, int dw, int dh, int border)
{
  std::vector<double> s(src, src + (size_t) w * h);
  std::vector<double> d = pyrdown_b(s, w, h, dw, dh, border);
  memcpy(dst, d.data(), d.size() * sizeof(double));
}

extern "C" void orc_pyrup(const double * src, int sw, int sh, double * dst, int dw, int dh)
{
  std::vector<std::vector<std::pair<int, double>>> tx, ty;
  pyrup_axis(sw, dw, tx);
  pyrup_axis(sh, dh, ty);
  std::vector<double> tmp((size_t) dw * sh);
  for( int y = 0; y < sh; ++y )
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( auto & pr : tx[x] ) a += pr.second * src[(size_t) y * sw + pr.first];
      tmp[(size_t) y * dw + x] = a;
    }
  for( int y = 0; y < dh; ++y )
    for( int x = 0; x < dw; ++x ) {
      double a = 0;
      for( auto & pr : ty[y] ) a += pr.second * tmp[(size_t) pr.first * dw + x];
      dst[(size_t) y * dw + x] = a;
    }
}

/* cv::pyrDown of a CV_8U mask (REFLECT_101, integer weights, rounded), then
 * cv::compare(>= 250) (c_frame_registration.cc:236-239) */
extern "C" void orc_mask_pyrdown_ge250(const uint8_t * src, int w, int h, uint8_t * dst, int dw, int dh)
{
  static const int k[5] = { 1, 4, 6, 4, 1 };
  for( int y = 0; y < dh; ++y )
    for( int x = 0; x < dw; ++x ) {
      int s = 0;
      for( int j = 0; j < 5; ++j ) {
        const int yy = border_index(2 * y + j - 2, h, ORC_BORDER_REFLECT101);
        int r = 0;
        for( int i = 0; i < 5; ++i ) r += k[i] * src[(size_t) yy * w + border_index(2 * x + i - 2, w, ORC_BORDER_REFLECT101)];
        s += k[j] * r;
      }
      dst[(size_t) y * dw + x] = ((s + 128) >> 8) >= 250 ? 255 : 0;
    }
}

/* scaleImage (c_frame_registration.cc:230-250): returns the scaled size */
extern "C" void orc_scale_image_size(int w, int h, double scale, int * dw, int * dh)
{
  if( std::abs(scale - 0.5) < 1e-2 ) *dw = (w + 1) / 2, *dh = (h + 1) / 2;
  else *dw = cv_round(w * scale), *dh = cv_round(h * scale);
}

extern "C" void orc_scale_image(const double * src, const uint8_t * mask, int w, int h, double scale, double * dst,
    uint8_t * dst_mask)
{
  int dw, dh;
  orc_scale_image_size(w, h, scale, &dw, &dh);
  if( std::abs(scale - 0.5) < 1e-2 ) {
    orc_pyrdown_border(src, w, h, dst, dw, dh, ORC_BORDER_REFLECT101);
    if( mask && dst_mask ) orc_mask_pyrdown_ge250(mask, w, h, dst_mask, dw, dh);
  }
  else {
    orc_resize_area(src, w, h, dst, dw, dh);
    if( mask && dst_mask ) {
      std::vector<double> m((size_t) w * h), md((size_t) dw * dh);
      for( size_t i = 0; i < m.size(); ++i ) m[i] = mask[i];
      orc_resize_area(m.data(), w, h, md.data(), dw, dh);
      for( size_t i = 0; i < md.size(); ++i ) dst_mask[i] = cv_round(md[i]) >= 250 ? 255 : 0;
    }
  }
}

/* ecc_normalize(src, mask, dst, lvl) (ecc2.cc:385-397): src minus the
 * pyrDown^lvl (BORDER_REPLICATE) / pyrUp (ecc_upscale sizes) background,
 * zero where the mask is 0 */
extern "C" void orc_ecc_normalize(const double * src, const uint8_t * mask, int w, int h, int lvl, double * dst)
{
  std::vector<int> ws(1, w), hs(1, h);
  std::vector<double> m(src, src + (size_t) w * h);
  for( int l = 0; l < std::max(lvl, 1); ++l ) {
    const int nw = (ws.back() + 1) / 2, nh = (hs.back() + 1) / 2;
    m = pyrdown_b(m, ws.back(), hs.back(), nw, nh, ORC_BORDER_REPLICATE);
    ws.push_back(nw), hs.push_back(nh);
  }
  // ecc_upscale: the chain of sizes from the destination, halved (rounding up)
  // until the downscaled size, then pyrUp through them coarse to fine
  for( int i = (int) ws.size() - 2; i >= 0; --i ) {
    std::vector<double> up((size_t) ws[i] * hs[i]);
    orc_pyrup(m.data(), ws[i + 1], hs[i + 1], up.data(), ws[i], hs[i]);
    m.swap(up);
  }
  for( size_t i = 0; i < (size_t) w * h; ++i ) dst[i] = (mask && !mask[i]) ? 0.0 : src[i] - m[i];
}

/* c_frame_registration with ECC registration only (no feature registration,
 * no eccflow): setup_reference_frame(reference, reference_mask) and
 * register_frame(current) for one frame. The returned state is the full
 * resolution transform of o->motion_type. status: 0 OK, 3 rho below the
 * gate (0.75 min_rho after the translation estimate, min_rho after the
 * final alignment) */
extern "C" int orc_register_frame(const orc_registration_opts * o, const double * ref, const uint8_t * ref_mask,
    int w, int h, const double * cur, double * state, double * rho_out, int * iters_out)
{
  const bool scaled = o->scale > 0 && o->scale != 1;
  int ew = w, eh = h;
  if( scaled ) orc_scale_image_size(w, h, o->scale, &ew, &eh);
  const size_t EN = (size_t) ew * eh;
  std::vector<double> er(EN), ec(EN);
  std::vector<uint8_t> em;
  if( ref_mask ) em.resize(EN);
  if( scaled ) {
    orc_scale_image(ref, ref_mask, w, h, o->scale, er.data(), ref_mask ? em.data() : nullptr);
    orc_scale_image(cur, nullptr, w, h, o->scale, ec.data(), nullptr);
  }
  else {
    memcpy(er.data(), ref, EN * sizeof(double));
    memcpy(ec.data(), cur, EN * sizeof(double));
    if( ref_mask ) memcpy(em.data(), ref_mask, EN);
  }
  if( o->normalization_scale > 0 && o->normalization_noise > 0 ) {
    orc_ecc_normalize(er.data(), ref_mask ? em.data() : nullptr, ew, eh, o->normalization_scale, er.data());
    orc_ecc_normalize(ec.data(), nullptr, ew, eh, o->normalization_scale, ec.data());
  }
  orc_ecch_opts eo;
  eo.epsx = o->eps;
  eo.reference_smooth_sigma = o->reference_smooth_sigma;
  eo.input_smooth_sigma = o->input_smooth_sigma;
  eo.update_step_scale = o->update_step_scale;
  eo.method = o->method;
  eo.max_iterations = o->max_iterations;
  eo.minimum_image_size = o->ecch_minimum_image_size;
  eo.maxlevel = o->ecch_max_level;
  eo.ic_jacobian_at_identity = 1;
  orc_model m = { o->motion_type, 0, 0, o->motion_type == ORC_MOTION_EUCLIDEAN ? 1 : 0 };
  orc_model_identity(&m, state);
  const uint8_t * rm = ref_mask ? em.data() : nullptr;
  int total = 0;
  if( o->motion_type != ORC_MOTION_TRANSLATION && o->estimate_translation_first && o->ecch_max_level != 0 ) {
    orc_model tm = { ORC_MOTION_TRANSLATION, 0, 0, 0 };
    double ts[16];
    orc_model_identity(&tm, ts);   // the translation of the default transform
    int it = 0;
    double e = 0, rho = 0;
    orc_ecch_align_pyramids(&tm, ts, &eo, er.data(), rm, ec.data(), ew, eh, &it, &e, &rho);
    total += it;
    *rho_out = rho;
    if( rho < 0.75 * o->min_rho ) {
      *iters_out = total;
      return 3;
    }
    // set_translation(): the translation of an identity transform of the model
    switch ( m.type ) {
    case ORC_MOTION_EUCLIDEAN:
    case ORC_MOTION_SCALED_EUCLIDEAN: state[0] = ts[0], state[1] = ts[1]; break;
    case ORC_MOTION_SEMI_QUADRATIC: state[2] = ts[0], state[6] = ts[1]; break;
    case ORC_MOTION_QUADRATIC: state[2] = ts[0], state[8] = ts[1]; break;
    default: state[2] = ts[0], state[5] = ts[1]; break;   // affine; homography with a22 = 1
    }
  }
  int it = 0;
  double e = 0, rho = 0;
  orc_ecch_align_pyramids(&m, state, &eo, er.data(), rm, ec.data(), ew, eh, &it, &e, &rho);
  total += it;
  *rho_out = rho;
  *iters_out = total;
  if( rho < o->min_rho ) return 3;
  if( scaled ) orc_model_scale(&m, state, 1.0 / o->scale);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* debayer NN2 (core/io/debayer.cc:828-1161, _debayer_nn2_interpolation): per
 * pixel, its own colour as it is; green at a red or blue site the mean of the
 * 4 cross neighbours; at a green site the colour of its row neighbours the
 * mean of those 2, the other colour the mean of the 2 column neighbours; red
 * at a blue site (and blue at a red one) the mean of the 4 diagonal
 * neighbours. Neighbours outside the frame reflect (BORDER_REFLECT_101: row
 * -1 is row 1, column w is column w - 2). Integer frames round the means
 * half up ((sum + n / 2) / n in integer arithmetic), float ones do not.
 * Output: B, G, R interleaved. colorid: 8 RGGB, 9 GRBG, 10 GBRG, 11 BGGR. */
namespace {

/* colour (0 B, 1 G, 2 R) of mosaic position (x, y) */
int bayer_color(int colorid, int x, int y)
{
  static const int pat[4][4] = {
    { 2, 1, 1, 0 },   // RGGB, index (y & 1) * 2 + (x & 1)
    { 1, 2, 0, 1 },   // GRBG
    { 1, 0, 2, 1 },   // GBRG
    { 0, 1, 1, 2 },   // BGGR
  };
  return pat[colorid - 8][(y & 1) * 2 + (x & 1)];
}

/* sums in the accumulation type A (int64 for integer frames, float for
 * float ones, added left to right in the order N W E S / NW NE SW SE / W E /
 * N S as the reference adds them) */
template<class T, class A>
void nn2(const T * src, int w, int h, int colorid, T * dst, bool integral)
{
  auto at = [&](int x, int y) -> A {
    x = x < 0 ? -x : (x >= w ? 2 * (w - 1) - x : x);
    y = y < 0 ? -y : (y >= h ? 2 * (h - 1) - y : y);
    return (A) src[(size_t) y * w + x];
  };
  auto mean = [&](A s, int n) -> T {
    if( integral ) return (T) (((long long) s + n / 2) / n);
    return (T) (s / (A) n);
  };
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      const int own = bayer_color(colorid, x, y);
      T out[3];
      for( int ch = 0; ch < 3; ++ch ) {
        if( ch == own ) out[ch] = (T) at(x, y);
        else if( ch == 1 ) out[ch] = mean(at(x, y - 1) + at(x - 1, y) + at(x + 1, y) + at(x, y + 1), 4);
        else if( own == 1 ) {
          if( bayer_color(colorid, x + 1, y) == ch ) out[ch] = mean(at(x - 1, y) + at(x + 1, y), 2);
          else out[ch] = mean(at(x, y - 1) + at(x, y + 1), 2);
        }
        else out[ch] = mean(at(x - 1, y - 1) + at(x + 1, y - 1) + at(x - 1, y + 1) + at(x + 1, y + 1), 4);
      }
      T * d = dst + ((size_t) y * w + x) * 3;
      d[0] = out[0], d[1] = out[1], d[2] = out[2];
    }
  }
}

}  // namespace

extern "C" int orc_debayer_nn2_u16(const uint16_t * src, int w, int h, int colorid, uint16_t * dst)
{
  if( (w & 1) || (h & 1) || colorid < 8 || colorid > 11 ) return -1;
  nn2<uint16_t, long long>(src, w, h, colorid, dst, true);
  return 0;
}

extern "C" int orc_debayer_nn2_f32(const float * src, int w, int h, int colorid, float * dst)
{
  if( (w & 1) || (h & 1) || colorid < 8 || colorid > 11 ) return -1;
  nn2<float, float>(src, w, h, colorid, dst, false);
  return 0;
}
