/*
 * sst_oracle_accum.cc -- FP64 restatements of the other frame accumulators
 * of core/average/c_frame_accumulation.cc:
 *   - c_frame_accumulation_with_fft (:704-900): per-frame DFT of the frame
 *     padded to the optimal DFT size (BORDER_REFLECT, fftGetOptimalSize,
 *     core/proc/fft.cc:17-57), spectral weights max(s, (|F|^2 s)^3) with
 *     s = 1 / area^2 (fftPower :940-980), weighted spectral mean, inverse DFT,
 *     crop;
 *   - c_laplacian_pyramid_focus_stacking (:464-688) with build_laplacian_pyramid
 *     / reconstruct_laplacian_pyramid (core/proc/laplacian_pyramid.cc:45-122)
 *     and linear_interpolation_inpaint (core/proc/inpaint/
 *     linear_interpolation_inpaint.cc);
 *   - c_canvas_average (:264-450): a growing canvas, first frame centred,
 *     maintainCanvasBoundaries shifts, remap + running weighted mean.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of the GPU accumulators.
 *
 * OpenCV primitives follow their documented semantics: cv::dft (forward
 * sum x e^{-2 pi i k n / N}, DFT_SCALE divides by the element count),
 * cv::getOptimalDFTSize (smallest 2^a 3^b 5^c >= n), cv::pyrDown / pyrUp
 * (orc_pyrdown_border / orc_pyrup), u8 pyrDown rounding (sum + 128) >> 8,
 * cv::sepFilter2D with BORDER_REFLECT_101, cv::meanStdDev (population).
 */
#include "sst_oracle.h"
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

typedef std::complex<double> cplx;

int reflect_idx(int p, int n)      // BORDER_REFLECT: fedcba|abcdefgh|hgfedcb
{
  if( n == 1 ) return 0;
  while ( p < 0 || p >= n ) p = p < 0 ? -p - 1 : 2 * n - p - 1;
  return p;
}

int reflect101_idx(int p, int n)   // BORDER_REFLECT_101: gfedcb|abcdefgh|gfedcba
{
  if( n == 1 ) return 0;
  while ( p < 0 || p >= n ) p = p < 0 ? -p : 2 * (n - 1) - p;
  return p;
}

/* in-place 1-D DFT of n points spaced `stride` apart; sign -1 forward */
void dft1(cplx * x, int n, size_t stride, int sign, std::vector<cplx> & tmp)
{
  tmp.resize(n);
  std::vector<cplx> tw(n);
  for( int k = 0; k < n; ++k ) tw[k] = std::polar(1.0, sign * 2.0 * M_PI * k / n);
  for( int k = 0; k < n; ++k ) {
    cplx s = 0;
    for( int j = 0; j < n; ++j ) s += x[(size_t) j * stride] * tw[(size_t) j * k % n];
    tmp[k] = s;
  }
  for( int k = 0; k < n; ++k ) x[(size_t) k * stride] = tmp[k];
}

void dft2(std::vector<cplx> & a, int w, int h, int sign)
{
  std::vector<cplx> tmp;
  for( int y = 0; y < h; ++y ) dft1(a.data() + (size_t) y * w, w, 1, sign, tmp);
  for( int x = 0; x < w; ++x ) dft1(a.data() + x, h, w, sign, tmp);
}

/* planar multi-channel image */
struct Img {
  int w = 0, h = 0, cn = 1;
  std::vector<double> d;
  Img() = default;
  Img(int w_, int h_, int cn_) : w(w_), h(h_), cn(cn_), d((size_t) w_ * h_ * cn_, 0.0) {}
  double * plane(int c) { return d.data() + (size_t) c * w * h; }
  const double * plane(int c) const { return d.data() + (size_t) c * w * h; }
};

Img pyrdown(const Img & s)
{
  Img o((s.w + 1) / 2, (s.h + 1) / 2, s.cn);
  for( int c = 0; c < s.cn; ++c ) orc_pyrdown_border(s.plane(c), s.w, s.h, o.plane(c), o.w, o.h, ORC_BORDER_REFLECT101);
  return o;
}

Img pyrup(const Img & s, int dw, int dh)
{
  Img o(dw, dh, s.cn);
  for( int c = 0; c < s.cn; ++c ) orc_pyrup(s.plane(c), s.w, s.h, o.plane(c), dw, dh);
  return o;
}

/* build_laplacian_pyramid (laplacian_pyramid.cc:45-96): levels while the next
 * size's smaller side is above minimum_image_size */
std::vector<Img> build_lap(const Img & img, int minimum_image_size)
{
  std::vector<Img> lp;
  lp.push_back(img);
  while ( true ) {
    const int nw = (lp.back().w + 1) / 2, nh = (lp.back().h + 1) / 2;
    if( std::min(nw, nh) <= minimum_image_size ) break;
    Img down = pyrdown(lp.back());
    Img up = pyrup(down, lp.back().w, lp.back().h);
    for( size_t i = 0; i < up.d.size(); ++i ) lp.back().d[i] -= up.d[i];
    lp.push_back(std::move(down));
  }
  return lp;
}

/* reconstruct_laplacian_pyramid (laplacian_pyramid.cc:98-122) */
Img reconstruct(const std::vector<Img> & p)
{
  Img cur = p.back();
  for( int i = (int) p.size() - 2; i >= 0; --i ) {
    cur = pyrup(cur, p[i].w, p[i].h);
    for( size_t k = 0; k < cur.d.size(); ++k ) cur.d[k] += p[i].d[k];
  }
  return cur;
}

/* cv::pyrDown of a u8 plane: 5 x 5 [1 4 6 4 1]^2 / 256, REFLECT_101, rounded */
std::vector<uint8_t> pyrdown_u8(const std::vector<uint8_t> & s, int w, int h, int dw, int dh)
{
  static const int k[5] = { 1, 4, 6, 4, 1 };
  std::vector<uint8_t> o((size_t) dw * dh);
  for( int y = 0; y < dh; ++y ) {
    for( int x = 0; x < dw; ++x ) {
      int acc = 0;
      for( int j = 0; j < 5; ++j ) {
        const int yy = reflect101_idx(2 * y - 2 + j, h);
        for( int i = 0; i < 5; ++i ) acc += k[j] * k[i] * s[(size_t) yy * w + reflect101_idx(2 * x - 2 + i, w)];
      }
      o[(size_t) y * dw + x] = (uint8_t) ((acc + 128) >> 8);
    }
  }
  return o;
}

/* apply_mask (c_frame_accumulation.cc:509-525) */
void apply_mask(std::vector<Img> & lp, const uint8_t * mask, int w, int h)
{
  if( !mask ) return;
  std::vector<uint8_t> m(mask, mask + (size_t) w * h);
  int mw = w, mh = h;
  for( size_t i = 0; i + 1 < lp.size(); ++i ) {
    if( i > 0 ) {
      const int nw = (mw + 1) / 2, nh = (mh + 1) / 2;
      m = pyrdown_u8(m, mw, mh, nw, nh);
      mw = nw, mh = nh;
    }
    size_t holes = 0;
    for( uint8_t v : m ) holes += v < 255;
    if( !holes ) break;
    Img & L = lp[i];
    for( int c = 0; c < L.cn; ++c ) {
      double * p = L.plane(c);
      for( size_t k = 0; k < m.size(); ++k )
        if( m[k] < 255 ) p[k] = 0;
    }
  }
}

/* cv::sepFilter2D(src, dst, -1, G, G, anchor, delta), BORDER_REFLECT_101 */
void sep_filter(double * p, int w, int h, const double * g, int k, double delta)
{
  const int r = k / 2;
  std::vector<double> t((size_t) w * h);
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      double s = 0;
      for( int i = 0; i < k; ++i ) s += g[i] * p[(size_t) y * w + reflect101_idx(x - r + i, w)];
      t[(size_t) y * w + x] = s;
    }
  }
  for( int y = 0; y < h; ++y ) {
    for( int x = 0; x < w; ++x ) {
      double s = 0;
      for( int j = 0; j < k; ++j ) s += g[j] * t[(size_t) reflect101_idx(y - r + j, h) * w + x];
      p[(size_t) y * w + x] = s + delta;
    }
  }
}

/* compute_energy (c_frame_accumulation.cc:527-551): w = lap^2 per channel, or
 * (sum of channels)^2 when avgc and cn > 1; smoothed by G (+1e-12); lap *= w */
Img compute_energy(Img & lap, const double * G, int gk, bool avgc)
{
  const size_t N = (size_t) lap.w * lap.h;
  Img w;
  if( !avgc || lap.cn == 1 ) {
    w = Img(lap.w, lap.h, lap.cn);
    for( size_t i = 0; i < w.d.size(); ++i ) w.d[i] = lap.d[i] * lap.d[i];
  }
  else {
    w = Img(lap.w, lap.h, 1);
    for( size_t i = 0; i < N; ++i ) {
      double s = 0;
      for( int c = 0; c < lap.cn; ++c ) s += lap.d[(size_t) c * N + i];
      w.d[i] = s * s;
    }
  }
  if( G ) for( int c = 0; c < w.cn; ++c ) sep_filter(w.plane(c), w.w, w.h, G, gk, 1e-12);
  for( int c = 0; c < lap.cn; ++c ) {
    const double * wp = w.plane(w.cn == lap.cn ? c : 0);
    double * lpc = lap.plane(c);
    for( size_t i = 0; i < N; ++i ) lpc[i] *= wp[i];
  }
  return w;
}

/* graystdev: the sum over channels of the population standard deviations */
double graystdev(const Img & m)
{
  const size_t N = (size_t) m.w * m.h;
  double sv = 0;
  for( int c = 0; c < m.cn; ++c ) {
    const double * p = m.plane(c);
    double mean = 0;
    for( size_t i = 0; i < N; ++i ) mean += p[i];
    mean /= N;
    double var = 0;
    for( size_t i = 0; i < N; ++i ) var += (p[i] - mean) * (p[i] - mean);
    sv += std::sqrt(var / N);
  }
  return sv;
}

/* linear_interpolation_inpaint (linear_interpolation_inpaint.cc): holes (mask
 * 0) filled from the nearest valid pixels of their row and column segment,
 * iterated until every hole is filled or no hole gains a value */
void linear_inpaint(Img & img, const uint8_t * mask_in)
{
  const int w = img.w, h = img.h, cn = img.cn;
  const size_t N = (size_t) w * h;
  std::vector<uint8_t> mask(mask_in, mask_in + N);
  long total = 0;
  for( uint8_t v : mask ) total += v == 0;
  if( total < 1 ) return;
  Img ih(w, h, cn), iv(w, h, cn);
  std::vector<double> hd(N), vd(N);
  while ( total > 0 ) {
    std::fill(hd.begin(), hd.end(), 0.0);
    std::fill(vd.begin(), vd.end(), 0.0);
    // rows (_interpolate_holes_h2)
    for( int y = 0; y < h; ++y ) {
      const uint8_t * m = mask.data() + (size_t) y * w;
      for( int start = 0; start < w; ) {
        while ( start < w && m[start] ) ++start;
        if( start >= w ) break;
        int end = start + 1;
        while ( end < w && !m[end] ) ++end;
        for( int x = start; x < end; ++x ) {
          const size_t i = (size_t) y * w + x;
          if( start > 0 && end < w ) {
            const int s = start - 1, e = end;
            hd[i] = std::max(x - s, e - x);
            for( int c = 0; c < cn; ++c ) {
              const double sv = img.plane(c)[(size_t) y * w + s], ev = img.plane(c)[(size_t) y * w + e];
              ih.plane(c)[i] = sv + (x - s) * ((ev - sv) * (1.0 / (end - start)));
            }
          }
          else if( start > 0 ) {
            hd[i] = x - (start - 1);
            for( int c = 0; c < cn; ++c ) ih.plane(c)[i] = img.plane(c)[(size_t) y * w + start - 1];
          }
          else if( end < w ) {
            hd[i] = end - x;
            for( int c = 0; c < cn; ++c ) ih.plane(c)[i] = img.plane(c)[(size_t) y * w + end];
          }
        }
        start = end;
      }
    }
    // columns (_interpolate_holes_v2)
    for( int x = 0; x < w; ++x ) {
      for( int start = 0; start < h; ) {
        while ( start < h && mask[(size_t) start * w + x] ) ++start;
        if( start >= h ) break;
        int end = start + 1;
        while ( end < h && !mask[(size_t) end * w + x] ) ++end;
        for( int y = start; y < end; ++y ) {
          const size_t i = (size_t) y * w + x;
          if( start > 0 && end < h ) {
            const int s = start - 1, e = end;
            vd[i] = std::max(y - s, e - y);
            for( int c = 0; c < cn; ++c ) {
              const double sv = img.plane(c)[(size_t) s * w + x], ev = img.plane(c)[(size_t) e * w + x];
              iv.plane(c)[i] = sv + (y - s) * ((ev - sv) * (1.0 / (end - start)));
            }
          }
          else if( start > 0 ) {
            vd[i] = y - (start - 1);
            for( int c = 0; c < cn; ++c ) iv.plane(c)[i] = img.plane(c)[(size_t) (start - 1) * w + x];
          }
          else if( end < h ) {
            vd[i] = end - y;
            for( int c = 0; c < cn; ++c ) iv.plane(c)[i] = img.plane(c)[(size_t) end * w + x];
          }
        }
        start = end;
      }
    }
    // fill (_fill_holes2)
    long filled = 0;
    for( size_t i = 0; i < N; ++i ) {
      if( mask[i] ) continue;
      const double dh = hd[i], dv = vd[i];
      if( dh > 0 && dv > 0 ) {
        const double dd = 1.0 / (dh + dv);
        for( int c = 0; c < cn; ++c ) img.plane(c)[i] = dd * (ih.plane(c)[i] * dv + iv.plane(c)[i] * dh);
      }
      else if( dv > 0 ) for( int c = 0; c < cn; ++c ) img.plane(c)[i] = iv.plane(c)[i];
      else if( dh > 0 ) for( int c = 0; c < cn; ++c ) img.plane(c)[i] = ih.plane(c)[i];
      else continue;
      mask[i] = 255, ++filled;
    }
    if( filled < 1 ) break;
    total -= filled;
  }
}

Img from_hwc(const double * src, int w, int h, int cn)
{
  Img m(w, h, cn);
  const size_t N = (size_t) w * h;
  for( size_t i = 0; i < N; ++i )
    for( int c = 0; c < cn; ++c ) m.d[(size_t) c * N + i] = src[i * cn + c];
  return m;
}

void to_hwc(const Img & m, double * dst)
{
  const size_t N = (size_t) m.w * m.h;
  for( size_t i = 0; i < N; ++i )
    for( int c = 0; c < m.cn; ++c ) dst[i * m.cn + c] = m.d[(size_t) c * N + i];
}

bool is_235(int m)
{
  for( int f : { 2, 3, 5 } ) while ( m % f == 0 ) m /= f;
  return m == 1;
}

}  // namespace

/* cv::getOptimalDFTSize: the smallest 2^a 3^b 5^c >= n */
extern "C" int orc_optimal_dft_size(int n)
{
  if( n <= 1 ) return 1;
  int m = n;
  while ( !is_235(m) ) ++m;
  return m;
}

/* c_frame_accumulation_with_fft: n frames (h x w x cn, interleaved) -> avg
 * (h x w x cn). Mono frames whose size is already optimal get their spectral
 * weights like every other frame (the reference leaves them empty there). */
extern "C" int orc_fft_average(const double * frames, int n, int w, int h, int cn, double * avg)
{
  if( n < 1 || w < 1 || h < 1 || cn < 1 ) return -1;
  const int fw = orc_optimal_dft_size(w), fh = orc_optimal_dft_size(h);
  const int top = (fh - h) / 2, left = (fw - w) / 2;
  const size_t F = (size_t) fw * fh;
  const double s = 1.0 / ((double) F * (double) F);
  for( int c = 0; c < cn; ++c ) {
    std::vector<cplx> A(F, 0.0);
    std::vector<double> W(F, 0.0);
    std::vector<cplx> P(F);
    for( int f = 0; f < n; ++f ) {
      const double * fr = frames + (size_t) f * w * h * cn;
      for( int y = 0; y < fh; ++y )
        for( int x = 0; x < fw; ++x )
          P[(size_t) y * fw + x] = fr[((size_t) reflect_idx(y - top, h) * w + reflect_idx(x - left, w)) * cn + c];
      dft2(P, fw, fh, -1);
      for( size_t k = 0; k < F; ++k ) {
        const double a = P[k].real(), b = P[k].imag();
        const double q = (a * a + b * b) * s;
        const double wk = std::max(s, q * q * q);
        A[k] += P[k] * wk;
        W[k] += wk;
      }
    }
    for( size_t k = 0; k < F; ++k ) A[k] /= W[k];
    dft2(A, fw, fh, +1);
    for( int y = 0; y < h; ++y )
      for( int x = 0; x < w; ++x )
        avg[((size_t) y * w + x) * cn + c] = A[(size_t) (y + top) * fw + x + left].real() / (double) F;
  }
  return 0;
}

/* c_laplacian_pyramid_focus_stacking: n frames (h x w x cn) with optional
 * u8 masks (n x h x w); policy 0 select_max_energy, 1 weighted_average;
 * G (gk taps, may be NULL) the smoothing kernel of the energies. -> avg
 * (h x w x cn). Returns the number of pyramid levels. */
extern "C" int orc_focus_stack(const double * frames, const uint8_t * masks, int n, int w, int h, int cn, int policy,
    int inpaint, int avgchannel, const double * G, int gk, double * avg)
{
  if( n < 1 || w < 1 || h < 1 || cn < 1 ) return -1;
  std::vector<Img> acc, wwp;
  for( int f = 0; f < n; ++f ) {
    Img img = from_hwc(frames + (size_t) f * w * h * cn, w, h, cn);
    const uint8_t * m = masks ? masks + (size_t) f * w * h : nullptr;
    if( inpaint && m ) linear_inpaint(img, m);
    std::vector<Img> pyr = build_lap(img, 8);
    apply_mask(pyr, m, w, h);
    const int L = (int) pyr.size();
    if( f == 0 ) {
      acc = std::move(pyr);
      if( policy == 1 ) {
        wwp.resize(L - 1);
        for( int i = 0; i < L - 1; ++i ) wwp[i] = compute_energy(acc[i], G, gk, avgchannel != 0);
      }
      continue;
    }
    const double sv0 = graystdev(acc.back()), sv1 = graystdev(pyr.back());
    const double a0 = sv0 / (sv0 + sv1), a1 = sv1 / (sv0 + sv1);
    for( size_t k = 0; k < acc.back().d.size(); ++k ) acc.back().d[k] = acc.back().d[k] * a0 + pyr.back().d[k] * a1;
    for( int i = 0; i < L - 1; ++i ) {
      if( policy == 0 ) {
        Img w0 = acc[i], w1 = pyr[i];
        for( double & v : w0.d ) v = std::fabs(v);
        for( double & v : w1.d ) v = std::fabs(v);
        if( G ) {
          for( int c = 0; c < cn; ++c ) {
            sep_filter(w0.plane(c), w0.w, w0.h, G, gk, 0.0);
            sep_filter(w1.plane(c), w1.w, w1.h, G, gk, 0.0);
          }
        }
        for( size_t k = 0; k < acc[i].d.size(); ++k )
          if( w1.d[k] > w0.d[k] ) acc[i].d[k] = pyr[i].d[k];
      }
      else {
        Img ww = compute_energy(pyr[i], G, gk, avgchannel != 0);
        for( size_t k = 0; k < acc[i].d.size(); ++k ) acc[i].d[k] += pyr[i].d[k];
        for( size_t k = 0; k < ww.d.size(); ++k ) wwp[i].d[k] += ww.d[k];
      }
    }
  }
  Img out;
  if( policy == 0 ) out = reconstruct(acc);
  else {
    std::vector<Img> lp(acc.size());
    const int L = (int) acc.size();
    for( int i = 0; i < L - 1; ++i ) {
      lp[i] = acc[i];
      const size_t N = (size_t) acc[i].w * acc[i].h;
      for( int c = 0; c < acc[i].cn; ++c ) {
        const double * wp = wwp[i].plane(wwp[i].cn == acc[i].cn ? c : 0);
        double * p = lp[i].plane(c);
        for( size_t k = 0; k < N; ++k ) p[k] /= wp[k];
      }
    }
    lp.back() = acc.back();
    out = reconstruct(lp);
  }
  to_hwc(out, avg);
  return (int) acc.size();
}

/* c_canvas_average over a sequence. Frame f (h x w x cn) comes with weights
 * (wkind 0 none, 1 u8 masks (n x h x w), 2 f64 weights (n x h x w)), a box
 * boxes[4f..4f+3] = x, y, width, height (width 0: no remap; the first frame is
 * never remapped) and, for boxes with width > 0, a remap of the box's size
 * (interleaved x, y), consecutive in `rmaps`. canvas: in (cw, ch) the
 * requested minimum size, out the canvas size; acc (ch x cw x cn) and W
 * (ch x cw) must hold max(request, 3/2 frame) sized planes. Per frame
 * status[f]: 0 added, 1 counted but not added (box clipped by the canvas),
 * -1 rejected (empty ROI). last[4]: the final bbox. */
extern "C" int orc_canvas_average(const double * frames, int n, int w, int h, int cn, int wkind, const void * weights,
    const int * boxes, const double * rmaps, int * canvas, double * acc, double * W, int * status, int * last)
{
  const int cw = std::max(canvas[0], 3 * w / 2), ch = std::max(canvas[1], 3 * h / 2);
  canvas[0] = cw, canvas[1] = ch;
  std::vector<double> A((size_t) cw * ch * cn, 0.0), Wt((size_t) cw * ch, 0.0);
  int lx = 0, ly = 0, lw = 0, lh = 0;
  size_t roff = 0;
  auto update = [&](int rx, int ry, int rw, int rh, const std::vector<double> & img, const std::vector<double> & wt) {
    for( int y = 0; y < rh; ++y ) {
      for( int x = 0; x < rw; ++x ) {
        const size_t i = (size_t) y * rw + x, o = (size_t) (ry + y) * cw + rx + x;
        const double wn = wt.empty() ? 1.0 : wt[i];
        if( !(wn > 0) ) continue;
        const double Wn = Wt[o] + wn, fac = wn / Wn;
        Wt[o] = Wn;
        for( int c = 0; c < cn; ++c ) A[o * cn + c] += (img[i * cn + c] - A[o * cn + c]) * fac;
      }
    }
  };
  for( int f = 0; f < n; ++f ) {
    const double * fr = frames + (size_t) f * w * h * cn;
    std::vector<double> img(fr, fr + (size_t) w * h * cn), wt;
    if( wkind == 1 ) {
      const uint8_t * m = (const uint8_t *) weights + (size_t) f * w * h;
      wt.resize((size_t) w * h);
      for( size_t i = 0; i < wt.size(); ++i ) wt[i] = m[i] ? 1.0 : 0.0;
    }
    else if( wkind == 2 ) {
      const double * p = (const double *) weights + (size_t) f * w * h;
      wt.assign(p, p + (size_t) w * h);
    }
    const int * b = boxes + 4 * f;
    if( f == 0 ) {
      const int tx = cw / 2 - w / 2, ty = ch / 2 - h / 2;
      update(tx, ty, w, h, img, wt);
      lx = tx, ly = ty, lw = w, lh = h;
      status[f] = 0;
      if( b[2] > 0 ) roff += (size_t) b[2] * b[3] * 2;
      continue;
    }
    if( b[2] <= 0 ) {
      const int x0 = std::max(lx, 0), y0 = std::max(ly, 0);
      const int x1 = std::min(lx + w, cw), y1 = std::min(ly + h, ch);
      const int rw = std::max(0, x1 - x0), rh = std::max(0, y1 - y0);
      if( rw == w && rh == h ) update(x0, y0, w, h, img, wt), status[f] = 0;
      else status[f] = 1;
      lx = x0, ly = y0, lw = rw, lh = rh;
      continue;
    }
    const double * rm = rmaps + roff;
    roff += (size_t) b[2] * b[3] * 2;
    int x0 = std::max(b[0], 0), y0 = std::max(b[1], 0);
    const int x1 = std::min(b[0] + b[2], cw), y1 = std::min(b[1] + b[3], ch);
    int rw = x1 - x0, rh = y1 - y0;
    if( rw <= 0 || rh <= 0 ) {
      status[f] = -1;
      continue;
    }
    // maintainCanvasBoundaries (c_frame_accumulation.cc:273-318)
    const int margin = 32;
    int sx = 0, sy = 0;
    if( x0 < margin ) sx = 2 * margin;
    else if( x0 + rw >= cw - margin ) sx = -2 * margin;
    if( y0 < margin ) sy = 2 * margin;
    else if( y0 + rh >= ch - margin ) sy = -2 * margin;
    if( sx || sy ) {
      const int copy_w = cw - std::abs(sx), copy_h = ch - std::abs(sy);
      if( copy_w > 0 && copy_h > 0 ) {
        const int srx = sx > 0 ? 0 : -sx, sry = sy > 0 ? 0 : -sy, dsx = sx > 0 ? sx : 0, dsy = sy > 0 ? sy : 0;
        std::vector<double> nA(A.size(), 0.0), nW(Wt.size(), 0.0);
        for( int y = 0; y < copy_h; ++y ) {
          for( int x = 0; x < copy_w; ++x ) {
            const size_t so = (size_t) (sry + y) * cw + srx + x, dso = (size_t) (dsy + y) * cw + dsx + x;
            nW[dso] = Wt[so];
            for( int c = 0; c < cn; ++c ) nA[dso * cn + c] = A[so * cn + c];
          }
        }
        A.swap(nA), Wt.swap(nW);
        x0 += sx, y0 += sy;
      }
    }
    if( x0 < 0 || y0 < 0 || x0 + rw > cw || y0 + rh > ch ) {
      status[f] = -1;
      continue;
    }
    // remap: image LINEAR / REPLICATE, u8 masks NEAREST / f64 weights LINEAR, CONSTANT 0
    const int bw = b[2], bh = b[3];
    std::vector<double> rimg((size_t) bw * bh * cn), rwt;
    std::vector<double> plane((size_t) w * h);
    for( int c = 0; c < cn; ++c ) {
      for( size_t i = 0; i < plane.size(); ++i ) plane[i] = img[i * cn + c];
      for( size_t i = 0; i < (size_t) bw * bh; ++i )
        rimg[i * cn + c] = orc_sample_bilinear(plane.data(), w, h, rm[2 * i], rm[2 * i + 1], ORC_BORDER_REPLICATE, 0.0);
    }
    if( wkind ) {
      rwt.resize((size_t) bw * bh);
      for( size_t i = 0; i < rwt.size(); ++i ) {
        if( wkind == 1 ) {
          const int xi = (int) std::nearbyint(rm[2 * i]), yi = (int) std::nearbyint(rm[2 * i + 1]);
          rwt[i] = (xi >= 0 && xi < w && yi >= 0 && yi < h) ? wt[(size_t) yi * w + xi] : 0.0;
        }
        else rwt[i] = orc_sample_bilinear(wt.data(), w, h, rm[2 * i], rm[2 * i + 1], ORC_BORDER_CONSTANT, 0.0);
      }
    }
    if( rw == bw && rh == bh ) update(x0, y0, rw, rh, rimg, rwt), status[f] = 0;
    else status[f] = 1;
    lx = x0, ly = y0, lw = rw, lh = rh;
  }
  memcpy(acc, A.data(), A.size() * sizeof(double));
  memcpy(W, Wt.data(), Wt.size() * sizeof(double));
  last[0] = lx, last[1] = ly, last[2] = lw, last[3] = lh;
  return 0;
}

/* linear_interpolation_inpaint(image, mask) on its own: image (h x w x cn)
 * in place */
extern "C" void orc_linear_inpaint(double * image, const uint8_t * mask, int w, int h, int cn)
{
  Img m = from_hwc(image, w, h, cn);
  linear_inpaint(m, mask);
  to_hwc(m, image);
}

namespace {

/* median_filter_bad_pixels / bayer_denoise on one plane view: the plane pixel
 * (x, y) is frame pixel (step x + ox, step y + oy) */
template<class T>
void bad_pixels_plane(const T * src, T * dst, int w, int step, int ox, int oy, int pw, int ph, int ks, float k,
    float mv, bool integral)
{
  const int r = ks / 2;
  auto at = [&](int x, int y) -> float { return (float) src[(size_t) (step * y + oy) * w + step * x + ox]; };
  std::vector<float> med((size_t) pw * ph), mad((size_t) pw * ph);
  std::vector<float> win(ks * ks);
  for( int y = 0; y < ph; ++y ) {
    for( int x = 0; x < pw; ++x ) {
      for( int j = 0; j < ks; ++j )
        for( int i = 0; i < ks; ++i )
          win[j * ks + i] = at(std::min(std::max(x + i - r, 0), pw - 1), std::min(std::max(y + j - r, 0), ph - 1));
      std::nth_element(win.begin(), win.begin() + ks * ks / 2, win.end());
      const float m = win[ks * ks / 2];
      med[(size_t) y * pw + x] = m;
      mad[(size_t) y * pw + x] = std::fabs(at(x, y) - m);
    }
  }
  for( int y = 0; y < ph; ++y ) {
    for( int x = 0; x < pw; ++x ) {
      double s = 0;
      for( int j = 0; j < ks; ++j )
        for( int i = 0; i < ks; ++i ) s += mad[(size_t) reflect101_idx(y + j - r, ph) * pw + reflect101_idx(x + i - r, pw)];
      const float q = integral ? (float) (((long long) s + ks * ks / 2) / (ks * ks)) : (float) (s * (1.0 / (ks * ks)));
      const float p = at(x, y), m = med[(size_t) y * pw + x];
      const float t = (float) ((double) k * q);
      const float thr = (float) ((double) t + mv);
      dst[(size_t) (step * y + oy) * w + step * x + ox] = (T) (std::fabs(m - p) > thr ? m : p);
    }
  }
}

template<class T>
int filter_bad_pixels(const T * src, int w, int h, int colorid, double threshold, T * dst, bool integral)
{
  const bool bayer = colorid >= 8 && colorid <= 11;
  if( bayer && ((w & 1) || (h & 1)) ) return -1;
  memcpy(dst, src, (size_t) w * h * sizeof(T));
  const float k = (float) threshold, mv = integral ? 1.f : 1.f / 256.f;
  if( bayer ) {
    for( int p = 0; p < 4; ++p ) bad_pixels_plane<T>(src, dst, w, 2, p & 1, p >> 1, w / 2, h / 2, 3, k, mv, integral);
  }
  else bad_pixels_plane<T>(src, dst, w, 1, 0, 0, w, h, 5, k, mv, integral);
  return 0;
}

}  // namespace

/* read_input_frame's bad-pixel filter (median_filter_bad_pixels,
 * core/proc/bad_pixels.cc:14-70; bayer_denoise, core/io/debayer.cc:1480-1612)
 * of one u16 or f32 frame; exact for u16 */
extern "C" int orc_filter_bad_pixels_u16(const uint16_t * src, int w, int h, int colorid, double threshold,
    uint16_t * dst)
{
  return filter_bad_pixels<uint16_t>(src, w, h, colorid, threshold, dst, true);
}

extern "C" int orc_filter_bad_pixels_f32(const float * src, int w, int h, int colorid, double threshold, float * dst)
{
  return filter_bad_pixels<float>(src, w, h, colorid, threshold, dst, false);
}
