/*
 * sst_taps.h -- host-built tap tables of separable resamplings (per output
 * index along one axis: K source indices and weights, zero weights pad):
 * cv::resize INTER_AREA / INTER_CUBIC, cv::pyrDown and cv::pyrUp, from the
 * functions' documented semantics.
 */
#pragma once
#include <math.h>
#include <algorithm>
#include <utility>
#include <vector>

#include "../../include/serstacker_gb300.h"

namespace {

/* per-axis tap tables (host build, FP64 weights rounded to f32) */
struct HostTaps {
  int K = 0;
  std::vector<int> idx;
  std::vector<float> w;
};

/* INTER_AREA: destination d averages source [d s, (d + 1) s), s = ssize / dsize;
 * partial cells at either end below 1e-3 of a pixel are dropped */
HostTaps area_taps(int ssize, int dsize)
{
  std::vector<std::vector<std::pair<int, double>>> t(dsize);
  const double scale = (double) ssize / dsize;
  size_t K = 1;
  for( int d = 0; d < dsize; ++d ) {
    const double f1 = d * scale, f2 = f1 + scale;
    const double cell = std::min(scale, ssize - f1);
    const int s1 = (int) ceil(f1), s2 = std::min((int) floor(f2), ssize);
    if( s1 - f1 > 1e-3 && s1 - 1 >= 0 ) t[d].push_back({ s1 - 1, (s1 - f1) / cell });
    for( int s = s1; s < s2; ++s ) t[d].push_back({ s, 1.0 / cell });
    if( s2 < ssize && f2 - s2 > 1e-3 ) t[d].push_back({ s2, std::min(std::min(f2 - s2, 1.0), cell) / cell });
    K = std::max(K, t[d].size());
  }
  HostTaps h;
  h.K = (int) K;
  h.idx.assign((size_t) dsize * K, 0);
  h.w.assign((size_t) dsize * K, 0.f);
  for( int d = 0; d < dsize; ++d ) {
    for( size_t k = 0; k < t[d].size(); ++k ) {
      h.idx[(size_t) d * K + k] = t[d][k].first;
      h.w[(size_t) d * K + k] = (float) t[d][k].second;
    }
  }
  return h;
}

/* INTER_CUBIC: Keys kernel a = -0.75 at (d + 0.5) s - 0.5, taps clamped to the image */
HostTaps cubic_taps(int ssize, int dsize)
{
  HostTaps h;
  h.K = 4;
  h.idx.resize((size_t) dsize * 4);
  h.w.resize((size_t) dsize * 4);
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
    for( int k = 0; k < 4; ++k ) {
      h.idx[(size_t) d * 4 + k] = std::min(std::max(sx - 1 + k, 0), ssize - 1);
      h.w[(size_t) d * 4 + k] = (float) w[k];
    }
  }
  return h;
}

/* identity (copy) taps for equal sizes */
HostTaps copy_taps(int n)
{
  HostTaps h;
  h.K = 1;
  h.idx.resize(n);
  h.w.assign(n, 1.f);
  for( int i = 0; i < n; ++i ) h.idx[i] = i;
  return h;
}

/* 5-tap pyrDown along one axis: dst d reads 2d - 2 .. 2d + 2 (REFLECT_101,
 * or BORDER_REPLICATE when `replicate`) */
HostTaps pyr_taps(int ssize, int dsize, bool replicate = false)
{
  HostTaps h;
  h.K = 5;
  h.idx.resize((size_t) dsize * 5);
  h.w.resize((size_t) dsize * 5);
  const float k[5] = { 1 / 16.f, 4 / 16.f, 6 / 16.f, 4 / 16.f, 1 / 16.f };
  for( int d = 0; d < dsize; ++d ) {
    for( int i = 0; i < 5; ++i ) {
      int s = 2 * d + i - 2;
      if( ssize == 1 ) s = 0;
      else if( replicate ) s = std::min(std::max(s, 0), ssize - 1);
      else {
        while ( s < 0 || s >= ssize ) s = s < 0 ? -s : 2 * ssize - 2 - s;
      }
      h.idx[(size_t) d * 5 + i] = s;
      h.w[(size_t) d * 5 + i] = k[i];
    }
  }
  return h;
}

/* cv::pyrUp along one axis: the source at the even positions of a 2 ssize
 * grid (zeros between), convolved with 2 x [1 4 6 4 1] / 16 under
 * BORDER_REFLECT_101 on that grid; dsize (2 ssize or 2 ssize - 1) keeps its
 * first dsize samples */
HostTaps pyrup_taps(int ssize, int dsize)
{
  const double k[5] = { 1 / 16., 4 / 16., 6 / 16., 4 / 16., 1 / 16. };
  const int n = 2 * ssize;
  std::vector<std::vector<std::pair<int, double>>> t(dsize);
  size_t K = 1;
  for( int d = 0; d < dsize; ++d ) {
    for( int i = -2; i <= 2; ++i ) {
      int u = d + i;
      if( n > 1 ) while ( u < 0 || u >= n ) u = u < 0 ? -u : 2 * (n - 1) - u;
      else u = 0;
      if( u & 1 ) continue;
      bool found = false;
      for( auto & pr : t[d] ) if( pr.first == u / 2 ) pr.second += 2 * k[i + 2], found = true;
      if( !found ) t[d].push_back({ u / 2, 2 * k[i + 2] });
    }
    K = std::max(K, t[d].size());
  }
  HostTaps h;
  h.K = (int) K;
  h.idx.assign((size_t) dsize * K, 0);
  h.w.assign((size_t) dsize * K, 0.f);
  for( int d = 0; d < dsize; ++d ) {
    for( size_t q = 0; q < t[d].size(); ++q ) {
      h.idx[(size_t) d * K + q] = t[d][q].first;
      h.w[(size_t) d * K + q] = (float) t[d][q].second;
    }
  }
  return h;
}

}  // namespace
