/*
 * sst_replicas.cu -- merge of partial accumulator states, for replicas that
 * each stack a contiguous range of the frames (one process per GPU) and
 * combine their compensated planes once at the end.
 *
 * A state is a run of groups of four planes: sum of w*I, its compensation,
 * sum of w, its compensation (c_weigthed_average: one group, c_bayer_average:
 * one group per channel B, G, R). The merge is error-free in the leading
 * terms: s = a + b is rounded, its rounding error e comes from TwoSum
 * (Knuth), and the compensation of the result is ca + cb + e. Merging the
 * partial states of ranks 0, 1, ..., N-1 in that fixed order gives the same
 * planes on every run.
 *
 * Host code only: the planes are small (a few x width x height) next to the
 * frames, and the merge runs once per sequence.
 */
#include <stddef.h>
#include <stdint.h>
#include "../../include/serstacker_gb300.h"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu

static inline void two_sum_merge(float & s, float & c, float s2, float c2)
{
  const float t = s + s2;
  const float bb = t - s;
  const float e = (s - (t - bb)) + (s2 - bb);
  c = (c + c2) + e;
  s = t;
}

extern "C" int sst_state_merge(float * dst, const float * src, int groups, size_t plane)
{
  if( !dst || !src || groups < 1 || plane == 0 ) return sst_internal_error(SST_ERR_INVALID_ARG, "sst_state_merge: invalid arguments");
  for( int g = 0; g < groups; ++g ) {
    float * D = dst + (size_t) g * 4 * plane;
    const float * S = src + (size_t) g * 4 * plane;
    for( size_t i = 0; i < plane; ++i ) {
      two_sum_merge(D[i], D[plane + i], S[i], S[plane + i]);
      two_sum_merge(D[2 * plane + i], D[3 * plane + i], S[2 * plane + i], S[3 * plane + i]);
    }
  }
  return SST_OK;
}
