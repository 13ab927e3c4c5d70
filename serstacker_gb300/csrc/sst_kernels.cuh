/*
 * sst_kernels.cuh -- device building blocks shared by the Gauss-Newton passes
 * and the adjoint: the steepest-descent rows of every motion model and the
 * tensor-core Gram-matrix accumulation.
 */
#pragma once
#include "sst_engine.cuh"

namespace sst {

/* ------------------------------------------------- steepest-descent images */

/* create_steepest_descent_images for one pixel (c_image_transform.cc:262-269,
 * 587-668, 1045-1070, 1319-1366, 1583-1612, 1834-1868). jc holds the per-frame
 * constants of model_sd_coeffs(). */
template<int JK, int M>
__device__ __forceinline__ void sd_pixel(const float * jc, float x, float y, float gx, float gy, float * J)
{
  if( JK == J_TRANS ) {
    J[0] = gx, J[1] = gy;
  }
  else if( JK == J_EUCL ) {
    const float sc = jc[0], sa = jc[1], ca = jc[2];
    const float xx = x - jc[3], yy = y - jc[4];
    J[0] = gx, J[1] = gy;
    const float u = ca * xx - sa * yy, v = sa * xx + ca * yy;
    J[2] = sc * (-gx * v + gy * u);
    if( M > 3 ) J[3 < M ? 3 : 0] = gx * u + gy * v;
  }
  else if( JK == J_AFFINE ) {
    J[0] = gx * x, J[1] = gx * y, J[2] = gx;
    J[3] = gy * x, J[4] = gy * y, J[5] = gy;
  }
  else if( JK == J_HOMOG ) {
    const float den = __fdividef(1.0f, fmaf(x, jc[6], fmaf(y, jc[7], 1.0f)));
    const float hatX = -fmaf(x, jc[0], fmaf(y, jc[1], jc[2])) * den;
    const float hatY = -fmaf(x, jc[3], fmaf(y, jc[4], jc[5])) * den;
    const float ggx = gx * den, ggy = gy * den;
    const float gg = hatX * ggx + hatY * ggy;
    J[0] = ggx * x, J[1] = ggx * y, J[2] = ggx;
    J[3] = ggy * x, J[4] = ggy * y, J[5] = ggy;
    J[6 < M ? 6 : 0] = gg * x;
    J[7 < M ? 7 : 0] = gg * y;
  }
  else if( JK == J_SEMIQ ) {
    const float xy = x * y;
    J[0] = gx * x, J[1] = gx * y, J[2] = gx, J[3] = gx * xy;
    J[4] = gy * x, J[5] = gy * y, J[6 < M ? 6 : 0] = gy, J[7 < M ? 7 : 0] = gy * xy;
  }
  else {
    const float xy = x * y, xx = x * x, yy = y * y;
    J[0] = gx * x, J[1] = gx * y, J[2] = gx, J[3] = gx * xy, J[4] = gx * xx, J[5] = gx * yy;
    J[6 < M ? 6 : 0] = gy * x, J[7 < M ? 7 : 0] = gy * y, J[8 < M ? 8 : 0] = gy;
    J[9 < M ? 9 : 0] = gy * xy, J[10 < M ? 10 : 0] = gy * xx, J[11 < M ? 11 : 0] = gy * yy;
  }
}

/* ---- tensor-core Gram matrix (3xTF32 mma.sync) */

/* f32 -> tf32 (round to nearest, ties away), as the b32 operand of mma */
__device__ __forceinline__ uint32_t to_tf32(float x)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

/* D = A B + D, A 16 x 8 (row), B 8 x 8 (col), tf32 operands, f32 accumulate */
__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
    uint32_t b0, uint32_t b1)
{
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

/* G += V^T V over the 32 pixels staged by one warp: sv holds 32 rows of 16
 * components (row stride GV_LD floats). A = V^T in k-chunks of 8 pixels,
 * B = V; the operands are split x = hi + lo (tf32 each) and the three
 * products hi.hi + hi.lo + lo.hi keep FP32-level accuracy. g0 holds
 * G[:, 0:8], g1 G[:, 8:16] in the m16n8 accumulator layout. */
constexpr int GV_LD = 24;   // 16 components + pad: conflict-free fragment loads

__device__ __forceinline__ void gram_accumulate(const float * sv, float (&g0)[4], float (&g1)[4])
{
  const int lane = threadIdx.x & 31, gq = lane >> 2, tq = lane & 3;
#pragma unroll
  for( int c = 0; c < 4; ++c ) {
    const float * r0 = sv + (8 * c + tq) * GV_LD, * r1 = sv + (8 * c + tq + 4) * GV_LD;
    const float x0 = r0[gq], x1 = r0[gq + 8], x2 = r1[gq], x3 = r1[gq + 8];
    const uint32_t h0 = to_tf32(x0), h1 = to_tf32(x1), h2 = to_tf32(x2), h3 = to_tf32(x3);
    const uint32_t l0 = to_tf32(x0 - __uint_as_float(h0)), l1 = to_tf32(x1 - __uint_as_float(h1));
    const uint32_t l2 = to_tf32(x2 - __uint_as_float(h2)), l3 = to_tf32(x3 - __uint_as_float(h3));
    // A fragment: rows (components) gq / gq + 8, columns (pixels) tq / tq + 4;
    // B fragment of the n-tile [n0, n0 + 8): rows (pixels) tq / tq + 4, column n0 + gq
    mma_tf32(g0, h0, h1, h2, h3, h0, h2);
    mma_tf32(g0, h0, h1, h2, h3, l0, l2);
    mma_tf32(g0, l0, l1, l2, l3, h0, h2);
    mma_tf32(g1, h0, h1, h2, h3, h1, h3);
    mma_tf32(g1, h0, h1, h2, h3, l1, l3);
    mma_tf32(g1, l0, l1, l2, l3, h1, h3);
  }
}

}  // namespace sst
