/*
 * sst_model.cuh -- the c_image_transform family in FP64, usable on host and
 * device: parameter packing, eps(), scale_transfrom(), invert_and_compose(),
 * conversion between models and the FP32 displacement coefficients consumed
 * by the per-pixel kernels.
 *
 * Transform state: 16 doubles.
 *   translation : tx ty                          (c_image_transform.cc:80-269)
 *   euclidean   : Tx Ty angle scale Cx Cy        (c_image_transform.cc:275-833)
 *   affine      : a00 a01 a02 a10 a11 a12        (c_image_transform.cc:837-1070)
 *   homography  : a00 a01 a02 a10 a11 a12 a20 a21, a22 = 1 (c_image_transform.cc:1074-1366)
 *   semi-quad.  : a00 a01 a02 a03 a10 a11 a12 a13 (c_image_transform.cc:1370-1612)
 *   quadratic   : a00..a05 a10..a15              (c_image_transform.cc:1616-1868)
 * The ECC parameter vector p (c_image_transform::parameters()) equals the
 * state except for euclidean, where it is the subset the fix flags leave free.
 */
#pragma once
#include <math.h>
#include <string.h>
#include "../../include/serstacker_gb300.h"

#ifdef __CUDACC__
#define SST_HD __host__ __device__
#else
#define SST_HD
#endif

namespace sst {

SST_HD inline bool is_euclid(int t) { return t == SST_MOTION_EUCLIDEAN || t == SST_MOTION_SCALED_EUCLIDEAN; }
SST_HD inline bool is_homog(int t) { return t == SST_MOTION_HOMOGRAPHY || t == SST_MOTION_EPIPOLAR_DEROTATION; }

SST_HD inline int model_nparams(const sst_motion_model & m)
{
  switch ( m.type ) {
  case SST_MOTION_TRANSLATION: return 2;
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN:
    return (m.fix_translation ? 0 : 2) + (m.fix_rotation ? 0 : 1) + (m.fix_scale ? 0 : 1);
  case SST_MOTION_AFFINE: return 6;
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: return 8;
  case SST_MOTION_SEMI_QUADRATIC: return 8;
  case SST_MOTION_QUADRATIC: return 12;
  }
  return 0;
}

SST_HD inline bool model_invertible(const sst_motion_model & m)
{
  return m.type != SST_MOTION_SEMI_QUADRATIC && m.type != SST_MOTION_QUADRATIC;
}

SST_HD inline void model_identity(const sst_motion_model & m, double * s)
{
  for( int i = 0; i < 16; ++i ) s[i] = 0;
  switch ( m.type ) {
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN: s[3] = 1; break;
  case SST_MOTION_AFFINE:
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: s[0] = 1, s[4] = 1; break;
  case SST_MOTION_SEMI_QUADRATIC: s[0] = 1, s[5] = 1; break;     // cv::Matx24f::eye()
  case SST_MOTION_QUADRATIC: s[0] = 1, s[7] = 1; break;          // cv::Matx26f::eye()
  }
}

SST_HD inline void model_get_params(const sst_motion_model & m, const double * s, double * p)
{
  if( is_euclid(m.type) ) {
    int i = 0;
    if( !m.fix_translation ) p[i++] = s[0], p[i++] = s[1];
    if( !m.fix_rotation ) p[i++] = s[2];
    if( !m.fix_scale ) p[i++] = s[3];
  }
  else {
    const int n = model_nparams(m);
    for( int i = 0; i < n; ++i ) p[i] = s[i];
  }
}

SST_HD inline void model_set_params(const sst_motion_model & m, double * s, const double * p)
{
  if( is_euclid(m.type) ) {
    int i = 0;
    if( !m.fix_translation ) s[0] = p[i++], s[1] = p[i++];
    if( !m.fix_rotation ) s[2] = p[i++];
    if( !m.fix_scale ) s[3] = p[i++];
  }
  else {
    const int n = model_nparams(m);
    for( int i = 0; i < n; ++i ) s[i] = p[i];
  }
}

SST_HD inline double sqd(double x) { return x * x; }

/* eps(dp, image_size) of each model; for euclidean a fixed component
 * contributes its stored absolute value (c_image_transform.cc:407-421,509-523) */
SST_HD inline double model_eps(const sst_motion_model & m, const double * s, const double * dp, int W, int H)
{
  switch ( m.type ) {
  case SST_MOTION_TRANSLATION:
    return sqrt(dp[0] * dp[0] + dp[1] * dp[1]);
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN: {
    int i = 0;
    double dTx, dTy, da, ds;
    if( m.fix_translation ) dTx = s[0], dTy = s[1];
    else dTx = dp[i++], dTy = dp[i++];
    da = m.fix_rotation ? s[2] : dp[i++];
    ds = m.fix_scale ? s[3] : dp[i++];
    const double sa = sin(da);
    const double mx = W > H ? W : H;
    return sqrt(sqd(dTx) + sqd(dTy) + sqd(W * sa) + sqd(H * sa) + sqd(mx * ds));
  }
  case SST_MOTION_AFFINE:
    return sqrt(sqd(W * dp[0]) + sqd(H * dp[1]) + sqd(dp[2]) + sqd(W * dp[3]) + sqd(H * dp[4]) + sqd(dp[5]));
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION:
    return sqrt(sqd(dp[2]) + sqd(dp[5]) + sqd(W * dp[0]) + sqd(H * dp[1]) + sqd(W * dp[3]) + sqd(H * dp[4]));
  case SST_MOTION_SEMI_QUADRATIC: {
    const double WH = (double) W * H;
    return sqrt(sqd(dp[2]) + sqd(dp[6]) + sqd(W * dp[0]) + sqd(H * dp[1]) + sqd(W * dp[4]) + sqd(H * dp[5]) +
        sqd(WH * dp[3]) + sqd(WH * dp[7]));
  }
  case SST_MOTION_QUADRATIC: {
    const double WH = (double) W * H, WW = (double) W * W, HH = (double) H * H;
    return sqrt(sqd(dp[2]) + sqd(dp[8]) + sqd(W * dp[0]) + sqd(H * dp[1]) + sqd(W * dp[6]) + sqd(H * dp[7]) +
        sqd(WH * dp[3]) + sqd(WH * dp[9]) + sqd(WW * dp[4]) + sqd(WW * dp[10]) + sqd(HH * dp[5]) + sqd(HH * dp[11]));
  }
  }
  return 0;
}

/* scale_transfrom(factor) */
SST_HD inline void model_scale(const sst_motion_model & m, double * a, double f)
{
  switch ( m.type ) {
  case SST_MOTION_TRANSLATION: a[0] *= f, a[1] *= f; break;
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN: a[0] *= f, a[1] *= f, a[4] *= f, a[5] *= f; break;
  case SST_MOTION_AFFINE: a[2] *= f, a[5] *= f; break;
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: a[2] *= f, a[5] *= f, a[6] /= f, a[7] /= f; break;
  case SST_MOTION_SEMI_QUADRATIC: a[2] *= f, a[3] /= f, a[6] *= f, a[7] /= f; break;
  case SST_MOTION_QUADRATIC:
    a[2] *= f, a[3] /= f, a[4] /= f, a[5] /= f;
    a[8] *= f, a[9] /= f, a[10] /= f, a[11] /= f;
    break;
  }
}

/* cv::invertAffineTransform */
SST_HD inline void invert_affine(const double * a, double * r)
{
  double D = a[0] * a[4] - a[1] * a[3];
  D = D != 0 ? 1.0 / D : 0.0;
  const double A11 = a[4] * D, A22 = a[0] * D, A12 = -a[1] * D, A21 = -a[3] * D;
  r[0] = A11, r[1] = A12, r[2] = -A11 * a[2] - A12 * a[5];
  r[3] = A21, r[4] = A22, r[5] = -A21 * a[2] - A22 * a[5];
}

SST_HD inline bool inv3(const double * a, double * r)
{
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
  const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  if( det == 0 ) {
    for( int i = 0; i < 9; ++i ) r[i] = 0;
    return false;
  }
  const double id = 1.0 / det;
  r[0] = c00 * id;
  r[1] = (a[2] * a[7] - a[1] * a[8]) * id;
  r[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  r[3] = c01 * id;
  r[4] = (a[0] * a[8] - a[2] * a[6]) * id;
  r[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  r[6] = c02 * id;
  r[7] = (a[1] * a[6] - a[0] * a[7]) * id;
  r[8] = (a[0] * a[4] - a[1] * a[3]) * id;
  return true;
}

SST_HD inline void euclid_matrix(double tX, double tY, double ang, double scl, double cX, double cY, double * M)
{
  const double sa = sin(ang), ca = cos(ang);
  M[0] = scl * ca, M[1] = -scl * sa, M[2] = tX - scl * ca * cX + scl * sa * cY;
  M[3] = scl * sa, M[4] = scl * ca, M[5] = tY - scl * sa * cX - scl * ca * cY;
}

/* invert_and_compose(p, dp): c_image_transform.h:159-167 (translation),
 * c_image_transform.cc:737-833 (euclidean), c_image_transform.h:309-317
 * (affine), c_image_transform.h:372-377 (homography). */
SST_HD inline bool model_invert_and_compose(const sst_motion_model & m, const double * s, const double * dp, double * out)
{
  for( int i = 0; i < 16; ++i ) out[i] = s[i];
  switch ( m.type ) {
  case SST_MOTION_TRANSLATION:
    out[0] = s[0] - dp[0], out[1] = s[1] - dp[1];
    return true;
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN: {
    const double Tx = s[0], Ty = s[1], angle = s[2], scale = s[3], Cx = s[4], Cy = s[5];
    int i = 0;
    double dTx = 0, dTy = 0, dA = 0, dS = 0;
    if( !m.fix_translation ) dTx = dp[i++], dTy = dp[i++];
    if( !m.fix_rotation ) dA = dp[i++];
    if( !m.fix_scale ) dS = dp[i++];
    const double scale_dp = m.fix_scale ? 1.0 : 1.0 + dS;
    double Mp[6], Mdp[6], Mi[6], R[6];
    euclid_matrix(Tx, Ty, angle, scale, Cx, Cy, Mp);
    euclid_matrix(dTx, dTy, dA, scale_dp, Cx, Cy, Mdp);
    invert_affine(Mdp, Mi);
    R[0] = Mp[0] * Mi[0] + Mp[1] * Mi[3];
    R[1] = Mp[0] * Mi[1] + Mp[1] * Mi[4];
    R[2] = Mp[0] * Mi[2] + Mp[1] * Mi[5] + Mp[2];
    R[3] = Mp[3] * Mi[0] + Mp[4] * Mi[3];
    R[4] = Mp[3] * Mi[1] + Mp[4] * Mi[4];
    R[5] = Mp[3] * Mi[2] + Mp[4] * Mi[5] + Mp[5];
    const double rs = m.fix_scale ? scale : sqrt(R[0] * R[0] + R[3] * R[3]);
    const double ra = m.fix_rotation ? angle : atan2(R[3], R[0]);
    const double rc = cos(ra), rsn = sin(ra);
    out[0] = m.fix_translation ? Tx : R[2] + rs * rc * Cx - rs * rsn * Cy;
    out[1] = m.fix_translation ? Ty : R[5] + rs * rsn * Cx + rs * rc * Cy;
    out[2] = ra;
    out[3] = rs;
    return true;
  }
  case SST_MOTION_AFFINE: {
    double a[6], b[6];
    invert_affine(s, a);
    for( int k = 0; k < 6; ++k ) a[k] += dp[k];
    invert_affine(a, b);
    for( int k = 0; k < 6; ++k ) out[k] = b[k];
    return true;
  }
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: {
    const double M[9] = { s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], 1.0 };
    double Mi[9], R[9];
    inv3(M, Mi);
    const double dM[9] = { dp[0], dp[1], dp[2], dp[3], dp[4], dp[5], dp[6], dp[7], 0.0 };
    for( int k = 0; k < 9; ++k ) Mi[k] += dM[k];
    inv3(Mi, R);
    const double nrm = 1.0 / R[8];
    for( int k = 0; k < 8; ++k ) out[k] = R[k] * nrm;
    return true;
  }
  }
  return false;
}

/* 2x3 affine view of a translation / euclidean / affine state */
SST_HD inline void model_affine_view(const sst_motion_model & m, const double * s, double * a)
{
  a[0] = 1, a[1] = 0, a[2] = 0, a[3] = 0, a[4] = 1, a[5] = 0;
  switch ( m.type ) {
  case SST_MOTION_TRANSLATION: a[2] = s[0], a[5] = s[1]; break;
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN: euclid_matrix(s[0], s[1], s[2], s[3], s[4], s[5], a); break;
  case SST_MOTION_AFFINE:
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: for( int i = 0; i < 6; ++i ) a[i] = s[i]; break;
  case SST_MOTION_SEMI_QUADRATIC:
    a[0] = s[0], a[1] = s[1], a[2] = s[2], a[3] = s[4], a[4] = s[5], a[5] = s[6];
    break;
  case SST_MOTION_QUADRATIC:
    a[0] = s[0], a[1] = s[1], a[2] = s[2], a[3] = s[6], a[4] = s[7], a[5] = s[8];
    break;
  }
}

/* Start state of a pass from the previous pass's result: a projective state
 * is kept, everything else goes through its affine view (the reference's
 * set_affine_matrix / set_matrix conversions, c_image_transform.cc:1447-1463). */
SST_HD inline void model_convert(const sst_motion_model & from, const double * s, const sst_motion_model & to, double * out)
{
  model_identity(to, out);
  double a[6];
  model_affine_view(from, s, a);
  switch ( to.type ) {
  case SST_MOTION_TRANSLATION: out[0] = a[2], out[1] = a[5]; break;
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN:
    out[0] = a[2], out[1] = a[5];
    out[2] = atan2(a[3], a[0]);
    if( !to.fix_scale ) out[3] = sqrt(a[0] * a[0] + a[3] * a[3]);
    break;
  case SST_MOTION_AFFINE: for( int i = 0; i < 6; ++i ) out[i] = a[i]; break;
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION:
    if( is_homog(from.type) ) for( int i = 0; i < 8; ++i ) out[i] = s[i];
    else for( int i = 0; i < 6; ++i ) out[i] = a[i];
    break;
  case SST_MOTION_SEMI_QUADRATIC:
    out[0] = a[0], out[1] = a[1], out[2] = a[2], out[4] = a[3], out[5] = a[4], out[6] = a[5];
    if( from.type == SST_MOTION_SEMI_QUADRATIC ) for( int i = 0; i < 8; ++i ) out[i] = s[i];
    break;
  case SST_MOTION_QUADRATIC:
    out[0] = a[0], out[1] = a[1], out[2] = a[2], out[6] = a[3], out[7] = a[4], out[8] = a[5];
    if( from.type == SST_MOTION_SEMI_QUADRATIC ) out[3] = s[3], out[9] = s[7];
    if( from.type == SST_MOTION_QUADRATIC ) for( int i = 0; i < 12; ++i ) out[i] = s[i];
    break;
  }
}

/* FP32 displacement coefficients (layout in sst_internal.cuh): 16 floats,
 * the translation's integer part in c[12], c[13] */
SST_HD inline void model_warp_coeffs(const sst_motion_model & m, const double * s, float * c)
{
  for( int i = 0; i < 16; ++i ) c[i] = 0.f;
  double tx, ty;
  if( m.type == SST_MOTION_SEMI_QUADRATIC ) tx = s[2], ty = s[6];
  else if( m.type == SST_MOTION_QUADRATIC ) tx = s[2], ty = s[8];
  else {
    double a[6];
    model_affine_view(m, s, a);
    tx = a[2], ty = a[5];
  }
  // integer part of the translation; non-finite or huge values keep 0
  const double Ix = (tx == tx && fabs(tx) < 1e6) ? floor(tx + 0.5) : 0.0;
  const double Iy = (ty == ty && fabs(ty) < 1e6) ? floor(ty + 0.5) : 0.0;
  c[12] = (float) Ix, c[13] = (float) Iy;
  if( m.type == SST_MOTION_SEMI_QUADRATIC ) {
    c[0] = (float) (s[0] - 1.0), c[1] = (float) s[1], c[2] = (float) (s[2] - Ix), c[3] = (float) s[3];
    c[6] = (float) s[4], c[7] = (float) (s[5] - 1.0), c[8] = (float) (s[6] - Iy), c[9] = (float) s[7];
    return;
  }
  if( m.type == SST_MOTION_QUADRATIC ) {
    c[0] = (float) (s[0] - 1.0), c[1] = (float) s[1], c[2] = (float) (s[2] - Ix);
    for( int i = 3; i < 6; ++i ) c[i] = (float) s[i];
    c[6] = (float) s[6], c[7] = (float) (s[7] - 1.0), c[8] = (float) (s[8] - Iy);
    for( int i = 9; i < 12; ++i ) c[i] = (float) s[i];
    return;
  }
  double a[6];
  model_affine_view(m, s, a);
  if( is_euclid(m.type) ) {
    // a00 - 1 = s cos - 1 computed without cancellation: -2 s sin^2(t/2) + (s - 1)
    const double h = sin(0.5 * s[2]);
    a[0] = s[3] * (-2.0 * h * h) + (s[3] - 1.0) + 1.0;
    a[4] = a[0];
    c[0] = (float) (s[3] * (-2.0 * h * h) + (s[3] - 1.0));
    c[4] = c[0];
  }
  else {
    c[0] = (float) (a[0] - 1.0);
    c[4] = (float) (a[4] - 1.0);
  }
  c[1] = (float) a[1], c[2] = (float) (a[2] - Ix);
  c[3] = (float) a[3], c[5] = (float) (a[5] - Iy);
  if( is_homog(m.type) ) c[6] = (float) s[6], c[7] = (float) s[7];
}

/* Per-frame constants of the steepest-descent images at the current state
 * (create_steepest_descent_images): euclidean {scale, sin, cos, Cx, Cy},
 * homography {a00 .. a21}. */
SST_HD inline void model_sd_coeffs(const sst_motion_model & m, const double * s, float * j)
{
  for( int i = 0; i < 8; ++i ) j[i] = 0.f;
  if( is_euclid(m.type) ) {
    j[0] = (float) s[3], j[1] = (float) sin(s[2]), j[2] = (float) cos(s[2]);
    j[3] = (float) s[4], j[4] = (float) s[5];
  }
  else if( is_homog(m.type) ) {
    for( int i = 0; i < 8; ++i ) j[i] = (float) s[i];
  }
}

/* FP64 Cholesky solve of A x = b, A n x n SPD (n <= 12). false if not SPD. */
SST_HD inline bool cholesky_solve(const double * A, const double * b, int n, double * x)
{
  double L[12 * 12];
  for( int i = 0; i < n; ++i ) {
    for( int j = 0; j <= i; ++j ) {
      double s = A[i * n + j];
      for( int k = 0; k < j; ++k ) s -= L[i * 12 + k] * L[j * 12 + k];
      if( i == j ) {
        if( !(s > 0) ) return false;
        L[i * 12 + i] = sqrt(s);
      }
      else {
        L[i * 12 + j] = s / L[j * 12 + j];
      }
    }
  }
  double y[12];
  for( int i = 0; i < n; ++i ) {
    double s = b[i];
    for( int k = 0; k < i; ++k ) s -= L[i * 12 + k] * y[k];
    y[i] = s / L[i * 12 + i];
  }
  for( int i = n - 1; i >= 0; --i ) {
    double s = y[i];
    for( int k = i + 1; k < n; ++k ) s -= L[k * 12 + i] * x[k];
    x[i] = s / L[i * 12 + i];
  }
  return true;
}

}  // namespace sst
