/*
 * sst_oracle_model.cc -- FP64 restatement of the c_image_transform family.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle of the parity tests, never part of the product).
 *
 * Follows core/proc/image_registration/c_image_transform.cc:
 *   translation    :   80-269   (create_remap 150-170, eps 136-139, SD 262-269)
 *   euclidean      :  275-833   (get_parameters 385-424, eps 509-523,
 *                                create_remap 525-555, SD 587-668,
 *                                invert_and_compose 737-833, scale 502-507)
 *   affine         :  837-1070  (eps 911-917, create_remap 919-937, SD 1045-1070,
 *                                invert_and_compose c_image_transform.h:309-317)
 *   homography     : 1074-1366  (matrix 1152-1164, scale 1186-1194, eps 1196-1205,
 *                                create_remap 1207-1223, SD 1319-1366,
 *                                invert_and_compose c_image_transform.h:372-377)
 *   semi-quadratic : 1370-1612  (scale 1498-1504, eps 1506-1529, SD 1583-1612)
 *   quadratic      : 1616-1868  (scale 1755-1765, eps 1767-1781, SD 1834-1868)
 *   factory        : image_transform.cc:32-60 (EUCLIDEAN = euclidean + fix_scale)
 */
#include "sst_oracle.h"
#include <cmath>
#include <cstring>
#include <algorithm>

static inline double sq(double x) { return x * x; }

extern "C" int orc_model_nparams(const orc_model * m)
{
  switch ( m->type ) {
  case ORC_MOTION_TRANSLATION: return 2;
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN:
    return (m->fix_translation ? 0 : 2) + (m->fix_rotation ? 0 : 1) + (m->fix_scale ? 0 : 1);
  case ORC_MOTION_AFFINE: return 6;
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION: return 8;
  case ORC_MOTION_SEMI_QUADRATIC: return 8;
  case ORC_MOTION_QUADRATIC: return 12;
  }
  return 0;
}

static inline bool is_euclid(const orc_model * m)
{
  return m->type == ORC_MOTION_EUCLIDEAN || m->type == ORC_MOTION_SCALED_EUCLIDEAN;
}

static inline bool is_homog(const orc_model * m)
{
  return m->type == ORC_MOTION_HOMOGRAPHY || m->type == ORC_MOTION_EPIPOLAR_DEROTATION;
}

extern "C" void orc_model_identity(const orc_model * m, double * s)
{
  memset(s, 0, 16 * sizeof(double));
  switch ( m->type ) {
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN:
    s[3] = 1;  // scale
    break;
  case ORC_MOTION_AFFINE:
    s[0] = 1, s[4] = 1;
    break;
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION:
    s[0] = 1, s[4] = 1;
    break;
  case ORC_MOTION_SEMI_QUADRATIC:   // cv::Matx24f::eye()
    s[0] = 1, s[5] = 1;
    break;
  case ORC_MOTION_QUADRATIC:        // cv::Matx26f::eye()
    s[0] = 1, s[7] = 1;
    break;
  }
}

/* c_euclidean_image_transform::update_parameters / set_parameters
 * (c_image_transform.cc:331-383) */
extern "C" void orc_model_get_params(const orc_model * m, const double * s, double * p)
{
  if( is_euclid(m) ) {
    int i = 0;
    if( !m->fix_translation ) p[i++] = s[0], p[i++] = s[1];
    if( !m->fix_rotation ) p[i++] = s[2];
    if( !m->fix_scale ) p[i++] = s[3];
  }
  else {
    memcpy(p, s, orc_model_nparams(m) * sizeof(double));
  }
}

extern "C" void orc_model_set_params(const orc_model * m, double * s, const double * p)
{
  if( is_euclid(m) ) {
    int i = 0;
    if( !m->fix_translation ) s[0] = p[i++], s[1] = p[i++];
    if( !m->fix_rotation ) s[2] = p[i++];
    if( !m->fix_scale ) s[3] = p[i++];
  }
  else {
    memcpy(s, p, orc_model_nparams(m) * sizeof(double));
  }
}

extern "C" void orc_model_warp(const orc_model * m, const double * a, double x, double y, double * X, double * Y)
{
  switch ( m->type ) {
  case ORC_MOTION_TRANSLATION:
    *X = x + a[0], *Y = y + a[1];
    break;
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN: {
    const double sa = std::sin(a[2]), ca = std::cos(a[2]), sc = a[3];
    const double xx = x - a[4], yy = y - a[5];
    *X = sc * (ca * xx - sa * yy) + a[0];
    *Y = sc * (sa * xx + ca * yy) + a[1];
    break;
  }
  case ORC_MOTION_AFFINE:
    *X = a[0] * x + a[1] * y + a[2];
    *Y = a[3] * x + a[4] * y + a[5];
    break;
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION: {
    const double w = a[6] * x + a[7] * y + 1.0;
    *X = (a[0] * x + a[1] * y + a[2]) / w;
    *Y = (a[3] * x + a[4] * y + a[5]) / w;
    break;
  }
  case ORC_MOTION_SEMI_QUADRATIC:
    *X = a[0] * x + a[1] * y + a[2] + a[3] * x * y;
    *Y = a[4] * x + a[5] * y + a[6] + a[7] * x * y;
    break;
  case ORC_MOTION_QUADRATIC:
    *X = a[0] * x + a[1] * y + a[2] + a[3] * x * y + a[4] * x * x + a[5] * y * y;
    *Y = a[6] * x + a[7] * y + a[8] + a[9] * x * y + a[10] * x * x + a[11] * y * y;
    break;
  default:
    *X = x, *Y = y;
  }
}

extern "C" void orc_model_sd(const orc_model * m, const double * a, double x, double y, double gx, double gy, double * J)
{
  switch ( m->type ) {
  case ORC_MOTION_TRANSLATION:
    J[0] = gx, J[1] = gy;
    break;
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN: {
    const double sa = std::sin(a[2]), ca = std::cos(a[2]), sc = a[3];
    const double xx = x - a[4], yy = y - a[5];
    int i = 0;
    if( !m->fix_translation ) J[i++] = gx, J[i++] = gy;
    if( !m->fix_rotation ) J[i++] = sc * (-gx * (sa * xx + ca * yy) + gy * (ca * xx - sa * yy));
    if( !m->fix_scale ) J[i++] = gx * (ca * xx - sa * yy) + gy * (sa * xx + ca * yy);
    break;
  }
  case ORC_MOTION_AFFINE:
    J[0] = gx * x, J[1] = gx * y, J[2] = gx;
    J[3] = gy * x, J[4] = gy * y, J[5] = gy;
    break;
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION: {
    const double den = 1.0 / (x * a[6] + y * a[7] + 1.0);
    const double hatX = -(x * a[0] + y * a[1] + a[2]) * den;
    const double hatY = -(x * a[3] + y * a[4] + a[5]) * den;
    const double ggx = gx * den, ggy = gy * den;
    const double gg = hatX * ggx + hatY * ggy;
    J[0] = ggx * x, J[1] = ggx * y, J[2] = ggx;
    J[3] = ggy * x, J[4] = ggy * y, J[5] = ggy;
    J[6] = gg * x, J[7] = gg * y;
    break;
  }
  case ORC_MOTION_SEMI_QUADRATIC:
    J[0] = gx * x, J[1] = gx * y, J[2] = gx, J[3] = gx * x * y;
    J[4] = gy * x, J[5] = gy * y, J[6] = gy, J[7] = gy * x * y;
    break;
  case ORC_MOTION_QUADRATIC:
    J[0] = gx * x, J[1] = gx * y, J[2] = gx, J[3] = gx * x * y, J[4] = gx * x * x, J[5] = gx * y * y;
    J[6] = gy * x, J[7] = gy * y, J[8] = gy, J[9] = gy * x * y, J[10] = gy * x * x, J[11] = gy * y * y;
    break;
  }
}

extern "C" double orc_model_eps(const orc_model * m, const double * s, const double * dp, int W, int H)
{
  switch ( m->type ) {
  case ORC_MOTION_TRANSLATION:
    return std::sqrt(dp[0] * dp[0] + dp[1] * dp[1]);
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN: {
    /* get_parameters(dp,...) returns the stored absolute value for a fixed
     * component (c_image_transform.cc:407-421), so a fixed scale contributes
     * max(W,H) * scale to eps. */
    int i = 0;
    double dTx, dTy, da, ds;
    if( m->fix_translation ) dTx = s[0], dTy = s[1];
    else dTx = dp[i++], dTy = dp[i++];
    da = m->fix_rotation ? s[2] : dp[i++];
    ds = m->fix_scale ? s[3] : dp[i++];
    const double sa = std::sin(da);
    return std::sqrt(sq(dTx) + sq(dTy) + sq(W * sa) + sq(H * sa) + sq(std::max(W, H) * ds));
  }
  case ORC_MOTION_AFFINE:
    return std::sqrt(sq(W * dp[0]) + sq(H * dp[1]) + sq(dp[2]) + sq(W * dp[3]) + sq(H * dp[4]) + sq(dp[5]));
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION:
    return std::sqrt(sq(dp[2]) + sq(dp[5]) + sq(W * dp[0]) + sq(H * dp[1]) + sq(W * dp[3]) + sq(H * dp[4]));
  case ORC_MOTION_SEMI_QUADRATIC: {
    const double WH = (double) W * H;
    return std::sqrt(sq(dp[2]) + sq(dp[6]) + sq(W * dp[0]) + sq(H * dp[1]) + sq(W * dp[4]) + sq(H * dp[5]) +
        sq(WH * dp[3]) + sq(WH * dp[7]));
  }
  case ORC_MOTION_QUADRATIC: {
    const double WH = (double) W * H, WW = (double) W * W, HH = (double) H * H;
    return std::sqrt(sq(dp[2]) + sq(dp[8]) + sq(W * dp[0]) + sq(H * dp[1]) + sq(W * dp[6]) + sq(H * dp[7]) +
        sq(WH * dp[3]) + sq(WH * dp[9]) + sq(WW * dp[4]) + sq(WW * dp[10]) + sq(HH * dp[5]) + sq(HH * dp[11]));
  }
  }
  return 0;
}

extern "C" void orc_model_scale(const orc_model * m, double * a, double f)
{
  switch ( m->type ) {
  case ORC_MOTION_TRANSLATION:
    a[0] *= f, a[1] *= f;
    break;
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN:
    a[0] *= f, a[1] *= f, a[4] *= f, a[5] *= f;
    break;
  case ORC_MOTION_AFFINE:
    a[2] *= f, a[5] *= f;
    break;
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION:
    a[2] *= f, a[5] *= f, a[6] /= f, a[7] /= f;
    break;
  case ORC_MOTION_SEMI_QUADRATIC:
    a[2] *= f, a[3] /= f, a[6] *= f, a[7] /= f;
    break;
  case ORC_MOTION_QUADRATIC:
    a[2] *= f, a[3] /= f, a[4] /= f, a[5] /= f;
    a[8] *= f, a[9] /= f, a[10] /= f, a[11] /= f;
    break;
  }
}

extern "C" int orc_model_invertible(const orc_model * m)
{
  return m->type != ORC_MOTION_SEMI_QUADRATIC && m->type != ORC_MOTION_QUADRATIC;
}

/* cv::invertAffineTransform semantics: a 2x3 -> 2x3 */
static void invert_affine(const double a[6], double r[6])
{
  double D = a[0] * a[4] - a[1] * a[3];
  D = D != 0 ? 1.0 / D : 0.0;
  const double A11 = a[4] * D, A22 = a[0] * D, A12 = -a[1] * D, A21 = -a[3] * D;
  r[0] = A11, r[1] = A12, r[2] = -A11 * a[2] - A12 * a[5];
  r[3] = A21, r[4] = A22, r[5] = -A21 * a[2] - A22 * a[5];
}

static bool inv3(const double a[9], double r[9])
{
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
  const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  if( det == 0 ) {
    memset(r, 0, 9 * sizeof(double));
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

static void euclid_matrix(double tX, double tY, double ang, double scl, double cX, double cY, double M[6])
{
  const double sa = std::sin(ang), ca = std::cos(ang);
  M[0] = scl * ca, M[1] = -scl * sa, M[2] = tX - scl * ca * cX + scl * sa * cY;
  M[3] = scl * sa, M[4] = scl * ca, M[5] = tY - scl * sa * cX - scl * ca * cY;
}

extern "C" int orc_model_invert_and_compose(const orc_model * m, const double * s, const double * dp, double * out)
{
  memcpy(out, s, 16 * sizeof(double));
  switch ( m->type ) {
  case ORC_MOTION_TRANSLATION:
    out[0] = s[0] - dp[0], out[1] = s[1] - dp[1];
    return 1;
  case ORC_MOTION_EUCLIDEAN:
  case ORC_MOTION_SCALED_EUCLIDEAN: {
    const double Tx = s[0], Ty = s[1], angle = s[2], scale = s[3], Cx = s[4], Cy = s[5];
    int i = 0;
    double dTx, dTy, dA, dS;
    if( m->fix_translation ) dTx = 0, dTy = 0;
    else dTx = dp[i++], dTy = dp[i++];
    if( m->fix_rotation ) dA = 0;
    else dA = dp[i++];
    if( m->fix_scale ) dS = 0;
    else dS = dp[i++];
    const double scale_dp = m->fix_scale ? 1.0 : 1.0 + dS;
    double Mp[6], Mdp[6], Mi[6];
    euclid_matrix(Tx, Ty, angle, scale, Cx, Cy, Mp);
    euclid_matrix(dTx, dTy, dA, scale_dp, Cx, Cy, Mdp);
    invert_affine(Mdp, Mi);
    // M_res = Mp * Mi (3x3 with last row 0 0 1)
    double R[6];
    R[0] = Mp[0] * Mi[0] + Mp[1] * Mi[3];
    R[1] = Mp[0] * Mi[1] + Mp[1] * Mi[4];
    R[2] = Mp[0] * Mi[2] + Mp[1] * Mi[5] + Mp[2];
    R[3] = Mp[3] * Mi[0] + Mp[4] * Mi[3];
    R[4] = Mp[3] * Mi[1] + Mp[4] * Mi[4];
    R[5] = Mp[3] * Mi[2] + Mp[4] * Mi[5] + Mp[5];
    const double rs = m->fix_scale ? scale : std::sqrt(R[0] * R[0] + R[3] * R[3]);
    const double ra = m->fix_rotation ? angle : std::atan2(R[3], R[0]);
    const double rc = std::cos(ra), rsn = std::sin(ra);
    out[0] = m->fix_translation ? Tx : R[2] + rs * rc * Cx - rs * rsn * Cy;
    out[1] = m->fix_translation ? Ty : R[5] + rs * rsn * Cx + rs * rc * Cy;
    out[2] = ra;
    out[3] = rs;
    return 1;
  }
  case ORC_MOTION_AFFINE: {
    double a[6], b[6];
    invert_affine(s, a);
    for( int k = 0; k < 6; ++k ) a[k] += dp[k];
    invert_affine(a, b);
    memcpy(out, b, 6 * sizeof(double));
    return 1;
  }
  case ORC_MOTION_HOMOGRAPHY:
  case ORC_MOTION_EPIPOLAR_DEROTATION: {
    const double M[9] = { s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], 1.0 };
    double Mi[9], R[9];
    inv3(M, Mi);
    const double dM[9] = { dp[0], dp[1], dp[2], dp[3], dp[4], dp[5], dp[6], dp[7], 0.0 };
    for( int k = 0; k < 9; ++k ) Mi[k] += dM[k];
    inv3(Mi, R);
    const double n = 1.0 / R[8];
    for( int k = 0; k < 8; ++k ) out[k] = R[k] * n;
    return 1;
  }
  }
  return 0;
}
