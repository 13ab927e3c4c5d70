/*
 * sst_oracle.h -- FP64 CPU restatement of SerStacker's frame registration +
 * stacking hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle of the parity tests of the
 * CUDA path and the timed CPU baseline; the product never links, loads or
 * calls it. It restates the algorithms of the reference files
 *   core/proc/image_registration/ecc2.cc
 *   core/proc/image_registration/c_image_transform.cc
 *   core/proc/image_registration/c_frame_registration.cc
 *   core/average/c_frame_accumulation.cc
 *   core/io/debayer.cc
 *   core/proc/sharpness_measure/c_local_variance_sharpness_measure.cc
 *   core/proc/inpaint/average_pyramid_inpaint.cc, core/proc/downstrike.cc
 * in double precision. OpenCV primitives the reference calls (sepFilter2D,
 * pyrDown, remap, meanStdDev, erode, resize NEAREST, Cholesky solve) are
 * re-implemented from their documented semantics; bilinear sampling is exact
 * (no 1/32 px grid) unless ORC_SNAP32 is requested.
 *
 * Parity status: unpinned by the reference (the reference ships no tests and
 * no golden data, and cannot be compiled here: OpenCV/TBB/libconfig absent).
 * The oracle is pinned by known-answer tests instead (tests/test_oracle.py).
 */
#pragma once
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* IMAGE_MOTION_TYPE values (image_transform.h:15-26) */
enum {
  ORC_MOTION_TRANSLATION = 0,
  ORC_MOTION_EUCLIDEAN = 1,
  ORC_MOTION_SCALED_EUCLIDEAN = 2,
  ORC_MOTION_AFFINE = 3,
  ORC_MOTION_HOMOGRAPHY = 4,
  ORC_MOTION_SEMI_QUADRATIC = 5,
  ORC_MOTION_QUADRATIC = 6,
  ORC_MOTION_EPIPOLAR_DEROTATION = 7,
};

/* ECC_ALIGN_METHOD values (ecc2.h:57-62) */
enum {
  ORC_ECC_FORWARD_ADDITIVE = 0,
  ORC_ECC_INVERSE_COMPOSITIONAL = 1,
  ORC_ECC_LM = 2,
  ORC_ECC_INVERSE_COMPOSITIONAL_LM = 3,
};

/* cv::BorderTypes values used on the path */
enum {
  ORC_BORDER_CONSTANT = 0,
  ORC_BORDER_REPLICATE = 1,
  ORC_BORDER_REFLECT = 2,
  ORC_BORDER_REFLECT101 = 4,
};

/* Motion model. The transform state is a vector of up to 16 doubles:
 *   translation : tx ty
 *   euclidean   : Tx Ty angle scale Cx Cy  (adjustable subset per fix flags)
 *   affine      : a00 a01 a02 a10 a11 a12
 *   homography  : a00 a01 a02 a10 a11 a12 a20 a21   (a22 = 1)
 *   semi-quad.  : a00 a01 a02 a03 a10 a11 a12 a13
 *   quadratic   : a00..a05 a10..a15
 * The ECC parameter vector p (c_image_transform::parameters()) equals the
 * state for every model but euclidean, where it is the adjustable subset. */
typedef struct orc_model {
  int type;
  int fix_translation, fix_rotation, fix_scale;
} orc_model;

int  orc_model_nparams(const orc_model * m);
void orc_model_identity(const orc_model * m, double * state);
void orc_model_get_params(const orc_model * m, const double * state, double * p);
void orc_model_set_params(const orc_model * m, double * state, const double * p);
void orc_model_warp(const orc_model * m, const double * state, double x, double y, double * X, double * Y);
void orc_model_sd(const orc_model * m, const double * state, double x, double y, double gx, double gy, double * J);
double orc_model_eps(const orc_model * m, const double * state, const double * dp, int w, int h);
void orc_model_scale(const orc_model * m, double * state, double factor);
int  orc_model_invert_and_compose(const orc_model * m, const double * state, const double * dp, double * out_state);
int  orc_model_invertible(const orc_model * m);

/* primitives */
int  orc_gaussian_kernel(double sigma, double * k /* >= 2*int(3 sigma)+1 */);
void orc_smooth(const double * src, int w, int h, double sigma, double * dst);
void orc_pyrdown(const double * src, int w, int h, double * dst, int dw, int dh);
void orc_resize_nearest_u8(const uint8_t * src, int w, int h, uint8_t * dst, int dw, int dh);
void orc_differentiate(const double * src, int w, int h, const uint8_t * valid, double * gx, double * gy);
double orc_sample_bilinear(const double * src, int w, int h, double sx, double sy, int border, double bval);
double orc_mask_coverage(const uint8_t * mask, int w, int h, double sx, double sy);
void orc_erode5(const uint8_t * src, int w, int h, int border_is_max, uint8_t * dst);
void orc_remap_model(const orc_model * m, const double * state, const double * src, int sw, int sh,
    int dw, int dh, int border, double bval, double * dst);

/* single-level ECC (c_ecc_align::align) */
typedef struct orc_align_opts {
  int method;
  int max_iterations;
  double max_eps;
  double update_step_scale;
  int ic_jacobian_at_identity;    /* 1: IC steepest-descent images at the identity warp */
} orc_align_opts;

typedef struct orc_level {
  int w, h;
  const double * ref;   const uint8_t * ref_mask;   /* mask may be NULL */
  const double * cur;   int cw, ch;  const uint8_t * cur_mask;
} orc_level;

/* returns the reference's align() bool; *iters, *eps filled. */
int orc_ecc_align(const orc_model * m, double * state, const orc_level * lvl, const orc_align_opts * o,
    int * iters, double * eps);

/* c_ecch: Gaussian pre-smooth, pyramid, coarse-to-fine align.
 * ref / cur are f64 images already converted (ecc_convert_input_image). */
typedef struct orc_ecch_opts {
  double epsx;
  double reference_smooth_sigma, input_smooth_sigma;
  double update_step_scale;
  int method, max_iterations, minimum_image_size, maxlevel;
  int ic_jacobian_at_identity;
} orc_ecch_opts;

int  orc_ecch_num_levels(int w, int h, const orc_ecch_opts * o);
int  orc_ecch_align(const orc_model * m, double * state, const orc_ecch_opts * o,
    const double * ref, const uint8_t * ref_mask, int w, int h,
    const double * cur, const uint8_t * cur_mask, int cw, int ch,
    int * iters, double * eps);

double orc_correlation(const double * cur, const uint8_t * cur_mask, int cw, int ch,
    const double * ref, const uint8_t * ref_mask, int w, int h, const orc_model * m, const double * state);

/* base_remap of a frame for stacking: LINEAR + border, mask LINEAR/CONSTANT >=255 + 5x5 erode */
void orc_stack_remap(const orc_model * m, const double * state, const double * src, int sw, int sh,
    int dw, int dh, int border, double * dst, uint8_t * dst_mask);

/* accumulators */
void orc_weighted_average_add(double * acc, double * accw, int w, int h, const double * src, const double * weights);
void orc_running_mean_add_f32(float * acc, float * accw, int w, int h, const float * src, const float * weights);
void orc_extract_bayer_planes_u16(const uint16_t * src, int w, int h, uint16_t * dst);
void orc_average_bayer_planes_u16(const uint16_t * src, int w, int h, uint16_t * dst);
void orc_bayer_pattern_mask(int colorid, int w, int h, uint8_t * dst);
void orc_warp_grid(const orc_model * m, const double * state, int w, int h, double * mapx, double * mapy);
void orc_bayer_accumulate(const double * src, int w, int h, const double * mapx, const double * mapy,
    const uint8_t * pattern, const double * weights, double * acc, double * cntr);

/* ------------------------------------------------------------- c_eccflow */

/* c_eccflow_options (ecc2.h:515-527); downscale: 0 recursive INTER_AREA
 * resize, 1 full INTER_AREA resize from level 0, 2 pyrDown */
typedef struct orc_flow_opts {
  double update_multiplier, scale_factor, noise_level;
  int max_iterations, support_scale, min_image_size, max_pyramid_level, downscale;
} orc_flow_opts;

/* cv::resize INTER_AREA (pixel-area relation) and INTER_CUBIC (a = -0.75) */
void orc_resize_area(const double * src, int sw, int sh, double * dst, int dw, int dh);
void orc_resize_cubic(const double * src, int sw, int sh, double * dst, int dw, int dh);
/* pyramid level sizes of c_eccflow::set_reference_image; returns the count */
int orc_eccflow_levels(int w, int h, const orc_flow_opts * o, int * ws, int * hs, int max_levels);
/* c_eccflow::compute_uv(current, rmap) after set_reference_image(reference):
 * flow (h x w x 2, interleaved u, v); init_flow may be NULL (zero start) */
int orc_eccflow(const orc_flow_opts * o, const double * ref, const double * cur, int w, int h,
    const double * init_flow, double * flow);
/* the same with reference / current masks (u8, 0 = invalid; either may be NULL) */
int orc_eccflow_masked(const orc_flow_opts * o, const double * ref, const uint8_t * ref_mask,
    const double * cur, const uint8_t * cur_mask, int w, int h, const double * init_flow, double * flow);

/* focus-stacking weights of a frame warped to the dw x dh grid:
 * W = (6 lap^2 + |grad|^2)^2 blurred by a Gaussian of sigma 3 */
void orc_focus_weights(const orc_model * m, const double * state, const double * src, int sw, int sh,
    int dw, int dh, double * out);

/* The warp residual objective of the adjoint: for frame f,
 *   r(x) = I_f(W(x; p_f) + u_f(x)) - T(x)   (bilinear, BORDER_REPLICATE)
 *   L_f = 1/2 sum_x r(x)^2
 * with its exact gradients: dL/dp (M) through the derivative of the
 * bilinear interpolant, dL/dT(x) = -r(x), and dL/du(x) = r(x) grad I.
 * flow may be NULL; grad outputs may be NULL. Returns L_f. */
double orc_warp_residual(const orc_model * m, const double * state, const double * img, const double * tmpl,
    const double * flow, int w, int h, double * grad_p, double * grad_t, double * grad_u);

/* sharpness weight of a frame: mean of the squared 5-point Laplacian over the
 * interior of a level image */
double orc_laplacian_energy(const double * img, int w, int h);

/* cv::resize INTER_LINEAR geometry (equal sizes copy) */
void orc_resize_linear(const double * src, int sw, int sh, double * dst, int dw, int dh);

/* size of the map compute_local_variance_map returns for a w x h image;
 * returns 1 when the map is upscaled to the image's size */
int orc_local_variance_size(int w, int h, int dscale, int uscale, int * mw, int * mh);

/* compute_local_variance_map: morphological gradient G (square of radius
 * max(1, kradius), BORDER_REPLICATE) of the image pyrDown'ed dscale times;
 * map = ds^3 G^3, INTER_AREA-reduced uscale halvings, plus 0.05 Q with
 * Q = ds^3 sum G^4 / sum G, INTER_LINEAR-upscaled to the image's size when the
 * gradient's size differs from it. Returns 0 (no map, q = 0) when sum G is
 * not positive, else 1 with the map (*mw x *mh, at most w x h) and q. */
/* average_pyramid_inpaint of a single-channel image with a u8 mask
 * (non-zero = valid): holes filled from 3 x 3 means over a downstrike /
 * upject pyramid of at most max_levels levels; the output mask is 255 where
 * a value was found */
void orc_average_pyramid_inpaint(const double * src, const uint8_t * mask, int w, int h, int max_levels,
    double * dst, uint8_t * dstmask);

int orc_local_variance_map(const double * img, int w, int h, int kradius, int dscale, int uscale,
    double depth_scale, double * map, int * mw, int * mh, double * q);

/* whole pipeline for the CPU baseline: register (ecch passes) + rho gate +
 * final warp + weighted stack of n frames. */
typedef struct orc_pipeline_opts {
  orc_ecch_opts ecch;
  int num_passes;
  int pass_motion[3];
  double min_rho;
  int border_mode;
  int use_laplacian_weights;
} orc_pipeline_opts;

int orc_register_and_stack(const orc_pipeline_opts * o,
    const double * ref, int w, int h,
    const uint16_t * frames, int n, double frame_scale,
    double * out_states /* n x 16 */, int * out_status, double * out_rho,
    double * acc, double * accw);

/* c_ecch::align + compute_correlation on w x h images (see sst_oracle.cc) */
int orc_ecch_align_pyramids(const orc_model * m, double * state, const orc_ecch_opts * o,
    const double * ref, const uint8_t * ref_mask, const double * cur, int w, int h, int * iters, double * eps,
    double * rho);

/* c_ecc_registration_options (c_frame_registration.h:47-63) with the
 * motion type of c_image_registration_options (:119-137) */
typedef struct orc_registration_opts {
  int motion_type;
  int method;
  double scale, eps, min_rho, input_smooth_sigma, reference_smooth_sigma, update_step_scale;
  int max_iterations, ecch_max_level, ecch_minimum_image_size;
  int normalization_scale;
  double normalization_noise;
  int estimate_translation_first;
} orc_registration_opts;

void orc_pyrdown_border(const double * src, int w, int h, double * dst, int dw, int dh, int border);
void orc_pyrup(const double * src, int sw, int sh, double * dst, int dw, int dh);
void orc_mask_pyrdown_ge250(const uint8_t * src, int w, int h, uint8_t * dst, int dw, int dh);
void orc_scale_image_size(int w, int h, double scale, int * dw, int * dh);
void orc_scale_image(const double * src, const uint8_t * mask, int w, int h, double scale, double * dst,
    uint8_t * dst_mask);
void orc_ecc_normalize(const double * src, const uint8_t * mask, int w, int h, int lvl, double * dst);
int orc_register_frame(const orc_registration_opts * o, const double * ref, const uint8_t * ref_mask,
    int w, int h, const double * cur, double * state, double * rho, int * iters);

/* lpg() (core/proc/lpg.cc:223-291) of a mono image already scaled to
 * [0, 1] (integer input / maxval); map w x h, metric = mean(map) (masked) */
int orc_lpg(const double * img, const uint8_t * mask, int w, int h, double k, double p, int dscale, int uscale,
    double * map, double * metric);

/* debayer NN2 (core/io/debayer.cc:828-1161): BGR interleaved output */
int orc_debayer_nn2_u16(const uint16_t * src, int w, int h, int colorid, uint16_t * dst);
int orc_debayer_nn2_f32(const float * src, int w, int h, int colorid, float * dst);

/* other accumulators (sst_oracle_accum.cc) */
int orc_optimal_dft_size(int n);
void orc_linear_inpaint(double * image, const uint8_t * mask, int w, int h, int cn);
int orc_filter_bad_pixels_u16(const uint16_t * src, int w, int h, int colorid, double threshold, uint16_t * dst);
int orc_filter_bad_pixels_f32(const float * src, int w, int h, int colorid, double threshold, float * dst);
int orc_fft_average(const double * frames, int n, int w, int h, int cn, double * avg);
int orc_focus_stack(const double * frames, const uint8_t * masks, int n, int w, int h, int cn, int policy,
    int inpaint, int avgchannel, const double * G, int gk, double * avg);
int orc_canvas_average(const double * frames, int n, int w, int h, int cn, int wkind, const void * weights,
    const int * boxes, const double * rmaps, int * canvas, double * acc, double * W, int * status, int * last);

void orc_set_num_threads(int n);
int  orc_get_num_threads(void);

#ifdef __cplusplus
}
#endif
