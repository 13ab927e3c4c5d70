/*
 * serstacker_gb300.h -- C ABI of the GB300 (sm_103a) frame registration +
 * stacking library (libsst_gb300.so).
 *
 * This is the drop-in boundary for SerStacker's registration and stacking hot
 * path. Every entry point names the reference interface it replaces
 * (paths relative to the SerStacker source tree). Plain C: pointers, sizes
 * and ints only; every call returns an int status (SST_OK = 0, negative on
 * error) and sst_last_error() describes the most recent failure of the
 * calling thread. No C++ exception crosses this boundary.
 *
 * Images are row-major. `depth` uses OpenCV depth codes (CV_8U = 0,
 * CV_16U = 2, CV_32F = 5). Buffers are host or device memory as stated by
 * each call's `on_device` flag; host buffers may be pageable or pinned
 * (pinned host memory is copied asynchronously).
 */
#ifndef SERSTACKER_GB300_H
#define SERSTACKER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define SST_OK                  0
#define SST_ERR_INVALID_ARG    -1
#define SST_ERR_CUDA           -2
#define SST_ERR_UNSUPPORTED    -3
#define SST_ERR_STATE          -4
#define SST_ERR_NOMEM          -5
#define SST_ERR_TIMEOUT        -6
#define SST_ERR_IO             -7

/* per-frame registration status */
#define SST_FRAME_OK              0
#define SST_FRAME_SINGULAR        1   /* Cholesky of the Gauss-Newton matrix failed (ecc2.cc:1331-1335) */
#define SST_FRAME_EMPTY_MASK      2   /* no valid pixel after warping */
#define SST_FRAME_LOW_RHO         3   /* rho < min_rho (c_frame_registration.cc:861-868) */
#define SST_FRAME_NAN             4   /* non-finite parameters */
#define SST_FRAME_NOT_INVERTIBLE  5   /* IC / IC-LM with a non-invertible model (ecc2.cc:1702-1705) */

/* IMAGE_MOTION_TYPE (core/proc/image_registration/image_transform.h:15-26) */
#define SST_MOTION_TRANSLATION          0
#define SST_MOTION_EUCLIDEAN            1   /* euclidean with fixed scale (image_transform.cc:35-39) */
#define SST_MOTION_SCALED_EUCLIDEAN     2
#define SST_MOTION_AFFINE               3
#define SST_MOTION_HOMOGRAPHY           4
#define SST_MOTION_SEMI_QUADRATIC       5
#define SST_MOTION_QUADRATIC            6
#define SST_MOTION_EPIPOLAR_DEROTATION  7

/* ECC_ALIGN_METHOD (core/proc/image_registration/ecc2.h:57-62) */
#define SST_ECC_FORWARD_ADDITIVE          0
#define SST_ECC_INVERSE_COMPOSITIONAL     1
#define SST_ECC_LM                        2
#define SST_ECC_INVERSE_COMPOSITIONAL_LM  3

/* cv::BorderTypes subset (ECC_BORDER_MODE, ecc2.h:44-54) */
#define SST_BORDER_CONSTANT    0
#define SST_BORDER_REPLICATE   1
#define SST_BORDER_REFLECT     2
#define SST_BORDER_REFLECT101  4

/* pixel depths (OpenCV codes) */
#define SST_DEPTH_U8   0
#define SST_DEPTH_U16  2
#define SST_DEPTH_F32  5
/* reported by SER files only (no compute entry point takes them) */
#define SST_DEPTH_S32  4
#define SST_DEPTH_F64  6

/* COLORID Bayer patterns (core/io/debayer.h:19-34) */
#define SST_COLORID_BAYER_RGGB  8
#define SST_COLORID_BAYER_GRBG  9
#define SST_COLORID_BAYER_GBRG 10
#define SST_COLORID_BAYER_BGGR 11

/* Motion model: the transform object of create_image_transform()
 * (core/proc/image_registration/image_transform.cc:32-60). The fix flags
 * apply to the euclidean models; EUCLIDEAN forces fix_scale = 1. The
 * euclidean centre is (0,0), as in the reference default
 * (c_image_transform.cc:275-286). */
typedef struct sst_motion_model {
  int32_t type;
  int32_t fix_translation;
  int32_t fix_rotation;
  int32_t fix_scale;
} sst_motion_model;

/* c_ecch_options (core/proc/image_registration/ecc2.h:158-172) with the
 * registration-level settings of c_ecc_registration_options
 * (core/proc/image_registration/c_frame_registration.h:47-63) that the
 * batched registration uses. */
typedef struct sst_ecch_options {
  double epsx;                     /* stop when eps(dp) < epsx at level 0; x2 per coarser level */
  double reference_smooth_sigma;   /* Gaussian pre-smooth of the reference (sepFilter2D, REPLICATE) */
  double input_smooth_sigma;       /* Gaussian pre-smooth of each frame */
  double update_step_scale;
  int32_t method;                  /* SST_ECC_* */
  int32_t interpolation;           /* only ECC_INTER_LINEAR (1) is accepted */
  int32_t max_iterations;
  int32_t minimum_image_size;
  int32_t maxlevel;                /* c_ecch maxlevel: number of pyramid levels limit */
  double min_rho;                  /* correlation gate after alignment; <= 0 reports rho without gating */
  int32_t ic_jacobian_at_identity; /* must be 1: IC steepest-descent images at the identity warp */
  int32_t reserved;
} sst_ecch_options;

/* The reference defaults of c_ecch_options (ecc2.h:158-172). */
void sst_ecch_options_default(sst_ecch_options * opts);

/* ---------------------------------------------------------------- library */

/* Human-readable description of the calling thread's last error. */
const char * sst_last_error(void);

/* Library version string. */
const char * sst_version(void);

/* Number of visible CUDA devices (0 when no driver / no GPU). */
int sst_device_count(void);

/* --------------------------------------------------- batched c_ecch engine */

typedef struct sst_ecch sst_ecch;

/* c_ecch::c_ecch(const c_ecch_options &) (ecc2.h:198-203). Allocates nothing
 * on the device until set_reference_image. */
int sst_ecch_create(sst_ecch ** out, const sst_ecch_options * opts);
int sst_ecch_destroy(sst_ecch * h);

/* c_ecch::set_reference_image(reference_image, reference_mask)
 * (ecc2.cc:984-1057): converts to f32 (ecc_convert_input_image,
 * ecc2.cc:345-382; `scale` multiplies the converted values), smooths with
 * reference_smooth_sigma, builds the pyramid (pyrDown, nearest mask resize)
 * and precomputes the inverse-compositional Gauss-Newton matrices per level.
 * mask may be NULL (u8, 0 = invalid). */
int sst_ecch_set_reference_image(sst_ecch * h, const void * image, int depth, int width, int height,
    size_t row_stride, double scale, const uint8_t * mask, size_t mask_stride, int on_device, void * stream);

/* Number of pyramid levels of the current reference (c_ecch::_pyramid.size()). */
int sst_ecch_num_levels(const sst_ecch * h);

/* Batched c_ecch::align(current_image, current_mask) (ecc2.cc:1123-1176)
 * for n frames, followed by compute_correlation (ecc2.cc:100-137) and the
 * min_rho gate of c_frame_registration::register_frame
 * (c_frame_registration.cc:852-868).
 *
 * frames : n images, frame k at frames + k * frame_stride (bytes)
 * passes : motion models run in sequence; pass k+1 starts from the result of
 *          pass k (e.g. AFFINE then HOMOGRAPHY). 1 <= num_passes <= 3.
 * params_inout : n x 12 floats. On input, when `use_initial_params` is
 *          non-zero, the initial parameter vector of the first pass at full
 *          resolution (c_image_transform::parameters() layout); otherwise
 *          the model's identity. On output, the final parameter vector of the
 *          last pass (first M entries).
 * status_out, iterations_out (summed over levels and passes), eps_out
 *          (level-0 eps of the last pass), rho_out: n entries each, may be NULL.
 * All frames of one call are registered together: one launch per
 * Gauss-Newton step covers every frame still iterating (per-frame
 * convergence masks), and the whole level x iteration schedule is replayed
 * as one CUDA graph. */
int sst_ecch_align_batch(sst_ecch * h, const void * frames, int depth, int n, int width, int height,
    size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int use_initial_params,
    float * params_inout, int32_t * status_out, int32_t * iterations_out, float * eps_out,
    float * rho_out, float * weight_out, void * stream);

/* The same registration, driven one frame at a time with one launch per
 * Gauss-Newton step and a host synchronisation after every step: the plain
 * one-frame-per-launch CUDA form the batched engine is measured against. */
int sst_ecch_align_plain(sst_ecch * h, const void * frames, int depth, int n, int width, int height,
    size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int use_initial_params,
    float * params_inout, int32_t * status_out, int32_t * iterations_out, float * eps_out,
    float * rho_out, float * weight_out, void * stream);

/* Timing of the last registration call, per motion pass and pyramid level
 * (the reference's c_image_registration_status::timings,
 * c_frame_registration.h:185-207, at level granularity): milliseconds
 * between CUDA events around the level's Gauss-Newton launches, the number
 * of frame-iterations executed, and their algorithmic bytes (16 B per pixel
 * and iteration for IC / IC-LM, 8 B for FA / LM). */
int sst_ecch_level_stats(sst_ecch * h, int pass, int level, float * ms, double * frame_iterations,
    double * algorithmic_bytes);

/* One level of the reference pyramid as the engine holds it: the converted,
 * pre-smoothed (reference_smooth_sigma) and pyrDown'ed reference, lw x lh
 * floats with packed rows (lw, lh: level 0 the image size, then
 * ((prev + 1) / 2) & ~1). Replaces c_ecch::reference_image() (ecc2.h:281) at
 * level 0 and c_ecc_align::reference_image() (ecc2.h:119) of the level's
 * aligner. out is host memory, or device memory when on_device != 0. */
int sst_ecch_reference_image(sst_ecch * h, int level, float * out, int on_device);

/* One level of frame `frame`'s pyramid from the last registration call (the
 * converted, pre-smoothed input_smooth_sigma image and its pyrDown levels).
 * Replaces c_ecch::current_image() (ecc2.h:284) / c_ecc_align::current_image()
 * (ecc2.h:122) for the frames of a batch. */
int sst_ecch_current_image(sst_ecch * h, int frame, int level, float * out, int on_device);

/* --------------------------------------------- weighted average accumulator */

typedef struct sst_weighted_average sst_weighted_average;

/* c_weigthed_average (core/average/c_frame_accumulation.h:39-63). The
 * accumulator holds compensated (Kahan-Babuska) FP32 sums of w*I and w;
 * compute() returns their ratio, which equals the reference's running mean
 * A += (I - A) w / W (c_frame_accumulation.cc:104-122) in exact arithmetic. */
int sst_weighted_average_create(sst_weighted_average ** out, int width, int height);
int sst_weighted_average_destroy(sst_weighted_average * h);

/* c_weigthed_average::clear (c_frame_accumulation.cc:164-169) */
int sst_weighted_average_clear(sst_weighted_average * h, void * stream);

/* c_weigthed_average::add(src, weights) (c_frame_accumulation.cc:182-221):
 * one already-warped frame; weights NULL, u8 mask (depth 0) or f32 (depth 5). */
int sst_weighted_average_add(sst_weighted_average * h, const void * src, int depth, size_t row_stride,
    double scale, const void * weights, int weights_depth, size_t weights_stride, int on_device, void * stream);

/* Batched remap + add: for each of n frames, warp the frame with its
 * parameters (c_frame_registration::base_remap, c_frame_registration.cc:
 * 1265-1340: LINEAR, `border`, mask LINEAR/CONSTANT >= 255 then 5x5 erode),
 * multiply the mask by the frame weight (c_image_stacking_pipeline.cc:
 * 1704-1714) and add (c_frame_accumulation.cc:182-221). Frames whose
 * status is not SST_FRAME_OK or whose weight is <= 0 are skipped. Each
 * output pixel is owned by one thread, which accumulates all n frames in
 * registers before one update of the accumulator. */
int sst_weighted_average_add_warped_batch(sst_weighted_average * h, const void * frames, int depth, int n,
    int src_width, int src_height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    const sst_motion_model * model, const float * params, const int32_t * status, const float * weights,
    int border, void * stream);

/* c_weigthed_average::compute(avg, mask) (c_frame_accumulation.cc:223-248):
 * avg (f32, width x height) and mask (u8, 255 where the weight sum > 0) are
 * host or device buffers per on_device; either may be NULL. */
int sst_weighted_average_compute(sst_weighted_average * h, float * avg, uint8_t * mask, int on_device, void * stream);

/* c_weigthed_average::get_acc_counters (c_frame_accumulation.cc:250-260): the weight sum. */
int sst_weighted_average_get_acc_counters(sst_weighted_average * h, float * accw, int on_device, void * stream);

/* c_weigthed_average::reinitialize(src, accw) (c_frame_accumulation.cc:171-180) */
int sst_weighted_average_reinitialize(sst_weighted_average * h, const float * avg, const float * accw,
    int on_device, void * stream);

/* c_frame_accumulation::accumulated_frames (c_frame_accumulation.h:29-32) */
int sst_weighted_average_accumulated_frames(const sst_weighted_average * h);

/* Checkpoint: the full compensated state (4 x width x height f32, sum,
 * compensation, weight sum, compensation) and the frame count. */
int sst_weighted_average_save_state(sst_weighted_average * h, float * state4, int32_t * frames, void * stream);
int sst_weighted_average_load_state(sst_weighted_average * h, const float * state4, int32_t frames, void * stream);

/* ------------------------------------------------ local-variance weights */

/* c_local_variance_map_options (c_local_variance_sharpness_measure.h:17-23):
 * kernel radius of the morphological gradient, pyrDown steps before it
 * (dscale) and INTER_AREA halvings of the map after it (uscale). The
 * channel option is the frame itself (mono frames; the Bayer pipeline uses
 * the 2x2-binned luminance). */
typedef struct sst_local_variance_options {
  int kradius;   /* 2; values below 1 act as 1; at most 16 */
  int dscale;    /* 1 */
  int uscale;    /* 3 */
} sst_local_variance_options;

void sst_local_variance_options_default(sst_local_variance_options * opts);

typedef struct sst_local_variance sst_local_variance;

/* c_local_variance_sharpness_measure (create_map, ..._measure.cc:252-262) */
int sst_local_variance_create(sst_local_variance ** out, const sst_local_variance_options * opts);
int sst_local_variance_destroy(sst_local_variance * h);

/* compute_local_variance_map (c_local_variance_sharpness_measure.cc:
 * 193-249) of n frames converted to FP32 by `scale`, with depthScale 20 (the
 * CV_32F frames of the stacking pipeline): `maps` receives n width x height
 * FP32 maps (may be NULL), `q` the n frame qualities Q (may be NULL). A
 * frame whose morphological gradient sums to zero has no map in the
 * reference: its q is 0 and its map is zero here. The map is always
 * returned at the frame's size: where the reference returns a reduced map
 * (dscale 0 with uscale > 0), it is upscaled with INTER_LINEAR here. */
int sst_local_variance_compute(sst_local_variance * h, const void * frames, int depth, int n, int width, int height,
    size_t row_stride, size_t frame_stride, double scale, int on_device, float * maps, double * q, void * stream);

/* c_frame_accumulation_options::sharpness_measure of the stacking pipeline:
 * the options of sst_stack_frames' weighting 3 (defaults until set). */
int sst_weighted_average_set_local_variance(sst_weighted_average * h, const sst_local_variance_options * opts);

/* ------------------------------------------------------------ LPG weights */

/* c_lpg_options (core/proc/sharpness_measure/c_lpg_sharpness_measure.h:
 * 22-28): k weighs the Laplacian against the gradient (alpha = k / (k + 1),
 * beta = 1 / (k + 1)), p the power of the map (0 and 1: none), dscale the
 * pyrDowns before the 5 x 5 operators, uscale the total pyrDowns of the map
 * before it is upscaled back. */
typedef struct sst_lpg_options {
  double k;
  double p;
  int32_t dscale;
  int32_t uscale;
} sst_lpg_options;

/* the reference defaults: k 2, p 2, dscale 2, uscale 6 */
void sst_lpg_options_default(sst_lpg_options * opts);

typedef struct sst_lpg sst_lpg;

/* c_lpg_sharpness_measure (c_lpg_sharpness_measure.h:44-80); opts NULL:
 * the defaults */
int sst_lpg_create(sst_lpg ** out, const sst_lpg_options * opts);
int sst_lpg_destroy(sst_lpg * h);

/* lpg() (core/proc/lpg.cc:223-291) of n mono frames: the map
 * alpha lap^2 + beta |grad|^2 + 1e-9 of the 5 x 5 noise-robust Laplacian and
 * extended Sobel gradient (lpg.cc:60-131) after dscale pyrDowns
 * (BORDER_REFLECT_101) of the frames converted to [0, 1] by their depth's
 * maximum and multiplied by 1 / (1 + dscale); then (uscale - dscale) further
 * pyrDowns, times (uscale - dscale), to the power p, and pyrUps back to the
 * frame size. `maps` (may be NULL) receives n packed width x height FP32 maps,
 * `metrics` (may be NULL) the n means of the maps over the nonzero pixels of
 * `masks` (NULL: all pixels). Frames, masks and maps are device pointers
 * when on_device, else host. SST_ERR_INVALID_ARG when the map would be
 * smaller than 5 x 5 after dscale. */
int sst_lpg_compute(sst_lpg * h, const void * frames, int depth, int n, int width, int height, size_t row_stride,
    size_t frame_stride, const uint8_t * masks, size_t mask_row_stride, size_t mask_frame_stride, int on_device,
    float * maps, double * metrics, void * stream);

/* ---------------------------------------------------- input calibration */

/* read_input_frame's dark / flat calibration of raw frames
 * (c_image_stacking_pipeline_base.cc:142-183), for n device frames into n
 * device FP32 frames: x = raw * scale (1 / 2^bpp), minus dark (when not
 * NULL), then x * 5 / flat (when not NULL): the reference passes the image
 * depth, CV_32F = 5, as cv::divide's scale argument. dark / flat are device
 * FP32 planes of the frame size. Strides in bytes (0: packed for dark, flat
 * and out). Enqueued on `stream`; the output feeds sst_stack_frames as
 * SST_DEPTH_F32 frames with scale 1. */
int sst_calibrate_frames(const void * frames, int depth, int n, int width, int height, size_t row_stride,
    size_t frame_stride, double scale, const float * dark, size_t dark_stride, const float * flat, size_t flat_stride,
    float * out, size_t out_row_stride, size_t out_frame_stride, void * stream);

/* nninterpolation (core/debayer.cc:828-1161), read_input_frame's
 * DEBAYER_NN2 (c_image_stacking_pipeline_base.cc:220-235): n device Bayer
 * frames (u8, u16 or f32; even width and height) into n device 3-channel BGR
 * frames of the same depth. colorid is the pattern: 8 RGGB, 9 GRBG, 10 GBRG,
 * 11 BGGR. At each pixel its own colour is copied; a green pixel takes red
 * and blue as the means of its two horizontal or vertical neighbours; a red
 * or blue pixel takes green as the mean of its 4 edge neighbours and the
 * other colour as the mean of its 4 diagonal neighbours (BORDER_REFLECT_101;
 * integer types round the means half up). Strides in bytes (dst rows hold
 * 3 * width elements). */
int sst_debayer_nn2(const void * frames, int depth, int n, int width, int height, size_t row_stride,
    size_t frame_stride, int colorid, void * dst, size_t dst_row_stride, size_t dst_frame_stride, void * stream);

/* read_input_frame's bad-pixel filter (c_image_stacking_pipeline_base.cc:
 * 200-216, input_options.filter_bad_pixels with bad_pixels_variation_threshold
 * k): Bayer frames (colorid 8..11, even sizes) take bayer_denoise
 * (core/io/debayer.cc:1480-1612): per Bayer plane (the 2 x 2 cell positions)
 * the 3 x 3 median (BORDER_REPLICATE) and mad = |p - median|, mad's
 * normalized 3 x 3 box mean (BORDER_REFLECT_101, rounded for integer
 * frames), and p -> median where |median - p| > k mad + minvar (1 for
 * integer frames, 1/256 for f32). Other frames take median_filter_bad_pixels
 * (core/proc/bad_pixels.cc:14-70), the same with 5 x 5 windows on the whole
 * frame. n device frames (u8, u16, f32, one channel) into n device frames;
 * dst may equal frames (strides in bytes, 0: packed). */
int sst_filter_bad_pixels(const void * frames, int depth, int n, int width, int height, size_t row_stride,
    size_t frame_stride, int colorid, double variation_threshold, void * dst, size_t dst_row_stride,
    size_t dst_frame_stride, void * stream);

/* ------------------------------------------------------ post-stack steps */

/* average_pyramid_inpaint (core/proc/inpaint/average_pyramid_inpaint.cc:
 * 18-126), applied by the stacking pipeline to the accumulated image and its
 * mask (c_image_stacking_pipeline.cc:763-767, max_levels 100): holes (mask 0)
 * are filled from 3 x 3 means over a downstrike / upject pyramid of at most
 * max_levels levels. dst / dst_mask receive the filled image and its mask
 * (255 where a value was found; a mask without holes is returned as it is).
 * Strides in bytes (0: packed). */
int sst_average_pyramid_inpaint(const float * src, size_t src_stride, const uint8_t * mask, size_t mask_stride,
    int width, int height, int max_levels, float * dst, size_t dst_stride, uint8_t * dst_mask,
    size_t dst_mask_stride, int on_device, void * stream);

/* ------------------------------------------------------ other accumulators */

/* cv::getOptimalDFTSize: the smallest 2^a 3^b 5^c >= n */
int sst_optimal_dft_size(int n);

typedef struct sst_fft_average sst_fft_average;

/* c_frame_accumulation_with_fft (core/average/c_frame_accumulation.cc:
 * 704-900). Frames are padded with BORDER_REFLECT to the optimal DFT size
 * (fftGetOptimalSize, core/proc/fft.cc:17-57, centred), transformed, and
 * their spectra averaged with per-bin weights max(s, (|F|^2 s)^3),
 * s = 1 / (DFT area)^2 (fftPower, c_frame_accumulation.cc:940-980); the
 * average is the inverse transform of the weighted mean spectrum, cropped
 * to the frame. Mono frames of an already optimal size get their weights
 * like the others (the reference leaves them empty there and fails). */
int sst_fft_average_create(sst_fft_average ** out);
int sst_fft_average_destroy(sst_fft_average * h);
int sst_fft_average_clear(sst_fft_average * h);
int sst_fft_average_accumulated_frames(const sst_fft_average * h);
/* the DFT size of the accumulated frames (0 x 0 before the first add) */
int sst_fft_average_size(const sst_fft_average * h, int * fft_width, int * fft_height);

/* add n frames (u8 / u16 / f32, `channels` interleaved channels, values
 * times `scale`); every frame of one accumulator has the same size and
 * channels. Host or device frames per on_device. */
int sst_fft_average_add(sst_fft_average * h, const void * frames, int depth, int n, int width, int height, int channels,
    size_t row_stride, size_t frame_stride, double scale, int on_device, void * stream);

/* avg (width x height x channels FP32, interleaved) and mask (u8, all 255 as
 * the reference returns it); either may be NULL; strides 0 = packed. */
int sst_fft_average_compute(sst_fft_average * h, float * avg, size_t avg_row_stride, uint8_t * mask,
    size_t mask_row_stride, int on_device, void * stream);

typedef struct sst_canvas_average sst_canvas_average;

/* c_canvas_average (c_frame_accumulation.cc:264-450); canvas_width /
 * canvas_height: setCanvasSize (0 = none). The canvas is max(requested,
 * 3/2 of the first frame) on each side. */
int sst_canvas_average_create(sst_canvas_average ** out, int canvas_width, int canvas_height);
int sst_canvas_average_destroy(sst_canvas_average * h);
int sst_canvas_average_clear(sst_canvas_average * h);
int sst_canvas_average_set_canvas_size(sst_canvas_average * h, int canvas_width, int canvas_height);

/* canvas size, last_bbox (x, y, width, height) and accumulated_frames; any
 * pointer may be NULL */
int sst_canvas_average_state(const sst_canvas_average * h, int * canvas_width, int * canvas_height, int * last_bbox,
    int * accumulated_frames);

/* c_canvas_average::add(image, weights_or_mask, rmap, new_canvas_bbox): the
 * first frame is centred on the new canvas; later frames without rmap and
 * bbox (bbox NULL or of zero size) land on the last box; with both, the box
 * is clipped to the canvas, the canvas contents shift by 64 px when the box
 * comes within 32 px of an edge (maintainCanvasBoundaries), and the image
 * remapped by rmap (bbox width x height x 2 floats, interleaved x, y;
 * LINEAR / BORDER_REPLICATE) with its weights (u8 mask: NEAREST, f32:
 * LINEAR; BORDER_CONSTANT 0; NULL: weight 1) updates the running mean
 * A += (I - A) w / W, W += w (_weighted_average_update, :20-129, FP32). A box
 * clipped by the canvas is counted but not added, as in the reference.
 * SST_ERR_INVALID_ARG for an empty box. */
int sst_canvas_average_add(sst_canvas_average * h, const void * image, int depth, int width, int height, int channels,
    size_t row_stride, double scale, const void * weights, int weights_depth, size_t weights_stride,
    const float * rmap, const int32_t * bbox, int on_device, void * stream);

/* c_canvas_average::compute(avg, mask, dscale, -1, rbbox): the canvas (or
 * the part inside rbbox, when given with a nonzero size) times dscale,
 * interleaved FP32, and mask = 255 where the weight sum is > 0. out_bbox
 * (may be NULL) receives the box returned. */
int sst_canvas_average_compute(sst_canvas_average * h, float * avg, size_t avg_row_stride, uint8_t * mask,
    size_t mask_row_stride, double dscale, const int32_t * rbbox, int32_t * out_bbox, int on_device, void * stream);

/* c_canvas_average::counter(): the weight plane (canvas size, FP32) */
int sst_canvas_average_counter(sst_canvas_average * h, float * W, size_t row_stride, int on_device, void * stream);

/* c_laplacian_pyramid_focus_stacking::fusing_policy
 * (c_frame_accumulation.h:153-156) */
#define SST_FOCUS_SELECT_MAX_ENERGY  0
#define SST_FOCUS_WEIGHTED_AVERAGE   1

/* c_laplacian_pyramid_focus_stacking::options (c_frame_accumulation.h:
 * 158-164): fusing_policy, inpaint_mask_holes (fill the mask holes of each
 * frame first), avgchannel (weighted_average: one weight from the channel
 * sum), kradius / ksigma (the Gaussian that smooths the energies:
 * getGaussianKernel(2 kradius + 1, ksigma); ksigma <= 0 takes the documented
 * default sigma 0.3 ((ksize - 1) / 2 - 1) + 0.8; none when both are 0) */
typedef struct sst_focus_stack_options {
  int32_t fusing_policy;
  int32_t inpaint_mask_holes;
  int32_t avgchannel;
  int32_t kradius;
  double ksigma;
} sst_focus_stack_options;

/* the reference defaults: select_max_energy, inpaint 1, avgchannel 1, no smoothing */
void sst_focus_stack_options_default(sst_focus_stack_options * opts);

typedef struct sst_focus_stack sst_focus_stack;

/* c_laplacian_pyramid_focus_stacking (c_frame_accumulation.cc:464-688);
 * opts NULL: the defaults */
int sst_focus_stack_create(sst_focus_stack ** out, const sst_focus_stack_options * opts);
int sst_focus_stack_destroy(sst_focus_stack * h);
int sst_focus_stack_clear(sst_focus_stack * h);
int sst_focus_stack_accumulated_frames(const sst_focus_stack * h);
/* the smoothing kernel's taps (k may be NULL to ask for *n; 0 taps: none) */
int sst_focus_stack_kernel(const sst_focus_stack * h, float * k, int * n);

/* add(src, mask) for n frames (u8 / u16 / f32 times `scale`, 1..4
 * interleaved channels, the same size for every frame): the Laplacian
 * pyramid (build_laplacian_pyramid, core/proc/laplacian_pyramid.cc:45-96,
 * minimum size 8) of each frame, after linear_interpolation_inpaint of its
 * mask holes when inpaint_mask_holes; the levels zeroed where the frame's
 * u8 mask pyramid is below 255; folded into the accumulated pyramid in
 * frame order. masks may be NULL. */
int sst_focus_stack_add(sst_focus_stack * h, const void * frames, int depth, int n, int width, int height, int channels,
    size_t row_stride, size_t frame_stride, double scale, const uint8_t * masks, size_t mask_row_stride,
    size_t mask_frame_stride, int on_device, void * stream);

/* compute(avg): reconstruct_laplacian_pyramid of the fused pyramid
 * (weighted_average: of acc / wwp), interleaved FP32 (stride 0 = packed) */
int sst_focus_stack_compute(sst_focus_stack * h, float * avg, size_t avg_row_stride, int on_device, void * stream);

/* linear_interpolation_inpaint(image, mask) (core/proc/inpaint/
 * linear_interpolation_inpaint.cc): the holes (mask 0) of an interleaved
 * FP32 image of 1..4 channels filled in place from the nearest valid pixels
 * of their row and column (a run of holes between s and e takes
 * sv + (x - s) (ev - sv) / run length; the two directions mix as
 * (h dv + v dh) / (dh + dv) with the distances dh, dv), repeated until no
 * hole gains a value. Strides in bytes (0: packed). */
int sst_linear_interpolation_inpaint(float * image, size_t row_stride, int width, int height, int channels,
    const uint8_t * mask, size_t mask_stride, int on_device, void * stream);

/* ------------------------------------------------------- stacking pipeline */

/* The per-frame body of the stacking pipeline for n frames
 * (c_image_stacking_pipeline.cc:1539-1790): register each frame against the
 * reference of `reg` (sst_ecch_align_batch semantics, min_rho gate), warp it
 * with the registered transform (base_remap, c_frame_registration.cc:
 * 1265-1340), weight it and add it to `acc`. `weighting`: 0 none; 1 the
 * frame's Laplacian-energy sharpness; 2 focus stacking: per pixel
 * W = (6 lap^2 + |grad|^2)^2 of the warped frame (5-point Laplacian and
 * central differences, BORDER_REPLICATE) blurred by a Gaussian of sigma 3;
 * 3 local-variance maps (compute_weights, c_image_stacking_pipeline.cc:
 * 2013-2020): the frame's sst_local_variance_compute map (options of
 * sst_weighted_average_set_local_variance) warped like the frame (bilinear,
 * BORDER_CONSTANT 0) and multiplied by the remapped mask
 * (c_image_stacking_pipeline.cc:1653-1658, 1704-1713); kradius <= 0 disables
 * the maps (weight 1), as weights_required does. Host frames are streamed to the
 * device in chunks whose copies overlap the registration of the previous
 * chunk; the chunks grow x 2.5 from a quarter of the chunk size set by
 * sst_set_chunk_frames up to it (the first copy is the only one that cannot
 * overlap). Outputs follow `on_device` and may be NULL. */
int sst_stack_frames(sst_ecch * reg, sst_weighted_average * acc, const void * frames, int depth, int n,
    int width, int height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int border, int weighting,
    float * params_out, int32_t * status_out, float * rho_out, float * weight_out, void * stream);

/* The Bayer form of the stacking loop body for n raw u16 mosaic frames of
 * width x height (both even): each frame's 2x2-binned luminance
 * (average_bayer_planes, core/io/debayer.cc:277-330) is registered against
 * the reference of `reg`, which must hold the binned reference (width/2 x
 * height/2); then the four Bayer planes of the raw frame
 * (extract_bayer_planes order, debayer.cc:96-147: cell positions (0,0),
 * (0,1), (1,0), (1,1)) are warped with the registered transform (the binned
 * and plane grids coincide) and added to acc[0..3], four width/2 x height/2
 * accumulators: the planar form of c_weigthed_average over the 4-channel
 * plane image. Weights, statuses, streaming and outputs as sst_stack_frames;
 * `scale` applies to the binned and the plane values alike. */
int sst_stack_bayer_frames(sst_ecch * reg, sst_weighted_average * const * acc, const void * frames, int n,
    int width, int height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    int num_passes, const sst_motion_model * passes, int border, int weighting,
    float * params_out, int32_t * status_out, float * rho_out, float * weight_out, void * stream);

/* Largest chunk of frames used by sst_stack_frames (default 512): device
 * frames are processed in chunks of this size; host frames in chunks growing
 * from a quarter of it, each chunk's host-to-device copy overlapping the
 * previous chunk's registration and stacking (two staging buffers of this
 * many frames). */
int sst_set_chunk_frames(sst_ecch * h, int frames);

/* Level iterations as CUDA graph WHILE loops (enable = 1, the default): each
 * pyramid level runs only the Gauss-Newton iterations some frame still needs.
 * enable = 0 selects the unrolled schedule (max_iterations + 1 pass / solve
 * launches per level, empty ones exit at once); the results are identical.
 * Kernel profilers do not profile single kernels of graphs that hold
 * conditional nodes, so per-kernel profiles use the unrolled schedule. */
int sst_ecch_set_level_loops(sst_ecch * h, int enable);

/* Launch shapes of the engine and the accumulator, chosen by the project's
 * autotuner (serstacker_gb300/autotune.py) per device and workload; a zero
 * field keeps the default. No counterpart in the reference (CPU code).
 *   pass_ctas_per_sm     CTAs per SM of the persistent Gauss-Newton pass
 *                        launches (0: the kernel's occupancy); results are
 *                        bitwise identical for every value
 *   pass_tile_w[c]       tile width of the staged IC / IC-LM pass on levels
 *                        of width class c (<= 192, <= 384, <= 768, wider
 *                        px): 64 or 128 (0: 64 up to 384 px, else 128); the
 *                        tile sums group differently, so results differ at
 *                        the rounding level
 *   corr_ctas_per_sm     CTAs per SM of the correlation launches (0: 4);
 *                        bitwise identical
 *   stack_max_chunks     CTAs a stack tile's frames may split over (0: 4);
 *                        the chunks' compensated partial sums are merged in
 *                        order (rounding-level differences)
 *   stack_items_per_slot (tile, chunk) CTAs aimed at per resident CTA slot
 *                        when splitting (0: 4) */
typedef struct sst_tuning {
  int32_t pass_ctas_per_sm;
  int32_t pass_tile_w[4];
  int32_t corr_ctas_per_sm;
  int32_t stack_max_chunks;
  int32_t stack_items_per_slot;
} sst_tuning;

/* the engine's fields (pass and correlation shapes); graphs are rebuilt */
int sst_ecch_set_tuning(sst_ecch * h, const sst_tuning * t);
int sst_ecch_get_tuning(const sst_ecch * h, sst_tuning * t);
/* the accumulator's fields (stack chunks) */
int sst_weighted_average_set_tuning(sst_weighted_average * h, const sst_tuning * t);

/* Number of kernels the library launched since the last call of this
 * function (graph replays count every kernel node they run). */
long long sst_kernel_launch_count(int reset);

/* ------------------------------------------------------------ SER input */

/* c_ser_file's header (core/io/c_ser_file.h:42-56) as read by c_ser_reader::open
 * (c_ser_file.cc:272-411). data_little_endian is the reference's inverted
 * reading of the LittleEndian field (1 when the field is 0). depth is an
 * SST_DEPTH_* code (SST_DEPTH_S32 for 17..32 bits, SST_DEPTH_F32 / _F64 for
 * -32 / -64), channels 3 for RGB / BGR, else 1. */
typedef struct sst_ser_info {
  int32_t luid, color_id, data_little_endian;
  int32_t width, height, bits_per_plane, frames;
  int32_t channels, bytes_per_plane, depth, has_timestamps;
  char observer[41], instrument[41], telescope[41];
  uint64_t date_time, date_time_utc;
} sst_ser_info;

typedef struct sst_ser_reader sst_ser_reader;

/* c_ser_reader::open: validates the header (file id, image size, pixel
 * format, color id) and reads the timestamp trailer when the file holds one;
 * the read position is frame 0. SST_ERR_IO for file errors, SST_ERR_UNSUPPORTED
 * for files the reference rejects. */
int sst_ser_open(sst_ser_reader ** out, const char * path);
int sst_ser_close(sst_ser_reader * r);
int sst_ser_get_info(const sst_ser_reader * r, sst_ser_info * info);

/* c_ser_file::timestamps: copies up to n timestamps, returns how many
 * (SST_ERR_STATE when the file has none) */
int sst_ser_timestamps(const sst_ser_reader * r, uint64_t * ts, int n);

/* c_ser_reader::curpos / seek (negative frames seek to 0; frames past the
 * end are rejected unless equal to the current position) */
int sst_ser_curpos(const sst_ser_reader * r);
int sst_ser_seek(sst_ser_reader * r, int frame);

/* c_ser_reader::read for up to n frames from the current position into host
 * memory, frame_stride bytes apart (0: packed); pixel data stored in the other
 * byte order than the host's is swapped. *frames_read receives the count
 * (0 at the end of the file). */
int sst_ser_read(sst_ser_reader * r, int n, void * dst, size_t frame_stride, int * frames_read);

/* c_ser_writer (core/io/c_ser_file.h:183-213, c_ser_file.cc:544-712):
 * create() writes the header of an empty file (LittleEndian field 0 on a
 * little-endian host, as the reference writes it); write() appends n frames
 * of the file's format from host memory (frame_stride 0: packed) with their
 * timestamps (NULL: UINT64_MAX each, the reference's default); the first
 * frame's timestamp becomes DateTime and DateTime_UTC. close() patches
 * FrameCount and appends the little-endian timestamp trailer. */
typedef struct sst_ser_writer sst_ser_writer;
int sst_ser_writer_create(sst_ser_writer ** out, const char * path, int width, int height, int color_id,
    int bits_per_plane);
int sst_ser_write(sst_ser_writer * w, const void * frames, int n, size_t frame_stride, const uint64_t * timestamps);
int sst_ser_writer_close(sst_ser_writer * w);

/* The stacking loop over frames [first, first + count) of a SER file (count
 * < 0: to the end): frames are read in chunks of `chunk` frames (0: 256; at
 * most 512 MB of frames per chunk) into
 * pinned host buffers, the next chunk from the file while the GPU registers
 * and stacks the current one, scaled by 1 / 2^bits_per_plane as
 * read_input_frame does (c_image_stacking_pipeline_base.cc:270-275), and
 * handed to sst_stack_frames (mono: acc[0]) or sst_stack_bayer_frames
 * (RGGB-family 16-bit Bayer: acc[0..3]). Outputs as those calls, for the
 * count frames (host memory). */
int sst_stack_ser(sst_ecch * reg, sst_weighted_average * const * acc, sst_ser_reader * ser, int first, int count,
    int chunk, int num_passes, const sst_motion_model * passes, int border, int weighting,
    float * params_out, int32_t * status_out, float * rho_out, float * weight_out, void * stream);

/* ----------------------------------------------------------- utilities */

/* c_frame_registration::base_remap of one frame (c_frame_registration.cc:
 * 1265-1340) with the transform of `model`/`params`: dst f32 (dst_width x
 * dst_height), dst_mask u8 (LINEAR/CONSTANT >= 255, 5x5 erode), either may
 * be NULL. Device buffers only. */
int sst_remap(const void * src, int depth, int src_width, int src_height, size_t row_stride, double scale,
    const sst_motion_model * model, const float * params, int border,
    float * dst, uint8_t * dst_mask, int dst_width, int dst_height, void * stream);

/* extract_bayer_planes (core/io/debayer.cc:96-147): u16 mosaic (even
 * width/height) -> 4 interleaved u16 planes of (width/2 x height/2), in the
 * mosaic order. Bit-exact. Device buffers. */
int sst_extract_bayer_planes_u16(const uint16_t * src, int width, int height, size_t row_stride,
    uint16_t * dst, void * stream);

/* average_bayer_planes (core/io/debayer.cc:277-330) of a raw mosaic:
 * (c1 + sum of the 2x2 block) / 4 in integer arithmetic. Bit-exact. */
int sst_average_bayer_planes_u16(const uint16_t * src, int width, int height, size_t row_stride,
    uint16_t * dst, void * stream);

/* ------------------------------------------------------------- c_eccflow */

/* ECCFlowDownscaleMethod (ecc2.h:509-513) */
#define SST_ECCFLOW_DOWNSCALE_RECURSIVE_RESIZE 0
#define SST_ECCFLOW_DOWNSCALE_FULL_RESIZE      1
#define SST_ECCFLOW_DOWNSCALE_PYRAMID          2

/* c_eccflow_options (ecc2.h:515-527). input_smooth_sigma and
 * reference_smooth_sigma are carried but, as in the reference, unused. */
typedef struct sst_eccflow_options {
  double update_multiplier;
  double scale_factor;
  double noise_level;
  double input_smooth_sigma;
  double reference_smooth_sigma;
  int32_t max_iterations;
  int32_t support_scale;
  int32_t min_image_size;
  int32_t max_pyramid_level;
  int32_t downscale;
  int32_t reserved;
} sst_eccflow_options;

typedef struct sst_eccflow sst_eccflow;

/* c_eccflow_options defaults (ecc2.h:515-527) */
void sst_eccflow_options_default(sst_eccflow_options * o);
int sst_eccflow_create(sst_eccflow ** out, const sst_eccflow_options * options);
int sst_eccflow_destroy(sst_eccflow * h);

/* c_eccflow::set_reference_image(reference) (ecc2.cc:2489-2672): the
 * reference pyramid, its gradients and the per-level 2x2 systems D. Values
 * are multiplied by `scale`. No mask (see _masked below). */
int sst_eccflow_set_reference_image(sst_eccflow * h, const void * image, int depth, int width, int height,
    size_t row_stride, double scale, int on_device, void * stream);

/* set_reference_image(reference, reference_mask) (ecc2.cc:2489-2672): as
 * sst_eccflow_set_reference_image, with a u8 reference mask (0 = invalid;
 * NULL: none). Each level's mask is the INTER_NEAREST resize of the mask of
 * the level its image comes from (downscale, ecc2.cc:2431-2456). */
int sst_eccflow_set_reference_image_masked(sst_eccflow * h, const void * image, int depth, int width, int height,
    size_t row_stride, double scale, const uint8_t * mask, size_t mask_stride, int on_device, void * stream);

/* number of pyramid levels of the current reference */
int sst_eccflow_num_levels(const sst_eccflow * h);

/* c_eccflow::compute(current, rmap) (ecc2.cc:2856-2865) for n frames of the
 * reference's size: rmap_out (n x height x width x 2 floats, interleaved
 * (x, y) as cv::Mat2f) receives identity + flow. init_rmap (same layout, or
 * NULL for a zero start) seeds the flow as the reference's input rmap does.
 * Buffers are host or device memory per on_device. */
int sst_eccflow_compute_batch(sst_eccflow * h, const void * frames, int depth, int n, size_t row_stride,
    size_t frame_stride, double scale, int on_device, const float * init_rmap, float * rmap_out, void * stream);

/* c_eccflow::compute(current, rmap, current_mask) for n frames with their u8
 * masks (n masks of the reference's size, mask_frame_stride bytes apart;
 * NULL: none): in every update the current mask is remapped INTER_NEAREST
 * (BORDER_CONSTANT 0) by the flow and ANDed with the reference mask, and the
 * update terms It gx, It gy are zero where that is 0 (compute_uv,
 * ecc2.cc:2253-2335). */
int sst_eccflow_compute_batch_masked(sst_eccflow * h, const void * frames, int depth, int n, size_t row_stride,
    size_t frame_stride, double scale, const uint8_t * masks, size_t mask_row_stride, size_t mask_frame_stride,
    int on_device, const float * init_rmap, float * rmap_out, void * stream);

/* -------------------------------------------- differentiable warp residual */

/* The ECC warp residual of n frames against a template and its adjoint (no
 * counterpart in the reference; the objective c_ecc_forward_additive and
 * c_ecclm minimise, ecc2.cc:1247-1365, 1444-1650):
 *   r_f(x) = I_f(W(x; p_f) + u_f(x)) - T(x)   (bilinear, BORDER_REPLICATE)
 *   L_f = 1/2 sum_x r_f(x)^2
 * frames: n x height x width f32 (frame_stride floats apart), tmpl: height x
 * width f32, params: n x 12 f32 (the model's parameter vectors), flow: n x
 * height x width x 2 f32 or NULL. Outputs (each may be NULL): loss (n f64),
 * grad_params (n x 12 f32: g_f dL_f/dp_f), grad_template (height x width f32:
 * sum_f g_f dL_f/dT), grad_flow (n x height x width x 2 f32: g_f dL_f/du_f),
 * hessian (n x 144 f64: the Gauss-Newton matrix J^T J, M x M row-major),
 * where g_f = grad_loss[f] (NULL: 1). The backward pass recomputes the warp
 * instead of storing it. Device buffers; stream ordered. Calls on one device
 * share scratch memory: do not overlap them. */
int sst_warp_residual(const float * frames, int n, int width, int height, size_t frame_stride,
    const float * tmpl, const sst_motion_model * model, const float * params, const float * flow,
    const double * grad_loss, double * loss, float * grad_params, float * grad_template, float * grad_flow,
    double * hessian, void * stream);

/* ------------------------------------------------------------ ROI batches */

/* One crop of a ROI batch: its reference and current images (same size),
 * as byte offsets into the reference and current pools with row strides. */
typedef struct sst_roi {
  int64_t ref_offset, cur_offset;
  int64_t ref_row_stride, cur_row_stride;
  int32_t width, height;
} sst_roi;

typedef struct sst_roi_batch sst_roi_batch;

/* A batch of independent c_ecch problems (ecc2.h:158-308): crop i is
 * registered against its own reference crop exactly as c_ecch(options)
 * with set_reference_image(reference crop) and align(current crop) would
 * (ecc2.cc:984-1176), for crops of different sizes in one schedule. The
 * options' method must be SST_ECC_FORWARD_ADDITIVE or SST_ECC_LM (the
 * quadratic models are not invertible, so IC and IC-LM cannot run them:
 * ecc2.cc:1702-1705). */
int sst_roi_batch_create(sst_roi_batch ** out, const sst_ecch_options * options);
int sst_roi_batch_destroy(sst_roi_batch * h);

/* Registers n crops (1..65535). Pools and outputs are host or device
 * memory per on_device; init_params (n x 12, NULL: identity) seeds the first
 * pass. Outputs per crop as sst_ecch_align_batch: params (n x 12), status,
 * iterations, eps, rho (min_rho gate of the options). Any output may be NULL. */
int sst_roi_batch_align(sst_roi_batch * h, int n, const sst_roi * rois, const void * ref_pool,
    const void * cur_pool, int depth, double scale, int on_device, int num_passes,
    const sst_motion_model * passes, const float * init_params, float * params_out, int32_t * status_out,
    int32_t * iters_out, float * eps_out, float * rho_out, void * stream);

/* Timing of one pass / level of the last call (CUDA events around its
 * launches), the frame-iterations and pixel-iterations it executed, and their
 * algorithmic bytes (8 per pixel-iteration: warped source and template). */
int sst_roi_batch_level_stats(sst_roi_batch * h, int pass, int level, float * ms, double * frame_iterations,
    double * pixel_iterations, double * algorithmic_bytes);

/* ------------------------------------------------ Bayer mosaic accumulator */

typedef struct sst_bayer_average sst_bayer_average;

/* c_bayer_average (core/average/c_frame_accumulation.h:222-262) with its
 * pattern set by set_bayer_pattern (c_frame_accumulation.cc:1138-1144).
 * width x height is the raw mosaic size of frames and accumulator alike.
 * colorid is one of SST_COLORID_BAYER_*; other patterns are rejected with
 * SST_ERR_UNSUPPORTED. */
int sst_bayer_average_create(sst_bayer_average ** out, int width, int height, int colorid);
int sst_bayer_average_destroy(sst_bayer_average * h);

/* c_bayer_average::clear (c_frame_accumulation.cc:1161-1168) */
int sst_bayer_average_clear(sst_bayer_average * h, void * stream);

/* set_remap + add for n raw mosaic frames (c_frame_accumulation.cc:
 * 1151-1203, _bayer_accumulate :988-1126, pipeline call site
 * c_image_stacking_pipeline.cc:1730-1749). With a model, frame f's remap is
 * the transform of params[f] (12 floats per frame) and the per-pixel weight
 * is the frame's remapped mask (LINEAR/CONSTANT >= 255, 5x5 erode) times
 * weights[f]; each output pixel gathers the four raw samples around its
 * truncated remap position into the colour channels of their mosaic
 * positions. Without a model (model NULL: no registration, empty rmap) each
 * raw sample goes to its own channel with weight weights[f]. Frames whose
 * status is not SST_FRAME_OK or whose weight is <= 0 are skipped; status
 * and weights may be NULL. Raw values are multiplied by `scale`. */
int sst_bayer_average_add_batch(sst_bayer_average * h, const void * frames, int depth, int n,
    size_t row_stride, size_t frame_stride, double scale, int on_device, const sst_motion_model * model,
    const float * params, const int32_t * status, const float * weights, void * stream);

/* c_bayer_average::compute (c_frame_accumulation.cc:1205-1238) and
 * get_acc_counters (:1240-1250): avg is width x height x 3 f32 (B, G, R
 * interleaved as the reference's Mat3f), 0 where a channel has no weight;
 * mask u8 is 255 where any channel has weight; accw is width x height x 3
 * f32, the channel weight sums with green halved. Any output may be NULL. */
int sst_bayer_average_compute(sst_bayer_average * h, float * avg, uint8_t * mask, float * accw,
    int on_device, void * stream);

/* c_frame_accumulation::accumulated_frames */
int sst_bayer_average_accumulated_frames(const sst_bayer_average * h);

/* Checkpoint: the 12 compensated planes (for channel B, G, R: sum of w*I,
 * its compensation, sum of w, its compensation; width x height f32 each) in
 * a host buffer, and the frame count. */
int sst_bayer_average_save_state(sst_bayer_average * h, float * state12, int32_t * frames, void * stream);
int sst_bayer_average_load_state(sst_bayer_average * h, const float * state12, int32_t frames, void * stream);

/* ------------------------------------------------ replicas: state merge */

/* Adds the accumulator state `src` into `dst` (host buffers), both `groups`
 * groups of four planes of `plane` floats (sum of w*I, its compensation, sum
 * of w, its compensation): 1 group for sst_weighted_average_save_state, 3 for
 * sst_bayer_average_save_state. The leading sums are merged with TwoSum, so
 * no rounding error is lost. Replicas that each stacked a contiguous range
 * of frames merge their states in rank order and load the result. Not in
 * the reference, whose stacking runs in one process. */
int sst_state_merge(float * dst, const float * src, int groups, size_t plane);

/* ------------------------------------------------------ frame registration */

/* color_channel_gray of color_channel_type (core/proc/extract_channel.h:31):
 * the registration channel of mono frames, which is the frame itself */
#define SST_COLOR_CHANNEL_GRAY 104

/* c_ecc_registration_options (core/proc/image_registration/
 * c_frame_registration.h:47-63), same fields and defaults */
typedef struct sst_ecc_registration_options {
  double scale;                     /* 0.5: ECC on scaleImage(frame): pyrDown at 0.5, INTER_AREA otherwise */
  double eps;                       /* 0.2: c_ecch epsx */
  double min_rho;                   /* 0.8: correlation gate after alignment */
  double input_smooth_sigma;        /* 1 */
  double reference_smooth_sigma;    /* 1 */
  double update_step_scale;         /* 1.5 */
  double normalization_noise;       /* 0.01 */
  int32_t se_radius;                /* 5 (planetary-disk masks only) */
  int32_t ecc_method;               /* SST_ECC_LM */
  int32_t max_iterations;           /* 50 */
  int32_t ecch_max_level;           /* 0 */
  int32_t ecch_minimum_image_size;  /* 16 */
  int32_t normalization_scale;      /* 0: ecc_normalize off; > 0: its pyramid level */
  int32_t ecch_estimate_translation_first;   /* 1 */
  int32_t replace_planetary_disk_with_mask;  /* 0; 1 is not supported */
} sst_ecc_registration_options;

/* c_eccflow_registration_options (c_frame_registration.h:88-100) */
typedef struct sst_eccflow_registration_options {
  double update_multiplier;         /* 1.5 */
  double input_smooth_sigma;        /* 0 */
  double reference_smooth_sigma;    /* 0 */
  double noise_level;               /* -1 */
  double scale_factor;              /* 0.75 */
  int32_t max_iterations;           /* 3 */
  int32_t support_scale;            /* 4 */
  int32_t min_image_size;           /* -1 */
  int32_t max_pyramid_level;        /* -1 */
  int32_t downscale_method;         /* SST_ECCFLOW_DOWNSCALE_RECURSIVE_RESIZE */
  int32_t reserved;
} sst_eccflow_registration_options;

/* c_image_registration_options (c_frame_registration.h:119-137). The
 * reference's defaults enable feature registration (AKAZE / ORB matching),
 * which is not part of this library: set enable_feature_registration = 0
 * and enable ECC and / or eccflow registration. */
typedef struct sst_image_registration_options {
  int32_t motion_type;              /* SST_MOTION_AFFINE */
  int32_t ecc_registration_channel; /* SST_COLOR_CHANNEL_GRAY (frames are mono) */
  int32_t interpolation;            /* ECC_INTER_LINEAR (1) */
  int32_t border_mode;              /* SST_BORDER_REFLECT101 */
  double border_value;              /* 0 */
  sst_ecc_registration_options ecc;
  sst_eccflow_registration_options eccflow;
  int32_t enable_feature_registration;               /* 1 in the reference; must be 0 */
  int32_t enable_ecc_registration;                   /* 0 */
  int32_t enable_eccflow_registration;               /* 0 */
  int32_t accumulate_and_compensate_turbulent_flow;  /* 0; 1 is not supported */
} sst_image_registration_options;

/* The reference defaults of the three option structs. */
void sst_image_registration_options_default(sst_image_registration_options * opts);

typedef struct sst_frame_registration sst_frame_registration;

/* c_frame_registration (c_frame_registration.h:210-356) with ECC and / or
 * eccflow registration of mono frames. */
int sst_frame_registration_create(sst_frame_registration ** out, const sst_image_registration_options * opts);
int sst_frame_registration_destroy(sst_frame_registration * h);

/* c_frame_registration::setup_reference_frame(reference_image, reference_mask)
 * (c_frame_registration.cc:565-719): the ECC reference is
 * scaleImage(reference, ecc.scale) (pyrDown at 0.5, INTER_AREA otherwise; the
 * mask pyrDown'ed / resized, then >= 250; c_frame_registration.cc:230-250),
 * ecc_normalize'd when normalization_scale > 0 and normalization_noise > 0
 * (ecc2.cc:385-397), and handed to c_ecch; the eccflow reference is the
 * full-size image and mask. Values are multiplied by `scale`. mask may be
 * NULL (u8, 0 = invalid). */
int sst_frame_registration_setup_reference_frame(sst_frame_registration * h, const void * image, int depth,
    int width, int height, size_t row_stride, double scale, const uint8_t * mask, size_t mask_stride,
    int on_device, void * stream);

/* c_frame_registration::register_frame (c_frame_registration.cc:721-964)
 * for n frames of the reference's size, registered together: each frame's
 * ECC image (scaleImage, ecc_normalize) is aligned by the batched c_ecch
 * engine, first as a translation with the gate rho >= 0.75 min_rho when
 * ecch_estimate_translation_first applies (motion_type not TRANSLATION,
 * ecch_max_level != 0), then with motion_type and the gate rho >= min_rho;
 * the result is scaled back by 1 / ecc.scale. With eccflow registration the
 * transform's remap at full size is refined by c_eccflow::compute.
 *   params_out     n x 12 floats: motion_type's parameter vector at full size
 *   status_out     SST_FRAME_* (SST_FRAME_LOW_RHO for either gate)
 *   rho_out        the last correlation computed for the frame
 *   iterations_out Gauss-Newton iterations over both passes and all levels
 *   rmap_out       n x height x width x 2 floats (interleaved x, y as
 *                  cv::Mat2f): the current remap (current_remap(),
 *                  c_frame_registration.h:308); may be NULL
 * Frames and outputs are host or device memory per on_device; outputs may be NULL. */
int sst_frame_registration_register_frames(sst_frame_registration * h, const void * frames, int depth, int n,
    int width, int height, size_t row_stride, size_t frame_stride, double scale, int on_device,
    float * params_out, int32_t * status_out, float * rho_out, int32_t * iterations_out, float * rmap_out,
    void * stream);

/* Frames registered per engine launch (default 256). */
int sst_frame_registration_set_chunk_frames(sst_frame_registration * h, int frames);

/* Size of the ECC images (the reference size scaled by scaleImage). */
int sst_frame_registration_ecc_size(const sst_frame_registration * h, int * width, int * height);

/* The ECC image (after scaleImage and ecc_normalize) of the reference
 * (frame = -1, with its ECC mask when mask_out is not NULL) or of frame
 * `frame` of the last chunk registered; out is ecc width x height floats. */
int sst_frame_registration_ecc_image(sst_frame_registration * h, int frame, float * out, uint8_t * mask_out,
    int on_device);

/* c_frame_registration::base_remap / custom_remap with a dense remap
 * (c_frame_registration.cc:1265-1386): dst (f32, dst_width x dst_height) =
 * cv::remap(src * scale, rmap, INTER_LINEAR, border, border_value); dst_mask
 * (u8) = remap of src_mask (all 255 when NULL) with LINEAR / BORDER_CONSTANT
 * 0, compared >= 255 and eroded 5 x 5. rmap is dst_width x dst_height x 2
 * floats. Either output may be NULL. Buffers are host or device memory per
 * on_device (packed dst rows). */
int sst_remap_rmap(const void * src, int depth, int src_width, int src_height, size_t row_stride, double scale,
    const float * rmap, int dst_width, int dst_height, int border, double border_value, const uint8_t * src_mask,
    size_t mask_stride, float * dst, uint8_t * dst_mask, int on_device, void * stream);

/* c_image_transform::scale_transfrom(factor) (c_image_transform.h:101;
 * per-model overrides c_image_transform.cc:130-1781) on a parameter vector
 * of `model`, in place (host memory). */
int sst_image_transform_scale(const sst_motion_model * model, float * params, double factor);

/* c_image_transform::create_remap(size, map) (c_image_transform.cc:150-170,
 * 525-555, 926-946, 1207-1223, 1531-1547, 1783-1798): rmap (width x height x
 * 2 floats, interleaved x, y) = W(x, y; params). Host or device memory per
 * on_device. */
int sst_image_transform_create_remap(const sst_motion_model * model, const float * params, int width, int height,
    float * rmap, int on_device, void * stream);

/* ------------------------------------------------ allocation-free stacking */

/* Largest batch the allocation-free entry point accepts. */
#define SST_NOALLOC_MAX_FRAMES 4096

/* Allocation-free variant of sst_weighted_average_add_warped_batch. This
 * entry point has no counterpart in the reference: SerStacker allocates its
 * accumulators with OpenCV and never runs on a GPU.
 *
 * It exists for callers that cannot let the library call cudaMalloc:
 *   - hosts that own all device memory through their own pool or arena (an
 *     allocation behind their back breaks their accounting, or fails once
 *     the pool has reserved the device);
 *   - real-time capture loops that cannot afford cudaMalloc's implicit
 *     device-wide synchronisation.
 * It warps, weights and accumulates n device-resident frames exactly like
 * sst_weighted_average_add_warped_batch (same kernels), but allocates
 * nothing: the per-frame scratch (warp coefficients and effective weights)
 * lives in a fixed device array of SST_NOALLOC_MAX_FRAMES entries that the
 * library declares at file scope, so every GPU that loads the library holds
 * it (about 272 KB) until the process exits, and the accumulator is the
 * caller's: acc_state holds 4 planes of dst_width x dst_height floats (sum
 * of w*I, its compensation, sum of w, its compensation), zeroed by the
 * caller before the first call and read back with any kernel or copy.
 *
 * All pointers are device pointers; params is n x 12 floats, status and
 * weights (n entries each) may be NULL. n > SST_NOALLOC_MAX_FRAMES is
 * rejected with SST_ERR_INVALID_ARG.
 *
 * The call returns once its work on `stream` has finished: it clears a
 * device error word before the launch and reads it back after it, and
 * returns SST_ERR_TIMEOUT (acc_state invalid: rebuild it) if a stacking
 * kernel raised it. The batched stacking kernels read the frames directly
 * and hold no waits, so none raises it today; the word stays the kernels'
 * error channel.
 *
 * The first call on each device looks up the device addresses of the
 * scratch array and of that word (cudaGetSymbolAddress) with that device
 * current: make that first call before capturing any stream. All calls share
 * the one array: calls whose work can overlap on the GPU (e.g. on unordered
 * streams) race and must not be issued concurrently. */
int sst_weighted_average_add_warped_batch_noalloc(const void * frames, int depth, int n,
    int src_width, int src_height, size_t row_stride, size_t frame_stride, double scale,
    const sst_motion_model * model, const float * params, const int32_t * status, const float * weights,
    int border, float * acc_state, int dst_width, int dst_height, void * stream);

#ifdef __cplusplus
}
#endif

#endif /* SERSTACKER_GB300_H */
