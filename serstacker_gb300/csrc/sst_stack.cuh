/*
 * sst_stack.cuh -- launch interface of the accumulation / remap kernels.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/serstacker_gb300.h"

namespace sst {

struct StackArgs {
  const uint8_t * frames;   // frame 0, row-major, depth per template
  size_t row_stride, frame_stride;
  int sw, sh;               // source frame size
  int n;
  float scale;              // value conversion factor (ecc_convert / bpp scaling)
  const float * coeffs;     // n x 16 FP32 displacement coefficients
  const float * weights;    // n effective weights (0 = skip frame)
  int dw, dh;               // accumulator size
  float * acc;              // 4 planes: S, cS, W, cW
  size_t plane;             // floats per plane
  int border;               // image border mode of the remap (SST_BORDER_*)
  const float * wmap = nullptr;   // optional per-pixel weight maps (n x plane, output grid)
  int * err = nullptr;            // optional error flag (set to 1 on a kernel-side failure; no kernel waits today)
  // optional scratch for frame chunks: (max_chunks - 1) x 4 planes of partial
  // sums, so that one tile's frames can be split over several CTAs
  float * part = nullptr;
  int max_chunks = 1;
  int items_per_slot = 4;         // (tile, chunk) CTAs aimed at per resident CTA slot
};

/* four Bayer planes of raw u16 mosaic frames, stacked into four accumulators */
struct BayerPlanesArgs {
  const uint8_t * frames;   // raw mosaic frame 0 (u16)
  size_t row_stride, frame_stride;
  int pw, ph;               // plane size = raw size / 2 = accumulator size
  int n;
  float scale;
  const float * coeffs;     // n x 16, plane coordinates
  const float * weights;    // n effective weights
  float * acc[4];           // 4 planes (S, cS, W, cW) per Bayer plane
  size_t plane;
  int border;
  const float * wmap = nullptr;   // optional per-pixel weight maps (n x plane)
};

cudaError_t launch_coeffs_from_params(const sst_motion_model & m, const float * params, int n, float * coeffs, cudaStream_t st);
cudaError_t launch_effective_weights(const float * weights, const int32_t * status, int n, float * out, cudaStream_t st);
cudaError_t launch_stack_add_warped(const StackArgs & a, int motion, int depth, cudaStream_t st);
cudaError_t launch_stack_add_plain(const void * src, int depth, size_t row_stride, double scale, const void * wts,
    int wdepth, size_t wstride, int w, int h, float * acc, size_t plane, cudaStream_t st);
cudaError_t launch_stack_compute(const float * acc, size_t plane, int n, float * avg, uint8_t * mask, float * accw, cudaStream_t st);
cudaError_t launch_stack_reinit(float * acc, size_t plane, int n, const float * avg, const float * accw, cudaStream_t st);
cudaError_t launch_remap(const void * src, int depth, int sw, int sh, size_t rs, double scale, int motion,
    const float * coeffs, int border, float * dst, uint8_t * dst_mask, int dw, int dh, cudaStream_t st);
cudaError_t launch_average_bayer_planes_batch(const void * src, int w, int h, size_t rs, size_t frame_stride, int n,
    uint16_t * dst, cudaStream_t st);
cudaError_t launch_stack_bayer_planes(const BayerPlanesArgs & a, int motion, cudaStream_t st);
/* focus weights W = (6 lap^2 + |grad|^2)^2 of each frame warped to the output grid */
cudaError_t launch_focus_energy(const void * frames, int depth, size_t row_stride, size_t frame_stride, int sw, int sh,
    double scale, int motion, const float * coeffs, int n, int dw, int dh, float * out, cudaStream_t st);
cudaError_t launch_bayer_planes(int op, const uint16_t * src, int w, int h, size_t rs, uint16_t * dst, cudaStream_t st);

}  // namespace sst
