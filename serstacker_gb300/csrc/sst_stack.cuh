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
cudaError_t launch_bayer_planes(int op, const uint16_t * src, int w, int h, size_t rs, uint16_t * dst, cudaStream_t st);

}  // namespace sst
