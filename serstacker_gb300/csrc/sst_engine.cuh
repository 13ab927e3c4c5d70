/*
 * sst_engine.cuh -- device data structures of the batched c_ecch engine and
 * the launch helpers shared by the kernel translation units and the C ABI.
 *
 * Execution model (one GPU): the frames of a batch live side by side in HBM
 * (one f32 pyramid per frame). A Gauss-Newton "step" is ONE kernel launch
 * over every frame that still iterates at the current pyramid level: the
 * launch walks a compacted list of active frames x tiles, each CTA reduces
 * its tile, and the last CTA to finish a frame (atomic ticket) combines the
 * frame's tile partials in a fixed order and runs that frame's FP64 solve /
 * convergence logic, appending the frame to the next step's active list if
 * it keeps iterating. Step k reads list k and writes list k+1, so the whole
 * level x iteration schedule is a static sequence of launches that is
 * captured once into a CUDA graph and replayed.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "sst_internal.cuh"
#include "sst_model.cuh"

namespace sst {

enum Method {
  M_FA = SST_ECC_FORWARD_ADDITIVE,
  M_IC = SST_ECC_INVERSE_COMPOSITIONAL,
  M_LM = SST_ECC_LM,
  M_ICLM = SST_ECC_INVERSE_COMPOSITIONAL_LM
};

/* steepest-descent image formula selector */
enum JacKind { J_TRANS = 0, J_EUCL = 1, J_AFFINE = 2, J_HOMOG = 3, J_SEMIQ = 4, J_QUAD = 5 };

__host__ __device__ inline int jac_kind(int motion)
{
  switch ( motion ) {
  case SST_MOTION_TRANSLATION: return J_TRANS;
  case SST_MOTION_EUCLIDEAN:
  case SST_MOTION_SCALED_EUCLIDEAN: return J_EUCL;
  case SST_MOTION_AFFINE: return J_AFFINE;
  case SST_MOTION_HOMOGRAPHY:
  case SST_MOTION_EPIPOLAR_DEROTATION: return J_HOMOG;
  case SST_MOTION_SEMI_QUADRATIC: return J_SEMIQ;
  default: return J_QUAD;
  }
}

enum Phase { PH_START = 0, PH_TRIAL = 1 };

/* Per-frame registration state (global memory, one per frame slot). */
struct FrameState {
  double state[16];     // accepted transform state
  double eval[16];      // state the next pass evaluates (== state, or an LM trial)
  double v[12];         // LM: J^T r at state; IC-LM: scaled J^T r at state
  double Hs[144];       // LM: J^T J at state
  double dpv[12];       // last Gauss-Newton delta
  double err, lambda, rmsold, eps, dpe, pad0;
  float wc[16];         // FP32 displacement coefficients of eval (current level)
  float jc[8];          // FP32 steepest-descent coefficients of eval
  int32_t n;            // iterations at the current level (reference counting)
  int32_t phase;
  int32_t converged;
  int32_t level_ok;
  int32_t status;       // SST_FRAME_*
  int32_t total_iters;
  float rho, weight;
};

/* Arguments of one Gauss-Newton pass launch (by value). */
struct PassArgs {
  const float * pyr;        // frame 0 level 0
  size_t pyr_stride;        // floats per frame
  size_t lvl_off;           // floats from a frame's level 0 to this level
  int w, h;                 // level size (reference == current)
  int tiles, tiles_x;       // tiles of this level for this kernel's tile shape
  const float * refT;       // reference level image
  const float2 * refG;      // reference level gradients (zero where the reference mask is 0)
  const float4 * refTG;     // packed {T, gx, gy, 0} of the level (one 128-bit load per pixel)
  const uint8_t * refM;     // reference level mask or nullptr
  const uint8_t * refMe;    // 5x5-eroded reference mask (LM) or nullptr
  const double * H;         // IC / IC-LM: M x M Gauss-Newton matrix at this level
  const double * Hinv;      // IC: its inverse (nullptr when H is not positive definite)
  double RMA;               // number of valid reference pixels
  float tshift;             // mean of the reference level (numerical shift for FA sums)
  float jc_id[8];           // identity steepest-descent coefficients (IC / IC-LM)
  FrameState * fs;
  double * partials;        // per frame: tiles x NS doubles
  size_t part_stride;       // doubles per frame
  unsigned * counters;      // per frame tile tickets
  const int * list_in;
  const int * count_in;
  int * list_out;
  int * count_out;
  sst_motion_model model;
  int M;
  double max_eps, step;
  int max_it;
  double scale_next;        // scale_transfrom factor to the next finer level, 0 at level 0
};

/* pointwise passes (IC, IC-LM, correlation): 128 x 64 pixel tiles, 256 threads */
constexpr int PW_TX = 128, PW_TY = 64;
/* stencil passes (FA, LM): 64 x 16 pixel tiles + 2 px halo, 256 threads */
constexpr int ST_TX = 64, ST_TY = 16;

inline int tiles_of(int w, int h, int tx, int ty, int * tiles_x)
{
  *tiles_x = (w + tx - 1) / tx;
  return *tiles_x * ((h + ty - 1) / ty);
}

/* kernel launchers (defined in the .cu files) */
cudaError_t launch_pass(int method, const PassArgs & a, int grid, cudaStream_t st);
__host__ __device__ int pass_num_sums(int method, int M);
cudaError_t launch_solve(int method, const PassArgs & a, int grid, cudaStream_t st);

struct LevelBeginArgs {
  FrameState * fs;
  int n;
  sst_motion_model model;
  int method;
  int * list_out;
  int * count_out;
  int level_is_first;
};
cudaError_t launch_level_begin(const LevelBeginArgs & a, cudaStream_t st);

struct PassBeginArgs {
  FrameState * fs;
  int n;
  int pass;
  sst_motion_model model, prev_model;
  const double * init_states;   // n x 16 or nullptr
  double scale_to_coarsest;
};
cudaError_t launch_pass_begin(const PassBeginArgs & a, cudaStream_t st);

struct CorrArgs {
  const float * pyr;
  size_t pyr_stride;
  int w, h, tiles, tiles_x;
  const float * refT;
  const uint8_t * refM;
  float tshift;
  FrameState * fs;
  int n;
  double * partials;
  size_t part_stride;
  unsigned * counters;
  sst_motion_model model;
  double min_rho;
};
cudaError_t launch_correlation(const CorrArgs & a, int grid, cudaStream_t st);

struct FinalizeArgs {
  FrameState * fs;
  int n;
  sst_motion_model model;
  const double * lap_partials;   // n x lap_tiles x 2
  int lap_tiles;
  float * params_out;            // n x 12
  int32_t * status_out, * iters_out;
  float * eps_out, * rho_out, * weight_out;
};
cudaError_t launch_finalize(const FinalizeArgs & a, cudaStream_t st);

/* pyramid / reference kernels (sst_pyramid.cu) */
cudaError_t launch_convert_smooth(const void * src, int depth, int n, int w, int h, size_t row_stride,
    size_t frame_stride, double scale, const float * gk, int ksize, float * dst, size_t dst_stride, cudaStream_t st);
cudaError_t launch_pyrdown(const float * src, int sw, int sh, size_t src_stride, float * dst, int dw, int dh,
    size_t dst_stride, int n, cudaStream_t st);
cudaError_t launch_resize_nearest_u8(const uint8_t * src, int sw, int sh, uint8_t * dst, int dw, int dh, cudaStream_t st);
cudaError_t launch_ref_gradients(const float * img, const uint8_t * mask, int w, int h, float2 * grad, cudaStream_t st);
cudaError_t launch_pack_reference(const float * img, const float2 * grad, size_t n, float4 * out, cudaStream_t st);
cudaError_t launch_erode5(const uint8_t * src, int w, int h, uint8_t * dst, cudaStream_t st);
cudaError_t launch_ref_hessian(const float2 * grad, int w, int h, int jkind, int M, const float * jc,
    double * partials, int * tiles_out, cudaStream_t st);
cudaError_t launch_ref_stats(const float * img, const uint8_t * mask, int w, int h, double * partials,
    int * tiles_out, cudaStream_t st);
cudaError_t launch_lap_energy(const float * pyr, size_t pyr_stride, size_t lvl_off, int w, int h, int n,
    double * partials, int tiles, cudaStream_t st);
int lap_tiles(int w, int h);

}  // namespace sst
