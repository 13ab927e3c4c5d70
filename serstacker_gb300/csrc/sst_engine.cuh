/*
 * sst_engine.cuh -- device data structures of the batched c_ecch engine and
 * the launch helpers shared by the kernel translation units and the C ABI.
 *
 * Execution model (one GPU): the frames of a batch live side by side in HBM
 * (one f32 pyramid per frame). A Gauss-Newton "step" is two launches over
 * every frame that still iterates at the current pyramid level: the pass
 * kernel walks a compacted list of active frames x tiles and stores one set
 * of FP64 partial sums per tile; the solve kernel gives each active frame a
 * warp that combines the frame's tile partials in a fixed order and runs the
 * frame's FP64 solve / convergence logic, appending the frame to the next
 * step's active list if it keeps iterating. Step k reads list k and writes
 * list k+1, so the whole level x iteration schedule is a static sequence of
 * launches that is captured once into a CUDA graph and replayed.
 *
 * ROI batches (frames of different sizes, each with its own reference) use
 * the same schedule with per-frame level geometry (RoiLevel): the pass
 * kernel maps its work index to (frame, tile) through a prefix sum of the
 * active frames' tile counts, rebuilt for every step by k_roi_scan.
 */
#pragma once
#include <cuda.h>            // CUtensorMap
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

/* Geometry of one frame at one pyramid level in a ROI batch. */
struct RoiLevel {
  size_t cur_off;           // floats from the current pool to this frame's level
  size_t ref_off;           // floats from the reference pool to this frame's level
  size_t part_off;          // doubles from the partials base to this frame's partials (all levels)
  int w, h;                 // level size; w == 0: the frame has no such level
  int tiles_x, tiles;       // stencil tiles (ST_TX x ST_TY) of the level
  int ctiles_x, ctiles;     // correlation tiles (PW_TX x PW_TY), level 0 only
  double scale_next;        // scale_transfrom factor to the next finer level (0 at level 0)
  double scale_first;       // level-0 entry: factor from level 0 to the frame's coarsest level
  float tshift;             // mean of the frame's reference (numerical shift of the FA sums)
  int pad;
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
  // ROI batches (roi != nullptr): per-frame geometry replaces pyr_stride / lvl_off / w / h / tiles
  const RoiLevel * roi;     // n x lmax entries
  int lmax, level;
  const int * tile_prefix;  // per entry of list_in: tiles of the entries before it (k_roi_scan)
  const int * tile_total;   // tiles of the whole list
  int * err;                // set to 1 when a bounded wait for a staged tile gave up
  int tile_w;               // staged IC / IC-LM pass: tile width (PW_TX, or 64 on narrow levels)
};

/* pointwise passes (IC, IC-LM, correlation): 128 x 32 pixel tiles, 256 threads */
constexpr int PW_TX = 128, PW_TY = 32;
/* stencil passes (FA, LM): 64 x 16 pixel tiles + 2 px halo, 256 threads */
constexpr int ST_TX = 64, ST_TY = 16;

inline int tiles_of(int w, int h, int tx, int ty, int * tiles_x)
{
  *tiles_x = (w + tx - 1) / tx;
  return *tiles_x * ((h + ty - 1) / ty);
}

/* kernel launchers (defined in the .cu files) */
cudaError_t launch_pass(int method, const PassArgs & a, int grid, cudaStream_t st, const CUtensorMap * map = nullptr);
bool encode_pass_level(const float * level_of_slot0, int w, int h, size_t pyr_stride, int frames, CUtensorMap * map,
    int tile_w = PW_TX);
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
  const RoiLevel * roi;     // ROI batches: frames without this level are not listed
  int lmax, level;
};
cudaError_t launch_level_begin(const LevelBeginArgs & a, cudaStream_t st);

/* One level's Gauss-Newton iterations as a graph WHILE loop: the pass reads
 * list A, the solve appends to list B, and the advance kernel moves B to A. */
struct LevelLoopArgs {
  int * cursor;             // iterations done at this level
  int * list_a;             // active frames of the next pass
  int * count_a;
  const int * list_b;       // frames the solve kept iterating
  int * count_b;
  int * hist;               // per iteration: active frames at its start (step history)
  int max_it;
  cudaGraphConditionalHandle handle;
};
cudaError_t launch_level_advance(const LevelLoopArgs & a, cudaStream_t st);
/* kernel launches made by the level loops since the last reset (3 per iteration) */
long long loop_launches(bool reset);

struct PassBeginArgs {
  FrameState * fs;
  int n;
  int pass;
  sst_motion_model model, prev_model;
  const double * init_states;   // n x 16 or nullptr
  double scale_to_coarsest;
  const RoiLevel * roi;          // ROI batches: per-frame factor (RoiLevel::scale_first)
  int lmax;
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
  const RoiLevel * roi;          // ROI batches: per-frame level-0 geometry
  int lmax;
  const int * tile_prefix;       // n + 1 correlation tile offsets (all frames)
  int * err;                     // set to 1 when a bounded wait for a staged tile gave up
};
cudaError_t launch_correlation(const CorrArgs & a, int grid, cudaStream_t st, const CUtensorMap * map = nullptr);

/* ROI batches: prefix sums of the active frames' tile counts for one step */
cudaError_t launch_roi_scan(const int * list, const int * count, const RoiLevel * roi, int lmax, int level,
    int * prefix, int * total, cudaStream_t st);

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

/* One image of a ragged batch job (grid.z = job): source at src_off (bytes
 * for convert, floats for pyrDown) of sw x sh with src_stride bytes per row
 * (convert), destination at dst_off floats of dw x dh. */
struct RaggedImg {
  size_t src_off, dst_off, src_stride;
  int sw, sh, dw, dh;
};

/* pyramid / reference kernels (sst_pyramid.cu) */
cudaError_t launch_convert_smooth_ragged(const void * src, int depth, const RaggedImg * jobs, int n, int max_w,
    int max_h, double scale, const float * gk, int ksize, float * dst, cudaStream_t st);
cudaError_t launch_pyrdown_ragged(const float * src, const RaggedImg * jobs, int n, int max_dw, int max_dh,
    float * dst, cudaStream_t st);
cudaError_t launch_roi_means(const float * pool, const RaggedImg * jobs, int n, double * sums, cudaStream_t st);
cudaError_t launch_convert_smooth(const void * src, int depth, int n, int w, int h, size_t row_stride,
    size_t frame_stride, double scale, const float * gk, int ksize, float * dst, size_t dst_stride, cudaStream_t st);
cudaError_t launch_pyrdown(const float * src, int sw, int sh, size_t src_stride, float * dst, int dw, int dh,
    size_t dst_stride, int n, cudaStream_t st);
cudaError_t launch_convert_pyr1(const void * src, int depth, int n, int w, int h, size_t row_stride,
    size_t frame_stride, double scale, const float * gk, int ksize, float * dst0, float * dst1, int dw, int dh,
    size_t dst_stride, int * err, cudaStream_t st, bool * done);
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
