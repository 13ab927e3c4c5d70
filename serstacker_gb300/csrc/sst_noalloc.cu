/*
 * sst_noalloc.cu -- allocation-free variant of the batched warp + weighted stack.
 *
 * sst_weighted_average_add_warped_batch() keeps its per-frame scratch (the
 * FP32 warp coefficients and the effective frame weights) in buffers the
 * accumulator object allocates with cudaMalloc. Some callers cannot allow
 * that: hosts that own every byte of device memory through their own pool or
 * arena (a cudaMalloc behind their back breaks their accounting, or fails
 * when the pool has reserved the device), and real-time capture loops that
 * must not pay cudaMalloc's implicit device-wide synchronisation. For them,
 * sst_weighted_average_add_warped_batch_noalloc() runs the same kernels with
 * that scratch placed in a fixed file-scope device array, and the caller
 * passes the accumulator planes it owns.
 *
 * The array holds SST_NOALLOC_MAX_FRAMES frames and is resident on every GPU
 * that loads the library, until the process exits. Every call shares it:
 * calls whose work overlaps on the GPU (different streams, no ordering) race
 * on it and must not be issued. Each call writes the scratch entries of its
 * n frames before reading them, so nothing there has to start at zero. The
 * one word that must start at zero, the stacking kernels' error flag
 * (StackArgs::err), is cleared on the stream before each launch and read back
 * after it: the call returns once its work on the stream has finished, with
 * SST_ERR_TIMEOUT if the flag was raised. (The batched kernels read the
 * frames directly and hold no bounded waits, so none raises it today.)
 */
#include <mutex>

#include "sst_engine.cuh"
#include "sst_stack.cuh"

int sst_internal_error(int code, const char * msg);   // sst_capi.cu

namespace {

/* per frame: SST_NCOEF warp coefficients and one effective weight */
static __device__ __align__(256) float g_noalloc_scratch[SST_NOALLOC_MAX_FRAMES * (SST_NCOEF + 1)];
/* the stacking kernels' error flag (StackArgs::err), raised by setting it to 1 */
static __device__ __align__(16) int g_noalloc_wait_flag;

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
float * g_noalloc_ptr[kMaxDevices] = { nullptr };
int * g_noalloc_flag_ptr[kMaxDevices] = { nullptr };

/* errors are reported through sst_last_error(), like every other entry point */
int fail(int code, const char * msg)
{
  return sst_internal_error(code, msg);
}

/* Device addresses of the scratch array and the wait flag on the current
 * device: looked up once per device, with that device current. */
int scratch_address(float ** out, int ** flag)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if( e != cudaSuccess ) return fail(SST_ERR_CUDA, cudaGetErrorString(e));
  if( dev < 0 || dev >= kMaxDevices ) return fail(SST_ERR_UNSUPPORTED, "device index out of range for the no-alloc scratch table");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if( !g_noalloc_ptr[dev] ) {
    void * p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if( e != cudaSuccess ) return fail(SST_ERR_CUDA, cudaGetErrorString(e));
    void * q = nullptr;
    e = cudaGetSymbolAddress(&q, g_noalloc_wait_flag);
    if( e != cudaSuccess ) return fail(SST_ERR_CUDA, cudaGetErrorString(e));
    g_noalloc_ptr[dev] = (float *) p;
    g_noalloc_flag_ptr[dev] = (int *) q;
  }
  *out = g_noalloc_ptr[dev];
  *flag = g_noalloc_flag_ptr[dev];
  return SST_OK;
}

}  // namespace

extern "C" int sst_weighted_average_add_warped_batch_noalloc(const void * frames, int depth, int n,
    int src_width, int src_height, size_t row_stride, size_t frame_stride, double scale,
    const sst_motion_model * model, const float * params, const int32_t * status, const float * weights,
    int border, float * acc_state, int dst_width, int dst_height, void * stream)
{
  if( !frames || !model || !params || !acc_state ) return fail(SST_ERR_INVALID_ARG, "NULL argument");
  if( n < 1 ) return fail(SST_ERR_INVALID_ARG, "n must be >= 1");
  if( n > SST_NOALLOC_MAX_FRAMES ) {
    return fail(SST_ERR_INVALID_ARG,
        "n exceeds SST_NOALLOC_MAX_FRAMES: split the batch or use sst_weighted_average_add_warped_batch");
  }
  const int bytes = depth == SST_DEPTH_U8 ? 1 : depth == SST_DEPTH_U16 ? 2 : depth == SST_DEPTH_F32 ? 4 : 0;
  if( !bytes ) return fail(SST_ERR_INVALID_ARG, "unsupported depth");
  if( src_width < 1 || src_height < 1 || dst_width < 1 || dst_height < 1 ) return fail(SST_ERR_INVALID_ARG, "invalid size");
  if( row_stride < (size_t) src_width * bytes || frame_stride < row_stride * src_height )
    return fail(SST_ERR_INVALID_ARG, "invalid strides");
  if( model->type < 0 || model->type > 7 ) return fail(SST_ERR_INVALID_ARG, "invalid motion type");
  if( border != SST_BORDER_CONSTANT && border != SST_BORDER_REPLICATE && border != SST_BORDER_REFLECT &&
      border != SST_BORDER_REFLECT101 )
    return fail(SST_ERR_UNSUPPORTED, "unsupported border mode");

  float * scratch = nullptr;
  int * wait_flag = nullptr;
  const int r = scratch_address(&scratch, &wait_flag);
  if( r != SST_OK ) return r;
  float * coeffs = scratch;
  float * weff = scratch + (size_t) SST_NOALLOC_MAX_FRAMES * SST_NCOEF;
  cudaStream_t st = (cudaStream_t) stream;

  cudaError_t e = sst::launch_coeffs_from_params(*model, params, n, coeffs, st);
  if( e == cudaSuccess ) e = sst::launch_effective_weights(weights, status, n, weff, st);
  if( e != cudaSuccess ) return fail(SST_ERR_CUDA, cudaGetErrorString(e));
  sst::StackArgs s;
  s.frames = (const uint8_t *) frames;
  s.row_stride = row_stride, s.frame_stride = frame_stride;
  s.sw = src_width, s.sh = src_height, s.n = n;
  s.scale = (float) scale;
  s.coeffs = coeffs;
  s.weights = weff;
  s.dw = dst_width, s.dh = dst_height;
  s.acc = acc_state;
  s.plane = (size_t) dst_width * dst_height;
  s.border = border;
  s.err = wait_flag;
  e = cudaMemsetAsync(wait_flag, 0, sizeof(int), st);
  if( e == cudaSuccess ) e = sst::launch_stack_add_warped(s, model->type, depth, st);
  if( e != cudaSuccess ) return fail(SST_ERR_CUDA, cudaGetErrorString(e));
  int raised = 0;
  e = cudaMemcpyAsync(&raised, wait_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
  if( e == cudaSuccess ) e = cudaStreamSynchronize(st);
  if( e != cudaSuccess ) return fail(SST_ERR_CUDA, cudaGetErrorString(e));
  if( raised ) {
    return fail(SST_ERR_TIMEOUT,
        "the stacking kernel raised its error flag; acc_state is invalid and must be rebuilt");
  }
  return SST_OK;
}
