/*
 * sst_tma.cuh -- tensor-memory-accelerator tile copies into shared memory,
 * completed on mbarriers, with bounded waits.
 *
 * Rules kept by every caller: the innermost coordinate of a tile copy times
 * the element size is a multiple of 16 bytes; the destination is 128-byte
 * aligned; the expected transaction bytes equal the whole box (out-of-range
 * elements are filled); every wait gives up after a fixed number of polls
 * and the kernel reports it instead of hanging.
 */
#pragma once
#include <cuda.h>            // CUtensorMap; the encoder is fetched through the runtime
#include <cuda_runtime.h>
#include <stdint.h>

namespace sst {

/* shared-memory address of a generic pointer into shared memory */
__device__ __forceinline__ uint32_t smem_u32(const void * p)
{
  return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t * bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t * bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t * bar, uint32_t parity)
{
  uint32_t done;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return done != 0;
}

/* bounded wait: gives up after a fixed number of polls (each poll may
 * suspend the thread for a short time) and reports it */
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t * bar, uint32_t parity)
{
  for( int i = 0; i < (1 << 20); ++i )
    if( mbar_try_wait(bar, parity) ) return true;
  return false;
}

/* Copies of a CTA's multi-buffer (up to 8 buffers) that the issuing thread
 * started and has not seen land, kept in one shared word by that thread
 * alone: bit b = a copy into buffer b is outstanding, bit 8 + b = the barrier
 * parity it completes. A CTA that gave up on a wait drains them (bounded
 * again) before it exits, so no copy writes into the shared memory of a
 * finished CTA. */
__device__ __forceinline__ void inflight_issued(uint32_t * w, int b, uint32_t parity)
{
  *w = (*w & ~(0x101u << b)) | (1u << b) | (parity << (b + 8));
}

__device__ __forceinline__ void inflight_landed(uint32_t * w, int b)
{
  *w &= ~(1u << b);
}

__device__ __forceinline__ void inflight_drain(uint32_t * w, uint64_t * bars, int nbuf = 2)
{
  for( int b = 0; b < nbuf; ++b )
    if( (*w >> b) & 1u ) mbar_wait_bounded(&bars[b], (*w >> (b + 8)) & 1u);
  *w = 0u;
}

/* 3-D tile copy (x, y, frame) of the tensor map into shared memory, completion on bar */
__device__ __forceinline__ void tma_load_3d(void * dst, const CUtensorMap * map, int x, int y, int z, uint64_t * bar)
{
  asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
               :: "r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
               : "memory");
}

/* cuTensorMapEncodeTiled of a 3-D tensor (x, y, z) with strides in bytes;
 * false when unavailable or when the layout breaks the TMA alignment rules */
bool encode_tensor_3d(CUtensorMap * map, CUtensorMapDataType dt, int esz, const void * base, const uint64_t * dims,
    const uint64_t * strides, const uint32_t * box);

}  // namespace sst
