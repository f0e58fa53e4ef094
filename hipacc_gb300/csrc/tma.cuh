// tma.cuh -- tensor-memory-accelerator (TMA) tile loads with mbarrier
// completion, plus the host-side tensor-map encoder.
//
// A CTA stages halo tiles with cp.async.bulk.tensor (issued by one thread,
// completion signalled on an mbarrier as transaction bytes).  Every wait is
// bounded: after kMaxSpins polls the waiting threads agree through a block
// vote, record HGB_ERR_TIMEOUT in the device status word and leave the
// kernel; no thread traps or spins forever.
#pragma once

#include <cuda.h>

#include "hgb_internal.cuh"

namespace hgb {

// ---------------------------------------------------------------- host
// Encode a 3-D tiled tensor map {width, height, batch} over an image batch.
// Returns HGB_OK, or an error when the layout is not TMA-legal (base not
// 16-byte aligned, pitch / batch stride not multiples of 16) -- callers then
// use their non-TMA path.
int make_tensor_map_3d(CUtensorMap *map, CUtensorMapDataType dt, int elem_size, const void *base, int width,
                       int height, int batch, int64_t pitch, int64_t bstride, int box_w, int box_h);
bool tma_legal(const void *base, int64_t pitch, int64_t bstride, int batch);
// device status word (HGB_OK or an error code recorded by a kernel)
int *device_status_word();

// ---------------------------------------------------------------- device
constexpr long long kMaxSpins = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait (at most `limit` polls); returns false on timeout (the caller
// votes and leaves)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, long long limit = kMaxSpins) {
  for (long long i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// One thread waits (bounded) for the barrier's phase and the CTA barrier that
// follows orders its acquire before every thread's reads of the landed bytes;
// the other threads sleep at the CTA barrier instead of polling the mbarrier
// (polling warps take issue slots from the CTAs that have work).  Same result
// on every thread: false when the wait expired.
__device__ __forceinline__ bool cta_wait(uint64_t *bar, unsigned parity, long long limit = kMaxSpins) {
  int late = 0;
  if (threadIdx.x == 0) late = !mbar_wait(bar, parity, limit);
  return !__syncthreads_or(late);
}

// order earlier generic-proxy accesses of shared memory before async-proxy
// (TMA) writes into it
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void record_status(int *status, int code) {
  if (status) atomicExch(status, code);
}

}  // namespace hgb
