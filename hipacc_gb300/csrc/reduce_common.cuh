// reduce_common.cuh -- block / grid combine helpers for single-pass reductions.
//
// The reference's single-pass reduction (runtime/hipacc_cu_red.hpp:140-346)
// takes an atomicInc ticket without a fence and relies on pre-Volta
// warp-synchronous code.  Here: warp shuffles (or redux.sync) inside a warp,
// shared memory across warps, one partial per block in the workspace, then a
// release fence + ticket; the block that takes the last ticket reads all
// partials with L1-bypassing loads (acquire side) in block order, so results
// are deterministic, and resets the ticket for the next launch.
#pragma once

#include "hgb_internal.cuh"

namespace hgb {

__device__ __forceinline__ unsigned int grid_blocks() { return gridDim.x * gridDim.y * gridDim.z; }
__device__ __forceinline__ unsigned int block_rank() {
  return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
}

// Call after thread 0 stored this block's partial.  Returns true (in all
// threads of the block) in the block that must combine.
__device__ __forceinline__ unsigned int ticket_acq_rel(unsigned int *t);
__device__ __forceinline__ bool take_last_ticket(unsigned int *ticket) {
  __shared__ bool s_last;
  __syncthreads();
  // thread 0 stored the block's partial; its acq_rel ticket releases it, and
  // in the last block acquires every other block's partial.  The barrier then
  // orders the other threads' reads of the partials after that acquire.
  if (threadIdx.x == 0) s_last = (ticket_acq_rel(ticket) == grid_blocks() - 1);
  __syncthreads();
  return s_last;
}

__device__ __forceinline__ void release_ticket(unsigned int *ticket) {
  if (threadIdx.x == 0) *ticket = 0u;
}

// Ticket increment with acquire-release semantics at GPU scope: it releases
// this thread's earlier (relaxed) accumulator atomics and, in the last CTA,
// acquires everyone's.
__device__ __forceinline__ unsigned int ticket_acq_rel(unsigned int *t) {
  unsigned int old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(t) : "memory");
  return old;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Single-pass integer reduction epilogue without a combine loop: thread 0 of
// every CTA folds its block value into the accumulators with relaxed atomics
// (no return value, so they issue as reductions) and takes the ticket; the CTA
// that takes the last ticket copies the accumulators out and zeroes them and
// the ticket for the next launch.  Only one atomic round trip per CTA.
__device__ __forceinline__ void accumulate_and_publish(unsigned long long *acc_sum, unsigned long long *acc_max,
                                                       unsigned int *ticket, unsigned long long bsum,
                                                       unsigned long long bmax, uint64_t *sum_dev,
                                                       uint32_t *max_dev) {
  if (threadIdx.x != 0) return;
  if (bsum) atomicAdd(acc_sum, bsum);
  if (bmax) atomicMax(acc_max, bmax);
  if (ticket_acq_rel(ticket) == grid_blocks() - 1) {
    const unsigned long long s = ld_relaxed_u64(acc_sum), m = ld_relaxed_u64(acc_max);
    if (sum_dev) *sum_dev = s;
    if (max_dev) *max_dev = (uint32_t)m;
    *acc_sum = 0ull;
    *acc_max = 0ull;
    *ticket = 0u;
  }
}

template <typename T>
__device__ __forceinline__ T shfl_down(T v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}

// two-sum of Kahan pairs (s, c): value = s + c
struct Kahan {
  float s, c;
};
__device__ __forceinline__ Kahan kahan_add(Kahan a, float x) {
  const float y = x - a.c;
  const float t = a.s + y;
  a.c = (t - a.s) - y;
  a.s = t;
  return a;
}
__device__ __forceinline__ Kahan kahan_merge(Kahan a, Kahan b) {
  // a.s + b.s exactly as s + e (Knuth two-sum), compensations folded into e
  const float s = a.s + b.s;
  const float bp = s - a.s;
  const float e = (a.s - (s - bp)) + (b.s - bp);
  Kahan r;
  r.s = s;
  r.c = -(e - a.c - b.c);  // stored as negative correction, value = s - c
  return r;
}

}  // namespace hgb
