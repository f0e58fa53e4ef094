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
__device__ __forceinline__ bool take_last_ticket(unsigned int *ticket) {
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    s_last = (t == grid_blocks() - 1);
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

__device__ __forceinline__ void release_ticket(unsigned int *ticket) {
  if (threadIdx.x == 0) *ticket = 0u;
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
