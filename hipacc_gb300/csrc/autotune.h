// autotune.h -- per-shape choice of kernel tile configuration.
//
// The reference fixes block shape and pixels-per-thread at compile time from
// per-device tables (include/hipacc/Device/TargetDescription.h:53-191) or the
// -use-config / -pixels-per-thread switches.  Here each operator has a small
// set of tile configurations; the first call for a (operator, dtype, shape,
// size class) key with autotuning on times every configuration with CUDA
// events and keeps the fastest.  Choices can be saved to and loaded from a
// JSON file.  While a stream is being captured nothing is timed: the stored
// choice (or configuration 0) is used.
#pragma once

#include <cuda_runtime.h>

#include "hgb_internal.cuh"

namespace hgb {

bool autotune_enabled();
int autotune_lookup(const char *key);  // -1 when unknown
void autotune_store(const char *key, int cfg, float ms);

template <typename F>
int autotune_run(const char *key, int ncfg, cudaStream_t st, F &&launch) {
  int cfg = autotune_lookup(key);
  if (cfg >= 0 && cfg < ncfg) return launch(cfg);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  if (!autotune_enabled() || ncfg <= 1 || cs != cudaStreamCaptureStatusNone) return launch(0);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = 0;
  float best_ms = 3.0e38f;
  for (int c = 0; c < ncfg; ++c) {
    int rc = launch(c);  // warm-up, also surfaces launch errors
    if (rc != HGB_OK) continue;
    cudaEventRecord(e0, st);
    for (int r = 0; r < 3; ++r) launch(c);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  autotune_store(key, best, best_ms / 3.0f);
  return launch(best);
}

}  // namespace hgb
