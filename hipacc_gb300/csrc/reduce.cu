// reduce.cu -- hgb_reduce: single-pass global reductions (kernels in
// reduce_kernels.cuh) with the per-device library workspace as scratch.
#include "reduce_kernels.cuh"

using namespace hgb;

extern "C" int hgb_reduce(const hgb_view *in, const hgb_window *winp, int op, void *result_dev, void *result_host,
                          void *stream) {
  HGB_REQUIRE(result_dev || result_host, "hgb_reduce: no result destination");
  RedParams p;
  int grid = 0;
  int rc = reduce_setup(in, winp, op, &p, &grid);
  if (rc) return rc;
  Workspace ws;
  rc = workspace_get((size_t)grid * 16 + 64, &ws);
  if (rc) return rc;
  p.partials = ws.base;
  // the 8-byte result slot sits behind the partials when no device result is given
  unsigned long long *slot = (unsigned long long *)((char *)ws.base + (size_t)grid * 16);
  p.result_dev = result_dev ? (unsigned long long *)result_dev : slot;
  p.ticket = ws.tickets + 1;
  p.acc = ws.acc + kSlotReduce;
  cudaStream_t st = (cudaStream_t)stream;
  rc = reduce_launch(in->dtype, op, p, grid, st);
  if (rc) return rc;
  if (result_host) {
    HGB_CHECK_CUDA(cudaMemcpyAsync(result_host, p.result_dev, 8, cudaMemcpyDeviceToHost, st));
    HGB_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return HGB_OK;
}
