// reduce_noalloc.cu -- hgb_reduce_noalloc: the global reduction of hgb_reduce
// for callers that cannot allocate device memory.
//
// hgb_reduce keeps its scratch (per-block partials, the last-block ticket, the
// integer accumulator, a result slot) in a per-device workspace that the
// library grows with cudaMalloc on first use.  Some callers cannot allow that:
// real-time frame loops that must never block in the CUDA allocator, and
// plug-ins inside a host program whose device memory is owned by the host's
// own allocator with a fixed budget.  This variant uses a fixed array in the
// library's own device memory instead and calls no allocating routine.
//
// Scratch: g_noalloc_scratch, a file-scope __device__ array of
// kNoAllocBytes (16 KiB of partials for up to kNoAllocMaxBlocks = 1024 blocks
// plus 256 bytes of control words).  Every GPU that loads the library holds it
// until the process exits.  A call whose launch would need more blocks is
// rejected with HGB_ERR_LIMIT (on a GB300 a launch uses at most SMs x 4 = 608).
//
// Every call shares the array and it keeps the last call's contents: each call
// clears the ticket and the accumulator with an ordered cudaMemsetAsync on its
// stream before the kernel.  Calls that overlap on the GPU (different streams
// without an ordering between them) race on the array.
//
// Set-up: host code cannot use the array's name as a device address (it is a
// host-side stand-in).  The first call on a device, with that device current,
// resolves the address once with cudaGetSymbolAddress and caches it per
// device.
#include <mutex>

#include "reduce_kernels.cuh"

namespace hgb {
namespace {

constexpr int kNoAllocMaxBlocks = 1024;
constexpr size_t kNoAllocPartialBytes = (size_t)kNoAllocMaxBlocks * 16;
constexpr size_t kNoAllocBytes = kNoAllocPartialBytes + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

int noalloc_scratch(void **ptr) {
  int dev = 0;
  HGB_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(HGB_ERR_LIMIT, "hgb_reduce_noalloc: device index too large");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "hgb_reduce_noalloc: cudaGetSymbolAddress");
    g_noalloc_ptr[dev] = p;
  }
  *ptr = g_noalloc_ptr[dev];
  return HGB_OK;
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_reduce_noalloc(const hgb_view *in, const hgb_window *winp, int op, void *result_dev,
                                  void *result_host, void *stream) {
  HGB_REQUIRE(result_dev || result_host, "hgb_reduce_noalloc: no result destination");
  RedParams p;
  int grid = 0;
  int rc = reduce_setup(in, winp, op, &p, &grid);
  if (rc) return rc;
  if (grid > kNoAllocMaxBlocks)
    return set_error(HGB_ERR_LIMIT, "hgb_reduce_noalloc: launch needs " + std::to_string(grid) +
                                        " block partials, the fixed scratch holds " +
                                        std::to_string(kNoAllocMaxBlocks));
  void *base = nullptr;
  rc = noalloc_scratch(&base);
  if (rc) return rc;
  char *ctrl = (char *)base + kNoAllocPartialBytes;  // acc (8 B), ticket (4 B), result slot at +16
  p.partials = base;
  p.acc = (unsigned long long *)ctrl;
  p.ticket = (unsigned int *)(ctrl + 8);
  p.result_dev = result_dev ? (unsigned long long *)result_dev : (unsigned long long *)(ctrl + 16);
  cudaStream_t st = (cudaStream_t)stream;
  HGB_CHECK_CUDA(cudaMemsetAsync(ctrl, 0, 16, st));
  rc = reduce_launch(in->dtype, op, p, grid, st);
  if (rc) return rc;
  if (result_host) {
    HGB_CHECK_CUDA(cudaMemcpyAsync(result_host, p.result_dev, 8, cudaMemcpyDeviceToHost, st));
    HGB_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return HGB_OK;
}
