// tma.cu -- host side of the TMA helpers: tensor-map encoding through the
// driver entry point (no link-time dependency on libcuda) and the device
// status word.
#include <cudaTypedefs.h>

#include <mutex>

#include "tma.cuh"

namespace hgb {

namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_once;

void resolve() {
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
}
}  // namespace

bool tma_legal(const void *base, int64_t pitch, int64_t bstride, int batch) {
  return ((uintptr_t)base % 16 == 0) && (pitch % 16 == 0) && (batch == 1 || bstride % 16 == 0);
}

int make_tensor_map_3d(CUtensorMap *map, CUtensorMapDataType dt, int elem_size, const void *base, int width,
                       int height, int batch, int64_t pitch, int64_t bstride, int box_w, int box_h) {
  std::call_once(g_once, resolve);
  if (!g_encode) return set_error(HGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  if (!tma_legal(base, pitch, bstride, batch)) return set_error(HGB_ERR_UNSUPPORTED, "layout not TMA-legal");
  cuuint64_t dims[3] = {(cuuint64_t)width, (cuuint64_t)height, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)pitch, (cuuint64_t)(batch > 1 ? bstride : pitch * height)};
  cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1u};
  cuuint32_t estr[3] = {1u, 1u, 1u};
  (void)elem_size;
  CUresult r = g_encode(map, dt, 3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(HGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled failed");
  return HGB_OK;
}

int *device_status_word() {
  Workspace ws;
  if (workspace_get(0, &ws) != HGB_OK) return nullptr;
  return reinterpret_cast<int *>(ws.tickets + (kTickets - 1));
}

}  // namespace hgb

using namespace hgb;

// Read (and clear) the device status word: HGB_OK, or the error a kernel
// recorded (HGB_ERR_TIMEOUT for an expired bounded wait).  Synchronises the
// device.
extern "C" HGB_API int hgb_device_status(int *status) {
  HGB_REQUIRE(status, "hgb_device_status: null argument");
  int *w = device_status_word();
  if (!w) return HGB_ERR_CUDA;
  HGB_CHECK_CUDA(cudaDeviceSynchronize());
  int v = 0;
  HGB_CHECK_CUDA(cudaMemcpy(&v, w, sizeof(int), cudaMemcpyDeviceToHost));
  const int zero = 0;
  HGB_CHECK_CUDA(cudaMemcpy(w, &zero, sizeof(int), cudaMemcpyHostToDevice));
  *status = v;
  return HGB_OK;
}
