// runtime.cu -- status codes, timing, workspace and image memory.
//
// Replaces the host runtime of the reference's CUDA back end
// (runtime/hipacc_cu.hpp, runtime/hipacc_cu.tpp, runtime/hipacc_cu_standalone.hpp)
// with explicit status codes instead of log-and-continue (checkErr,
// runtime/hipacc_base.hpp:112-129) and a reused per-device workspace instead
// of per-call cudaMalloc/cudaFree (runtime/hipacc_cu.tpp:331-391).
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "hgb_internal.cuh"

namespace hgb {

namespace {
thread_local std::string t_last_error;
thread_local float t_last_timing_ms = 0.0f;
bool g_timing = false;

struct DeviceState {
  Workspace ws;
  int sms = 0;
};
std::mutex g_mu;
std::vector<DeviceState> g_dev;

DeviceState &dev_state(int dev) {
  if ((int)g_dev.size() <= dev) g_dev.resize(dev + 1);
  return g_dev[dev];
}
}  // namespace

int set_error(int status, const std::string &msg) {
  t_last_error = msg;
  return status;
}

int cuda_error(cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return set_error(e == cudaErrorMemoryAllocation ? HGB_ERR_ALLOC : HGB_ERR_CUDA, m);
}

cudaEvent_t before_launch(cudaStream_t stream) {
  if (!g_timing) return nullptr;
  cudaEvent_t ev = nullptr;
  if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
  cudaEventRecord(ev, stream);
  return ev;
}

int after_launch(const char *kernel, cudaStream_t stream, cudaEvent_t start) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    if (start) cudaEventDestroy(start);
    return cuda_error(e, kernel);
  }
  if (start) {
    cudaEvent_t stop;
    cudaEventCreate(&stop);
    cudaEventRecord(stop, stream);
    e = cudaEventSynchronize(stop);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, start, stop);
    t_last_timing_ms = ms;
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    if (e != cudaSuccess) return cuda_error(e, kernel);
  }
  return HGB_OK;
}

int workspace_get(size_t bytes, Workspace *ws) {
  int dev = 0;
  HGB_CHECK_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState &st = dev_state(dev);
  if (!st.ws.tickets) {
    // accumulators first (8-byte aligned), tickets behind them
    void *t = nullptr;
    const size_t nb = kAcc * sizeof(unsigned long long) + kTickets * sizeof(unsigned int);
    HGB_CHECK_CUDA(cudaMalloc(&t, nb));
    HGB_CHECK_CUDA(cudaMemset(t, 0, nb));
    HGB_CHECK_CUDA(cudaDeviceSynchronize());
    st.ws.acc = (unsigned long long *)t;
    st.ws.tickets = (unsigned int *)((char *)t + kAcc * sizeof(unsigned long long));
  }
  if (st.ws.bytes < bytes) {
    // Growing replaces the buffer: wait for every stream of the device that
    // may still use the old one.
    if (st.ws.base) {
      HGB_CHECK_CUDA(cudaDeviceSynchronize());
      cudaFree(st.ws.base);
      st.ws.base = nullptr;
      st.ws.bytes = 0;
    }
    size_t nb = 1 << 20;
    while (nb < bytes) nb <<= 1;
    void *p = nullptr;
    HGB_CHECK_CUDA(cudaMalloc(&p, nb));
    st.ws.base = p;
    st.ws.bytes = nb;
  }
  *ws = st.ws;
  return HGB_OK;
}

int ensure_dynamic_smem(const void *kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> done;
  int dev = 0;
  HGB_CHECK_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t &have = done[{dev, kernel}];
  if (have >= bytes) return HGB_OK;
  HGB_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  have = bytes;
  return HGB_OK;
}

int resident_ctas(const void *kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<int, const void *, int, size_t>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_tuple(dev, kernel, threads, smem);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) n = 1;
  cache[key] = n;
  return n;
}

int num_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState &st = dev_state(dev);
  if (!st.sms) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    st.sms = v > 0 ? v : 148;
  }
  return st.sms;
}

int check_view(const hgb_view *v, const char *name) {
  if (!v) return set_error(HGB_ERR_INVALID, std::string(name) + ": null view");
  if (!v->data) return set_error(HGB_ERR_INVALID, std::string(name) + ": null data pointer");
  const int es = dtype_size(v->dtype);
  if (es == 0) return set_error(HGB_ERR_INVALID, std::string(name) + ": unknown dtype");
  if (v->width <= 0 || v->height <= 0 || v->batch <= 0)
    return set_error(HGB_ERR_INVALID, std::string(name) + ": empty or negative size");
  if (v->pitch < (int64_t)v->width * es)
    return set_error(HGB_ERR_INVALID, std::string(name) + ": pitch smaller than a row");
  if (v->batch > 1 && v->batch_stride < v->pitch * v->height)
    return set_error(HGB_ERR_INVALID, std::string(name) + ": batch_stride smaller than an image");
  if (((uintptr_t)v->data) % es != 0 || v->pitch % es != 0)
    return set_error(HGB_ERR_INVALID, std::string(name) + ": misaligned data or pitch");
  return HGB_OK;
}

int check_window(const hgb_window &w, const hgb_view &v, const char *name) {
  if (w.width <= 0 || w.height <= 0 || w.offset_x < 0 || w.offset_y < 0 || w.offset_x + w.width > v.width ||
      w.offset_y + w.height > v.height)
    return set_error(HGB_ERR_INVALID, std::string(name) + ": window outside the image");
  return HGB_OK;
}

}  // namespace hgb

using namespace hgb;

struct hgb_image {
  hgb_view view;
  int alignment;
};

extern "C" {

int hgb_abi_version(void) { return HGB_ABI_VERSION; }

const char *hgb_last_error(void) { return t_last_error.c_str(); }

int hgb_init(int device, char *name, size_t name_len) {
  int n = 0;
  HGB_CHECK_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return set_error(HGB_ERR_INVALID, "hgb_init: no such device");
  HGB_CHECK_CUDA(cudaSetDevice(device));
  HGB_CHECK_CUDA(cudaFree(nullptr));  // create the primary context
  if (name && name_len) {
    cudaDeviceProp p;
    HGB_CHECK_CUDA(cudaGetDeviceProperties(&p, device));
    snprintf(name, name_len, "%s (sm_%d%d, %d SMs)", p.name, p.major, p.minor, p.multiProcessorCount);
  }
  return HGB_OK;
}

int hgb_set_timing(int on) {
  g_timing = on != 0;
  return HGB_OK;
}

float hgb_last_kernel_timing(void) { return t_last_timing_ms; }

int hgb_workspace_reserve(size_t bytes) {
  Workspace ws;
  return workspace_get(bytes, &ws);
}

int hgb_image_create(int dtype, int width, int height, int alignment, const void *host_init, hgb_image **out) {
  HGB_REQUIRE(out, "hgb_image_create: null out");
  const int es = dtype_size(dtype);
  HGB_REQUIRE(es > 0, "hgb_image_create: unknown dtype");
  HGB_REQUIRE(width > 0 && height > 0, "hgb_image_create: empty image");
  if (alignment <= 0) alignment = 256;
  // hipaccCreateMemory: stride rounded up to the alignment (runtime/hipacc_cu.tpp:50-68)
  alignment = (alignment + es - 1) / es * es;
  int64_t pitch = ((int64_t)width * es + alignment - 1) / alignment * alignment;
  void *p = nullptr;
  HGB_CHECK_CUDA(cudaMalloc(&p, (size_t)pitch * height));
  hgb_image *img = new hgb_image;
  img->view.data = p;
  img->view.dtype = dtype;
  img->view.width = width;
  img->view.height = height;
  img->view.batch = 1;
  img->view.pitch = pitch;
  img->view.batch_stride = pitch * height;
  img->alignment = alignment;
  if (host_init) {
    cudaError_t e = cudaMemcpy2D(p, pitch, host_init, (size_t)width * es, (size_t)width * es, height,
                                 cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(p);
      delete img;
      return cuda_error(e, "hgb_image_create: write");
    }
  } else {
    cudaMemset(p, 0, (size_t)pitch * height);
  }
  *out = img;
  return HGB_OK;
}

int hgb_image_destroy(hgb_image *img) {
  if (!img) return HGB_OK;
  cudaError_t e = cudaFree(img->view.data);
  delete img;
  if (e != cudaSuccess) return cuda_error(e, "hgb_image_destroy");
  return HGB_OK;
}

int hgb_image_get_view(const hgb_image *img, hgb_view *out) {
  HGB_REQUIRE(img && out, "hgb_image_get_view: null argument");
  *out = img->view;
  return HGB_OK;
}

int hgb_image_write(hgb_image *img, const void *host, void *stream) {
  HGB_REQUIRE(img && host, "hgb_image_write: null argument");
  const hgb_view &v = img->view;
  const size_t row = (size_t)v.width * dtype_size(v.dtype);
  HGB_CHECK_CUDA(cudaMemcpy2DAsync(v.data, v.pitch, host, row, row, v.height, cudaMemcpyHostToDevice,
                                   (cudaStream_t)stream));
  return HGB_OK;
}

int hgb_image_read(const hgb_image *img, void *host, void *stream) {
  HGB_REQUIRE(img && host, "hgb_image_read: null argument");
  const hgb_view &v = img->view;
  const size_t row = (size_t)v.width * dtype_size(v.dtype);
  HGB_CHECK_CUDA(cudaMemcpy2DAsync(host, row, v.data, v.pitch, row, v.height, cudaMemcpyDeviceToHost,
                                   (cudaStream_t)stream));
  HGB_CHECK_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return HGB_OK;
}

int hgb_image_read_async(const hgb_image *img, void *host, void *stream) {
  HGB_REQUIRE(img && host, "hgb_image_read_async: null argument");
  const hgb_view &v = img->view;
  const size_t row = (size_t)v.width * dtype_size(v.dtype);
  HGB_CHECK_CUDA(cudaMemcpy2DAsync(host, row, v.data, v.pitch, row, v.height, cudaMemcpyDeviceToHost,
                                   (cudaStream_t)stream));
  return HGB_OK;
}

int hgb_stream_create(void **stream) {
  HGB_REQUIRE(stream, "hgb_stream_create: null argument");
  cudaStream_t s = nullptr;
  HGB_CHECK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = s;
  return HGB_OK;
}

int hgb_stream_destroy(void *stream) {
  if (!stream) return HGB_OK;
  HGB_CHECK_CUDA(cudaStreamDestroy((cudaStream_t)stream));
  return HGB_OK;
}

int hgb_stream_synchronize(void *stream) {
  HGB_CHECK_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return HGB_OK;
}

int hgb_stream_wait(void *waiter, void *signaller) {
  cudaEvent_t e = nullptr;
  HGB_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaError_t err = cudaEventRecord(e, (cudaStream_t)signaller);
  if (err == cudaSuccess) err = cudaStreamWaitEvent((cudaStream_t)waiter, e, 0);
  cudaEventDestroy(e);  // released once the recorded work completes
  if (err != cudaSuccess) return cuda_error(err, "hgb_stream_wait");
  return HGB_OK;
}

int hgb_graph_begin(void *stream) {
  HGB_REQUIRE(stream, "hgb_graph_begin: the legacy default stream cannot be recorded");
  HGB_CHECK_CUDA(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
  return HGB_OK;
}

int hgb_graph_end(void *stream, hgb_graph **out) {
  HGB_REQUIRE(stream && out, "hgb_graph_end: null argument");
  cudaGraph_t g = nullptr;
  HGB_CHECK_CUDA(cudaStreamEndCapture((cudaStream_t)stream, &g));
  cudaGraphExec_t x = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_error(e, "hgb_graph_end: instantiate");
  *out = reinterpret_cast<hgb_graph *>(x);
  return HGB_OK;
}

int hgb_graph_launch(const hgb_graph *graph, void *stream) {
  HGB_REQUIRE(graph, "hgb_graph_launch: null graph");
  HGB_CHECK_CUDA(cudaGraphLaunch((cudaGraphExec_t)graph, (cudaStream_t)stream));
  return HGB_OK;
}

int hgb_graph_destroy(hgb_graph *graph) {
  if (!graph) return HGB_OK;
  HGB_CHECK_CUDA(cudaGraphExecDestroy((cudaGraphExec_t)graph));
  return HGB_OK;
}

int hgb_image_copy(const hgb_image *src, hgb_image *dst, void *stream) {
  HGB_REQUIRE(src && dst, "hgb_image_copy: null argument");
  HGB_REQUIRE(src->view.width == dst->view.width && src->view.height == dst->view.height &&
                  src->view.dtype == dst->view.dtype,
              "hgb_image_copy: images differ in size or type");
  const size_t row = (size_t)src->view.width * dtype_size(src->view.dtype);
  HGB_CHECK_CUDA(cudaMemcpy2DAsync(dst->view.data, dst->view.pitch, src->view.data, src->view.pitch, row,
                                   src->view.height, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return HGB_OK;
}

int hgb_image_copy_region(const hgb_image *src, const hgb_window *src_win, hgb_image *dst,
                          const hgb_window *dst_win, void *stream) {
  HGB_REQUIRE(src && dst, "hgb_image_copy_region: null argument");
  HGB_REQUIRE(src->view.dtype == dst->view.dtype, "hgb_image_copy_region: dtype mismatch");
  hgb_window sw = window_or_full(src_win, src->view), dw = window_or_full(dst_win, dst->view);
  int rc = check_window(sw, src->view, "src_win");
  if (rc) return rc;
  rc = check_window(dw, dst->view, "dst_win");
  if (rc) return rc;
  HGB_REQUIRE(sw.width == dw.width && sw.height == dw.height, "hgb_image_copy_region: window sizes differ");
  const int es = dtype_size(src->view.dtype);
  const char *s = (const char *)src->view.data + sw.offset_y * src->view.pitch + (int64_t)sw.offset_x * es;
  char *d = (char *)dst->view.data + dw.offset_y * dst->view.pitch + (int64_t)dw.offset_x * es;
  HGB_CHECK_CUDA(cudaMemcpy2DAsync(d, dst->view.pitch, s, src->view.pitch, (size_t)sw.width * es, sw.height,
                                   cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return HGB_OK;
}

}  // extern "C"
