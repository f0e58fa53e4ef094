// hipacc.hpp -- C++ host surface of libhipacc_gb300 in the shape of Hipacc's
// DSL and CUDA runtime (dsl/hipacc.hpp, dsl/image.hpp, dsl/mask.hpp,
// dsl/iterationspace.hpp, dsl/kernel.hpp, dsl/pyramid.hpp,
// runtime/hipacc_cu.hpp, runtime/hipacc_base.hpp).
//
// A Hipacc program declares Images, BoundaryConditions, Accessors, Masks /
// Domains and IterationSpaces, and runs Kernel objects with execute() and
// reduced_data().  Hipacc's compiler turns each user Kernel subclass into a
// generated CUDA kernel; without that compiler, this header provides the
// operator families of the hot path as ready Kernel classes that keep the
// reference's constructor arguments and member calls and run the
// hand-written sm_103a kernels of libhipacc_gb300.so through its C ABI
// (include/hipacc_gb300.h):
//   Convolution<T>      Kernel::convolve(Mask, Reduce, mask()*input(mask));
//                       T = uchar writes (uchar)(result + 0.5f), saturated
//   DomainReduce<T>     Kernel::reduce(Domain, Reduce, input(dom))
//   Separable<T>        the 1xK + Kx1 pair of convolutions, fused
//   BilateralFilter<T>  the bilateral sample's iterate(Domain, ...) body
//   SobelMagnitude      min(|reduce(dx)| + |reduce(dy)|, 255), u8, with the
//                       sum / max of the result fused (reduced_data)
//   ColorConversion     uchar4 -> uchar weighted sum >> shift
//   Copy<T>             output() = input() (NN / LF accessors resample)
//   Difference<T>       output() = input1() - input2() (input2 may be LF)
//   Reduction<T>        output() = input(); reduced_data() with Reduce
// Images live in device memory (pitched, hipaccCreateMemory) with a host
// mirror that Image::data() refreshes (hipaccReadMemory semantics).
// Every failing library call throws hipacc::Error with the library message.
#ifndef HIPACC_GB300_HIPACC_HPP
#define HIPACC_GB300_HIPACC_HPP

#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <type_traits>
#include <string>
#include <vector>

#include "../hipacc_gb300.h"

namespace hipacc {

typedef unsigned char uchar;
struct uchar4 {
  uchar x, y, z, w;
};

enum class Boundary : uint8_t { UNDEFINED = 0, CLAMP, REPEAT, MIRROR, CONSTANT };  // dsl/image.hpp:46-52
enum class Interpolate : uint8_t { NO = 0, NN, LF, B5, CF, L3 };                    // dsl/image.hpp:54-61
enum class Reduce : uint8_t { SUM = 0, MIN, MAX, PROD, MEDIAN };                    // dsl/kernel.hpp:48-54

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(int status, const char *what) {
  if (status != HGB_OK) throw Error(status, std::string(what) + ": " + hgb_last_error());
}

// ---------------------------------------------------------------- runtime
// hipaccInitCUDA (runtime/hipacc_cu_standalone.hpp:113-163)
inline std::string hipaccInitCUDA(int device = 0) {
  char name[256] = {0};
  check(hgb_init(device, name, sizeof(name)), "hipaccInitCUDA");
  return name;
}
// -time-kernels (runtime/hipacc_cu_standalone.hpp:297-326) and
// hipacc_last_kernel_timing (runtime/hipacc_base.hpp:64-66)
inline void hipaccEnableTiming(bool on) { check(hgb_set_timing(on ? 1 : 0), "hipaccEnableTiming"); }
inline float hipacc_last_kernel_timing() { return hgb_last_kernel_timing(); }

// The stream every call below is queued on (the stream of an
// ExecutionParameter, runtime/hipacc_cu_standalone.hpp:293-295); nullptr is
// the legacy default stream.  Per thread.
inline void *&current_stream() {
  static thread_local void *s = nullptr;
  return s;
}
inline void hipaccSetStream(void *stream) { current_stream() = stream; }

// A stream owned by the library (for hosts compiled without the CUDA headers).
class Stream {
 public:
  Stream() { check(hgb_stream_create(&s_), "hgb_stream_create"); }
  ~Stream() { hgb_stream_destroy(s_); }
  Stream(const Stream &) = delete;
  Stream &operator=(const Stream &) = delete;
  void *get() const { return s_; }
  void synchronize() const { check(hgb_stream_synchronize(s_), "hgb_stream_synchronize"); }
  // this stream waits for the work queued so far on `other` (fork / join)
  void wait(const Stream &other) const { check(hgb_stream_wait(s_, other.s_), "hgb_stream_wait"); }

 private:
  void *s_ = nullptr;
};

// Whole-program graph (Hipacc's CUDA-graph mode, hipaccLaunchKernelCudaGraph,
// runtime/hipacc_cu_standalone.hpp:331-356): between begin() and end() the
// kernels executed on this thread are recorded on the graph's stream instead of
// running; launch() replays them all with one launch.  Only device work can be
// recorded: read images back (Image::data(), reduced_data()) after launch().
class CudaGraph {
 public:
  CudaGraph() = default;
  ~CudaGraph() { hgb_graph_destroy(g_); }
  CudaGraph(const CudaGraph &) = delete;
  CudaGraph &operator=(const CudaGraph &) = delete;
  void begin() {
    saved_ = current_stream();
    current_stream() = stream_.get();
    check(hgb_graph_begin(stream_.get()), "CudaGraph::begin");
  }
  void end() {
    hgb_graph *g = nullptr;
    const int st = hgb_graph_end(stream_.get(), &g);
    current_stream() = saved_;
    check(st, "CudaGraph::end");
    hgb_graph_destroy(g_);
    g_ = g;
  }
  void launch() { check(hgb_graph_launch(g_, stream_.get()), "CudaGraph::launch"); }
  void synchronize() { stream_.synchronize(); }
  Stream &stream() { return stream_; }

 private:
  Stream stream_;
  hgb_graph *g_ = nullptr;
  void *saved_ = nullptr;
};

template <typename T> struct dtype_of;
template <> struct dtype_of<uchar> { static constexpr int value = HGB_U8; };
template <> struct dtype_of<uchar4> { static constexpr int value = HGB_U8X4; };
template <> struct dtype_of<short> { static constexpr int value = HGB_I16; };
template <> struct dtype_of<unsigned short> { static constexpr int value = HGB_U16; };
template <> struct dtype_of<int> { static constexpr int value = HGB_I32; };
template <> struct dtype_of<unsigned int> { static constexpr int value = HGB_U32; };
template <> struct dtype_of<unsigned long long> { static constexpr int value = HGB_U64; };
template <> struct dtype_of<float> { static constexpr int value = HGB_F32; };
template <> struct dtype_of<double> { static constexpr int value = HGB_F64; };

// ---------------------------------------------------------------- images
// HipaccImageCudaRaw (runtime/hipacc_cu.hpp:113-160): device memory with a
// pitched row layout and a host mirror.
template <typename T>
class Image {
 public:
  Image(int width, int height, const T *init = nullptr) : w_(width), h_(height), host_((size_t)width * height) {
    hgb_image *p = nullptr;
    check(hgb_image_create(dtype_of<T>::value, width, height, 256, init, &p), "hipaccCreateMemory");
    img_.reset(p, [](hgb_image *q) { hgb_image_destroy(q); });
    if (init) std::memcpy(host_.data(), init, sizeof(T) * host_.size());
  }
  int width() const { return w_; }
  int height() const { return h_; }
  // hipaccReadMemory: refresh the host mirror and return it
  T *data() {
    check(hgb_image_read(img_.get(), host_.data(), current_stream()), "hipaccReadMemory");
    return host_.data();
  }
  // hipaccWriteMemory
  Image &operator=(const T *other) {
    check(hgb_image_write(img_.get(), other, current_stream()), "hipaccWriteMemory");
    std::memcpy(host_.data(), other, sizeof(T) * host_.size());
    return *this;
  }
  hgb_view view() const {
    hgb_view v;
    check(hgb_image_get_view(img_.get(), &v), "image view");
    return v;
  }
  hgb_image *handle() const { return img_.get(); }

 private:
  int w_, h_;
  std::shared_ptr<hgb_image> img_;
  std::vector<T> host_;
};

// runtime-level names over the same images (runtime/hipacc_cu.tpp:50-193,
// runtime/hipacc_cu_standalone.hpp:165-216)
template <typename T>
inline std::shared_ptr<Image<T>> hipaccCreateMemory(const T *host, int width, int height) {
  return std::make_shared<Image<T>>(width, height, host);
}
template <typename T>
inline void hipaccWriteMemory(std::shared_ptr<Image<T>> &img, const T *host) {
  *img = host;
}
template <typename T>
inline T *hipaccReadMemory(const std::shared_ptr<Image<T>> &img) {
  return img->data();
}
template <typename T>
inline void hipaccCopyMemory(const std::shared_ptr<Image<T>> &src, std::shared_ptr<Image<T>> &dst) {
  check(hgb_image_copy(src->handle(), dst->handle(), current_stream()), "hipaccCopyMemory");
}

// ---------------------------------------------------------------- masks
class MaskBase {  // dsl/mask.hpp:37-85
 public:
  MaskBase(int sx, int sy) : sx_(sx), sy_(sy), domain_((size_t)sx * sy, 1) {}
  virtual ~MaskBase() {}
  int size_x() const { return sx_; }
  int size_y() const { return sy_; }
  const uint8_t *domain() const { return domain_.data(); }

 protected:
  int sx_, sy_;
  std::vector<uint8_t> domain_;
  friend class Domain;
};

template <typename T>
class Mask : public MaskBase {  // dsl/mask.hpp:231-305: zero coefficients are Domain holes
 public:
  template <int SY, int SX>
  explicit Mask(const T (&m)[SY][SX]) : MaskBase(SX, SY), coef_((size_t)SX * SY) {
    for (int y = 0; y < SY; ++y)
      for (int x = 0; x < SX; ++x) {
        coef_[(size_t)y * SX + x] = m[y][x];
        domain_[(size_t)y * SX + x] = m[y][x] != T(0);
      }
  }
  Mask(int sx, int sy, const T *m) : MaskBase(sx, sy), coef_(m, m + (size_t)sx * sy) {
    for (size_t i = 0; i < coef_.size(); ++i) domain_[i] = coef_[i] != T(0);
  }
  const T *coefficients() const { return coef_.data(); }

 private:
  std::vector<T> coef_;
};

class Domain : public MaskBase {  // dsl/mask.hpp:88-228
 public:
  Domain(int sx, int sy) : MaskBase(sx, sy) {}
  template <int SY, int SX>
  explicit Domain(const uchar (&d)[SY][SX]) : MaskBase(SX, SY) {
    for (int y = 0; y < SY; ++y)
      for (int x = 0; x < SX; ++x) domain_[(size_t)y * SX + x] = d[y][x] != 0;
  }
  explicit Domain(const MaskBase &m) : MaskBase(m.size_x(), m.size_y()) { domain_.assign(m.domain(), m.domain() + (size_t)sx_ * sy_); }
};

// ---------------------------------------------------------------- accessors
template <typename T>
class BoundaryCondition {  // dsl/image.hpp:215-308; the constant is honoured
 public:
  BoundaryCondition(Image<T> &img, int sx, int sy, Boundary mode) : img_(&img), sx_(sx), sy_(sy), mode_(mode) {}
  BoundaryCondition(Image<T> &img, int size, Boundary mode) : BoundaryCondition(img, size, size, mode) {}
  BoundaryCondition(Image<T> &img, const MaskBase &m, Boundary mode) : BoundaryCondition(img, m.size_x(), m.size_y(), mode) {}
  BoundaryCondition(Image<T> &img, int sx, int sy, Boundary mode, T val)
      : img_(&img), sx_(sx), sy_(sy), mode_(mode), const_(val) {}
  BoundaryCondition(Image<T> &img, int size, Boundary mode, T val) : BoundaryCondition(img, size, size, mode, val) {}
  BoundaryCondition(Image<T> &img, const MaskBase &m, Boundary mode, T val)
      : BoundaryCondition(img, m.size_x(), m.size_y(), mode, val) {}
  Image<T> &image() const { return *img_; }
  Boundary mode() const { return mode_; }
  T constant() const { return const_; }

 private:
  Image<T> *img_;
  int sx_, sy_;
  Boundary mode_;
  T const_{};
};

template <typename T>
class Accessor {  // dsl/image.hpp:557-710
 public:
  explicit Accessor(Image<T> &img, Interpolate im = Interpolate::NO)
      : bc_(img, 0, 0, Boundary::CLAMP), win_{0, 0, img.width(), img.height()}, im_(im) {}
  Accessor(Image<T> &img, int w, int h, int xf, int yf, Interpolate im = Interpolate::NO)
      : bc_(img, 0, 0, Boundary::CLAMP), win_{xf, yf, w, h}, im_(im) {}
  explicit Accessor(const BoundaryCondition<T> &bc, Interpolate im = Interpolate::NO)
      : bc_(bc), win_{0, 0, bc.image().width(), bc.image().height()}, im_(im) {}
  Accessor(const BoundaryCondition<T> &bc, int w, int h, int xf, int yf, Interpolate im = Interpolate::NO)
      : bc_(bc), win_{xf, yf, w, h}, im_(im) {}
  Image<T> &image() const { return bc_.image(); }
  const hgb_window &window() const { return win_; }
  Boundary mode() const { return bc_.mode(); }
  T constant() const { return bc_.constant(); }
  Interpolate interpolation() const { return im_; }

 private:
  BoundaryCondition<T> bc_;
  hgb_window win_;
  Interpolate im_;
};

template <typename T>
class IterationSpace {  // dsl/iterationspace.hpp:118-133
 public:
  explicit IterationSpace(Image<T> &img) : img_(&img), win_{0, 0, img.width(), img.height()} {}
  IterationSpace(Image<T> &img, int w, int h) : img_(&img), win_{0, 0, w, h} {}
  IterationSpace(Image<T> &img, int w, int h, int ox, int oy) : img_(&img), win_{ox, oy, w, h} {}
  Image<T> &image() const { return *img_; }
  const hgb_window &window() const { return win_; }

 private:
  Image<T> *img_;
  hgb_window win_;
};

// ---------------------------------------------------------------- kernels
// Kernel<T> (dsl/kernel.hpp:56-238): execute() launches once per object,
// reduced_data() reduces the output image.
template <typename T>
class Kernel {
 public:
  explicit Kernel(IterationSpace<T> &it) : it_(it) {}
  virtual ~Kernel() {}
  void execute() {
    if (!executed_) {
      launch();
      executed_ = true;
    }
  }
  T reduced_data() {
    execute();
    return reduce_output();
  }

 protected:
  virtual void launch() = 0;
  virtual T reduce_output() { throw Error(HGB_ERR_UNSUPPORTED, "this kernel defines no reduction"); }
  hgb_view out_view() const { return it_.image().view(); }
  const hgb_window *out_window() const { return &it_.window(); }
  IterationSpace<T> &it_;
  bool executed_ = false;
};

template <typename T>
inline T reduce_image(const Image<T> &img, const hgb_window &win, Reduce op) {
  hgb_view v = img.view();
  unsigned char raw[8];
  check(hgb_reduce(&v, &win, (int)op, nullptr, raw, current_stream()), "reduced_data");
  if (std::is_floating_point<T>::value) {
    double d;
    std::memcpy(&d, raw, 8);
    return (T)d;
  }
  unsigned long long u;
  std::memcpy(&u, raw, 8);
  return (T)u;
}

// convolve(mask, mode, mask() * input(mask))
template <typename T>
class Convolution : public Kernel<T> {
 public:
  Convolution(IterationSpace<T> &it, Accessor<T> &in, Mask<float> &m, Reduce mode = Reduce::SUM)
      : Kernel<T>(it), in_(in), m_(m), mode_(mode) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    check(hgb_local_op(&iv, &in_.window(), &ov, this->out_window(), m_.coefficients(), nullptr, nullptr, m_.size_x(),
                       m_.size_y(), (int)mode_, (int)in_.mode(), (float)in_.constant(), current_stream()),
          "Convolution::execute");
  }
  Accessor<T> &in_;
  Mask<float> &m_;
  Reduce mode_;
};

// reduce(domain, mode, input(dom))
template <typename T>
class DomainReduce : public Kernel<T> {
 public:
  DomainReduce(IterationSpace<T> &it, Accessor<T> &in, Domain &d, Reduce mode) : Kernel<T>(it), in_(in), d_(d), mode_(mode) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    check(hgb_local_op(&iv, &in_.window(), &ov, this->out_window(), nullptr, nullptr, d_.domain(), d_.size_x(),
                       d_.size_y(), (int)mode_, (int)in_.mode(), (float)in_.constant(), current_stream()),
          "DomainReduce::execute");
  }
  Accessor<T> &in_;
  Domain &d_;
  Reduce mode_;
};

template <typename T>
class Separable : public Kernel<T> {
 public:
  Separable(IterationSpace<T> &it, Accessor<T> &in, std::vector<float> row, std::vector<float> col)
      : Kernel<T>(it), in_(in), row_(std::move(row)), col_(std::move(col)) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    check(hgb_separable(&iv, &ov, row_.data(), col_.data(), (int)row_.size(), (int)in_.mode(), (float)in_.constant(),
                        current_stream()),
          "Separable::execute");
  }
  Accessor<T> &in_;
  std::vector<float> row_, col_;
};

template <typename T>
class BilateralFilter : public Kernel<T> {
 public:
  BilateralFilter(IterationSpace<T> &it, Accessor<T> &in, Mask<float> &spatial, float sigma_r)
      : Kernel<T>(it), in_(in), m_(spatial), sigma_r_(sigma_r) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    check(hgb_bilateral(&iv, &ov, m_.coefficients(), m_.size_x(), sigma_r_, (int)in_.mode(), (float)in_.constant(), 0,
                        current_stream()),
          "BilateralFilter::execute");
  }
  Accessor<T> &in_;
  Mask<float> &m_;
  float sigma_r_;
};

// min(|reduce(dom_x, SUM, mx * in)| + |reduce(dom_y, SUM, my * in)|, 255);
// reduced_data(Reduce::SUM / MAX) returns the fused sum / max of the result
class SobelMagnitude : public Kernel<uchar> {
 public:
  SobelMagnitude(IterationSpace<uchar> &it, Accessor<uchar> &in, Mask<int> &mx, Mask<int> &my)
      : Kernel<uchar>(it), in_(in), mx_(mx), my_(my) {
    // device slots of the fused sum and max (created here, so execute() allocates nothing)
    hgb_image *d = nullptr;
    check(hgb_image_create(HGB_U64, 2, 1, 256, nullptr, &d), "SobelMagnitude scratch");
    scratch_.reset(d, [](hgb_image *p) { hgb_image_destroy(p); });
  }
  unsigned long long reduced_sum() {
    fetch();
    return host_[0];
  }
  uchar reduced_max() {
    fetch();
    return (uchar)host_[1];
  }

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view(), sv;
    hgb_image_get_view(scratch_.get(), &sv);
    uint64_t *sum = (uint64_t *)sv.data;
    uint32_t *mx = (uint32_t *)((char *)sv.data + 8);
    check(hgb_sobel_mag(&iv, &ov, mx_.coefficients(), my_.coefficients(), mx_.size_x(), (int)in_.mode(),
                        (int)in_.constant(), sum, mx, current_stream()),
          "SobelMagnitude::execute");
  }
  // read the two scalars back (synchronises the current stream); read on
  // every call, since a replayed graph rewrites them without a launch() here
  void fetch() {
    execute();
    unsigned long long tmp[2] = {0, 0};
    check(hgb_image_read(scratch_.get(), tmp, current_stream()), "SobelMagnitude::reduced_data");
    host_[0] = tmp[0];
    host_[1] = tmp[1] & 0xffffffffull;
  }
  uchar reduce_output() override {
    fetch();
    return (uchar)host_[1];
  }
  std::shared_ptr<hgb_image> scratch_;
  Accessor<uchar> &in_;
  Mask<int> &mx_, &my_;
  unsigned long long host_[2] = {0, 0};
};

class ColorConversion : public Kernel<uchar> {
 public:
  ColorConversion(IterationSpace<uchar> &it, Accessor<uchar4> &in, int wr = 77, int wg = 150, int wb = 29, int shift = 8)
      : Kernel<uchar>(it), in_(in), wr_(wr), wg_(wg), wb_(wb), sh_(shift) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    check(hgb_point_gray(&iv, &ov, wr_, wg_, wb_, sh_, current_stream()), "ColorConversion::execute");
  }
  Accessor<uchar4> &in_;
  int wr_, wg_, wb_, sh_;
};

// The Harris corner program of samples-public/3_Preprocessing/Harris_Corner
// (3x3; derivatives, squares, Gaussians, response) as one kernel object: the
// accessor's boundary applies to every local operator of the chain.  mode 0
// runs it fused, mode 1 as the reference's nine launches.
class HarrisCorner : public Kernel<uchar> {
 public:
  HarrisCorner(IterationSpace<uchar> &it, Accessor<uchar> &in, float k = 0.04f, float threshold = 20000.0f,
               int mode = 0)
      : Kernel<uchar>(it), in_(in), k_(k), thr_(threshold), mode_(mode) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    check(hgb_harris_corner(&iv, &ov, k_, thr_, (int)in_.mode(), mode_, current_stream()), "HarrisCorner::execute");
  }
  Accessor<uchar> &in_;
  float k_, thr_;
  int mode_;
};

// The Unsharp program of samples-public/1_Local_Operators/Unsharp (3x3;
// luminance, blur, sharpen, ratio, scale) as one kernel object; the accessor's
// boundary applies to the blur.  mode 0 fused, mode 1 the reference's five
// launches.
class UnsharpMask : public Kernel<uchar4> {
 public:
  UnsharpMask(IterationSpace<uchar4> &it, Accessor<uchar4> &in, int mode = 0) : Kernel<uchar4>(it), in_(in), mode_(mode) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    check(hgb_unsharp(&iv, &ov, (int)in_.mode(), mode_, current_stream()), "UnsharpMask::execute");
  }
  Accessor<uchar4> &in_;
  int mode_;
};

// output() = input(): a plain copy, or a resampling read for NN / LF accessors
template <typename T>
class Copy : public Kernel<T> {
 public:
  Copy(IterationSpace<T> &it, Accessor<T> &in) : Kernel<T>(it), in_(in) {}

 protected:
  void launch() override {
    hgb_view iv = in_.image().view(), ov = this->out_view();
    if (in_.interpolation() == Interpolate::NO) {
      check(hgb_image_copy_region(in_.image().handle(), &in_.window(), this->it_.image().handle(), this->out_window(),
                                  current_stream()),
            "Copy::execute");
    } else {
      check(hgb_resample(&iv, &ov, (int)in_.interpolation(), current_stream()), "Copy::execute");
    }
  }
  Accessor<T> &in_;
};

// output() = input1() - input2(); input2 may be a linear-filtering accessor
template <typename T>
class Difference : public Kernel<T> {
 public:
  Difference(IterationSpace<T> &it, Accessor<T> &a, Accessor<T> &b) : Kernel<T>(it), a_(a), b_(b) {}

 protected:
  void launch() override {
    hgb_view av = a_.image().view(), bv = b_.image().view(), ov = this->out_view();
    if (b_.interpolation() != Interpolate::NO) {
      Image<T> tmp(ov.width, ov.height);
      hgb_view tv = tmp.view();
      check(hgb_resample(&bv, &tv, (int)b_.interpolation(), current_stream()), "Difference::execute");
      check(hgb_point_binary(0, &av, &tv, &ov, 1.0f, 1.0f, current_stream()), "Difference::execute");
    } else {
      check(hgb_point_binary(0, &av, &bv, &ov, 1.0f, 1.0f, current_stream()), "Difference::execute");
    }
  }
  Accessor<T> &a_, &b_;
};

// output() = input(); reduce(l, r) by Reduce
template <typename T>
class Reduction : public Kernel<T> {
 public:
  Reduction(IterationSpace<T> &it, Accessor<T> &in, Reduce op) : Kernel<T>(it), in_(in), op_(op) {}

 protected:
  void launch() override {}
  T reduce_output() override { return reduce_image<T>(in_.image(), in_.window(), op_); }
  Accessor<T> &in_;
  Reduce op_;
};

// ---------------------------------------------------------------- pyramids
// Pyramid<T> and traverse (dsl/pyramid.hpp:97-318): levels of floor(w/2^l).
class PyramidBase {
 public:
  explicit PyramidBase(int depth) : depth_(depth) {}
  virtual ~PyramidBase() {}
  int depth() const { return depth_; }
  int level() const { return level_; }
  bool is_top_level() const { return level_ == 0; }
  bool is_bottom_level() const { return level_ == depth_ - 1; }
  void increment() { ++level_; }
  void decrement() { --level_; }
  void reset() { level_ = 0; }

 private:
  int depth_;
  int level_ = 0;
};

template <typename T>
class Pyramid : public PyramidBase {
 public:
  Pyramid(Image<T> &img, int depth) : PyramidBase(depth) {
    levels_.emplace_back(std::shared_ptr<Image<T>>(&img, [](Image<T> *) {}));
    int w = img.width() / 2, h = img.height() / 2;
    for (int i = 1; i < depth; ++i) {
      if (w < 1 || h < 1) throw Error(HGB_ERR_INVALID, "Pyramid stages too deep for image size");
      levels_.push_back(std::make_shared<Image<T>>(w, h));
      w /= 2;
      h /= 2;
    }
  }
  Image<T> &operator()(int relative) {
    const int l = level() + relative;
    if (l < 0 || l >= (int)levels_.size()) throw Error(HGB_ERR_INVALID, "Accessed pyramid stage is out of bounds");
    return *levels_[(size_t)l];
  }

 private:
  std::vector<std::shared_ptr<Image<T>>> levels_;
};

namespace detail {
inline std::vector<const std::function<void()> *> &traverse_funcs() {
  static std::vector<const std::function<void()> *> v;
  return v;
}
inline std::vector<std::vector<PyramidBase *>> &traverse_pyrs() {
  static std::vector<std::vector<PyramidBase *>> v;
  return v;
}
}  // namespace detail

inline void traverse(std::vector<PyramidBase *> pyrs, const std::function<void()> &f) {
  for (auto *p : pyrs) p->reset();
  detail::traverse_pyrs().push_back(pyrs);
  detail::traverse_funcs().push_back(&f);
  f();
  detail::traverse_funcs().pop_back();
  detail::traverse_pyrs().pop_back();
}
inline void traverse(PyramidBase &p0, const std::function<void()> &f) { traverse(std::vector<PyramidBase *>{&p0}, f); }
inline void traverse(PyramidBase &p0, PyramidBase &p1, const std::function<void()> &f) {
  traverse(std::vector<PyramidBase *>{&p0, &p1}, f);
}
inline void traverse(PyramidBase &p0, PyramidBase &p1, PyramidBase &p2, const std::function<void()> &f) {
  traverse(std::vector<PyramidBase *>{&p0, &p1, &p2}, f);
}
// recursion into the next level (dsl/pyramid.hpp:306-318)
inline void traverse(int loop = 1, const std::function<void()> &between = [] {}) {
  if (detail::traverse_pyrs().empty()) throw Error(HGB_ERR_INVALID, "traverse recursion called outside of traverse");
  auto pyrs = detail::traverse_pyrs().back();
  if (pyrs.at(0)->is_bottom_level()) return;
  for (auto *p : pyrs) p->increment();
  for (int i = 0; i < loop; ++i) {
    (*detail::traverse_funcs().back())();
    if (i < loop - 1) between();
  }
  for (auto *p : pyrs) p->decrement();
}

// Batched form: the Laplacian pyramids of many FP32 images in one persistent
// launch (hgb_pyramid_plan).
class LaplacianPyramidBatch {
 public:
  LaplacianPyramidBatch(const std::vector<int> &w, const std::vector<int> &h, int levels, const float mask5[25],
                        Boundary b = Boundary::MIRROR) {
    hgb_pyramid_plan *p = nullptr;
    check(hgb_pyramid_plan_create((int)w.size(), w.data(), h.data(), levels, mask5, (int)b, &p), "pyramid plan");
    plan_.reset(p, [](hgb_pyramid_plan *q) { hgb_pyramid_plan_destroy(q); });
  }
  hgb_view gauss(int image, int level) const {
    hgb_view g, l;
    check(hgb_pyramid_level_view(plan_.get(), image, level, &g, &l), "pyramid view");
    return g;
  }
  hgb_view laplace(int image, int level) const {
    hgb_view g, l;
    check(hgb_pyramid_level_view(plan_.get(), image, level, &g, &l), "pyramid view");
    return l;
  }
  void decompose(int mode = 0) { check(hgb_pyramid_decompose(plan_.get(), mode, current_stream()), "pyramid decompose"); }
  void collapse() { check(hgb_pyramid_collapse(plan_.get(), current_stream()), "pyramid collapse"); }

 private:
  std::shared_ptr<hgb_pyramid_plan> plan_;
};

}  // namespace hipacc

#endif  // HIPACC_GB300_HIPACC_HPP
