// ref_dsl.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own DSL headers (dsl/hipacc.hpp, dsl/kernel.hpp,
// dsl/image.hpp, dsl/mask.hpp, dsl/pyramid.hpp), which execute every kernel
// on the CPU when no Hipacc compiler is involved (dsl/kernel.hpp:94-119).
// Built by oracle/Makefile against the headers where they lie in the
// reference tree, into oracle/_ref/ (never shipped, never committed).  Used to
// pin the restated oracle (hgb_oracle.cpp) and to generate tests/golden/.
//
// Kernel bodies mirror the sample programs:
//   convolve:  samples-public/1_Local_Operators/Gaussian_Blur/src/main.cpp:56-61 (float and
//              the sample's own uchar form with `+ 0.5f`)
//   erode / dilate: samples-public/1_Local_Operators/Erode/src/main.cpp, Dilate/src/main.cpp
//   Sobel:     samples-public/3_Preprocessing/Sobel/src/main.cpp:56-67
//   bilateral: samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77
//   reduction: samples-public/2_Global_Operators/Reduction_Sum/src/main.cpp:50-62
//   pyramid:   samples-public/5_Other/Gaussian_Laplacian_Pyramid/src/main.cpp:199-231
//   Harris:    samples-public/3_Preprocessing/Harris_Corner/src/main.cpp:56-166,258-307 (3x3)
//   Unsharp:   samples-public/1_Local_Operators/Unsharp/src/main.cpp:53-149,203-247 (3x3)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>

#include "hipacc.hpp"

using namespace hipacc;

namespace {

class ConvK : public Kernel<float> {
  Accessor<float> &in;
  Mask<float> &mask;

 public:
  ConvK(IterationSpace<float> &it, Accessor<float> &in, Mask<float> &m) : Kernel(it), in(in), mask(m) {
    add_accessor(&in);
  }
  void kernel() {
    output() = convolve(mask, Reduce::SUM, [&]() -> float { return mask() * in(mask); });
  }
};

class DomRedK : public Kernel<float> {
  Accessor<float> &in;
  Domain &dom;
  Reduce mode;

 public:
  DomRedK(IterationSpace<float> &it, Accessor<float> &in, Domain &d, Reduce mode)
      : Kernel(it), in(in), dom(d), mode(mode) {
    add_accessor(&in);
  }
  void kernel() {
    output() = reduce(dom, mode, [&]() -> float { return in(dom); });
  }
};

// the Gaussian-blur sample's u8 body: (uchar)(convolve(...) + 0.5f)
class ConvU8K : public Kernel<uchar> {
  Accessor<uchar> &in;
  Mask<float> &mask;

 public:
  ConvU8K(IterationSpace<uchar> &it, Accessor<uchar> &in, Mask<float> &m) : Kernel(it), in(in), mask(m) {
    add_accessor(&in);
  }
  void kernel() {
    output() = (uchar)(convolve(mask, Reduce::SUM, [&]() -> float { return mask() * in(mask); }) + 0.5f);
  }
};

// the Erode / Dilate samples' body: reduce(dom, MIN / MAX) over uchar
class DomRedU8K : public Kernel<uchar> {
  Accessor<uchar> &in;
  Domain &dom;
  Reduce mode;

 public:
  DomRedU8K(IterationSpace<uchar> &it, Accessor<uchar> &in, Domain &d, Reduce mode)
      : Kernel(it), in(in), dom(d), mode(mode) {
    add_accessor(&in);
  }
  void kernel() {
    output() = reduce(dom, mode, [&]() -> uchar { return in(dom); });
  }
};

class SobelK : public Kernel<uchar> {
  Accessor<uchar> &in;
  Domain &dx, &dy;
  Mask<int> &mx, &my;

 public:
  SobelK(IterationSpace<uchar> &it, Accessor<uchar> &in, Domain &dx, Domain &dy, Mask<int> &mx,
         Mask<int> &my)
      : Kernel(it), in(in), dx(dx), dy(dy), mx(mx), my(my) {
    add_accessor(&in);
  }
  void kernel() {
    int gx = reduce(dx, Reduce::SUM, [&]() -> int { return mx(dx) * in(dx); });
    int gy = reduce(dy, Reduce::SUM, [&]() -> int { return my(dy) * in(dy); });
    int m = std::abs(gx) + std::abs(gy);
    output() = (uchar)(m > 255 ? 255 : m);
  }
};

class GrayK : public Kernel<uchar> {
  Accessor<uchar4> &in;

 public:
  GrayK(IterationSpace<uchar> &it, Accessor<uchar4> &in) : Kernel(it), in(in) { add_accessor(&in); }
  void kernel() {
    uchar4 p = in();
    output() = (uchar)((77 * p.x + 150 * p.y + 29 * p.z) >> 8);
  }
};

template <typename T>
class CopyK : public Kernel<T> {
  Accessor<T> &in;

 public:
  CopyK(IterationSpace<T> &it, Accessor<T> &in) : Kernel<T>(it), in(in) { this->add_accessor(&in); }
  void kernel() { this->output() = in(); }
};

class SumU64K : public Kernel<uint64_t> {
  Accessor<uchar> &in;

 public:
  SumU64K(IterationSpace<uint64_t> &it, Accessor<uchar> &in) : Kernel(it), in(in) { add_accessor(&in); }
  void kernel() { output() = (uint64_t)in(); }
  uint64_t reduce(uint64_t l, uint64_t r) const { return l + r; }
};

class MaxU8K : public Kernel<uchar> {
  Accessor<uchar> &in;

 public:
  MaxU8K(IterationSpace<uchar> &it, Accessor<uchar> &in) : Kernel(it), in(in) { add_accessor(&in); }
  void kernel() { output() = in(); }
  uchar reduce(uchar l, uchar r) const { return l > r ? l : r; }
};

class RedF32K : public Kernel<float> {
  Accessor<float> &in;
  int op;

 public:
  RedF32K(IterationSpace<float> &it, Accessor<float> &in, int op) : Kernel(it), in(in), op(op) {
    add_accessor(&in);
  }
  void kernel() { output() = in(); }
  float reduce(float l, float r) const {
    switch (op) {
      case 0: return l + r;
      case 1: return l < r ? l : r;
      case 2: return l > r ? l : r;
      default: return l * r;
    }
  }
};

class BilateralK : public Kernel<float> {
  Accessor<float> &in;
  Mask<float> &mask;
  Domain &dom;
  float sigma_r;

 public:
  BilateralK(IterationSpace<float> &it, Accessor<float> &in, Mask<float> &m, Domain &d, float s)
      : Kernel(it), in(in), mask(m), dom(d), sigma_r(s) {
    add_accessor(&in);
  }
  void kernel() {
    float c_r = 0.5f / (sigma_r * sigma_r);
    float d = 0.0f;
    float p = 0.0f;
    float center = in();
    iterate(dom, [&]() -> void {
      float diff = in(dom) - center;
      float s = expf(-c_r * diff * diff) * mask(dom);
      d += s;
      p += s * in(dom);
    });
    output() = p / d;
  }
};

class DoGK : public Kernel<float> {
  Accessor<float> &a, &b;

 public:
  DoGK(IterationSpace<float> &it, Accessor<float> &a, Accessor<float> &b) : Kernel(it), a(a), b(b) {
    add_accessor(&a);
    add_accessor(&b);
  }
  void kernel() { output() = a() - b(); }
};

template <typename T>
BoundaryCondition<T> make_bc(Image<T> &img, MaskBase &m, int bmode) {
  if (bmode == (int)Boundary::CONSTANT) return BoundaryCondition<T>(img, m, Boundary::CONSTANT, T{});
  return BoundaryCondition<T>(img, m, (Boundary)bmode);
}

template <int MH, int MW>
void conv_sized(const float *in, int w, int h, const float *coef, int bmode, int dom_mode, int red,
                float *out) {
  float c[MH][MW];
  std::memcpy(c, coef, sizeof(c));
  Mask<float> mask(c);
  Image<float> IN(w, h, const_cast<float *>(in));
  Image<float> OUT(w, h);
  BoundaryCondition<float> bc = make_bc(IN, mask, bmode);
  Accessor<float> acc(bc);
  IterationSpace<float> it(OUT);
  if (dom_mode) {
    Domain dom(mask);
    DomRedK k(it, acc, dom, (Reduce)red);
    k.execute();
  } else {
    ConvK k(it, acc, mask);
    k.execute();
  }
  std::memcpy(out, OUT.data(), sizeof(float) * (size_t)w * h);
}

template <int MH, int MW>
void conv_u8_sized(const uint8_t *in, int w, int h, const float *coef, int bmode, int dom_mode, int red,
                   uint8_t *out) {
  float c[MH][MW];
  std::memcpy(c, coef, sizeof(c));
  Mask<float> mask(c);
  Image<uchar> IN(w, h, const_cast<uchar *>(in));
  Image<uchar> OUT(w, h);
  BoundaryCondition<uchar> bc = make_bc(IN, mask, bmode);
  Accessor<uchar> acc(bc);
  IterationSpace<uchar> it(OUT);
  if (dom_mode) {
    Domain dom(mask);
    DomRedU8K k(it, acc, dom, (Reduce)red);
    k.execute();
  } else {
    ConvU8K k(it, acc, mask);
    k.execute();
  }
  std::memcpy(out, OUT.data(), (size_t)w * h);
}

template <int S>
void sobel_sized(const uint8_t *in, int w, int h, const int *cx, const int *cy, int bmode, uint8_t *out) {
  int ax[S][S], ay[S][S];
  std::memcpy(ax, cx, sizeof(ax));
  std::memcpy(ay, cy, sizeof(ay));
  Mask<int> mx(ax), my(ay);
  Domain dx(mx), dy(my);
  Image<uchar> IN(w, h, const_cast<uchar *>(in));
  Image<uchar> OUT(w, h);
  BoundaryCondition<uchar> bc = make_bc(IN, dx, bmode);
  Accessor<uchar> acc(bc);
  IterationSpace<uchar> it(OUT);
  SobelK k(it, acc, dx, dy, mx, my);
  k.execute();
  std::memcpy(out, OUT.data(), (size_t)w * h);
}

template <int S>
void bilateral_sized(const float *in, int w, int h, const float *coef, float sigma_r, int bmode, float *out) {
  float c[S][S];
  std::memcpy(c, coef, sizeof(c));
  Mask<float> mask(c);
  Domain dom(mask);
  Image<float> IN(w, h, const_cast<float *>(in));
  Image<float> OUT(w, h);
  BoundaryCondition<float> bc = make_bc(IN, dom, bmode);
  Accessor<float> acc(bc);
  IterationSpace<float> it(OUT);
  BilateralK k(it, acc, mask, dom, sigma_r);
  k.execute();
  std::memcpy(out, OUT.data(), sizeof(float) * (size_t)w * h);
}

// ---- Harris corner sample (3x3): derivative masks over Domains, squares,
// integer Gaussian with a divisor, response threshold
class HarrisDerivK : public Kernel<short> {
  Accessor<uchar> &in;
  Mask<char> &mask;
  Domain &dom;

 public:
  HarrisDerivK(IterationSpace<short> &it, Accessor<uchar> &in, Mask<char> &m, Domain &d)
      : Kernel(it), in(in), mask(m), dom(d) {
    add_accessor(&in);
  }
  void kernel() {
    short sum = 0;
    sum += reduce(dom, Reduce::SUM, [&]() -> short { return in(dom) * mask(dom); });
    output() = sum / 6;
  }
};

class HarrisSq1K : public Kernel<short> {
  Accessor<short> &in;

 public:
  HarrisSq1K(IterationSpace<short> &it, Accessor<short> &in) : Kernel(it), in(in) { add_accessor(&in); }
  void kernel() {
    short v = in();
    output() = v * v;
  }
};

class HarrisSq2K : public Kernel<short> {
  Accessor<short> &a, &b;

 public:
  HarrisSq2K(IterationSpace<short> &it, Accessor<short> &a, Accessor<short> &b) : Kernel(it), a(a), b(b) {
    add_accessor(&a);
    add_accessor(&b);
  }
  void kernel() { output() = a() * b(); }
};

class HarrisGaussK : public Kernel<short> {
  Accessor<short> &in;
  Mask<uchar> &mask;
  short norm;

 public:
  HarrisGaussK(IterationSpace<short> &it, Accessor<short> &in, Mask<uchar> &m, short norm)
      : Kernel(it), in(in), mask(m), norm(norm) {
    add_accessor(&in);
  }
  void kernel() {
    int sum = 0;
    sum += convolve(mask, Reduce::SUM, [&]() -> int { return in(mask) * mask(); });
    output() = sum / norm;
  }
};

class HarrisRespK : public Kernel<uchar> {
  Accessor<short> &dx, &dy, &dxy;
  float k, threshold;

 public:
  HarrisRespK(IterationSpace<uchar> &it, Accessor<short> &dx, Accessor<short> &dy, Accessor<short> &dxy, float k,
              float threshold)
      : Kernel(it), dx(dx), dy(dy), dxy(dxy), k(k), threshold(threshold) {
    add_accessor(&dx);
    add_accessor(&dy);
    add_accessor(&dxy);
  }
  void kernel() {
    int x = dx();
    int y = dy();
    int xy = dxy();
    float R = 0;
    R = ((x * y) - (xy * xy)) - (k * (x + y) * (x + y));
    uchar out = 0;
    if (R > threshold) out = 1;
    output() = out;
  }
};

template <typename T>
BoundaryCondition<T> make_bc_t(Image<T> &img, MaskBase &m, int bmode) {
  switch (bmode) {
    case 2: return BoundaryCondition<T>(img, m, Boundary::REPEAT);
    case 3: return BoundaryCondition<T>(img, m, Boundary::MIRROR);
    default: return BoundaryCondition<T>(img, m, Boundary::CLAMP);
  }
}

// ---- Unsharp sample (3x3): gamma-corrected luminance, blur, sharpen, ratio, scale
class UnsGrayK : public Kernel<float> {
  Accessor<uchar4> &in;

 public:
  UnsGrayK(IterationSpace<float> &it, Accessor<uchar4> &in) : Kernel(it), in(in) { add_accessor(&in); }
  void kernel() {
    uchar4 pixel = in();
    float c = 1.0f / 2.2f;
    float xg = powf((float)pixel.x, c);
    float yg = powf((float)pixel.y, c);
    float zg = powf((float)pixel.z, c);
    output() = 0.2126f * xg + 0.7152 * yg + 0.0722 * zg;
  }
};

class UnsSharpK : public Kernel<float> {
  Accessor<float> &gray, &blur;

 public:
  UnsSharpK(IterationSpace<float> &it, Accessor<float> &g, Accessor<float> &b) : Kernel(it), gray(g), blur(b) {
    add_accessor(&gray);
    add_accessor(&blur);
  }
  void kernel() { output() = 2 * gray() - blur(); }
};

class UnsRatioK : public Kernel<float> {
  Accessor<float> &gray, &sharp;

 public:
  UnsRatioK(IterationSpace<float> &it, Accessor<float> &g, Accessor<float> &s) : Kernel(it), gray(g), sharp(s) {
    add_accessor(&gray);
    add_accessor(&sharp);
  }
  void kernel() {
    float pixel = gray();
    pixel = std::max(pixel, 0.01f);
    output() = sharp() / pixel;
  }
};

class UnsScaleK : public Kernel<uchar4> {
  Accessor<uchar4> &in;
  Accessor<float> &ratio;

 public:
  UnsScaleK(IterationSpace<uchar4> &it, Accessor<uchar4> &in, Accessor<float> &r) : Kernel(it), in(in), ratio(r) {
    add_accessor(&in);
    add_accessor(&ratio);
  }
  void kernel() {
    uchar4 v = in();
    float r = ratio();
    v.x *= r;
    v.y *= r;
    v.z *= r;
    output() = v;
  }
};

}  // namespace

extern "C" {

// The Harris corner program of the sample (3x3 masks, k, threshold) with the
// boundary bmode (1 CLAMP as the sample, 2 REPEAT, 3 MIRROR) on every local
// operator; out is 0 / 1 per pixel
void ref_harris_u8(const uint8_t *input, int w, int h, int bmode, float k, float threshold, uint8_t *out) {
  const short norm = 16;
  const uchar cxy[3][3] = {{1, 2, 1}, {2, 4, 2}, {1, 2, 1}};
  const char cx[3][3] = {{-1, 0, 1}, {-1, 0, 1}, {-1, 0, 1}};
  const char cy[3][3] = {{-1, -1, -1}, {0, 0, 0}, {1, 1, 1}};
  Image<uchar> IN(w, h, const_cast<uint8_t *>(input));
  Image<uchar> OUT(w, h);
  Image<short> dx(w, h), dy(w, h), dxy(w, h), sx(w, h), sy(w, h), sxy(w, h);
  Mask<uchar> maskxy(cxy);
  Mask<char> maskx(cx), masky(cy);
  Domain domx(maskx), domy(masky);
  IterationSpace<short> iter_dx(dx), iter_dy(dy), iter_sx(sx), iter_sy(sy), iter_sxy(sxy), iter_dxy(dxy);
  BoundaryCondition<uchar> bound_in = make_bc_t<uchar>(IN, maskx, bmode);
  Accessor<uchar> acc_in(bound_in);
  HarrisDerivK derivx(iter_dx, acc_in, maskx, domx);
  derivx.execute();
  HarrisDerivK derivy(iter_dy, acc_in, masky, domy);
  derivy.execute();
  Accessor<short> acc_dx(dx), acc_dy(dy);
  HarrisSq1K squarex(iter_sx, acc_dx);
  squarex.execute();
  HarrisSq1K squarey(iter_sy, acc_dy);
  squarey.execute();
  HarrisSq2K squarexy(iter_sxy, acc_dx, acc_dy);
  squarexy.execute();
  BoundaryCondition<short> bound_sx = make_bc_t<short>(sx, maskxy, bmode);
  Accessor<short> acc_sx(bound_sx);
  HarrisGaussK gaussx(iter_dx, acc_sx, maskxy, norm);
  gaussx.execute();
  BoundaryCondition<short> bound_sy = make_bc_t<short>(sy, maskxy, bmode);
  Accessor<short> acc_sy(bound_sy);
  HarrisGaussK gaussy(iter_dy, acc_sy, maskxy, norm);
  gaussy.execute();
  BoundaryCondition<short> bound_sxy = make_bc_t<short>(sxy, maskxy, bmode);
  Accessor<short> acc_sxy(bound_sxy);
  HarrisGaussK gaussxy(iter_dxy, acc_sxy, maskxy, norm);
  gaussxy.execute();
  IterationSpace<uchar> iter_out(OUT);
  Accessor<short> acc_dxy(dxy);
  HarrisRespK harris(iter_out, acc_dx, acc_dy, acc_dxy, k, threshold);
  harris.execute();
  std::memcpy(out, OUT.data(), (size_t)w * h);
}

// The Unsharp program of the sample (3x3 mask) with the blur's boundary bmode;
// gray_out (may be NULL) receives the luminance image
void ref_unsharp_u8x4(const uint8_t *rgba, int w, int h, int bmode, uint8_t *out, float *gray_out) {
  const float coef[3][3] = {{0.057118f, 0.124758f, 0.057118f},
                            {0.124758f, 0.272496f, 0.124758f},
                            {0.057118f, 0.124758f, 0.057118f}};
  Image<uchar4> IN(w, h, reinterpret_cast<uchar4 *>(const_cast<uint8_t *>(rgba)));
  Image<float> gray(w, h), blur(w, h), sharp(w, h), ratio(w, h);
  Image<uchar4> OUT(w, h);
  Mask<float> mask(coef);
  IterationSpace<float> iterGray(gray);
  Accessor<uchar4> accIn(IN);
  UnsGrayK g(iterGray, accIn);
  g.execute();
  BoundaryCondition<float> bound = make_bc_t<float>(gray, mask, bmode);
  Accessor<float> accGrayBound(bound);
  Accessor<float> accGray(gray);
  IterationSpace<float> iterBlur(blur);
  ConvK gb(iterBlur, accGrayBound, mask);
  gb.execute();
  IterationSpace<float> iterSharp(sharp);
  Accessor<float> accBlur(blur);
  UnsSharpK sh(iterSharp, accGray, accBlur);
  sh.execute();
  IterationSpace<float> iterRatio(ratio);
  Accessor<float> accSharp(sharp);
  UnsRatioK ra(iterRatio, accGray, accSharp);
  ra.execute();
  IterationSpace<uchar4> iter(OUT);
  Accessor<float> accRatio(ratio);
  UnsScaleK us(iter, accIn, accRatio);
  us.execute();
  std::memcpy(out, OUT.data(), (size_t)w * h * 4);
  if (gray_out) std::memcpy(gray_out, gray.data(), sizeof(float) * (size_t)w * h);
}

// returns 0 on success, -1 for an unsupported mask size
int ref_conv_f32(const float *in, int w, int h, const float *coef, int mw, int mh, int bmode, int dom_mode,
                 int red, float *out) {
#define HGB_CASE(H, W) \
  if (mh == H && mw == W) { conv_sized<H, W>(in, w, h, coef, bmode, dom_mode, red, out); return 0; }
  HGB_CASE(3, 3) HGB_CASE(5, 5) HGB_CASE(7, 7) HGB_CASE(9, 9) HGB_CASE(13, 13)
  HGB_CASE(1, 3) HGB_CASE(3, 1) HGB_CASE(1, 5) HGB_CASE(5, 1) HGB_CASE(1, 9) HGB_CASE(9, 1)
  HGB_CASE(3, 5) HGB_CASE(5, 3) HGB_CASE(1, 7) HGB_CASE(7, 1) HGB_CASE(1, 13) HGB_CASE(13, 1)
#undef HGB_CASE
  return -1;
}

// u8 images: the Gaussian-blur sample's convolution (dom_mode 0) or the
// Erode / Dilate samples' Domain reduction (dom_mode 1, red MIN or MAX)
int ref_conv_u8(const uint8_t *in, int w, int h, const float *coef, int mw, int mh, int bmode, int dom_mode,
                int red, uint8_t *out) {
#define HGB_CASE(H, W) \
  if (mh == H && mw == W) { conv_u8_sized<H, W>(in, w, h, coef, bmode, dom_mode, red, out); return 0; }
  HGB_CASE(3, 3) HGB_CASE(5, 5) HGB_CASE(7, 7) HGB_CASE(1, 5) HGB_CASE(5, 1)
#undef HGB_CASE
  return -1;
}

int ref_sobel_mag_u8(const uint8_t *in, int w, int h, const int *cx, const int *cy, int size, int bmode,
                     uint8_t *out) {
  if (size == 3) { sobel_sized<3>(in, w, h, cx, cy, bmode, out); return 0; }
  if (size == 5) { sobel_sized<5>(in, w, h, cx, cy, bmode, out); return 0; }
  if (size == 7) { sobel_sized<7>(in, w, h, cx, cy, bmode, out); return 0; }
  return -1;
}

void ref_gray_u8(const uint8_t *rgba, int w, int h, uint8_t *out) {
  Image<uchar4> IN(w, h, reinterpret_cast<uchar4 *>(const_cast<uint8_t *>(rgba)));
  Image<uchar> OUT(w, h);
  Accessor<uchar4> acc(IN);
  IterationSpace<uchar> it(OUT);
  GrayK k(it, acc);
  k.execute();
  std::memcpy(out, OUT.data(), (size_t)w * h);
}

uint64_t ref_sum_u8_u64(const uint8_t *in, int w, int h) {
  Image<uchar> IN(w, h, const_cast<uint8_t *>(in));
  Image<uint64_t> OUT(w, h);
  Accessor<uchar> acc(IN);
  IterationSpace<uint64_t> it(OUT);
  SumU64K k(it, acc);
  k.execute();
  return k.reduced_data();
}

uint32_t ref_max_u8(const uint8_t *in, int w, int h) {
  Image<uchar> IN(w, h, const_cast<uint8_t *>(in));
  Image<uchar> OUT(w, h);
  Accessor<uchar> acc(IN);
  IterationSpace<uchar> it(OUT);
  MaxU8K k(it, acc);
  k.execute();
  return k.reduced_data();
}

float ref_reduce_f32(const float *in, int w, int h, int op) {
  Image<float> IN(w, h, const_cast<float *>(in));
  Image<float> OUT(w, h);
  Accessor<float> acc(IN);
  IterationSpace<float> it(OUT);
  RedF32K k(it, acc, op);
  k.execute();
  return k.reduced_data();
}

int ref_bilateral_f32(const float *in, int w, int h, const float *coef, int size, float sigma_r, int bmode,
                      float *out) {
  if (size == 5) { bilateral_sized<5>(in, w, h, coef, sigma_r, bmode, out); return 0; }
  if (size == 9) { bilateral_sized<9>(in, w, h, coef, sigma_r, bmode, out); return 0; }
  if (size == 13) { bilateral_sized<13>(in, w, h, coef, sigma_r, bmode, out); return 0; }
  return -1;
}

// imode: 1 = NN, 2 = LF (hipacc::Interpolate numbering, dsl/image.hpp:54-61)
void ref_resample_f32(const float *src, int sw, int sh, float *dst, int dw, int dh, int imode) {
  Image<float> IN(sw, sh, const_cast<float *>(src));
  Image<float> OUT(dw, dh);
  Accessor<float> acc(IN, (Interpolate)imode);
  IterationSpace<float> it(OUT);
  CopyK<float> k(it, acc);
  k.execute();
  std::memcpy(dst, OUT.data(), sizeof(float) * (size_t)dw * dh);
}

// Laplacian pyramid through the DSL's Pyramid/traverse.  gauss_out holds the
// levels 0..depth-1 back to back, lap_out the levels 0..depth-2.
void ref_pyramid_f32(const float *img, int w, int h, int depth, const float *coef5, int bmode,
                     float *gauss_out, float *lap_out) {
  float c[5][5];
  std::memcpy(c, coef5, sizeof(c));
  Mask<float> mask(c);
  Image<float> gaus(w, h, const_cast<float *>(img));
  Image<float> tmp(w, h);
  Image<float> lap(w, h);
  Pyramid<float> pgaus(gaus, depth);
  Pyramid<float> ptmp(tmp, depth);
  Pyramid<float> plap(lap, depth);
  traverse(pgaus, ptmp, plap, [&]() {
    if (!pgaus.is_top_level()) {
      BoundaryCondition<float> bound = make_bc(pgaus(-1), mask, bmode);
      Accessor<float> acc1(bound);
      IterationSpace<float> iter1(ptmp(-1));
      ConvK blur(iter1, acc1, mask);
      blur.execute();

      Accessor<float> acc2(ptmp(-1), Interpolate::NN);
      IterationSpace<float> iter2(pgaus(0));
      CopyK<float> sub(iter2, acc2);
      sub.execute();

      Accessor<float> acc3(pgaus(-1));
      Accessor<float> acc4(pgaus(0), Interpolate::LF);
      IterationSpace<float> iter3(plap(-1));
      DoGK dog(iter3, acc3, acc4);
      dog.execute();
    }
    traverse();
  });
  size_t og = 0, ol = 0;
  for (int l = 0; l < depth; ++l) {
    Image<float> &g = pgaus(l);
    const size_t n = (size_t)g.width() * g.height();
    std::memcpy(gauss_out + og, g.data(), sizeof(float) * n);
    og += n;
    if (l + 1 < depth) {
      std::memcpy(lap_out + ol, plap(l).data(), sizeof(float) * n);
      ol += n;
    }
  }
}

}  // extern "C"
