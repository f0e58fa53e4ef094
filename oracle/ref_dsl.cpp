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

}  // namespace

extern "C" {

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
