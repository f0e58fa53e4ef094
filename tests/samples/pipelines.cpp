// The Harris corner and Unsharp programs (samples-public/3_Preprocessing/
// Harris_Corner, samples-public/1_Local_Operators/Unsharp, 3x3) recorded once
// into a whole-program CudaGraph, Hipacc's CUDA-graph mode
// (samples-public/common/config/cuda-graph.conf): the fused kernels on one
// branch and the reference's launch structure (nine and five launches, which
// share the library workspace and so stay on one stream) on the other, joined
// at the end.  Every replayed result is checked against plain CPU loops of the
// samples' kernel bodies, bit for bit; then new inputs are written and the
// same graph is replayed and checked again.
#include <hipacc_gb300/hipacc.hpp>

#include <algorithm>
#include <cstdint>

#include "common.hpp"

using namespace hipacc;

// structured test images: rectangles of random grey levels plus noise
static std::vector<unsigned char> blocks(int w, int h, unsigned seed) {
  std::mt19937_64 g(seed);
  std::vector<int> img((size_t)w * h, (int)(g() % 256));
  for (int n = 0; n < 40; ++n) {
    const int x0 = (int)(g() % (w - 2)), y0 = (int)(g() % (h - 2));
    const int x1 = x0 + 2 + (int)(g() % (w - x0 - 1)), y1 = y0 + 2 + (int)(g() % (h - y0 - 1));
    const int v = (int)(g() % 256);
    for (int y = y0; y < std::min(y1, h); ++y)
      for (int x = x0; x < std::min(x1, w); ++x) img[(size_t)y * w + x] = v;
  }
  std::vector<unsigned char> out(img.size());
  for (size_t i = 0; i < img.size(); ++i) out[i] = (unsigned char)clampi(img[i] + (int)(g() % 13) - 6, 0, 255);
  return out;
}

// the Harris sample's kernels, CLAMP everywhere
static std::vector<unsigned char> cpu_harris(const std::vector<unsigned char> &in, int w, int h, float k, float thr) {
  std::vector<short> sx((size_t)w * h), sy(sx.size()), sxy(sx.size());
  auto at = [&](int x, int y) { return (int)in[(size_t)clampi(y, 0, h - 1) * w + clampi(x, 0, w - 1)]; };
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      short ax = 0, ay = 0;
      for (int j = -1; j <= 1; ++j) {
        ax = (short)(ax - at(x - 1, y + j));
        ax = (short)(ax + at(x + 1, y + j));
      }
      for (int i = -1; i <= 1; ++i) ay = (short)(ay - at(x + i, y - 1));
      for (int i = -1; i <= 1; ++i) ay = (short)(ay + at(x + i, y + 1));
      const short dx = (short)(ax / 6), dy = (short)(ay / 6);
      sx[(size_t)y * w + x] = (short)(dx * dx);
      sy[(size_t)y * w + x] = (short)(dy * dy);
      sxy[(size_t)y * w + x] = (short)(dx * dy);
    }
  std::vector<unsigned char> out((size_t)w * h);
  const int m[3][3] = {{1, 2, 1}, {2, 4, 2}, {1, 2, 1}};
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      int a = 0, b = 0, c = 0;
      for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) {
          const size_t q = (size_t)clampi(y + j, 0, h - 1) * w + clampi(x + i, 0, w - 1);
          a += sx[q] * m[j + 1][i + 1];
          b += sy[q] * m[j + 1][i + 1];
          c += sxy[q] * m[j + 1][i + 1];
        }
      const int gx = (short)(a / 16), gy = (short)(b / 16), gxy = (short)(c / 16);
      volatile float det = (float)(gx * gy - gxy * gxy), tr = (float)(gx + gy);
      volatile float kt = k * tr;
      volatile float kt2 = kt * tr;
      volatile float R = det - kt2;
      out[(size_t)y * w + x] = R > thr ? 1 : 0;
    }
  return out;
}

// the Unsharp sample's kernels, CLAMP for the blur
static std::vector<unsigned char> cpu_unsharp(const std::vector<unsigned char> &in, int w, int h) {
  std::vector<float> gray((size_t)w * h);
  const float c = 1.0f / 2.2f;
  for (size_t p = 0; p < gray.size(); ++p) {
    volatile float xg = powf((float)in[4 * p], c), yg = powf((float)in[4 * p + 1], c), zg = powf((float)in[4 * p + 2], c);
    // every product and sum rounded on its own (no fused multiply-add)
    volatile float t0 = 0.2126f * xg;
    volatile double p1 = 0.7152 * (double)yg, p2 = 0.0722 * (double)zg;
    volatile double s1 = (double)t0 + p1;
    gray[p] = (float)(s1 + p2);
  }
  const float m[3][3] = {{0.057118f, 0.124758f, 0.057118f}, {0.124758f, 0.272496f, 0.124758f},
                         {0.057118f, 0.124758f, 0.057118f}};
  std::vector<unsigned char> out(in.size());
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      volatile float blur = 0.0f;
      for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) {
          volatile float t = m[j + 1][i + 1] * gray[(size_t)clampi(y + j, 0, h - 1) * w + clampi(x + i, 0, w - 1)];
          blur = blur + t;
        }
      const size_t p = (size_t)y * w + x;
      volatile float g2 = 2.0f * gray[p];
      volatile float sharp = g2 - blur;
      volatile float ratio = sharp / std::max(gray[p], 0.01f);
      for (int ch = 0; ch < 3; ++ch) {
        volatile float v = (float)in[4 * p + ch] * ratio;
        out[4 * p + ch] = (unsigned char)((int)v & 0xff);
      }
      out[4 * p + 3] = in[4 * p + 3];
    }
  return out;
}

int main() {
  hipaccInitCUDA(0);
  const int w = 403, h = 302;
  const float k = 0.04f, thr = 20000.0f;
  std::vector<unsigned char> gin = blocks(w, h, 41);
  std::vector<unsigned char> cin(4 * (size_t)w * h);
  for (int ch = 0; ch < 4; ++ch) {
    std::vector<unsigned char> b = blocks(w, h, 50 + ch);
    for (size_t p = 0; p < b.size(); ++p) cin[4 * p + ch] = b[p];
  }
  Image<uchar> hin(w, h, gin.data()), hout_f(w, h), hout_p(w, h);
  Image<uchar4> uin(w, h, reinterpret_cast<const uchar4 *>(cin.data())), uout_f(w, h), uout_p(w, h);
  const int dom[3][3] = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}};
  Mask<int> m3(dom);
  BoundaryCondition<uchar> hb(hin, m3, Boundary::CLAMP);
  Accessor<uchar> ha(hb);
  BoundaryCondition<uchar4> ub(uin, m3, Boundary::CLAMP);
  Accessor<uchar4> ua(ub);
  IterationSpace<uchar> hi_f(hout_f), hi_p(hout_p);
  IterationSpace<uchar4> ui_f(uout_f), ui_p(uout_p);
  HarrisCorner harris_f(hi_f, ha, k, thr, 0), harris_p(hi_p, ha, k, thr, 1);
  UnsharpMask unsharp_f(ui_f, ua, 0), unsharp_p(ui_p, ua, 1);

  // eager warm-up: the first calls size the workspace and upload tables
  HarrisCorner hw(hi_p, ha, k, thr, 1);
  hw.execute();
  UnsharpMask uw(ui_p, ua, 1);
  uw.execute();
  UnsharpMask uw0(ui_f, ua, 0);
  uw0.execute();

  CudaGraph graph;
  Stream side;
  graph.begin();
  side.wait(graph.stream());  // fork
  hipaccSetStream(side.get());
  harris_f.execute();
  unsharp_f.execute();
  hipaccSetStream(graph.stream().get());
  harris_p.execute();
  unsharp_p.execute();
  graph.stream().wait(side);  // join
  graph.end();

  for (int round = 0; round < 2; ++round) {
    for (int i = 0; i < 5; ++i) graph.launch();
    graph.synchronize();
    const std::vector<unsigned char> rh = cpu_harris(gin, w, h, k, thr), ru = cpu_unsharp(cin, w, h);
    const uchar *a = hout_f.data(), *b = hout_p.data();
    size_t corners = 0;
    for (size_t p = 0; p < rh.size(); ++p) {
      REQUIRE(a[p] == rh[p] && b[p] == rh[p]);
      corners += rh[p];
    }
    REQUIRE(corners > 0 && corners < rh.size() / 2);
    const unsigned char *c = reinterpret_cast<const unsigned char *>(uout_f.data());
    const unsigned char *d = reinterpret_cast<const unsigned char *>(uout_p.data());
    for (size_t p = 0; p < ru.size(); ++p) REQUIRE(c[p] == ru[p] && d[p] == ru[p]);
    std::printf("round %d: %zu corners, unsharp equal\n", round, corners);
    // new inputs into the same device images for the next replay
    gin = blocks(w, h, 141 + round);
    for (int ch = 0; ch < 4; ++ch) {
      std::vector<unsigned char> bb = blocks(w, h, 150 + 4 * round + ch);
      for (size_t p = 0; p < bb.size(); ++p) cin[4 * p + ch] = bb[p];
    }
    hin = gin.data();
    uin = reinterpret_cast<const uchar4 *>(cin.data());
  }
  std::printf("Test PASSED\n");
  return 0;
}
