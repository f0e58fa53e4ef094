// pyramid.cu -- Laplacian pyramids of many images of uneven sizes.
//
// Reference structure (samples-public/5_Other/Gaussian_Laplacian_Pyramid/src/main.cpp:199-248,
// dsl/pyramid.hpp:97-318): for each level l of each image, three kernels run
// one after the other, driven by the host's recursive traverse():
//   blur:        T_l     = conv5x5(G_l) with the boundary mode
//   subsample:   G_{l+1} = T_l read through a nearest-neighbour accessor
//                (x = (int)(scale/2 + scale*x'), scale = w_l / w_{l+1},
//                 lib/AST/Interpolate.cpp:85-113)
//   difference:  L_l     = G_l - LF(G_{l+1}) (linear filtering accessor with
//                CLAMP taps, runtime/hipacc_cu_interpolate.hpp:173-216)
// Level sizes are floor(w / 2^l) (dsl/pyramid.hpp:103-114).
//
// GB300 form: one level-tile kernel does all three for a 64 x 32 tile of L_l:
// it stages the G_l region it needs once in shared memory with one TMA load
// (a tensor map per image and level, built with the plan; cells outside the
// level are patched through the boundary remap), evaluates the blur
// only at the nearest-neighbour sample positions of the G_{l+1} tile plus a
// one-pixel halo (kept in shared memory), writes the G_{l+1} pixels the tile
// owns, and writes L_l from the staged G_l and the shared G_{l+1} values.
// Arithmetic order equals the reference's (blur taps row-major with fused
// multiply-add; LF as w_a*a, then three fused multiply-adds), so results are
// bit-identical to the three-kernel program.
//
// Launch forms (hgb_pyramid_decompose mode):
//   0  one persistent launch over a work-list of every level of every image.
//      CTAs claim tiles in list order (levels ascending) from an atomic
//      counter; a tile of level l waits (bounded, acquire) until its image's
//      level l-1 tiles are done, then publishes its own completion (release).
//      Tiles are claimed in order and only wait on earlier tiles, so resident
//      CTAs always make progress.
//   1  one launch per level over all images (the level barrier is the launch
//      boundary).
//   2  the reference's launch structure: per image and level, a blur over the
//      full level, a subsample and a difference launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cstdio>

#include "autotune.h"
#include "local_op.cuh"
#include "tma.cuh"

namespace hgb {
namespace {

// Tile configuration of the level-tile kernels: an L_l tile of TW x TH pixels,
// NT threads.  The G_{l+1} tile with its halo is GW x GH; the staged G_l region
// is bounded by SW x SH, and its TMA box is BW x BH (the x origin is rounded
// down to a multiple of 4 floats, 16 bytes, so the box is 4 floats wider).
template <int TW_, int TH_, int NT_>
struct PyCfg {
  static constexpr int TW = TW_, TH = TH_, NT = NT_;
  static constexpr int GW = TW / 2 + 2, GH = TH / 2 + 2;
  static constexpr int SW = TW + 12, SH = TH + 12;
  static constexpr int BW = SW + 4, BH = SH;
  static constexpr int MIN_CTAS = 1280 / NT;  // ten CTAs of 128 threads per SM
};
// configurations the autotuner chooses from (config 0 is the default; the
// collapse uses its work-list).  64 x 32 at 128 threads and ten CTAs per SM
// measured 1.30 -> 1.01 ms per batch against 256 threads and five CTAs.
using PyCfg0 = PyCfg<64, 32, 128>;
using PyCfg1 = PyCfg<64, 16, 128>;
using PyCfg2 = PyCfg<32, 32, 128>;
using PyCfg3 = PyCfg<64, 32, 256>;
constexpr int kPyCfgs = 4;
constexpr int PY_TW = 64, PY_TH = 32;  // config 0, the collapse's tiles
constexpr int kPyClaim = 4;            // tiles per claim of a persistent CTA

struct LevelMeta {
  float *g;    // Gaussian level
  float *lap;  // Laplacian level (null for the last level)
  int w, h;
  int pitch;   // floats
  int pad;
};

// A tile of the work-list.  The origin of its staged G_l box (bx, by) is
// computed with the plan, so that a CTA can issue the box's TMA load right
// after reading its tile record; the kernel recomputes it and checks.
struct __align__(16) PyrTile {
  int img, level, x0, y0;
  int bx, by, pad0, pad1;
};

struct PyrParams {
  const LevelMeta *meta;  // [img * levels + l]
  const CUtensorMap *maps;  // [img * levels + l]: G_l tensor maps, box BW x BH of the configuration
  const PyrTile *tiles;
  int ntiles;
  int levels;
  unsigned int *done;       // [img * levels + l]: finished tiles of level l
  const int *ntiles_il;     // [img * levels + l]: tiles of level l
  unsigned int *work;       // claim counter (persistent form)
  unsigned int *abort;      // set when a tile failed: dependants stop waiting (persistent form)
  int *status;
  long long max_polls;      // limit of every bounded wait
  int single;               // pyr_persistent_kernel: 0 persistent, 1 one tile per CTA, 2 static level 0
  int nlevel0;              // tiles of level 0 (the head of the work-list)
  int inject_kind;          // wait test (hgb_pyramid_plan_wait_test): 0 none, 1 withhold, 2 no copy
  int inject_level;
  float mask[25];
  int bmode;
  long long *trace;         // persistent form, when set: one PyrTrace record per CTA
};

// Per-CTA trace of the single-launch forms (thread 0's view): start and end
// (global timer, ns, and the SM clock), SM clock cycles spent in tile claims,
// in level waits and in tiles (work, barrier and publish), tiles taken, and
// waits that had to poll.
struct PyrTrace {
  long long t0, t1, c0, c1, claim, wait, tile, counts;  // counts: tiles | polled waits << 32
};
static_assert(sizeof(PyrTrace) == 8 * sizeof(long long), "trace record");

__device__ __forceinline__ long long global_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ float ld_level(const float *p, bool coherent) {
  // levels written inside the same persistent launch must bypass the
  // non-coherent read-only path
  return coherent ? __ldcg(p) : __ldg(p);
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add(unsigned int *p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Linear-filtering taps of one column (or row) of an L_l tile: the two
// G_{l+1} indices (tile-relative) and the weights f and 1 - f.
struct LfTap {
  int a, c;
  float f, g;
};

__device__ __forceinline__ LfTap lf_tap(float s, int x, int n, int origin) {
  float b = __fmaf_rn(s, (float)x, s * 0.5f) - 0.5f;
  b = b < 0.0f ? 0.0f : b;
  const int i = (int)b;
  const float f = b - (float)i;
  LfTap t;
  t.a = min(i, n - 1) - origin;
  t.c = min(i + 1, n - 1) - origin;
  t.f = f;
  t.g = 1.0f - f;
  return t;
}

// Five consecutive staged values of a row: two 8-byte loads and one 4-byte
// load, the 4-byte one first when the row position is odd.
template <bool ODD>
__device__ __forceinline__ void load5(const float *row, float v[5]) {
  if (ODD) {
    v[0] = row[0];
    const float2 a = *reinterpret_cast<const float2 *>(row + 1), b = *reinterpret_cast<const float2 *>(row + 3);
    v[1] = a.x; v[2] = a.y; v[3] = b.x; v[4] = b.y;
  } else {
    const float2 a = *reinterpret_cast<const float2 *>(row), b = *reinterpret_cast<const float2 *>(row + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    v[4] = row[4];
  }
}

// 5x5 blur at two samples of one column whose top rows are D apart: rows
// 0..D+4 of `src` are read once; each sample's 25 taps stay row-major fused
// multiply-adds (the reference's order).
template <int D, bool ODD, int BW>
__device__ __forceinline__ void blur_pair(const float *mask, const float *src, float &a0, float &a1) {
  float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
  for (int R = 0; R < D + 5; ++R) {
    float v[5];
    load5<ODD>(src + R * BW, v);
    if (R < 5) {
#pragma unroll
      for (int mx = 0; mx < 5; ++mx) s0 = __fmaf_rn(mask[R * 5 + mx], v[mx], s0);
    }
    if (R >= D) {
#pragma unroll
      for (int mx = 0; mx < 5; ++mx) s1 = __fmaf_rn(mask[(R - D) * 5 + mx], v[mx], s1);
    }
  }
  a0 = s0;
  a1 = s1;
}

template <int BW>
__device__ __forceinline__ float blur_one(const float *mask, const float *src) {
  float acc = 0.0f;
#pragma unroll
  for (int my = 0; my < 5; ++my)
#pragma unroll
    for (int mx = 0; mx < 5; ++mx) acc = __fmaf_rn(mask[my * 5 + mx], src[my * BW + mx], acc);
  return acc;
}

// One TW x TH tile of L_level (and the owned part of G_{level+1}).
// `bar` is the CTA's mbarrier and `phase` its next phase parity.
template <class C>
__device__ bool pyr_tile(const PyrParams &p, const PyrTile t, float *stage, float *gt, LfTap *cols, LfTap *rows,
                         int *ncx, int *ncy, uint64_t *bar, unsigned &phase, bool coherent) {
  // ---- stage the G_l box [by, by + BH) x [bx, bx + BW) with one TMA load
  if (threadIdx.x == 0) {
    // in the single-launch forms the previous tile's patch wrote `stage` with
    // generic stores, and a level above 0 was written by other CTAs of this
    // launch (generic stores, acquired by the level wait): order them before
    // the copy.  Level 0 was written before the launch and needs only the
    // shared-memory fence.
    if (coherent) {
      if (t.level > 0)
        asm volatile("fence.proxy.async;" ::: "memory");
      else
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    mbar_expect_tx(bar, C::BW * C::BH * 4);
    // wait test kind 2: the bytes are expected but no copy is issued, so the
    // barrier's phase never completes (nothing is in flight when the wait expires)
    if (!(p.inject_kind == 2 && t.level == p.inject_level))
      tma_load_3d(stage, &p.maps[t.img * p.levels + t.level], t.bx, t.by, 0, bar);
  }
  const LevelMeta A = p.meta[t.img * p.levels + t.level];
  const LevelMeta B = p.meta[t.img * p.levels + t.level + 1];
  const int wl = A.w, hl = A.h, wn = B.w, hn = B.h;
  // nearest-neighbour scale G_l -> G_{l+1} and linear-filtering scale G_{l+1} -> L_l
  const float Sx = (float)wl / (float)wn, Sy = (float)hl / (float)hn;
  const float sx = (float)wn / (float)wl, sy = (float)hn / (float)hl;
  const int gx0 = max(0, t.x0 / 2 - 1), gx1 = min(wn, t.x0 / 2 + C::TW / 2 + 1);
  const int gy0 = max(0, t.y0 / 2 - 1), gy1 = min(hn, t.y0 / 2 + C::TH / 2 + 1);
  auto nn = [](float S, int x, int lim) {
    int v = (int)__fmaf_rn(S, (float)x, S * 0.5f);
    return v < lim ? v : lim - 1;
  };
  const int rx0 = nn(Sx, gx0, wl) - 2;
  const int ry0 = nn(Sy, gy0, hl) - 2;
  // the box origin: x rounded down to a multiple of 4 floats (16 bytes)
  const int bx0 = rx0 & ~3, ox = rx0 - bx0;
  // while the box lands: the linear-filtering taps of the tile's columns and
  // rows, and the staged positions of the blur's nearest-neighbour samples
  for (int i = threadIdx.x; i < C::TW + C::TH + C::GW + C::GH; i += C::NT) {
    if (i < C::TW) {
      cols[i] = lf_tap(sx, t.x0 + i, wn, gx0);
    } else if (i < C::TW + C::TH) {
      rows[i - C::TW] = lf_tap(sy, t.y0 + i - C::TW, hn, gy0);
    } else if (i < C::TW + C::TH + C::GW) {
      const int q = i - C::TW - C::TH;
      ncx[q] = nn(Sx, gx0 + q, wl) - 2 - rx0 + ox;
    } else {
      const int r = i - C::TW - C::TH - C::GW;
      ncy[r] = nn(Sy, gy0 + r, hl) - 2 - ry0;
    }
  }
  const bool landed = cta_wait(bar, phase, p.max_polls);
  phase ^= 1u;
  if (!landed) {
    if (threadIdx.x == 0) {
      record_status(p.status, HGB_ERR_TIMEOUT);
      mbar_wait(bar, phase ^ 1u, p.max_polls);  // the copy may still land: wait once more (bounded)
    }
    return false;
  }
  if (t.bx != bx0 || t.by != ry0) {  // the plan's box origin disagrees (not expected): leave with an error
    if (threadIdx.x == 0) record_status(p.status, HGB_ERR_INTERNAL);
    return false;
  }
  if (bx0 < 0 || bx0 + C::BW > wl || ry0 < 0 || ry0 + C::BH > hl) {
    // box cells outside the level (zero-filled by TMA) through the boundary
    // remap: left / right columns, top / bottom rows.  The tile reads at most
    // two columns (rows) past the level's last one (the blur's reach from the
    // last nearest-neighbour position w_l - 1), so the patch stops there.
    const int cw = min(C::BW, wl + 2 - bx0), ch = min(C::BH, hl + 2 - ry0);  // box part the tile reads
    const int nl = max(0, min(cw, -bx0)), rs = max(0, min(cw, wl - bx0));
    const int nt = max(0, min(ch, -ry0)), bs = max(0, min(ch, hl - ry0));
    const int ncl = nl * ch, ncr = (cw - rs) * ch, nrt = nt * cw, nrb = (ch - bs) * cw;
    for (int c = threadIdx.x; c < ncl + ncr + nrt + nrb; c += C::NT) {
      int r, q;
      if (c < ncl) {
        r = c / nl;
        q = c - r * nl;
      } else if (c < ncl + ncr) {
        const int d = c - ncl, n = cw - rs;
        r = d / n;
        q = rs + (d - r * n);
      } else if (c < ncl + ncr + nrt) {
        const int d = c - ncl - ncr;
        r = d / cw;
        q = d - r * cw;
      } else {
        const int d = c - ncl - ncr - nrt;
        const int rr = d / cw;
        r = bs + rr;
        q = d - rr * cw;
      }
      const int yy = remap(p.bmode, ry0 + r, 0, hl), xx = remap(p.bmode, bx0 + q, 0, wl);
      stage[r * C::BW + q] = (yy == (int)0x80000000 || xx == (int)0x80000000)
                                 ? 0.0f
                                 : ld_level(A.g + (int64_t)yy * A.pitch + xx, coherent);
    }
    __syncthreads();
  }
  // ---- G_{l+1} on the tile + halo: blur at the nearest-neighbour positions,
  // two vertically adjacent samples per thread (they share 3 of their 5 rows
  // when their G_l rows are 2 apart, 2 when 3 apart)
  const int gw = gx1 - gx0, gh = gy1 - gy0;
  const int ownx0 = t.x0 / 2, owny0 = t.y0 / 2;
  auto put = [&](int q, int r, float v) {
    gt[r * C::GW + q] = v;
    // owned pixels of G_{l+1}: x' in [x0/2, x0/2 + TW/2), y' likewise
    const int xp = gx0 + q, yp = gy0 + r;
    if (xp >= ownx0 && xp < ownx0 + C::TW / 2 && yp >= owny0 && yp < owny0 + C::TH / 2)
      __stwb(B.g + (int64_t)yp * B.pitch + xp, v);
  };
  for (int c = threadIdx.x; c < C::GW * (C::GH / 2); c += C::NT) {
    const int r2 = c / C::GW, q = c - r2 * C::GW;  // constant divisor
    const int r = 2 * r2;
    if (q >= gw || r >= gh) continue;
    const int cx = ncx[q];
    const int2 cy = *reinterpret_cast<const int2 *>(ncy + r);  // rows of samples r and r + 1 (r even)
    const int cy0 = cy.x;
    const bool two = r + 1 < gh;
    const int d = two ? cy.y - cy0 : 0;
    const float *src = stage + cy0 * C::BW + cx;
    float a0, a1 = 0.0f;
    if (d == 2) {
      if (cx & 1) blur_pair<2, true, C::BW>(p.mask, src, a0, a1); else blur_pair<2, false, C::BW>(p.mask, src, a0, a1);
    } else if (d == 3) {
      if (cx & 1) blur_pair<3, true, C::BW>(p.mask, src, a0, a1); else blur_pair<3, false, C::BW>(p.mask, src, a0, a1);
    } else {
      a0 = blur_one<C::BW>(p.mask, src);
      if (two) a1 = blur_one<C::BW>(p.mask, src + d * C::BW);
    }
    put(q, r, a0);
    if (two) put(q, r + 1, a1);
  }
  __syncthreads();
  // ---- L_l = G_l - LF(G_{l+1}): a thread per pair of columns, rows strided;
  // the two columns' arithmetic as packed FP32 (per-lane rounding unchanged)
  const int tx = threadIdx.x % (C::TW / 2);
  const int x = t.x0 + 2 * tx;
  if (x < wl) {
    const LfTap c0 = cols[2 * tx], c1 = cols[2 * tx + 1];
    const f2 cg = f2_pack(c0.g, c1.g), cf = f2_pack(c0.f, c1.f);
    const float *gcol = stage + (x - rx0 + ox);  // even: x and bx0 are even
    const bool pair = x + 1 < wl;
#pragma unroll 1
    for (int r = threadIdx.x / (C::TW / 2); r < C::TH; r += C::NT / (C::TW / 2)) {
      const int y = t.y0 + r;
      if (y >= hl) break;
      const LfTap cy = rows[r];
      const f2 yg = f2_pack(cy.g, cy.g), yf = f2_pack(cy.f, cy.f);
      const f2 wa = f2_mul(cg, yg), wb = f2_mul(cf, yg), wc = f2_mul(cg, yf), wd = f2_mul(cf, yf);
      const float *ga = gt + cy.a * C::GW, *gc = gt + cy.c * C::GW;
      f2 lf = f2_mul(wa, f2_pack(ga[c0.a], ga[c1.a]));
      lf = f2_fma(wb, f2_pack(ga[c0.c], ga[c1.c]), lf);
      lf = f2_fma(wc, f2_pack(gc[c0.a], gc[c1.a]), lf);
      lf = f2_fma(wd, f2_pack(gc[c0.c], gc[c1.c]), lf);
      const float2 g = *reinterpret_cast<const float2 *>(gcol + (y - ry0) * C::BW);
      const f2 v = f2_sub(f2_pack(g.x, g.y), lf);
      float *dst = A.lap + (int64_t)y * A.pitch + x;
      if (pair)
        __stwb(reinterpret_cast<float2 *>(dst), make_float2(f2_lo(v), f2_hi(v)));
      else
        __stwb(dst, f2_lo(v));
    }
  }
  return true;
}

template <class C>
__global__ void __launch_bounds__(C::NT, C::MIN_CTAS) pyr_level_kernel(const __grid_constant__ PyrParams p, int first) {
  __shared__ __align__(128) float stage[C::BW * C::BH];
  __shared__ float gt[C::GW * C::GH];
  __shared__ LfTap cols[C::TW], rows[C::TH];
  __shared__ __align__(8) int ncx[C::GW], ncy[C::GH];
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  unsigned phase = 0;
  pyr_tile<C>(p, p.tiles[first + blockIdx.x], stage, gt, cols, rows, ncx, ncy, &bar, phase, false);
}

// One launch over the whole work-list.  p.single = 0: persistent CTAs (one
// wave) claim tiles until the list ends; p.single = 1: a CTA per tile, each
// claiming one tile when the hardware starts it.  Either way a tile only waits
// on tiles claimed before it, so the claimers of what it waits for are running
// or done.
template <class C, bool TRACE>
__global__ void __launch_bounds__(C::NT, C::MIN_CTAS) pyr_persistent_kernel(const __grid_constant__ PyrParams p) {
  __shared__ __align__(128) float stage[C::BW * C::BH];
  __shared__ float gt[C::GW * C::GH];
  __shared__ LfTap cols[C::TW], rows[C::TH];
  __shared__ __align__(8) int ncx[C::GW], ncy[C::GH];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_t;
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  unsigned phase = 0;
  // single == 2 (a cooperative, co-resident grid): the level-0 tiles, which
  // wait on nothing, are taken round-robin without an atomic; the later levels
  // are claimed.  Otherwise every tile is claimed, kPyClaim consecutive tiles
  // per atomic for persistent CTAs (the claim counter is one address for the
  // whole launch); tiles are processed in list order.
  int claim_base = 0, claim_left = 0;
  int static_next = p.single == 2 ? (int)blockIdx.x : p.nlevel0;
  // the trace record lives in shared memory (thread 0 only), so that it costs
  // the tile loop no registers
  __shared__ PyrTrace tr;
  if (TRACE && threadIdx.x == 0) {
    tr = PyrTrace{};
    tr.t0 = global_ns();
    tr.c0 = clock64();
  }
  auto trace_out = [&]() {
    if (TRACE && threadIdx.x == 0) {
      tr.t1 = global_ns();
      tr.c1 = clock64();
      reinterpret_cast<PyrTrace *>(p.trace)[blockIdx.x] = tr;
    }
  };
  for (;;) {
    if (threadIdx.x == 0) {
      int t;
      if (static_next < p.nlevel0) {
        t = static_next;
        static_next += gridDim.x;
      } else {
        if (claim_left == 0) {
          const int chunk = p.single == 1 ? 1 : kPyClaim;
          if (TRACE) tr.c1 = clock64();
          claim_base = (int)atomicAdd(p.work, (unsigned)chunk) + (p.single == 2 ? p.nlevel0 : 0);
          if (TRACE) tr.claim += clock64() - tr.c1;
          claim_left = chunk;
        }
        t = claim_base++;
        --claim_left;
      }
      s_t = t;
      s_ok = 1;
      if (t < p.ntiles) {
        const PyrTile tl = p.tiles[t];
        if (tl.level > 0) {
          // wait (bounded) until the image's previous level is complete; a
          // failed tile anywhere in the launch ends every wait at once
          const int k = tl.img * p.levels + tl.level - 1;
          const unsigned int need = (unsigned int)p.ntiles_il[k];
          long long spins = 0;
          if (TRACE) tr.c1 = clock64();
          while (ld_acquire_u32(&p.done[k]) < need) {
            if (ld_acquire_u32(p.abort)) {
              s_ok = 0;
              break;
            }
            if (++spins > p.max_polls) {
              s_ok = 0;
              record_status(p.status, HGB_ERR_TIMEOUT);
              atomicExch(p.abort, 1u);
              break;
            }
            __nanosleep(64);
          }
          if (TRACE) {
            tr.wait += clock64() - tr.c1;
            if (spins) tr.counts += 1ll << 32;
          }
        }
        // wait test kind 1: the tile is claimed but never published
        if (s_ok == 1 && tl.level == p.inject_level && p.inject_kind == 1) s_ok = 2;
      }
    }
    __syncthreads();
    const int t = s_t;
    if (t >= p.ntiles || s_ok == 0) {
      trace_out();
      return;
    }
    const PyrTile tl = p.tiles[t];
    if (TRACE && threadIdx.x == 0) tr.c1 = clock64();  // tile start (c1 is final only at exit)
    if (s_ok == 2) {  // uniform: every thread read s_ok after the barrier
      if (p.single == 1) return;
      __syncthreads();  // s_t / s_ok are read before thread 0 claims again
      continue;
    }
    if (!pyr_tile<C>(p, tl, stage, gt, cols, rows, ncx, ncy, &bar, phase, true)) {
      if (threadIdx.x == 0) atomicExch(p.abort, 1u);
      return;
    }
    __syncthreads();
    if (threadIdx.x == 0) red_release_add(&p.done[tl.img * p.levels + tl.level], 1u);
    if (TRACE && threadIdx.x == 0) {
      tr.tile += clock64() - tr.c1;
      tr.counts += 1;
    }
    if (p.single == 1) {
      trace_out();
      return;
    }
  }
}

// ---- reference launch structure: difference with a linear-filtering accessor
__global__ void __launch_bounds__(256) pyr_dog_kernel(LevelMeta A, LevelMeta B) {
  const int x = blockIdx.x * 64 + (threadIdx.x & 63), y = blockIdx.y * 4 + (threadIdx.x >> 6);
  if (x >= A.w || y >= A.h) return;
  const float sx = (float)B.w / (float)A.w, sy = (float)B.h / (float)A.h;
  float xb = __fmaf_rn(sx, (float)x, sx * 0.5f) - 0.5f;
  float yb = __fmaf_rn(sy, (float)y, sy * 0.5f) - 0.5f;
  xb = xb < 0.0f ? 0.0f : xb;
  yb = yb < 0.0f ? 0.0f : yb;
  const int xi = (int)xb, yi = (int)yb;
  const float xf = xb - (float)xi, yf = yb - (float)yi;
  const int xa = min(xi, B.w - 1), xc = min(xi + 1, B.w - 1), ya = min(yi, B.h - 1), yc = min(yi + 1, B.h - 1);
  const float wa = __fmul_rn(1.0f - xf, 1.0f - yf), wb = __fmul_rn(xf, 1.0f - yf);
  const float wc = __fmul_rn(1.0f - xf, yf), wd = __fmul_rn(xf, yf);
  float lf = __fmul_rn(wa, __ldg(B.g + (int64_t)ya * B.pitch + xa));
  lf = __fmaf_rn(wb, __ldg(B.g + (int64_t)ya * B.pitch + xc), lf);
  lf = __fmaf_rn(wc, __ldg(B.g + (int64_t)yc * B.pitch + xa), lf);
  lf = __fmaf_rn(wd, __ldg(B.g + (int64_t)yc * B.pitch + xc), lf);
  A.lap[(int64_t)y * A.pitch + x] = __fsub_rn(__ldg(A.g + (int64_t)y * A.pitch + x), lf);
}

// ---- collapse (Restore): G_l = LF(G_{l+1}) + L_l, one launch per level
__global__ void __launch_bounds__(256) pyr_restore_kernel(const __grid_constant__ PyrParams p, int first) {
  const PyrTile t = p.tiles[first + blockIdx.x];
  const LevelMeta A = p.meta[t.img * p.levels + t.level];
  const LevelMeta B = p.meta[t.img * p.levels + t.level + 1];
  const float sx = (float)B.w / (float)A.w, sy = (float)B.h / (float)A.h;
  for (int c = threadIdx.x; c < PY_TW * PY_TH; c += blockDim.x) {
    const int x = t.x0 + c % PY_TW, y = t.y0 + c / PY_TW;
    if (x >= A.w || y >= A.h) continue;
    float xb = __fmaf_rn(sx, (float)x, sx * 0.5f) - 0.5f;
    float yb = __fmaf_rn(sy, (float)y, sy * 0.5f) - 0.5f;
    xb = xb < 0.0f ? 0.0f : xb;
    yb = yb < 0.0f ? 0.0f : yb;
    const int xi = (int)xb, yi = (int)yb;
    const float xf = xb - (float)xi, yf = yb - (float)yi;
    const int xa = min(xi, B.w - 1), xc = min(xi + 1, B.w - 1), ya = min(yi, B.h - 1), yc = min(yi + 1, B.h - 1);
    const float wa = __fmul_rn(1.0f - xf, 1.0f - yf), wb = __fmul_rn(xf, 1.0f - yf);
    const float wc = __fmul_rn(1.0f - xf, yf), wd = __fmul_rn(xf, yf);
    float lf = __fmul_rn(wa, B.g[(int64_t)ya * B.pitch + xa]);
    lf = __fmaf_rn(wb, B.g[(int64_t)ya * B.pitch + xc], lf);
    lf = __fmaf_rn(wc, B.g[(int64_t)yc * B.pitch + xa], lf);
    lf = __fmaf_rn(wd, B.g[(int64_t)yc * B.pitch + xc], lf);
    A.g[(int64_t)y * A.pitch + x] = __fadd_rn(lf, A.lap[(int64_t)y * A.pitch + x]);
  }
}

}  // namespace
}  // namespace hgb

using namespace hgb;

// Work-list, tensor maps and tile counts of one tile configuration
struct PyrConfigData {
  std::vector<int> level_first;    // first tile of each level in the list
  std::vector<int> level_count;
  CUtensorMap *d_maps = nullptr;   // G_l tensor maps, [img * levels + l]
  PyrTile *d_tiles = nullptr;
  int *d_ntiles = nullptr;         // tiles of level l of image i, [img * levels + l]
  int ntiles = 0;
  int persistent_ctas = 0;
};

struct hgb_pyramid_plan {
  int n = 0, levels = 0, bmode = 0;
  float mask[25];
  std::vector<int> w0, h0;
  std::vector<LevelMeta> meta;     // host copy
  void *arena = nullptr;           // all levels of all images
  void *tmp = nullptr;             // blur buffer of the reference launch structure
  LevelMeta *d_meta = nullptr;
  unsigned int *d_ctrl = nullptr;  // done counters [n*levels] + claim counter + abort flag
  PyrConfigData cfg[kPyCfgs];
  long long max_polls = kMaxSpins;
  int inject_kind = 0, inject_level = 0;
  long long *trace = nullptr;  // device buffer of PyrTrace records (hgb_pyramid_plan_trace)
  long long trace_cap = 0;     // records it holds
};

namespace {

template <class C>
int build_config(hgb_pyramid_plan *P, int c) {
  PyrConfigData &D = P->cfg[c];
  const int n = P->n, levels = P->levels;
  // work-list: levels ascending, then images, then tiles row-major
  std::vector<PyrTile> tiles;
  std::vector<int> nil((size_t)n * levels, 0);
  for (int l = 0; l + 1 < levels; ++l) {
    D.level_first.push_back((int)tiles.size());
    for (int i = 0; i < n; ++i) {
      const LevelMeta &m = P->meta[(size_t)i * levels + l];
      const LevelMeta &mn = P->meta[(size_t)i * levels + l + 1];
      const float Sx = (float)m.w / (float)mn.w, Sy = (float)m.h / (float)mn.h;
      auto nn = [](float S, int v, int lim) {
        const int r = (int)std::fmaf(S, (float)v, S * 0.5f);
        return r < lim ? r : lim - 1;
      };
      for (int y = 0; y < m.h; y += C::TH)
        for (int x = 0; x < m.w; x += C::TW) {
          // the kernel's box origin, with the same single-precision arithmetic
          const int rx0 = nn(Sx, std::max(0, x / 2 - 1), m.w) - 2, ry0 = nn(Sy, std::max(0, y / 2 - 1), m.h) - 2;
          tiles.push_back(PyrTile{i, l, x, y, rx0 & ~3, ry0, 0, 0});
        }
      nil[(size_t)i * levels + l] = cdiv(m.w, C::TW) * cdiv(m.h, C::TH);
    }
    D.level_count.push_back((int)tiles.size() - D.level_first.back());
  }
  D.ntiles = (int)tiles.size();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pyr_persistent_kernel<C, false>, C::NT, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  D.persistent_ctas = num_sms() * per_sm;
  // tensor maps of every Gaussian level a tile stages
  std::vector<CUtensorMap> maps(P->meta.size());
  memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
  for (size_t k = 0; k < P->meta.size(); ++k) {
    if ((int)(k % levels) + 1 >= levels) continue;
    const LevelMeta &m = P->meta[k];
    const int rc = make_tensor_map_3d(&maps[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, m.g, m.w, m.h, 1,
                                      (int64_t)m.pitch * 4, (int64_t)m.pitch * 4 * m.h, C::BW, C::BH);
    if (rc != HGB_OK) return rc;
  }
  cudaError_t e = cudaMalloc((void **)&D.d_tiles, tiles.size() * sizeof(PyrTile));
  if (e == cudaSuccess) e = cudaMalloc((void **)&D.d_ntiles, nil.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void **)&D.d_maps, maps.size() * sizeof(CUtensorMap));
  if (e == cudaSuccess)
    e = cudaMemcpy(D.d_tiles, tiles.data(), tiles.size() * sizeof(PyrTile), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(D.d_ntiles, nil.data(), nil.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(D.d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_error(e, "hgb_pyramid_plan_create: work-list upload");
  return HGB_OK;
}

void free_config(PyrConfigData &D) {
  cudaFree(D.d_maps);
  cudaFree(D.d_tiles);
  cudaFree(D.d_ntiles);
  D.d_maps = nullptr;
  D.d_tiles = nullptr;
  D.d_ntiles = nullptr;
}

}  // namespace

extern "C" {

int hgb_pyramid_plan_create(int n_images, const int *widths, const int *heights, int levels, const float *mask5,
                            int boundary, hgb_pyramid_plan **out) {
  HGB_REQUIRE(out && widths && heights && mask5, "hgb_pyramid_plan_create: null argument");
  HGB_REQUIRE(n_images >= 1 && levels >= 2 && levels <= 16, "hgb_pyramid_plan_create: need >= 1 image, 2..16 levels");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_pyramid_plan_create: bad boundary");
  for (int i = 0; i < n_images; ++i)
    HGB_REQUIRE((widths[i] >> (levels - 1)) >= 1 && (heights[i] >> (levels - 1)) >= 1,
                "hgb_pyramid_plan_create: pyramid stages too deep for an image size");
  hgb_pyramid_plan *P = new hgb_pyramid_plan;
  P->n = n_images;
  P->levels = levels;
  P->bmode = boundary;
  memcpy(P->mask, mask5, sizeof(P->mask));
  P->w0.assign(widths, widths + n_images);
  P->h0.assign(heights, heights + n_images);
  // arena layout: per image, per level: G then L, rows padded to 16 floats
  size_t bytes = 0, tmp_bytes = 0;
  std::vector<size_t> goff, loff;
  P->meta.resize((size_t)n_images * levels);
  for (int i = 0; i < n_images; ++i) {
    int w = widths[i], h = heights[i];
    for (int l = 0; l < levels; ++l) {
      LevelMeta &m = P->meta[(size_t)i * levels + l];
      m.w = w;
      m.h = h;
      m.pitch = (w + 15) / 16 * 16;
      goff.push_back(bytes);
      bytes += (size_t)m.pitch * h * 4;
      loff.push_back(bytes);
      if (l + 1 < levels) bytes += (size_t)m.pitch * h * 4;
      if (l == 0) tmp_bytes = std::max(tmp_bytes, (size_t)m.pitch * h * 4);
      w /= 2;
      h /= 2;
    }
  }
  cudaError_t e = cudaMalloc(&P->arena, bytes);
  if (e == cudaSuccess) e = cudaMemset(P->arena, 0, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&P->tmp, tmp_bytes);
  if (e == cudaSuccess) e = cudaMalloc((void **)&P->d_meta, P->meta.size() * sizeof(LevelMeta));
  if (e == cudaSuccess) e = cudaMalloc((void **)&P->d_ctrl, ((size_t)n_images * levels + 2) * sizeof(unsigned int));
  if (e != cudaSuccess) {
    hgb_pyramid_plan_destroy(P);
    return cuda_error(e, "hgb_pyramid_plan_create: allocation");
  }
  for (size_t k = 0; k < P->meta.size(); ++k) {
    P->meta[k].g = (float *)((char *)P->arena + goff[k]);
    P->meta[k].lap = ((int)(k % levels) + 1 < levels) ? (float *)((char *)P->arena + loff[k]) : nullptr;
  }
  e = cudaMemcpy(P->d_meta, P->meta.data(), P->meta.size() * sizeof(LevelMeta), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    hgb_pyramid_plan_destroy(P);
    return cuda_error(e, "hgb_pyramid_plan_create: upload");
  }
  int rc = build_config<PyCfg0>(P, 0);
  if (rc == HGB_OK) rc = build_config<PyCfg1>(P, 1);
  if (rc == HGB_OK) rc = build_config<PyCfg2>(P, 2);
  if (rc == HGB_OK) rc = build_config<PyCfg3>(P, 3);
  if (rc != HGB_OK) {
    hgb_pyramid_plan_destroy(P);
    return rc;
  }
  *out = P;
  return HGB_OK;
}

int hgb_pyramid_plan_destroy(hgb_pyramid_plan *P) {
  if (!P) return HGB_OK;
  cudaFree(P->arena);
  cudaFree(P->tmp);
  cudaFree(P->d_meta);
  cudaFree(P->d_ctrl);
  for (int c = 0; c < kPyCfgs; ++c) free_config(P->cfg[c]);
  delete P;
  return HGB_OK;
}

int hgb_pyramid_level_view(const hgb_pyramid_plan *P, int image, int level, hgb_view *gauss, hgb_view *lap) {
  HGB_REQUIRE(P, "hgb_pyramid_level_view: null plan");
  HGB_REQUIRE(image >= 0 && image < P->n && level >= 0 && level < P->levels, "hgb_pyramid_level_view: bad index");
  const LevelMeta &m = P->meta[(size_t)image * P->levels + level];
  hgb_view v;
  v.dtype = HGB_F32;
  v.width = m.w;
  v.height = m.h;
  v.batch = 1;
  v.pitch = (int64_t)m.pitch * 4;
  v.batch_stride = v.pitch * m.h;
  if (gauss) {
    *gauss = v;
    gauss->data = m.g;
  }
  if (lap) {
    *lap = v;
    lap->data = m.lap;
  }
  return HGB_OK;
}

static void fill_params(const hgb_pyramid_plan *P, int c, PyrParams *p) {
  memset(p, 0, sizeof(*p));
  const PyrConfigData &D = P->cfg[c];
  p->meta = P->d_meta;
  p->maps = D.d_maps;
  p->tiles = D.d_tiles;
  p->ntiles = D.ntiles;
  p->levels = P->levels;
  p->done = P->d_ctrl;
  p->ntiles_il = D.d_ntiles;
  p->work = P->d_ctrl + (size_t)P->n * P->levels;
  p->abort = p->work + 1;
  p->status = device_status_word();
  p->max_polls = P->max_polls;
  p->inject_kind = P->inject_kind;
  p->inject_level = P->inject_level;
  memcpy(p->mask, P->mask, sizeof(p->mask));
  p->bmode = P->bmode;
}

}  // extern "C"

template <class C>
static int launch_decompose(const hgb_pyramid_plan *P, int c, int mode, int single, cudaStream_t st) {
  const PyrConfigData &D = P->cfg[c];
  PyrParams p;
  fill_params(P, c, &p);
  if (mode == 0) {
    HGB_CHECK_CUDA(cudaMemsetAsync(P->d_ctrl, 0, ((size_t)P->n * P->levels + 2) * sizeof(unsigned int), st));
    p.single = single;
    p.nlevel0 = D.level_count[0];
    const int grid = single == 1 ? D.ntiles : std::min(D.persistent_ctas, D.ntiles);
    p.trace = (P->trace && grid <= P->trace_cap) ? P->trace : nullptr;
    cudaEvent_t ev = before_launch(st);
    // the traced instantiation only when a trace buffer is set (measurement)
    const void *kern =
        p.trace ? (const void *)pyr_persistent_kernel<C, true> : (const void *)pyr_persistent_kernel<C, false>;
    if (single == 2) {
      // co-residency of the whole grid is what makes the static level-0 share
      // safe: a cooperative launch fails instead of running a partial grid
      void *args[] = {(void *)&p};
      HGB_CHECK_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(C::NT), args, 0, st));
    } else if (p.trace) {
      pyr_persistent_kernel<C, true><<<grid, C::NT, 0, st>>>(p);
    } else {
      pyr_persistent_kernel<C, false><<<grid, C::NT, 0, st>>>(p);
    }
    return after_launch("pyr_persistent_kernel", st, ev);
  }
  for (int l = 0; l + 1 < P->levels; ++l) {
    cudaEvent_t ev = before_launch(st);
    pyr_level_kernel<C><<<D.level_count[l], C::NT, 0, st>>>(p, D.level_first[l]);
    const int rc = after_launch("pyr_level_kernel", st, ev);
    if (rc) return rc;
  }
  return HGB_OK;
}

static int launch_cfg(const hgb_pyramid_plan *P, int c, int mode, int single, cudaStream_t st) {
  switch (c) {
    case 1: return launch_decompose<PyCfg1>(P, c, mode, single, st);
    case 2: return launch_decompose<PyCfg2>(P, c, mode, single, st);
    case 3: return launch_decompose<PyCfg3>(P, c, mode, single, st);
    default: return launch_decompose<PyCfg0>(P, c, mode, single, st);
  }
}

extern "C" {

int hgb_pyramid_decompose(hgb_pyramid_plan *P, int mode, void *stream) {
  HGB_REQUIRE(P, "hgb_pyramid_decompose: null plan");
  HGB_REQUIRE(mode >= 0 && mode <= 2, "hgb_pyramid_decompose: mode must be 0, 1 or 2");
  cudaStream_t st = (cudaStream_t)stream;
  if (mode == 0 || mode == 1) {
    // tile configuration (tile shape, threads) and, for the single launch,
    // persistent CTAs or one CTA per tile: autotuned per batch shape
    int64_t px = 0;
    for (int i = 0; i < P->n; ++i) px += (int64_t)P->w0[i] * P->h0[i];
    int lg = 0;
    while ((int64_t(1) << lg) < px) ++lg;
    char key[96];
    snprintf(key, sizeof(key), "pyramid:m%d:n%d:l%d:px2^%d", mode, P->n, P->levels, lg);
    const int ncfg = mode == 0 ? 3 * kPyCfgs : kPyCfgs;
    return autotune_run(key, ncfg, st, [&](int k) {
      return launch_cfg(P, k % kPyCfgs, mode, mode == 0 ? k / kPyCfgs : 0, st);
    });
  }
  PyrParams p;
  fill_params(P, 0, &p);
  // mode 2: the reference's kernels, per image and level
  for (int i = 0; i < P->n; ++i) {
    for (int l = 0; l + 1 < P->levels; ++l) {
      const LevelMeta &A = P->meta[(size_t)i * P->levels + l];
      const LevelMeta &B = P->meta[(size_t)i * P->levels + l + 1];
      hgb_view ga{A.g, HGB_F32, A.w, A.h, 1, (int64_t)A.pitch * 4, (int64_t)A.pitch * 4 * A.h};
      hgb_view tv{P->tmp, HGB_F32, A.w, A.h, 1, (int64_t)A.pitch * 4, (int64_t)A.pitch * 4 * A.h};
      hgb_view gb{B.g, HGB_F32, B.w, B.h, 1, (int64_t)B.pitch * 4, (int64_t)B.pitch * 4 * B.h};
      int rc = hgb_local_op(&ga, nullptr, &tv, nullptr, P->mask, nullptr, nullptr, 5, 5, HGB_REDUCE_SUM, P->bmode, 0.0f,
                            stream);
      if (rc) return rc;
      rc = hgb_resample(&tv, &gb, 1, stream);
      if (rc) return rc;
      cudaEvent_t ev = before_launch(st);
      pyr_dog_kernel<<<dim3(cdiv(A.w, 64), cdiv(A.h, 4)), 256, 0, st>>>(A, B);
      rc = after_launch("pyr_dog_kernel", st, ev);
      if (rc) return rc;
    }
  }
  return HGB_OK;
}

int hgb_pyramid_plan_trace(hgb_pyramid_plan *P, long long *trace_dev, long long capacity) {
  HGB_REQUIRE(P, "hgb_pyramid_plan_trace: null plan");
  HGB_REQUIRE(capacity >= 0 && (trace_dev != nullptr || capacity == 0), "hgb_pyramid_plan_trace: bad buffer");
  P->trace = trace_dev;
  P->trace_cap = capacity;
  return HGB_OK;
}

int hgb_pyramid_plan_wait_test(hgb_pyramid_plan *P, long long max_polls, int kind, int level) {
  HGB_REQUIRE(P, "hgb_pyramid_plan_wait_test: null plan");
  HGB_REQUIRE(max_polls >= 0, "hgb_pyramid_plan_wait_test: negative poll limit");
  HGB_REQUIRE(kind >= 0 && kind <= 2, "hgb_pyramid_plan_wait_test: kind must be 0, 1 or 2");
  HGB_REQUIRE(level >= 0 && level + 1 < P->levels, "hgb_pyramid_plan_wait_test: level has no tiles");
  P->max_polls = max_polls > 0 ? max_polls : kMaxSpins;
  P->inject_kind = kind;
  P->inject_level = level;
  return HGB_OK;
}

int hgb_pyramid_collapse(hgb_pyramid_plan *P, void *stream) {
  HGB_REQUIRE(P, "hgb_pyramid_collapse: null plan");
  cudaStream_t st = (cudaStream_t)stream;
  PyrParams p;
  fill_params(P, 0, &p);
  for (int l = P->levels - 2; l >= 0; --l) {
    cudaEvent_t ev = before_launch(st);
    pyr_restore_kernel<<<P->cfg[0].level_count[l], 256, 0, st>>>(p, P->cfg[0].level_first[l]);
    const int rc = after_launch("pyr_restore_kernel", st, ev);
    if (rc) return rc;
  }
  return HGB_OK;
}

}  // extern "C"
