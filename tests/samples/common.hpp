// Shared helpers of the sample programs (seeded inputs, comparisons).
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

inline std::vector<float> random_floats(int n, unsigned seed) {
  std::mt19937_64 g(seed);
  std::uniform_real_distribution<float> d(0.0f, 1.0f);
  std::vector<float> v((size_t)n);
  for (auto &x : v) x = d(g);
  return v;
}
inline std::vector<unsigned char> random_bytes(int n, unsigned seed) {
  std::mt19937_64 g(seed);
  std::uniform_int_distribution<int> d(0, 255);
  std::vector<unsigned char> v((size_t)n);
  for (auto &x : v) x = (unsigned char)d(g);
  return v;
}
inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline int mirror(int v, int n) {
  while (v < 0 || v >= n) {
    if (v >= n) v = n - (v + 1 - n);
    if (v < 0) v = -v - 1;
  }
  return v;
}
#define REQUIRE(c)                                                      \
  do {                                                                  \
    if (!(c)) {                                                         \
      std::fprintf(stderr, "Test FAILED: %s (line %d)\n", #c, __LINE__); \
      std::exit(1);                                                     \
    }                                                                   \
  } while (0)
