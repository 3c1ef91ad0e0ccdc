// rmat_hash.hpp — the counter-based R-MAT draw shared by the host generator
// (rmat.cpp) and the device generator (rmat_gpu.cu).  Everything is integer
// arithmetic, so both produce the same edge multiset on x86 and Arm.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define OG_HD __host__ __device__ __forceinline__
#else
#define OG_HD inline
#endif

namespace og {

// splitmix64 finaliser (Steele, Lea, Flood 2014).
OG_HD uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

struct RmatDraw {
  uint32_t scale;
  uint32_t t1, t2, t3;  // a, a+b, a+b+c scaled to 2^32
  uint64_t seed;
  uint64_t pmul[3], padd[3];  // permutation constants (odd multipliers)
  bool permute;

  // Edge tuple i: `scale` quadrant choices, two per 64-bit hash.
  OG_HD void tuple(uint64_t i, uint32_t &u, uint32_t &v) const {
    const uint64_t base = mix64(seed + (i + 1) * 0x9e3779b97f4a7c15ull);
    uint32_t a = 0, b = 0;
    uint64_t h = 0;
    for (uint32_t l = 0; l < scale; l++) {
      uint32_t r;
      if ((l & 1) == 0) {
        h = mix64(base + (uint64_t)(l + 1) * 0xd1b54a32d192ed03ull);
        r = (uint32_t)h;
      } else {
        r = (uint32_t)(h >> 32);
      }
      const uint32_t ub = r >= t2;                   // quadrants c, d: lower half
      const uint32_t vb = (r >= t1 && r < t2) || r >= t3;  // quadrants b, d: right half
      a = (a << 1) | ub;
      b = (b << 1) | vb;
    }
    if (permute) {
      a = perm(a);
      b = perm(b);
    }
    u = a;
    v = b;
  }

  // Bijection on [0, 2^scale): odd multiply, xor-shift, add (each invertible mod 2^scale).
  OG_HD uint32_t perm(uint32_t x) const {
    if (scale == 0) return x;
    const uint64_t m = (scale >= 64) ? ~0ull : ((1ull << scale) - 1);
    const uint32_t sh = (scale + 1) / 2;
    uint64_t y = x;
    for (int r = 0; r < 3; r++) {
      y = (y * pmul[r]) & m;
      y ^= y >> sh;
      y = (y + padd[r]) & m;
    }
    return (uint32_t)y;
  }
};

inline RmatDraw make_rmat_draw(uint32_t scale, double a, double b, double c,
                               uint64_t seed, bool permute) {
  RmatDraw d;
  d.scale = scale;
  auto thr = [](double p) -> uint32_t {
    if (p <= 0) return 0;
    if (p >= 1) return 0xFFFFFFFFu;
    return (uint32_t)(p * 4294967296.0);
  };
  d.t1 = thr(a);
  d.t2 = thr(a + b);
  d.t3 = thr(a + b + c);
  d.seed = seed;
  d.permute = permute;
  for (int r = 0; r < 3; r++) {
    d.pmul[r] = mix64(seed ^ (0x5851f42d4c957f2dull + (uint64_t)r)) | 1ull;
    d.padd[r] = mix64(seed ^ (0x14057b7ef767814full + 7ull * (uint64_t)r));
  }
  return d;
}

// Weight of the undirected edge {u, v}: the same in both directions.
OG_HD uint32_t edge_weight(uint64_t wseed, uint32_t u, uint32_t v, uint32_t wmin,
                           uint32_t wmax) {
  const uint32_t lo = u < v ? u : v, hi = u < v ? v : u;
  const uint64_t h = mix64(wseed ^ mix64(((uint64_t)lo << 32) | hi));
  const uint64_t range = (uint64_t)wmax - wmin + 1;
  return wmin + (uint32_t)(h % range);
}

}  // namespace og
