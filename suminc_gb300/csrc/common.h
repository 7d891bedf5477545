// Shared host/device definitions: status plumbing, the counter-based hash
// used by every generator, the R-MAT edge draw and the edge-weight rule.
// Host and device evaluate the same integer arithmetic, so the GPU generator
// and the host generator produce identical graphs.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define SG_HD __host__ __device__ __forceinline__
#else
#define SG_HD inline
#endif

namespace sg {

constexpr uint32_t kInvalidVid = 0xFFFFFFFFu;

// splitmix64 finaliser (Steele, Lea, Flood: "Fast splittable pseudorandom
// number generators", OOPSLA 2014).
SG_HD uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// R-MAT quadrant thresholds on a 24-bit uniform integer.
struct RmatParams {
  uint64_t seed_key;  // mix64(seed ^ const)
  uint32_t ta, tab, tabc;
  int scale;
};

inline RmatParams make_rmat_params(int scale, double a, double b, double c,
                                   uint64_t seed) {
  RmatParams p;
  p.seed_key = mix64(seed ^ 0x5851F42D4C957F2Dull);
  const double s = 16777216.0;
  p.ta = (uint32_t)(a * s);
  p.tab = (uint32_t)((a + b) * s);
  p.tabc = (uint32_t)((a + b + c) * s);
  p.scale = scale;
  return p;
}

// Draw number i of the R-MAT stream: s levels of quadrant descent, most
// significant bit first, two 24-bit uniforms per 64-bit hash.  Returns
// (src << 32) | dst.  Quadrants: a -> (0,0), b -> (0,1), c -> (1,0),
// d -> (1,1) (Chakrabarti, Zhan, Faloutsos, SDM 2004).
SG_HD uint64_t rmat_draw(const RmatParams& p, uint64_t i) {
  uint32_t s = 0, d = 0;
  uint64_t h = 0;
  for (int l = 0; l < p.scale; ++l) {
    uint32_t r;
    if ((l & 1) == 0) {
      h = mix64(p.seed_key + i * 32u + (uint64_t)(l >> 1));
      r = (uint32_t)(h >> 40);
    } else {
      r = (uint32_t)((h >> 16) & 0xFFFFFFu);
    }
    uint32_t sb, db;
    if (r < p.ta) {
      sb = 0; db = 0;
    } else if (r < p.tab) {
      sb = 0; db = 1;
    } else if (r < p.tabc) {
      sb = 1; db = 0;
    } else {
      sb = 1; db = 1;
    }
    s = (s << 1) | sb;
    d = (d << 1) | db;
  }
  return ((uint64_t)s << 32) | d;
}

// Edge weight as a pure function of (weight seed, src, dst), so it does not
// depend on draw order.  kind 1: integer U[lo,hi]; kind 2: float U[lo,hi].
struct WeightParams {
  uint64_t key;
  int kind;
  double lo, hi;
  uint32_t span;  // integer kind: hi - lo + 1
};

inline WeightParams make_weight_params(uint64_t seed, int kind, double lo,
                                       double hi) {
  WeightParams w;
  w.key = mix64(seed ^ 0xD1B54A32D192ED03ull);
  w.kind = kind;
  w.lo = lo;
  w.hi = hi;
  w.span = kind == 1 ? (uint32_t)(hi - lo + 1.0) : 0u;
  return w;
}

SG_HD float edge_weight(const WeightParams& wp, uint64_t edge_key) {
  const uint64_t h = mix64(wp.key ^ edge_key);
  if (wp.kind == 1) {
    return (float)(wp.lo + (double)(h % wp.span));
  }
  // float kind: lo + (hi - lo) * u, u = 24-bit fraction; both roundings are
  // explicit so the host and device agree bit for bit.
  const double u = (double)(h >> 40) * (1.0 / 16777216.0);
#ifdef __CUDA_ARCH__
  const double v = __dadd_rn(wp.lo, __dmul_rn(wp.hi - wp.lo, u));
#else
  volatile double prod = (wp.hi - wp.lo) * u;  // no fused multiply-add
  const double v = wp.lo + prod;
#endif
  return (float)v;
}

}  // namespace sg
