// crand.h -- the C library's rand() stream (glibc: random() with its default
// state), restated so that a device loop draws exactly the numbers the
// reference's randomReal (MathLibrary.cpp:27-33: srand(seed), rand()) draws.
//
// The generator is the additive feedback generator of BSD random(3) in its
// degree-31 form: 31 words r[], a front index f and a rear index b three
// apart; each output adds r[b] into r[f] (mod 2^32) and returns that word
// shifted right by one (31 bits), then both indexes advance around the ring.
// Seeding (srandom) fills r[0] = seed (1 for a zero seed) and
// r[i] = 16807 r[i-1] mod (2^31 - 1) by Schrage's decomposition
// (127773 = (2^31 - 1) / 16807, 2836 = (2^31 - 1) mod 16807), sets f = 3,
// b = 0 and discards the first 310 outputs.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define MCGPU_HD __host__ __device__ __forceinline__
#else
#define MCGPU_HD inline
#endif

namespace mcgpu {

struct CRand {
  int32_t r[31];
  int32_t f, b;
};

MCGPU_HD int32_t crand_next(CRand& g) {
  const uint32_t v = (uint32_t)g.r[g.f] + (uint32_t)g.r[g.b];
  g.r[g.f] = (int32_t)v;
  if (++g.f >= 31) {
    g.f = 0;
    ++g.b;
  } else if (++g.b >= 31) {
    g.b = 0;
  }
  return (int32_t)(v >> 1);
}

inline void crand_seed(CRand& g, unsigned int seed) {
  if (seed == 0) seed = 1;
  int32_t word = (int32_t)seed;
  g.r[0] = word;
  for (int i = 1; i < 31; i++) {
    const long long hi = word / 127773, lo = word % 127773;
    long long w = 16807 * lo - 2836 * hi;
    if (w < 0) w += 2147483647;
    word = (int32_t)w;
    g.r[i] = word;
  }
  g.f = 3;
  g.b = 0;
  for (int k = 0; k < 310; k++) (void)crand_next(g);
}

}  // namespace mcgpu
