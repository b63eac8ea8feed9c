#pragma once
// TEST INFRASTRUCTURE ONLY.  The reference renderer's curand calls
// (mpm/csrc/integrator.cu:1309-1373), served by the counter-based generator
// the product's renderer uses: SplitMix64 (Steele, Lea & Flood, OOPSLA 2014)
// of (seed, subsequence) as the key, one more SplitMix64 per draw of
// key + draw_index * 0x9E3779B97F4A7C15, 24 bits mapped to (0, 1].
#include <stdint.h>
struct curandState {
  unsigned long long key, ctr;
};
static inline unsigned long long dex_splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline void curand_init(unsigned long long seed, unsigned long long subsequence, unsigned long long offset,
                        curandState *st) {
  st->key = dex_splitmix64(((unsigned long long)(uint32_t)seed << 32) ^ (unsigned long long)(uint32_t)subsequence);
  st->ctr = offset;
}
inline float curand_uniform(curandState *st) {
  ++st->ctr;
  const unsigned long long h = dex_splitmix64(st->key + st->ctr * 0x9E3779B97F4A7C15ull);
  return (float)((h >> 40) + 1ull) * (1.f / 16777216.f);
}
