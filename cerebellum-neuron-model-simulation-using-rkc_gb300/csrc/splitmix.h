// Counter-based uniform draws: the SplitMix64 finaliser (Steele, Lea & Flood
// 2014) over a seed, an index and a counter, as a double in (0, 1] like
// curand_uniform.  Used for the mossy fibres' Poisson draws and for the
// Purkinje target draws of the reference's wiring rules; the oracle carries
// the same formula.
#pragma once

#ifdef __CUDACC__
#define GBRKC_HD __host__ __device__
#else
#define GBRKC_HD
#endif

namespace gbrkc {

GBRKC_HD inline double splitmix_uniform(unsigned long long seed, long long id, long long counter) {
  unsigned long long z = seed ^ ((unsigned long long)id * 0xD1B54A32D192ED03ull) ^
                         ((unsigned long long)counter * 0x9E3779B97F4A7C15ull);
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)((z >> 11) + 1ull) * 0x1p-53;
}

}  // namespace gbrkc
