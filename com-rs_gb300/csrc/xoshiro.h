// The xoshiro256** generator of crates/com-core/src/rng.rs, bit-identical, for kernels
// and for host code (the progressive-edge-growth construction draws from it too).
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define CB_HD __host__ __device__ __forceinline__
#else
#define CB_HD inline
#endif

namespace cbd {

// rng.rs:49-117, :270-278
struct Xoshiro {
  uint64_t s0, s1, s2, s3;
};

CB_HD uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

CB_HD uint64_t splitmix64(uint64_t& st) {
  st += 0x9E3779B97F4A7C15ull;
  uint64_t z = st;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

CB_HD Xoshiro xoshiro_seed(uint64_t seed) {
  Xoshiro r;
  uint64_t st = seed;
  r.s0 = splitmix64(st);
  r.s1 = splitmix64(st);
  r.s2 = splitmix64(st);
  r.s3 = splitmix64(st);
  return r;
}

// stream(base_seed, experiment, condition, trial) with the experiment already hashed
CB_HD Xoshiro stream(uint64_t base_seed, uint64_t name_hash, uint64_t cond, uint64_t trial) {
  uint64_t st = base_seed ^ name_hash;
  uint64_t a = splitmix64(st);
  st = a ^ cond;
  uint64_t b = splitmix64(st);
  st = b ^ trial;
  return xoshiro_seed(splitmix64(st));
}

CB_HD void xoshiro_advance(Xoshiro& r) {
  uint64_t t = r.s1 << 17;
  r.s2 ^= r.s0;
  r.s3 ^= r.s1;
  r.s1 ^= r.s2;
  r.s0 ^= r.s3;
  r.s2 ^= t;
  r.s3 = rotl64(r.s3, 45);
}

CB_HD uint64_t xoshiro_next(Xoshiro& r) {
  uint64_t result = rotl64(r.s1 * 5, 7) * 9;
  xoshiro_advance(r);
  return result;
}

// Rng::uniform (rng.rs:115-117): the top 53 bits over 2^53
CB_HD double xoshiro_uniform(Xoshiro& r) { return (double)(xoshiro_next(r) >> 11) * (1.0 / 9007199254740992.0); }

// Rng::below (rng.rs:125-128): floor(uniform * n), at most n - 1
CB_HD uint64_t xoshiro_below(Xoshiro& r, uint64_t n) {
  const uint64_t v = (uint64_t)(xoshiro_uniform(r) * (double)n);
  return v < n - 1 ? v : n - 1;
}

}  // namespace cbd
