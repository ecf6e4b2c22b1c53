// ckr_rng.h — counter-based random numbers shared by host and device code.
//
// The reference seeds a Mersenne Twister from clock() at every call site
// (src/random.cpp:104, src/domainSampler.cpp:55), so its streams cannot be
// reproduced.  This library replaces it with a stateless hash: every random
// number is a pure function of (seed, pixel or ray index, counter), which
// makes GPU and CPU consume identical streams and makes renders resumable.
//
// Mixer: the splitmix64 finaliser (Steele, Lea, Flood 2014).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CKR_HD __host__ __device__ __forceinline__
#else
#define CKR_HD inline
#endif

CKR_HD uint64_t ckr_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Stream key for (seed, index), e.g. the per-pixel seed hash(seed, pixel).
CKR_HD uint64_t ckr_key(uint64_t seed, uint64_t index) {
  return ckr_mix64(seed * 0x9E3779B97F4A7C15ull + ckr_mix64(index + 0x632BE59BD9B4E019ull));
}

// The counter-th 32-bit draw of a stream.
CKR_HD uint32_t ckr_draw_u32(uint64_t key, uint32_t counter) {
  return (uint32_t)(ckr_mix64(key + (uint64_t)(counter + 1u) * 0xD1B54A32D192ED03ull) >> 32);
}

// Uniform in [0, 1) with 24 bits: exactly representable in FP32 and FP64, so
// the FP64 oracle and the FP32 kernels see the same value.
CKR_HD float ckr_draw_f(uint64_t key, uint32_t counter) {
  return (float)(ckr_draw_u32(key, counter) >> 8) * (1.0f / 16777216.0f);
}
