// Counter-based random numbers shared bit-for-bit by the CUDA kernels and the
// CPU oracle.
//
// Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11): a 10-round
// multiply/xor network over a 128-bit counter and a 64-bit key.  Each MC trial
// draws from counter (trial_lo, trial_hi, lane, 0) under key (seed_lo, seed_hi
// ^ chain), so a trial's proposal and uniform depend only on (seed, chain,
// trial) and never on how trials are scheduled.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CEMC_HD __host__ __device__ __forceinline__
#else
#define CEMC_HD static inline
#endif

typedef struct {
  uint32_t v[4];
} cemc_u32x4;

CEMC_HD uint32_t cemc_mulhi32(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}

CEMC_HD cemc_u32x4 cemc_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                       uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#if defined(__CUDACC__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * c0;
    const uint64_t p1 = (uint64_t)M1 * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  cemc_u32x4 out;
  out.v[0] = c0;
  out.v[1] = c1;
  out.v[2] = c2;
  out.v[3] = c3;
  return out;
}

// Uniform double in [0, 1) with 53 random bits from two words.
CEMC_HD double cemc_u01_53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Uniform integer in [0, n) by multiply-high (exact, identical on CPU and GPU).
CEMC_HD uint32_t cemc_below(uint32_t w, uint32_t n) { return cemc_mulhi32(w, n); }

// Draws of one trial.  lane 0 carries the site/symbol choices, lane 1 the
// second site of a swap and the Metropolis uniform of a swap.
CEMC_HD cemc_u32x4 cemc_trial_draw(uint64_t seed, uint32_t chain, uint64_t trial, uint32_t lane) {
  return cemc_philox4x32_10((uint32_t)trial, (uint32_t)(trial >> 32), lane, 0u, (uint32_t)seed,
                            (uint32_t)(seed >> 32) ^ chain);
}
