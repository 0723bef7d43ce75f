/*
 * philox.h -- TEST INFRASTRUCTURE (oracle).  Counter-based Philox4x32-10
 * generator (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11), written from the published
 * round function.  Defines the per-track uniform stream shared by the
 * reference harness and the CPU port:
 *   counter = (k >> 1, track id, 0, 0x48455045), key = (seed lo, seed hi);
 *   uniform = (52 random bits + 0.5) * 2^-52, from words (0,1) for even k and
 *   words (2,3) for odd k.
 */
#ifndef HEPEM_ORACLE_PHILOX_H
#define HEPEM_ORACLE_PHILOX_H

#include <stdint.h>

static inline void oracle_philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * c[0];
    const uint64_t p1 = (uint64_t)M1 * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += W0; k1 += W1;
  }
}

static inline double oracle_philox_uniform(uint64_t seed, int32_t id, int32_t k) {
  uint32_t c[4] = {(uint32_t)k >> 1, (uint32_t)id, 0u, 0x48455045u};
  oracle_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint32_t a = (k & 1) ? c[2] : c[0];
  const uint32_t b = (k & 1) ? c[3] : c[1];
  const uint64_t bits52 = ((uint64_t)a << 20) | (uint64_t)(b >> 12);
  return ((double)bits52 + 0.5) * (1.0 / 4503599627370496.0);
}

#endif
