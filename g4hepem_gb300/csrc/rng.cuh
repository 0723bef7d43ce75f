// rng.cuh -- per-track uniform streams on the device.
//
// Replaces the consumer-supplied G4HepEmRandomEngine::flat()/flatArray()
// (reference G4HepEm/G4HepEmRun/include/G4HepEmRandomEngine.hh:40-51) and
// carries its Gauss cache (:50-70) and Poisson sampler (:74-97) as per-track
// state.  Stream k of track `id`: uniforms[k] while k < n, then
// Philox4x32-10 (Salmon et al., SC'11) at counter (k>>1, id, 0, 0x48455045),
// key = seed, which is also how the buffer is meant to be filled.
#pragma once

#include <cstdint>
#include <cstring>

#include "vdt.cuh"

namespace hepem {

__host__ __device__ __forceinline__ void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                                       uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// (bits52 + 0.5) 2^-52 = (2 bits52 + 1) 2^-53 exactly, built from its bits
// (integer operations only: no integer-to-FP64 conversion, no FP64 multiply)
__host__ __device__ __forceinline__ double u52_to_double(uint64_t bits52) {
  const uint64_t v = 2 * bits52 + 1;  // odd, < 2^53
#ifdef __CUDA_ARCH__
  const int p = 63 - __clzll((long long)v);
#else
  const int p = 63 - __builtin_clzll(v);
#endif
  const uint64_t bits = ((uint64_t)(p - 53 + 1023) << 52) | ((v << (52 - p)) & 0xFFFFFFFFFFFFFull);
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)bits);
#else
  double d;
  memcpy(&d, &bits, sizeof d);
  return d;
#endif
}

__host__ __device__ __forceinline__ double philox_uniform(uint64_t seed, int32_t id, int32_t k) {
  uint32_t c0 = (uint32_t)k >> 1, c1 = (uint32_t)id, c2 = 0u, c3 = 0x48455045u;
  philox4x32_10(c0, c1, c2, c3, (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint32_t a = (k & 1) ? c2 : c0;
  const uint32_t b = (k & 1) ? c3 : c1;
  return u52_to_double(((uint64_t)a << 20) | (uint64_t)(b >> 12));
}


struct Rng {
  const double* u;        // this track's buffered stream
  int32_t n;              // buffered length
  int32_t cursor;         // next index
  int32_t id;
  uint32_t overflow;      // read past the buffer
  uint64_t seed;
  bool gaussValid;
  double gaussValue;
  // u holds the stream's first n values drawn ahead by the library (the
  // caller passed no uniforms): every draw still counts as past the caller's
  // buffer, as if drawn here
  bool filled = false;

  __device__ __forceinline__ double flat() {
    double v;
    if (cursor < n) {
      v = __ldg(u + cursor);
      if (filled) overflow = 1u;
    } else {
      overflow = 1u;
      v = philox_uniform(seed, id, cursor);
    }
    ++cursor;
    return v;
  }
  __device__ __forceinline__ void flat2(double* v) { v[0] = flat(); v[1] = flat(); }
  __device__ __forceinline__ void flat3(double* v) { v[0] = flat(); v[1] = flat(); v[2] = flat(); }

  // polar Marsaglia with cached second value (G4HepEmRandomEngine.hh:50-67)
  __device__ double gauss(double mean, double sd) {
    if (gaussValid) {
      gaussValid = false;
      return gaussValue * sd + mean;
    }
    double r, v1, v2;
    do {
      const double a = flat(), b = flat();
      v1 = 2. * a - 1.;
      v2 = 2. * b - 1.;
      r = v1 * v1 + v2 * v2;
    } while (r > 1.);
    const double fac = sqrt(-2. * vdt_log(r) / r);
    gaussValue = v1 * fac;
    gaussValid = true;
    return v2 * fac * sd + mean;
  }

  // G4HepEmRandomEngine.hh:74-97
  __device__ int poisson(double mean) {
    int number = 0;
    if (mean <= 16) {
      const double position = flat();
      double pv = vdt_exp(-mean);
      double ps = pv;
      while (ps <= position) {
        ++number;
        pv *= mean / number;
        ps += pv;
      }
      return number;
    }
    const double a = flat(), b = flat();
    const double t = sqrt(-2. * vdt_log(a)) * cos(6.2831853071795862 * b);
    const double value = mean + t * sqrt(mean) + 0.5;
    return value < 0. ? 0 : value >= 2.E+9 ? (int)2.E+9 : (int)value;
  }
};

}  // namespace hepem
