// vdt.cuh -- log / exp by the VDT (Cephes) Pade method, in device code.
//
// The reference evaluates G4HepEmLog / G4HepEmExp / G4HepEmPow on the host
// with the VDT method (G4HepEm/G4HepEmRun/include/G4HepEmLog.hh:228-271,
// G4HepEmExp.hh:182-226, G4HepEmMath.hh:37-88): frexp-style mantissa/exponent
// split, a rational (Pade) approximation and a two-constant ln2 reduction.
// Device code here evaluates the same published method with the same
// coefficients and operation order, one IEEE-rounded operation at a time
// (files including this one are compiled with --fmad=false), so the results
// are bit-identical to the reference host values.  The coefficient tables are
// the published Cephes / VDT 0.3.7 ones and must match the reference exactly.
#pragma once

#include <climits>
#include <cstdint>

namespace hepem {

// On GB300 every FP64 instruction -- conversions and comparisons included --
// takes FP64-pipe time, which the FP64 step is short of.  The helpers below
// do the exact ones with integer operations and give the same results bit
// for bit as the conversion and comparison instructions they replace.

// (double)k, exactly, from the bits
__device__ __forceinline__ double int_to_double_exact(int32_t k) {
  if (k == 0) return 0.0;
  const uint32_t a = k < 0 ? (uint32_t)(-(int64_t)k) : (uint32_t)k;
  const int e = 31 - __clz(a);  // 2^e <= a < 2^(e+1)
  const uint64_t mant = ((uint64_t)a << (52 - e)) & 0xFFFFFFFFFFFFFull;
  return __longlong_as_double((long long)(((uint64_t)(k < 0) << 63) | ((uint64_t)(1023 + e) << 52) | mant));
}

// truncation toward zero to int32 as cvt.rzi.s32.f64 does it (saturating;
// NaN gives 0)
__device__ __forceinline__ int32_t double_to_int_rz_exact(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  const bool neg = (b >> 63) != 0;
  if (e < 0) return 0;
  if (e == 1024 && (b & 0xFFFFFFFFFFFFFull)) return 0;
  if (e >= 31) return neg ? INT32_MIN : INT32_MAX;
  const int32_t t = (int32_t)(((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) >> (52 - e));
  return neg ? -t : t;
}

// x > c and x < -c for a finite constant c > 0, as the FP64 comparisons
// (false for NaN)
__device__ __forceinline__ bool dgreater_const(double x, double c) {
  const long long b = __double_as_longlong(x);
  return b > __double_as_longlong(c) && b <= 0x7FF0000000000000LL;
}
__device__ __forceinline__ bool dless_neg_const(double x, double c) {
  const long long b = __double_as_longlong(x);
  const long long m = b & 0x7FFFFFFFFFFFFFFFLL;
  return b < 0 && m > __double_as_longlong(c) && m <= 0x7FF0000000000000LL;
}

__device__ __forceinline__ double vdt_log(double x) {
  const double x0 = x;
  uint64_t n = (uint64_t)__double_as_longlong(x);
  int32_t ei = (int32_t)(n >> 52) - 1023;
  n = (n & 0x800FFFFFFFFFFFFFULL) | 0x3FE0000000000000ULL;
  // x = n in [0.5, 1) with the sign of x0; x > 1/sqrt(2) on the bits, and
  // x += x as one more in the exponent (exact)
  if ((long long)n > __double_as_longlong(0.70710678118654752440))
    ei += 1;
  else
    n += 1ull << 52;
  x = __longlong_as_double((long long)n);
  const double fe = int_to_double_exact(ei);
  x -= 1.0;
  double px = 1.01875663804580931796E-4;
  px = __dadd_rn(__dmul_rn(px, x), 4.97494994976747001425E-1);
  px = __dadd_rn(__dmul_rn(px, x), 4.70579119878881725854E0);
  px = __dadd_rn(__dmul_rn(px, x), 1.44989225341610930846E1);
  px = __dadd_rn(__dmul_rn(px, x), 1.79368678507819816313E1);
  px = __dadd_rn(__dmul_rn(px, x), 7.70838733755885391666E0);
  const double x2 = __dmul_rn(x, x);
  px = __dmul_rn(px, x);
  px = __dmul_rn(px, x2);
  double qx = __dadd_rn(x, 1.12873587189167450590E1);
  qx = __dadd_rn(__dmul_rn(qx, x), 4.52279145837532221105E1);
  qx = __dadd_rn(__dmul_rn(qx, x), 8.29875266912776603211E1);
  qx = __dadd_rn(__dmul_rn(qx, x), 7.11544750618563894466E1);
  qx = __dadd_rn(__dmul_rn(qx, x), 2.31251620126765340583E1);
  double res = __ddiv_rn(px, qx);
  res = __dsub_rn(res, __dmul_rn(fe, 2.121944400546905827679e-4));
  res = __dsub_rn(res, __dmul_rn(0.5, x2));
  res = __dadd_rn(x, res);
  res = __dadd_rn(res, __dmul_rn(fe, 0.693359375));
  const long long b0 = __double_as_longlong(x0);
  if (dgreater_const(x0, 1e307)) res = __longlong_as_double(0x7FF0000000000000LL);
  // x0 < 0: negative, not -0 and not NaN
  if (b0 < 0 && (b0 & 0x7FFFFFFFFFFFFFFFLL) != 0 && (b0 & 0x7FFFFFFFFFFFFFFFLL) <= 0x7FF0000000000000LL)
    res = __longlong_as_double((long long)0xFFF8000000000000ULL);
  return res;
}

__device__ __forceinline__ double vdt_exp(double x0) {
  double x = x0;
  const double t = __dadd_rn(__dmul_rn(1.4426950408889634073599, x), 0.5);
  // floor as the reference computes it: truncate, minus the sign bit of
  // (float)t, which is the sign bit of t
  int32_t fl = double_to_int_rz_exact(t);
  fl -= (int32_t)((uint64_t)__double_as_longlong(t) >> 63);
  double px = int_to_double_exact(fl);
  const int32_t n = fl;
  x = __dsub_rn(x, __dmul_rn(px, 6.93145751953125E-1));
  x = __dsub_rn(x, __dmul_rn(px, 1.42860682030941723212E-6));
  const double xx = __dmul_rn(x, x);
  px = 1.26177193074810590878E-4;
  px = __dmul_rn(px, xx);
  px = __dadd_rn(px, 3.02994407707441961300E-2);
  px = __dmul_rn(px, xx);
  px = __dadd_rn(px, 9.99999999999999999910E-1);
  px = __dmul_rn(px, x);
  double qx = 3.00198505138664455042E-6;
  qx = __dmul_rn(qx, xx);
  qx = __dadd_rn(qx, 2.52448340349684104192E-3);
  qx = __dmul_rn(qx, xx);
  qx = __dadd_rn(qx, 2.27265548208155028766E-1);
  qx = __dmul_rn(qx, xx);
  qx = __dadd_rn(qx, 2.00000000000000000009E0);
  x = __ddiv_rn(px, __dsub_rn(qx, px));
  x = __dadd_rn(1.0, __dmul_rn(2.0, x));
  x = __dmul_rn(x, __longlong_as_double((long long)((((uint64_t)(int64_t)n) + 1023) << 52)));
  if (dgreater_const(x0, 708.0)) x = __longlong_as_double(0x7FF0000000000000LL);
  if (dless_neg_const(x0, 708.0)) x = 0.;
  return x;
}

__device__ __forceinline__ double vdt_pow(double x, double a) { return vdt_exp(__dmul_rn(a, vdt_log(x))); }

}  // namespace hepem
