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

#include <cstdint>

namespace hepem {

__device__ __forceinline__ double vdt_log(double x) {
  const double x0 = x;
  uint64_t n = (uint64_t)__double_as_longlong(x);
  double fe = (double)((int32_t)(n >> 52) - 1023);
  n = (n & 0x800FFFFFFFFFFFFFULL) | 0x3FE0000000000000ULL;
  x = __longlong_as_double((long long)n);
  if (x > 0.70710678118654752440) fe += 1.0; else x += x;
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
  if (x0 > 1e307) res = __longlong_as_double(0x7FF0000000000000LL);
  if (x0 < 0) res = __longlong_as_double((long long)0xFFF8000000000000ULL);
  return res;
}

__device__ __forceinline__ double vdt_exp(double x0) {
  double x = x0;
  const double t = __dadd_rn(__dmul_rn(1.4426950408889634073599, x), 0.5);
  // floor as the reference computes it: truncate, minus the sign bit of (float)t
  int32_t fl = __double2int_rz(t);
  fl -= (int32_t)(((uint32_t)__float_as_uint(__double2float_rn(t))) >> 31);
  double px = (double)fl;
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
  if (x0 > 708) x = __longlong_as_double(0x7FF0000000000000LL);
  if (x0 < -708) x = 0.;
  return x;
}

__device__ __forceinline__ double vdt_pow(double x, double a) { return vdt_exp(__dmul_rn(a, vdt_log(x))); }

}  // namespace hepem
