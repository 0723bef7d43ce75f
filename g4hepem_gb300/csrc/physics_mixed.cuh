// physics_mixed.cuh -- the precision form: the e+- stage A (HowFar,
// continuous step, MSC, energy loss fluctuations, delta-interaction test;
// MixedEl), the gamma stage A (HowFar and interaction choice; MixedG) and the
// FP32 interaction models (MixedB).
//
// The same algorithms as Physics (physics.cuh; G4HepEmElectronManager.icc:35-483,
// G4HepEmGammaManager.icc:27-130, the UMSC, fluctuation and interaction
// models), with the table lookups and the sampling arithmetic in FP32 from
// FP32 tables (DevElData32, DevGamma32) and FP32 parameter records.  FP64 is
// kept for: the decisions on exact inputs (energy against table thresholds,
// compared as integer bit patterns), the range->energy inversion of the mean
// energy loss, the polar-method acceptance of Gaussian samples, the accepted
// photon energy / epsilon of the relativistic brem and pair production, the
// kinematic limits, and the energy / deposit bookkeeping.  Conversions between
// FP64 and FP32 are integer bit operations (d2f, f2d): on this GPU they would
// otherwise run on the FP64 pipe.
//
// Guarded decisions.  Every branch that changes a discrete outcome (the
// winning process, whether MSC limits the step or scatters, Gaussian or
// Poisson sampling, Poisson counts, rejection-loop acceptances, target
// elements, the delta-interaction test, the tracking cut) compares FP32 values
// that carry a relative error of ~1e-6.  A comparison whose operands are
// closer than kGuardTol (relative) sets `trip`: the caller then discards the
// track's FP32 result and steps it again with the FP64 code (Physics), which
// gives the FP64 outcome bit for bit.  So the discrete outcomes of the
// precision form are those of the FP64 path; the tripped fraction is reported.
#pragma once

#include "physics.cuh"

namespace hepem {

constexpr float kGuardTol = 2.44140625e-4f;  // 2^-12
constexpr float kLargeF = 1.0E+20f;

// ---- FP64 <-> FP32 conversions with integer operations ---------------------------------
// Conversions between double and float issue on the FP64 pipe, which on this
// GPU runs at 1/64 of the FP32 rate; for the values of this path (normal
// floats, no NaN) the bit patterns are converted with integer operations.
// d2f truncates the mantissa (error < 1 float ulp); f2d is exact.
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned sign = hi & 0x80000000u;
  const int ef = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  if (ef <= 0) return __uint_as_float(sign);                  // zero, or below the float range
  if (ef >= 255) return __uint_as_float(sign | 0x7F800000u);  // beyond the float range
  const unsigned m = ((hi & 0xFFFFFu) << 3) | ((unsigned)b >> 29);
  return __uint_as_float(sign | ((unsigned)ef << 23) | m);
}
__device__ __forceinline__ double f2d(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0u) return __longlong_as_double((long long)sign);  // zero (subnormals flushed)
  const unsigned long long ed = e == 255u ? 0x7FFull : (unsigned long long)(e - 127u + 1023u);
  return __longlong_as_double((long long)(sign | (ed << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}
// 1 - u for a uniform u in (0, 1) to float precision, without FP64 arithmetic:
// for u >= 1/2, 1 - u = (2^52 - mantissa) 2^-53 is formed exactly in integers
__device__ __forceinline__ float one_minus_u(double u) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(u);
  if ((b >> 52) < 1022ull) return 1.0f - d2f(u);  // u < 1/2: no cancellation
  if ((b >> 52) > 1022ull) return 0.0f;           // u >= 1
  const unsigned long long k = (1ull << 52) - (b & 0xFFFFFFFFFFFFFull);
  if (k == 0ull) return 0.0f;
  const int p = 63 - __clzll((long long)k);                  // k = 1.x 2^p
  const unsigned m = (unsigned)((k << (63 - p)) >> 40) & 0x7FFFFFu;
  return __uint_as_float(((unsigned)(p - 53 + 127) << 23) | m);
}
// x <= 0 for a double without NaN, from its bit pattern
__device__ __forceinline__ bool nonpositive(double x) {
  const long long b = __double_as_longlong(x);
  return b <= 0 || b == (long long)0x8000000000000000ull;
}
// a < b for doubles a, b >= 0 (no NaN, no -0): the bit patterns order as integers
__device__ __forceinline__ bool dless(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b);
}
// max(x, 0) for a double without NaN
__device__ __forceinline__ double dpos(double x) { return __double_as_longlong(x) < 0 ? 0.0 : x; }

// x^2 (c[0] + c[1] x + ... + c[N-1] x^(N-1)), Horner
template <int N>
__device__ __forceinline__ float series2(float x, const float (&c)[N]) {
  float a = c[N - 1];
#pragma unroll
  for (int k = N - 2; k >= 0; --k) a = fmaf(a, x, c[k]);
  return a * x * x;
}
// Non-negative functions of the true -> geometrical path length conversion,
// each by its power series where the direct form cancels (truncation < 1e-8
// relative in the series' range):
//   g(x) = x + (1 - x) ln(1 - x)   = sum_{k>=2} x^k / (k (k-1)),        0 <= x < 1
//   h(y) = e^y - 1 - y             = sum_{k>=2} y^k / k!,               y <= 0
//   P(b) = 1 - e^-b (1 + b)        = sum_{k>=2} (-1)^k (k-1) b^k / k!,  b >= 0
//   Q(u) = u - 1 + e^-u            = sum_{k>=2} (-1)^k u^k / k!,        u >= 0
__device__ __forceinline__ float geom_g(float x) {
  if (x >= 0.25f) return x + (1.f - x) * log1pf(-x);
  const float c[13] = {1.f / 2, 1.f / 6, 1.f / 12, 1.f / 20, 1.f / 30, 1.f / 42, 1.f / 56,
                       1.f / 72, 1.f / 90, 1.f / 110, 1.f / 132, 1.f / 156, 1.f / 182};
  return series2(x, c);
}
__device__ __forceinline__ float geom_h(float y) {
  if (y <= -0.5f) return expm1f(y) - y;
  const float c[9] = {1.f / 2, 1.f / 6, 1.f / 24, 1.f / 120, 1.f / 720, 1.f / 5040, 1.f / 40320, 1.f / 362880,
                      1.f / 3628800};
  return series2(y, c);
}
__device__ __forceinline__ float geom_p(float b) {
  if (b >= 0.5f) return -expm1f(-b) - b * expf(-b);
  const float c[10] = {1.f / 2, -2.f / 6, 3.f / 24, -4.f / 120, 5.f / 720, -6.f / 5040, 7.f / 40320,
                       -8.f / 362880, 9.f / 3628800, -10.f / 39916800};
  return series2(b, c);
}
__device__ __forceinline__ float geom_q(float u) {
  if (u >= 0.5f) return u + expm1f(-u);
  const float c[9] = {1.f / 2, -1.f / 6, 1.f / 24, -1.f / 120, 1.f / 720, -1.f / 5040, 1.f / 40320,
                      -1.f / 362880, 1.f / 3628800};
  return series2(u, c);
}

__device__ __forceinline__ float fmx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fmn(float a, float b) { return a < b ? a : b; }

// ---- FP32 interpolation (the formulas of G4HepEmRunUtils.icc:49-237) --------------
__device__ __forceinline__ float spline32(float x1, float x2, float y1, float y2, float s1, float s2, float x) {
  const float dl = x2 - x1;
  const float b = fmx(0.f, fmn(1.f, (x - x1) / dl));
  const float c0 = (2.0f - b) * s1;
  const float c1 = (1.0f + b) * s2;
  return y1 + b * (y2 - y1) + (b * (b - 1.0f)) * (c0 + c1) * (dl * dl * 0.16666667f);
}
__device__ __forceinline__ int bin32(float lx, float lxm, float ild, int nd) {
  return (int)fmx(0.f, fmn((lx - lxm) * ild, (float)(nd - 2)));
}
__device__ __forceinline__ float spline_log_xy32(int nd, const float* xd, const float* yd, float x, float lx,
                                                 float lxm, float ild) {
  const float xv = fmx(ld(xd), fmn(ld(xd + nd - 1), x));
  const int i = bin32(lx, lxm, ild, nd);
  return spline32(ld(xd + i), ld(xd + i + 1), ld(yd + 2 * i), ld(yd + 2 * i + 2), ld(yd + 2 * i + 1),
                  ld(yd + 2 * i + 3), xv);
}
__device__ __forceinline__ float spline_log_3_32(int nd, const float* d, float x, float lx, float lxm, float ild) {
  const float xv = fmx(ld(d), fmn(ld(d + 3 * (nd - 1)), x));
  const int i = 3 * bin32(lx, lxm, ild, nd);
  return spline32(ld(d + i), ld(d + i + 3), ld(d + i + 1), ld(d + i + 4), ld(d + i + 2), ld(d + i + 5), xv);
}
// The same over (x, y, y'') triplets with the offset x - x1 taken in FP64
// (d64: the FP64 table).  The restricted cross sections start from zero at a
// threshold knot: just above it y ~ (x - x1), and the FP32 rounding of x
// (~6e-8 x) would be a relative error ~6e-8 x / (x - x1) of the cross section.
__device__ __forceinline__ float spline_log_3_32x(int nd, const float* d, const double* d64, double x, float lx,
                                                  float lxm, float ild) {
  const int i = 3 * bin32(lx, lxm, ild, nd);
  const double x1 = ld(d64 + i), x2 = ld(d64 + i + 3);
  const float dl = d2f(x2 - x1);
  const float b = fmx(0.f, fmn(1.f, d2f(x - x1) / dl));
  const float s1 = ld(d + i + 2), s2 = ld(d + i + 5), y1 = ld(d + i + 1), y2 = ld(d + i + 4);
  return y1 + b * (y2 - y1) + (b * (b - 1.0f)) * ((2.0f - b) * s1 + (1.0f + b) * s2) * (dl * dl * 0.16666667f);
}
__device__ __forceinline__ int lower_bin32(const float* xd, int num, float x, int step) {
  int ml = -1, mu = num - 1;
  while (abs(mu - ml) > 1) {
    const int mav = (ml + mu) / 2;
    if (x < ld(xd + step * mav)) mu = mav; else ml = mav;
  }
  return mu - 1;
}
__device__ __forceinline__ void rotate32(float* d, const float* r) {
  float up = r[0] * r[0] + r[1] * r[1];
  if (up > 0.f) {
    up = sqrtf(up);
    const float px = d[0], py = d[1], pz = d[2];
    d[0] = (r[0] * r[2] * px - r[1] * py) / up + r[0] * pz;
    d[1] = (r[1] * r[2] * px + r[0] * py) / up + r[1] * pz;
    d[2] = -up * px + r[2] * pz;
  } else if (r[2] < 0.f) {
    d[0] = -d[0];
    d[2] = -d[2];
  }
}
// rotation to the frame of the unit vector r, in FP32 where it is well
// conditioned; within ~6 degrees of the z axis the division by the transverse
// length sqrt(r0^2 + r1^2) amplifies FP32 rounding, and FP64 is used (rd: r in FP64)
// (the FP64 branch is out of line: it is rare, and one copy keeps the code small)
static __device__ __noinline__ float3 rotate64(float3 d, double r0, double r1, double r2) {
  double v[3] = {d.x, d.y, d.z};
  const double r[3] = {r0, r1, r2};
  rotate(v, r);
  return make_float3((float)v[0], (float)v[1], (float)v[2]);
}
__device__ __forceinline__ void rotate_mixed(float* d, const float* r, const double* rd) {
  if (r[0] * r[0] + r[1] * r[1] > 0.01f) {
    rotate32(d, r);
    return;
  }
  const float3 o = rotate64(make_float3(d[0], d[1], d[2]), rd[0], rd[1], rd[2]);
  d[0] = o.x;
  d[1] = o.y;
  d[2] = o.z;
}
// -ln(u) for u in (0,1) to FP32 accuracy, also for u close to 1
__device__ __forceinline__ float neg_log_u(double u) {
  return dless(0.5, u) ? -log1pf(-one_minus_u(u)) : -logf(d2f(u));
}

// ---- FP32 e+- table accessors (G4HepEmElectronManager.icc:486-599) -----------------
__device__ __forceinline__ float rest_range32(const DevElData32& f, int nL, int imc, float e, float le) {
  return fmx(0.f, spline_log_xy32(nL, f.lossGrid, f.loss + 5 * nL * imc, e, le, f.lossLogMin, f.lossILD));
}
__device__ __forceinline__ float rest_dedx32(const DevElData32& f, int nL, int imc, float e, float le) {
  return fmx(0.f, spline_log_xy32(nL, f.lossGrid, f.loss + nL * (5 * imc + 2), e, le, f.lossLogMin, f.lossILD));
}
__device__ __forceinline__ float inv_range32(const DevElData32& f, int nL, int imc, float r) {
  const float* R = f.loss + 5 * nL * imc;
  const float rmin = ld(R);
  if (r < rmin) {
    const float q = r / rmin;
    return fmx(0.f, ld(f.lossGrid) * q * q);
  }
  const int i = lower_bin32(R, nL, r, 2);
  const float* S2 = R + 4 * nL;
  return fmx(0.f, spline32(ld(R + 2 * i), ld(R + 2 * (i + 1)), ld(f.lossGrid + i), ld(f.lossGrid + i + 1),
                           ld(S2 + i), ld(S2 + i + 1), r));
}
__device__ __forceinline__ float transport_mfp32(const DevElData32& f, int nL, int imat, float e, float le) {
  const float v = fmx(0.f, spline_log_xy32(nL, f.lossGrid, f.tr1 + 2 * nL * imat, e, le, f.lossLogMin, f.lossILD));
  return v > 0.f ? 1.f / v : kLargeF;
}
// restricted macroscopic cross section (at the energy e, exact threshold test)
__device__ __forceinline__ float rest_macxs32(const DevElData& d, const DevElData32& f, int imc, double e, float ef,
                                              float le, bool ioni) {
  const int i0 = ld(d.xsStart + imc);
  const int st = ioni ? i0 : i0 + 3 * (int)ld(f.xs + i0) + 5;
  const int nd = (int)ld(f.xs + st);
  if (dless(e, ld(d.xs + st + 5))) return 0.f;
  return fmx(0.f, spline_log_3_32x(nd, f.xs + st + 5, d.xs + st + 5, e, le, ld(f.xs + st + 3), ld(f.xs + st + 4)));
}
// the cross section for stepping, max over [0.8 e, e]: continuous in e at
// both switches (e at the energy of the maximum, 0.8 e at it), so they are
// taken in FP32; the threshold test is exact
__device__ __forceinline__ float rest_macxs_stepping32(const DevElData& d, const DevElData32& f, int imc, double e,
                                                       float ef, float le, bool ioni) {
  const int i0 = ld(d.xsStart + imc);
  const int st = ioni ? i0 : i0 + 3 * (int)ld(f.xs + i0) + 5;
  const int nd = (int)ld(f.xs + st);
  const float maxE = ld(f.xs + st + 1);
  float ee = ef;
  if (ef > maxE) {
    const float er = 0.8f * ef;
    if (er < maxE) return fmx(0.f, ld(f.xs + st + 2));
    ee = er;
    le += -0.22314355f;  // log(0.8)
    if (ee < ld(f.xs + st + 5)) return 0.f;
    return fmx(0.f, spline_log_3_32(nd, f.xs + st + 5, ee, le, ld(f.xs + st + 3), ld(f.xs + st + 4)));
  }
  if (dless(e, ld(d.xs + st + 5))) return 0.f;
  return fmx(0.f, spline_log_3_32x(nd, f.xs + st + 5, d.xs + st + 5, e, le, ld(f.xs + st + 3), ld(f.xs + st + 4)));
}
__device__ __forceinline__ float nuc_macxs32(const DevElData& d, const DevElData32& f, int imat, double e, float ef,
                                             float le) {
  if (dless(e, ld(d.nucGrid))) return 0.f;
  const int n = d.nNuc;
  return fmx(0.f, spline_log_xy32(n, f.nucGrid, f.nuc + imat * 2 * n, ef, le, f.nucLogMin, f.nucILD));
}

// ---- FP64 range <-> energy for the mean energy loss ----------------------------------
// The reference's splines (G4HepEmRunUtils.icc:49-99) in FP64 where the
// inversion needs it, at a few FP64 operations: the interval is located on the
// FP32 copy and made exact by comparing the FP64 knots (integer comparisons of
// positive values); the interpolation variable is an FP32 quotient refined by
// one FP64 residual step (relative error ~1e-14 instead of an FP64 division);
// the curvature term, a small fraction of y, is evaluated in FP32.
__device__ __forceinline__ double spline64_lite(double x1, double x2, double y1, double y2, float s1, float s2,
                                                double x) {
  const double dl = x2 - x1, dx = x - x1;
  const float dlf = d2f(dl);
  const float b0 = d2f(dx) / dlf;
  const double res = fma(-f2d(b0), dl, dx);
  const double b = f2d(b0) + f2d(d2f(res) / dlf);
  const float bf = d2f(b);
  const float curv = (bf * (bf - 1.0f)) * ((2.0f - bf) * s1 + (1.0f + bf) * s2) * (dlf * dlf * 0.166666666667f);
  return fma(b, y2 - y1, y1) + f2d(curv);
}
// restricted range at e (lef: FP32 log e for the interval)
__device__ __forceinline__ double rest_range64(const DevElData& d, const DevElData32& f, int imc, double e,
                                               float lef) {
  const int n = d.nLoss;
  const double* xd = d.lossGrid;
  const double x0 = ld(xd), xn = ld(xd + n - 1);
  const double xv = dless(e, x0) ? x0 : dless(xn, e) ? xn : e;
  int i = bin32(lef, f.lossLogMin, f.lossILD, n);
  if (i > 0 && dless(xv, ld(xd + i))) --i;
  else if (i < n - 2 && !dless(xv, ld(xd + i + 1))) ++i;
  const double* yd = d.loss + 5 * n * imc;
  const float* yf = f.loss + 5 * n * imc;
  return dpos(spline64_lite(ld(xd + i), ld(xd + i + 1), ld(yd + 2 * i), ld(yd + 2 * i + 2), ld(yf + 2 * i + 1),
                            ld(yf + 2 * i + 3), xv));
}
// energy of the restricted range r (G4HepEmElectronManager.icc:547-561)
__device__ __forceinline__ double inv_range64(const DevElData& d, const DevElData32& f, int imc, double r) {
  const int n = d.nLoss;
  const double* R = d.loss + 5 * n * imc;
  const double rmin = ld(R);
  if (dless(r, rmin)) {  // (also r < 0)
    const double q = r / rmin;
    return dpos(ld(d.lossGrid) * q * q);
  }
  const float* Rf = f.loss + 5 * n * imc;
  const double rn = ld(R + 2 * (n - 1));
  const double rv = dless(rn, r) ? rn : r;
  int i = lower_bin32(Rf, n, d2f(rv), 2);
  i = i < 0 ? 0 : i;
  if (i > 0 && dless(rv, ld(R + 2 * i))) --i;
  else if (i < n - 2 && !dless(rv, ld(R + 2 * (i + 1)))) ++i;
  const float* S2 = Rf + 4 * n;
  return dpos(spline64_lite(ld(R + 2 * i), ld(R + 2 * (i + 1)), ld(d.lossGrid + i), ld(d.lossGrid + i + 1),
                            ld(S2 + i), ld(S2 + i + 1), rv));
}
__device__ __forceinline__ float annih_macxs32(float e, float ne) {
  const float tau = e * (float)kInvMec2;
  const float gam = tau + 1.0f;
  const float gam2 = gam * gam;
  const float bg2 = tau * (tau + 2.0f);
  const float bg = sqrtf(bg2);
  return ne * (float)kPir02 * (((gam2 + 4.f * gam + 1.f) * logf(gam + bg) - (gam + 3.f) * bg) / (bg2 * (gam + 1.f)));
}

// ---- the e+- stage A in FP32 ------------------------------------------------------------
// The step limits that the FP32 HowFar of MixedEl leaves for its Perform:
// lengths, mean free paths and interaction lengths left in FP32, the MSC
// state, and the provenance of values equal by construction (kL32*), which
// Perform's comparisons decide exactly.
constexpr uint32_t kL32FirstStep = 1u << 0, kL32Active = 1u << 1, kL32Displace = 1u << 2, kL32StepFn = 1u << 3,
                   kL32PIsRange = 1u << 4, kL32TsIsP = 1u << 5, kL32TsIsTlm = 1u << 6, kL32AtRange = 1u << 7;
struct ElLimit32 {
  float range, pstep, gstep, trueStep, zPath, lambtr1, delta, initRange, dynFactor, tlimitMin;
  float mfp[4], nia[4];
  int winner;
  uint32_t bits;
};

struct MixedEl {
  const DevTables& T;
  Rng& rng;
  Track& t;
  bool trip;
  int tripLine;  // source line of the first guard that tripped (diagnostics)

  __device__ __forceinline__ void set_trip(int line = __builtin_LINE()) {
    if (!trip) tripLine = line;
    trip = true;
  }

  // guarded comparisons: a < b / a <= b with a trip when the operands are too close
  __device__ __forceinline__ void near(float a, float b, int line = __builtin_LINE()) {
    if (fabsf(a - b) <= kGuardTol * fmx(fabsf(a), fabsf(b))) set_trip(line);
  }
  __device__ __forceinline__ bool lt(float a, float b, int line = __builtin_LINE()) {
    near(a, b, line);
    return a < b;
  }
  __device__ __forceinline__ bool le(float a, float b, int line = __builtin_LINE()) {
    near(a, b, line);
    return a <= b;
  }

  __device__ __forceinline__ const DevElData& eld() const { return t.isEl ? T.el[0] : T.el[1]; }
  __device__ __forceinline__ const DevElData32& elf() const { return t.isEl ? T.el32[0] : T.el32[1]; }

  // Gaussian of the polar method with the cached second value (rng.cuh); the
  // acceptance test is the FP64 one of the reference, the transform FP32
  __device__ float gauss(float mean, float sd) {
    if (rng.gaussValid) {
      rng.gaussValid = false;
      return d2f(rng.gaussValue) * sd + mean;
    }
    double r, v1, v2;
    int it = 0;
    do {
      const double a = rng.flat(), b = rng.flat();
      // the acceptance r > 1 is the FP64 path's decision: evaluated with its
      // rounding (no contraction into FMA)
      v1 = __dsub_rn(__dmul_rn(2., a), 1.);
      v2 = __dsub_rn(__dmul_rn(2., b), 1.);
      r = __dadd_rn(__dmul_rn(v1, v1), __dmul_rn(v2, v2));
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (dless(1.0, r));
    const float rf = d2f(r);
    // ln r to FP32 accuracy on both ends of (0, 1]; 1 - r is exact for r >= 1/2
    const float lr = dless(r, 0.5) ? logf(rf) : log1pf(-one_minus_u(r));
    const float fac = sqrtf(-2.f * lr / rf);
    rng.gaussValue = f2d(d2f(v1) * fac);
    rng.gaussValid = true;
    return d2f(v2) * fac * sd + mean;
  }

  __device__ int poisson(float mean) {
    int number = 0;
    if (le(mean, 16.f)) {
      const float position = d2f(rng.flat());
      float pv = expf(-mean);
      float ps = pv;
      // the cumulative carries the FP32 error of the mean (~1e-6 of mean times
      // the largest Poisson probability, <= 2e-6) and of its sum (<= 2e-6): an
      // absolute margin of 8e-6 covers both
      for (;;) {
        if (fabsf(ps - position) <= 8.0e-6f) set_trip();
        if (!(ps <= position)) break;
        ++number;
        pv *= mean / number;
        ps += pv;
        if (number >= 4096) { t.flags |= kFlagLoopCap; break; }
      }
      return number;
    }
    const double a = rng.flat(), b = rng.flat();
    float sb, cb;
    sincospif(2.f * d2f(b), &sb, &cb);
    const float tt = sqrtf(2.f * neg_log_u(a)) * cb;
    const float value = mean + tt * sqrtf(mean) + 0.5f;
    // the integer part is a discrete outcome: guard the distance to the nearest integer
    const float fl = floorf(value);
    if (value - fl < kGuardTol * fmx(1.f, value) || fl + 1.f - value < kGuardTol * fmx(1.f, value)) set_trip();
    return value < 0.f ? 0 : value >= 2.E+9f ? (int)2.E+9 : (int)value;
  }

  __device__ float gauss_loss(float me, float s2) {
    const float twom = 2.f * me;
    if (lt(me * me, 0.0625f * s2)) return twom * d2f(rng.flat());
    const float sig = sqrtf(s2);
    float el;
    int it = 0;
    do {
      el = gauss(me, sig);
      if (fabsf(el) <= kGuardTol * sig) set_trip();
      near(el, twom);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (el < 0.f || el > twom);
    return el;
  }

  // Urban fluctuation model (G4HepEmElectronEnergyLossFluctuation.icc:11-111);
  // the sampled terms (all >= 0) are summed with compensation (Neumaier), so
  // that the sum carries the terms' own FP32 accuracy
  float fsum, fcomp;
  __device__ __forceinline__ void fadd(float x) {
    const float s = fsum + x;
    fcomp += fabsf(fsum) >= fabsf(x) ? (fsum - s) + x : (x - s) + fsum;
    fsum = s;
  }
  __device__ float fluct(float tcut, float excE, float meanE) {
    const float scaling = fmn(1.f + 5.E-4f / tcut, 1.5f);
    const float meanLoss = meanE / scaling;
    const float rate = 0.56f, e0 = 1.E-5f, nmax = 8.f;
    const float w1 = tcut / e0;
    float a3 = meanLoss * (tcut - e0) / (e0 * tcut * logf(w1));
    float a1 = 0.f;
    float e1 = excE;
    fsum = 0.f;
    fcomp = 0.f;
    HEPEM_TR(1, 18, a3);
    if (lt(excE, tcut)) {
      const float a1t = meanLoss * (1.f - rate) / excE;
      const float d0 = a1t < 42.f ? .1f + (4.f - .1f) * sqrtf(a1t / 42.f) : 4.f;
      a1 = a1t / d0;
      e1 *= d0;
      a3 *= rate;
      if (lt(nmax, a1)) {
        const float em = a1 * e1;
        fadd(gauss_loss(em, em * e1));
      } else {
        const int p = poisson(a1);
        HEPEM_TR(1, 17, p);
        // ((p + 1) - 2u) e1 as ((p - 1) + 2 (1 - u)) e1: no cancellation for p = 1, u -> 1
        if (p > 0) fadd(((float)(p - 1) + 2.f * one_minus_u(rng.flat())) * e1);
      }
    }
    if (a3 > 0.f) {
      // The reference's differences a3 - nam, alfa - 1 and tcut - w3 cancel for
      // thick steps (a3 >> nmax); their closed forms are used here:
      //   alfa - 1 = a3 (w1 - 1) / (w1 nmax + a3),  nam = a3^2 / (nmax + a3),
      //   a3 - nam = a3 nmax / (nmax + a3),  (tcut - w3) / tcut = nmax (w1 - 1) / (w1 nmax + a3)
      float p3 = a3;
      float alfa = 1.f;
      float w = (w1 - 1.f) / w1;
      if (lt(nmax, a3)) {
        const float den = w1 * nmax + a3;
        alfa = w1 * (nmax + a3) / den;
        const float am1 = a3 * (w1 - 1.f) / den;
        const float alfa1 = alfa * logf(alfa) / am1;
        const float nam = a3 * a3 / (nmax + a3);
        const float em = nam * e0 * alfa1;
        const float s2 = e0 * e0 * nam * (alfa - alfa1 * alfa1);
        fadd(gauss_loss(em, s2));
        p3 = a3 * nmax / (nmax + a3);
        w = nmax * (w1 - 1.f) / den;
      }
      const float w3 = alfa * e0;
      if (lt(w3, tcut)) {
        int nnb = poisson(p3);
        HEPEM_TR(1, 19, p3);
        HEPEM_TR(1, 20, nnb);
        if (nnb > kMaxIter) { nnb = kMaxIter; t.flags |= kFlagLoopCap; }
        // 1 - w u as (1 - w) + w (1 - u): no cancellation in the Landau tail (u -> 1/w)
        const float omw = w3 / tcut;
        for (int k = 0; k < nnb; ++k) fadd(w3 / (omw + w * one_minus_u(rng.flat())));
      }
    }
    return (fsum + fcomp) * scaling;
  }

  // Urban MSC cos(theta) (G4HepEmElectronInteractionUMSC.icc:153-270), given
  // as 1 - cos and 1 + cos, each to FP32 relative precision
  struct CosT {
    float omc, opc;
  };
  // cos = -1 + 2 u for a uniform u
  __device__ static CosT cos_uniform(double u) { return CosT{2.f * one_minus_u(u), 2.f * d2f(u)}; }
  // d0 = 3 <x^2> - 1 and d1 = 2 <x> - d0, given without cancellation (cos_theta)
  __device__ CosT simple_scatter(float xm, float d0, float d1) {
    const float a = 1.f + 4.f * d0 / d1;
    const float prob = (2.f + a) * xm / a;
    const double r0 = rng.flat(), r1 = rng.flat();
    if (!lt(d2f(r0), prob)) return cos_uniform(r1);
    // cos = -1 + 2 pw, pw = r1^(1/(1+a)): 1 + cos = 2 pw, 1 - cos = -2 expm1(ln pw)
    const float lg = (1.f / (1.f + a)) * -neg_log_u(r1);
    const float pw = expf(lg);
    return CosT{pw < 0.5f ? 2.f - 2.f * pw : -2.f * expm1f(lg), 2.f * pw};
  }

  __device__ float theta0_of(float srl, float postE, float preE, const DevMat32& md) {
    const float me = (float)kMec2;
    const float postInv = (postE + me) / (postE * (postE + 2.f * me));
    const float inv = preE != postE ? sqrtf(postInv * (preE + me) / (preE * (preE + 2.f * me))) : postInv;
    float y = srl;
    if (!t.isEl && T.mscPosCor) y = srl * pos_correction32(preE * postE, ld(&md.zeff));
    return 13.6f * sqrtf(y) * inv * (ld(&md.theta[0]) + ld(&md.theta[1]) * logf(y));
  }

  __device__ static float pos_correction32(float eekin, float zeff) {
    const float ff = 1.f + zeff * (1.84035E-4f * zeff - 1.86427E-2f) + 0.41125f;
    const float a = 0.994f - 4.08E-3f * zeff;
    const float b = 7.16f + (52.6f + 365.f / zeff) / zeff;
    const float tu = sqrtf(eekin) * (float)kInvMec2;
    const float x = sqrtf(tu * (tu + 2.f) / ((tu + 1.f) * (tu + 1.f)));
    if (x < 0.6f) return ff * a * (1.f - expf(-b * x));
    const float c = 1.00f - 4.47E-3f * zeff;
    const float d = 1.21E-3f * zeff;
    if (x > 0.9f) return ff * (c + d * expf(113.0f * (x - 1.f)));
    const float yl = a * (1.f - expf(-b * 0.6f));
    const float yh = c + d * expf(113.0f * (0.9f - 1.f));
    const float y0 = (yh - yl) / (0.9f - 0.6f);
    const float y1 = yl - y0 * 0.6f;
    return ff * (y0 * x + y1);
  }

  bool exactCos;  // cos_theta returned an exact 1.0 of the reference's own shortcuts

  __device__ CosT cos_theta(float pstep, float preE, float preMFP, float postE, float postMFP, float tlimMin,
                            const DevMat32& md, bool pIsTlm) {
    exactCos = false;
    const float iPre = 1.0f / preMFP;
    const float dR = preMFP - postMFP;
    const float tau = lt(0.01f * preMFP, fabsf(dR)) ? pstep * logf(preMFP / postMFP) / dR : pstep * iPre;
    if (lt(8.0f, tau)) return cos_uniform(rng.flat());
    if (lt(tau, 1.0E-16f)) {
      exactCos = true;
      return CosT{0.f, 2.f};
    }
    // <x> = xm and <x^2> = x2m of the reference (with its 0.333333); the simple
    // model needs d0 = 3 x2m - 1 and d1 = 2 xm - d0, formed here so that the
    // small-tau cancellations of the direct differences do not occur
    float xm, d0, d1;
    if (tau < 0.01f) {
      xm = 1.0f - tau * (1.0f - 0.5f * tau);
      d0 = 2.0f - tau * (5.0f - 6.25f * tau) * 0.999999f;
      d1 = tau * (4.999995f - 2.0f) + tau * tau * (1.0f - 6.2499938f);
    } else {
      xm = expf(-tau);
      d0 = 1.999998f * expf(-2.5f * tau) - 1.0e-6f;
      d1 = 3.0e-6f + 2.0f * expm1f(-tau) - 1.999998f * expm1f(-2.5f * tau);
    }
    if (lt(postE, 0.5f * preE)) return simple_scatter(xm, d0, d1);
    const float radLen = ld(&md.radLength);
    const float tsmall = fmn(tlimMin, 1.0f);
    // pstep == tlimitMin by construction when the MSC limit chose it
    const bool notSmall = (pIsTlm && tlimMin <= 1.0f) ? false : lt(tsmall, pstep);
    const float theta0 = notSmall ? theta0_of(pstep / radLen, postE, preE, md)
                                  : theta0_of(tsmall / radLen, postE, preE, md) * sqrtf(pstep / tsmall);
    if (lt((float)kPi * 0.166666f, theta0)) return simple_scatter(xm, d0, d1);
    const float th2 = theta0 * theta0;
    if (lt(th2, 1.0E-16f)) {
      exactCos = true;
      return CosT{0.f, 2.f};
    }
    const float dumtau = notSmall ? tau : tsmall * iPre;
    const float u = exp2f(0.1666666f * log2f(dumtau));
    const float dumxsi = ld(&md.tail[0]) + u * (ld(&md.tail[1]) + u * ld(&md.tail[2])) +
                         ld(&md.tail[3]) * logf(pstep / (tau * radLen));
    const float xsi = fmx(dumxsi, 1.9f);
    // the reference moves c off the poles of its formulas at 2 and 3
    const bool pole3 = lt(fabsf(xsi - 3.f), 0.001f), pole2 = lt(fabsf(xsi - 2.f), 0.001f);
    const float c = pole3 ? 3.001f : pole2 ? 2.001f : xsi;
    const float c1 = c - 1.f;
    const float ea = expf(-xsi);
    const float eaa = 1.f / (1.f - ea);
    float thex = th2 * (1.0f - th2 * 0.0833333f);
    if (th2 > 0.01f) {
      const float q = 2.0f * sinpif(theta0 * (float)(0.5 / kPi));
      thex = q * q;
    }
    const float xmean1 = 1.f - (1.f - (1.f + xsi) * ea) * thex * eaa;
    if (le(xmean1, 0.999f * xm)) return simple_scatter(xm, d0, d1);
    const float x0 = 1.f - xsi * thex;
    const float bx = c * thex;
    const float b = bx + x0;
    const float b1 = b + 1.f;
    const float dd = powf(bx / b1, c1);  // bx^c1 / b1^c1
    const float xmean2 = (x0 + dd - (bx - b1 * dd) / (c - 2.f)) / (1.f - dd);
    const float f1x0 = ea * eaa;
    const float f2x0 = c1 / (c * (1.f - dd));
    const float prob = f2x0 / (f1x0 + f2x0);
    const float qprb = xm / (prob * xmean1 + (1.f - prob) * xmean2);
    const double r0 = rng.flat(), r1 = rng.flat(), r2 = rng.flat();
    if (lt(d2f(r0), qprb)) {
      // log(ea + r2/eaa) = log(1 - (1 - r2)(1 - ea)): log1p keeps small angles
      if (lt(d2f(r1), prob)) {
        const float omc = -(log1pf(-one_minus_u(r2) * (1.f - ea)) * thex);
        return CosT{omc, 2.f - omc};
      }
      const float var0 = (1.0f - dd) * d2f(r2);
      if (lt(var0, 0.01f * dd)) {
        const float var = var0 / (dd * c1);
        const float opc = var * (1.0f - var * 0.5f * c) * b1;
        return CosT{2.f - opc, opc};
      }
      const float omc = -(thex * (c - xsi - c * powf(var0 + dd, -1.f / c1)));
      return CosT{omc, 2.f - omc};
    }
    return cos_uniform(r1);
  }

  // ---- the stage: HowFar + Perform up to the pending discrete interaction ------------
  // stage_a() returns the interaction queue of the pending interaction or -1 (as
  // Physics::el_perform_until_discrete); valid only if !trip on return.  Its two
  // halves are howfar(), the step limits of G4HepEmElectronManager::HowFar in FP32
  // (kept in an ElLimit32), and perform(), Perform from those limits; the split
  // entry points run them as two kernels.
  __device__ void howfar(ElLimit32& h) {
    const DevElData& d = eld();
    const DevElData32& f = elf();
    const int nL = d.nLoss;
    const int imc = t.imc;
    const int cMat = ld(&T.couples[imc].mat), cRegion = ld(&T.couples[imc].region);
    const DevRegion32& reg = T.regions32[cRegion];
    const DevMat32& md = T.mats32[cMat];
    // -- HowFar (G4HepEmElectronManager.icc:35-101)
#pragma unroll
    for (int ip = 0; ip < 4; ++ip)
      if (nonpositive(t.nia[ip])) t.nia[ip] = f2d(neg_log_u(rng.flat()));
    const double e = t.e;
    const float ef = d2f(e), lef = logf(ef);
    const float range = rest_range32(f, nL, imc, ef, lef);
    const float frange = ld(&reg.finalRange), drange = ld(&reg.dRoverRange);
    // The step function.  Some later comparisons of the reference meet values
    // that are equal by construction (pstep == range, trueStep == pstep,
    // trueStep == tlimitMin); their provenance is tracked here so that those
    // comparisons are decided exactly and only the others are guarded.
    const bool stepFn = lt(frange, range);
    float pstep = stepFn ? range * drange + frange * (1.0f - drange) * (2.0f - frange / range) : range;
    bool pIsRange = !stepFn;  // pstep == range
    HEPEM_TR(1, 0, range);
    HEPEM_TR(1, 1, pstep);
    int winner = -1;
    float mx[4], mfp[4], nia[4];
    mx[0] = rest_macxs_stepping32(d, f, imc, e, ef, lef, true);
    mx[1] = rest_macxs_stepping32(d, f, imc, e, ef, lef, false);
    mx[2] = t.isEl ? 0.f : annih_macxs32(0.8f * ef, ld(&md.elDensity));
    mx[3] = nuc_macxs32(d, f, cMat, e, ef, lef);
#pragma unroll
    for (int ip = 0; ip < 4; ++ip) {
      nia[ip] = d2f(t.nia[ip]);
      mfp[ip] = mx[ip] > 0.f ? 1.f / mx[ip] : kLargeF;
      const float lim = mfp[ip] * nia[ip];
      if (lt(lim, pstep)) { pstep = lim; winner = ip; pIsRange = false; }
    }
    HEPEM_TR(1, 2, mx[0]);
    HEPEM_TR(1, 3, mx[1]);
    HEPEM_TR(1, 6, pstep);
    HEPEM_TR(1, 7, winner);
    // MSC step limit and true -> geometrical length (UMSC.icc:19-126, Manager.icc:602-650)
    float trueStep = pstep, zPath = pstep, lambtr1 = kLargeF;
    float delta = 0.f;  // trueStep - zPath, kept without cancellation (lateral displacement)
    float initRange = d2f(t.msc.initRange), dynFactor = d2f(t.msc.dynFactor);
    float tlimitMin = d2f(t.msc.tlimitMin);
    bool firstStep = t.msc.firstStep;
    bool active = false, displace = false;
    bool tsIsP = true, tsIsTlm = false;  // trueStep == pstep / == tlimitMin
    bool atRange = pIsRange;             // trueStep == range
    float gstep = pstep;
    if (lt(5.E-8f, pstep) && dless(1.0E-3, e)) {
      active = true;
      lambtr1 = transport_mfp32(f, nL, cMat, ef, lef);
      // -- step limit
      const float kTLimitMinfix = 1.0E-8f;
      const float safety = d2f(t.safety);
      displace = true;
      if (lt(trueStep, kTLimitMinfix) || lt(range * ld(&md.umscPar), safety)) {
        displace = false;
      } else {
        const float rf = ld(&reg.mscRangeFactor), sf = ld(&reg.mscSafetyFactor);
        float tlimit;
        bool tlimIsRange = false, tlimIsTlm = false;  // tlimit == range / == tlimitMin
        if (!ld(&reg.mscMinimal)) {
          if (firstStep || t.onBoundary) {
            const float l1 = lambtr1;
            initRange = fmx(range, l1);
            dynFactor = l1 > 1.0f ? rf * (0.75f + 0.25f * l1) : rf;
            const float stepMin = l1 * 1.0E-3f / (2.0E-3f + ef * (ld(&md.stepMin[0]) + ef * ld(&md.stepMin[1])));
            const float d0 = t.isEl ? 0.87f * ld(&md.zeff23) : 0.70f * ld(&md.zeffSqrt);
            const float d1 = dless(5.0E-3, e) ? d0 * stepMin : d0 * stepMin * 0.5f * (1.0f + ef * 200.0f);
            tlimitMin = fmx(d1, kTLimitMinfix);
            firstStep = false;
          }
          float cand;
          if (lt(safety, range)) {
            cand = fmx(initRange * dynFactor, sf * safety);
            tlimIsRange = false;
          } else {
            cand = range;
            tlimIsRange = true;
          }
          near(cand, tlimitMin);
          tlimIsTlm = !(cand > tlimitMin);
          tlimIsRange = tlimIsRange && !tlimIsTlm;
          tlimit = fmx(cand, tlimitMin);
        } else {
          if (t.onBoundary) {
            const float tmp = range > lambtr1 ? rf * range : rf * lambtr1;
            initRange = fmx(tmp, 10.f * kTLimitMinfix);
          }
          tlimit = initRange;
        }
        // reference: if (tlimit < trueStep) { d0 = tlimit > tlimitMin ? max(gauss, tlimitMin) : tlimitMin;
        //                                     trueStep = min(d0, trueStep) }
        HEPEM_TR(1, 24, tlimit);
        const bool limits = (tlimIsRange && pIsRange) ? false : lt(tlimit, trueStep);
        if (limits) {
          float d0;
          bool d0IsTlm;
          if (!tlimIsTlm && lt(tlimitMin, tlimit)) {
            const float gs = gauss(tlimit, 0.1f * (tlimit - tlimitMin));
            near(gs, tlimitMin);
            d0IsTlm = !(gs > tlimitMin);
            d0 = fmx(gs, tlimitMin);
          } else {
            d0 = tlimitMin;
            d0IsTlm = true;
          }
          HEPEM_TR(1, 25, d0);
          near(d0, trueStep);
          if (d0 < trueStep) {
            trueStep = d0;
            tsIsP = false;
            tsIsTlm = d0IsTlm;
          }
        }
      }
      HEPEM_TR(1, 8, lambtr1);
      HEPEM_TR(1, 10, trueStep);
      // -- true -> geometrical.  trueStep <= pstep <= range: trueStep == range
      // only by construction (the reference then takes its trueStep == range branch)
      atRange = tsIsP && pIsRange;
      if (!atRange) near(trueStep, range);
      trueStep = fmn(trueStep, range);
      zPath = trueStep;
      if (!lt(trueStep, 1.0E-6f)) {
        const float tau = trueStep / lambtr1;
        if (lt(tau, 1.0e-16f)) {
          zPath = fmn(trueStep, lambtr1);
        } else if (lt(trueStep, range * 0.05f)) {
          // zPath = lambda (1 - exp(-tau)); trueStep - zPath = lambda g(tau),
          // g = exp(-tau) - 1 + tau, by its series where it cancels
          const float g = tau < 0.1f
              ? tau * tau * (0.5f - tau * (0.16666667f - tau * (0.041666668f - tau * (0.0083333338f - tau *
                                                                                    0.0013888889f))))
              : tau + expm1f(-tau);
          delta = lambtr1 * g;
          zPath = trueStep - delta;
          // below ~1e-12 the reference's own rounding decides whether zPath < trueStep
          if (tau < 1.0e-12f) set_trip();
        } else {
          // the range-based conversions (UMSC.icc:105-126) in forms without
          // cancellation, so that trueStep - zPath (the displacement length)
          // keeps the inputs' FP32 accuracy where zPath is close to trueStep.
          // Below m_e c^2, with x = trueStep / range and q = range / lambda:
          //   trueStep - zPath = range (q g(x) + (1 - x) h(q ln(1 - x))) / (1 + q);
          // above, with lambda1 the transport mfp at E(range - trueStep),
          // b = ln(lambda / lambda1), s = trueStep / (lambda (1 - e^-b)), u = s b:
          //   trueStep - zPath = trueStep (u P(b) + b e^-b Q(u)) / ((b + u)(1 - e^-b))
          // (g, h, P, Q >= 0: geom_g .. geom_q)
          float dz;
          if (dless(e, kMec2) || atRange) {
            const float q = range / lambtr1;
            if (atRange) {
              dz = range * q / (1.f + q);
            } else {
              const float x = trueStep / range;
              dz = range * (q * geom_g(x) + (1.f - x) * geom_h(q * log1pf(-x))) / (1.f + q);
            }
          } else {
            const float rfin = fmx(range - trueStep, 0.01f * range);
            const float t1 = inv_range32(f, nL, imc, rfin);
            const float l1 = transport_mfp32(f, nL, cMat, t1, logf(t1));
            const float b = logf(lambtr1 / l1);
            if (!(b > 1.0e-6f)) set_trip();  // lambda1 >= lambda: left to the FP64 code
            const float omea = -expm1f(-b);
            const float u = trueStep / (lambtr1 * omea) * b;
            dz = trueStep * (u * geom_p(b) + b * expf(-b) * geom_q(u)) / ((b + u) * omea);
          }
          // the reference displaces only when zPath < trueStep
          if (!(dz >= 1.0e-9f * trueStep)) set_trip();
          zPath = trueStep - dz;
          delta = dz;
        }
        if (delta == 0.f) delta = trueStep - zPath;
        if (zPath > lambtr1) {
          zPath = lambtr1;
          delta = trueStep - zPath;
        }
      }
      HEPEM_TR(1, 11, zPath);
      if (!tsIsP) {  // the MSC limit is below the proposed step
        winner = -2;
        pstep = trueStep;
      }
      gstep = fmn(zPath, pstep);
      // the geometrical step equals zPath here (zPath <= true length <= pstep);
      // the geometry-shortened case of the reference is left to the FP64 code
      if (gstep < zPath) set_trip();
    }
    h.range = range;
    h.pstep = pstep;
    h.gstep = gstep;
    h.trueStep = trueStep;
    h.zPath = zPath;
    h.lambtr1 = lambtr1;
    h.delta = delta;
    h.initRange = initRange;
    h.dynFactor = dynFactor;
    h.tlimitMin = tlimitMin;
#pragma unroll
    for (int ip = 0; ip < 4; ++ip) {
      h.mfp[ip] = mfp[ip];
      h.nia[ip] = nia[ip];
    }
    h.winner = winner;
    h.bits = (firstStep ? kL32FirstStep : 0u) | (active ? kL32Active : 0u) | (displace ? kL32Displace : 0u) |
             (stepFn ? kL32StepFn : 0u) | (pIsRange ? kL32PIsRange : 0u) | (tsIsP ? kL32TsIsP : 0u) |
             (tsIsTlm ? kL32TsIsTlm : 0u) | (atRange ? kL32AtRange : 0u);
  }

  __device__ int perform(const ElLimit32& h) {
    const DevElData& d = eld();
    const DevElData32& f = elf();
    const int nL = d.nLoss;
    const int imc = t.imc;
    const int cMat = ld(&T.couples[imc].mat), cRegion = ld(&T.couples[imc].region);
    const DevRegion32& reg = T.regions32[cRegion];
    const DevMat32& md = T.mats32[cMat];
    const double e = t.e;
    const float ef = d2f(e), lef = logf(ef);
    const float range = h.range;
    float pstep = h.pstep, gstep = h.gstep, trueStep = h.trueStep, zPath = h.zPath, lambtr1 = h.lambtr1;
    const float delta = h.delta;
    const float initRange = h.initRange, dynFactor = h.dynFactor, tlimitMin = h.tlimitMin;
    float mfp[4], nia[4];
#pragma unroll
    for (int ip = 0; ip < 4; ++ip) {
      mfp[ip] = h.mfp[ip];
      nia[ip] = h.nia[ip];
    }
    const int winner = h.winner;
    const bool firstStep = h.bits & kL32FirstStep;
    bool active = h.bits & kL32Active;
    const bool displace = h.bits & kL32Displace, stepFn = h.bits & kL32StepFn, pIsRange = h.bits & kL32PIsRange;
    const bool tsIsP = h.bits & kL32TsIsP, tsIsTlm = h.bits & kL32TsIsTlm, atRange = h.bits & kL32AtRange;
    t.winner = winner;
    t.gstep = f2d(gstep);
    t.msc.initRange = f2d(initRange);
    t.msc.dynFactor = f2d(dynFactor);
    t.msc.tlimitMin = f2d(tlimitMin);
    t.msc.firstStep = firstStep;
    t.msc.disp[0] = t.msc.disp[1] = t.msc.disp[2] = 0.;
#pragma unroll
    for (int ip = 0; ip < 4; ++ip) t.mfp[ip] = f2d(mfp[ip]);

    // -- Perform: continuous part (G4HepEmElectronManager.icc:375-405).  With
    // no geometry the geometrical step is the one HowFar proposed, so the
    // true length is the MSC true length.
    t.edep = 0.0;
    t.pstep = t.gstep;
    if (!(gstep > 0.f)) return -1;
    float p = gstep;
    bool pAtRange = pIsRange && winner == -1;  // p == range
    bool pIsStepFn = stepFn && winner == -1;   // p is the step-function value
    if (active) {
      p = trueStep;
      pAtRange = atRange;
      pIsStepFn = pIsStepFn && tsIsP;
      if (le(p, 5.E-8f) || atRange) active = false;
    }
    t.pstep = f2d(p);
#pragma unroll
    for (int i = 0; i < 4; ++i) t.nia[i] = f2d(nia[i] - p / mfp[i]);
    // mean energy loss (G4HepEmElectronManager.icc:216-259); the range->energy
    // inversion in FP64
    const double preE = e;
    const float preEf = ef;
    if (pAtRange || !dless(T.minLossE, e)) {
      t.edep = e;
      t.setE(0.0);
      return t.isEl ? -1 : kQAnnihRest;
    }
    const float elossF = p * rest_dedx32(f, nL, imc, ef, lef);
    double eloss = f2d(elossF);
    if (lt(ld(&reg.linELossLimit) * ef, elossF)) {
      const double range64 = rest_range64(d, f, imc, e, lef);
      double rp;
      if (pIsStepFn) {
        // range - p of the step function, (1 - dR/R)(range - finalRange)^2 / range,
        // in FP64 without the cancellation of range - p (range close to finalRange)
        const DevRegion& r64 = T.regions[cRegion];
        const double dF = range64 - ld(&r64.finalRange);
        rp = (1.0 - ld(&r64.dRoverRange)) * dF * dF / range64;
      } else {
        rp = range64 - f2d(p);
        // E(range - p) is ill-conditioned when p is close to the range: it
        // inherits p's FP32 error (~3e-7) times 0.6 p / (range - p); keep that
        // below ~5e-6 (range - p >= range / 25)
        if (range - p < 0.04f * range) set_trip();
      }
      eloss = e - inv_range64(d, f, imc, rp);
    }
    eloss = dpos(eloss);
    HEPEM_TR(1, 14, eloss);
    if (!dless(eloss, e)) {  // only after the inversion, where p close to the range has tripped
      t.setE(0.0);
      t.edep = e;
      return t.isEl ? -1 : kQAnnihRest;
    }
    double postE = e - eloss;
    t.setE(postE);
    t.edep = eloss;
    // MSC angular deflection and displacement (G4HepEmElectronManager.icc:261-322)
    if (active && lt(fmx(1.0E-8f, 1.0e-16f * lambtr1), p)) {
      float pE = preEf, pLE = lef;
      if (lt(range * 0.01f, p)) {
        pE = d2f(postE);
        pLE = logf(pE);
      }
      const float postMFP = transport_mfp32(f, nL, cMat, pE, pLE);
      const CosT ct = cos_theta(p, preEf, lambtr1, pE, postMFP, tlimitMin, md, tsIsTlm);
      HEPEM_TR(1, 21, 1.0 - (double)ct.omc);
      // the reference skips the deflection when cos(theta) rounds to +-1 in
      // FP64: a computed value within a few ulp of that is undecidable here
      const float mc = fmn(ct.omc, ct.opc);
      if (!exactCos && mc < 1.0E-15f) set_trip();
      if (mc > 0.f) {
        const float sth = sqrtf(ct.omc * ct.opc);
        const float cost = ct.omc < 1.f ? 1.f - ct.omc : ct.opc - 1.f;
        const double uphi = rng.flat();
        const float phiN = 2.f * d2f(uphi);  // phi / pi
        float sp, cp;
        sincospif(phiN, &sp, &cp);
        float dir[3] = {sth * cp, sth * sp, cost};
        const float tdir[3] = {d2f(t.dir[0]), d2f(t.dir[1]), d2f(t.dir[2])};
        float disp[3] = {0.f, 0.f, 0.f};
        bool dsp = displace && T.mscDisplacement;
        if (dsp && delta > 0.f) {
          const float r = 0.73f * sqrtf(delta * (p + zPath));
          HEPEM_TR(1, 22, r);
          HEPEM_TR(1, 23, delta);
          const float cbeta = 2.16f;
          const double r0 = rng.flat(), r1 = rng.flat();
          // -ln(1 - r0 (1 - e^-cbeta pi)) / cbeta, with 1 - r0 (1 - q) = (1 - r0) + r0 q:
          // no cancellation as r0 -> 1
          const float q = expf(-cbeta * (float)kPi);
          const float psi = -logf(one_minus_u(r0) + d2f(r0) * q) / cbeta;
          const float psiN = psi * (float)(1.0 / kPi);
          const float phN = lt(d2f(r1), 0.5f) ? phiN + psiN : phiN - psiN;
          float s2, c2;
          sincospif(phN, &s2, &c2);
          disp[0] = r * c2;
          disp[1] = r * s2;
          rotate_mixed(disp, tdir, t.dir);
        } else {
          dsp = false;
        }
        rotate_mixed(dir, tdir, t.dir);
        // renormalise (one Newton step on the reciprocal square root) so that
        // repeated steps keep unit directions
        const float n2 = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
        float inv = rsqrtf(n2);
        inv = inv * (1.5f - 0.5f * n2 * inv * inv);
        t.dir[0] = f2d(dir[0] * inv);
        t.dir[1] = f2d(dir[1] * inv);
        t.dir[2] = f2d(dir[2] * inv);
        if (dsp) {
          t.msc.disp[0] = f2d(disp[0]);
          t.msc.disp[1] = f2d(disp[1]);
          t.msc.disp[2] = f2d(disp[2]);
        }
      }
    }
    // energy loss fluctuations (G4HepEmElectronManager.icc:324-368)
    double finalE = postE;
    if (ld(&reg.eLossFluct) && lt(1.E-5f, d2f(eloss))) {
      const float tmax = t.isEl ? 0.5f * preEf : preEf;
      const float tcut = fmn(ld(&T.couples32[imc].elCut), tmax);
      eloss = f2d(fmx(fluct(tcut, ld(&md.meanExc), d2f(eloss)), 0.f));
      finalE = preE - eloss;
      HEPEM_TR(1, 15, eloss);
      // the final energy inherits eloss's relative error (~3e-7) times
      // eloss / finalE: keep that below ~3e-6
      if (d2f(finalE) < 0.1f * preEf) set_trip();
    }
    if (le(d2f(finalE), T.elTrackingCut32)) {
      t.setE(0.0);
      t.edep = preE;
      return t.isEl ? -1 : kQAnnihRest;
    }
    t.setE(finalE);
    t.edep = eloss;
    // the delta-interaction test (G4HepEmElectronManager.icc:408-423)
    const int ip = t.winner;
    if (ip < 0 || t.onBoundary) return -1;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k == ip) t.nia[k] = -1.0;
    const float fe = d2f(finalE), lfe = logf(fe);
    const float mxp = ip < 2 ? rest_macxs32(d, f, imc, finalE, fe, lfe, ip == 0)
                   : (ip < 3 ? annih_macxs32(fe, ld(&md.elDensity)) : nuc_macxs32(d, f, cMat, finalE, fe, lfe));
    const double u = rng.flat();
    const float mfpw = ip == 0 ? mfp[0] : ip == 1 ? mfp[1] : ip == 2 ? mfp[2] : mfp[3];
    if (mxp <= 0.f || !lt(d2f(u), mxp * mfpw)) return -1;
    switch (ip) {
      case 0: return t.isEl ? kQIoniEm : kQIoniEp;
      case 1: near(fe, T.bremModelLim32); return dless(finalE, T.bremModelLim) ? kQBremSB : kQBremRB;
      case 2: return kQAnnihFlight;
      default: return -1;
    }
  }

  __device__ int stage_a() {
    ElLimit32 h;
    howfar(h);
    return perform(h);
  }
};

// ---- the gamma stage A in FP32 ---------------------------------------------------------
// G4HepEmGammaManager HowFar + SelectInteraction (G4HepEmGammaManager.icc:27-130;
// Physics::gamma_howfar / gamma_select): the total macroscopic cross section,
// the step and the interaction choice from the FP32 table copy.  The energy
// windows of the table are chosen exactly (the cross section is discontinuous
// between them), the interaction choice is guarded as in MixedEl, and the
// photoelectric cross section that the photoelectric model's element selection
// uses is evaluated in FP64 for the tracks that pick it.

// spline over a row of 9 of the gamma window-2 table (G4HepEmRunUtils.icc)
__device__ __forceinline__ float spline_log_9_32(int nd, const float* d, float x, float lx, float lxm, float ild,
                                                 int iwhich) {
  const int i0 = 9 * bin32(lx, lxm, ild, nd);
  const int i1 = i0 + 9;
  const int w = (iwhich - 1) * 2 + 1;
  return spline32(ld(d + i0), ld(d + i1), ld(d + i0 + w), ld(d + i1 + w), ld(d + i0 + w + 1), ld(d + i1 + w + 1), x);
}

// FP64 photoelectric cross section of the window of e, as Physics::gamma_total_xs
// and Physics::gamma_select leave it in Track::peXS (out of line: rare)
static __device__ __noinline__ double gamma_pe_xs64(const DevTables& T, int imat, double e) {
  const DevGamma& g = T.gm;
  const double le = vdt_log(e);
  if (e > g.eMax1) {
    const int st = imat * g.dataPerMat + g.nData0 + g.nData1;
    return spline_log_9(g.nE2, g.mx + st, e, le, g.logEMin2, g.ild2, 4);
  }
  if (e > g.eMax0) {
    const double* d = g.mx + imat * g.dataPerMat + g.nData0;
    const int i3 = 3 * bin_of(le, g.logEMin1, g.ild1, g.nE1);
    const int j3 = i3 + 3;
    const double x0 = ld(d + i3);
    const double dl = ld(d + j3) - x0;
    const double b = dmax_(0., dmin_(1., (e - x0) / dl));
    return dmax_(0.0, ld(d + i3 + 2) + b * (ld(d + j3 + 2) - ld(d + i3 + 2)));
  }
  const DevMat& m = T.mats[imat];
  const int n = ld(&m.nSandia), off = ld(&m.sandiaOff);
  int iv = 0;
  if (e >= ld(T.sandiaE + off)) {
    for (int i = n - 1; i >= 0; --i)
      if (e >= ld(T.sandiaE + off + i)) { iv = i; break; }
  }
  const double* c = T.sandiaC + 4 * (off + iv);
  const double inv = 1 / e;
  return dmax_(0.0, inv * (ld(c) + inv * (ld(c + 1) + inv * (ld(c + 2) + inv * ld(c + 3)))));
}

// The FP64 interaction choice of Physics::gamma_select for a drawn uniform u,
// from the FP64 total cross section (out of line: taken only when the FP32
// choice is too close to call), with the photoelectric cross section that the
// FP64 path leaves in Track::peXS.  The track's couple and energy come by
// value: a reference to the caller's track or stream would keep them in local
// memory for the whole kernel.
struct GammaSelect64 {
  int winner;
  double peXS;
};
static __device__ __noinline__ GammaSelect64 gamma_select64(const DevTables& T, int imc, double e, double u) {
  Track t;
  t.imc = imc;
  t.setE(e);
  t.peXS = 0.0;
  Rng rng;  // nothing is drawn here
  rng.u = nullptr;
  rng.n = 0;
  rng.cursor = 0;
  rng.id = 0;
  rng.overflow = 0u;
  rng.seed = 0;
  rng.gaussValid = false;
  rng.gaussValue = 0.0;
  Physics P{T, rng, t};
  const double tot = P.gamma_total_xs();
  const double tmfp = tot > 0. ? 1. / tot : kLarge;
  const DevGamma& g = T.gm;
  if (e > g.eMax1) {
    const double le = t.logE();
    const int st = ld(&T.couples[imc].mat) * g.dataPerMat + g.nData0 + g.nData1;
    double mx = 0.0, cp = 0.0;
    int pid = 2;
    do {
      mx = pid < 5 ? spline_log_9(g.nE2, g.mx + st, e, le, g.logEMin2, g.ild2, pid) : 0.0;
      cp += mx * tmfp;
      ++pid;
    } while (pid < 6 && u > cp);
    return {pid - 3, mx};
  }
  return {(u > tmfp * t.peXS) ? 1 : 2, t.peXS};
}

// What the FP32 HowFar of MixedG leaves for its Perform.
struct GammaLimit32 {
  float tot, mfp, pe, nia0, gstep;
};

struct MixedG {
  const DevTables& T;
  Rng& rng;
  Track& t;
  bool trip;
  int tripLine;

  __device__ __forceinline__ void set_trip(int line = __builtin_LINE()) {
    if (!trip) tripLine = line;
    trip = true;
  }
  __device__ __forceinline__ void near(float a, float b, int line = __builtin_LINE()) {
    if (fabsf(a - b) <= kGuardTol * fmx(fabsf(a), fabsf(b))) set_trip(line);
  }

  // Sandia photoabsorption cross section (Physics::macxs_pe) in FP32; the
  // interval is found with exact comparisons
  __device__ float macxs_pe32(int imat, double e, float ef) {
    const DevMat& m = T.mats[imat];
    const int n = ld(&m.nSandia), off = ld(&m.sandiaOff);
    int iv = 0;
    if (!dless(e, ld(T.sandiaE + off))) {
      for (int i = n - 1; i >= 0; --i)
        if (!dless(e, ld(T.sandiaE + off + i))) { iv = i; break; }
    }
    const double* c = T.sandiaC + 4 * (off + iv);
    const float inv = 1.f / ef;
    return inv * (d2f(ld(c)) + inv * (d2f(ld(c + 1)) + inv * (d2f(ld(c + 2)) + inv * d2f(ld(c + 3)))));
  }

  // HowFar + SelectInteraction + the first part of Perform, as the FP64 stage
  // (stage_a_gamma_kernel): returns the interaction queue, -1 (no interaction
  // or on a boundary) or -2 (no interaction: tracking cut); valid if !trip.
  // howfar() is the HowFar half (total cross section, mean free path and the
  // proposed step in FP32, kept in a GammaLimit32), perform() the rest with
  // the geometrical step gstep (the proposed one in stage_a).
  __device__ int stage_a() {
    GammaLimit32 q;
    howfar(q);
    return perform(q, q.gstep);
  }

  __device__ void howfar(GammaLimit32& q) {
    const DevGamma& g = T.gm;
    const DevGamma32& h = T.gm32;
    if (nonpositive(t.nia[0])) t.nia[0] = f2d(neg_log_u(rng.flat()));
    const double e = t.e;
    const float ef = d2f(e), lef = logf(ef);
    const int imat = ld(&T.couples[t.imc].mat);
    const bool w2 = dless(g.eMax1, e), w1 = !w2 && dless(g.eMax0, e);
    float tot, pe = 0.f;
    if (w2) {
      const int st2 = imat * g.dataPerMat + g.nData0 + g.nData1;
      tot = spline_log_9_32(g.nE2, h.mx + st2, ef, lef, h.logEMin2, h.ild2, 1);
    } else if (w1) {
      const float* d = h.mx + imat * g.dataPerMat + g.nData0;
      const int i3 = 3 * bin32(lef, h.logEMin1, h.ild1, g.nE1);
      const int j3 = i3 + 3;
      const float x0 = ld(d + i3);
      const float b = fmx(0.f, fmn(1.f, (ef - x0) / (ld(d + j3) - x0)));
      tot = fmx(0.f, ld(d + i3 + 1) + b * (ld(d + j3 + 1) - ld(d + i3 + 1)));
      pe = fmx(0.f, ld(d + i3 + 2) + b * (ld(d + j3 + 2) - ld(d + i3 + 2)));
    } else {
      const float* d = h.mx + imat * g.dataPerMat;
      const int i2 = 2 * bin32(lef, h.logEMin0, h.ild0, g.nE0);
      const float x1 = ld(d + i2);
      const float b = fmx(0.f, fmn(1.f, (ef - x1) / (ld(d + i2 + 2) - x1)));
      const float y1 = ld(d + i2 + 1);
      pe = fmx(0.f, macxs_pe32(imat, e, ef));
      tot = y1 + b * (ld(d + i2 + 3) - y1) + pe;
    }
    q.tot = tot;
    q.mfp = tot > 0.f ? 1.f / tot : kLargeF;
    q.pe = pe;
    q.nia0 = d2f(t.nia[0]);
    q.gstep = q.mfp * q.nia0;
  }

  // gstep: the geometrical step made (FP32)
  __device__ int perform(const GammaLimit32& q, float gstep) {
    const DevGamma& g = T.gm;
    const DevGamma32& h = T.gm32;
    const double e = t.e;
    const float ef = d2f(e), lef = logf(ef);
    const int imat = ld(&T.couples[t.imc].mat);
    const bool w2 = dless(g.eMax1, e);
    const int st2 = w2 ? imat * g.dataPerMat + g.nData0 + g.nData1 : 0;
    const float mfp = q.mfp, pe = q.pe, nia0 = q.nia0;
    t.mfp[0] = f2d(mfp);
    t.gstep = f2d(gstep);
    t.pstep = t.gstep;
    t.edep = 0.0;
    if (t.onBoundary) {
      t.nia[0] = f2d(nia0 - gstep / mfp);
      return -1;
    }
    // SelectInteraction; a choice whose FP32 operands are too close to call is
    // made again in FP64 (gamma_select64) instead of sending the track back
    const double ud = rng.flat();
    const float u = d2f(ud);
    bool tie = false;
    int winner;
    if (w2) {
      float cp = 0.f;
      int pid = 2;
      do {
        const float mx = pid < 5 ? spline_log_9_32(g.nE2, h.mx + st2, ef, lef, h.logEMin2, h.ild2, pid) : 0.f;
        cp += mx * mfp;
        tie = tie || fabsf(u - cp) <= kGuardTol * fmx(fabsf(u), fabsf(cp));
        ++pid;
      } while (pid < 6 && u > cp);
      winner = pid - 3;
    } else {
      tie = fabsf(u - mfp * pe) <= kGuardTol * fmx(fabsf(u), fabsf(mfp * pe));
      winner = u > mfp * pe ? 1 : 2;
    }
    if (tie) {
      const GammaSelect64 s64 = gamma_select64(T, t.imc, t.e, ud);
      winner = s64.winner;
      t.peXS = winner == 2 ? s64.peXS : 0.0;
    } else {
      t.peXS = winner == 2 ? gamma_pe_xs64(T, imat, e) : 0.0;
    }
    t.winner = winner;
    // Perform up to the interaction: nia -= gstep / mfp after SelectInteraction set it to -1
    t.nia[0] = winner == 0 ? -1.0 : f2d(-1.f - gstep / mfp);
    switch (winner) {
      case 0: return kQConversion;
      case 1: return kQCompton;
      case 2: return kQPhotoelectric;
      default: return -2;
    }
  }
};

// ---- stage B of the precision form: the costly interaction models ---------------------
// Bethe-Heitler pair production, Seltzer-Berger and relativistic brem, the
// modified-Tsai angles, Moller/Bhabha and Klein-Nishina Compton with their
// rejection functions in FP32; FP64 is kept for the kinematic limits (e.g.
// eps0 = m c^2 / E, the photon-energy sampling of the relativistic model near
// the dielectric cut-off, the positron-correction velocities near the end
// point), the target-element selection and the energy bookkeeping.  Guards as
// in MixedEl: a tripped track is left to the FP64 interaction kernel.
struct MixedB {
  const DevTables& T;
  Rng& rng;
  Track& t;
  bool trip;
  int tripLine;  // source line of the first guard that tripped (diagnostics)

  __device__ __forceinline__ void set_trip(int line = __builtin_LINE()) {
    if (!trip) tripLine = line;
    trip = true;
  }

  __device__ __forceinline__ void near(float a, float b, int line = __builtin_LINE()) {
    if (fabsf(a - b) <= kGuardTol * fmx(fabsf(a), fabsf(b))) set_trip(line);
  }
  __device__ __forceinline__ void neard(double a, double b, int line = __builtin_LINE()) {
    if (fabs(a - b) <= (double)kGuardTol * fmax(fabs(a), fabs(b))) set_trip(line);
  }
  __device__ __forceinline__ bool lt(float a, float b, int line = __builtin_LINE()) {
    near(a, b, line);
    return a < b;
  }
  __device__ __forceinline__ const DevElData& eld() const { return t.isEl ? T.el[0] : T.el[1]; }
  __device__ __forceinline__ const DevCouple& couple() const { return T.couples[t.imc]; }

  // modified-Tsai polar angle (G4HepEmInteractionUtils.icc:10-22) as the pair
  // 1 - cos = 2 w^2, 1 + cos = 2 (1 - w)(1 + w), w = u / umax, in FP32.  Near the
  // backward limit w -> 1, 1 + cos carries u's relative error times 1 / (1 - w):
  // for w > 0.9 the accepted u is recomputed in FP64.
  __device__ void tsai_pair(double E, float& omc, float& opc) {
    const float umax = 2.0f * (1.0f + d2f(E) * (float)kInvMec2);
    float u;
    double r01;
    bool low;
    int it = 0;
    do {
      const double r0 = rng.flat(), r1 = rng.flat(), r2 = rng.flat();
      r01 = r0 * r1;
      low = dless(r2, 0.25);
      const float uu = neg_log_u(r01);
      u = low ? uu * 1.6f : uu * 0.533333333f;
      near(u, umax);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (u > umax);
    const float w = u / umax;
    if (w > 0.9f) {
      const double umax64 = 2.0 * (1.0 + E * kInvMec2);
      const double w64 = -vdt_log(r01) * (low ? 1.6 : 0.533333333) / umax64;
      omc = d2f(2.0 * w64 * w64);
      opc = d2f(2.0 * (1.0 - w64) * (1.0 + w64));
      return;
    }
    omc = 2.0f * w * w;
    opc = 2.0f * (1.0f - w) * (1.0f + w);
  }
  // a unit vector at polar angle (1 - cos, 1 + cos) and azimuth pi phiN about the
  // direction rd (FP64 input), in FP32 (FP64 rotation close to the z axis)
  __device__ static void dir_about(float omc, float opc, float phiN, const double* rd, double* out) {
    float sp, cp;
    sincospif(phiN, &sp, &cp);
    const float st = sqrtf(fmx(0.f, omc * opc));
    float v[3] = {st * cp, st * sp, omc < 1.f ? 1.f - omc : opc - 1.f};
    const float r[3] = {d2f(rd[0]), d2f(rd[1]), d2f(rd[2])};
    rotate_mixed(v, r, rd);
    out[0] = f2d(v[0]);
    out[1] = f2d(v[1]);
    out[2] = f2d(v[2]);
  }

  // The secondaries of an e+- interaction are rotated to the frame of the
  // track direction, whose azimuthal axes turn by (direction error) / sin(theta_z)
  // close to the z axis: within sin(theta_z) < 0.063 the FP32-stepped direction
  // (error ~3e-7) would not give the FP64 secondary directions to ~5e-6, and the
  // FP64 code takes the track.
  bool dirExact;  // the track direction is an exact input (not stepped in FP32): no guard
  __device__ __forceinline__ void frame_guard() {
    if (dirExact) return;
    const float x = d2f(t.dir[0]), y = d2f(t.dir[1]);
    if (x * x + y * y < 0.004f) set_trip();
  }

  // the e+- target element of a brem model: the reference selector's
  // interpolation in FP32, its comparisons with u guarded (E carries the FP32
  // continuous loss; the interpolated cumulatives are continuous across the
  // energy knots, so the bin may come from the FP32 log)
  __device__ int select_brem_target(double E, double le, double u, int which) {
    const DevElData& d = eld();
    const int st = ld(d.selStart[which] + t.imc);
    const double* D = d.sel[which] + st;
    const int nd = (int)ld(D);
    const int ne = (int)ld(D + 1);
    const double* x = D + 4;
    const double x0 = ld(x), xn = ld(x + ne * (nd - 1));
    const double xv = dless(E, x0) ? x0 : dless(xn, E) ? xn : E;
    int ie = (int)((d2f(le) - d2f(ld(D + 2))) * d2f(ld(D + 3)));
    ie = ie < 0 ? 0 : (ie > nd - 2 ? nd - 2 : ie);
    int i0 = ie * ne, i1 = i0 + ne;
    const double x1 = ld(x + i0++), x2 = ld(x + i1++);
    const float b = fmx(0.f, fmn(1.f, d2f(xv - x1) / d2f(x2 - x1)));
    const float uf = d2f(u);
    int k = 0;
    while (k < ne - 1) {
      const float c0 = d2f(ld(x + i0 + k));
      const float c = c0 + b * (d2f(ld(x + i1 + k)) - c0);
      near(uf, c);
      if (!(uf > c)) break;
      ++k;
    }
    return k;
  }

  // unit vector along a x - b y (a, b >= 0; x, y unit vectors): the difference
  // in FP64 (it may cancel), its normalisation in FP32; returns |a x - b y|^2
  __device__ static float unit_diff(double a, const double* x, double b, const double* y, double* out) {
    const float fx = d2f(a * x[0] - b * y[0]), fy = d2f(a * x[1] - b * y[1]), fz = d2f(a * x[2] - b * y[2]);
    const float n2 = fx * fx + fy * fy + fz * fz;
    float inv = rsqrtf(n2);
    inv = inv * (1.5f - 0.5f * n2 * inv * inv);
    out[0] = f2d(fx * inv);
    out[1] = f2d(fy * inv);
    out[2] = f2d(fz * inv);
    return n2;
  }

  // ---- Moller / Bhabha (G4HepEmElectronInteractionIoni.icc:19-138) ------------------
  __device__ void ioni() {
    const double E = t.e;
    const double cut = couple().elCut;
    const double tmaxE = t.isEl ? 0.5 * E : E;
    near(d2f(tmaxE), d2f(cut));
    if (!dless(cut, tmaxE)) return;
    frame_guard();
    const float Ef = d2f(E);
    const float xmin = d2f(cut) / Ef;
    float x, omx = 1.f;
    int it = 0;
    if (t.isEl) {
      const float xmax = 0.5f;
      const float gam = Ef * (float)kInvMec2 + 1.0f;
      const float g2 = gam * gam;
      const float xmm = xmin * xmax;
      const float gg = (2.0f * gam - 1.0f) / g2;
      const float y = 1.f - xmax;
      const float gf = 1.0f - gg * xmax + xmax * xmax * (1.0f - gg + (1.0f - gg * y) / (y * y));
      float dum, g;
      do {
        const double r0 = rng.flat(), r1 = rng.flat();
        x = xmm / (xmin * one_minus_u(r0) + xmax * d2f(r0));
        const float xx = 1.0f - x;
        dum = 1.0f - gg * x + x * x * (1.0f - gg + (1.0f - gg * xx) / (xx * xx));
        g = gf * d2f(r1);
        near(g, dum);
        if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
      } while (g > dum);
    } else {
      const float xmax = 1.0f;
      const float gam = Ef * (float)kInvMec2 + 1.0f;
      const float g2 = gam * gam;
      const float b2 = 1.f - 1.f / g2;
      const float xmm = xmin * xmax;
      const float y = 1.0f / (1.0f + gam);
      const float y2 = y * y;
      const float y12 = 1.0f - 2.0f * y;
      const float c1 = 2.0f - y2;
      const float c2 = y12 * (3.0f + y2);
      const float y122 = y12 * y12;
      const float c4 = y122 * y12;
      const float c3 = c4 + y122;
      const float xmax2 = xmax * xmax;
      const float gf = 1.0f + (xmax2 * c4 - xmin * xmin * xmin * c3 + xmax2 * c2 - xmin * c1) * b2;
      float dum, g;
      do {
        const double r0 = rng.flat(), r1 = rng.flat();
        const float den = xmin * one_minus_u(r0) + xmax * d2f(r0);
        x = xmm / den;
        omx = d2f(r0) * (1.f - xmin) / den;  // 1 - x, xmax = 1
        const float xx = x * x;
        dum = 1.0f + (xx * xx * c4 - x * xx * c3 + xx * c2 - x * c1) * b2;
        g = gf * d2f(r1);
        near(g, dum);
        if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
      } while (g > dum);
    }
    const double dE = f2d(x) * E;
    Sec& s = t.addSec(0);
    // the polar angle in FP64 (cos close to 1 at high energy), 1 -+ cos to FP32
    const double eTot = E + kMec2;
    const double pTot = sqrt(E * (eTot + kMec2));
    const double dP = sqrt(dE * (dE + 2.0 * kMec2));
    const double cost = dE * (eTot + kMec2) / (dP * pTot);
    const double ct = dmax_(-1.0, dmin_(cost, 1.0));
    dir_about(d2f(1.0 - ct), d2f(1.0 + ct), 2.f * d2f(rng.flat()), t.dir, s.dir);
    unit_diff(pTot, t.dir, dP, s.dir, t.dir);
    const double eAfter = !t.isEl && omx < 0.5f ? E * f2d(omx) : E - dE;
    t.setE(eAfter);
    s.e = E - eAfter;
    if (eAfter * (eAfter + 2.0 * kMec2) < 4.0e-4 * pTot * pTot) set_trip();  // as in brem
  }

  // ---- bremsstrahlung (G4HepEmElectronInteractionBrem.icc:35-344) -------------------
  // 1 - k/E of the last sample_sb, kept without cancellation (photon taking
  // nearly all the energy); < 0: not set, the electron keeps E - k
  double omk;

  __device__ void brem(bool sbModel) {
    const double E = t.e;
    const double gcut = ld(&couple().gamCut);
    near(d2f(E), d2f(gcut));
    if (!dless(gcut, E)) return;
    frame_guard();
    omk = -1.0;
    // log E in FP32 (error < 2e-6): the target selection only bins with it,
    // and the Seltzer-Berger energy-bin choice that uses it is guarded by 2e-5
    const double le = f2d(logf(d2f(E)));
    const double k = sbModel ? sample_sb(E, le) : sample_rb(E, le);
    Sec& s = t.addSec(2);
    float omc, opc;
    tsai_pair(E, omc, opc);
    dir_about(omc, opc, 2.f * d2f(rng.flat()), t.dir, s.dir);
    const double eTot = E + kMec2;
    const double pTot = sqrt(E * (eTot + kMec2));
    unit_diff(pTot, t.dir, k, s.dir, t.dir);
    // the smaller of the two energies is formed directly, the other as the
    // complement, so that E is shared exactly
    const double eAfter = omk >= 0.0 && omk < 0.5 ? E * omk : E - k;
    t.setE(eAfter);
    s.e = E - eAfter;
    // the electron's new direction is a difference of momenta ~ pTot: its
    // error is the incoming direction's (~1e-7, FP32 MSC) times pTot / p_after
    if (eAfter * (eAfter + 2.0 * kMec2) < 4.0e-4 * pTot * pTot) set_trip();
  }

  // first index i (a multiple of 3) with v[i] > val, as Physics::lin_search;
  // these cumulatives and val are >= 0, so their bit patterns order as integers
  __device__ static int lin_search_bits(const double* v, int size, double val) {
    int i = 0;
    const int s3 = 3 * size;
    while (i + 9 < s3) {
      if (dless(val, ld(v + i))) return i;
      if (dless(val, ld(v + i + 3))) return i + 3;
      if (dless(val, ld(v + i + 6))) return i + 6;
      if (dless(val, ld(v + i + 9))) return i + 9;
      i += 12;
    }
    while (i < s3) {
      if (dless(val, ld(v + i))) break;
      i += 3;
    }
    return i;
  }

  __device__ double sample_sb(double E, double le) {
    const DevCouple c = couple();
    const double gcut = c.gamCut, lgcut = c.logGamCut;
    const DevMat& md = T.mats[c.mat];
    const int nElem = ld(&md.nElem);
    const int ei = nElem > 1 ? select_brem_target(E, le, rng.flat(), 1) : 0;
    const int Z = ld(T.matElemZ + ld(&md.elemOff) + ei);
    const DevSB& sb = T.sb;
    const int st = ld(sb.startPerZ + Z);
    const int gci = ld(sb.gcIdx + ld(sb.gcStart + t.imc) + ei);
    bool corner = false, simple = false;
    int ie = (int)ld(sb.data + st + 2);
    neard(E, ld(sb.elE + ie));
    if (E < ld(sb.elE + ie)) {
      const double val = (le - sb.logMinE) * sb.ildE;
      ie = (int)val;
      double pH = val - ie;
      // le carries the FP32 log's error: pH to ~1e-5 absolute
      if (pH < 2e-5 || pH > 1.0 - 2e-5) set_trip();
      if (ie < 0 || ie > kNumElEnergySB - 2) { t.flags |= kFlagBadIndex; return E; }
      if (ld(sb.elE + ie) <= gcut) {
        pH = (le - lgcut) / (ld(sb.lelE + ie + 1) - lgcut);
        corner = true;
      }
      const double u = rng.flat();
      neard(u, pH);
      if (fabs(u - pH) < 2e-5) set_trip();
      if (u < pH) ++ie;
      else if (corner) simple = true;
    }
    const int minIE = (int)ld(sb.data + st + 1);
    const int maxIE = (int)ld(sb.data + st + 2);
    if (ie < minIE || ie > maxIE) { t.flags |= kFlagBadIndex; return E; }
    const int ncut = (int)ld(sb.data + st + 3);
    const int size1 = ncut + 3 * kNumKappaSB;
    const int tst = st + 4 + (ie - minIE) * size1;
    const double minV = ld(sb.data + tst + gci);
    const double* Tb = sb.data + tst + ncut;
    const float lkt = d2f(lgcut - le) / d2f(lgcut - ld(sb.lelE + ie));
    const float Ef = d2f(E);
    const float pe = Ef + (float)kMec2;
    const float dsc = d2f(ld(&md.densityCor)) * pe * pe;
    // positron correction: the velocity at E - gcut is fixed, the one at E - k
    // is evaluated in FP64 (kinematic end point k -> E)
    double ib1 = 0.0;
    if (!t.isEl) {
      const double e1 = E - gcut;
      ib1 = (e1 + kMec2) / sqrt(e1 * (e1 + 2.0 * kMec2));
    }
    const float zfac = (float)(kAlpha * k2Pi) * (float)Z;
    double k = 0.0;
    float sup = 1.0f, r1f = 0.f;
    double r1;
    int it = 0;
    do {
      const double r0 = rng.flat();
      r1 = rng.flat();
      float kappa = 1.0f;
      float kf;
      if (!simple) {
        const double cum = r0 * (1.0 - minV) + minV;
        int i3 = lin_search_bits(Tb, kNumKappaSB, cum) - 3;
        if (i3 > 3 * (kNumKappaSB - 2)) { i3 = 3 * (kNumKappaSB - 2); t.flags |= kFlagBadIndex; }
        if (i3 < 0) { i3 = 0; t.flags |= kFlagBadIndex; }
        const int i = i3 / 3;
        const double cL = ld(Tb + i3), cH = ld(Tb + i3 + 3);
        const float pA = d2f(ld(Tb + i3 + 1)), pB = d2f(ld(Tb + i3 + 2));
        const float lKL = d2f(ld(sb.lkappa + i)), lKH = d2f(ld(sb.lkappa + i + 1));
        // the rational inverse interpolation lk = lKL + m2/m3 (lKH - lKL) written as
        // lKH - (lKH - lKL)(1 - m1)(1 - pB m1)/m3, exact in the top bin (lKH = 0);
        // m1 and 1 - m1 from FP64 differences of the cumulatives
        const float dc = d2f(cH - cL);
        const float m1 = d2f(cum - cL) / dc, om1 = d2f(cH - cum) / dc;
        const float m3 = 1.0f + m1 * (pA + pB * m1);
        const float lk = lKH - (lKH - lKL) * om1 * (1.0f - pB * m1) / m3;
        kappa = expf(lk * lkt);
        k = f2d(kappa) * E;
        kf = kappa * Ef;
        omk = f2d(-expm1f(lk * lkt));
      } else {
        const double om = r0 * (1.0 - gcut / E);
        k = (1.0 - om) * E;
        omk = om;
        kf = d2f(k);
      }
      const float ik = 1.0f / kf;
      sup = 1.0f / (1.0f + dsc * ik * ik);
      if (!t.isEl) {
        const double e2 = omk >= 0.0 && omk < 0.5 ? E * omk : E - k;
        const double ib2 = (e2 + kMec2) / sqrt(e2 * (e2 + 2.0 * kMec2));
        const float dum = zfac * (float)(ib1 - ib2);
        near(dum, -12.f);
        sup = dum > -12.f ? sup * expf(dum) : 0.f;
      }
      r1f = d2f(r1);
      near(r1f, sup);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (r1f > sup);
    return k;
  }

  __device__ static void lpm_functions32(float& xiS, float& gS, float& phiS, float eg, float et, float elpm,
                                         float z23, float ilS1, float ilS1c, float dcor, float times) {
    const float sqrt2 = 1.41421356f;
    const float red = eg / et;
    const float sP = sqrtf(0.125f * red * elpm / (times * (1.0f - red) * et));
    const float s1 = z23 / (184.15f * 184.15f);
    const float cond = sqrt2 * s1;
    float xiSP = 2.0f;
    if (sP > 1.0f) {
      xiSP = 1.0f;
    } else if (sP > cond) {
      const float h = logf(sP) * ilS1c;
      xiSP = 1.0f + h - 0.08f * (1.0f - h) * h * (2.0f - h) * ilS1c;
    }
    xiS = xiSP;
    const float s = sP / sqrtf(xiSP);
    float sh = s;
    if (dcor != 0.0f) {
      sh *= (1.0f + dcor / (eg * eg));
      xiS = 2.0f;
      if (sh > 1.0f) xiS = 1.0f;
      else if (sh > s1) xiS = 1.0f + logf(sh) * ilS1;
    }
    if (sh < 2.0f) {
      float val = sh * 20.0f;
      int il = (int)val;
      val -= il;
      il *= 2;
      il = il < 0 ? 0 : (il > 78 ? 78 : il);
      const float f0 = d2f(kFuncLPM[il]), f1 = d2f(kFuncLPM[il + 1]);
      gS = (d2f(kFuncLPM[il + 2]) - f0) * val + f0;
      phiS = (d2f(kFuncLPM[il + 3]) - f1) * val + f1;
    } else {
      float ss = 1.0f / (sh * sh);
      ss *= ss;
      gS = 1.0f - 0.0230655f * ss;
      phiS = 1.0f - 0.01190476f * ss;
    }
    if (xiS * phiS > 1.0f || sh > 0.57f) xiS = 1.0f / phiS;
  }

  __device__ double sample_rb(double E, double le) {
    const DevCouple c = couple();
    const double gcut = c.gamCut;
    const DevMat& md = T.mats[c.mat];
    const int nElem = ld(&md.nElem);
    const int ei = nElem > 1 ? select_brem_target(E, le, rng.flat(), 2) : 0;
    const int Z = ld(T.matElemZ + ld(&md.elemOff) + ei);
    const float dZ = (float)Z;
    const DevElem& el = T.elems[Z < kMaxZ ? Z : kMaxZ];
    const double dens = kMigdal * ld(&md.elDensity);
    const double lpmE = kLPM * ld(&md.radLength);
    const double lpmLim = sqrt(dens) * lpmE;
    const double pte = E + kMec2;
    const double dcor = dens * pte * pte;
    neard(pte, lpmLim);
    const bool lpm = pte > lpmLim;
    const float zf1 = d2f(ld(&el.zFactor1));
    const float zf2 = (1.f + 1.f / dZ) / 12.f;
    const float fmax = zf1 + zf2;
    // photon energy k^2 = exp(xmin + r0 xr) - dcor: in the loop in FP32 as
    // gcut^2 e^y + dcor (e^y - 1), y = r0 xr, without the cancellation of the
    // difference; the accepted k in FP64 by the reference's own formula
    const double xmin = vdt_log(gcut * gcut + dcor);
    const double xr = vdt_log(E * E + dcor) - xmin;
    const float xrf = d2f(xr), gcut2f = d2f(gcut * gcut);
    const float ptef = d2f(pte), lpmEf = d2f(lpmE), dcorf = d2f(dcor);
    const float z23 = d2f(ld(&el.Z23)), ilS1 = d2f(ld(&el.ilVarS1)), ilS1c = d2f(ld(&el.ilVarS1Cond));
    const float z13 = d2f(ld(&el.Z13)), lz = d2f(ld(&el.logZ)), coul = d2f(ld(&el.coulomb));
    double r0, r1;
    float fv, g;
    int it = 0;
    do {
      r0 = rng.flat();
      r1 = rng.flat();
      const float yk = d2f(r0) * xrf;
      const float kf = sqrtf(gcut2f * expf(yk) + dcorf * expm1f(yk));
      const float y = kf / ptef;
      const float omy = 1.f - y;
      const float d0 = 0.25f * y * y;
      if (lpm) {
        float xiS, gS, phiS;
        lpm_functions32(xiS, gS, phiS, kf, ptef, lpmEf, z23, ilS1, ilS1c, dcorf, 1.0f);
        const float t1 = xiS * (d0 * gS + (omy + 2.0f * d0) * phiS);
        fv = t1 * zf1 + omy * zf2;
      } else {
        const float d1 = omy + 3.f * d0;
        if (Z < 5) {
          fv = d1 * zf1 + omy * zf2;
        } else {
          const float d2 = y / (ptef - kf);
          const float gam = d2 * 100.f * (float)kMec2 / z13;
          const float eps = gam / z13;
          const float g2 = gam * gam;
          const float phi1 = 16.863f - 2.0f * log1pf(0.311877f * g2) + 2.4f * expf(-0.9f * gam) +
                             1.6f * expf(-1.5f * gam);
          const float phi2 = 2.0f / (3.0f + 19.5f * gam + 18.0f * g2);
          const float e2 = eps * eps;
          const float psi1 = 24.34f - 2.0f * log1pf(13.111641f * e2) + 2.8f * expf(-8.0f * eps) +
                             1.2f * expf(-29.2f * eps);
          const float psi2 = 2.0f / (3.0f + 120.0f * eps + 1200.0f * e2);
          const float Fz = lz / 3.f + coul;
          const float iz = 1.f / dZ;
          fv = d1 * ((0.25f * phi1 - Fz) + (0.25f * psi1 - 2.f * lz / 3.f) * iz) + 0.125f * omy * (phi2 + psi2 * iz);
        }
      }
      fv = fmx(0.0f, fv);
      g = fmax * d2f(r1);
      near(fv, g);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (fv < g);
    return sqrt(dmax_(vdt_exp(xmin + r0 * xr) - dcor, 0.0));
  }

  // ---- annihilation in flight (G4HepEmPositronInteractionAnnihilation.icc) -----------
  // the FP64 model (it is cheap) with its rejection test guarded
  __device__ void annihilate_in_flight() {
    frame_guard();
    const double E = t.e;
    Sec& g1 = t.addSec(2);
    Sec& g2 = t.addSec(2);
    const double tau = E * kInvMec2;
    const double gam = tau + 1.0;
    const double tau2 = tau + 2.0;
    const double sq = sqrt(tau / tau2) * 0.5;
    const double emin = 0.5 - sq, emax = 0.5 + sq;
    const double eq = emax / emin;
    const double tau4 = tau2 * tau2;
    double eps, rf, r1;
    int it = 0;
    do {
      const double r0 = rng.flat();
      r1 = rng.flat();
      eps = emin * vdt_exp(vdt_log(eq) * r0);
      rf = 1. - eps + (2. * gam * eps - 1.) / (eps * tau4);
      neard(rf, r1);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (rf < r1);
    const double sqg = sqrt(tau * tau2);
    const double cost = dmin_(1., dmax_(-1., (eps * tau2 - 1.) / (eps * sqg)));
    const double sint = sqrt((1. + cost) * (1. - cost));
    const double phi = k2Pi * rng.flat();
    const double initE = E + 2. * kMec2;
    const double e1 = eps * initE;
    g1.e = e1;
    double sp, cp;
    sincos(phi, &sp, &cp);
    g1.dir[0] = sint * cp;
    g1.dir[1] = sint * sp;
    g1.dir[2] = cost;
    rotate(g1.dir, t.dir);
    g2.e = initE - e1;
    const double ip = sqrt(E * (E + 2 * kMec2));
    const double px = ip * t.dir[0] - g1.dir[0] * e1;
    const double py = ip * t.dir[1] - g1.dir[1] * e1;
    const double pz = ip * t.dir[2] - g1.dir[2] * e1;
    const double p2 = px * px + py * py + pz * pz;
    if (p2 < 4.0e-4 * ip * ip) set_trip();  // second photon from a difference of momenta, as in brem
    const double nrm = 1.0 / sqrt(p2);
    g2.dir[0] = px * nrm; g2.dir[1] = py * nrm; g2.dir[2] = pz * nrm;
    t.setE(0.0);
  }

  // ---- pair production (G4HepEmGammaInteractionConversion.icc:19-274) ---------------
  __device__ static float screen1(float d) {
    return d > 1.4f ? 42.038f - 8.29f * logf(d + 0.958f) : 42.184f - d * (7.444f - 1.623f * d);
  }
  __device__ static float screen2(float d) {
    return d > 1.4f ? 42.038f - 8.29f * logf(d + 0.958f) : 41.326f - d * (5.848f - 0.902f * d);
  }
  __device__ static void phi12(float d, float& p1, float& p2) {
    if (d > 1.4f) {
      p1 = 21.0190f - 4.145f * logf(d + 0.958f);
      p2 = p1;
    } else {
      p1 = 20.806f - d * (3.190f - 0.5710f * d);
      p2 = 20.234f - d * (2.126f - 0.0903f * d);
    }
  }

  // the pair-production target element (Physics::conv_target): interpolation
  // in FP32, comparisons with u guarded; the energy bin from the FP32 log (the
  // cumulatives are continuous across the energy knots)
  __device__ int conv_target32(int imat, double e, double u) {
    const DevGamma& g = T.gm;
    const double* D = g.conv + ld(g.convStart + imat);
    const int nd = g.convN;
    const int ne = (int)ld(D);
    const double* x = g.convGrid;
    const double x0 = ld(x), xn = ld(x + nd - 1);
    const double xv = dless(e, x0) ? x0 : dless(xn, e) ? xn : e;
    int ie = (int)((logf(d2f(e)) - d2f(g.convLogMin)) * d2f(g.convILD));
    ie = ie < 0 ? 0 : (ie > nd - 2 ? nd - 2 : ie);
    const double x1 = ld(x + ie), x2 = ld(x + ie + 1);
    const float b = fmx(0.f, fmn(1.f, d2f(xv - x1) / d2f(x2 - x1)));
    const int i0 = ie * (ne - 1) + 1;
    const int i1 = i0 + (ne - 1);
    const float uf = d2f(u);
    int k = 0;
    while (k < ne - 1) {
      const float c0 = d2f(ld(D + i0 + k));
      const float c = c0 + b * (d2f(ld(D + i1 + k)) - c0);
      near(uf, c);
      if (!(uf > c)) break;
      ++k;
    }
    return k;
  }

  __device__ void conversion() {
    const double E = t.e;
    if (dless(E, 2. * kMec2)) return;
    const int imat = couple().mat;
    const DevMat& md = T.mats[imat];
    const int nElem = ld(&md.nElem);
    // the photon energy is exact here (gammas carry no FP32 continuous loss):
    // the FP64 target selection is the reference's own
    int ei = 0;
    if (nElem > 1) ei = conv_target32(imat, E, rng.flat());
    const int Z = ld(T.matElemZ + ld(&md.elemOff) + ei);
    const DevElem& el = T.elems[Z < kMaxZ ? Z : kMaxZ];
    // kinematic limits in FP64
    const double eps0 = kMec2 / E;
    // eps and dlt = eps - eps0: the kinetic energy of the lepton that takes
    // eps is E dlt, which near the threshold the difference eps E - m c^2 loses
    double eps = 0.0, dlt = 0.0;
    if (E < 2.0) {
      dlt = (0.5 - eps0) * rng.flat();
      eps = eps0 + dlt;
    } else {
      const double df = eps0 * 136. / ld(&el.Z13);
      const double dmn = 4. * df;
      const double dmx = E < 50.0 ? ld(&el.deltaMaxLow) : ld(&el.deltaMaxHigh);
      const double lz13 = 0.333333 * ld(&el.logZ);
      const double FZ = E < 50.0 ? 8. * lz13 : 8. * (lz13 + ld(&el.coulomb));
      const double epsp = 0.5 - 0.5 * sqrt(1. - dmn / dmx);
      const double epsMin = dmax_(eps0, epsp);
      const double epsRange = 0.5 - epsMin;
      const float dmnf = d2f(dmn), FZf = d2f(FZ), dff = d2f(df);
      float F10, F20;
      if (dmnf > 1.4f) {
        F10 = 42.038f - 8.29f * logf(dmnf + 0.958f);
        F20 = F10;
      } else {
        F10 = 42.184f - dmnf * (7.444f - 1.623f * dmnf);
        F20 = 41.326f - dmnf * (5.848f - 0.902f * dmnf);
      }
      F10 -= FZf;
      F20 -= FZf;
      const float epsRf = d2f(epsRange), epsMinf = d2f(epsMin);
      const float N1 = fmx(F10 * epsRf * epsRf, 0.f);
      const float N2 = fmx(1.5f * F20, 0.f);
      const float cond = N1 / (N1 + N2);
      const float iF10 = 1.f / F10, iF20 = 1.f / F20;
      double r1;
      bool first;
      float gr, r2f;
      int it = 0;
      const bool lpmRegime = !dless(E, 100000.0);
      const float lpmEf = d2f(kLPM * ld(&md.radLength));
      const float z23 = d2f(ld(&el.Z23)), il1 = d2f(ld(&el.ilVarS1)), il1c = d2f(ld(&el.ilVarS1Cond));
      const float Ef = d2f(E);
      do {
        const double r0 = rng.flat();
        r1 = rng.flat();
        r2f = d2f(rng.flat());
        first = lt(d2f(r0), cond);
        const float ef = first ? 0.5f - epsRf * cbrtf(d2f(r1)) : epsMinf + epsRf * d2f(r1);
        const float dd = dff / (ef * (1.f - ef));
        if (!lpmRegime) {
          gr = first ? (screen1(dd) - FZf) * iF10 : (screen2(dd) - FZf) * iF20;
        } else {
          float xiS, gS, phiS, p1, p2;
          phi12(dd, p1, p2);
          lpm_functions32(xiS, gS, phiS, Ef, ef * Ef, lpmEf, z23, il1, il1c, 0.0f, -1.0f);
          gr = first ? xiS * ((2.f * phiS + gS) * p1 - gS * p2 - phiS * FZf) * iF10
                     : xiS * ((phiS + 0.5f * gS) * p1 + 0.5f * gS * p2 - 0.5f * (gS + phiS) * FZf) * iF20;
        }
        near(gr, r2f);
        if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
      } while (gr < r2f);
      // the accepted eps and dlt = eps - eps0 in FP64
      if (first) {
        const double cr = f2d(cbrtf(d2f(r1)));
        eps = 0.5 - epsRange * cr;
        // 1 - cbrt(r1) = (1 - r1) / (1 + c + c^2)
        dlt = (epsMin - eps0) + epsRange * ((1.0 - r1) / (1.0 + cr + cr * cr));
      } else {
        eps = epsMin + epsRange * r1;
        dlt = (epsMin - eps0) + epsRange * r1;
      }
    }
    // kinetic energies: E dlt for the eps lepton, the rest of E - 2 m c^2 for the other
    const double kEps = E * dlt;
    const double kOther = dmax_(0., (E - 2.0 * kMec2) - kEps);
    double eK, pK;
    if (dless(0.5, rng.flat())) {
      eK = kOther;
      pK = kEps;
    } else {
      pK = kOther;
      eK = kEps;
    }
    Sec& se = t.addSec(0);
    Sec& sp = t.addSec(1);
    // the positron opposite in azimuth: phi + pi
    const float phiN = 2.f * d2f(rng.flat());
    float omc, opc;
    tsai_pair(eK, omc, opc);
    dir_about(omc, opc, phiN, t.dir, se.dir);
    tsai_pair(pK, omc, opc);
    dir_about(omc, opc, phiN + 1.f, t.dir, sp.dir);
    se.e = eK;
    sp.e = pK;
    t.setE(0.0);
  }

  // ---- Klein-Nishina Compton (G4HepEmGammaInteractionCompton.icc:17-103) ------------
  __device__ void compton() {
    const double E = t.e;
    const double thr = 0.0001;
    if (E < thr) return;
    const double org[3] = {t.dir[0], t.dir[1], t.dir[2]};
    const float kappa = d2f(E) * (float)kInvMec2;
    const float eps0 = 1.f / (1.f + 2.f * kappa);
    const float eps02 = eps0 * eps0;
    const float al1 = log1pf(2.f * kappa);
    const float al2 = al1 + 0.5f * (1.f - eps02);
    // 1 - cos = (1 - eps)/(eps kappa) and 1 + cos = (eps - eps0)(1 + 2 kappa)/(eps kappa)
    // are both formed from differences computed without cancellation
    float eps, ome, omc, opc, s2, gf, r2f = 0.f;
    double r2;
    int it = 0;
    do {
      const double r0 = rng.flat(), r1 = rng.flat();
      r2 = rng.flat();
      const float r1f = d2f(r1), omr1 = one_minus_u(r1);
      float dlt;  // eps - eps0
      if (lt(al2 * d2f(r0), al1)) {
        eps = expf(-al1 * r1f);
        ome = -expm1f(-al1 * r1f);
        dlt = eps0 * expm1f(al1 * omr1);
      } else {
        const float eps2 = eps02 + (1.f - eps02) * r1f;
        eps = sqrtf(eps2);
        ome = (1.f - eps02) * omr1 / (1.f + eps);
        dlt = (1.f - eps02) * r1f / (eps + eps0);
      }
      omc = ome / (eps * kappa);
      opc = dlt * (1.f + 2.f * kappa) / (eps * kappa);
      s2 = omc * opc;
      gf = 1.f - eps * s2 / (1.f + eps * eps);
      r2f = d2f(r2);
      near(gf, r2f);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (gf < r2f);
    dir_about(omc, opc, 2.f * d2f(rng.flat()), org, t.dir);
    // energies: the smaller share is computed directly, the other by difference
    double post, se;
    if (eps < 0.5f) {
      post = E * f2d(eps);
      se = E - post;
    } else {
      se = E * f2d(ome);
      post = E - se;
    }
    near(d2f(se), 1.0e-4f);
    near(d2f(post), 1.0e-4f);
    double dep = 0.0;
    if (dless(thr, se)) {
      Sec& s = t.addSec(0);
      const float q2 = unit_diff(E, org, post, t.dir, s.dir);
      // the electron direction is a difference of ~E-sized vectors built with
      // the FP32 photon angle: its error grows as E / |q|
      const float Ef2 = d2f(E);
      if (q2 < 4.0e-4f * Ef2 * Ef2) set_trip();
      s.e = se;
    } else {
      dep += se;
    }
    if (dless(thr, post)) {
      t.setE(post);
    } else {
      dep += post;
      t.setE(0.0);
    }
    t.edep = dep;
  }
};

}  // namespace hepem
