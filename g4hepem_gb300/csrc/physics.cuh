// physics.cuh -- G4HepEmRun stepping physics, FP64, device code.
//
// One physics step of one track: G4HepEmElectronManager::HowFar + Perform for
// e-/e+ and G4HepEmGammaManager::HowFar + SelectInteraction + Perform for
// gammas (reference G4HepEm/G4HepEmRun/include/*.icc, cited per function),
// evaluated on the device table image (tables.h).  Floating-point expressions
// keep the reference operand order and this file is compiled with
// --fmad=false, so with the VDT log/exp of vdt.cuh the discrete outcomes and
// all values that do not pass through sin/cos/pow are bit-identical to the
// reference host functions; sin/cos/pow are CUDA's (<= 2 ulp).
//
// Differences from the reference, all for robustness on a shared GPU:
//  * every rejection / search loop is bounded (kMaxIter); a track that hits
//    the bound stops sampling and gets kFlagLoopCap (the reference would spin);
//  * table indices derived from data are clamped to the table, with
//    kFlagBadIndex where the reference would read outside its arrays.
#pragma once

#include <cstdint>

#include "rng.cuh"
#include "tables.h"
#include "vdt.cuh"

namespace hepem {

// interaction queues of the batched form
enum : int {
  kQIoniEm = 0, kQIoniEp, kQBremSB, kQBremRB, kQAnnihFlight, kQAnnihRest, kQConversion, kQCompton,
  kQPhotoelectric, kNumQueues
};

constexpr uint8_t kFlagRngOverflow = 1u;
constexpr uint8_t kFlagLoopCap = 2u;
constexpr uint8_t kFlagBadInput = 4u;
constexpr uint8_t kFlagBadIndex = 8u;
constexpr int kMaxIter = 1 << 16;

// G4HepEmConstants.hh:7-29
constexpr double kPi = 3.1415926535897931e+00;
constexpr double k2Pi = 2.0 * kPi;
constexpr double kMec2 = 5.1099890999999997e-01;
constexpr double kInvMec2 = 1.0 / kMec2;
constexpr double kAlpha = 7.2973525653052150e-03;
constexpr double kPir02 = 2.4946724123674787e-23;
constexpr double kMigdal = 5.2804955733859579e-30;
constexpr double kLPM = 7.6843819381368661e+05;
constexpr double kLarge = 1.0E+20;

// Diagnostics build only (-DHEPEM_TRACE): intermediate values of one track
// (id g_traceId) of the FP64 physics (row 0) and of the precision form (row 1).
#ifdef HEPEM_TRACE
static __device__ int g_traceId = -1;
static __device__ double g_trace[2][64];
#define HEPEM_TR(row, slot, v)                               \
  do {                                                       \
    if (rng.id == g_traceId) g_trace[row][slot] = (double)(v); \
  } while (0)
#else
#define HEPEM_TR(row, slot, v) ((void)0)
#endif

template <class T>
__device__ __forceinline__ T ld(const T* p) { return __ldg(p); }
__device__ __forceinline__ double dmax_(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin_(double a, double b) { return a < b ? a : b; }

// LPM functions G(s), Phi(s) on s in [0,2], ds = 0.05 (G4HepEmInteractionUtils.hh:20-36)
__device__ __constant__ const double kFuncLPM[84] = {
    0.0000E+00, 0.0000E+00, 6.9163E-02, 2.5747E-01, 2.0597E-01, 4.4573E-01, 3.5098E-01, 5.8373E-01,
    4.8095E-01, 6.8530E-01, 5.8926E-01, 7.6040E-01, 6.7626E-01, 8.1626E-01, 7.4479E-01, 8.5805E-01,
    7.9826E-01, 8.8952E-01, 8.4003E-01, 9.1338E-01, 8.7258E-01, 9.3159E-01, 8.9794E-01, 9.4558E-01,
    9.1776E-01, 9.5640E-01, 9.3332E-01, 9.6483E-01, 9.4560E-01, 9.7143E-01, 9.5535E-01, 9.7664E-01,
    9.6313E-01, 9.8078E-01, 9.6939E-01, 9.8408E-01, 9.7444E-01, 9.8673E-01, 9.7855E-01, 9.8888E-01,
    9.8191E-01, 9.9062E-01, 9.8467E-01, 9.9204E-01, 9.8695E-01, 9.9321E-01, 9.8884E-01, 9.9417E-01,
    9.9042E-01, 9.9497E-01, 9.9174E-01, 9.9564E-01, 9.9285E-01, 9.9619E-01, 9.9379E-01, 9.9666E-01,
    9.9458E-01, 9.9706E-01, 9.9526E-01, 9.9739E-01, 9.9583E-01, 9.9768E-01, 9.9632E-01, 9.9794E-01,
    9.9674E-01, 9.9818E-01, 9.9710E-01, 9.9839E-01, 9.9741E-01, 9.9857E-01, 9.9767E-01, 9.9873E-01,
    9.9790E-01, 9.9887E-01, 9.9809E-01, 9.9898E-01, 9.9826E-01, 9.9909E-01, 9.9840E-01, 9.9918E-01,
    9.9856E-01, 9.9926E-01, 0.0, 0.0};

// ---- interpolation (G4HepEmRunUtils.icc:49-237) ---------------------------------
__device__ __forceinline__ double spline(double x1, double x2, double y1, double y2, double s1, double s2, double x) {
  const double dl = x2 - x1;
  const double b = dmax_(0., dmin_(1., (x - x1) / dl));
  const double os = 0.166666666667;
  const double c0 = (2.0 - b) * s1;
  const double c1 = (1.0 + b) * s2;
  return y1 + b * (y2 - y1) + (b * (b - 1.0)) * (c0 + c1) * (dl * dl * os);
}
// (int)max(0, min(v, hi)) for an integer hi >= 0, as the FP64 min/max and the
// truncation give it (NaN: hi), in integer operations on the bits of v
__device__ __forceinline__ int clamp_trunc(double v, int hi) {
  const long long b = __double_as_longlong(v);
  if (b <= 0) return 0;  // +0, -0 and negative values
  const int e = (int)(b >> 52) - 1023;
  if (e < 0) return 0;
  if (e >= 31) return hi;  // also inf and NaN
  const int t = (int)(((b & 0xFFFFFFFFFFFFFLL) | (1LL << 52)) >> (52 - e));
  return t < hi ? t : hi;
}
__device__ __forceinline__ int bin_of(double lx, double lxm, double ild, int nd) {
  return clamp_trunc((lx - lxm) * ild, nd - 2);
}
__device__ __forceinline__ double spline_log_xy(int nd, const double* xd, const double* yd, double x, double lx,
                                                double lxm, double ild) {
  const double xv = dmax_(ld(xd), dmin_(ld(xd + nd - 1), x));
  const int i = bin_of(lx, lxm, ild, nd);
  // (y_i, y''_i) pairs are adjacent but only 8-byte aligned (5*N doubles per couple)
  return spline(ld(xd + i), ld(xd + i + 1), ld(yd + 2 * i), ld(yd + 2 * i + 2), ld(yd + 2 * i + 1),
                ld(yd + 2 * i + 3), xv);
}
__device__ __forceinline__ double spline_log_3(int nd, const double* d, double x, double lx, double lxm, double ild) {
  const double xv = dmax_(ld(d), dmin_(ld(d + 3 * (nd - 1)), x));
  const int i = 3 * bin_of(lx, lxm, ild, nd);
  return spline(ld(d + i), ld(d + i + 3), ld(d + i + 1), ld(d + i + 4), ld(d + i + 2), ld(d + i + 5), xv);
}
__device__ __forceinline__ double spline_log_9(int nd, const double* d, double x, double lx, double lxm, double ild,
                                               int iwhich) {
  const int i0 = 9 * bin_of(lx, lxm, ild, nd);
  const int i1 = i0 + 9;
  const int w = (iwhich - 1) * 2 + 1;
  return spline(ld(d + i0), ld(d + i1), ld(d + i0 + w), ld(d + i1 + w), ld(d + i0 + w + 1), ld(d + i1 + w + 1), x);
}
__device__ __forceinline__ int lower_bin(const double* xd, int num, double x, int step) {
  int ml = -1, mu = num - 1;
  while (abs(mu - ml) > 1) {
    const int mav = (ml + mu) / 2;  // (int)(0.5 * (ml + mu)): both truncate toward 0
    if (x < ld(xd + step * mav)) mu = mav; else ml = mav;
  }
  return mu - 1;
}
__device__ __forceinline__ void rotate(double* d, const double* r) {
  double up = r[0] * r[0] + r[1] * r[1];
  if (up > 0.) {
    up = sqrt(up);
    const double px = d[0], py = d[1], pz = d[2];
    d[0] = (r[0] * r[2] * px - r[1] * py) / up + r[0] * pz;
    d[1] = (r[1] * r[2] * px + r[0] * py) / up + r[1] * pz;
    d[2] = -up * px + r[2] * pz;
  } else if (r[2] < 0.) {
    d[0] = -d[0];
    d[2] = -d[2];
  }
}

// ---- electron table accessors (G4HepEmElectronManager.icc:486-599) ---------------
__device__ __forceinline__ double rest_range(const DevElData& d, int imc, double e, double le) {
  const int n = d.nLoss;
  return dmax_(0.0, spline_log_xy(n, d.lossGrid, d.loss + 5 * n * imc, e, le, d.lossLogMin, d.lossILD));
}
__device__ __forceinline__ double rest_dedx(const DevElData& d, int imc, double e, double le) {
  const int n = d.nLoss;
  return dmax_(0.0, spline_log_xy(n, d.lossGrid, d.loss + n * (5 * imc + 2), e, le, d.lossLogMin, d.lossILD));
}
__device__ __forceinline__ double inv_range(const DevElData& d, int imc, double r) {
  const int n = d.nLoss;
  const double* R = d.loss + 5 * n * imc;
  const double rmin = ld(R);
  if (r < rmin) {
    const double q = r / rmin;
    return dmax_(0.0, ld(d.lossGrid) * q * q);
  }
  const int i = lower_bin(R, n, r, 2);
  const double* S2 = R + 4 * n;
  return dmax_(0.0, spline(ld(R + 2 * i), ld(R + 2 * (i + 1)), ld(d.lossGrid + i), ld(d.lossGrid + i + 1), ld(S2 + i),
                           ld(S2 + i + 1), r));
}
__device__ __forceinline__ double rest_macxs(const DevElData& d, int imc, double e, double le, bool ioni) {
  const int i0 = ld(d.xsStart + imc);
  const int st = ioni ? i0 : i0 + 3 * double_to_int_rz_exact(ld(d.xs + i0)) + 5;
  const int nd = double_to_int_rz_exact(ld(d.xs + st));
  if (e < ld(d.xs + st + 5)) return 0.0;
  return dmax_(0.0, spline_log_3(nd, d.xs + st + 5, e, le, ld(d.xs + st + 3), ld(d.xs + st + 4)));
}
__device__ __forceinline__ double nuc_macxs(const DevElData& d, int imat, double e, double le) {
  if (e < ld(d.nucGrid)) return 0.0;
  const int n = d.nNuc;
  return dmax_(0.0, spline_log_xy(n, d.nucGrid, d.nuc + imat * 2 * n, e, le, d.nucLogMin, d.nucILD));
}
__device__ __forceinline__ double rest_macxs_stepping(const DevElData& d, int imc, double e, double le, bool ioni) {
  const double log08 = -0.22314355131420971;
  const int i0 = ld(d.xsStart + imc);
  const int st = ioni ? i0 : i0 + 3 * double_to_int_rz_exact(ld(d.xs + i0)) + 5;
  const int nd = double_to_int_rz_exact(ld(d.xs + st));
  const double minE = ld(d.xs + st + 5), maxE = ld(d.xs + st + 1), maxV = ld(d.xs + st + 2);
  if (e > maxE) {
    const double er = 0.8 * e;
    if (er < maxE) return dmax_(0.0, maxV);
    e = er;
    le += log08;
  }
  if (e < minE) return 0.0;
  return dmax_(0.0, spline_log_3(nd, d.xs + st + 5, e, le, ld(d.xs + st + 3), ld(d.xs + st + 4)));
}
__device__ __forceinline__ double transport_mfp(const DevElData& d, int imat, double e, double le) {
  const int n = d.nLoss;
  const double v = dmax_(0.0, spline_log_xy(n, d.lossGrid, d.tr1 + 2 * n * imat, e, le, d.lossLogMin, d.lossILD));
  return v > 0. ? 1. / v : kLarge;
}
__device__ __forceinline__ double annih_macxs(double e, double ne) {
  const double tau = e * kInvMec2;
  const double gam = tau + 1.0;
  const double gam2 = gam * gam;
  const double bg2 = tau * (tau + 2.0);
  const double bg = sqrt(bg2);
  return ne * kPir02 * ((gam2 + 4. * gam + 1.) * vdt_log(gam + bg) - (gam + 3.) * bg) / (bg2 * (gam + 1.));
}

// ---- per-track register state -------------------------------------------------------
struct Msc {
  double lambtr1, trueStep, zPath, disp[3], dir[3], initRange, dynFactor, tlimitMin, par1, par2, par3;
  bool noScatter, displace, firstStep, active;
};

struct Sec {
  int8_t type;
  double e, dir[3];
};

struct Track {
  double e, le, dir[3], nia[4], mfp[4], safety, edep, gstep, pstep, range, preE, preLE, peXS;
  int imc, winner;
  bool isEl, onBoundary;
  uint8_t flags;
  Msc msc;
  int nsec;
  Sec sec[2];
  __device__ __forceinline__ void setE(double v) { e = v; le = 100.0; }
  __device__ __forceinline__ double logE() {
    if (le > 99.0) le = (e > 0.) ? vdt_log(e) : -30;
    return le;
  }
  __device__ __forceinline__ Sec& addSec(int8_t type) {
    Sec& s = sec[nsec < 2 ? nsec : 1];
    ++nsec;
    s.type = type;
    return s;
  }
};

struct Physics {
  const DevTables& T;
  Rng& rng;
  Track& t;

  __device__ __forceinline__ const DevElData& eld() const { return t.isEl ? T.el[0] : T.el[1]; }
  __device__ __forceinline__ const DevCouple& couple() const { return T.couples[t.imc]; }
  __device__ __forceinline__ const DevRegion& region() const { return T.regions[T.couples[t.imc].region]; }

  // ================= e+- HowFar (G4HepEmElectronManager.icc:35-169) ================
  __device__ void el_howfar() {
#pragma unroll
    for (int ip = 0; ip < 4; ++ip)
      if (t.nia[ip] <= 0.) t.nia[ip] = -vdt_log(rng.flat());
    const DevElData& d = eld();
    const double e = t.e, le = t.logE();
    const int imc = t.imc;
    const DevCouple c = couple();
    const DevRegion& reg = T.regions[c.region];
    const double range = rest_range(d, imc, e, le);
    t.range = range;
    const double frange = ld(&reg.finalRange), drange = ld(&reg.dRoverRange);
    double pstep = range > frange ? range * drange + frange * (1.0 - drange) * (2.0 - frange / range) : range;
    HEPEM_TR(0, 0, range);
    HEPEM_TR(0, 1, pstep);
    int winner = -1;
    double mx[4];
    mx[0] = rest_macxs_stepping(d, imc, e, le, true);
    mx[1] = rest_macxs_stepping(d, imc, e, le, false);
    mx[2] = t.isEl ? 0.0 : annih_macxs(0.8 * e, ld(&T.mats[c.mat].elDensity));
    mx[3] = nuc_macxs(d, c.mat, e, le);
#pragma unroll
    for (int ip = 0; ip < 4; ++ip) {
      const double mfp = mx[ip] > 0. ? 1. / mx[ip] : kLarge;
      t.mfp[ip] = mfp;
      const double lim = mfp * t.nia[ip];
      if (lim < pstep) { pstep = lim; winner = ip; }
    }
    t.pstep = pstep;
    t.winner = winner;
    t.gstep = pstep;
    HEPEM_TR(0, 2, mx[0]);
    HEPEM_TR(0, 3, mx[1]);
    HEPEM_TR(0, 6, pstep);
    HEPEM_TR(0, 7, winner);
    Msc& m = t.msc;
    m.trueStep = pstep;
    m.zPath = pstep;
    m.active = false;
    m.disp[0] = m.disp[1] = m.disp[2] = 0.;
    m.dir[0] = 0.; m.dir[1] = 0.; m.dir[2] = 1.;
    if (pstep > 5.E-8 && e > 1.0E-3) {
      m.active = true;
      m.lambtr1 = transport_mfp(d, c.mat, e, le);
      msc_step_limit(e, c.mat, range, reg);
      HEPEM_TR(0, 8, m.lambtr1);
      HEPEM_TR(0, 10, m.trueStep);
      true_to_geom(e, range, c.mat);
      HEPEM_TR(0, 11, m.zPath);
      if (m.trueStep < pstep) {
        t.winner = -2;
        pstep = m.trueStep;
        t.pstep = pstep;
      }
      t.gstep = dmin_(m.zPath, pstep);
    }
  }

  // G4HepEmElectronInteractionUMSC.icc:19-126
  __device__ void msc_step_limit(double e, int imat, double range, const DevRegion& reg) {
    Msc& m = t.msc;
    const DevMat& md = T.mats[imat];
    m.noScatter = false;
    m.displace = true;
    const double kTLimitMinfix = 1.0E-8;
    if (m.trueStep < kTLimitMinfix || range * ld(&md.umscPar) < t.safety) {
      m.displace = false;
      return;
    }
    const double rf = ld(&reg.mscRangeFactor), sf = ld(&reg.mscSafetyFactor);
    double tlimit = 0.0;
    if (!ld(&reg.mscMinimal)) {
      if (m.firstStep || t.onBoundary) {
        const double l1 = m.lambtr1;
        m.initRange = dmax_(range, l1);
        m.dynFactor = l1 > 1.0 ? rf * (0.75 + 0.25 * l1) : rf;
        const double stepMin = l1 * 1.0E-3 / (2.0E-3 + e * (ld(&md.stepMin[0]) + e * ld(&md.stepMin[1])));
        const double d0 = t.isEl ? 0.87 * ld(&md.zeff23) : 0.70 * ld(&md.zeffSqrt);
        const double d1 = e > 5.0E-3 ? d0 * stepMin : d0 * stepMin * 0.5 * (1.0 + e * 200.0);
        m.tlimitMin = dmax_(d1, kTLimitMinfix);
        m.firstStep = false;
      }
      const double tlm = m.tlimitMin;
      tlimit = range > t.safety ? dmax_(dmax_(m.initRange * m.dynFactor, sf * t.safety), tlm) : dmax_(range, tlm);
    } else {
      if (t.onBoundary) {
        const double l1 = m.lambtr1;
        const double tmp = range > l1 ? rf * range : rf * l1;
        m.initRange = dmax_(tmp, 10 * kTLimitMinfix);
      }
      tlimit = m.initRange;
    }
    const double tlm = m.tlimitMin;
    HEPEM_TR(0, 24, tlimit);
    if (tlimit < m.trueStep) {
      const double d0 = tlimit > tlm ? dmax_(rng.gauss(tlimit, 0.1 * (tlimit - tlm)), tlm) : tlm;
      HEPEM_TR(0, 25, d0);
      m.trueStep = dmin_(d0, m.trueStep);
    }
  }

  // G4HepEmElectronManager.icc:602-650
  __device__ void true_to_geom(double e, double range, int imat) {
    Msc& m = t.msc;
    m.par1 = -1.; m.par2 = 0.; m.par3 = 0.;
    m.trueStep = dmin_(m.trueStep, range);
    m.zPath = m.trueStep;
    if (m.trueStep < 1.0E-6) return;
    const double tau = m.trueStep / m.lambtr1;
    if (tau < 1.0e-16) {
      m.zPath = dmin_(m.trueStep, m.lambtr1);
    } else if (m.trueStep < range * 0.05) {
      m.zPath = tau < 1.0e-6 ? m.trueStep * (1. - 0.5 * tau) : m.lambtr1 * (1. - vdt_exp(-tau));
    } else if (e < kMec2 || m.trueStep == range) {
      m.par1 = 1. / range;
      m.par2 = 1. / (m.par1 * m.lambtr1);
      m.par3 = 1. + m.par2;
      m.zPath = 1. / (m.par1 * m.par3);
      if (m.trueStep < range) m.zPath *= (1. - vdt_pow(1. - m.trueStep / range, m.par3));
    } else {
      const double rfin = dmax_(range - m.trueStep, 0.01 * range);
      const DevElData& d = eld();
      const double t1 = inv_range(d, t.imc, rfin);
      const double l1 = transport_mfp(d, imat, t1, vdt_log(t1));
      m.par1 = (m.lambtr1 - l1) / (m.lambtr1 * m.trueStep);
      m.par2 = 1. / (m.par1 * m.lambtr1);
      m.par3 = 1. + m.par2;
      m.zPath = (1. - vdt_pow(l1 / m.lambtr1, m.par3)) / (m.par1 * m.par3);
    }
    m.zPath = dmin_(m.zPath, m.lambtr1);
  }

  // G4HepEmElectronManager.icc:653-691
  __device__ void geom_to_true(double range, double g) {
    Msc& m = t.msc;
    m.zPath = g;
    if (g < 1.0E-6) {
      m.trueStep = g;
      return;
    }
    double tl = g;
    if (g > m.lambtr1 * 1.0e-16) {
      if (m.par1 < 0.) {
        tl = -m.lambtr1 * vdt_log(1. - g / m.lambtr1);
      } else {
        const double dum = m.par1 * m.par3 * g;
        tl = dum < 1. ? (1. - vdt_pow(1. - dum, 1. / m.par3)) / m.par1 : range;
      }
      if (tl < g) tl = g;
    }
    m.trueStep = tl;
  }

  // ================= e+- Perform (G4HepEmElectronManager.icc:171-483) ================
  // returns: 0 nothing more, 1 discrete interaction pending in t.winner
  __device__ void el_perform() {
    t.edep = 0;
    t.pstep = t.gstep;
    if (t.gstep <= 0.) return;
    if (el_continuous()) {
      if (!t.isEl) annihilate_at_rest();
      return;
    }
    el_discrete();
  }

  __device__ bool el_continuous() {
    t.preE = t.e;
    t.preLE = t.logE();
    {
      const double g = t.gstep;
      double p = g;
      Msc& m = t.msc;
      if (m.active) {
        p = m.trueStep;
        if (g < m.zPath) {
          geom_to_true(t.range, g);
          p = dmin_(p, m.trueStep);
          m.trueStep = p;
        }
        if (p <= 5.E-8 || t.range <= p) m.active = false;
      }
      t.pstep = p;
    }
    const double pstep = t.pstep;
    if (pstep <= 0.0) return false;
#pragma unroll
    for (int i = 0; i < 4; ++i) t.nia[i] -= pstep / t.mfp[i];
    if (mean_loss()) return true;
    sample_msc();
    return loss_fluct();
  }

  __device__ bool mean_loss() {
    const double pstep = t.pstep, e = t.e, range = t.range;
    if (pstep >= range || e <= T.minLossE) {
      t.edep = e;
      t.setE(0.0);
      return true;
    }
    const DevElData& d = eld();
    const double le = t.logE();
    double eloss = pstep * rest_dedx(d, t.imc, e, le);
    if (eloss > e * ld(&region().linELossLimit)) {
      const double post = range - pstep;
      eloss = e - inv_range(d, t.imc, post);
    }
    eloss = dmax_(eloss, 0.0);
    HEPEM_TR(0, 14, eloss);
    if (eloss >= e) {
      eloss = e;
      t.setE(0);
      t.edep = eloss;
      return true;
    }
    t.setE(e - eloss);
    t.edep = eloss;
    return false;
  }

  __device__ void sample_msc() {
    const double pstep = t.pstep, preE = t.preE, range = t.range;
    Msc& m = t.msc;
    if (m.active && pstep > dmax_(1.0E-8, 1.0e-16 * m.lambtr1)) {
      double postE = preE;
      double postLE = t.preLE;
      if (pstep > range * 0.01) {
        postE = t.e;
        postLE = t.logE();
      }
      const int imat = couple().mat;
      const double postMFP = transport_mfp(eld(), imat, postE, postLE);
      msc_scatter(pstep, preE, m.lambtr1, postE, postMFP, imat);
      if (!m.noScatter) {
        rotate(m.dir, t.dir);
        if (m.displace) rotate(m.disp, t.dir);
        t.dir[0] = m.dir[0]; t.dir[1] = m.dir[1]; t.dir[2] = m.dir[2];
      }
    }
  }

  // G4HepEmElectronInteractionUMSC.icc:129-150, 342-357
  __device__ void msc_scatter(double pstep, double preE, double preMFP, double postE, double postMFP, int imat) {
    Msc& m = t.msc;
    const double cost = msc_cos_theta(pstep, preE, preMFP, postE, postMFP, m.tlimitMin, imat);
    HEPEM_TR(0, 21, cost);
    if (fabs(cost) >= 1.0) {
      m.noScatter = true;
      return;
    }
    const double sth = sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = k2Pi * rng.flat();
    double sp, cp;
    sincos(phi, &sp, &cp);
    m.dir[0] = sth * cp;
    m.dir[1] = sth * sp;
    m.dir[2] = cost;
    m.displace = m.displace && T.mscDisplacement;
    if (m.displace && pstep > m.zPath) {
      const double r = 0.73 * sqrt((pstep - m.zPath) * (pstep + m.zPath));
      HEPEM_TR(0, 22, r);
      HEPEM_TR(0, 23, pstep - m.zPath);
      const double cbeta = 2.16;
      const double cbeta1 = 1. - vdt_exp(-cbeta * kPi);
      const double r0 = rng.flat(), r1 = rng.flat();
      const double psi = -vdt_log(1. - r0 * cbeta1) / cbeta;
      const double ph = r1 < 0.5 ? phi + psi : phi - psi;
      double s2, c2;
      sincos(ph, &s2, &c2);
      m.disp[0] = r * c2;
      m.disp[1] = r * s2;
      m.disp[2] = 0.0;
    }
  }

  // G4HepEmElectronInteractionUMSC.icc:153-270
  __device__ double msc_cos_theta(double pstep, double preE, double preMFP, double postE, double postMFP,
                                  double tlimMin, int imat) {
    const DevMat& md = T.mats[imat];
    const double iPre = 1.0 / preMFP;
    const double dR = preMFP - postMFP;
    const double tau = fabs(dR) > 0.01 * preMFP ? pstep * vdt_log(preMFP / postMFP) / dR : pstep * iPre;
    if (tau > 8.0) return 2.0 * rng.flat() - 1.0;
    if (tau < 1.0E-16) return 1.0;
    double xm, x2m;
    if (tau < 0.01) {
      xm = 1.0 - tau * (1.0 - 0.5 * tau);
      x2m = 1.0 - tau * (5.0 - 6.25 * tau) * 0.333333;
    } else {
      xm = vdt_exp(-tau);
      x2m = (1.0 + 2.0 * vdt_exp(-2.5 * tau)) * 0.333333;
    }
    if (postE < 0.5 * preE) return simple_scatter(xm, x2m);
    const double radLen = ld(&md.radLength);
    const double tsmall = dmin_(tlimMin, 1.0);
    const bool notSmall = pstep > tsmall;
    const double theta0 = notSmall ? theta0_of(pstep / radLen, postE, preE, imat)
                                   : theta0_of(tsmall / radLen, postE, preE, imat) * sqrt(pstep / tsmall);
    if (theta0 > kPi * 0.166666) return simple_scatter(xm, x2m);
    const double th2 = theta0 * theta0;
    if (th2 < 1.0E-16) return 1.0;
    const double dumtau = notSmall ? tau : tsmall * iPre;
    const double u = vdt_pow(dumtau, 0.1666666);
    const double dumxsi = ld(&md.tail[0]) + u * (ld(&md.tail[1]) + u * ld(&md.tail[2])) +
                          ld(&md.tail[3]) * vdt_log(pstep / (tau * radLen));
    const double xsi = dmax_(dumxsi, 1.9);
    const double c = fabs(xsi - 3.) < 0.001 ? 3.001 : fabs(xsi - 2.) < 0.001 ? 2.001 : xsi;
    const double c1 = c - 1.;
    const double ea = vdt_exp(-xsi);
    const double eaa = 1. / (1. - ea);
    double thex = th2 * (1.0 - th2 * 0.0833333);
    if (th2 > 0.01) {
      const double q = 2.0 * sin(0.5 * theta0);
      thex = q * q;
    }
    const double xmean1 = 1. - (1. - (1. + xsi) * ea) * thex * eaa;
    if (xmean1 <= 0.999 * xm) return simple_scatter(xm, x2m);
    const double x0 = 1. - xsi * thex;
    const double bx = c * thex;
    const double b = bx + x0;
    const double b1 = b + 1.;
    const double eb1 = vdt_pow(b1, c1);
    const double ebx = vdt_pow(bx, c1);
    const double dd = ebx / eb1;
    const double xmean2 = (x0 + dd - (bx - b1 * dd) / (c - 2.)) / (1. - dd);
    const double f1x0 = ea * eaa;
    const double f2x0 = c1 / (c * (1. - dd));
    const double prob = f2x0 / (f1x0 + f2x0);
    const double qprb = xm / (prob * xmean1 + (1. - prob) * xmean2);
    const double r0 = rng.flat(), r1 = rng.flat(), r2 = rng.flat();
    if (r0 < qprb) {
      if (r1 < prob) return 1. + vdt_log(ea + r2 / eaa) * thex;
      const double var0 = (1.0 - dd) * r2;
      if (var0 < 0.01 * dd) {
        const double var = var0 / (dd * c1);
        return -1.0 + var * (1.0 - var * 0.5 * c) * b1;
      }
      return 1.0 + thex * (c - xsi - c * vdt_pow(var0 + dd, -1. / c1));
    }
    return 2.0 * r1 - 1.0;
  }

  __device__ double simple_scatter(double xm, double x2m) {
    const double d0 = 3. * x2m - 1;
    const double d1 = 2. * xm - d0;
    const double a = 1. + 4. * d0 / d1;
    const double prob = (2. + a) * xm / a;
    const double r0 = rng.flat(), r1 = rng.flat();
    return r0 < prob ? -1. + 2. * vdt_pow(r1, 1. / (1. + a)) : -1. + 2. * r1;
  }

  // G4HepEmElectronInteractionUMSC.icc:291-339
  __device__ double theta0_of(double srl, double postE, double preE, int imat) {
    const DevMat& md = T.mats[imat];
    const double postInv = (postE + kMec2) / (postE * (postE + 2. * kMec2));
    const double inv = preE != postE ? sqrt(postInv * (preE + kMec2) / (preE * (preE + 2. * kMec2))) : postInv;
    const double y = (t.isEl || !T.mscPosCor) ? srl : srl * pos_correction(preE * postE, ld(&md.zeff));
    return 13.6 * sqrt(y) * inv * (ld(&md.theta[0]) + ld(&md.theta[1]) * vdt_log(y));
  }

  __device__ static double pos_correction(double eekin, double zeff) {
    const double ff = 1. + zeff * (1.84035E-4 * zeff - 1.86427E-2) + 0.41125;
    const double a = 0.994 - 4.08E-3 * zeff;
    const double b = 7.16 + (52.6 + 365. / zeff) / zeff;
    const double tu = sqrt(eekin) * kInvMec2;
    const double x = sqrt(tu * (tu + 2.) / ((tu + 1.) * (tu + 1.)));
    if (x < 0.6) return ff * a * (1. - vdt_exp(-b * x));
    const double c = 1.00 - 4.47E-3 * zeff;
    const double d = 1.21E-3 * zeff;
    if (x > 0.9) return ff * (c + d * vdt_exp(113.0 * (x - 1.)));
    const double yl = a * (1. - vdt_exp(-b * 0.6));
    const double yh = c + d * vdt_exp(113.0 * (0.9 - 1.));
    const double y0 = (yh - yl) / (0.9 - 0.6);
    const double y1 = yl - y0 * 0.6;
    return ff * (y0 * x + y1);
  }

  // G4HepEmElectronManager.icc:324-368, G4HepEmElectronEnergyLossFluctuation.icc:11-111
  __device__ bool loss_fluct() {
    const double pstep = t.pstep, preE = t.preE;
    double finalE = t.e;
    double eloss = t.edep;
    const DevCouple c = couple();
    if (ld(&T.regions[c.region].eLossFluct) && eloss > 1.E-5) {
      const double tmax = t.isEl ? 0.5 * preE : preE;
      const double tcut = dmin_(c.elCut, tmax);
      eloss = fluct(tcut, ld(&T.mats[c.mat].meanExc), eloss);
      eloss = dmax_(eloss, 0.0);
      finalE = preE - eloss;
      HEPEM_TR(0, 15, eloss);
    }
    (void)pstep;
    if (finalE <= T.elTrackingCut) {
      eloss = preE;
      finalE = 0.0;
      t.setE(finalE);
      t.edep = eloss;
      return true;
    }
    t.setE(finalE);
    t.edep = eloss;
    return false;
  }

  __device__ double fluct(double tcut, double excE, double meanE) {
    const double scaling = dmin_(1. + 5.E-4 / tcut, 1.5);
    const double meanLoss = meanE / scaling;
    const double rate = 0.56, e0 = 1.E-5, nmax = 8.;
    const double w1 = tcut / e0;
    double a3 = meanLoss * (tcut - e0) / (e0 * tcut * vdt_log(w1));
    double a1 = 0.;
    double e1 = excE;
    double eloss = 0.0;
    HEPEM_TR(0, 18, a3);
    if (tcut > excE) {
      const double a1t = meanLoss * (1. - rate) / excE;
      const double d0 = a1t < 42. ? .1 + (4. - .1) * sqrt(a1t / 42.) : 4.;
      a1 = a1t / d0;
      e1 *= d0;
      a3 *= rate;
      if (a1 > nmax) {
        const double em = a1 * e1;
        eloss = gauss_loss(em, em * e1);
      } else {
        const int p = poisson_capped(a1);
        HEPEM_TR(0, 17, p);
        eloss = p > 0 ? ((p + 1) - 2. * rng.flat()) * e1 : 0.;
      }
    }
    if (a3 > 0.) {
      double p3 = a3;
      double alfa = 1.;
      if (a3 > nmax) {
        alfa = w1 * (nmax + a3) / (w1 * nmax + a3);
        const double alfa1 = alfa * vdt_log(alfa) / (alfa - 1.);
        const double nam = a3 * w1 * (alfa - 1.) / ((w1 - 1.) * alfa);
        const double em = nam * e0 * alfa1;
        const double s2 = e0 * e0 * nam * (alfa - alfa1 * alfa1);
        eloss += gauss_loss(em, s2);
        p3 = a3 - nam;
      }
      const double w3 = alfa * e0;
      if (tcut > w3) {
        const double w = (tcut - w3) / tcut;
        int nnb = poisson_capped(p3);
        HEPEM_TR(0, 19, p3);
        HEPEM_TR(0, 20, nnb);
        if (nnb > kMaxIter) { nnb = kMaxIter; t.flags |= kFlagLoopCap; }
        for (int k = 0; k < nnb; ++k) eloss += w3 / (1. - w * rng.flat());
      }
    }
    return eloss * scaling;
  }

  // Poisson of G4HepEmRandomEngine.hh:74-97 with a bounded inversion loop
  __device__ int poisson_capped(double mean) {
    int number = 0;
    if (mean <= 16) {
      const double position = rng.flat();
      double pv = vdt_exp(-mean);
      double ps = pv;
      while (ps <= position) {
        ++number;
        pv *= mean / number;
        ps += pv;
        if (number >= 4096) { t.flags |= kFlagLoopCap; break; }
      }
      return number;
    }
    const double a = rng.flat(), b = rng.flat();
    double sb, cb;
    sincos(k2Pi * b, &sb, &cb);
    const double tt = sqrt(-2. * vdt_log(a)) * cb;
    const double value = mean + tt * sqrt(mean) + 0.5;
    return value < 0. ? 0 : value >= 2.E+9 ? (int)2.E+9 : (int)value;
  }

  __device__ double gauss_loss(double me, double s2) {
    const double twom = 2. * me;
    if (me * me < 0.0625 * s2) return twom * rng.flat();
    const double sig = sqrt(s2);
    double el;
    int it = 0;
    do {
      el = rng.gauss(me, sig);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (el < 0. || el > twom);
    return el;
  }

  // Perform split at the discrete interaction: continuous part, the
  // delta-interaction test, and the choice of the interaction to sample
  // (G4HepEmElectronManager.icc:425-483).  Returns the queue of the pending
  // interaction, or -1.
  __device__ int el_perform_until_discrete() {
    t.edep = 0;
    t.pstep = t.gstep;
    if (t.gstep <= 0.) return -1;
    if (el_continuous()) return t.isEl ? -1 : kQAnnihRest;
    const int ip = t.winner;
    if (ip < 0 || t.onBoundary) return -1;
    t.nia[ip] = -1.0;
    const DevElData& d = eld();
    const DevCouple c = couple();
    const double e = t.e, le = t.logE();
    const double mx = ip < 2 ? rest_macxs(d, t.imc, e, le, ip == 0)
                     : (ip < 3 ? annih_macxs(e, ld(&T.mats[c.mat].elDensity)) : nuc_macxs(d, c.mat, e, le));
    const double u = rng.flat();
    if (mx <= 0.0 || u > mx * t.mfp[ip]) return -1;
    switch (ip) {
      case 0: return t.isEl ? kQIoniEm : kQIoniEp;
      case 1: return e < T.bremModelLim ? kQBremSB : kQBremRB;
      case 2: return kQAnnihFlight;
      default: return -1;
    }
  }

  // Gamma Perform up to the interaction (G4HepEmGammaManager.icc:54-81);
  // returns the queue of the pending interaction or -1 (the tracking cut of
  // :97-104 is then applied by the caller when no interaction is pending).
  __device__ int gamma_perform_until_interaction() {
    t.nia[0] -= t.gstep / t.mfp[0];
    t.edep = 0.0;
    if (t.onBoundary) return -1;
    const int ip = t.winner;
    if (ip >= 0 && ip < 4) t.nia[ip] = -1.0;
    switch (ip) {
      case 0: return kQConversion;
      case 1: return kQCompton;
      case 2: return kQPhotoelectric;
      default: return -2;  // no interaction, tracking cut still applies
    }
  }

  __device__ void gamma_tracking_cut() {
    const double fe = t.e;
    if (fe > 0.0 && fe <= T.gammaTrackingCut) {
      t.setE(0.0);
      t.edep += fe;
    }
  }

  // G4HepEmElectronManager.icc:408-459
  __device__ void el_discrete() {
    const int ip = t.winner;
    if (ip < 0 || t.onBoundary) return;
    t.nia[ip] = -1.0;
    const DevElData& d = eld();
    const DevCouple c = couple();
    const double e = t.e, le = t.logE();
    const double mx = ip < 2 ? rest_macxs(d, t.imc, e, le, ip == 0)
                     : (ip < 3 ? annih_macxs(e, ld(&T.mats[c.mat].elDensity)) : nuc_macxs(d, c.mat, e, le));
    const double u = rng.flat();
    if (mx <= 0.0 || u > mx * t.mfp[ip]) return;
    switch (ip) {
      case 0: ioni(); break;
      case 1: brem(e < T.bremModelLim); break;
      case 2: annihilate_in_flight(); break;
      default: break;
    }
  }

  // ================= Moller-Bhabha (G4HepEmElectronInteractionIoni.icc:19-138) =========
  __device__ void ioni() {
    const double E = t.e;
    const double cut = couple().elCut;
    const double tmaxE = t.isEl ? 0.5 * E : E;
    if (tmaxE <= cut) return;
    const double dE = t.isEl ? moller(cut, E) : bhabha(cut, E);
    Sec& s = t.addSec(0);
    const double eTot = E + kMec2;
    const double pTot = sqrt(E * (eTot + kMec2));
    const double dP = sqrt(dE * (dE + 2.0 * kMec2));
    const double cost = dE * (eTot + kMec2) / (dP * pTot);
    const double ct = dmax_(-1.0, dmin_(cost, 1.0));
    const double st = sqrt((1.0 - ct) * (1.0 + ct));
    const double phi = k2Pi * rng.flat();
    double sp, cp;
    sincos(phi, &sp, &cp);
    s.dir[0] = st * cp;
    s.dir[1] = st * sp;
    s.dir[2] = ct;
    rotate(s.dir, t.dir);
    t.dir[0] = pTot * t.dir[0] - dP * s.dir[0];
    t.dir[1] = pTot * t.dir[1] - dP * s.dir[1];
    t.dir[2] = pTot * t.dir[2] - dP * s.dir[2];
    const double nrm = 1.0 / sqrt(t.dir[0] * t.dir[0] + t.dir[1] * t.dir[1] + t.dir[2] * t.dir[2]);
    t.dir[0] *= nrm; t.dir[1] *= nrm; t.dir[2] *= nrm;
    t.setE(E - dE);
    s.e = dE;
  }

  __device__ double moller(double cut, double E) {
    const double xmin = cut / E;
    const double xmax = 0.5 * E / E;
    const double gam = E * kInvMec2 + 1.0;
    const double g2 = gam * gam;
    const double xmm = xmin * xmax;
    const double gg = (2.0 * gam - 1.0) / g2;
    const double y = 1. - xmax;
    const double gf = 1.0 - gg * xmax + xmax * xmax * (1.0 - gg + (1.0 - gg * y) / (y * y));
    double dum, r0, r1, x;
    int it = 0;
    do {
      r0 = rng.flat(); r1 = rng.flat();
      x = xmm / (xmin * (1.0 - r0) + xmax * r0);
      const double xx = 1.0 - x;
      dum = 1.0 - gg * x + x * x * (1.0 - gg + (1.0 - gg * xx) / (xx * xx));
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (gf * r1 > dum);
    return x * E;
  }

  __device__ double bhabha(double cut, double E) {
    const double xmin = cut / E;
    const double xmax = E / E;
    const double gam = E * kInvMec2 + 1.0;
    const double g2 = gam * gam;
    const double b2 = 1. - 1. / g2;
    const double xmm = xmin * xmax;
    const double y = 1.0 / (1.0 + gam);
    const double y2 = y * y;
    const double y12 = 1.0 - 2.0 * y;
    const double c1 = 2.0 - y2;
    const double c2 = y12 * (3.0 + y2);
    const double y122 = y12 * y12;
    const double c4 = y122 * y12;
    const double c3 = c4 + y122;
    const double xmax2 = xmax * xmax;
    const double gf = 1.0 + (xmax2 * c4 - xmin * xmin * xmin * c3 + xmax2 * c2 - xmin * c1) * b2;
    double dum, r0, r1, x;
    int it = 0;
    do {
      r0 = rng.flat(); r1 = rng.flat();
      x = xmm / (xmin * (1.0 - r0) + xmax * r0);
      const double xx = x * x;
      dum = 1.0 + (xx * xx * c4 - x * xx * c3 + xx * c2 - x * c1) * b2;
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (gf * r1 > dum);
    return x * E;
  }

  // ================= bremsstrahlung (G4HepEmElectronInteractionBrem.icc:35-344) =========
  __device__ void brem(bool sbModel) {
    const double E = t.e;
    const double le = t.logE();
    if (E <= couple().gamCut) return;
    const double k = sbModel ? sample_sb(E, le) : sample_rb(E, le);
    Sec& s = t.addSec(2);
    const double cost = tsai_cost(E);
    const double sint = sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = k2Pi * rng.flat();
    double sp, cp;
    sincos(phi, &sp, &cp);
    s.dir[0] = sint * cp;
    s.dir[1] = sint * sp;
    s.dir[2] = cost;
    rotate(s.dir, t.dir);
    const double eTot = E + kMec2;
    const double pTot = sqrt(E * (eTot + kMec2));
    t.dir[0] = pTot * t.dir[0] - k * s.dir[0];
    t.dir[1] = pTot * t.dir[1] - k * s.dir[1];
    t.dir[2] = pTot * t.dir[2] - k * s.dir[2];
    const double nrm = 1.0 / sqrt(t.dir[0] * t.dir[0] + t.dir[1] * t.dir[1] + t.dir[2] * t.dir[2]);
    t.dir[0] *= nrm; t.dir[1] *= nrm; t.dir[2] *= nrm;
    t.setE(E - k);
    s.e = k;
  }

  __device__ int select_brem_target(double E, double le, double u, int which) {
    const DevElData& d = eld();
    const int st = ld(d.selStart[which] + t.imc);
    const double* D = d.sel[which] + st;
    const int nd = double_to_int_rz_exact(ld(D));
    const int ne = double_to_int_rz_exact(ld(D + 1));
    const double* x = D + 4;
    const double xv = dmax_(ld(x), dmin_(ld(x + ne * (nd - 1)), E));
    const int ie = clamp_trunc((le - ld(D + 2)) * ld(D + 3), nd - 2);
    int i0 = ie * ne, i1 = i0 + ne;
    const double x1 = ld(x + i0++), x2 = ld(x + i1++);
    const double b = dmax_(0., dmin_(1., (xv - x1) / (x2 - x1)));
    int k = 0;
    while (k < ne - 1 && u > ld(x + i0 + k) + b * (ld(x + i1 + k) - ld(x + i0 + k))) ++k;
    return k;
  }

  __device__ static int lin_search(const double* v, int size, double val) {
    int i = 0;
    const int s3 = 3 * size;
    while (i + 9 < s3) {
      if (ld(v + i) > val) return i;
      if (ld(v + i + 3) > val) return i + 3;
      if (ld(v + i + 6) > val) return i + 6;
      if (ld(v + i + 9) > val) return i + 9;
      i += 12;
    }
    while (i < s3) {
      if (ld(v + i) > val) break;
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
    const double dZ = int_to_double_exact(Z);
    const DevSB& sb = T.sb;
    const int st = ld(sb.startPerZ + Z);
    const int gci = ld(sb.gcIdx + ld(sb.gcStart + t.imc) + ei);
    bool corner = false, simple = false;
    int ie = double_to_int_rz_exact(ld(sb.data + st + 2));
    if (E < ld(sb.elE + ie)) {
      const double val = (le - sb.logMinE) * sb.ildE;
      ie = double_to_int_rz_exact(val);
      double pH = val - int_to_double_exact(ie);
      if (ie < 0 || ie > kNumElEnergySB - 2) { t.flags |= kFlagBadIndex; return E; }
      if (ld(sb.elE + ie) <= gcut) {
        pH = (le - lgcut) / (ld(sb.lelE + ie + 1) - lgcut);
        corner = true;
      }
      if (rng.flat() < pH) ++ie;
      else if (corner) simple = true;
    }
    const int minIE = double_to_int_rz_exact(ld(sb.data + st + 1));
    const int maxIE = double_to_int_rz_exact(ld(sb.data + st + 2));
    if (ie < minIE || ie > maxIE) { t.flags |= kFlagBadIndex; return E; }
    const int ncut = double_to_int_rz_exact(ld(sb.data + st + 3));
    const int size1 = ncut + 3 * kNumKappaSB;
    const int tst = st + 4 + (ie - minIE) * size1;
    const double minV = ld(sb.data + tst + gci);
    const double* Tb = sb.data + tst + ncut;
    const double lkt = (lgcut - le) / (lgcut - ld(sb.lelE + ie));
    const double pe = E + kMec2;
    const double dsc = ld(&md.densityCor) * pe * pe;
    double sup = 1.0, r0, r1, k = 0.0;
    int it = 0;
    do {
      r0 = rng.flat(); r1 = rng.flat();
      double kappa = 1.0;
      if (!simple) {
        const double cum = r0 * (1.0 - minV) + minV;
        int i3 = lin_search(Tb, kNumKappaSB, cum) - 3;
        if (i3 > 3 * (kNumKappaSB - 2)) { i3 = 3 * (kNumKappaSB - 2); t.flags |= kFlagBadIndex; }
        if (i3 < 0) { i3 = 0; t.flags |= kFlagBadIndex; }
        const int i = i3 / 3;
        const double cL = ld(Tb + i3), pA = ld(Tb + i3 + 1), pB = ld(Tb + i3 + 2), cH = ld(Tb + i3 + 3);
        const double lKL = ld(sb.lkappa + i), lKH = ld(sb.lkappa + i + 1);
        const double m1 = (cum - cL) / (cH - cL);
        const double m2 = (1.0 + pA + pB) * m1;
        const double m3 = 1.0 + m1 * (pA + pB * m1);
        const double lk = lKL + m2 / m3 * (lKH - lKL);
        kappa = vdt_exp(lk * lkt);
      } else {
        kappa = 1.0 - r0 * (1.0 - gcut / E);
      }
      k = kappa * E;
      const double ik = 1.0 / k;
      sup = 1.0 / (1.0 + dsc * ik * ik);
      if (!t.isEl) {
        const double e1 = E - gcut;
        const double ib1 = (e1 + kMec2) / sqrt(e1 * (e1 + 2.0 * kMec2));
        const double e2 = E - k;
        const double ib2 = (e2 + kMec2) / sqrt(e2 * (e2 + 2.0 * kMec2));
        const double dum = kAlpha * k2Pi * dZ * (ib1 - ib2);
        sup = dum > -12. ? sup * vdt_exp(dum) : 0.;
      }
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (r1 > sup);
    return k;
  }

  __device__ double sample_rb(double E, double le) {
    const DevCouple c = couple();
    const double gcut = c.gamCut;
    const DevMat& md = T.mats[c.mat];
    const int nElem = ld(&md.nElem);
    const int ei = nElem > 1 ? select_brem_target(E, le, rng.flat(), 2) : 0;
    const int Z = ld(T.matElemZ + ld(&md.elemOff) + ei);
    const double dZ = (double)Z;
    const DevElem& el = T.elems[Z < kMaxZ ? Z : kMaxZ];
    const double dens = kMigdal * ld(&md.elDensity);
    const double lpmE = kLPM * ld(&md.radLength);
    const double lpmLim = sqrt(dens) * lpmE;
    const double pte = E + kMec2;
    const double dcor = dens * pte * pte;
    const bool lpm = pte > lpmLim;
    const double zf1 = ld(&el.zFactor1);
    const double zf2 = (1. + 1. / dZ) / 12.;
    const double fmax = zf1 + zf2;
    const double xmin = vdt_log(gcut * gcut + dcor);
    const double xr = vdt_log(E * E + dcor) - xmin;
    double r0, r1, k, fv;
    int it = 0;
    do {
      r0 = rng.flat(); r1 = rng.flat();
      k = sqrt(dmax_(vdt_exp(xmin + r0 * xr) - dcor, 0.0));
      const double y = k / pte;
      const double omy = 1. - y;
      const double d0 = 0.25 * y * y;
      if (lpm) {
        double xiS, gS, phiS;
        lpm_functions(xiS, gS, phiS, k, pte, lpmE, ld(&el.Z23), ld(&el.ilVarS1), ld(&el.ilVarS1Cond), dcor, 1.0);
        const double t1 = xiS * (d0 * gS + (omy + 2.0 * d0) * phiS);
        fv = t1 * zf1 + omy * zf2;
      } else {
        const double d1 = omy + 3. * d0;
        if (Z < 5) {
          fv = d1 * zf1 + omy * zf2;
        } else {
          const double z13 = ld(&el.Z13);
          const double d2 = y / (pte - k);
          const double gam = d2 * 100. * kMec2 / z13;
          const double eps = gam / z13;
          const double g2 = gam * gam;
          const double phi1 = 16.863 - 2.0 * vdt_log(1.0 + 0.311877 * g2) + 2.4 * vdt_exp(-0.9 * gam) +
                              1.6 * vdt_exp(-1.5 * gam);
          const double phi2 = 2.0 / (3.0 + 19.5 * gam + 18.0 * g2);
          const double e2 = eps * eps;
          const double psi1 = 24.34 - 2.0 * vdt_log(1.0 + 13.111641 * e2) + 2.8 * vdt_exp(-8.0 * eps) +
                              1.2 * vdt_exp(-29.2 * eps);
          const double psi2 = 2.0 / (3.0 + 120.0 * eps + 1200.0 * e2);
          const double lz = ld(&el.logZ);
          const double Fz = lz / 3. + ld(&el.coulomb);
          const double iz = 1. / dZ;
          fv = d1 * ((0.25 * phi1 - Fz) + (0.25 * psi1 - 2. * lz / 3.) * iz) + 0.125 * omy * (phi2 + psi2 * iz);
        }
      }
      fv = dmax_(0.0, fv);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (fv < fmax * r1);
    return k;
  }

  // G4HepEmInteractionUtils.icc:10-22
  __device__ double tsai_cost(double E) {
    const double umax = 2.0 * (1.0 + E * kInvMec2);
    double u;
    int it = 0;
    do {
      const double r0 = rng.flat(), r1 = rng.flat(), r2 = rng.flat();
      const double uu = -vdt_log(r0 * r1);
      u = 0.25 > r2 ? uu * 1.6 : uu * 0.533333333;
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (u > umax);
    return 1.0 - 2.0 * u * u / (umax * umax);
  }

  // G4HepEmInteractionUtils.icc:26-76
  __device__ static void lpm_functions(double& xiS, double& gS, double& phiS, double eg, double et, double elpm,
                                       double z23, double ilS1, double ilS1c, double dcor, double times) {
    const double sqrt2 = 1.414213562373095;
    const double red = eg / et;
    const double sP = sqrt(0.125 * red * elpm / (times * (1.0 - red) * et));
    const double s1 = z23 / (184.15 * 184.15);
    const double cond = sqrt2 * s1;
    double xiSP = 2.0;
    if (sP > 1.0) {
      xiSP = 1.0;
    } else if (sP > cond) {
      const double h = vdt_log(sP) * ilS1c;
      xiSP = 1.0 + h - 0.08 * (1.0 - h) * h * (2.0 - h) * ilS1c;
    }
    xiS = xiSP;
    const double s = sP / sqrt(xiSP);
    double sh = s;
    if (dcor != 0.0) {
      sh *= (1.0 + dcor / (eg * eg));
      xiS = 2.0;
      if (sh > 1.0) xiS = 1.0;
      else if (sh > s1) xiS = 1.0 + vdt_log(sh) * ilS1;
    }
    if (sh < 2.0) {
      double val = sh * 20.0;
      int il = double_to_int_rz_exact(val);
      val -= int_to_double_exact(il);
      il *= 2;
      il = il < 0 ? 0 : (il > 78 ? 78 : il);
      gS = (kFuncLPM[il + 2] - kFuncLPM[il]) * val + kFuncLPM[il];
      phiS = (kFuncLPM[il + 3] - kFuncLPM[il + 1]) * val + kFuncLPM[il + 1];
    } else {
      double ss = 1.0 / (sh * sh);
      ss *= ss;
      gS = 1.0 - 0.0230655 * ss;
      phiS = 1.0 - 0.01190476 * ss;
    }
    if (xiS * phiS > 1.0 || sh > 0.57) xiS = 1.0 / phiS;
  }

  // ================= positron annihilation (G4HepEmPositronInteractionAnnihilation.icc) ===
  __device__ void annihilate_at_rest() {
    const double cost = 2. * rng.flat() - 1.;
    const double sint = sqrt((1. - cost) * (1. + cost));
    const double phi = k2Pi * rng.flat();
    Sec& g1 = t.addSec(2);
    Sec& g2 = t.addSec(2);
    double sp, cp;
    sincos(phi, &sp, &cp);
    g1.dir[0] = sint * cp;
    g1.dir[1] = sint * sp;
    g1.dir[2] = cost;
    g2.dir[0] = -g1.dir[0]; g2.dir[1] = -g1.dir[1]; g2.dir[2] = -g1.dir[2];
    g1.e = kMec2;
    g2.e = kMec2;
  }

  __device__ void annihilate_in_flight() {
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
    const double nrm = 1.0 / sqrt(px * px + py * py + pz * pz);
    g2.dir[0] = px * nrm; g2.dir[1] = py * nrm; g2.dir[2] = pz * nrm;
    t.setE(0.0);
  }

  // ================= gamma (G4HepEmGammaManager.icc:27-219) ===========================
  __device__ double macxs_pe(int imat, double e) {
    const DevMat& m = T.mats[imat];
    const int n = ld(&m.nSandia), off = ld(&m.sandiaOff);
    int iv = 0;
    if (e >= ld(T.sandiaE + off)) {
      for (int i = n - 1; i >= 0; --i)
        if (e >= ld(T.sandiaE + off + i)) { iv = i; break; }
    }
    const double* c = T.sandiaC + 4 * (off + iv);
    const double inv = 1 / e;
    return inv * (ld(c) + inv * (ld(c + 1) + inv * (ld(c + 2) + inv * ld(c + 3))));
  }

  __device__ double gamma_total_xs() {
    const double e = t.e, le = t.logE();
    const int imat = couple().mat;
    const DevGamma& g = T.gm;
    if (e > g.eMax1) {
      const int st = imat * g.dataPerMat + g.nData0 + g.nData1;
      return spline_log_9(g.nE2, g.mx + st, e, le, g.logEMin2, g.ild2, 1);
    }
    if (e > g.eMax0) {
      const double* d = g.mx + imat * g.dataPerMat + g.nData0;
      const int i3 = 3 * bin_of(le, g.logEMin1, g.ild1, g.nE1);
      const int j3 = i3 + 3;
      const double x0 = ld(d + i3);
      const double dl = ld(d + j3) - x0;
      const double b = dmax_(0., dmin_(1., (e - x0) / dl));
      const double tot = dmax_(0.0, ld(d + i3 + 1) + b * (ld(d + j3 + 1) - ld(d + i3 + 1)));
      t.peXS = dmax_(0.0, ld(d + i3 + 2) + b * (ld(d + j3 + 2) - ld(d + i3 + 2)));
      return tot;
    }
    const double* d = g.mx + imat * g.dataPerMat;
    const int i2 = 2 * bin_of(le, g.logEMin0, g.ild0, g.nE0);
    const double x1 = ld(d + i2), x2 = ld(d + i2 + 2);
    const double dl = x2 - x1;
    const double b = dmax_(0., dmin_(1., (e - x1) / dl));
    const double y1 = ld(d + i2 + 1);
    const double comp = y1 + b * (ld(d + i2 + 3) - y1);
    const double pe = dmax_(0.0, macxs_pe(imat, e));
    t.peXS = pe;
    return comp + pe;
  }

  __device__ void gamma_howfar() {
    if (t.nia[0] <= 0.0) t.nia[0] = -vdt_log(rng.flat());
    const double tot = gamma_total_xs();
    const double mfp = tot > 0. ? 1. / tot : kLarge;
    t.mfp[0] = mfp;
    t.gstep = mfp * t.nia[0];
  }

  __device__ void gamma_select() {
    const double u = rng.flat();
    const double e = t.e;
    const double tmfp = t.mfp[0];
    t.nia[0] = -1.0;
    const DevGamma& g = T.gm;
    if (e > g.eMax1) {
      const double le = t.logE();
      const int st = couple().mat * g.dataPerMat + g.nData0 + g.nData1;
      double mx = 0.0, cp = 0.0;
      int pid = 2;
      // after the PE column the reference evaluates one more (unused) column
      // when the cumulative is still below u: that is gamma-nuclear (winner 3)
      do {
        mx = pid < 5 ? spline_log_9(g.nE2, g.mx + st, e, le, g.logEMin2, g.ild2, pid) : 0.0;
        cp += mx * tmfp;
        ++pid;
      } while (pid < 6 && u > cp);
      t.winner = pid - 3;
      t.peXS = mx;
      return;
    }
    t.winner = (u > tmfp * t.peXS) ? 1 : 2;
  }

  __device__ void gamma_perform() {
    t.nia[0] -= t.gstep / t.mfp[0];
    t.edep = 0.0;
    if (t.onBoundary) return;
    const int ip = t.winner;
    if (ip >= 0 && ip < 4) t.nia[ip] = -1.0;
    switch (ip) {
      case 0: conversion(); break;
      case 1: compton(); break;
      case 2: photoelectric(); break;
      default: break;
    }
    const double fe = t.e;
    if (fe > 0.0 && fe <= T.gammaTrackingCut) {
      t.setE(0.0);
      t.edep += fe;
    }
  }

  // ================= conversion (G4HepEmGammaInteractionConversion.icc:19-274) =========
  __device__ int conv_target(int imat, double e, double le, double u) {
    const DevGamma& g = T.gm;
    const double* D = g.conv + ld(g.convStart + imat);
    const int nd = g.convN;
    const int ne = double_to_int_rz_exact(ld(D));
    const double* x = g.convGrid;
    const double xv = dmax_(ld(x), dmin_(ld(x + nd - 1), e));
    const int ie = clamp_trunc((le - g.convLogMin) * g.convILD, nd - 2);
    const double x1 = ld(x + ie), x2 = ld(x + ie + 1);
    const double b = dmax_(0., dmin_(1., (xv - x1) / (x2 - x1)));
    const int i0 = ie * (ne - 1) + 1;
    const int i1 = i0 + (ne - 1);
    int k = 0;
    while (k < ne - 1 && u > ld(D + i0 + k) + b * (ld(D + i1 + k) - ld(D + i0 + k))) ++k;
    return k;
  }

  __device__ static double screen1(double d) {
    return d > 1.4 ? 42.038 - 8.29 * vdt_log(d + 0.958) : 42.184 - d * (7.444 - 1.623 * d);
  }
  __device__ static double screen2(double d) {
    return d > 1.4 ? 42.038 - 8.29 * vdt_log(d + 0.958) : 41.326 - d * (5.848 - 0.902 * d);
  }
  __device__ static void phi12(double d, double& p1, double& p2) {
    if (d > 1.4) {
      p1 = 21.0190 - 4.145 * vdt_log(d + 0.958);
      p2 = p1;
    } else {
      p1 = 20.806 - d * (3.190 - 0.5710 * d);
      p2 = 20.234 - d * (2.126 - 0.0903 * d);
    }
  }

  __device__ void conversion() {
    const double E = t.e;
    if (E < 2. * kMec2) return;
    const double le = t.logE();
    const int imat = couple().mat;
    const DevMat& md = T.mats[imat];
    const int nElem = ld(&md.nElem);
    const int ei = nElem > 1 ? conv_target(imat, E, le, rng.flat()) : 0;
    const int Z = ld(T.matElemZ + ld(&md.elemOff) + ei);
    const double lpmE = kLPM * ld(&md.radLength);
    const DevElem& el = T.elems[Z < kMaxZ ? Z : kMaxZ];
    const double eps0 = kMec2 / E;
    double eps = 0.0;
    if (E < 2.0) {
      eps = eps0 + (0.5 - eps0) * rng.flat();
    } else {
      const double df = eps0 * 136. / ld(&el.Z13);
      const double dmn = 4. * df;
      const double dmx = E < 50.0 ? ld(&el.deltaMaxLow) : ld(&el.deltaMaxHigh);
      const double lz13 = 0.333333 * ld(&el.logZ);
      const double FZ = E < 50.0 ? 8. * lz13 : 8. * (lz13 + ld(&el.coulomb));
      const double epsp = 0.5 - 0.5 * sqrt(1. - dmn / dmx);
      const double epsMin = dmax_(eps0, epsp);
      const double epsRange = 0.5 - epsMin;
      double F10, F20;
      if (dmn > 1.4) {
        F10 = 42.038 - 8.29 * vdt_log(dmn + 0.958);
        F20 = F10;
      } else {
        F10 = 42.184 - dmn * (7.444 - 1.623 * dmn);
        F20 = 41.326 - dmn * (5.848 - 0.902 * dmn);
      }
      F10 -= FZ;
      F20 -= FZ;
      const double N1 = dmax_(F10 * epsRange * epsRange, 0.);
      const double N2 = dmax_(1.5 * F20, 0.);
      const double cond = N1 / (N1 + N2);
      const double iF10 = 1. / F10, iF20 = 1. / F20;
      double r2, gr;
      int it = 0;
      if (E < 100000.0) {
        do {
          const double r0 = rng.flat(), r1 = rng.flat();
          r2 = rng.flat();
          if (cond > r0) {
            eps = 0.5 - epsRange * cbrt(r1);  // reference: std::pow(u, 1./3.) of the host libm
            gr = (screen1(df / (eps * (1. - eps))) - FZ) * iF10;
          } else {
            eps = epsMin + epsRange * r1;
            gr = (screen2(df / (eps * (1. - eps))) - FZ) * iF20;
          }
          if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
        } while (gr < r2);
      } else {
        const double z23 = ld(&el.Z23), il1 = ld(&el.ilVarS1), il1c = ld(&el.ilVarS1Cond);
        do {
          const double r0 = rng.flat(), r1 = rng.flat();
          r2 = rng.flat();
          double xiS, gS, phiS, p1, p2;
          if (cond > r0) {
            eps = 0.5 - epsRange * cbrt(r1);  // reference: std::pow(u, 1./3.) of the host libm
            phi12(df / (eps * (1. - eps)), p1, p2);
            lpm_functions(xiS, gS, phiS, E, eps * E, lpmE, z23, il1, il1c, 0.0, -1.0);
            gr = xiS * ((2. * phiS + gS) * p1 - gS * p2 - phiS * FZ) * iF10;
          } else {
            eps = epsMin + epsRange * r1;
            phi12(df / (eps * (1. - eps)), p1, p2);
            lpm_functions(xiS, gS, phiS, E, eps * E, lpmE, z23, il1, il1c, 0.0, -1.0);
            gr = xiS * ((phiS + 0.5 * gS) * p1 + 0.5 * gS * p2 - 0.5 * (gS + phiS) * FZ) * iF20;
          }
          if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
        } while (gr < r2);
      }
    }
    double eT, pT;
    if (rng.flat() > 0.5) {
      eT = (1. - eps) * E;
      pT = eps * E;
    } else {
      pT = (1. - eps) * E;
      eT = eps * E;
    }
    const double eK = dmax_(0., eT - kMec2);
    const double pK = dmax_(0., pT - kMec2);
    Sec& se = t.addSec(0);
    Sec& sp = t.addSec(1);
    const double phi = k2Pi * rng.flat();
    double sph, cph;
    sincos(phi, &sph, &cph);
    const double ce = tsai_cost(eK);
    const double st = sqrt((1.0 - ce) * (1.0 + ce));
    se.dir[0] = st * cph; se.dir[1] = st * sph; se.dir[2] = ce;
    rotate(se.dir, t.dir);
    const double cpo = tsai_cost(pK);
    const double stp = sqrt((1.0 - cpo) * (1.0 + cpo));
    sp.dir[0] = -stp * cph; sp.dir[1] = -stp * sph; sp.dir[2] = cpo;
    rotate(sp.dir, t.dir);
    se.e = eK;
    sp.e = pK;
    t.setE(0.0);
  }

  // ================= Compton (G4HepEmGammaInteractionCompton.icc:17-103) ===============
  __device__ void compton() {
    const double E = t.e;
    const double thr = 0.0001;
    if (E < thr) return;
    const double org[3] = {t.dir[0], t.dir[1], t.dir[2]};
    const double kappa = E * kInvMec2;
    const double eps0 = 1. / (1. + 2. * kappa);
    const double eps02 = eps0 * eps0;
    const double al1 = -vdt_log(eps0);
    const double al2 = al1 + 0.5 * (1. - eps02);
    double eps, eps2, gf, omc, s2, r2;
    int it = 0;
    do {
      const double r0 = rng.flat(), r1 = rng.flat();
      r2 = rng.flat();
      if (al1 > al2 * r0) {
        eps = vdt_exp(-al1 * r1);
        eps2 = eps * eps;
      } else {
        eps2 = eps02 + (1. - eps02) * r1;
        eps = sqrt(eps2);
      }
      omc = (1. - eps) / (eps * kappa);
      s2 = omc * (2. - omc);
      gf = 1. - eps * s2 / (1. + eps2);
      if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
    } while (gf < r2);
    const double cost = 1.0 - omc;
    const double sint = sqrt(dmax_(0., s2));
    const double phi = k2Pi * rng.flat();
    double sp, cp;
    sincos(phi, &sp, &cp);
    t.dir[0] = sint * cp;
    t.dir[1] = sint * sp;
    t.dir[2] = cost;
    rotate(t.dir, org);
    const double post = E * eps;
    const double se = E - post;
    double dep = 0.0;
    if (se > thr) {
      Sec& s = t.addSec(0);
      s.dir[0] = E * org[0] - post * t.dir[0];
      s.dir[1] = E * org[1] - post * t.dir[1];
      s.dir[2] = E * org[2] - post * t.dir[2];
      const double nrm = 1.0 / sqrt(s.dir[0] * s.dir[0] + s.dir[1] * s.dir[1] + s.dir[2] * s.dir[2]);
      s.dir[0] *= nrm; s.dir[1] *= nrm; s.dir[2] *= nrm;
      s.e = se;
    } else {
      dep += se;
    }
    if (post > thr) {
      t.setE(post);
    } else {
      dep += post;
      t.setE(0.0);
    }
    t.edep = dep;
  }

  // ================= photoelectric (G4HepEmGammaInteractionPhotoelectric.icc) ==========
  __device__ void photoelectric() {
    const double E = t.e;
    const int imat = couple().mat;
    const DevMat& md = T.mats[imat];
    const int nElem = ld(&md.nElem), eoff = ld(&md.elemOff);
    int ie = 0;
    if (nElem > 1) {
      const double x = rng.flat() * t.peXS;
      double sum = 0;
      const double inv = 1 / E;
      for (int i = 0; i < nElem; i++) {
        const DevElem& el = T.elems[ld(T.matElemZ + eoff + i)];
        const int n = ld(&el.nSandia), off = ld(&el.sandiaOff);
        int iv = 0;
        if (E >= ld(T.sandiaE + off)) {
          for (int j = n - 1; j >= 0; j--)
            if (E >= ld(T.sandiaE + off + j)) { iv = j; break; }
        }
        const double* c = T.sandiaC + 4 * (off + iv);
        sum += ld(T.matElemN + eoff + i) * inv * (ld(c) + inv * (ld(c + 1) + inv * (ld(c + 2) + inv * ld(c + 3))));
        if (x <= sum) { ie = i; break; }
      }
    }
    const double bind = ld(&T.elems[ld(T.matElemZ + eoff + ie)].kShell);
    const double pe = E - bind;
    if (pe > 0.000001) {
      Sec& s = t.addSec(0);
      const double tau = pe * kInvMec2;
      const double gamma = 1.0 + tau;
      const double beta = sqrt(tau * (tau + 2.0)) / gamma;
      const double ac = (1.0 - beta) / beta;
      const double a1 = 0.5 * beta * gamma * tau * (gamma - 2.0);
      const double a2 = ac + 2.0;
      const double gtmax = 2.0 * (a1 + 1.0 / ac);
      double ts, gtr, r1;
      int it = 0;
      do {
        const double r0 = rng.flat();
        r1 = rng.flat();
        ts = 2.0 * ac * (2.0 * r0 + a2 * sqrt(r0)) / (a2 * a2 - 4.0 * r0);
        gtr = (2.0 - ts) * (a1 + 1.0 / (ac + ts));
        if (++it >= kMaxIter) { t.flags |= kFlagLoopCap; break; }
      } while (r1 * gtmax > gtr);
      const double ct = 1.0 - ts;
      const double st = sqrt(ts * (2.0 - ts));
      const double phi = k2Pi * rng.flat();
      double sp, cp;
      sincos(phi, &sp, &cp);
      s.dir[0] = st * cp;
      s.dir[1] = st * sp;
      s.dir[2] = ct;
      rotate(s.dir, t.dir);
      s.e = pe;
      t.edep = bind;
    } else {
      t.edep = E;
    }
    t.setE(0.0);
  }
};

}  // namespace hepem
