/*
 * hepem_port.cpp -- TEST INFRASTRUCTURE (oracle).
 *
 * Scalar CPU restatement of the reference G4HepEmRun stepping physics: one
 * track at a time, double precision, every floating-point expression in the
 * operand order of the reference so that results agree bit for bit where the
 * reference itself is deterministic (log/exp by the VDT/Cephes Pade method,
 * no contracted multiply-adds; sin/cos/pow/sqrt from the host libm).
 * It is the oracle of the GPU path on hosts without the reference sources and
 * the timed CPU baseline; it is pinned against the reference itself by
 * tests/golden (vectors written by oracle/_ref) and by tests that run both.
 *
 * Functions cite the reference file:line they restate (paths relative to
 * G4HepEm/G4HepEmRun/include/).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "g4hepem_gb300.h"
#include "hepem_port.h"
#include "philox.h"

namespace port {
namespace {

// ---- constants (G4HepEmConstants.hh:7-29) --------------------------------
const double kPi = 3.1415926535897931e+00;
const double k2Pi = 2.0 * kPi;
const double kMec2 = 5.1099890999999997e-01;
const double kInvMec2 = 1.0 / kMec2;
const double kAlpha = 7.2973525653052150e-03;
const double kPir02 = 2.4946724123674787e-23;
const double kMigdal = 5.2804955733859579e-30;
const double kLPM = 7.6843819381368661e+05;
const double kLarge = 1.0E+20;

inline double dmax(double a, double b) { return a > b ? a : b; }
inline double dmin(double a, double b) { return a < b ? a : b; }

// ---- VDT/Cephes log and exp (G4HepEmLog.hh:228-271, G4HepEmExp.hh:182-226) --
inline uint64_t bits_of(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
inline double of_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

double vlog(double x) {
  const double x0 = x;
  uint64_t n = bits_of(x);
  double fe = (double)((int32_t)(n >> 52) - 1023);
  n = (n & 0x800FFFFFFFFFFFFFULL) | 0x3FE0000000000000ULL;
  x = of_bits(n);
  if (x > 0.70710678118654752440) fe += 1.0; else x += x;
  x -= 1.0;
  double px = 1.01875663804580931796E-4;
  px = px * x + 4.97494994976747001425E-1;
  px = px * x + 4.70579119878881725854E0;
  px = px * x + 1.44989225341610930846E1;
  px = px * x + 1.79368678507819816313E1;
  px = px * x + 7.70838733755885391666E0;
  const double x2 = x * x;
  px *= x;
  px *= x2;
  double qx = x + 1.12873587189167450590E1;
  qx = qx * x + 4.52279145837532221105E1;
  qx = qx * x + 8.29875266912776603211E1;
  qx = qx * x + 7.11544750618563894466E1;
  qx = qx * x + 2.31251620126765340583E1;
  double res = px / qx;
  res -= fe * 2.121944400546905827679e-4;
  res -= 0.5 * x2;
  res = x + res;
  res += fe * 0.693359375;
  if (x0 > 1e307) res = INFINITY;
  if (x0 < 0) res = -NAN;
  return res;
}

double vexp(double x0) {
  double x = x0;
  const double t = 1.4426950408889634073599 * x + 0.5;
  int32_t fl = (int32_t)t;
  float tf = (float)t;
  uint32_t tb; memcpy(&tb, &tf, 4);
  fl -= (int32_t)(tb >> 31);
  double px = (double)fl;
  const int32_t n = (int32_t)px;
  x -= px * 6.93145751953125E-1;
  x -= px * 1.42860682030941723212E-6;
  const double xx = x * x;
  px = 1.26177193074810590878E-4;
  px *= xx;
  px += 3.02994407707441961300E-2;
  px *= xx;
  px += 9.99999999999999999910E-1;
  px *= x;
  double qx = 3.00198505138664455042E-6;
  qx *= xx;
  qx += 2.52448340349684104192E-3;
  qx *= xx;
  qx += 2.27265548208155028766E-1;
  qx *= xx;
  qx += 2.00000000000000000009E0;
  x = px / (qx - px);
  x = 1.0 + 2.0 * x;
  x *= of_bits((((uint64_t)n) + 1023) << 52);
  if (x0 > 708) x = INFINITY;
  if (x0 < -708) x = 0.;
  return x;
}

inline double vpow(double x, double a) { return vexp(a * vlog(x)); }

// ---- per-track uniform stream + Gauss/Poisson (G4HepEmRandomEngine.hh:40-97) --
struct Rng {
  const double* u;
  int32_t n;
  int32_t cursor;
  uint64_t seed;
  int32_t id;
  bool overflow;
  bool gaussValid;
  double gaussValue;
  double flat() {
    double v = cursor < n ? u[cursor] : (overflow = true, oracle_philox_uniform(seed, id, cursor));
    ++cursor;
    return v;
  }
  void flatArray(int k, double* v) { for (int i = 0; i < k; ++i) v[i] = flat(); }
  double gauss(double mean, double sd) {
    if (gaussValid) { gaussValid = false; return gaussValue * sd + mean; }
    double r, v1, v2, rnd[2];
    do {
      flatArray(2, rnd);
      v1 = 2. * rnd[0] - 1.;
      v2 = 2. * rnd[1] - 1.;
      r = v1 * v1 + v2 * v2;
    } while (r > 1.);
    const double fac = std::sqrt(-2. * vlog(r) / r);
    gaussValue = v1 * fac;
    gaussValid = true;
    return v2 * fac * sd + mean;
  }
  int poisson(double mean) {
    int number = 0;
    if (mean <= 16) {
      const double position = flat();
      double pv = vexp(-mean);
      double ps = pv;
      while (ps <= position) {
        ++number;
        pv *= mean / number;
        ps += pv;
      }
      return number;
    }
    double rnd[2];
    flatArray(2, rnd);
    const double t = std::sqrt(-2. * vlog(rnd[0])) * std::cos(k2Pi * rnd[1]);
    double value = mean + t * std::sqrt(mean) + 0.5;
    return value < 0. ? 0 : value >= 2.E+9 ? (int)2.E+9 : (int)value;
  }
};

// ---- interpolation helpers (G4HepEmRunUtils.icc:49-237) ------------------------
double spline(double x1, double x2, double y1, double y2, double s1, double s2, double x) {
  const double dl = x2 - x1;
  const double b = dmax(0., dmin(1., (x - x1) / dl));
  const double os = 0.166666666667;
  const double c0 = (2.0 - b) * s1;
  const double c1 = (1.0 + b) * s2;
  return y1 + b * (y2 - y1) + (b * (b - 1.0)) * (c0 + c1) * (dl * dl * os);
}
double linear(double x1, double x2, double y1, double y2, double x) {
  const double dl = x2 - x1;
  const double b = dmax(0., dmin(1., (x - x1) / dl));
  return y1 + b * (y2 - y1);
}
inline int bin_of(double logx, double logxmin, double ild, int ndata) {
  return (int)dmax(0., dmin((logx - logxmin) * ild, ndata - 2.));
}
// y and y'' interleaved, separate x grid
double spline_log_xy(int nd, const double* xd, const double* yd, double x, double lx, double lxm, double ild) {
  const double xv = dmax(xd[0], dmin(xd[nd - 1], x));
  const int i = bin_of(lx, lxm, ild, nd);
  return spline(xd[i], xd[i + 1], yd[2 * i], yd[2 * i + 2], yd[2 * i + 1], yd[2 * i + 3], xv);
}
// x, y, y'' interleaved
double spline_log_3(int nd, const double* d, double x, double lx, double lxm, double ild) {
  const double xv = dmax(d[0], dmin(d[3 * (nd - 1)], x));
  const int i = 3 * bin_of(lx, lxm, ild, nd);
  return spline(d[i], d[i + 3], d[i + 1], d[i + 4], d[i + 2], d[i + 5], xv);
}
// stride-9 gamma window-2 rows, one of the 4 quantities (iwhich = 1..4)
double spline_log_9(int nd, const double* d, double x, double lx, double lxm, double ild, int iwhich) {
  const int i0 = 9 * bin_of(lx, lxm, ild, nd);
  const int i1 = i0 + 9;
  const int w = (iwhich - 1) * 2 + 1;
  return spline(d[i0], d[i1], d[i0 + w], d[i1 + w], d[i0 + w + 1], d[i1 + w + 1], x);
}
int lower_bin(const double* xd, int num, double x, int step) {
  int ml = -1, mu = num - 1;
  while (std::abs(mu - ml) > 1) {
    const int mav = 0.5 * (ml + mu);
    if (x < xd[step * mav]) mu = mav; else ml = mav;
  }
  return mu - 1;
}
void rotate(double* d, const double* r) {
  double up = r[0] * r[0] + r[1] * r[1];
  if (up > 0.) {
    up = std::sqrt(up);
    const double px = d[0], py = d[1], pz = d[2];
    d[0] = (r[0] * r[2] * px - r[1] * py) / up + r[0] * pz;
    d[1] = (r[1] * r[2] * px + r[0] * py) / up + r[1] * pz;
    d[2] = -up * px + r[2] * pz;
  } else if (r[2] < 0.) {
    d[0] = -d[0];
    d[2] = -d[2];
  }
}

// ---- track data ----------------------------------------------------------------
struct Msc {                    // G4HepEmMSCTrackData.hh:112-131
  double lambtr1 = 0, trueStep = 0, zPath = 0, disp[3] = {0, 0, 0}, dir[3] = {0, 0, 1};
  double initRange = 1e21, dynFactor = 0.04, tlimitMin = 1e-7, par1 = -1, par2 = 0, par3 = 0;
  bool noScatter = false, displace = false, firstStep = true, active = false;
};

struct Track {                  // G4HepEmTrack + G4HepEmElectronTrack + G4HepEmGammaTrack
  double e = 0, le = 100.0, dir[3] = {0, 0, 0}, charge = 0, edep = 0, gstep = 0;
  double mfp[4] = {-1, -1, -1, -1}, nia[4] = {-1, -1, -1, -1}, safety = 0;
  int id = -1, imc = -1, winner = -1;
  bool onBoundary = false;
  double range = 0, pstep = 0, preE = 0, preLE = 0, peXS = 0;
  Msc msc;
  void setE(double v) { e = v; le = 100.0; }
  double logE() {
    if (le > 99.0) le = (e > 0.) ? vlog(e) : -30;
    return le;
  }
};

struct Secondary { int type; double e; double dir[3]; };

struct Step {
  const State& S;
  Rng& rng;
  Track t;
  Secondary sec[2];
  int nsec = 0;
  Step(const State& s, Rng& r) : S(s), rng(r) {}
  Secondary& addSec(int type) { Secondary& s = sec[nsec < 2 ? nsec : 1]; ++nsec; s.type = type; return s; }

  const ElData& eld() const { return t.charge < 0.0 ? S.el[0] : S.el[1]; }
  bool isElectron() const { return t.charge < 0.0; }
  const Couple& couple() const { return S.couples[t.imc]; }
  const Mat& mat() const { return S.mats[S.couples[t.imc].mat]; }
  const Region& region() const { return S.pars.regions[S.couples[t.imc].region]; }

  // ---- electron table accessors (G4HepEmElectronManager.icc:486-599) ------------
  static double restRange(const ElData& d, int imc, double e, double le) {
    const int n = d.nLoss;
    return dmax(0.0, spline_log_xy(n, d.lossGrid.data(), &d.loss[5 * n * imc], e, le, d.lossLogMin, d.lossILD));
  }
  static double restDEDX(const ElData& d, int imc, double e, double le) {
    const int n = d.nLoss;
    return dmax(0.0, spline_log_xy(n, d.lossGrid.data(), &d.loss[n * (5 * imc + 2)], e, le, d.lossLogMin, d.lossILD));
  }
  static double invRange(const ElData& d, int imc, double r) {
    const int n = d.nLoss;
    const int s = 5 * n * imc;
    const double rmin = d.loss[s];
    if (r < rmin) {
      const double q = r / rmin;
      return dmax(0.0, d.lossGrid[0] * q * q);
    }
    const int i = lower_bin(&d.loss[s], n, r, 2);
    const double* R = &d.loss[s];
    const double* S2 = &d.loss[s + 4 * n];
    return dmax(0.0, spline(R[2 * i], R[2 * (i + 1)], d.lossGrid[i], d.lossGrid[i + 1], S2[i], S2[i + 1], r));
  }
  static double restMacXS(const ElData& d, int imc, double e, double le, bool ioni) {
    const int i0 = d.xsStart[imc];
    const int nIoni = (int)d.xs[i0];
    const int st = ioni ? i0 : i0 + 3 * nIoni + 5;
    const int nd = (int)d.xs[st];
    if (e < d.xs[st + 5]) return 0.0;
    return dmax(0.0, spline_log_3(nd, &d.xs[st + 5], e, le, d.xs[st + 3], d.xs[st + 4]));
  }
  static double nucMacXS(const ElData& d, int imat, double e, double le) {
    if (e < d.nucGrid[0]) return 0.0;
    const int n = d.nNuc;
    return dmax(0.0, spline_log_xy(n, d.nucGrid.data(), &d.nuc[imat * 2 * n], e, le, d.nucLogMin, d.nucILD));
  }
  static double restMacXSStepping(const ElData& d, int imc, double e, double le, bool ioni) {
    const double log08 = -0.22314355131420971;
    const int i0 = d.xsStart[imc];
    const int nIoni = (int)d.xs[i0];
    const int st = ioni ? i0 : i0 + 3 * nIoni + 5;
    const int nd = (int)d.xs[st];
    const double minE = d.xs[st + 5], maxE = d.xs[st + 1], maxV = d.xs[st + 2];
    if (e > maxE) {
      const double er = 0.8 * e;
      if (er < maxE) return dmax(0.0, maxV);
      e = er;
      le += log08;
    }
    if (e < minE) return 0.0;
    return dmax(0.0, spline_log_3(nd, &d.xs[st + 5], e, le, d.xs[st + 3], d.xs[st + 4]));
  }
  static double transportMFP(const ElData& d, int imat, double e, double le) {
    const int n = d.nLoss;
    const double v = dmax(0.0, spline_log_xy(n, d.lossGrid.data(), &d.tr1[2 * n * imat], e, le, d.lossLogMin, d.lossILD));
    return v > 0. ? 1. / v : kLarge;
  }
  static double annihXS(double e, double ne) {
    const double tau = e * kInvMec2;
    const double gam = tau + 1.0;
    const double gam2 = gam * gam;
    const double bg2 = tau * (tau + 2.0);
    const double bg = std::sqrt(bg2);
    return ne * kPir02 * ((gam2 + 4. * gam + 1.) * vlog(gam + bg) - (gam + 3.) * bg) / (bg2 * (gam + 1.));
  }

  // ---- e+- HowFar (G4HepEmElectronManager.icc:35-169) ----------------------------
  void elHowFar() {
    for (int ip = 0; ip < 4; ++ip)
      if (t.nia[ip] <= 0.) t.nia[ip] = -vlog(rng.flat());
    // discrete / continuous limit (:48-101)
    const ElData& d = eld();
    const double e = t.e, le = t.logE();
    const int imc = t.imc;
    const double range = restRange(d, imc, e, le);
    t.range = range;
    const Region& reg = region();
    const double frange = reg.finalRange, drange = reg.dRoverRange;
    double pstep = range > frange ? range * drange + frange * (1.0 - drange) * (2.0 - frange / range) : range;
    int winner = -1;
    const int imat = couple().mat;
    double mx[4];
    mx[0] = restMacXSStepping(d, imc, e, le, true);
    mx[1] = restMacXSStepping(d, imc, e, le, false);
    mx[2] = isElectron() ? 0.0 : annihXS(0.8 * e, S.mats[imat].elDensity);
    mx[3] = nucMacXS(d, imat, e, le);
    for (int ip = 0; ip < 4; ++ip) {
      const double mfp = mx[ip] > 0. ? 1. / mx[ip] : kLarge;
      t.mfp[ip] = mfp;
      const double lim = mfp * t.nia[ip];
      if (lim < pstep) { pstep = lim; winner = ip; }
    }
    t.pstep = pstep;
    t.winner = winner;
    t.gstep = pstep;
    // MSC (:103-164)
    Msc& m = t.msc;
    m.trueStep = pstep;
    m.zPath = pstep;
    m.active = false;
    m.disp[0] = m.disp[1] = m.disp[2] = 0.;
    m.dir[0] = 0.; m.dir[1] = 0.; m.dir[2] = 1.;
    if (pstep > 5.E-8 && e > 1.0E-3) {
      m.active = true;
      m.lambtr1 = transportMFP(d, imat, e, le);
      mscStepLimit(e, imat, range);
      trueToGeom(e, range);
      if (m.trueStep < pstep) {
        t.winner = -2;
        pstep = m.trueStep;
        t.pstep = pstep;
      }
      t.gstep = dmin(m.zPath, pstep);
    }
  }

  // G4HepEmElectronInteractionUMSC.icc:19-126
  void mscStepLimit(double e, int imat, double range) {
    Msc& m = t.msc;
    const Mat& md = S.mats[imat];
    const Region& reg = region();
    m.noScatter = false;
    m.displace = true;
    const double kTLimitMinfix = 1.0E-8;
    if (m.trueStep < kTLimitMinfix || range * md.umscPar < t.safety) {
      m.displace = false;
      return;
    }
    const double rf = reg.mscRangeFactor, sf = reg.mscSafetyFactor;
    double tlimit = 0.0;
    if (!reg.mscMinimal) {
      if (m.firstStep || t.onBoundary) {
        const double l1 = m.lambtr1;
        m.initRange = dmax(range, l1);
        m.dynFactor = l1 > 1.0 ? rf * (0.75 + 0.25 * l1) : rf;
        const double stepMin = l1 * 1.0E-3 / (2.0E-3 + e * (md.stepMin[0] + e * md.stepMin[1]));
        const double d0 = isElectron() ? 0.87 * md.zeff23 : 0.70 * md.zeffSqrt;
        const double d1 = e > 5.0E-3 ? d0 * stepMin : d0 * stepMin * 0.5 * (1.0 + e * 200.0);
        m.tlimitMin = dmax(d1, kTLimitMinfix);
        m.firstStep = false;
      }
      const double tlm = m.tlimitMin;
      tlimit = range > t.safety ? dmax(dmax(m.initRange * m.dynFactor, sf * t.safety), tlm) : dmax(range, tlm);
    } else {
      if (t.onBoundary) {
        const double l1 = m.lambtr1;
        const double tmp = range > l1 ? rf * range : rf * l1;
        m.initRange = dmax(tmp, 10 * kTLimitMinfix);
      }
      tlimit = m.initRange;
    }
    const double tlm = m.tlimitMin;
    if (tlimit < m.trueStep) {
      const double d0 = tlimit > tlm ? dmax(rng.gauss(tlimit, 0.1 * (tlimit - tlm)), tlm) : tlm;
      m.trueStep = dmin(d0, m.trueStep);
    }
  }

  // G4HepEmElectronManager.icc:602-650
  void trueToGeom(double e, double range) {
    Msc& m = t.msc;
    m.par1 = -1.; m.par2 = 0.; m.par3 = 0.;
    m.trueStep = dmin(m.trueStep, range);
    m.zPath = m.trueStep;
    if (m.trueStep < 1.0E-6) return;
    const double tau = m.trueStep / m.lambtr1;
    if (tau < 1.0e-16) {
      m.zPath = dmin(m.trueStep, m.lambtr1);
    } else if (m.trueStep < range * 0.05) {
      m.zPath = tau < 1.0e-6 ? m.trueStep * (1. - 0.5 * tau) : m.lambtr1 * (1. - vexp(-tau));
    } else if (e < kMec2 || m.trueStep == range) {
      m.par1 = 1. / range;
      m.par2 = 1. / (m.par1 * m.lambtr1);
      m.par3 = 1. + m.par2;
      m.zPath = 1. / (m.par1 * m.par3);
      if (m.trueStep < range) m.zPath *= (1. - vpow(1. - m.trueStep / range, m.par3));
    } else {
      const double rfin = dmax(range - m.trueStep, 0.01 * range);
      const ElData& d = eld();
      const double t1 = invRange(d, t.imc, rfin);
      const double l1 = transportMFP(d, couple().mat, t1, vlog(t1));
      m.par1 = (m.lambtr1 - l1) / (m.lambtr1 * m.trueStep);
      m.par2 = 1. / (m.par1 * m.lambtr1);
      m.par3 = 1. + m.par2;
      m.zPath = (1. - vpow(l1 / m.lambtr1, m.par3)) / (m.par1 * m.par3);
    }
    m.zPath = dmin(m.zPath, m.lambtr1);
  }

  // G4HepEmElectronManager.icc:653-691
  void geomToTrue(double range, double g) {
    Msc& m = t.msc;
    m.zPath = g;
    if (g < 1.0E-6) {
      m.trueStep = g;
      return;
    }
    double tl = g;
    if (g > m.lambtr1 * 1.0e-16) {
      if (m.par1 < 0.) {
        tl = -m.lambtr1 * vlog(1. - g / m.lambtr1);
      } else {
        const double dum = m.par1 * m.par3 * g;
        tl = dum < 1. ? (1. - vpow(1. - dum, 1. / m.par3)) / m.par1 : range;
      }
      if (tl < g) tl = g;
    }
    m.trueStep = tl;
  }

  // ---- e+- Perform (G4HepEmElectronManager.icc:171-483) -----------------------------
  void elPerform() {
    t.edep = 0;
    t.pstep = t.gstep;
    const bool isEl = isElectron();
    if (t.gstep <= 0.) return;
    const bool stopped = elContinuous();
    if (stopped) {
      if (!isEl) annihilateAtRest();
      return;
    }
    elDiscrete();
  }

  bool elContinuous() {
    t.preE = t.e;
    t.preLE = t.logE();
    // UpdatePStepLength (:171-203)
    {
      const double g = t.gstep;
      double p = g;
      Msc& m = t.msc;
      if (m.active) {
        p = m.trueStep;
        if (g < m.zPath) {
          geomToTrue(t.range, g);
          p = dmin(p, m.trueStep);
          m.trueStep = p;
        }
        if (p <= 5.E-8 || t.range <= p) m.active = false;
      }
      t.pstep = p;
    }
    const double pstep = t.pstep;
    if (pstep <= 0.0) return false;
    for (int i = 0; i < 4; ++i) t.nia[i] -= pstep / t.mfp[i];
    if (meanLoss()) return true;
    sampleMSC();
    return lossFluct();
  }

  // :216-259
  bool meanLoss() {
    const double pstep = t.pstep;
    const double e = t.e;
    const double range = t.range;
    if (pstep >= range || e <= S.pars.minLossE) {
      t.edep = e;
      t.setE(0.0);
      return true;
    }
    const ElData& d = eld();
    const int imc = t.imc;
    const double le = t.logE();
    double eloss = pstep * restDEDX(d, imc, e, le);
    if (eloss > e * region().linELossLimit) {
      const double post = range - pstep;
      eloss = e - invRange(d, imc, post);
    }
    eloss = dmax(eloss, 0.0);
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

  // :261-322
  void sampleMSC() {
    const double pstep = t.pstep;
    const bool isEl = isElectron();
    const double preE = t.preE;
    const double range = t.range;
    const ElData& d = eld();
    Msc& m = t.msc;
    if (m.active && pstep > dmax(1.0E-8, 1.0e-16 * m.lambtr1)) {
      double postE = preE;
      double postLE = t.preLE;
      if (pstep > range * 0.01) {
        postE = t.e;
        postLE = t.logE();
      }
      const int imat = couple().mat;
      const double postMFP = transportMFP(d, imat, postE, postLE);
      mscScatter(pstep, preE, m.lambtr1, postE, postMFP, imat, isEl, S.pars.mscPosCor, S.pars.mscDisplacement);
      if (!m.noScatter) {
        rotate(m.dir, t.dir);
        if (m.displace) rotate(m.disp, t.dir);
        t.dir[0] = m.dir[0]; t.dir[1] = m.dir[1]; t.dir[2] = m.dir[2];
      }
    }
  }

  // G4HepEmElectronInteractionUMSC.icc:129-150
  void mscScatter(double pstep, double preE, double preMFP, double postE, double postMFP, int imat, bool isEl,
                  bool posCor, bool isDisplace) {
    Msc& m = t.msc;
    const Mat& md = S.mats[imat];
    const double cost = mscCosTheta(pstep, preE, preMFP, postE, postMFP, m.tlimitMin, md.radLength, md.zeff,
                                    md.tail, md.theta, isEl, posCor);
    if (std::abs(cost) >= 1.0) {
      m.noScatter = true;
      return;
    }
    const double sth = std::sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = k2Pi * rng.flat();
    m.dir[0] = sth * std::cos(phi);
    m.dir[1] = sth * std::sin(phi);
    m.dir[2] = cost;
    m.displace = m.displace && isDisplace;
    if (m.displace && pstep > m.zPath) {
      // SampleDisplacement (:342-357)
      const double r = 0.73 * std::sqrt((pstep - m.zPath) * (pstep + m.zPath));
      const double cbeta = 2.16;
      const double cbeta1 = 1. - vexp(-cbeta * kPi);
      double rnd[2];
      rng.flatArray(2, rnd);
      const double psi = -vlog(1. - rnd[0] * cbeta1) / cbeta;
      const double ph = rnd[1] < 0.5 ? phi + psi : phi - psi;
      m.disp[0] = r * std::cos(ph);
      m.disp[1] = r * std::sin(ph);
      m.disp[2] = 0.0;
    }
  }

  // :153-270
  double mscCosTheta(double pstep, double preE, double preMFP, double postE, double postMFP, double tlimMin,
                     double radLen, double zeff, const double* tail, const double* thc, bool isEl, bool posCor) {
    const double iPre = 1.0 / preMFP;
    const double dR = preMFP - postMFP;
    const double tau = std::abs(dR) > 0.01 * preMFP ? pstep * vlog(preMFP / postMFP) / dR : pstep * iPre;
    if (tau > 8.0) return 2.0 * rng.flat() - 1.0;
    if (tau < 1.0E-16) return 1.0;
    double xm, x2m;
    if (tau < 0.01) {
      xm = 1.0 - tau * (1.0 - 0.5 * tau);
      x2m = 1.0 - tau * (5.0 - 6.25 * tau) * 0.333333;
    } else {
      xm = vexp(-tau);
      x2m = (1.0 + 2.0 * vexp(-2.5 * tau)) * 0.333333;
    }
    if (postE < 0.5 * preE) return simpleScatter(xm, x2m);
    const double tsmall = dmin(tlimMin, 1.0);
    const bool notSmall = pstep > tsmall;
    const double theta0 = notSmall
        ? theta0Of(pstep / radLen, postE, preE, zeff, thc, isEl, posCor)
        : theta0Of(tsmall / radLen, postE, preE, zeff, thc, isEl, posCor) * std::sqrt(pstep / tsmall);
    if (theta0 > kPi * 0.166666) return simpleScatter(xm, x2m);
    const double th2 = theta0 * theta0;
    if (th2 < 1.0E-16) return 1.0;
    const double dumtau = notSmall ? tau : tsmall * iPre;
    const double u = vpow(dumtau, 0.1666666);
    const double dumxsi = tail[0] + u * (tail[1] + u * tail[2]) + tail[3] * vlog(pstep / (tau * radLen));
    const double xsi = dmax(dumxsi, 1.9);
    const double c = std::abs(xsi - 3.) < 0.001 ? 3.001 : std::abs(xsi - 2.) < 0.001 ? 2.001 : xsi;
    const double c1 = c - 1.;
    const double ea = vexp(-xsi);
    const double eaa = 1. / (1. - ea);
    double thex = th2 * (1.0 - th2 * 0.0833333);
    if (th2 > 0.01) {
      const double q = 2.0 * std::sin(0.5 * theta0);
      thex = q * q;
    }
    const double xmean1 = 1. - (1. - (1. + xsi) * ea) * thex * eaa;
    if (xmean1 <= 0.999 * xm) return simpleScatter(xm, x2m);
    const double x0 = 1. - xsi * thex;
    const double bx = c * thex;
    const double b = bx + x0;
    const double b1 = b + 1.;
    const double eb1 = vpow(b1, c1);
    const double ebx = vpow(bx, c1);
    const double dd = ebx / eb1;
    const double xmean2 = (x0 + dd - (bx - b1 * dd) / (c - 2.)) / (1. - dd);
    const double f1x0 = ea * eaa;
    const double f2x0 = c1 / (c * (1. - dd));
    const double prob = f2x0 / (f1x0 + f2x0);
    const double qprb = xm / (prob * xmean1 + (1. - prob) * xmean2);
    double r[3];
    rng.flatArray(3, r);
    if (r[0] < qprb) {
      if (r[1] < prob) return 1. + vlog(ea + r[2] / eaa) * thex;
      const double var0 = (1.0 - dd) * r[2];
      if (var0 < 0.01 * dd) {
        const double var = var0 / (dd * c1);
        return -1.0 + var * (1.0 - var * 0.5 * c) * b1;
      }
      return 1.0 + thex * (c - xsi - c * vpow(var0 + dd, -1. / c1));
    }
    return 2.0 * r[1] - 1.0;
  }

  double simpleScatter(double xm, double x2m) {
    const double d0 = 3. * x2m - 1;
    const double d1 = 2. * xm - d0;
    const double a = 1. + 4. * d0 / d1;
    const double prob = (2. + a) * xm / a;
    double r[2];
    rng.flatArray(2, r);
    return r[0] < prob ? -1. + 2. * vpow(r[1], 1. / (1. + a)) : -1. + 2. * r[1];
  }

  static double theta0Of(double srl, double postE, double preE, double zeff, const double* thc, bool isEl,
                         bool posCor) {
    const double postInv = (postE + kMec2) / (postE * (postE + 2. * kMec2));
    const double inv = preE != postE ? std::sqrt(postInv * (preE + kMec2) / (preE * (preE + 2. * kMec2))) : postInv;
    const double y = (isEl || !posCor) ? srl : srl * posCorrection(preE * postE, zeff);
    return 13.6 * std::sqrt(y) * inv * (thc[0] + thc[1] * vlog(y));
  }

  static double posCorrection(double eekin, double zeff) {
    const double ff = 1. + zeff * (1.84035E-4 * zeff - 1.86427E-2) + 0.41125;
    const double a = 0.994 - 4.08E-3 * zeff;
    const double b = 7.16 + (52.6 + 365. / zeff) / zeff;
    const double tu = std::sqrt(eekin) * kInvMec2;
    const double x = std::sqrt(tu * (tu + 2.) / ((tu + 1.) * (tu + 1.)));
    if (x < 0.6) return ff * a * (1. - vexp(-b * x));
    const double c = 1.00 - 4.47E-3 * zeff;
    const double d = 1.21E-3 * zeff;
    if (x > 0.9) return ff * (c + d * vexp(113.0 * (x - 1.)));
    const double yl = a * (1. - vexp(-b * 0.6));
    const double yh = c + d * vexp(113.0 * (0.9 - 1.));
    const double y0 = (yh - yl) / (0.9 - 0.6);
    const double y1 = yl - y0 * 0.6;
    return ff * (y0 * x + y1);
  }

  // :324-368 and G4HepEmElectronEnergyLossFluctuation.icc:11-111
  bool lossFluct() {
    const double pstep = t.pstep;
    const bool isEl = isElectron();
    const double preE = t.preE;
    double finalE = t.e;
    double eloss = t.edep;
    const int fl = region().eLossFluct;
    if (fl && eloss > 1.E-5) {
      const Couple& c = couple();
      const double tmax = isEl ? 0.5 * preE : preE;
      const double tcut = dmin(c.elCut, tmax);
      eloss = fluct(tcut, S.mats[c.mat].meanExc, pstep, eloss);
      eloss = dmax(eloss, 0.0);
      finalE = preE - eloss;
    }
    if (finalE <= S.pars.electronTrackingCut) {
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

  double fluct(double tcut, double excE, double /*step*/, double meanE) {
    const double scaling = dmin(1. + 5.E-4 / tcut, 1.5);
    const double meanLoss = meanE / scaling;
    const double rate = 0.56, e0 = 1.E-5, nmax = 8.;
    const double w1 = tcut / e0;
    double a3 = meanLoss * (tcut - e0) / (e0 * tcut * vlog(w1));
    double a1 = 0.;
    double e1 = excE;
    double eloss = 0.0;
    if (tcut > excE) {
      const double a1t = meanLoss * (1. - rate) / excE;
      const double d0 = a1t < 42. ? .1 + (4. - .1) * std::sqrt(a1t / 42.) : 4.;
      a1 = a1t / d0;
      e1 *= d0;
      a3 *= rate;
      if (a1 > nmax) {
        const double em = a1 * e1;
        eloss = gaussLoss(em, em * e1);
      } else {
        const int p = rng.poisson(a1);
        eloss = p > 0 ? ((p + 1) - 2. * rng.flat()) * e1 : 0.;
      }
    }
    if (a3 > 0.) {
      double p3 = a3;
      double alfa = 1.;
      if (a3 > nmax) {
        alfa = w1 * (nmax + a3) / (w1 * nmax + a3);
        const double alfa1 = alfa * vlog(alfa) / (alfa - 1.);
        const double nam = a3 * w1 * (alfa - 1.) / ((w1 - 1.) * alfa);
        const double em = nam * e0 * alfa1;
        const double s2 = e0 * e0 * nam * (alfa - alfa1 * alfa1);
        eloss += gaussLoss(em, s2);
        p3 = a3 - nam;
      }
      const double w3 = alfa * e0;
      if (tcut > w3) {
        const double w = (tcut - w3) / tcut;
        const int nnb = rng.poisson(p3);
        if (nnb > 0) {
          // the reference draws in blocks of 8 then the tail; the stream order
          // is the same as drawing one by one
          for (int k = 0; k < nnb; ++k) eloss += w3 / (1. - w * rng.flat());
        }
      }
    }
    return eloss * scaling;
  }

  double gaussLoss(double me, double s2) {
    const double twom = 2. * me;
    if (me * me < 0.0625 * s2) return twom * rng.flat();
    const double sig = std::sqrt(s2);
    double el;
    do {
      el = rng.gauss(me, sig);
    } while (el < 0. || el > twom);
    return el;
  }

  // :408-459
  void elDiscrete() {
    const bool isEl = isElectron();
    const int ip = t.winner;
    if (ip < 0 || t.onBoundary) return;
    t.nia[ip] = -1.0;
    // CheckDelta
    {
      const ElData& d = eld();
      const int imat = couple().mat;
      const double e = t.e, le = t.logE();
      const double mx = ip < 2 ? restMacXS(d, t.imc, e, le, ip == 0)
                       : (ip < 3 ? annihXS(e, S.mats[imat].elDensity) : nucMacXS(d, imat, e, le));
      const double u = rng.flat();
      if (mx <= 0.0 || u > mx * t.mfp[ip]) return;
    }
    const double e = t.e;
    switch (ip) {
      case 0: ioni(isEl); break;
      case 1: brem(isEl, e < S.pars.bremModelLim); break;
      case 2: annihilateInFlight(); break;
      default: break;
    }
  }

  // ---- Moller-Bhabha (G4HepEmElectronInteractionIoni.icc:19-138) ---------------------
  void ioni(bool isEl) {
    const double E = t.e;
    const double cut = couple().elCut;
    const double tmaxE = isEl ? 0.5 * E : E;
    if (tmaxE <= cut) return;
    const double dE = isEl ? moller(cut, E) : bhabha(cut, E);
    Secondary& s = addSec(0);
    const double eTot = E + kMec2;
    const double pTot = std::sqrt(E * (eTot + kMec2));
    const double dP = std::sqrt(dE * (dE + 2.0 * kMec2));
    const double cost = dE * (eTot + kMec2) / (dP * pTot);
    const double ct = dmax(-1.0, dmin(cost, 1.0));
    const double st = std::sqrt((1.0 - ct) * (1.0 + ct));
    const double phi = k2Pi * rng.flat();
    s.dir[0] = st * std::cos(phi);
    s.dir[1] = st * std::sin(phi);
    s.dir[2] = ct;
    rotate(s.dir, t.dir);
    t.dir[0] = pTot * t.dir[0] - dP * s.dir[0];
    t.dir[1] = pTot * t.dir[1] - dP * s.dir[1];
    t.dir[2] = pTot * t.dir[2] - dP * s.dir[2];
    const double nrm = 1.0 / std::sqrt(t.dir[0] * t.dir[0] + t.dir[1] * t.dir[1] + t.dir[2] * t.dir[2]);
    t.dir[0] *= nrm; t.dir[1] *= nrm; t.dir[2] *= nrm;
    t.setE(E - dE);
    s.e = dE;
  }

  double moller(double cut, double E) {
    const double xmin = cut / E;
    const double xmax = 0.5 * E / E;
    const double gam = E * kInvMec2 + 1.0;
    const double g2 = gam * gam;
    const double xmm = xmin * xmax;
    const double gg = (2.0 * gam - 1.0) / g2;
    const double y = 1. - xmax;
    const double gf = 1.0 - gg * xmax + xmax * xmax * (1.0 - gg + (1.0 - gg * y) / (y * y));
    double dum, r[2], x;
    do {
      rng.flatArray(2, r);
      x = xmm / (xmin * (1.0 - r[0]) + xmax * r[0]);
      const double xx = 1.0 - x;
      dum = 1.0 - gg * x + x * x * (1.0 - gg + (1.0 - gg * xx) / (xx * xx));
    } while (gf * r[1] > dum);
    return x * E;
  }

  double bhabha(double cut, double E) {
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
    double dum, r[2], x;
    do {
      rng.flatArray(2, r);
      x = xmm / (xmin * (1.0 - r[0]) + xmax * r[0]);
      const double xx = x * x;
      dum = 1.0 + (xx * xx * c4 - x * xx * c3 + xx * c2 - x * c1) * b2;
    } while (gf * r[1] > dum);
    return x * E;
  }

  // ---- bremsstrahlung (G4HepEmElectronInteractionBrem.icc:35-344) ---------------------
  void brem(bool isEl, bool sbModel) {
    const double E = t.e;
    const double le = t.logE();
    const Couple& c = couple();
    if (E <= c.gamCut) return;
    const double k = sbModel ? sampleSB(E, le, isEl) : sampleRB(E, le, isEl);
    Secondary& s = addSec(2);
    // SampleDirections (:298-323)
    const double cost = tsaiCost(E);
    const double sint = std::sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = k2Pi * rng.flat();
    s.dir[0] = sint * std::cos(phi);
    s.dir[1] = sint * std::sin(phi);
    s.dir[2] = cost;
    rotate(s.dir, t.dir);
    const double eTot = E + kMec2;
    const double pTot = std::sqrt(E * (eTot + kMec2));
    t.dir[0] = pTot * t.dir[0] - k * s.dir[0];
    t.dir[1] = pTot * t.dir[1] - k * s.dir[1];
    t.dir[2] = pTot * t.dir[2] - k * s.dir[2];
    const double nrm = 1.0 / std::sqrt(t.dir[0] * t.dir[0] + t.dir[1] * t.dir[1] + t.dir[2] * t.dir[2]);
    t.dir[0] *= nrm; t.dir[1] *= nrm; t.dir[2] *= nrm;
    t.setE(E - k);
    s.e = k;
  }

  int selectBremTarget(double E, double le, double u, bool sb) {
    const ElData& d = eld();
    const int st = sb ? d.selSBStart[t.imc] : d.selRBStart[t.imc];
    const double* D = sb ? &d.selSB[st] : &d.selRB[st];
    const int nd = (int)D[0];
    const int ne = (int)D[1];
    const double* x = &D[4];
    const double xv = dmax(x[0], dmin(x[ne * (nd - 1)], E));
    const int ie = (int)dmax(0.0, dmin((le - D[2]) * D[3], nd - 2.0));
    int i0 = ie * ne, i1 = i0 + ne;
    const double x1 = x[i0++], x2 = x[i1++];
    const double b = dmax(0., dmin(1., (xv - x1) / (x2 - x1)));
    int k = 0;
    while (k < ne - 1 && u > x[i0 + k] + b * (x[i1 + k] - x[i0 + k])) ++k;
    return k;
  }

  static int linSearch(const double* v, int size, double val) {
    int i = 0;
    const int s3 = 3 * size;
    while (i + 9 < s3) {
      if (v[i] > val) return i;
      if (v[i + 3] > val) return i + 3;
      if (v[i + 6] > val) return i + 6;
      if (v[i + 9] > val) return i + 9;
      i += 12;
    }
    while (i < s3) {
      if (v[i] > val) break;
      i += 3;
    }
    return i;
  }

  double sampleSB(double E, double le, bool isEl) {
    const Couple& c = couple();
    const double gcut = c.gamCut, lgcut = c.logGamCut;
    const Mat& md = S.mats[c.mat];
    const int ei = md.elems.size() > 1 ? selectBremTarget(E, le, rng.flat(), true) : 0;
    const int Z = md.elems[ei];
    const double dZ = (double)Z;
    const SB& sb = S.sb;
    const int st = sb.startPerZ[Z];
    const int gci = sb.gcIdx[sb.gcStart[t.imc] + ei];
    bool corner = false, simple = false;
    int ie = (int)sb.data[st + 2];
    if (E < sb.elE[ie]) {
      const double val = (le - sb.logMinE) * sb.ildE;
      ie = (int)val;
      double pH = val - ie;
      if (sb.elE[ie] <= gcut) {
        pH = (le - lgcut) / (sb.lelE[ie + 1] - lgcut);
        corner = true;
      }
      if (rng.flat() < pH) ++ie;
      else if (corner) simple = true;
    }
    const int minIE = (int)sb.data[st + 1];
    const int ncut = (int)sb.data[st + 3];
    const int size1 = (int)(ncut + 3 * sb.numKappa);
    const int tst = st + 4 + (ie - minIE) * size1;
    const double minV = sb.data[tst + gci];
    const double* T = &sb.data[tst + ncut];
    const double lkt = (lgcut - le) / (lgcut - sb.lelE[ie]);
    const double pe = E + kMec2;
    const double dsc = md.densityCor * pe * pe;
    double sup = 1.0, r[2], k = 0.0;
    do {
      rng.flatArray(2, r);
      double kappa = 1.0;
      if (!simple) {
        const double cum = r[0] * (1.0 - minV) + minV;
        const int i3 = linSearch(T, sb.numKappa, cum) - 3;
        const int i = i3 / 3;
        const double cL = T[i3], pA = T[i3 + 1], pB = T[i3 + 2], cH = T[i3 + 3];
        const double lKL = sb.lkappa[i], lKH = sb.lkappa[i + 1];
        const double m1 = (cum - cL) / (cH - cL);
        const double m2 = (1.0 + pA + pB) * m1;
        const double m3 = 1.0 + m1 * (pA + pB * m1);
        const double lk = lKL + m2 / m3 * (lKH - lKL);
        kappa = vexp(lk * lkt);
      } else {
        kappa = 1.0 - r[0] * (1.0 - gcut / E);
      }
      k = kappa * E;
      const double ik = 1.0 / k;
      sup = 1.0 / (1.0 + dsc * ik * ik);
      if (!isEl) {
        const double e1 = E - gcut;
        const double ib1 = (e1 + kMec2) / std::sqrt(e1 * (e1 + 2.0 * kMec2));
        const double e2 = E - k;
        const double ib2 = (e2 + kMec2) / std::sqrt(e2 * (e2 + 2.0 * kMec2));
        const double dum = kAlpha * k2Pi * dZ * (ib1 - ib2);
        sup = dum > -12. ? sup * vexp(dum) : 0.;
      }
    } while (r[1] > sup);
    return k;
  }

  double sampleRB(double E, double le, bool isEl) {
    const Couple& c = couple();
    const double gcut = c.gamCut;
    const Mat& md = S.mats[c.mat];
    const int ei = md.elems.size() > 1 ? selectBremTarget(E, le, rng.flat(), false) : 0;
    const int Z = md.elems[ei];
    const double dZ = (double)Z;
    const Elem& el = S.elem[Z < 120 ? Z : 120];
    const double dens = kMigdal * md.elDensity;
    const double lpmE = kLPM * md.radLength;
    const double lpmLim = std::sqrt(dens) * lpmE;
    const double pte = E + kMec2;
    const double dcor = dens * pte * pte;
    const bool lpm = pte > lpmLim;
    const double zf1 = el.zFactor1;
    const double zf2 = (1. + 1. / dZ) / 12.;
    const double fmax = zf1 + zf2;
    const double xmin = vlog(gcut * gcut + dcor);
    const double xr = vlog(E * E + dcor) - xmin;
    double r[2], k, fv;
    do {
      rng.flatArray(2, r);
      k = std::sqrt(dmax(vexp(xmin + r[0] * xr) - dcor, 0.0));
      const double y = k / pte;
      const double omy = 1. - y;
      const double d0 = 0.25 * y * y;
      if (lpm) {
        double xiS, gS, phiS;
        lpmFunctions(xiS, gS, phiS, k, pte, lpmE, el.Z23, el.ilVarS1, el.ilVarS1Cond, dcor, 1.0);
        const double t1 = xiS * (d0 * gS + (omy + 2.0 * d0) * phiS);
        fv = t1 * zf1 + omy * zf2;
      } else {
        const double d1 = omy + 3. * d0;
        if (Z < 5) {
          fv = d1 * zf1 + omy * zf2;
        } else {
          const double d2 = y / (pte - k);
          const double gam = d2 * 100. * kMec2 / el.Z13;
          const double eps = gam / el.Z13;
          const double g2 = gam * gam;
          const double phi1 = 16.863 - 2.0 * vlog(1.0 + 0.311877 * g2) + 2.4 * vexp(-0.9 * gam) + 1.6 * vexp(-1.5 * gam);
          const double phi2 = 2.0 / (3.0 + 19.5 * gam + 18.0 * g2);
          const double e2 = eps * eps;
          const double psi1 = 24.34 - 2.0 * vlog(1.0 + 13.111641 * e2) + 2.8 * vexp(-8.0 * eps) + 1.2 * vexp(-29.2 * eps);
          const double psi2 = 2.0 / (3.0 + 120.0 * eps + 1200.0 * e2);
          const double lz = el.logZ;
          const double Fz = lz / 3. + el.coulomb;
          const double iz = 1. / dZ;
          fv = d1 * ((0.25 * phi1 - Fz) + (0.25 * psi1 - 2. * lz / 3.) * iz) + 0.125 * omy * (phi2 + psi2 * iz);
        }
      }
      fv = dmax(0.0, fv);
    } while (fv < fmax * r[1]);
    return k;
  }

  // G4HepEmInteractionUtils.icc:10-76
  double tsaiCost(double E) {
    const double umax = 2.0 * (1.0 + E * kInvMec2);
    double r[3], u;
    do {
      rng.flatArray(3, r);
      const double uu = -vlog(r[0] * r[1]);
      u = 0.25 > r[2] ? uu * 1.6 : uu * 0.533333333;
    } while (u > umax);
    return 1.0 - 2.0 * u * u / (umax * umax);
  }

  static void lpmFunctions(double& xiS, double& gS, double& phiS, double eg, double et, double elpm, double z23,
                           double ilS1, double ilS1c, double dcor, double times) {
    static const double kFuncLPM[] = {
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
      9.9856E-01, 9.9926E-01};
    const double sqrt2 = 1.414213562373095;
    const double red = eg / et;
    const double sP = std::sqrt(0.125 * red * elpm / (times * (1.0 - red) * et));
    const double s1 = z23 / (184.15 * 184.15);
    const double cond = sqrt2 * s1;
    double xiSP = 2.0;
    if (sP > 1.0) {
      xiSP = 1.0;
    } else if (sP > cond) {
      const double h = vlog(sP) * ilS1c;
      xiSP = 1.0 + h - 0.08 * (1.0 - h) * h * (2.0 - h) * ilS1c;
    }
    xiS = xiSP;
    const double s = sP / std::sqrt(xiSP);
    double sh = s;
    if (dcor != 0.0) {
      sh *= (1.0 + dcor / (eg * eg));
      xiS = 2.0;
      if (sh > 1.0) xiS = 1.0;
      else if (sh > s1) xiS = 1.0 + vlog(sh) * ilS1;
    }
    if (sh < 2.0) {
      double val = sh * 20.0;
      int il = (int)val;
      val -= il;
      il *= 2;
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

  // ---- positron annihilation (G4HepEmPositronInteractionAnnihilation.icc:15-119) -------
  void annihilateAtRest() {
    const double cost = 2. * rng.flat() - 1.;
    const double sint = std::sqrt((1. - cost) * (1. + cost));
    const double phi = k2Pi * rng.flat();
    Secondary& g1 = addSec(2);
    Secondary& g2 = addSec(2);
    g1.dir[0] = sint * std::cos(phi);
    g1.dir[1] = sint * std::sin(phi);
    g1.dir[2] = cost;
    g2.dir[0] = -g1.dir[0]; g2.dir[1] = -g1.dir[1]; g2.dir[2] = -g1.dir[2];
    g1.e = kMec2;
    g2.e = kMec2;
  }

  void annihilateInFlight() {
    const double E = t.e;
    Secondary& g1 = addSec(2);
    Secondary& g2 = addSec(2);
    const double tau = E * kInvMec2;
    const double gam = tau + 1.0;
    const double tau2 = tau + 2.0;
    const double sq = std::sqrt(tau / tau2) * 0.5;
    const double emin = 0.5 - sq, emax = 0.5 + sq;
    const double eq = emax / emin;
    const double tau4 = tau2 * tau2;
    double eps, rf, r[2];
    do {
      rng.flatArray(2, r);
      eps = emin * vexp(vlog(eq) * r[0]);
      rf = 1. - eps + (2. * gam * eps - 1.) / (eps * tau4);
    } while (rf < r[1]);
    const double sqg = std::sqrt(tau * tau2);
    const double cost = dmin(1., dmax(-1., (eps * tau2 - 1.) / (eps * sqg)));
    const double sint = std::sqrt((1. + cost) * (1. - cost));
    const double phi = k2Pi * rng.flat();
    const double initE = E + 2. * kMec2;
    const double e1 = eps * initE;
    g1.e = e1;
    g1.dir[0] = sint * std::cos(phi);
    g1.dir[1] = sint * std::sin(phi);
    g1.dir[2] = cost;
    rotate(g1.dir, t.dir);
    g2.e = initE - e1;
    const double ip = std::sqrt(E * (E + 2 * kMec2));
    const double px = ip * t.dir[0] - g1.dir[0] * e1;
    const double py = ip * t.dir[1] - g1.dir[1] * e1;
    const double pz = ip * t.dir[2] - g1.dir[2] * e1;
    const double nrm = 1.0 / std::sqrt(px * px + py * py + pz * pz);
    g2.dir[0] = px * nrm; g2.dir[1] = py * nrm; g2.dir[2] = pz * nrm;
    t.setE(0.0);
  }

  // ---- gamma (G4HepEmGammaManager.icc:27-219) -----------------------------------------
  double macXSPE(int imat, double e) {
    const Mat& m = S.mats[imat];
    int iv = 0;
    const int n = (int)m.sandiaE.size();
    if (e >= m.sandiaE[0]) {
      for (int i = n - 1; i >= 0; --i)
        if (e >= m.sandiaE[i]) { iv = i; break; }
    }
    const double* c = &m.sandiaC[4 * iv];
    const double inv = 1 / e;
    return inv * (c[0] + inv * (c[1] + inv * (c[2] + inv * c[3])));
  }

  double gammaTotalXS() {
    const double e = t.e, le = t.logE();
    const int imat = couple().mat;
    const Gamma& g = S.gm;
    if (e > g.eMax1) {
      const int st = imat * g.dataPerMat + g.nData0 + g.nData1;
      return spline_log_9(g.nE2, &g.mx[st], e, le, g.logEMin2, g.ild2, 1);
    }
    if (e > g.eMax0) {
      const int st = imat * g.dataPerMat + g.nData0;
      const double* d = &g.mx[st];
      const int i3 = 3 * bin_of(le, g.logEMin1, g.ild1, g.nE1);
      const int j3 = i3 + 3;
      const double dl = d[j3] - d[i3];
      const double b = dmax(0., dmin(1., (e - d[i3]) / dl));
      double res[2];
      for (int i = 1; i < 3; ++i) res[i - 1] = dmax(0.0, d[i3 + i] + b * (d[j3 + i] - d[i3 + i]));
      t.peXS = res[1];
      return res[0];
    }
    const int st = imat * g.dataPerMat;
    const double* d = &g.mx[st];
    const int i2 = 2 * bin_of(le, g.logEMin0, g.ild0, g.nE0);
    const double comp = linear(d[i2], d[i2 + 2], d[i2 + 1], d[i2 + 3], e);
    const double pe = dmax(0.0, macXSPE(imat, e));
    t.peXS = pe;
    return comp + pe;
  }

  void gammaHowFar() {
    if (t.nia[0] <= 0.0) t.nia[0] = -vlog(rng.flat());
    const double tot = gammaTotalXS();
    const double mfp = tot > 0. ? 1. / tot : kLarge;
    t.mfp[0] = mfp;
    t.gstep = mfp * t.nia[0];
  }

  void gammaSelect() {
    const double u = rng.flat();
    const double e = t.e;
    const double tmfp = t.mfp[0];
    t.nia[0] = -1.0;
    const Gamma& g = S.gm;
    if (e > g.eMax1) {
      const double le = t.logE();
      const int imat = couple().mat;
      const int st = imat * g.dataPerMat + g.nData0 + g.nData1;
      double mx = 0.0, cp = 0.0;
      int pid = 2;
      // the reference evaluates a fifth column after the PE one when the
      // cumulative is still below u; its value is not used (winner 3)
      do {
        mx = pid < 5 ? spline_log_9(g.nE2, &g.mx[st], e, le, g.logEMin2, g.ild2, pid) : 0.0;
        cp += mx * tmfp;
        ++pid;
      } while (pid < 6 && u > cp);
      t.winner = pid - 3;
      t.peXS = mx;
      return;
    }
    t.winner = (u > tmfp * t.peXS) ? 1 : 2;
  }

  void gammaPerform() {
    // UpdateNumIALeft
    t.nia[0] -= t.gstep / t.mfp[0];
    t.edep = 0.0;
    if (t.onBoundary) return;
    const int ip = t.winner;
    t.nia[ip] = -1.0;
    switch (ip) {
      case 0: conversion(); break;
      case 1: compton(); break;
      case 2: photoelectric(); break;
      default: break;
    }
    const double fe = t.e;
    if (fe > 0.0 && fe <= S.pars.gammaTrackingCut) {
      t.setE(0.0);
      t.edep += fe;
    }
  }

  // ---- conversion (G4HepEmGammaInteractionConversion.icc:19-274) ------------------------
  int convTarget(int imat, double e, double le, double u) {
    const Gamma& g = S.gm;
    const double* D = &g.conv[g.convStart[imat]];
    const int nd = g.convN;
    const int ne = (int)D[0];
    const double* x = g.convGrid.data();
    const double xv = dmax(x[0], dmin(x[nd - 1], e));
    const int ie = (int)dmax(0.0, dmin((le - g.convLogMin) * g.convILD, nd - 2.0));
    const double x1 = x[ie], x2 = x[ie + 1];
    const double b = dmax(0., dmin(1., (xv - x1) / (x2 - x1)));
    const int i0 = ie * (ne - 1) + 1;
    const int i1 = i0 + (ne - 1);
    int k = 0;
    while (k < ne - 1 && u > D[i0 + k] + b * (D[i1 + k] - D[i0 + k])) ++k;
    return k;
  }

  static double screen1(double d) { return d > 1.4 ? 42.038 - 8.29 * vlog(d + 0.958) : 42.184 - d * (7.444 - 1.623 * d); }
  static double screen2(double d) { return d > 1.4 ? 42.038 - 8.29 * vlog(d + 0.958) : 41.326 - d * (5.848 - 0.902 * d); }
  static void phi12(double d, double& p1, double& p2) {
    if (d > 1.4) {
      p1 = 21.0190 - 4.145 * vlog(d + 0.958);
      p2 = p1;
    } else {
      p1 = 20.806 - d * (3.190 - 0.5710 * d);
      p2 = 20.234 - d * (2.126 - 0.0903 * d);
    }
  }

  void conversion() {
    const double E = t.e;
    if (E < 2. * kMec2) return;
    const double le = t.logE();
    const int imat = couple().mat;
    const Mat& md = S.mats[imat];
    const int ei = md.elems.size() > 1 ? convTarget(imat, E, le, rng.flat()) : 0;
    const int Z = md.elems[ei];
    const double lpmE = kLPM * md.radLength;
    const Elem& el = S.elem[Z < 120 ? Z : 120];
    const double eps0 = kMec2 / E;
    double eps = 0.0;
    if (E < 2.0) {
      eps = eps0 + (0.5 - eps0) * rng.flat();
    } else {
      const double df = eps0 * 136. / el.Z13;
      const double dmin_ = 4. * df;
      const double dmax_ = E < 50.0 ? el.deltaMaxLow : el.deltaMaxHigh;
      const double lz13 = 0.333333 * el.logZ;
      const double FZ = E < 50.0 ? 8. * lz13 : 8. * (lz13 + el.coulomb);
      const double epsp = 0.5 - 0.5 * std::sqrt(1. - dmin_ / dmax_);
      const double epsMin = dmax(eps0, epsp);
      const double epsRange = 0.5 - epsMin;
      double F10, F20;
      if (dmin_ > 1.4) {
        F10 = 42.038 - 8.29 * vlog(dmin_ + 0.958);
        F20 = F10;
      } else {
        F10 = 42.184 - dmin_ * (7.444 - 1.623 * dmin_);
        F20 = 41.326 - dmin_ * (5.848 - 0.902 * dmin_);
      }
      F10 -= FZ;
      F20 -= FZ;
      const double N1 = dmax(F10 * epsRange * epsRange, 0.);
      const double N2 = dmax(1.5 * F20, 0.);
      const double cond = N1 / (N1 + N2);
      const double iF10 = 1. / F10, iF20 = 1. / F20;
      double r[3], gr;
      if (E < 100000.0) {
        do {
          rng.flatArray(3, r);
          if (cond > r[0]) {
            eps = 0.5 - epsRange * std::pow(r[1], 1. / 3.);
            gr = (screen1(df / (eps * (1. - eps))) - FZ) * iF10;
          } else {
            eps = epsMin + epsRange * r[1];
            gr = (screen2(df / (eps * (1. - eps))) - FZ) * iF20;
          }
        } while (gr < r[2]);
      } else {
        do {
          rng.flatArray(3, r);
          double xiS, gS, phiS, p1, p2;
          if (cond > r[0]) {
            eps = 0.5 - epsRange * std::pow(r[1], 1. / 3.);
            phi12(df / (eps * (1. - eps)), p1, p2);
            lpmFunctions(xiS, gS, phiS, E, eps * E, lpmE, el.Z23, el.ilVarS1, el.ilVarS1Cond, 0.0, -1.0);
            gr = xiS * ((2. * phiS + gS) * p1 - gS * p2 - phiS * FZ) * iF10;
          } else {
            eps = epsMin + epsRange * r[1];
            phi12(df / (eps * (1. - eps)), p1, p2);
            lpmFunctions(xiS, gS, phiS, E, eps * E, lpmE, el.Z23, el.ilVarS1, el.ilVarS1Cond, 0.0, -1.0);
            gr = xiS * ((phiS + 0.5 * gS) * p1 + 0.5 * gS * p2 - 0.5 * (gS + phiS) * FZ) * iF20;
          }
        } while (gr < r[2]);
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
    const double eK = dmax(0., eT - kMec2);
    const double pK = dmax(0., pT - kMec2);
    Secondary& se = addSec(0);
    Secondary& sp = addSec(1);
    const double phi = k2Pi * rng.flat();
    const double cp = std::cos(phi), sp_ = std::sin(phi);
    const double ce = tsaiCost(eK);
    const double st = std::sqrt((1.0 - ce) * (1.0 + ce));
    se.dir[0] = st * cp; se.dir[1] = st * sp_; se.dir[2] = ce;
    rotate(se.dir, t.dir);
    const double cpo = tsaiCost(pK);
    const double stp = std::sqrt((1.0 - cpo) * (1.0 + cpo));
    sp.dir[0] = -stp * cp; sp.dir[1] = -stp * sp_; sp.dir[2] = cpo;
    rotate(sp.dir, t.dir);
    se.e = eK;
    sp.e = pK;
    t.setE(0.0);
  }

  // ---- Compton (G4HepEmGammaInteractionCompton.icc:17-103) ------------------------------
  void compton() {
    const double E = t.e;
    const double thr = 0.0001;
    if (E < thr) return;
    const double org[3] = {t.dir[0], t.dir[1], t.dir[2]};
    const double kappa = E * kInvMec2;
    const double eps0 = 1. / (1. + 2. * kappa);
    const double eps02 = eps0 * eps0;
    const double al1 = -vlog(eps0);
    const double al2 = al1 + 0.5 * (1. - eps02);
    double eps, eps2, gf, omc, s2, r[3];
    do {
      rng.flatArray(3, r);
      if (al1 > al2 * r[0]) {
        eps = vexp(-al1 * r[1]);
        eps2 = eps * eps;
      } else {
        eps2 = eps02 + (1. - eps02) * r[1];
        eps = std::sqrt(eps2);
      }
      omc = (1. - eps) / (eps * kappa);
      s2 = omc * (2. - omc);
      gf = 1. - eps * s2 / (1. + eps2);
    } while (gf < r[2]);
    const double cost = 1.0 - omc;
    const double sint = std::sqrt(dmax(0., s2));
    const double phi = k2Pi * rng.flat();
    t.dir[0] = sint * std::cos(phi);
    t.dir[1] = sint * std::sin(phi);
    t.dir[2] = cost;
    rotate(t.dir, org);
    const double post = E * eps;
    const double se = E - post;
    double dep = 0.0;
    if (se > thr) {
      Secondary& s = addSec(0);
      s.dir[0] = E * org[0] - post * t.dir[0];
      s.dir[1] = E * org[1] - post * t.dir[1];
      s.dir[2] = E * org[2] - post * t.dir[2];
      const double nrm = 1.0 / std::sqrt(s.dir[0] * s.dir[0] + s.dir[1] * s.dir[1] + s.dir[2] * s.dir[2]);
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

  // ---- photoelectric (G4HepEmGammaInteractionPhotoelectric.icc:13-121) -------------------
  void photoelectric() {
    const double E = t.e;
    const int imat = couple().mat;
    const Mat& md = S.mats[imat];
    int ie = 0;
    if (md.elems.size() > 1) {
      const double x = rng.flat() * t.peXS;
      double sum = 0;
      const double inv = 1 / E;
      for (int i = 0; i < (int)md.elems.size(); i++) {
        const Elem& el = S.elem[md.elems[i]];
        int iv = 0;
        if (E >= el.sandiaE[0]) {
          for (int j = (int)el.sandiaE.size() - 1; j >= 0; j--)
            if (E >= el.sandiaE[j]) { iv = j; break; }
        }
        const double* c = &el.sandiaC[4 * iv];
        sum += md.natoms[i] * inv * (c[0] + inv * (c[1] + inv * (c[2] + inv * c[3])));
        if (x <= sum) { ie = i; break; }
      }
    }
    const double bind = S.elem[md.elems[ie]].kShell;
    const double pe = E - bind;
    if (pe > 0.000001) {
      Secondary& s = addSec(0);
      const double tau = pe * kInvMec2;
      const double gamma = 1.0 + tau;
      const double beta = std::sqrt(tau * (tau + 2.0)) / gamma;
      const double ac = (1.0 - beta) / beta;
      const double a1 = 0.5 * beta * gamma * tau * (gamma - 2.0);
      const double a2 = ac + 2.0;
      const double gtmax = 2.0 * (a1 + 1.0 / ac);
      double ts, gtr, r[2];
      do {
        rng.flatArray(2, r);
        ts = 2.0 * ac * (2.0 * r[0] + a2 * std::sqrt(r[0])) / (a2 * a2 - 4.0 * r[0]);
        gtr = (2.0 - ts) * (a1 + 1.0 / (ac + ts));
      } while (r[1] * gtmax > gtr);
      const double ct = 1.0 - ts;
      const double st = std::sqrt(ts * (2.0 - ts));
      const double phi = k2Pi * rng.flat();
      s.dir[0] = st * std::cos(phi);
      s.dir[1] = st * std::sin(phi);
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

// Transport between HowFar and Perform (the caller's geometry): the
// geometrical step made is gfrac[i] times the proposed one, the track leaves
// with direction nd*[i] and post-step boundary status post[i]; proposed[i]
// receives HowFar's geometrical step.  Null: no geometry (the step is the
// proposed one, direction and boundary status unchanged).
struct Geo {
  const double *gfrac, *ndx, *ndy, *ndz;
  const uint8_t* post;
  double* proposed;
};

int step_range(const State& S, int64_t b, int64_t e, const hepem_track_state* in, hepem_track_state* out,
               const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res, const Geo* geo = nullptr) {
  for (int64_t i = b; i < e; ++i) {
    Rng rng{uniforms + i * (int64_t)nu, nu, in->rng_cursor[i], seed, in->id[i], false,
            in->gauss_valid[i] != 0, in->gauss_value[i]};
    Step s(S, rng);
    Track& t = s.t;
    const int type = in->type[i];
    t.setE(in->ekin[i]);
    t.dir[0] = in->dir_x[i]; t.dir[1] = in->dir_y[i]; t.dir[2] = in->dir_z[i];
    t.imc = in->imc[i];
    t.id = in->id[i];
    t.onBoundary = in->on_boundary[i] != 0;
    t.nia[0] = in->nia0[i];
    double pstep;
    if (type == 2) {
      t.charge = 0.0;
      s.gammaHowFar();
      if (geo) {
        // G4HepEmProcess.cc:167-197: the step made, the direction after
        // transport, and the post-step boundary status
        geo->proposed[i] = t.gstep;
        t.gstep = geo->gfrac[i] * t.gstep;
        t.dir[0] = geo->ndx[i]; t.dir[1] = geo->ndy[i]; t.dir[2] = geo->ndz[i];
        t.onBoundary = geo->post[i] != 0;
      }
      if (t.onBoundary) {
        t.nia[0] -= t.gstep / t.mfp[0];
      } else {
        s.gammaSelect();
        s.gammaPerform();
      }
      pstep = t.gstep;
    } else {
      t.charge = type == 0 ? -1.0 : 1.0;
      t.nia[1] = in->nia1[i]; t.nia[2] = in->nia2[i]; t.nia[3] = in->nia3[i];
      t.safety = in->safety[i];
      t.msc.initRange = in->msc_init_range[i];
      t.msc.dynFactor = in->msc_dyn_factor[i];
      t.msc.tlimitMin = in->msc_tlimit_min[i];
      t.msc.firstStep = in->msc_first_step[i] != 0;
      s.elHowFar();
      if (geo) {
        geo->proposed[i] = t.gstep;
        t.gstep = geo->gfrac[i] * t.gstep;
        t.dir[0] = geo->ndx[i]; t.dir[1] = geo->ndy[i]; t.dir[2] = geo->ndz[i];
        t.onBoundary = geo->post[i] != 0;
      }
      s.elPerform();
      pstep = t.pstep;
    }
    if (s.nsec > 2) return -1;
    out->ekin[i] = t.e;
    out->dir_x[i] = t.dir[0]; out->dir_y[i] = t.dir[1]; out->dir_z[i] = t.dir[2];
    out->nia0[i] = t.nia[0];
    if (type != 2) {
      out->nia1[i] = t.nia[1]; out->nia2[i] = t.nia[2]; out->nia3[i] = t.nia[3];
      out->msc_init_range[i] = t.msc.initRange;
      out->msc_dyn_factor[i] = t.msc.dynFactor;
      out->msc_tlimit_min[i] = t.msc.tlimitMin;
      out->msc_first_step[i] = t.msc.firstStep ? 1 : 0;
    } else if (out != in) {
      out->nia1[i] = in->nia1[i]; out->nia2[i] = in->nia2[i]; out->nia3[i] = in->nia3[i];
      out->msc_init_range[i] = in->msc_init_range[i];
      out->msc_dyn_factor[i] = in->msc_dyn_factor[i];
      out->msc_tlimit_min[i] = in->msc_tlimit_min[i];
      out->msc_first_step[i] = in->msc_first_step[i];
    }
    out->gauss_valid[i] = rng.gaussValid ? 1 : 0;
    out->gauss_value[i] = rng.gaussValue;
    out->rng_cursor[i] = rng.cursor;
    if (out != in) {
      out->type[i] = in->type[i];
      out->imc[i] = in->imc[i];
      out->id[i] = in->id[i];
      out->safety[i] = in->safety[i];
      out->on_boundary[i] = in->on_boundary[i];
    }
    if (geo) out->on_boundary[i] = geo->post[i];
    res->edep[i] = t.edep;
    res->gstep[i] = t.gstep;
    res->pstep[i] = pstep;
    res->winner[i] = (int8_t)t.winner;
    const bool mscOut = type != 2;
    res->disp_x[i] = mscOut ? t.msc.disp[0] : 0.0;
    res->disp_y[i] = mscOut ? t.msc.disp[1] : 0.0;
    res->disp_z[i] = mscOut ? t.msc.disp[2] : 0.0;
    res->flags[i] = rng.overflow ? 1 : 0;
    res->n_sec[i] = (int8_t)s.nsec;
    for (int k = 0; k < s.nsec; ++k) {
      res->sec_type[2 * i + k] = (int8_t)s.sec[k].type;
      res->sec_ekin[2 * i + k] = s.sec[k].e;
      res->sec_dir_x[2 * i + k] = s.sec[k].dir[0];
      res->sec_dir_y[2 * i + k] = s.sec[k].dir[1];
      res->sec_dir_z[2 * i + k] = s.sec[k].dir[2];
    }
  }
  return 0;
}

// ---- Woodcock gamma tracking in a layered box (G4HepEmWoodcockHelper.cc:146-299) ------
// The reference helper navigates a Geant4 geometry; here the geometry is a box
// of slabs along z and the helper's loop is restated over it, with the
// track's own uniform stream (G4UniformRand in the reference).
struct BoxGeo {
  double hx, hy;
  int nl, wdt;
  const double* zb;
  const int32_t* limc;
  double elim;
};

double box_dist_out(const BoxGeo& b, const double* p, const double* v) {
  double d = 1.0e300;
  if (v[0] > 0.) d = dmin(d, (b.hx - p[0]) / v[0]);
  else if (v[0] < 0.) d = dmin(d, (-b.hx - p[0]) / v[0]);
  if (v[1] > 0.) d = dmin(d, (b.hy - p[1]) / v[1]);
  else if (v[1] < 0.) d = dmin(d, (-b.hy - p[1]) / v[1]);
  if (v[2] > 0.) d = dmin(d, (b.zb[b.nl] - p[2]) / v[2]);
  else if (v[2] < 0.) d = dmin(d, (b.zb[0] - p[2]) / v[2]);
  return dmax(d, 0.0);
}

int box_layer(const BoxGeo& b, double z) {
  if (!(z > b.zb[0])) return 0;
  if (!(z < b.zb[b.nl])) return b.nl - 1;
  int lo = 0, hi = b.nl;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (z < b.zb[mid]) hi = mid; else lo = mid;
  }
  return lo;
}

void woodcock_one(const State& S, const BoxGeo& b, int64_t i, const hepem_track_state* in, hepem_track_state* out,
                  double* px, double* py, double* pz, const double* uniforms, int32_t nu, uint64_t seed,
                  hepem_step_out* res, uint8_t* reached) {
  const double kDblMax = 1.7976931348623157e308;
  Rng rng{uniforms + i * (int64_t)nu, nu, in->rng_cursor[i], seed, in->id[i], false, in->gauss_valid[i] != 0,
          in->gauss_value[i]};
  Step s(S, rng);
  Track& t = s.t;
  const int type = in->type[i];
  t.setE(in->ekin[i]);
  t.dir[0] = in->dir_x[i]; t.dir[1] = in->dir_y[i]; t.dir[2] = in->dir_z[i];
  t.imc = in->imc[i];
  t.id = in->id[i];
  t.onBoundary = in->on_boundary[i] != 0;
  t.nia[0] = in->nia0[i];
  t.charge = 0.0;
  double p[3] = {px[i], py[i], pz[i]};
  bool boundary = false;
  const bool bad = type != 2 || !(t.imc >= 0 && t.imc < (int)S.couples.size()) || !(t.e > 0.0) || !(t.e < 1.0e300);
  uint8_t flags = 0;
  if (bad) {
    flags = 4;
  } else if (t.e > b.elim) {
    double dist = dmax(box_dist_out(b, p, t.dir) - 1.0E-3, 0.0);
    t.imc = b.wdt;
    const double wdtMX = s.gammaTotalXS();
    const double wdtMFP = wdtMX > 0.0 ? 1.0 / wdtMX : kDblMax;
    const double wdtPE = t.peXS;
    const int wdtMat = S.couples[b.wdt].mat;
    double mx = 0.0, step = 0.0;
    int prev = -1, it = 0;
    bool stop = false;
    while (!stop) {
      const double ps = wdtMFP < kDblMax ? -vlog(rng.flat()) * wdtMFP : kDblMax;
      if (dist < ps) {
        step += dist;
        boundary = true;
        stop = true;
      } else {
        step += ps;
        dist -= ps;
        const int imc = b.limc[box_layer(b, p[2] + step * t.dir[2])];
        if (S.couples[imc].mat != wdtMat) {
          if (imc != prev) {
            prev = imc;
            t.imc = imc;
            mx = s.gammaTotalXS();
          }
          stop = mx * wdtMFP > rng.flat();
          if (stop) t.mfp[0] = mx > 0.0 ? 1.0 / mx : kDblMax;
        } else {
          stop = true;
          t.imc = b.wdt;
          t.mfp[0] = wdtMFP;
          t.peXS = wdtPE;
        }
      }
      if (++it >= (1 << 16)) {
        flags |= 2;
        boundary = true;
        break;
      }
    }
    for (int k = 0; k < 3; ++k) p[k] += step * t.dir[k];
    t.gstep = step;
    t.nia[0] = -1.0;
    t.winner = -1;
    if (!boundary) {
      s.gammaSelect();
      t.edep = 0.0;
      if (t.winner == 0) s.conversion();
      if (t.winner == 1) s.compton();
      if (t.winner == 2) s.photoelectric();
      const double fe = t.e;
      if (fe > 0.0 && fe <= S.pars.gammaTrackingCut) {
        t.setE(0.0);
        t.edep += fe;
      }
    }
    t.imc = b.limc[box_layer(b, p[2])];
  } else {
    t.imc = b.limc[box_layer(b, p[2])];
    s.gammaHowFar();
    s.gammaSelect();
    s.gammaPerform();
    for (int k = 0; k < 3; ++k) p[k] += t.gstep * t.dir[k];
    t.imc = b.limc[box_layer(b, p[2])];
  }
  px[i] = p[0]; py[i] = p[1]; pz[i] = p[2];
  out->ekin[i] = t.e;
  out->dir_x[i] = t.dir[0]; out->dir_y[i] = t.dir[1]; out->dir_z[i] = t.dir[2];
  out->nia0[i] = t.nia[0];
  if (out != in) {
    out->nia1[i] = in->nia1[i]; out->nia2[i] = in->nia2[i]; out->nia3[i] = in->nia3[i];
    out->msc_init_range[i] = in->msc_init_range[i];
    out->msc_dyn_factor[i] = in->msc_dyn_factor[i];
    out->msc_tlimit_min[i] = in->msc_tlimit_min[i];
    out->msc_first_step[i] = in->msc_first_step[i];
    out->type[i] = in->type[i];
    out->id[i] = in->id[i];
    out->safety[i] = in->safety[i];
    out->on_boundary[i] = in->on_boundary[i];
  }
  out->imc[i] = bad ? in->imc[i] : t.imc;
  out->gauss_valid[i] = rng.gaussValid ? 1 : 0;
  out->gauss_value[i] = rng.gaussValue;
  out->rng_cursor[i] = rng.cursor;
  res->edep[i] = t.edep;
  res->gstep[i] = t.gstep;
  res->pstep[i] = t.gstep;
  res->winner[i] = (int8_t)t.winner;
  res->disp_x[i] = res->disp_y[i] = res->disp_z[i] = 0.0;
  res->flags[i] = (uint8_t)(flags | (rng.overflow ? 1 : 0));
  res->n_sec[i] = (int8_t)(s.nsec > 2 ? 2 : s.nsec);
  for (int k = 0; k < s.nsec && k < 2; ++k) {
    res->sec_type[2 * i + k] = (int8_t)s.sec[k].type;
    res->sec_ekin[2 * i + k] = s.sec[k].e;
    res->sec_dir_x[2 * i + k] = s.sec[k].dir[0];
    res->sec_dir_y[2 * i + k] = s.sec[k].dir[1];
    res->sec_dir_z[2 * i + k] = s.sec[k].dir[2];
  }
  if (reached) reached[i] = boundary ? 1 : 0;
}

}  // namespace
}  // namespace port

extern "C" {

int port_woodcock_gamma(void* st, int64_t n, const hepem_track_state* in, hepem_track_state* out, double* px,
                        double* py, double* pz, double hx, double hy, int nl, int wdt, const double* zb,
                        const int32_t* limc, double elim, const double* u, int32_t nu, uint64_t seed,
                        hepem_step_out* res, uint8_t* reached) {
  const port::State& S = *static_cast<port::State*>(st);
  port::BoxGeo b{hx, hy, nl, wdt, zb, limc, elim};
  for (int64_t i = 0; i < n; ++i) port::woodcock_one(S, b, i, in, out, px, py, pz, u, nu, seed, res, reached);
  return 0;
}


void* port_load_state(const char* path) {
  const char* err = nullptr;
  return port::load_state(path, &err);
}

void port_free_state(void* s) { delete static_cast<port::State*>(s); }

double port_philox_uniform(uint64_t seed, int32_t id, int32_t k) { return oracle_philox_uniform(seed, id, k); }

void port_fill_uniforms(int64_t n, const int32_t* id, int32_t nu, uint64_t seed, double* u) {
  for (int64_t i = 0; i < n; ++i)
    for (int32_t k = 0; k < nu; ++k) u[i * nu + k] = oracle_philox_uniform(seed, id[i], k);
}

void port_vdt_log(int64_t n, const double* x, double* y) { for (int64_t i = 0; i < n; ++i) y[i] = port::vlog(x[i]); }
void port_vdt_exp(int64_t n, const double* x, double* y) { for (int64_t i = 0; i < n; ++i) y[i] = port::vexp(x[i]); }

void port_electron_lookup(void* st, int64_t n, int is_pos, const double* ekin, const int32_t* imc, double* xi,
                          double* xb, double* dedx, double* range, double* invr) {
  const port::State& S = *static_cast<port::State*>(st);
  const port::ElData& d = S.el[is_pos ? 1 : 0];
  using St = port::Step;
  for (int64_t i = 0; i < n; ++i) {
    const double e = ekin[i], le = port::vlog(e);
    xi[i] = St::restMacXS(d, imc[i], e, le, true);
    xb[i] = St::restMacXS(d, imc[i], e, le, false);
    dedx[i] = St::restDEDX(d, imc[i], e, le);
    range[i] = St::restRange(d, imc[i], e, le);
    invr[i] = St::invRange(d, imc[i], 0.5 * range[i]);
  }
}

// Step-limit cross sections of HowFarToDiscreteInteraction and the transport
// mean free path (G4HepEmElectronManager.icc:534-599), per (E, couple).
void port_electron_xs_stepping(void* st, int64_t n, int is_pos, const double* ekin, const int32_t* imc,
                               double* xi, double* xb, double* xa, double* xn, double* tr) {
  const port::State& S = *static_cast<port::State*>(st);
  const port::ElData& d = S.el[is_pos ? 1 : 0];
  using St = port::Step;
  for (int64_t i = 0; i < n; ++i) {
    const double e = ekin[i], le = port::vlog(e);
    const int imat = S.couples[imc[i]].mat;
    xi[i] = St::restMacXSStepping(d, imc[i], e, le, true);
    xb[i] = St::restMacXSStepping(d, imc[i], e, le, false);
    xa[i] = is_pos ? St::annihXS(0.8 * e, S.mats[imat].elDensity) : 0.0;
    xn[i] = St::nucMacXS(d, imat, e, le);
    tr[i] = St::transportMFP(d, imat, e, le);
  }
}

// Target element of Seltzer-Berger (is_sb) or relativistic brem for a given
// uniform (G4HepEmElectronInteractionBrem.icc SelectTargetAtom); 0 for
// single-element materials, where the reference draws nothing.
void port_brem_select_target(void* st, int64_t n, int is_pos, int is_sb, const double* ekin, const int32_t* imc,
                             const double* urnd, int32_t* elem) {
  const port::State& S = *static_cast<port::State*>(st);
  for (int64_t i = 0; i < n; ++i) {
    if (S.mats[S.couples[imc[i]].mat].elems.size() < 2) { elem[i] = 0; continue; }
    port::Rng rng{&urnd[i], 1, 0, 0, 0, false, false, 0.0};
    port::Step P(S, rng);
    P.t.imc = imc[i];
    P.t.charge = is_pos ? 1.0 : -1.0;
    elem[i] = P.selectBremTarget(ekin[i], port::vlog(ekin[i]), urnd[i], is_sb != 0);
  }
}

// Gamma total macroscopic cross section and the interaction chosen with a
// given uniform (G4HepEmGammaManager.icc:108-219, the pair the reference's
// gamma cross-section test checks); PE cross section when the winner is PE.
void port_gamma_xs(void* st, int64_t n, const double* ekin, const int32_t* imc, const double* urnd,
                   double* xs_tot, double* xs_pe, int32_t* winner) {
  const port::State& S = *static_cast<port::State*>(st);
  for (int64_t i = 0; i < n; ++i) {
    port::Rng rng{&urnd[i], 1, 0, 0, 0, false, false, 0.0};
    port::Step P(S, rng);
    P.t.imc = imc[i];
    P.t.setE(ekin[i]);
    const double tot = P.gammaTotalXS();
    xs_tot[i] = tot;
    P.t.mfp[0] = tot > 0. ? 1. / tot : port::kLarge;
    P.gammaSelect();
    winner[i] = P.t.winner;
    xs_pe[i] = P.t.winner == 2 ? P.t.peXS : 0.0;
  }
}

// Target element of gamma conversion for a given uniform
// (G4HepEmGammaInteractionConversion.icc SelectTargetAtom).
void port_conv_select_target(void* st, int64_t n, const double* ekin, const int32_t* imc, const double* urnd,
                             int32_t* elem) {
  const port::State& S = *static_cast<port::State*>(st);
  for (int64_t i = 0; i < n; ++i) {
    const int imat = S.couples[imc[i]].mat;
    if (S.mats[imat].elems.size() < 2) { elem[i] = 0; continue; }
    port::Rng rng{&urnd[i], 1, 0, 0, 0, false, false, 0.0};
    port::Step P(S, rng);
    elem[i] = P.convTarget(imat, ekin[i], port::vlog(ekin[i]), urnd[i]);
  }
}

int port_step(void* st, int64_t n, const hepem_track_state* in, hepem_track_state* out, const double* u,
              int32_t nu, uint64_t seed, hepem_step_out* res) {
  return port::step_range(*static_cast<port::State*>(st), 0, n, in, out, u, nu, seed, res);
}

// HowFar, the caller's transport (step gfrac * proposed, direction nd*,
// post-step boundary status post), then Perform, in the order of
// G4HepEmProcess (apps/examples/TestEm3/src/G4HepEmProcess.cc:119-197);
// proposed[i] receives HowFar's geometrical step.
int port_step_geom(void* st, int64_t n, const hepem_track_state* in, hepem_track_state* out, const double* u,
                   int32_t nu, uint64_t seed, const double* gfrac, const double* ndx, const double* ndy,
                   const double* ndz, const uint8_t* post, double* proposed, hepem_step_out* res) {
  const port::Geo geo{gfrac, ndx, ndy, ndz, post, proposed};
  return port::step_range(*static_cast<port::State*>(st), 0, n, in, out, u, nu, seed, res, &geo);
}

// The same over `threads` host threads (static partition of the batch).
int port_step_mt(void* st, int64_t n, const hepem_track_state* in, hepem_track_state* out, const double* u,
                 int32_t nu, uint64_t seed, hepem_step_out* res, int threads) {
  if (threads <= 1) return port_step(st, n, in, out, u, nu, seed, res);
  std::vector<std::thread> pool;
  std::vector<int> rc(threads, 0);
  const int64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
    if (b >= e) break;
    pool.emplace_back([&, t, b, e] {
      rc[t] = port::step_range(*static_cast<port::State*>(st), b, e, in, out, u, nu, seed, res);
    });
  }
  for (auto& th : pool) th.join();
  for (int r : rc) if (r) return r;
  return 0;
}

}  // extern "C"
