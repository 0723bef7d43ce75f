// kernels_fp64.cu -- plain FP64 kernels of the drop-in path (compiled with
// --fmad=false: no contracted multiply-adds, so the arithmetic is the
// reference's operation by operation).
//
//  lookup_kernel  : the electron table lookups, the reference functions
//                   GetRestMacXSec / GetRestDEDX / GetRestRange / GetInvRange
//                   (G4HepEm/G4HepEmRun/include/G4HepEmElectronManager.icc:486-532)
//  step_kernel    : one HowFar + Perform per track
//  fill_uniforms  : the per-track Philox streams of the C-ABI contract
#include <cstdint>

#include "g4hepem_gb300.h"
#include "kernels.h"
#include "physics.cuh"
#include "physics_mixed.cuh"
#include "step_io.cuh"

namespace hepem {

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) lookup_kernel(const __grid_constant__ DevTables T, int64_t n, int pos,
                                                     const double* __restrict__ ekin, const int32_t* __restrict__ imc,
                                                     double* __restrict__ xi, double* __restrict__ xb,
                                                     double* __restrict__ dedx, double* __restrict__ range,
                                                     double* __restrict__ invr) {
  const DevElData& d = T.el[pos ? 1 : 0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double e = ekin[i];
    int c = imc[i];
    const bool bad = !(c >= 0 && c < T.nCouples) || !(e > 0.0) || !(e < 1.0e300);
    if (bad) c = 0;
    const double le = vdt_log(e);
    const double a = rest_macxs(d, c, e, le, true);
    const double b = rest_macxs(d, c, e, le, false);
    const double s = rest_dedx(d, c, e, le);
    const double r = rest_range(d, c, e, le);
    const double q = inv_range(d, c, 0.5 * r);
    const double nan = __longlong_as_double(0x7FF8000000000000LL);
    xi[i] = bad ? nan : a;
    xb[i] = bad ? nan : b;
    dedx[i] = bad ? nan : s;
    range[i] = bad ? nan : r;
    invr[i] = bad ? nan : q;
  }
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ void step_one(const DevTables& T, int64_t i, const hepem_track_state& in,
                                         const hepem_track_state& out, const double* uniforms, int nu,
                                         uint64_t seed, const hepem_step_out& res, StepCount& cnt) {
  const int type = in.type[i];
  Track t;
  t.imc = in.imc[i];
  t.setE(in.ekin[i]);
  t.flags = 0;
  t.nsec = 0;
  const bool bad = !(type >= 0 && type <= 2) || !(t.imc >= 0 && t.imc < T.nCouples) || !(t.e > 0.0) ||
                   !(t.e < 1.0e300);
  Rng rng;
  rng.u = uniforms + i * (int64_t)nu;
  rng.n = nu;
  rng.cursor = in.rng_cursor[i];
  rng.id = in.id[i];
  rng.overflow = 0u;
  rng.seed = seed;
  rng.gaussValid = in.gauss_valid[i] != 0;
  rng.gaussValue = in.gauss_value[i];
  t.dir[0] = in.dir_x[i];
  t.dir[1] = in.dir_y[i];
  t.dir[2] = in.dir_z[i];
  t.onBoundary = in.on_boundary[i] != 0;
  t.nia[0] = in.nia0[i];
  t.winner = -1;
  t.edep = 0.0;
  t.gstep = 0.0;
  t.pstep = 0.0;
  Physics P{T, rng, t};
  double nia1 = in.nia1[i], nia2 = in.nia2[i], nia3 = in.nia3[i];
  double mir = in.msc_init_range[i], mdf = in.msc_dyn_factor[i], mtm = in.msc_tlimit_min[i];
  uint8_t mfs = in.msc_first_step[i];
  t.msc.disp[0] = t.msc.disp[1] = t.msc.disp[2] = 0.0;
  if (bad) {
    t.flags |= kFlagBadInput;
  } else if (type == 2) {
    t.isEl = false;
    P.gamma_howfar();
    if (t.onBoundary) {
      t.nia[0] -= t.gstep / t.mfp[0];
    } else {
      P.gamma_select();
      P.gamma_perform();
    }
    t.pstep = t.gstep;
  } else {
    t.isEl = type == 0;
    t.nia[1] = nia1; t.nia[2] = nia2; t.nia[3] = nia3;
    t.safety = in.safety[i];
    t.msc.initRange = mir;
    t.msc.dynFactor = mdf;
    t.msc.tlimitMin = mtm;
    t.msc.firstStep = mfs != 0;
    P.el_howfar();
    P.el_perform();
    nia1 = t.nia[1]; nia2 = t.nia[2]; nia3 = t.nia[3];
    mir = t.msc.initRange; mdf = t.msc.dynFactor; mtm = t.msc.tlimitMin;
    mfs = t.msc.firstStep ? 1 : 0;
  }
  if (rng.overflow) t.flags |= kFlagRngOverflow;
  // state out (out may alias in: every input was read above)
  out.ekin[i] = t.e;
  out.dir_x[i] = t.dir[0];
  out.dir_y[i] = t.dir[1];
  out.dir_z[i] = t.dir[2];
  out.nia0[i] = t.nia[0];
  out.nia1[i] = nia1;
  out.nia2[i] = nia2;
  out.nia3[i] = nia3;
  out.msc_init_range[i] = mir;
  out.msc_dyn_factor[i] = mdf;
  out.msc_tlimit_min[i] = mtm;
  out.msc_first_step[i] = mfs;
  out.gauss_valid[i] = rng.gaussValid ? 1 : 0;
  out.gauss_value[i] = rng.gaussValue;
  out.rng_cursor[i] = rng.cursor;
  if (out.type != in.type) {
    out.type[i] = (int8_t)type;
    out.imc[i] = in.imc[i];
    out.id[i] = in.id[i];
    out.safety[i] = in.safety[i];
    out.on_boundary[i] = in.on_boundary[i];
  }
  res.edep[i] = t.edep;
  res.gstep[i] = t.gstep;
  res.pstep[i] = t.pstep;
  res.winner[i] = (int8_t)t.winner;
  const bool charged = type != 2 && !bad;
  res.disp_x[i] = charged ? t.msc.disp[0] : 0.0;
  res.disp_y[i] = charged ? t.msc.disp[1] : 0.0;
  res.disp_z[i] = charged ? t.msc.disp[2] : 0.0;
  res.flags[i] = t.flags;
  const int ns = t.nsec > 2 ? 2 : t.nsec;
  res.n_sec[i] = (int8_t)ns;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (k < ns) {
      res.sec_type[2 * i + k] = t.sec[k].type;
      res.sec_ekin[2 * i + k] = t.sec[k].e;
      res.sec_dir_x[2 * i + k] = t.sec[k].dir[0];
      res.sec_dir_y[2 * i + k] = t.sec[k].dir[1];
      res.sec_dir_z[2 * i + k] = t.sec[k].dir[2];
    }
  }
  cnt.steps += 1;
  cnt.uniforms += (uint32_t)(rng.cursor - in.rng_cursor[i]);
  cnt.overflow += rng.overflow;
  cnt.secondaries += ns;
  if (!bad && t.winner >= 0 && t.winner < 4) count_inter(cnt, (type == 2 ? 4 : 0) + t.winner);
}

__global__ void __launch_bounds__(256) step_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                   const hepem_track_state in, const hepem_track_state out,
                                                   const double* __restrict__ uniforms, int nu, uint64_t seed,
                                                   const hepem_step_out res, hepem_step_counters* counters) {
  StepCount cnt = {};
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    if (i < n) step_one(T, i, in, out, uniforms, nu, seed, res, cnt);
  }
  if (counters) add_counters(cnt, counters);
}

// ---- the step split at the geometry: HowFar, then Perform ----------------------------
// howfar_kernel: G4HepEmElectronManager::HowFar / G4HepEmGammaManager::HowFar
// (G4HepEmElectronManager.icc:35-169, G4HepEmGammaManager.icc:27-48) per track;
// the proposed geometrical step to gstep, the rest of what Perform needs to the
// step-limit record; the track state is left as it was.
__global__ void __launch_bounds__(256) howfar_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                     const hepem_track_state in, const double* __restrict__ uniforms,
                                                     int nu, uint64_t seed, double* __restrict__ gstep,
                                                     const Limits L, hepem_step_counters* counters) {
  StepCount cnt = {};
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    if (i >= n) continue;
    const int type = in.type[i];
    Track t;
    Rng rng;
    const bool bad = track_input_bad(T, type, in.imc[i], in.ekin[i]);
    load_track(in, i, t, rng, uniforms, nu, seed, bad ? 2 : type);
    if (bad) {
      t.flags |= kFlagBadInput;
      t.mfp[0] = kLarge;
      t.peXS = 0.0;
      store_limits64(L, i, t, rng, 2, gstep);
      continue;
    }
    Physics P{T, rng, t};
    if (type == 2) {
      t.isEl = false;
      P.gamma_howfar();
    } else {
      P.el_howfar();
    }
    store_limits64(L, i, t, rng, type, gstep);
    cnt.uniforms += (uint32_t)(rng.cursor - in.rng_cursor[i]);
    cnt.overflow += rng.overflow;
  }
  if (counters) add_counters(cnt, counters);
}

// perform_kernel: the rest of the step with the geometrical step gstep[i]
// that transport made, the direction and the post-step boundary status in
// the state: e+- G4HepEmElectronManager::Perform (.icc:171-483, with
// UpdatePStepLength's geometrical -> true conversion); gamma on a boundary
// UpdateNumIALeft only, else SelectInteraction + Perform, as the reference
// client (apps/examples/TestEm3/src/G4HepEmProcess.cc:160-197).
__global__ void __launch_bounds__(256) perform_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                      const hepem_track_state in, const hepem_track_state out,
                                                      const double* __restrict__ gstep, const Limits L,
                                                      const double* __restrict__ uniforms, int nu, uint64_t seed,
                                                      const hepem_step_out res, hepem_step_counters* counters) {
  StepCount cnt = {};
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    if (i >= n) continue;
    const int type = in.type[i];
    Track t;
    Rng rng;
    const bool bad = track_input_bad(T, type, in.imc[i], in.ekin[i]);
    load_track(in, i, t, rng, uniforms, nu, seed, bad ? 2 : type);
    if (bad) {
      t.flags |= kFlagBadInput;
      t.gstep = gstep[i];
      t.pstep = t.gstep;
      store_track(in, out, res, i, t, rng, 2, true);
      res.n_sec[i] = 0;
      cnt.steps += 1;
      continue;
    }
    load_limits64(L, i, t, rng, type, gstep);
    const int32_t c0 = rng.cursor;
    Physics P{T, rng, t};
    if (type == 2) {
      t.isEl = false;
      if (t.onBoundary) {
        t.nia[0] -= t.gstep / t.mfp[0];
      } else {
        P.gamma_select();
        P.gamma_perform();
      }
      t.pstep = t.gstep;
    } else {
      P.el_perform();
    }
    store_track(in, out, res, i, t, rng, type, false);
    store_secondaries(res, i, t, 0);
    const int ns = t.nsec > 2 ? 2 : t.nsec;
    cnt.steps += 1;
    cnt.uniforms += (uint32_t)(rng.cursor - c0);
    cnt.overflow += rng.overflow;
    cnt.secondaries += ns;
    if (t.winner >= 0 && t.winner < 4) count_inter(cnt, (type == 2 ? 4 : 0) + t.winner);
  }
  if (counters) add_counters(cnt, counters);
}

// the same lookups from the FP32 tables of the precision form (FP32 arithmetic)
__global__ void __launch_bounds__(256) lookup_mixed_kernel(const __grid_constant__ DevTables T, int64_t n, int pos,
                                                           const double* __restrict__ ekin,
                                                           const int32_t* __restrict__ imc, double* __restrict__ xi,
                                                           double* __restrict__ xb, double* __restrict__ dedx,
                                                           double* __restrict__ range, double* __restrict__ invr) {
  const DevElData& d = T.el[pos ? 1 : 0];
  const DevElData32& f = T.el32[pos ? 1 : 0];
  const int nL = d.nLoss;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double e = ekin[i];
    int c = imc[i];
    const bool bad = !(c >= 0 && c < T.nCouples) || !(e > 0.0) || !(e < 1.0e300);
    if (bad) c = 0;
    const float ef = (float)e, le = logf(ef);
    const float a = rest_macxs32(d, f, c, e, ef, le, true);
    const float b = rest_macxs32(d, f, c, e, ef, le, false);
    const float s = rest_dedx32(f, nL, c, ef, le);
    const float r = rest_range32(f, nL, c, ef, le);
    const float q = inv_range32(f, nL, c, 0.5f * r);
    const double nan = __longlong_as_double(0x7FF8000000000000LL);
    xi[i] = bad ? nan : (double)a;
    xb[i] = bad ? nan : (double)b;
    dedx[i] = bad ? nan : (double)s;
    range[i] = bad ? nan : (double)r;
    invr[i] = bad ? nan : (double)q;
  }
}

static int grid_for(int64_t n, int block, int sms);

// ---- Woodcock gamma tracking in a layered box (G4HepEmWoodcockHelper.cc:146-299) --------
struct BoxGeo {
  double hx, hy;
  int nl, wdt;
  const double* zb;
  const int32_t* limc;
  double elim;
};

// distance from p (inside) to the box surface along v (the box solid's DistanceToOut)
__device__ __forceinline__ double box_dist_out(const BoxGeo& b, const double* p, const double* v) {
  double d = 1.0e300;
  if (v[0] > 0.) d = dmin_(d, (b.hx - p[0]) / v[0]);
  else if (v[0] < 0.) d = dmin_(d, (-b.hx - p[0]) / v[0]);
  if (v[1] > 0.) d = dmin_(d, (b.hy - p[1]) / v[1]);
  else if (v[1] < 0.) d = dmin_(d, (-b.hy - p[1]) / v[1]);
  if (v[2] > 0.) d = dmin_(d, (ld(b.zb + b.nl) - p[2]) / v[2]);
  else if (v[2] < 0.) d = dmin_(d, (ld(b.zb) - p[2]) / v[2]);
  return dmax_(d, 0.0);
}

// layer that contains z (clamped to the box)
__device__ __forceinline__ int box_layer(const BoxGeo& b, double z) {
  if (!(z > ld(b.zb))) return 0;
  if (!(z < ld(b.zb + b.nl))) return b.nl - 1;
  int lo = 0, hi = b.nl;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (z < ld(b.zb + mid)) hi = mid; else lo = mid;
  }
  return lo;
}

// The tracks in energy order: the Woodcock loop's number of steps and the
// interaction that ends it follow the energy, so a warp of neighbouring
// energies stays converged (2.35x faster than batch order on a calorimeter
// of Pb and lAr).  A counting sort into quarter-octave bins of the energy
// (the exponent and the top two mantissa bits) gives the order; each track's
// result does not depend on it.
constexpr int kWdtBins = 256;
constexpr int64_t kWdtSortMin = 1 << 16;  // smaller batches run in batch order
__device__ __forceinline__ int wdt_bin(double e) {
  const long long bits = __double_as_longlong(e);
  if (!(e > 0.0)) return 0;
  const int b = ((int)((bits >> 52) & 0x7FF) - 1023 + 16) * 4 + (int)((bits >> 50) & 3);
  return b < 0 ? 0 : (b >= kWdtBins ? kWdtBins - 1 : b);
}
__global__ void __launch_bounds__(256) wdt_hist_kernel(int64_t n, const double* __restrict__ ekin,
                                                       uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[kWdtBins];
  for (int k = threadIdx.x; k < kWdtBins; k += blockDim.x) sh[k] = 0;
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&sh[wdt_bin(ekin[i])], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < kWdtBins; k += blockDim.x)
    if (sh[k]) atomicAdd(&hist[k], sh[k]);
}
// exclusive sums of the histogram into the scatter cursors (one block)
__global__ void wdt_scan_kernel(const uint32_t* __restrict__ hist, uint32_t* __restrict__ cursor) {
  if (threadIdx.x == 0) {
    uint32_t sum = 0;
    for (int k = 0; k < kWdtBins; ++k) {
      cursor[k] = sum;
      sum += hist[k];
    }
  }
}
// perm[cursor[bin]++] = i, one atomic per distinct bin in a warp
__global__ void __launch_bounds__(256) wdt_scatter_kernel(int64_t n, const double* __restrict__ ekin,
                                                          uint32_t* __restrict__ cursor, int32_t* __restrict__ perm) {
  const unsigned full = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const int key = i < n ? wdt_bin(ekin[i]) : -1;
    const unsigned same = __match_any_sync(full, key);
    const int leader = __ffs(same) - 1;
    uint32_t b = 0;
    if (key >= 0 && lane == leader) b = atomicAdd(&cursor[key], (uint32_t)__popc(same));
    b = __shfl_sync(full, b, leader);
    if (key >= 0) perm[b + (uint32_t)__popc(same & ((1u << lane) - 1u))] = (int32_t)i;
  }
}

__global__ void __launch_bounds__(256) woodcock_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                       const hepem_track_state in, const hepem_track_state out,
                                                       double* __restrict__ px, double* __restrict__ py,
                                                       double* __restrict__ pz, const BoxGeo b,
                                                       const double* __restrict__ uniforms, int nu, uint64_t seed,
                                                       const hepem_step_out res, uint8_t* __restrict__ reached,
                                                       const int32_t* __restrict__ perm) {
  const double kDblMax = 1.7976931348623157e308;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? (int64_t)perm[j] : j;
    const int type = in.type[i];
    Track t;
    Rng rng;
    load_track(in, i, t, rng, uniforms, nu, seed, 2);
    t.isEl = false;
    double p[3] = {px[i], py[i], pz[i]};
    bool boundary = false;
    const bool bad = type != 2 || track_input_bad(T, 2, t.imc, t.e);
    if (bad) {
      t.flags = kFlagBadInput;
    } else if (t.e > b.elim) {
      Physics P{T, rng, t};
      double dist = dmax_(box_dist_out(b, p, t.dir) - 1.0E-3, 0.0);
      t.imc = b.wdt;
      const double wdtMX = P.gamma_total_xs();
      const double wdtMFP = wdtMX > 0.0 ? 1.0 / wdtMX : kDblMax;
      const double wdtPE = t.peXS;
      const int wdtMat = T.couples[b.wdt].mat;
      double mx = 0.0, step = 0.0;
      int prev = -1, it = 0;
      bool stop = false;
      while (!stop) {
        const double ps = wdtMFP < kDblMax ? -vdt_log(rng.flat()) * wdtMFP : kDblMax;
        if (dist < ps) {
          step += dist;
          boundary = true;
          stop = true;
        } else {
          step += ps;
          dist -= ps;
          const int imc = ld(b.limc + box_layer(b, p[2] + step * t.dir[2]));
          if (T.couples[imc].mat != wdtMat) {
            if (imc != prev) {
              prev = imc;
              t.imc = imc;
              mx = P.gamma_total_xs();
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
        if (++it >= kMaxIter) {
          t.flags |= kFlagLoopCap;
          boundary = true;
          break;
        }
      }
      for (int k = 0; k < 3; ++k) p[k] += step * t.dir[k];
      t.gstep = step;
      t.nia[0] = -1.0;
      t.winner = -1;
      if (!boundary) {
        // interaction at the end point (G4HepEmTrackingManager.cc:1094-1110)
        P.gamma_select();
        t.edep = 0.0;
        if (t.winner == 0) P.conversion();
        if (t.winner == 1) P.compton();
        if (t.winner == 2) P.photoelectric();
        P.gamma_tracking_cut();
      }
      t.imc = ld(b.limc + box_layer(b, p[2]));
    } else {
      // an ordinary step in the current layer
      Physics P{T, rng, t};
      t.imc = ld(b.limc + box_layer(b, p[2]));
      P.gamma_howfar();
      P.gamma_select();
      P.gamma_perform();
      for (int k = 0; k < 3; ++k) p[k] += t.gstep * t.dir[k];
      t.imc = ld(b.limc + box_layer(b, p[2]));
    }
    t.pstep = t.gstep;
    px[i] = p[0];
    py[i] = p[1];
    pz[i] = p[2];
    store_track(in, out, res, i, t, rng, 2, bad);
    out.imc[i] = bad ? in.imc[i] : t.imc;
    store_secondaries(res, i, t, 0);
    if (reached) reached[i] = boundary ? 1 : 0;
  }
}

cudaError_t launch_woodcock(const DevTables& T, int64_t n, const hepem_track_state& in,
                            const hepem_track_state& out, double* px, double* py, double* pz,
                            const hepem_layered_box& box, const double* uniforms, int nu, uint64_t seed,
                            const hepem_step_out& res, uint8_t* reached, cudaStream_t s, int sms) {
  if (n <= 0) return cudaSuccess;
  BoxGeo b{box.half_x, box.half_y, box.n_layers, box.wdt_imc, box.z_bounds, box.layer_imc, box.energy_limit};
  int32_t* perm = nullptr;
  void* ws = nullptr;
  if (n >= kWdtSortMin) {
    cudaError_t e = cudaMallocAsync(&ws, 8 * (size_t)kWdtBins + 4 * (size_t)n, s);
    if (e != cudaSuccess) return e;
    uint32_t* hist = static_cast<uint32_t*>(ws);
    uint32_t* cursor = hist + kWdtBins;
    perm = reinterpret_cast<int32_t*>(cursor + kWdtBins);
    e = cudaMemsetAsync(hist, 0, 4 * (size_t)kWdtBins, s);
    if (e != cudaSuccess) {
      cudaFreeAsync(ws, s);
      return e;
    }
    const int g = grid_for(n, 256, sms);
    wdt_hist_kernel<<<g, 256, 0, s>>>(n, in.ekin, hist);
    wdt_scan_kernel<<<1, 32, 0, s>>>(hist, cursor);
    wdt_scatter_kernel<<<g, 256, 0, s>>>(n, in.ekin, cursor, perm);
  }
  woodcock_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(T, n, in, out, px, py, pz, b, uniforms, nu, seed, res,
                                                         reached, perm);
  const cudaError_t e = cudaGetLastError();
  if (ws) {
    const cudaError_t f = cudaFreeAsync(ws, s);
    if (e == cudaSuccess && f != cudaSuccess) return f;
  }
  return e;
}

// one warp per track, one Philox block per lane: uniforms k and k + 1 (k even)
// share the counter (k >> 1, id, 0, c), so a lane writes both, and a warp
// writes the track's row contiguously
__global__ void fill_uniforms_kernel(int64_t n, const int32_t* __restrict__ id, int nu, uint64_t seed,
                                     double* __restrict__ u) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const int32_t tid = id[i];
    double* row = u + i * nu;
    for (int k = 2 * lane; k < nu; k += 64) {
      uint32_t c0 = (uint32_t)k >> 1, c1 = (uint32_t)tid, c2 = 0u, c3 = 0x48455045u;
      philox4x32_10(c0, c1, c2, c3, (uint32_t)seed, (uint32_t)(seed >> 32));
      row[k] = u52_to_double(((uint64_t)c0 << 20) | (uint64_t)(c1 >> 12));
      if (k + 1 < nu) row[k + 1] = u52_to_double(((uint64_t)c2 << 20) | (uint64_t)(c3 >> 12));
    }
  }
}

// ---- host launchers ---------------------------------------------------------------
static int grid_for(int64_t n, int block, int sms) {
  const int64_t need = (n + block - 1) / block;
  const int64_t cap = (int64_t)sms * 32;
  return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

cudaError_t launch_lookup(const DevTables& T, int64_t n, int pos, const double* ekin, const int32_t* imc, double* xi,
                          double* xb, double* dedx, double* range, double* invr, cudaStream_t s, int sms) {
  if (n <= 0) return cudaSuccess;
  lookup_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(T, n, pos, ekin, imc, xi, xb, dedx, range, invr);
  return cudaGetLastError();
}

cudaError_t launch_lookup_mixed(const DevTables& T, int64_t n, int pos, const double* ekin, const int32_t* imc,
                                double* xi, double* xb, double* dedx, double* range, double* invr, cudaStream_t s,
                                int sms) {
  if (n <= 0) return cudaSuccess;
  lookup_mixed_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(T, n, pos, ekin, imc, xi, xb, dedx, range, invr);
  return cudaGetLastError();
}

cudaError_t launch_step(const DevTables& T, int64_t n, const hepem_track_state& in, const hepem_track_state& out,
                        const double* uniforms, int nu, uint64_t seed, const hepem_step_out& res,
                        hepem_step_counters* counters, cudaStream_t s, int sms) {
  if (n <= 0) return cudaSuccess;
  step_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(T, n, in, out, uniforms, nu, seed, res, counters);
  return cudaGetLastError();
}

cudaError_t launch_howfar(const DevTables& T, int64_t n, const hepem_track_state& in, const double* uniforms, int nu,
                          uint64_t seed, double* gstep, const Limits& L, hepem_step_counters* counters,
                          cudaStream_t s, int sms) {
  if (n <= 0) return cudaSuccess;
  howfar_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(T, n, in, uniforms, nu, seed, gstep, L, counters);
  return cudaGetLastError();
}

cudaError_t launch_perform(const DevTables& T, int64_t n, const hepem_track_state& in, const hepem_track_state& out,
                           const double* gstep, const Limits& L, const double* uniforms, int nu, uint64_t seed,
                           const hepem_step_out& res, hepem_step_counters* counters, cudaStream_t s, int sms) {
  if (n <= 0) return cudaSuccess;
  perform_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(T, n, in, out, gstep, L, uniforms, nu, seed, res, counters);
  return cudaGetLastError();
}

cudaError_t launch_fill_uniforms(int64_t n, const int32_t* id, int nu, uint64_t seed, double* u, cudaStream_t s,
                                 int sms) {
  if (n <= 0 || nu <= 0) return cudaSuccess;
  fill_uniforms_kernel<<<grid_for(n * 32, 256, sms), 256, 0, s>>>(n, id, nu, seed, u);
  return cudaGetLastError();
}

}  // namespace hepem
