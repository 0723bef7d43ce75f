// step_io.cuh -- loading / storing the SoA track batch of the C-ABI, warp-level
// counter reduction and queue pushes, shared by the plain and batched kernels.
#pragma once

#include <cstdint>

#include "g4hepem_gb300.h"
#include "kernels.h"
#include "physics.cuh"

namespace hepem {

struct StepCount {
  uint32_t steps, uniforms, overflow, secondaries, inter[8], fallback;
};
// inter[k] += 1 for k = w in [0, 8) (constant indices: the counters stay in registers)
__device__ __forceinline__ void count_inter(StepCount& c, int w) {
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (w == k) c.inter[k] += 1;
}

// Block-level sum of the step counters: warp reduce, then one atomic per block.
// Every thread of the block must call it.
__device__ __forceinline__ void add_counters(const StepCount& c, hepem_step_counters* g) {
  if (!g) return;
  __shared__ uint32_t s[13];
  if (threadIdx.x < 13) s[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t v[13] = {c.steps, c.uniforms, c.overflow, c.secondaries, c.inter[0], c.inter[1], c.inter[2],
                          c.inter[3], c.inter[4], c.inter[5], c.inter[6], c.inter[7], c.fallback};
#pragma unroll
  for (int k = 0; k < 13; ++k) {
    const uint32_t w = __reduce_add_sync(0xFFFFFFFFu, v[k]);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&s[k], w);
  }
  __syncthreads();
  if (threadIdx.x < 13 && s[threadIdx.x]) {
    unsigned long long* dst = threadIdx.x < 4    ? (unsigned long long*)&g->steps + threadIdx.x
                              : threadIdx.x < 12 ? (unsigned long long*)&g->interactions[threadIdx.x - 4]
                                                 : (unsigned long long*)&g->fp64_fallback;
    atomicAdd(dst, (unsigned long long)s[threadIdx.x]);
  }
}

// Warp-aggregated append of `value` to queue `key` (key < 0: nothing).  All 32
// lanes of the warp must call it together.
__device__ __forceinline__ void warp_push(int key, int32_t value, int32_t* const* queues, uint32_t* counts,
                                         double pe = 0.0, double* peQueue = nullptr, int peKey = -1) {
  const unsigned full = 0xFFFFFFFFu;
  const unsigned same = __match_any_sync(full, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(same) - 1;
  const unsigned below = same & ((1u << lane) - 1u);
  uint32_t base = 0;
  if (key >= 0 && lane == leader) base = atomicAdd(&counts[key], (uint32_t)__popc(same));
  base = __shfl_sync(full, base, leader);
  if (key >= 0) {
    const uint32_t pos = base + (uint32_t)__popc(below);
    queues[key][pos] = value;
    if (key == peKey) peQueue[pos] = pe;
  }
}

__device__ __forceinline__ bool track_input_bad(const DevTables& T, int type, int imc, double e) {
  return !(type >= 0 && type <= 2) || !(imc >= 0 && imc < T.nCouples) || !(e > 0.0) || !(e < 1.0e300);
}

// Read the persistent state of track i into registers (see hepem_track_state).
__device__ __forceinline__ void load_track(const hepem_track_state& in, int64_t i, Track& t, Rng& rng,
                                           const double* uniforms, int nu, uint64_t seed, int type) {
  t.imc = in.imc[i];
  t.setE(in.ekin[i]);
  t.flags = 0;
  t.nsec = 0;
  t.dir[0] = in.dir_x[i];
  t.dir[1] = in.dir_y[i];
  t.dir[2] = in.dir_z[i];
  t.onBoundary = in.on_boundary[i] != 0;
  t.nia[0] = in.nia0[i];
  t.winner = -1;
  t.edep = 0.0;
  t.gstep = 0.0;
  t.pstep = 0.0;
  t.isEl = type == 0;
  t.msc.disp[0] = t.msc.disp[1] = t.msc.disp[2] = 0.0;
  rng.u = uniforms + i * (int64_t)nu;
  rng.n = nu;
  rng.cursor = in.rng_cursor[i];
  rng.id = in.id[i];
  rng.overflow = 0u;
  rng.seed = seed;
  rng.gaussValid = in.gauss_valid[i] != 0;
  rng.gaussValue = in.gauss_value[i];
  if (type != 2) {
    t.nia[1] = in.nia1[i];
    t.nia[2] = in.nia2[i];
    t.nia[3] = in.nia3[i];
    t.safety = in.safety[i];
    t.msc.initRange = in.msc_init_range[i];
    t.msc.dynFactor = in.msc_dyn_factor[i];
    t.msc.tlimitMin = in.msc_tlimit_min[i];
    t.msc.firstStep = in.msc_first_step[i] != 0;
  }
}

// Write the state and step results of track i (secondaries excluded).
__device__ __forceinline__ void store_track(const hepem_track_state& in, const hepem_track_state& out,
                                            const hepem_step_out& res, int64_t i, const Track& t, const Rng& rng,
                                            int type, bool bad) {
  const bool charged = type != 2 && !bad;
  out.ekin[i] = t.e;
  out.dir_x[i] = t.dir[0];
  out.dir_y[i] = t.dir[1];
  out.dir_z[i] = t.dir[2];
  out.nia0[i] = t.nia[0];
  if (charged) {
    out.nia1[i] = t.nia[1];
    out.nia2[i] = t.nia[2];
    out.nia3[i] = t.nia[3];
    out.msc_init_range[i] = t.msc.initRange;
    out.msc_dyn_factor[i] = t.msc.dynFactor;
    out.msc_tlimit_min[i] = t.msc.tlimitMin;
    out.msc_first_step[i] = t.msc.firstStep ? 1 : 0;
  } else if (out.nia1 != in.nia1) {
    out.nia1[i] = in.nia1[i];
    out.nia2[i] = in.nia2[i];
    out.nia3[i] = in.nia3[i];
    out.msc_init_range[i] = in.msc_init_range[i];
    out.msc_dyn_factor[i] = in.msc_dyn_factor[i];
    out.msc_tlimit_min[i] = in.msc_tlimit_min[i];
    out.msc_first_step[i] = in.msc_first_step[i];
  }
  out.gauss_valid[i] = rng.gaussValid ? 1 : 0;
  out.gauss_value[i] = rng.gaussValue;
  out.rng_cursor[i] = rng.cursor;
  if (out.type != in.type) {
    out.type[i] = in.type[i];
    out.imc[i] = in.imc[i];
    out.id[i] = in.id[i];
    out.safety[i] = in.safety[i];
    out.on_boundary[i] = in.on_boundary[i];
  }
  res.edep[i] = t.edep;
  res.gstep[i] = t.gstep;
  res.pstep[i] = t.pstep;
  res.winner[i] = (int8_t)t.winner;
  res.disp_x[i] = charged ? t.msc.disp[0] : 0.0;
  res.disp_y[i] = charged ? t.msc.disp[1] : 0.0;
  res.disp_z[i] = charged ? t.msc.disp[2] : 0.0;
  res.flags[i] = t.flags | (rng.overflow ? kFlagRngOverflow : 0);
}

// ---- the step-limit record (kernels.h: Limits) ----------------------------------------
// After the FP64 HowFar of track i (Physics::el_howfar / gamma_howfar):
// the proposed geometrical step to gstep[i], everything else Perform needs to
// the record.  preBoundary: the pre-step boundary status HowFar used.
__device__ __forceinline__ void store_limits64(const Limits& L, int64_t i, const Track& t, const Rng& rng, int type,
                                               double* gstep) {
  const bool charged = type != 2;
  gstep[i] = t.gstep;
  L.d[kLProposed][i] = t.gstep;
  L.d[kLPstep][i] = t.pstep;
  L.d[kLMfp0][i] = t.mfp[0];
  L.d[kLNia0][i] = t.nia[0];
  L.d[kLGauss][i] = rng.gaussValue;
  L.cursor[i] = rng.cursor;
  L.winner[i] = (int8_t)t.winner;
  uint32_t b = (rng.gaussValid ? kLimGaussValid : 0u) | (t.onBoundary ? kLimPreBoundary : 0u) |
               ((uint32_t)(t.flags | (rng.overflow ? kFlagRngOverflow : 0)) << kLimFlagsShift);
  if (charged) {
    const Msc& m = t.msc;
    L.d[kLRange][i] = t.range;
#pragma unroll
    for (int k = 1; k < 4; ++k) {
      L.d[kLMfp0 + k][i] = t.mfp[k];
      L.d[kLNia0 + k][i] = t.nia[k];
    }
    L.d[kLLambtr1][i] = m.lambtr1;
    L.d[kLTrueStep][i] = m.trueStep;
    L.d[kLZPath][i] = m.zPath;
    L.d[kLPar1][i] = m.par1;
    L.d[kLPar2][i] = m.par2;
    L.d[kLPar3][i] = m.par3;
    L.d[kLInitRange][i] = m.initRange;
    L.d[kLDynFactor][i] = m.dynFactor;
    L.d[kLTlimitMin][i] = m.tlimitMin;
    b |= (m.active ? kLimMscActive : 0u) | (m.displace ? kLimMscDisplace : 0u) | (m.firstStep ? kLimFirstStep : 0u);
  } else {
    L.d[kLPeXS][i] = t.peXS;
  }
  L.bits[i] = b;
}

// Before the FP64 Perform of track i: the caller's geometrical step and the
// record over the state that load_track read (the state keeps the direction
// and the post-step boundary status that transport left).
__device__ __forceinline__ void load_limits64(const Limits& L, int64_t i, Track& t, Rng& rng, int type,
                                              const double* gstep) {
  const uint32_t b = L.bits[i];
  t.gstep = gstep[i];
  t.pstep = L.d[kLPstep][i];
  t.mfp[0] = L.d[kLMfp0][i];
  t.nia[0] = L.d[kLNia0][i];
  t.winner = L.winner[i];
  t.flags |= (uint8_t)((b >> kLimFlagsShift) & 0xFFu);
  rng.cursor = L.cursor[i];
  rng.gaussValid = (b & kLimGaussValid) != 0;
  rng.gaussValue = L.d[kLGauss][i];
  if (type != 2) {
    Msc& m = t.msc;
    t.range = L.d[kLRange][i];
#pragma unroll
    for (int k = 1; k < 4; ++k) {
      t.mfp[k] = L.d[kLMfp0 + k][i];
      t.nia[k] = L.d[kLNia0 + k][i];
    }
    m.lambtr1 = L.d[kLLambtr1][i];
    m.trueStep = L.d[kLTrueStep][i];
    m.zPath = L.d[kLZPath][i];
    m.par1 = L.d[kLPar1][i];
    m.par2 = L.d[kLPar2][i];
    m.par3 = L.d[kLPar3][i];
    m.initRange = L.d[kLInitRange][i];
    m.dynFactor = L.d[kLDynFactor][i];
    m.tlimitMin = L.d[kLTlimitMin][i];
    m.active = (b & kLimMscActive) != 0;
    m.displace = (b & kLimMscDisplace) != 0;
    m.firstStep = (b & kLimFirstStep) != 0;
    m.noScatter = false;
  } else {
    t.peXS = L.d[kLPeXS][i];
  }
}

__device__ __forceinline__ void store_secondaries(const hepem_step_out& res, int64_t i, const Track& t, int first) {
  const int ns = t.nsec > 2 ? 2 : t.nsec;
  res.n_sec[i] = (int8_t)ns;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (k >= first && k < ns) {
      res.sec_type[2 * i + k] = t.sec[k].type;
      res.sec_ekin[2 * i + k] = t.sec[k].e;
      res.sec_dir_x[2 * i + k] = t.sec[k].dir[0];
      res.sec_dir_y[2 * i + k] = t.sec[k].dir[1];
      res.sec_dir_z[2 * i + k] = t.sec[k].dir[2];
    }
  }
}

}  // namespace hepem
