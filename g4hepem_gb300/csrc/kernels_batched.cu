// kernels_batched.cu -- the batched form of the FP64 step (compiled with
// --fmad=false, same physics code as the plain form, bit-identical results).
//
// The plain kernel runs one track per thread through HowFar + Perform; in a
// mixed batch a warp then holds e-, e+ and gammas that take different branches
// and different interaction models, and the FP64 pipe -- the scarce resource of
// GB300 -- executes every branch for the whole warp.  Here the step is
// re-scheduled so that warps are coherent:
//   1. sort       : a counting sort (histogram, scan, warp-aggregated scatter)
//                   orders the tracks by particle, couple and energy bin, so
//                   that warps hold similar tracks; malformed tracks are
//                   flagged and finished here;
//   2. stage A    : e+- ranges: HowFar, continuous loss, MSC, fluctuations,
//                   the delta-interaction test; gamma range: HowFar and the
//                   interaction choice.  Each track that has a discrete
//                   interaction left is appended to the queue of that model;
//   3. stage B    : one kernel per interaction queue (Moller, Bhabha,
//                   Seltzer-Berger brem, relativistic brem, annihilation in
//                   flight / at rest, conversion, Compton, photoelectric).
// Stage kernels use persistent grids sized from occupancy and read their item
// counts from device memory, so the host never synchronises inside a step.
#include <cuda_runtime.h>

#include <cstdint>

#include "g4hepem_gb300.h"
#include "kernels.h"
#include "physics_mixed.cuh"
#include "step_io.cuh"
#include "trace.h"

// This file is compiled twice.  As itself (the FP64 unit, -fmad=false: the
// FP64 path is bit-exact only without contraction) it holds the sort, the
// FP64 stage kernels, the FP64 fallback and the host side.  Included by
// kernels_batched_mixed.cu with HEPEM_MIXED_UNIT defined, it holds the FP32
// stage kernels of the precision form, compiled with contraction (FFMA) on.
#ifdef HEPEM_MIXED_UNIT
#define HEPEM_FP64_UNIT 0
#else
#define HEPEM_FP64_UNIT 1
#endif

namespace hepem {

// Diagnostics build only (-DHEPEM_TRIP_SITES): count, per source line of
// physics_mixed.cuh, the guards that sent a track of the precision form to
// its FP64 fallback (read with hepem_debug_trip_sites).
#ifdef HEPEM_TRIP_SITES
static __device__ unsigned long long g_tripSites[4096];
#define HEPEM_COUNT_TRIP(line) atomicAdd(&g_tripSites[(line) & 4095], 1ull)
#else
#define HEPEM_COUNT_TRIP(line) ((void)0)
#endif

// Tracks are ordered by a sort key (particle, couple bin, energy bin) with a
// counting sort, so that the warps of a stage hold tracks of one particle in
// one material at similar energies and take the same branches (FP64 form; the
// precision form only splits e+- from gammas, see launch_step_batched).
constexpr int kMaxSortEBins = 32;   // log2(E) bins over 1 keV - 100 TeV (the launch configuration picks 8..32)
constexpr int kSortCoupleBins = 64; // couples beyond 64 share bins (imc % 64)
constexpr int kMaxSortKeys = 3 * kSortCoupleBins * kMaxSortEBins;

struct Work {
  uint32_t* counts;               // [0..2] e-, e+, gamma tracks (oneChargedKey: e+-, 0, gamma),
                                  // [3..3+kNumQueues] queues + FP64 fallback
  uint32_t* hist;                 // [kMaxSortKeys] tracks per sort key
  uint32_t* cursor;               // [kMaxSortKeys] scatter cursors
  int32_t* perm;                  // [n] valid tracks in sort-key order
  int32_t* queue[kNumQueues + 1];  // interaction queues; [kNumQueues]: tracks the precision form re-steps in FP64
  double* peXS;                   // parallel to queue[kQPhotoelectric]
  uint8_t* fbKind;                // parallel to queue[kNumQueues]: what the precision form redoes in FP64
  const uint64_t* seeds;          // per-track RNG keys (serving), or null: one key per call
  // precision form: the pre-step state of the tracks (the input batch, or for
  // in-place steps a copy that stage A takes of the e+- tracks it queues)
  hepem_track_state pre;
  bool preCopy;
  // precision form: e- and e+ share one sort key (one list in batch order)
  bool oneChargedKey;
  // the split step (kPhaseHowFar / kPhasePerform): the geometrical steps
  // (proposed / made) and the step-limit record
  double* gstep;
  Limits limits;
  int phase;
  // the batch: n tracks, active[0..n) of larger arrays or all; with nDev,
  // *nDev tracks (n is then an upper bound, set by the launch)
  int64_t n;
  const int32_t* active;
  const uint32_t* nDev;
  // no caller uniforms: the first kPrefill values of each stepped track's
  // stream, row prefillPos[i] (active list) or i, or null
  const double* prefill;
  const int32_t* prefillPos;
};

// the track's stream values drawn ahead (Work::prefill), when there are any
__device__ __forceinline__ void use_prefill(const Work& w, int64_t i, Rng& rng) {
  if (w.prefill) {
    const int64_t row = w.prefillPos ? (int64_t)w.prefillPos[i] : i;
    rng.u = w.prefill + row * kPrefill;
    rng.n = kPrefill;
    rng.filled = true;
  }
}

__device__ __forceinline__ uint64_t key_of(const Work& w, int64_t i, uint64_t seed) {
  return w.seeds ? w.seeds[i] : seed;
}

#if HEPEM_FP64_UNIT
const char* stage_name(int i) {
  static const char* names[kNumStageEvents - 1] = {
      "sort", "stage_a_charged", "stage_a_gamma", "ioni_e-", "ioni_e+", "brem_sb", "brem_rb",
      "annihilation_in_flight", "annihilation_at_rest", "conversion", "compton", "photoelectric"};
  return (i >= 0 && i < kNumStageEvents - 1) ? names[i] : "";
}

static size_t rnd(size_t b) { return (b + 255) / 256 * 256; }

size_t batched_workspace_bytes(int64_t n) {
  return rnd(64 * sizeof(uint32_t)) + 2 * rnd(kMaxSortKeys * sizeof(uint32_t)) +
         (2 + kNumQueues) * rnd(sizeof(int32_t) * (size_t)n) + rnd(sizeof(double) * (size_t)n) + rnd((size_t)n);
}

size_t mixed_pre_state_bytes(int64_t n) {
  // ekin, dir x3, nia x4, msc x3, gauss value: 12 doubles; cursor; first step, gauss valid
  return 12 * rnd(sizeof(double) * (size_t)n) + rnd(sizeof(int32_t) * (size_t)n) + 2 * rnd((size_t)n);
}

hepem_track_state carve_pre_state(void* mem, int64_t n, const hepem_track_state& in) {
  uint8_t* p = static_cast<uint8_t*>(mem);
  auto dbl = [&]() {
    double* r = reinterpret_cast<double*>(p);
    p += rnd(sizeof(double) * (size_t)n);
    return r;
  };
  hepem_track_state s = in;  // type, imc, id, safety, on_boundary: the input's
  s.ekin = dbl();
  s.dir_x = dbl();
  s.dir_y = dbl();
  s.dir_z = dbl();
  s.nia0 = dbl();
  s.nia1 = dbl();
  s.nia2 = dbl();
  s.nia3 = dbl();
  s.msc_init_range = dbl();
  s.msc_dyn_factor = dbl();
  s.msc_tlimit_min = dbl();
  s.gauss_value = dbl();
  s.rng_cursor = reinterpret_cast<int32_t*>(p);
  p += rnd(sizeof(int32_t) * (size_t)n);
  s.msc_first_step = p;
  p += rnd((size_t)n);
  s.gauss_valid = p;
  return s;
}

static Work carve(void* ws, int64_t n) {
  uint8_t* p = static_cast<uint8_t*>(ws);
  Work w;
  w.oneChargedKey = false;
  w.gstep = nullptr;
  w.limits = Limits{};
  w.phase = kPhaseStep;
  w.n = n;
  w.active = nullptr;
  w.nDev = nullptr;
  w.prefill = nullptr;
  w.prefillPos = nullptr;
  w.counts = reinterpret_cast<uint32_t*>(p);
  p += rnd(64 * sizeof(uint32_t));
  w.hist = reinterpret_cast<uint32_t*>(p);
  p += rnd(kMaxSortKeys * sizeof(uint32_t));
  w.cursor = reinterpret_cast<uint32_t*>(p);
  p += rnd(kMaxSortKeys * sizeof(uint32_t));
  w.perm = reinterpret_cast<int32_t*>(p);
  p += rnd(sizeof(int32_t) * (size_t)n);
  for (int k = 0; k <= kNumQueues; ++k) {
    w.queue[k] = reinterpret_cast<int32_t*>(p);
    p += rnd(sizeof(int32_t) * (size_t)n);
  }
  w.peXS = reinterpret_cast<double*>(p);
  p += rnd(sizeof(double) * (size_t)n);
  w.fbKind = p;
  return w;
}

__device__ __forceinline__ int sort_key(int type, int imc, double e, int ncb, int neb, bool oneChargedKey) {
  // Gammas keep their batch order (one key): their stage is light on FP64 and
  // latency bound, so coalesced loads matter more there than branch coherence.
  if (type == 2) return 2 * ncb * neb;
  // the precision form (ncb = neb = 1) keeps e- and e+ in one list: the e+
  // alone are too sparse in the batch for their loads to share sectors
  if (oneChargedKey) return 0;
  // log2(1 keV / MeV) = -9.9658, log2(100 TeV / 1 keV) = 36.5412
  int eb = (int)((__log2f((float)e) + 9.965784f) * ((float)neb / 36.541209f));
  eb = eb < 0 ? 0 : (eb >= neb ? neb - 1 : eb);
  return ((type * ncb) + (imc % ncb)) * neb + eb;
}

// ---- 0. no caller uniforms: the first kPrefill values of each stream --------------
// Row p of `pre` (track i = active[p], or p) gets stream values 0..kPrefill-1
// of track i, the same values Rng::flat draws in place (rng.cuh: Philox block
// (k >> 1, id, 0, 0x48455045) keyed by the track's seed, two values a block);
// pos[i] = p for an active list.
__global__ void __launch_bounds__(256) prefill_kernel(int64_t n, const int32_t* __restrict__ active,
                                                      const uint32_t* __restrict__ nDev,
                                                      const hepem_track_state in,
                                                      const uint64_t* __restrict__ seeds, uint64_t seed,
                                                      double* __restrict__ pre, int32_t* __restrict__ pos) {
  if (nDev && (int64_t)*nDev < n) n = *nDev;
  constexpr int kPairs = kPrefill / 2;
  const int64_t total = n * kPairs;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = g / kPairs;
    const uint32_t pair = (uint32_t)(g - p * kPairs);
    const int64_t i = active ? (int64_t)active[p] : p;
    const uint64_t key = seeds ? seeds[i] : seed;
    uint32_t c0 = pair, c1 = (uint32_t)in.id[i], c2 = 0u, c3 = 0x48455045u;
    philox4x32_10(c0, c1, c2, c3, (uint32_t)key, (uint32_t)(key >> 32));
    double2 v;
    v.x = u52_to_double(((uint64_t)c0 << 20) | (uint64_t)(c1 >> 12));
    v.y = u52_to_double(((uint64_t)c2 << 20) | (uint64_t)(c3 >> 12));
    reinterpret_cast<double2*>(pre + p * kPrefill)[pair] = v;
    if (pos && pair == 0) pos[i] = (int32_t)p;
  }
}

// ---- 1. sort: histogram, scan, scatter ----------------------------------------------
__global__ void __launch_bounds__(256) sort_hist_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                        const int32_t* __restrict__ active,
                                                        const hepem_track_state in, const hepem_track_state out,
                                                        const hepem_step_out res, const Work w, int ncb,
                                                        int neb, hepem_step_counters* counters) {
  extern __shared__ uint32_t sh[];
  const int nkeys = 3 * ncb * neb;
  for (int k = threadIdx.x; k < nkeys; k += blockDim.x) sh[k] = 0;
  __syncthreads();
  if (w.nDev && (int64_t)*w.nDev < n) n = *w.nDev;
  StepCount cnt = {};
  const int lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    int key = -1;
    if (j < n) {
      const int64_t i = active ? (int64_t)active[j] : j;
      const int type = in.type[i];
      const int imc = in.imc[i];
      const double e = in.ekin[i];
      if (track_input_bad(T, type, imc, e)) {
        if (w.phase == kPhaseHowFar) {
          // no step limit: flagged in the record, passed through by Perform
          w.gstep[i] = 0.0;
          w.limits.d[kLProposed][i] = 0.0;
          w.limits.bits[i] = (uint32_t)kFlagBadInput << kLimFlagsShift;
        } else {
          // pass the track through unchanged, flagged
          Track t;
          Rng rng;
          load_track(in, i, t, rng, nullptr, 0, 0, 2);
          t.flags = kFlagBadInput;
          if (w.phase == kPhasePerform) {
            t.gstep = w.gstep[i];
            t.pstep = t.gstep;
          }
          store_track(in, out, res, i, t, rng, 2, true);
          res.n_sec[i] = 0;
          cnt.steps += 1;
        }
      } else {
        key = sort_key(type, imc, e, ncb, neb, w.oneChargedKey);
      }
    }
    // warp-aggregated: one shared atomic per distinct key in the warp
    const unsigned same = __match_any_sync(0xFFFFFFFFu, key);
    if (key >= 0 && lane == __ffs(same) - 1) atomicAdd(&sh[key], (uint32_t)__popc(same));
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nkeys; k += blockDim.x)
    if (sh[k]) atomicAdd(&w.hist[k], sh[k]);
  add_counters(cnt, counters);
}

// one block: exclusive scan of the histogram into the scatter cursors, and
// the number of tracks of each particle type
__global__ void __launch_bounds__(1024) sort_scan_kernel(const Work w, int ncb, int neb) {
  __shared__ uint32_t partial[1024];
  const int nkeys = 3 * ncb * neb;
  const int per = (nkeys + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per;
  uint32_t s = 0;
  for (int k = b; k < b + per && k < nkeys; ++k) s += w.hist[k];
  partial[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < (int)blockDim.x; off <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)off ? partial[threadIdx.x - off] : 0u;
    __syncthreads();
    partial[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = partial[threadIdx.x] - s;
  for (int k = b; k < b + per && k < nkeys; ++k) {
    w.cursor[k] = run;
    run += w.hist[k];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    uint32_t c = 0;
    for (int k = threadIdx.x * ncb * neb; k < (threadIdx.x + 1) * ncb * neb; ++k) c += w.hist[k];
    w.counts[threadIdx.x] = c;
  }
}

// Scatter in tiles of 2048 tracks: ranks within the tile from shared-memory
// counters (warp-aggregated), then one global atomic per key and tile reserves
// the tile's range of each key.  (The order within a key is not fixed; no
// result depends on it.)
constexpr int kScatterItems = 8;
__global__ void __launch_bounds__(256) sort_scatter_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                           const int32_t* __restrict__ active,
                                                           const hepem_track_state in, const Work w, int ncb,
                                                           int neb) {
  extern __shared__ uint32_t sh[];
  const int nkeys = 3 * ncb * neb;
  const int lane = threadIdx.x & 31;
  const int64_t tile = 256 * kScatterItems;
  if (w.nDev && (int64_t)*w.nDev < n) n = *w.nDev;
  for (int64_t base = blockIdx.x * tile; base < n; base += (int64_t)gridDim.x * tile) {
    for (int k = threadIdx.x; k < nkeys; k += 256) sh[k] = 0;
    __syncthreads();
    int key[kScatterItems];
    uint32_t rank[kScatterItems];
    int32_t idx[kScatterItems];
#pragma unroll
    for (int it = 0; it < kScatterItems; ++it) {
      const int64_t j = base + it * 256 + threadIdx.x;
      key[it] = -1;
      idx[it] = 0;
      if (j < n) {
        const int64_t i = active ? (int64_t)active[j] : j;
        idx[it] = (int32_t)i;
        const int type = in.type[i];
        const int imc = in.imc[i];
        const double e = in.ekin[i];
        if (!track_input_bad(T, type, imc, e)) key[it] = sort_key(type, imc, e, ncb, neb, w.oneChargedKey);
      }
      // warp-aggregated: one shared atomic per distinct key in the warp
      const unsigned same = __match_any_sync(0xFFFFFFFFu, key[it]);
      const int leader = __ffs(same) - 1;
      uint32_t b = 0;
      if (key[it] >= 0 && lane == leader) b = atomicAdd(&sh[key[it]], (uint32_t)__popc(same));
      b = __shfl_sync(0xFFFFFFFFu, b, leader);
      rank[it] = b + __popc(same & ((1u << lane) - 1u));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nkeys; k += 256) {
      const uint32_t c = sh[k];
      if (c) sh[k] = atomicAdd(&w.cursor[k], c);
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kScatterItems; ++it)
      if (key[it] >= 0) w.perm[sh[key[it]] + rank[it]] = idx[it];
    __syncthreads();
  }
}

#endif  // HEPEM_FP64_UNIT

// ---- the FP32 step-limit record of the precision form's split step -------------------
// The values of ElLimit32 / GammaLimit32 widened to FP64 (exactly) in the
// record of kernels.h, with kLimFp32 set and the provenance bits of
// ElLimit32 in bits kLimProvShift...
__device__ __forceinline__ void store_limits32(const Limits& L, int64_t i, const ElLimit32& h, const Track& t,
                                               const Rng& rng, double* gstep) {
  gstep[i] = f2d(h.gstep);
  L.d[kLProposed][i] = f2d(h.gstep);
  L.d[kLPstep][i] = f2d(h.pstep);
  L.d[kLRange][i] = f2d(h.range);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    L.d[kLMfp0 + k][i] = f2d(h.mfp[k]);
    L.d[kLNia0 + k][i] = f2d(h.nia[k]);
  }
  L.d[kLLambtr1][i] = f2d(h.lambtr1);
  L.d[kLTrueStep][i] = f2d(h.trueStep);
  L.d[kLZPath][i] = f2d(h.zPath);
  L.d[kLDelta][i] = f2d(h.delta);
  L.d[kLInitRange][i] = f2d(h.initRange);
  L.d[kLDynFactor][i] = f2d(h.dynFactor);
  L.d[kLTlimitMin][i] = f2d(h.tlimitMin);
  L.d[kLGauss][i] = rng.gaussValue;
  L.cursor[i] = rng.cursor;
  L.winner[i] = (int8_t)h.winner;
  L.bits[i] = kLimFp32 | (rng.gaussValid ? kLimGaussValid : 0u) | (t.onBoundary ? kLimPreBoundary : 0u) |
              (h.bits << kLimProvShift) |
              ((uint32_t)(t.flags | (rng.overflow ? kFlagRngOverflow : 0)) << kLimFlagsShift);
}

__device__ __forceinline__ void load_limits32(const Limits& L, int64_t i, ElLimit32& h, Track& t, Rng& rng) {
  const uint32_t b = L.bits[i];
  h.gstep = d2f(L.d[kLProposed][i]);
  h.pstep = d2f(L.d[kLPstep][i]);
  h.range = d2f(L.d[kLRange][i]);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    h.mfp[k] = d2f(L.d[kLMfp0 + k][i]);
    h.nia[k] = d2f(L.d[kLNia0 + k][i]);
  }
  h.lambtr1 = d2f(L.d[kLLambtr1][i]);
  h.trueStep = d2f(L.d[kLTrueStep][i]);
  h.zPath = d2f(L.d[kLZPath][i]);
  h.delta = d2f(L.d[kLDelta][i]);
  h.initRange = d2f(L.d[kLInitRange][i]);
  h.dynFactor = d2f(L.d[kLDynFactor][i]);
  h.tlimitMin = d2f(L.d[kLTlimitMin][i]);
  h.winner = L.winner[i];
  h.bits = (b >> kLimProvShift) & 0xFFu;
  rng.cursor = L.cursor[i];
  rng.gaussValid = (b & kLimGaussValid) != 0;
  rng.gaussValue = L.d[kLGauss][i];
  t.flags |= (uint8_t)((b >> kLimFlagsShift) & 0xFFu);
}

__device__ __forceinline__ void store_glimits32(const Limits& L, int64_t i, const GammaLimit32& q, const Track& t,
                                                const Rng& rng, double* gstep) {
  gstep[i] = f2d(q.gstep);
  L.d[kLProposed][i] = f2d(q.gstep);
  L.d[kLPstep][i] = f2d(q.gstep);
  L.d[kLMfp0][i] = f2d(q.mfp);
  L.d[kLNia0][i] = f2d(q.nia0);
  L.d[kLPeXS][i] = f2d(q.pe);
  L.d[kLGauss][i] = rng.gaussValue;
  L.cursor[i] = rng.cursor;
  L.winner[i] = -1;
  L.bits[i] = kLimFp32 | (rng.gaussValid ? kLimGaussValid : 0u) | (t.onBoundary ? kLimPreBoundary : 0u) |
              ((uint32_t)(t.flags | (rng.overflow ? kFlagRngOverflow : 0)) << kLimFlagsShift);
}

__device__ __forceinline__ void load_glimits32(const Limits& L, int64_t i, GammaLimit32& q, Track& t, Rng& rng) {
  const uint32_t b = L.bits[i];
  q.gstep = d2f(L.d[kLProposed][i]);
  q.mfp = d2f(L.d[kLMfp0][i]);
  q.nia0 = d2f(L.d[kLNia0][i]);
  q.pe = d2f(L.d[kLPeXS][i]);
  t.nia[0] = L.d[kLNia0][i];
  rng.cursor = L.cursor[i];
  rng.gaussValid = (b & kLimGaussValid) != 0;
  rng.gaussValue = L.d[kLGauss][i];
  t.flags |= (uint8_t)((b >> kLimFlagsShift) & 0xFFu);
}

// ---- 2. stage A -----------------------------------------------------------------------
// copy of the mutable pre-step state of track i (precision form, in-place steps)
__device__ __forceinline__ void save_pre(const hepem_track_state& in, const hepem_track_state& pre, int64_t i) {
  pre.ekin[i] = in.ekin[i];
  pre.dir_x[i] = in.dir_x[i];
  pre.dir_y[i] = in.dir_y[i];
  pre.dir_z[i] = in.dir_z[i];
  pre.nia0[i] = in.nia0[i];
  pre.nia1[i] = in.nia1[i];
  pre.nia2[i] = in.nia2[i];
  pre.nia3[i] = in.nia3[i];
  pre.msc_init_range[i] = in.msc_init_range[i];
  pre.msc_dyn_factor[i] = in.msc_dyn_factor[i];
  pre.msc_tlimit_min[i] = in.msc_tlimit_min[i];
  pre.msc_first_step[i] = in.msc_first_step[i];
  pre.gauss_valid[i] = in.gauss_valid[i];
  pre.gauss_value[i] = in.gauss_value[i];
  pre.rng_cursor[i] = in.rng_cursor[i];
}

// MODE kStageFp64: the FP64 physics over the e+- tracks in sort order.
// MODE kStageMixed: the precision form (physics_mixed.cuh) over the same
//   tracks; a track whose FP32 pass tripped a guard is not stored but appended
//   to the fallback list, whose tracks one last kernel steps in FP64.
enum { kStageFp64 = 0, kStageMixed = 1 };

// fallback list of the precision form: queue[kNumQueues] with its kinds and
// the count in counts[kFbCount].  Kind 0: the e+- stage A tripped (the track
// was not stored); kind 1 + Q: interaction model Q tripped; kind kFbGammaA:
// the gamma stage A tripped (the track was not stored).
constexpr int kFbCount = 3 + kNumQueues;
constexpr uint8_t kFbGammaA = 1 + kNumQueues;

// warp-aggregated append to the fallback list; all 32 lanes call it
__device__ __forceinline__ void fb_push(bool trip, int32_t idx, uint8_t kind, const Work& w) {
  const unsigned m = __ballot_sync(0xFFFFFFFFu, trip);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&w.counts[kFbCount], (uint32_t)__popc(m));
  base = __shfl_sync(0xFFFFFFFFu, base, leader);
  if (trip) {
    const uint32_t pos = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
    w.queue[kNumQueues][pos] = idx;
    w.fbKind[pos] = kind;
  }
}

// The FP32 stages are latency bound (dependent table gathers and special
// functions per track): they are compiled for more resident warps per SM
// (stage A e+-: 32 warps, 64 registers; stage A gamma and stage B: 24 warps,
// 80 registers); the FP64 stages keep their registers (their FP64 pipe is the
// limit).
#ifndef HEPEM_MIXED_A_WARPS
#define HEPEM_MIXED_A_WARPS 32
#endif
#ifndef HEPEM_MIXED_B_WARPS
#define HEPEM_MIXED_B_WARPS 24
#endif
#ifndef HEPEM_MIXED_G_WARPS
#define HEPEM_MIXED_G_WARPS 24
#endif
// PHASE kPhaseStep: HowFar and Perform up to the interaction (the fused step);
// kPhaseHowFar: HowFar only, into the step-limit record (nothing queued);
// kPhasePerform: Perform from the record with the caller's geometrical step.
// Stage A of one e+- track idx: HowFar + Perform up to the pending discrete
// interaction.  Returns the queue of that interaction (-1: none); tripped =
// the precision form handed the track to its FP64 fallback (nothing stored).
template <int MODE, int PHASE>
__device__ __forceinline__ int charged_item(const DevTables& T, const hepem_track_state& in,
                                            const hepem_track_state& out, const double* uniforms, int nu,
                                            uint64_t seed, const hepem_step_out& res, const Work& w, int32_t idx,
                                            int type, bool& tripped, StepCount& cnt) {
  int key = -1;
  Track t;
  Rng rng;
  load_track(in, idx, t, rng, uniforms, nu, key_of(w, idx, seed), type);
  use_prefill(w, idx, rng);
  int32_t c0 = rng.cursor;
  if (MODE == kStageMixed) {
    MixedEl M{T, rng, t, false};
    if (PHASE == kPhaseStep) {
      key = M.stage_a();
    } else if (PHASE == kPhaseHowFar) {
      ElLimit32 h;
      M.howfar(h);
      if (!M.trip) store_limits32(w.limits, idx, h, t, rng, w.gstep);
    } else {
      ElLimit32 h;
      load_limits32(w.limits, idx, h, t, rng);
      c0 = rng.cursor;
      // an FP64 record (its HowFar tripped), or a step that transport
      // shortened (the geometrical -> true conversion): the FP64 code
      if (!(w.limits.bits[idx] & kLimFp32) || w.gstep[idx] != f2d(h.gstep))
        M.set_trip();
      else
        key = M.perform(h);
    }
    tripped = M.trip;
    if (tripped) HEPEM_COUNT_TRIP(M.tripLine);
  } else {
    Physics P{T, rng, t};
    if (PHASE == kPhaseStep) {
      P.el_howfar();
      key = P.el_perform_until_discrete();
    } else if (PHASE == kPhaseHowFar) {
      P.el_howfar();
      store_limits64(w.limits, idx, t, rng, type, w.gstep);
    } else {
      load_limits64(w.limits, idx, t, rng, type, w.gstep);
      c0 = rng.cursor;
      key = P.el_perform_until_discrete();
    }
  }
  if (PHASE == kPhaseHowFar) {
    key = -1;
    if (!tripped) {
      cnt.uniforms += (uint32_t)(rng.cursor - c0);
      cnt.overflow += rng.overflow;
    }
  } else if (tripped) {
    key = -1;
  } else {
    if (MODE == kStageMixed && w.preCopy && key >= 0 && key != kQAnnihRest) save_pre(in, w.pre, idx);
    store_track(in, out, res, idx, t, rng, type, false);
    res.n_sec[idx] = 0;
    cnt.steps += 1;
    cnt.uniforms += (uint32_t)(rng.cursor - c0);
    cnt.overflow += rng.overflow;
    if (t.winner >= 0 && t.winner < 4) count_inter(cnt, t.winner);
  }
  return key;
}

// Stage A of one gamma idx: HowFar, the interaction choice and Perform up to
// the interaction; pe = the photoelectric cross section for its model.
// MODE kStageMixed: from the FP32 table (MixedG); a tripped gamma is not
// stored but goes to the fallback list.
template <int MODE, int PHASE>
__device__ __forceinline__ int gamma_item(const DevTables& T, const hepem_track_state& in,
                                          const hepem_track_state& out, const double* uniforms, int nu,
                                          uint64_t seed, const hepem_step_out& res, const Work& w, int32_t idx,
                                          double& pe, bool& tripped, StepCount& cnt) {
  int key = -1;
  Track t;
  Rng rng;
  load_track(in, idx, t, rng, uniforms, nu, key_of(w, idx, seed), 2);
  use_prefill(w, idx, rng);
  int32_t c0 = rng.cursor;
  t.isEl = false;
  if (MODE == kStageMixed) {
    MixedG G{T, rng, t, false};
    if (PHASE == kPhaseStep) {
      key = G.stage_a();
    } else if (PHASE == kPhaseHowFar) {
      GammaLimit32 q;
      G.howfar(q);
      store_glimits32(w.limits, idx, q, t, rng, w.gstep);
    } else {
      GammaLimit32 q;
      load_glimits32(w.limits, idx, q, t, rng);
      c0 = rng.cursor;
      const double g = w.gstep[idx];
      key = G.perform(q, d2f(g));
      t.gstep = g;
      t.pstep = g;
    }
    tripped = G.trip;
    if (tripped) {
      HEPEM_COUNT_TRIP(G.tripLine);
      key = -1;
    }
  } else {
    Physics P{T, rng, t};
    if (PHASE == kPhaseHowFar) {
      P.gamma_howfar();
      store_limits64(w.limits, idx, t, rng, 2, w.gstep);
    } else {
      if (PHASE == kPhaseStep) {
        P.gamma_howfar();
      } else {
        load_limits64(w.limits, idx, t, rng, 2, w.gstep);
        c0 = rng.cursor;
      }
      if (t.onBoundary) {
        t.nia[0] -= t.gstep / t.mfp[0];
      } else {
        P.gamma_select();
        key = P.gamma_perform_until_interaction();
      }
      t.pstep = t.gstep;
    }
  }
  if (PHASE == kPhaseHowFar) {
    key = -1;
    cnt.uniforms += (uint32_t)(rng.cursor - c0);
    cnt.overflow += rng.overflow;
  } else if (!tripped) {
    if (key == -2) {
      Physics P{T, rng, t};
      P.gamma_tracking_cut();
      key = -1;
    }
    pe = t.peXS;
    store_track(in, out, res, idx, t, rng, 2, false);
    res.n_sec[idx] = 0;
    cnt.steps += 1;
    cnt.uniforms += (uint32_t)(rng.cursor - c0);
    cnt.overflow += rng.overflow;
    if (t.winner >= 0 && t.winner < 4) count_inter(cnt, 4 + t.winner);
  }
  return key;
}

// PHASE kPhaseStep: HowFar and Perform up to the interaction (the fused step);
// kPhaseHowFar: HowFar only, into the step-limit record (nothing queued);
// kPhasePerform: Perform from the record with the caller's geometrical step.
// The e+- tracks in sort order (perm[0, nEm + nEp)).
template <int BS, int MODE, int PHASE = kPhaseStep>
__global__ void __launch_bounds__(BS, MODE == kStageMixed ? HEPEM_MIXED_A_WARPS * 32 / BS : 1)
    stage_a_charged_kernel(const __grid_constant__ DevTables T, const hepem_track_state in,
                           const hepem_track_state out, const double* __restrict__ uniforms, int nu, uint64_t seed,
                           const hepem_step_out res, const Work w, hepem_step_counters* counters) {
  const uint32_t nEm = w.counts[0], nEp = w.counts[1];
  const int64_t total = (int64_t)nEm + nEp;
  StepCount cnt = {};
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < total; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    int key = -1;
    int32_t idx = 0;
    bool tripped = false;
    if (j < total) {
      idx = w.perm[j];
      const int type = w.oneChargedKey ? (int)in.type[idx] : (j < nEm ? 0 : 1);
      key = charged_item<MODE, PHASE>(T, in, out, uniforms, nu, seed, res, w, idx, type, tripped, cnt);
    }
    warp_push(key, idx, w.queue, w.counts + 3);
    if (MODE == kStageMixed) fb_push(tripped, idx, 0, w);
  }
  add_counters(cnt, counters);
}

// The gammas in sort order (perm[nEm + nEp, ...)).
template <int BS, int MODE, int PHASE = kPhaseStep>
__global__ void __launch_bounds__(BS, MODE == kStageMixed ? HEPEM_MIXED_G_WARPS * 32 / BS : 1)
    stage_a_gamma_kernel(const __grid_constant__ DevTables T,
                                                            const hepem_track_state in, const hepem_track_state out,
                                                            const double* __restrict__ uniforms, int nu,
                                                            uint64_t seed, const hepem_step_out res, const Work w,
                                                            hepem_step_counters* counters) {
  const int64_t total = w.counts[2];
  StepCount cnt = {};
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < total; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    int key = -1;
    int32_t idx = 0;
    double pe = 0.0;
    bool tripped = false;
    if (j < total) {
      idx = w.perm[w.counts[0] + w.counts[1] + j];
      key = gamma_item<MODE, PHASE>(T, in, out, uniforms, nu, seed, res, w, idx, pe, tripped, cnt);
    }
    warp_push(key, idx, w.queue, w.counts + 3, pe, w.peXS, kQPhotoelectric);
    if (MODE == kStageMixed) fb_push(tripped, idx, kFbGammaA, w);
  }
  add_counters(cnt, counters);
}

// ---- 3. stage B: one interaction model per kernel ------------------------------------------
// e+- models: their input energy carries the FP32 continuous loss
__host__ __device__ constexpr bool charged_model(int q) {
  return q == kQIoniEm || q == kQIoniEp || q == kQBremSB || q == kQBremRB || q == kQAnnihFlight;
}

// one interaction of model Q for track i (j: its queue position, for the
// photoelectric cross section; < 0 when not queued).  MIXED: the FP32 model,
// which returns true (storing nothing) when a guard tripped.
template <int Q, bool MIXED>
__device__ bool stage_b_one(const DevTables& T, const hepem_track_state& in, const hepem_track_state& out,
                            const double* uniforms, int nu, uint64_t seed, const hepem_step_out& res, const Work& w,
                            int32_t i, int64_t j, StepCount& cnt) {
  Track t;
  Rng rng;
  t.imc = in.imc[i];
  t.setE(out.ekin[i]);
  t.dir[0] = out.dir_x[i];
  t.dir[1] = out.dir_y[i];
  t.dir[2] = out.dir_z[i];
  t.isEl = (Q == kQIoniEm) || ((Q == kQBremSB || Q == kQBremRB) && in.type[i] == 0);
  t.flags = res.flags[i];
  t.nsec = 0;
  rng.u = uniforms + (int64_t)i * nu;
  rng.n = nu;
  use_prefill(w, i, rng);
  rng.cursor = out.rng_cursor[i];
  rng.id = in.id[i];
  rng.overflow = 0u;
  rng.seed = key_of(w, i, seed);
  rng.gaussValid = out.gauss_valid[i] != 0;
  rng.gaussValue = out.gauss_value[i];
  const int32_t c0 = rng.cursor;
  if (MIXED) {
    MixedB M{T, rng, t, false};
    if (Q == kQIoniEm || Q == kQIoniEp) M.ioni();
    if (Q == kQBremSB) M.brem(true);
    if (Q == kQBremRB) M.brem(false);
    if (Q == kQAnnihFlight) M.annihilate_in_flight();
    if (Q >= kQConversion) {
      t.edep = 0.0;
      if (Q == kQConversion) M.conversion();
      if (Q == kQCompton) M.compton();
    }
    if (M.trip) {
      HEPEM_COUNT_TRIP(M.tripLine);
      return true;
    }
  } else {
    Physics P{T, rng, t};
    if (Q == kQIoniEm || Q == kQIoniEp) P.ioni();
    if (Q == kQBremSB) P.brem(true);
    if (Q == kQBremRB) P.brem(false);
    if (Q == kQAnnihFlight) P.annihilate_in_flight();
    if (Q == kQAnnihRest) P.annihilate_at_rest();
    if (Q >= kQConversion) {
      t.edep = 0.0;
      t.peXS = (Q == kQPhotoelectric && j >= 0) ? w.peXS[j] : 0.0;
      if (Q == kQConversion) P.conversion();
      if (Q == kQCompton) P.compton();
      if (Q == kQPhotoelectric) P.photoelectric();
    }
  }
  if (Q >= kQConversion) {
    Physics P{T, rng, t};
    P.gamma_tracking_cut();
    res.edep[i] = t.edep;
  }
  out.ekin[i] = t.e;
  if (Q != kQAnnihRest) {
    out.dir_x[i] = t.dir[0];
    out.dir_y[i] = t.dir[1];
    out.dir_z[i] = t.dir[2];
  }
  out.gauss_valid[i] = rng.gaussValid ? 1 : 0;
  out.gauss_value[i] = rng.gaussValue;
  out.rng_cursor[i] = rng.cursor;
  const bool firstOverflow = rng.overflow && !(t.flags & kFlagRngOverflow);
  res.flags[i] = t.flags | (rng.overflow ? kFlagRngOverflow : 0);
  store_secondaries(res, i, t, 0);
  cnt.uniforms += (uint32_t)(rng.cursor - c0);
  cnt.overflow += firstOverflow ? 1u : 0u;
  cnt.secondaries += (uint32_t)(t.nsec > 2 ? 2 : t.nsec);
  return false;
}

template <int Q, int BS, int MODE>
__global__ void __launch_bounds__(BS, MODE == kStageMixed ? HEPEM_MIXED_B_WARPS * 32 / BS : 1) stage_b_kernel(const __grid_constant__ DevTables T,
                                                      const hepem_track_state in, const hepem_track_state out,
                                                      const double* __restrict__ uniforms, int nu, uint64_t seed,
                                                      const hepem_step_out res, const Work w,
                                                      hepem_step_counters* counters) {
  const int64_t total = w.counts[3 + Q];
  const int32_t* q = w.queue[Q];
  StepCount cnt = {};
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < total; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    bool tripped = false;
    int32_t i = 0;
    if (j < total) {
      i = q[j];
      tripped = stage_b_one<Q, MODE == kStageMixed>(T, in, out, uniforms, nu, seed, res, w, i, j, cnt);
    }
    if (MODE == kStageMixed) fb_push(tripped, i, (uint8_t)(1 + Q), w);
  }
  add_counters(cnt, counters);
}

// Precision form, last kernel of the step: the FP64 redo of every track on
// the fallback list.  A tripped e+- stage A, or a tripped e+- interaction, is
// stepped again entirely in FP64 from its pre-step state (the interaction's
// input energy carries the FP32 continuous loss, so the FP64 interaction
// alone would not give the FP64 path's outcome at the near-tie that tripped
// the guard).  A tripped gamma interaction has exact inputs: only the FP64
// interaction is redone.  One launch for all of them keeps the latency of
// these few long FP64 threads to one kernel's tail.
template <int Q>
__device__ __forceinline__ void interaction_fp64(Physics& P) {
  if (Q == kQIoniEm || Q == kQIoniEp) P.ioni();
  if (Q == kQBremSB) P.brem(true);
  if (Q == kQBremRB) P.brem(false);
  if (Q == kQAnnihFlight) P.annihilate_in_flight();
  if (Q == kQAnnihRest) P.annihilate_at_rest();
}

#if HEPEM_FP64_UNIT
// PHASE kPhaseHowFar: the FP64 HowFar of a track whose FP32 HowFar tripped,
// into the step-limit record.  kPhasePerform: the whole step again in FP64:
// HowFar from the pre-step state with the pre-step boundary status (the state
// is the pre-step one: HowFar left it unchanged), then the caller's transport
// (its geometrical step, unless it is the proposed one, the direction and the
// post-step boundary status in the state), then Perform.  An unshortened step
// is the FP64 proposed one, as in the fused step (results equal to it).
template <int PHASE>
__device__ void charged_full_step(const DevTables& T, const hepem_track_state& in, const hepem_track_state& out,
                                  const double* uniforms, int nu, uint64_t seed, const hepem_step_out& res,
                                  const Work& w, int32_t i, bool fromStageA, StepCount& cnt) {
  const hepem_track_state& src = fromStageA ? in : w.pre;
  const int type = in.type[i];
  Track t;
  Rng rng;
  load_track(src, i, t, rng, uniforms, nu, key_of(w, i, seed), type);
  use_prefill(w, i, rng);
  Physics P{T, rng, t};
  int32_t c0 = rng.cursor;
  if (PHASE == kPhaseHowFar) {
    P.el_howfar();
    store_limits64(w.limits, i, t, rng, type, w.gstep);
    cnt.uniforms += (uint32_t)(rng.cursor - c0);
    cnt.overflow += rng.overflow;
    cnt.fallback += 1;
    return;
  }
  if (PHASE == kPhasePerform) {
    const bool post = t.onBoundary;
    t.onBoundary = (w.limits.bits[i] & kLimPreBoundary) != 0;
    P.el_howfar();
    const double g = w.gstep[i];
    if (g != w.limits.d[kLProposed][i]) t.gstep = g;
    t.onBoundary = post;
    c0 = rng.cursor;
  } else {
    P.el_howfar();
  }
  const int key = P.el_perform_until_discrete();
  const int32_t cA = rng.cursor;
  const uint32_t ovA = rng.overflow;
  switch (key) {
    case kQIoniEm: interaction_fp64<kQIoniEm>(P); break;
    case kQIoniEp: interaction_fp64<kQIoniEp>(P); break;
    case kQBremSB: interaction_fp64<kQBremSB>(P); break;
    case kQBremRB: interaction_fp64<kQBremRB>(P); break;
    case kQAnnihFlight: interaction_fp64<kQAnnihFlight>(P); break;
    case kQAnnihRest: interaction_fp64<kQAnnihRest>(P); break;
    default: break;
  }
  store_track(in, out, res, i, t, rng, type, false);
  store_secondaries(res, i, t, 0);
  if (fromStageA) {
    // stage A counted nothing for this track
    cnt.steps += 1;
    cnt.uniforms += (uint32_t)(rng.cursor - c0);
    cnt.overflow += rng.overflow;
    if (t.winner >= 0 && t.winner < 4) count_inter(cnt, t.winner);
  } else {
    cnt.uniforms += (uint32_t)(rng.cursor - cA);
    cnt.overflow += (rng.overflow && !ovA) ? 1u : 0u;
  }
  cnt.secondaries += (uint32_t)(t.nsec > 2 ? 2 : t.nsec);
  cnt.fallback += 1;
}

// the FP64 step of a gamma whose FP32 stage A tripped: stage A as
// stage_a_gamma_kernel (MODE kStageFp64) and its interaction as stage_b_one,
// in one thread from the unchanged input state
__device__ void gamma_full_step(const DevTables& T, const hepem_track_state& in, const hepem_track_state& out,
                                const double* uniforms, int nu, uint64_t seed, const hepem_step_out& res,
                                const Work& w, int32_t i, StepCount& cnt) {
  Track t;
  Rng rng;
  load_track(in, i, t, rng, uniforms, nu, key_of(w, i, seed), 2);
  use_prefill(w, i, rng);
  const int32_t c0 = rng.cursor;
  t.isEl = false;
  Physics P{T, rng, t};
  P.gamma_howfar();
  int key = -1;
  if (t.onBoundary) {
    t.nia[0] -= t.gstep / t.mfp[0];
  } else {
    P.gamma_select();
    key = P.gamma_perform_until_interaction();
  }
  t.pstep = t.gstep;
  if (key == kQConversion) P.conversion();
  if (key == kQCompton) P.compton();
  if (key == kQPhotoelectric) P.photoelectric();
  if (key != -1) P.gamma_tracking_cut();
  store_track(in, out, res, i, t, rng, 2, false);
  store_secondaries(res, i, t, 0);
  cnt.steps += 1;
  cnt.uniforms += (uint32_t)(rng.cursor - c0);
  cnt.overflow += rng.overflow;
  if (t.winner >= 0 && t.winner < 4) count_inter(cnt, 4 + t.winner);
  cnt.secondaries += (uint32_t)(t.nsec > 2 ? 2 : t.nsec);
  cnt.fallback += 1;
}

template <int BS, int PHASE = kPhaseStep>
__global__ void __launch_bounds__(BS) final_fallback_kernel(const __grid_constant__ DevTables T,
                                                             const hepem_track_state in, const hepem_track_state out,
                                                             const double* __restrict__ uniforms, int nu,
                                                             uint64_t seed, const hepem_step_out res, const Work w,
                                                             hepem_step_counters* counters) {
  const int64_t total = w.counts[kFbCount];
  StepCount cnt = {};
  // every block takes an equal contiguous share of the list: the few (~1% of
  // the tracks), long FP64 steps spread over every SM's FP64 pipe instead of
  // filling the first blocks, and a share holds mostly one kind (the list is
  // appended kernel by kernel)
  const int64_t per = (total + gridDim.x - 1) / gridDim.x;
  const int64_t j0 = (int64_t)blockIdx.x * per;
  const int64_t j1 = j0 + per < total ? j0 + per : total;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const int32_t i = w.queue[kNumQueues][j];
    const int kind = w.fbKind[j];
    if (kind == kFbGammaA) {
      gamma_full_step(T, in, out, uniforms, nu, seed, res, w, i, cnt);
    } else if (kind == 0 || charged_model(kind - 1)) {
      charged_full_step<PHASE>(T, in, out, uniforms, nu, seed, res, w, i, kind == 0, cnt);
    } else {
      if (kind - 1 == kQConversion)
        stage_b_one<kQConversion, false>(T, in, out, uniforms, nu, seed, res, w, i, -1, cnt);
      else if (kind - 1 == kQCompton)
        stage_b_one<kQCompton, false>(T, in, out, uniforms, nu, seed, res, w, i, -1, cnt);
      cnt.fallback += 1;
    }
  }
  add_counters(cnt, counters);
}

#endif  // HEPEM_FP64_UNIT

// ---- host side -------------------------------------------------------------------------------
// The eleven stage kernels share one signature; each exists for 128, 256 and
// 512 threads per block, and the launch configuration picks one of them and
// the number of CTAs per SM for every kernel.
using StageFn = void (*)(DevTables, hepem_track_state, hepem_track_state, const double*, int, uint64_t,
                         hepem_step_out, Work, hepem_step_counters*);
constexpr int kBlockSizes[3] = {128, 256, 512};

static int bs_index(int bs) { return bs == 128 ? 0 : (bs == 512 ? 2 : 1); }

template <int BS>
static void stage_table(StageFn* f) {
  f[0] = stage_a_charged_kernel<BS, kStageFp64>;
  f[1] = stage_a_gamma_kernel<BS, kStageFp64>;
  f[2] = stage_b_kernel<0, BS, kStageFp64>;
  f[3] = stage_b_kernel<1, BS, kStageFp64>;
  f[4] = stage_b_kernel<2, BS, kStageFp64>;
  f[5] = stage_b_kernel<3, BS, kStageFp64>;
  f[6] = stage_b_kernel<4, BS, kStageFp64>;
  f[7] = stage_b_kernel<5, BS, kStageFp64>;
  f[8] = stage_b_kernel<6, BS, kStageFp64>;
  f[9] = stage_b_kernel<7, BS, kStageFp64>;
  f[10] = stage_b_kernel<8, BS, kStageFp64>;
}

// precision form: [kernel index] -> its FP32 kernel (null: FP64 only)
template <int BS>
static void mixed_table(StageFn* m) {
  for (int k = 0; k < kNumStageKernels; ++k) m[k] = nullptr;
  m[0] = stage_a_charged_kernel<BS, kStageMixed>;
  m[1] = stage_a_gamma_kernel<BS, kStageMixed>;
  m[2 + kQIoniEm] = stage_b_kernel<kQIoniEm, BS, kStageMixed>;
  m[2 + kQIoniEp] = stage_b_kernel<kQIoniEp, BS, kStageMixed>;
  m[2 + kQBremSB] = stage_b_kernel<kQBremSB, BS, kStageMixed>;
  m[2 + kQBremRB] = stage_b_kernel<kQBremRB, BS, kStageMixed>;
  m[2 + kQAnnihFlight] = stage_b_kernel<kQAnnihFlight, BS, kStageMixed>;
  m[2 + kQConversion] = stage_b_kernel<kQConversion, BS, kStageMixed>;
  m[2 + kQCompton] = stage_b_kernel<kQCompton, BS, kStageMixed>;
}

// the stage A kernels of the split step (256 threads): [phase - 1][0 e+-, 1 gamma]
template <int MODE>
static void split_table(StageFn (*f)[2]) {
  f[0][0] = stage_a_charged_kernel<256, MODE, kPhaseHowFar>;
  f[0][1] = stage_a_gamma_kernel<256, MODE, kPhaseHowFar>;
  f[1][0] = stage_a_charged_kernel<256, MODE, kPhasePerform>;
  f[1][1] = stage_a_gamma_kernel<256, MODE, kPhasePerform>;
}

#if !HEPEM_FP64_UNIT
// the precision form's stage kernels of this unit, for the FP64 unit's table
void mixed_stage_table(int b, StageFn* m) {
  if (b == 0) mixed_table<128>(m);
  else if (b == 2) mixed_table<512>(m);
  else mixed_table<256>(m);
}
void mixed_split_table(StageFn (*m)[2]) { split_table<kStageMixed>(m); }
#else
void mixed_stage_table(int b, StageFn* m);  // kernels_batched_mixed.cu
void mixed_split_table(StageFn (*m)[2]);

struct StageKernels {
  StageFn fn[3][kNumStageKernels];
  int occ[3][kNumStageKernels];  // resident CTAs per SM
  StageFn mixed[3][kNumStageKernels];  // precision form (null: FP64 only)
  int occMixed[3][kNumStageKernels];
  StageFn final_[3];                   // precision form: the FP64 fallback kernel
  int occFinal[3];
  // the split step (256 threads per block): stage A of HowFar / Perform,
  // [phase - 1][0 e+-, 1 gamma], FP64 and FP32; the fallback of each phase
  StageFn split[2][2], splitMixed[2][2], finalSplit[2];
  int occSplit[2][2], occSplitMixed[2][2], occFinalSplit[2];
};

static int occupancy_of(StageFn f, int bs) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, bs, 0) != cudaSuccess || per < 1) per = 1;
  return per;
}

// kernel table and occupancies (thread-safe one-time initialisation)
static const StageKernels& stage_kernels() {
  static const StageKernels K = [] {
    StageKernels r;
    stage_table<128>(r.fn[0]);
    stage_table<256>(r.fn[1]);
    stage_table<512>(r.fn[2]);
    mixed_stage_table(0, r.mixed[0]);
    mixed_stage_table(1, r.mixed[1]);
    mixed_stage_table(2, r.mixed[2]);
    r.final_[0] = final_fallback_kernel<128>;
    r.final_[1] = final_fallback_kernel<256>;
    r.final_[2] = final_fallback_kernel<512>;
    for (int b = 0; b < 3; ++b) {
      for (int k = 0; k < kNumStageKernels; ++k) {
        r.occ[b][k] = occupancy_of(r.fn[b][k], kBlockSizes[b]);
        r.occMixed[b][k] = r.mixed[b][k] ? occupancy_of(r.mixed[b][k], kBlockSizes[b]) : 0;
      }
      r.occFinal[b] = occupancy_of(r.final_[b], kBlockSizes[b]);
    }
    split_table<kStageFp64>(r.split);
    mixed_split_table(r.splitMixed);
    r.finalSplit[0] = final_fallback_kernel<256, kPhaseHowFar>;
    r.finalSplit[1] = final_fallback_kernel<256, kPhasePerform>;
    for (int ph = 0; ph < 2; ++ph) {
      for (int q = 0; q < 2; ++q) {
        r.occSplit[ph][q] = occupancy_of(r.split[ph][q], 256);
        r.occSplitMixed[ph][q] = occupancy_of(r.splitMixed[ph][q], 256);
      }
      r.occFinalSplit[ph] = occupancy_of(r.finalSplit[ph], 256);
    }
    return r;
  }();
  return K;
}

int stage_occupancy(int kernel, int block) { return stage_kernels().occ[bs_index(block)][kernel]; }

LaunchCfg default_launch_cfg() {
  LaunchCfg c;
  for (int k = 0; k < kNumStageKernels; ++k) {
    c.block[k] = 256;
    c.ctasPerSM[k] = 0;
  }
  c.sortEBins = kMaxSortEBins;
  return c;
}

bool valid_launch_cfg(const LaunchCfg& c) {
  for (int k = 0; k < kNumStageKernels; ++k) {
    if (c.block[k] != 128 && c.block[k] != 256 && c.block[k] != 512) return false;
    if (c.ctasPerSM[k] < 0 || c.ctasPerSM[k] > 64) return false;
  }
  return c.sortEBins == 8 || c.sortEBins == 16 || c.sortEBins == 32;
}

cudaError_t launch_step_batched(const DevTables& T, int64_t n, const hepem_track_state& in,
                                const hepem_track_state& out, const double* uniforms, int nu, uint64_t seed,
                                const hepem_step_out& res, hepem_step_counters* counters, void* workspace,
                                cudaStream_t s, int sms, const BatchOpts& o) {
  if (n <= 0) return cudaSuccess;
  const StageKernels& K = stage_kernels();
  static const LaunchCfg kDefault = default_launch_cfg();
  const LaunchCfg& cfg = o.cfg ? *o.cfg : kDefault;
  Work w = carve(workspace, n);
  w.seeds = o.seeds;
  w.pre = in;
  w.preCopy = false;
  w.oneChargedKey = o.mixed;
  if (o.mixed && o.preState) {
    w.pre = *o.preState;
    w.preCopy = true;
  }
  w.phase = o.phase;
  w.gstep = o.gstep;
  w.limits = o.limits;
  // The FP64 stages are bound by the FP64 pipe and gain from warps of one
  // couple and energy range; the precision form's stages are bound by the
  // latency of their state gathers and gain more from keeping each particle
  // list in batch order (neighbouring tracks share memory sectors: stage A
  // of e+- takes 2.2x less time): it sorts into two lists only, e+- (e- and
  // e+ together: the step 4% faster than with an e+ list of its own) and
  // gammas.
  const int ncb = o.mixed ? 1 : (T.nCouples < kSortCoupleBins ? T.nCouples : kSortCoupleBins);
  const int neb = o.mixed ? 1 : cfg.sortEBins;
  const int nkeys = 3 * ncb * neb;
  cudaError_t e = cudaMemsetAsync(w.counts, 0, 64 * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.hist, 0, nkeys * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  int k = 0;
  auto mark = [&]() {
    if (o.ev) cudaEventRecord(o.ev[k++], s);
  };
  const int64_t blocks = (n + 255) / 256;
  const int gC = (int)(blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8);
  w.active = o.active;
  w.nDev = o.nDev;
  TraceStages trace(n);
  if (o.prefill && wants_prefill(n, nu)) {
    trace.next("prefill");
    double* pre = static_cast<double*>(o.prefill);
    int32_t* pos = o.active
                       ? reinterpret_cast<int32_t*>(static_cast<uint8_t*>(o.prefill) + prefill_bytes(n, 0))
                       : nullptr;
    const int64_t pb = (n * (kPrefill / 2) + 255) / 256;
    const int gP = (int)(pb < (int64_t)sms * 16 ? pb : (int64_t)sms * 16);
    prefill_kernel<<<gP, 256, 0, s>>>(n, o.active, o.nDev, in, o.seeds, seed, pre, pos);
    w.prefill = pre;
    w.prefillPos = pos;
  }
  trace.next("sort");
  mark();
  sort_hist_kernel<<<gC, 256, nkeys * sizeof(uint32_t), s>>>(T, n, o.active, in, out, res, w, ncb, neb, counters);
  sort_scan_kernel<<<1, 1024, 0, s>>>(w, ncb, neb);
  const int64_t nt = (n + 256 * kScatterItems - 1) / (256 * kScatterItems);
  const int gS = (int)(nt < (int64_t)sms * 8 ? nt : (int64_t)sms * 8);
  sort_scatter_kernel<<<gS, 256, nkeys * sizeof(uint32_t), s>>>(T, n, o.active, in, w, ncb, neb);
  mark();
  // the stage kernels: with a table window, launched with it as a launch
  // attribute (the caller's stream is left as it is)
  cudaError_t le = cudaSuccess;
  auto stage = [&](StageFn f, int grid, int block, cudaStream_t st) {
    if (o.tableBytes == 0) {
      f<<<grid, block, 0, st>>>(T, in, out, uniforms, nu, seed, res, w, counters);
      return;
    }
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[0].val.accessPolicyWindow.base_ptr = const_cast<void*>(o.tableBase);
    attr[0].val.accessPolicyWindow.num_bytes = o.tableBytes;
    attr[0].val.accessPolicyWindow.hitRatio = o.tableHitRatio;
    attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(block);
    lc.dynamicSmemBytes = 0;
    lc.stream = st;
    lc.attrs = attr;
    lc.numAttrs = 1;
    const cudaError_t x = cudaLaunchKernelEx(&lc, f, T, in, out, uniforms, nu, seed, res, w, counters);
    if (le == cudaSuccess) le = x;
  };
  // stage kernel q (0, 1: stage A of e+- / gammas, of the phase; 2..: the
  // interaction queues) on stream st: the precision form's FP32 kernel where
  // one exists, else the FP64 one, at the configured block size and CTAs per SM
  auto launch_q = [&](int q, cudaStream_t st) {
    trace.next(stage_name(q + 1));
    if (q < 2 && o.phase != kPhaseStep) {
      const int ph = o.phase - 1;
      if (o.mixed)
        stage(K.splitMixed[ph][q], sms * K.occSplitMixed[ph][q], 256, st);
      else
        stage(K.split[ph][q], sms * K.occSplit[ph][q], 256, st);
      return;
    }
    const int b = bs_index(cfg.block[q]);
    const bool fp32 = o.mixed && K.mixed[b][q];
    const int occ = fp32 ? K.occMixed[b][q] : K.occ[b][q];
    const int per = cfg.ctasPerSM[q] > 0 && cfg.ctasPerSM[q] < occ ? cfg.ctasPerSM[q] : occ;
    stage(fp32 ? K.mixed[b][q] : K.fn[b][q], sms * per, kBlockSizes[b], st);
  };
  // the precision form's FP64 fallback kernel of the phase (after every stage)
  auto launch_final = [&](cudaStream_t st) {
    trace.next("fp64_fallback");
    if (o.phase == kPhaseHowFar)
      stage(K.finalSplit[0], sms * K.occFinalSplit[0], 256, st);
    else if (o.phase == kPhasePerform)
      stage(K.finalSplit[1], sms * K.occFinalSplit[1], 256, st);
    else
      stage(K.final_[1], sms * K.occFinal[1], 256, st);
  };
  SideStreams* sd = o.ev ? nullptr : o.side;
  if (!sd) {
    // one stream, stage by stage (the stage events of hepem_profile_stages
    // time each stage alone)
    const int qEnd = o.phase == kPhaseHowFar ? 2 : kNumStageKernels;
    for (int q = 0; q < qEnd; ++q) {
      launch_q(q, s);
      if (o.mixed && q == kNumStageKernels - 1) launch_final(s);
      mark();
    }
    if (o.phase == kPhaseHowFar && o.mixed) launch_final(s);
  } else {
    // Independent stages overlap: each kernel's last, slowest tracks leave
    // its SMs idle, which the kernels on the other streams fill.  The gamma
    // chain (stage A, conversion, Compton, photoelectric) runs on side
    // stream 0 beside the e+- chain; after the e+- stage A the two
    // bremsstrahlung queues go to side streams 1 and 2 and the other e+-
    // queues stay on the caller's stream, which then waits for all three
    // and runs the FP64 fallback.  The enqueue holds the lock, so that
    // another thread's use of the same side streams and events cannot
    // interleave with these waits.
    std::lock_guard<std::mutex> lock(sd->mu);
    auto fork = [&](cudaEvent_t ev, cudaStream_t to) {
      if (cudaEventRecord(ev, s) == cudaSuccess) cudaStreamWaitEvent(to, ev, 0);
    };
    auto join = [&](cudaStream_t from, cudaEvent_t ev) {
      if (cudaEventRecord(ev, from) == cudaSuccess) cudaStreamWaitEvent(s, ev, 0);
    };
    fork(sd->ev[0], sd->st[0]);
    launch_q(0, s);
    launch_q(1, sd->st[0]);
    if (o.phase == kPhaseHowFar) {
      join(sd->st[0], sd->ev[2]);
      if (o.mixed) launch_final(s);
    } else {
      if (cudaEventRecord(sd->ev[1], s) == cudaSuccess) {
        cudaStreamWaitEvent(sd->st[1], sd->ev[1], 0);
        cudaStreamWaitEvent(sd->st[2], sd->ev[1], 0);
      }
      launch_q(2 + kQBremSB, sd->st[1]);
      launch_q(2 + kQBremRB, sd->st[2]);
      for (int q = 2; q < kNumStageKernels; ++q) {
        const int Q = q - 2;
        if (Q == kQBremSB || Q == kQBremRB) continue;
        // queues before kQConversion are filled by the e+- stage A, the rest by the gamma one
        launch_q(q, Q < kQConversion ? s : sd->st[0]);
      }
      join(sd->st[0], sd->ev[2]);
      join(sd->st[1], sd->ev[3]);
      join(sd->st[2], sd->ev[4]);
      if (o.mixed) launch_final(s);
    }
  }
  const cudaError_t e2 = cudaGetLastError();
  return le != cudaSuccess ? le : e2;
}

// ---- sub-batches: index list and per-track RNG keys --------------------------------------
__global__ void __launch_bounds__(256) subbatch_index_kernel(const hepem_subbatch* __restrict__ batches,
                                                             const int64_t* __restrict__ prefix, int nb,
                                                             int64_t total, int32_t* __restrict__ active,
                                                             uint64_t* __restrict__ keys) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nb - 1;  // prefix[lo] <= p < prefix[lo + 1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (prefix[mid] <= p) lo = mid; else hi = mid - 1;
    }
    const int64_t i = batches[lo].offset + (p - prefix[lo]);
    active[p] = (int32_t)i;
    keys[i] = batches[lo].seed;
  }
}

cudaError_t launch_subbatch_index(const hepem_subbatch* batches, const int64_t* prefix, int nb, int64_t total,
                                  int32_t* active, uint64_t* keys, cudaStream_t s, int sms) {
  if (total <= 0 || nb <= 0) return cudaSuccess;
  const int64_t blocks = (total + 255) / 256;
  const int g = (int)(blocks < (int64_t)sms * 16 ? blocks : (int64_t)sms * 16);
  subbatch_index_kernel<<<g, 256, 0, s>>>(batches, prefix, nb, total, active, keys);
  return cudaGetLastError();
}

// ---- 4. per-model sampling (interaction unit tests and distribution checks) -------------
// n independent draws of one interaction model at a fixed energy and couple:
// draw i is a track with id i, direction +z and the pure Philox stream of
// (seed, i).  MIXED: the FP32 model of the precision form, a draw that trips
// a guard is redone by the FP64 model (counted in nFallback).
__device__ __forceinline__ void sample_init(Track& t, Rng& rng, int model, double ekin, int imc, int64_t i,
                                            uint64_t seed) {
  t.imc = imc;
  t.setE(ekin);
  t.dir[0] = 0.0; t.dir[1] = 0.0; t.dir[2] = 1.0;
  t.isEl = model != kSampleBhabha;
  t.flags = 0;
  t.nsec = 0;
  t.edep = 0.0;
  t.peXS = 0.0;
  rng.u = nullptr;
  rng.n = 0;
  rng.cursor = 0;
  rng.id = (int32_t)i;
  rng.overflow = 0u;
  rng.seed = seed;
  rng.gaussValid = false;
  rng.gaussValue = 0.0;
}

template <class M>
__device__ __forceinline__ void sample_run(M& m, int model) {
  switch (model) {
    case kSampleSB: m.brem(true); break;
    case kSampleRB: m.brem(false); break;
    case kSampleMoller:
    case kSampleBhabha: m.ioni(); break;
    case kSampleCompton: m.compton(); break;
    case kSampleConversion: m.conversion(); break;
    default: break;
  }
}

__device__ __forceinline__ double sample_value(const Track& t, int model) {
  if (model == kSampleCompton) return t.e;            // scattered photon energy
  return t.nsec > 0 ? t.sec[0].e : 0.0;               // photon, delta ray, or pair electron
}

template <bool MIXED>
__global__ void __launch_bounds__(256) sample_kernel(const __grid_constant__ DevTables T, int model, int64_t n,
                                                     double ekin, int imc, uint64_t seed, double* __restrict__ out,
                                                     unsigned long long* nFallback) {
  uint32_t fb = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    Track t;
    Rng rng;
    sample_init(t, rng, model, ekin, imc, i, seed);
    bool redo = !MIXED;
    if (MIXED) {
      MixedB mb{T, rng, t, false};
      mb.dirExact = true;
      sample_run(mb, model);
      if (mb.trip) {
        redo = true;
        ++fb;
        sample_init(t, rng, model, ekin, imc, i, seed);
      }
    }
    if (redo) {
      Physics P{T, rng, t};
      sample_run(P, model);
    }
    out[i] = sample_value(t, model);
  }
  if (MIXED && nFallback) {
    const uint32_t w = __reduce_add_sync(0xFFFFFFFFu, fb);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(nFallback, (unsigned long long)w);
  }
}

cudaError_t launch_sample(const DevTables& T, int model, int mixed, int64_t n, double ekin, int imc, uint64_t seed,
                          double* out, unsigned long long* nFallback, cudaStream_t s, int sms) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 255) / 256;
  const int g = (int)(blocks < (int64_t)sms * 16 ? blocks : (int64_t)sms * 16);
  if (mixed)
    sample_kernel<true><<<g, 256, 0, s>>>(T, model, n, ekin, imc, seed, out, nFallback);
  else
    sample_kernel<false><<<g, 256, 0, s>>>(T, model, n, ekin, imc, seed, out, nFallback);
  return cudaGetLastError();
}
#endif  // HEPEM_FP64_UNIT

// ---- 5. the quantities of the reference's device tests -----------------------------------
// One function of the path per kernel, on given energies, couples and
// uniforms: the step-limit cross sections of e+- (G4HepEmElectronManager.icc:
// 534-599, testing/ElectronXSections/src/ResMacXSecs.cu:16-33), the target
// element of brem (G4HepEmElectronInteractionBrem SelectTargetAtom,
// testing/ElectronTargetElementSelector/src/ElemSelector.cu:14-30) and of
// pair production (G4HepEmGammaInteractionConversion SelectTargetAtom,
// testing/GammaTargetElementSelector/src/GammaElemSelector.cu:14-27), the
// gamma total cross section and the interaction it selects
// (G4HepEmGammaManager.icc:108-219, testing/GammaXSections/src/
// GammaMacXSecs.cu:20-30).  MIXED: the FP32 code of the precision form, where
// a selection too close to call is made again in FP64 as in the step.
template <bool MIXED>
__global__ void __launch_bounds__(256) probe_kernel(const __grid_constant__ DevTables T, const ProbeArgs a) {
  const double nan = __longlong_as_double(0x7FF8000000000000LL);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double e = a.ekin[i];
    const int c = a.imc[i];
    if (track_input_bad(T, 0, c, e)) {
      if (a.kind == kProbeElXs || a.kind == kProbeGammaXs)
        for (int k = 0; k < 5; ++k)
          if (a.out[k]) a.out[k][i] = nan;
      if (a.iout) a.iout[i] = -1;
      continue;
    }
    const int imat = ld(&T.couples[c].mat);
    Track t;
    Rng rng;
    t.imc = c;
    t.setE(e);
    t.isEl = !a.positron;
    t.flags = 0;
    t.nsec = 0;
    t.onBoundary = false;
    t.nia[0] = 1.0;
    t.peXS = 0.0;
    rng.u = a.urnd ? a.urnd + i : nullptr;
    rng.n = a.urnd ? 1 : 0;
    rng.cursor = 0;
    rng.id = (int32_t)i;
    rng.overflow = 0u;
    rng.seed = 0;
    rng.gaussValid = false;
    rng.gaussValue = 0.0;
    if (a.kind == kProbeElXs) {
      const DevElData& d = T.el[a.positron ? 1 : 0];
      double v[5];
      if (MIXED) {
        const DevElData32& f = T.el32[a.positron ? 1 : 0];
        const float ef = d2f(e), lef = logf(ef);
        v[0] = (double)rest_macxs_stepping32(d, f, c, e, ef, lef, true);
        v[1] = (double)rest_macxs_stepping32(d, f, c, e, ef, lef, false);
        v[2] = a.positron ? (double)annih_macxs32(0.8f * ef, ld(&T.mats32[imat].elDensity)) : 0.0;
        v[3] = (double)nuc_macxs32(d, f, imat, e, ef, lef);
        v[4] = (double)transport_mfp32(f, d.nLoss, imat, ef, lef);
      } else {
        const double le = vdt_log(e);
        v[0] = rest_macxs_stepping(d, c, e, le, true);
        v[1] = rest_macxs_stepping(d, c, e, le, false);
        v[2] = a.positron ? annih_macxs(0.8 * e, ld(&T.mats[imat].elDensity)) : 0.0;
        v[3] = nuc_macxs(d, imat, e, le);
        v[4] = transport_mfp(d, imat, e, le);
      }
      for (int k = 0; k < 5; ++k) a.out[k][i] = v[k];
    } else if (a.kind == kProbeBremTarget || a.kind == kProbeConvTarget) {
      int k = 0;
      if (ld(&T.mats[imat].nElem) > 1) {
        const double u = a.urnd[i];
        bool redo = !MIXED;
        if (MIXED) {
          MixedB M{T, rng, t, false};
          k = a.kind == kProbeBremTarget ? M.select_brem_target(e, f2d(logf(d2f(e))), u, a.sb ? 1 : 2)
                                         : M.conv_target32(imat, e, u);
          redo = M.trip;
        }
        if (redo) {
          Physics P{T, rng, t};
          k = a.kind == kProbeBremTarget ? P.select_brem_target(e, vdt_log(e), u, a.sb ? 1 : 2)
                                         : P.conv_target(imat, e, vdt_log(e), u);
        }
      }
      a.iout[i] = k;
    } else {
      double tot;
      if (MIXED) {
        MixedG G{T, rng, t, false};
        GammaLimit32 q;
        G.howfar(q);
        tot = (double)q.tot;
        G.perform(q, 0.f);
      } else {
        Physics P{T, rng, t};
        tot = P.gamma_total_xs();
        t.mfp[0] = tot > 0. ? 1. / tot : kLarge;
        P.gamma_select();
      }
      a.out[0][i] = tot;
      a.out[1][i] = t.winner == 2 ? t.peXS : 0.0;
      a.iout[i] = t.winner;
    }
  }
}

static int probe_grid(int64_t n, int sms) {
  const int64_t b = (n + 255) / 256;
  return (int)(b < (int64_t)sms * 16 ? (b > 0 ? b : 1) : (int64_t)sms * 16);
}

#if HEPEM_FP64_UNIT
cudaError_t launch_probe_mixed(const DevTables& T, const ProbeArgs& a, cudaStream_t s, int sms);
cudaError_t launch_probe(const DevTables& T, const ProbeArgs& a, int mixed, cudaStream_t s, int sms) {
  if (a.n <= 0) return cudaSuccess;
  if (mixed) return launch_probe_mixed(T, a, s, sms);
  probe_kernel<false><<<probe_grid(a.n, sms), 256, 0, s>>>(T, a);
  return cudaGetLastError();
}
#else
cudaError_t launch_probe_mixed(const DevTables& T, const ProbeArgs& a, cudaStream_t s, int sms) {
  probe_kernel<true><<<probe_grid(a.n, sms), 256, 0, s>>>(T, a);
  return cudaGetLastError();
}
#endif

}  // namespace hepem

// diagnostics exports: the trip counters of the precision form's kernels live
// in the FP32 unit, the trace rows in both (FP64 row 0 here, row 1 there)
#if defined(HEPEM_TRIP_SITES) && !HEPEM_FP64_UNIT
extern "C" int hepem_debug_trip_sites(unsigned long long* out, int reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, hepem::g_tripSites, sizeof(unsigned long long) * 4096);
  if (e == cudaSuccess && reset) {
    static const unsigned long long zero[4096] = {};
    e = cudaMemcpyToSymbol(hepem::g_tripSites, zero, sizeof(zero));
  }
  return e == cudaSuccess ? 0 : 3;
}
#endif

#ifdef HEPEM_TRACE
#if HEPEM_FP64_UNIT
extern "C" int hepem_debug_trace(int id, double* out128) {
#else
extern "C" int hepem_debug_trace_mixed(int id, double* out128) {
#endif
  if (id >= -1) {
    static const double zero[128] = {};
    if (cudaMemcpyToSymbol(hepem::g_trace, zero, sizeof(zero)) != cudaSuccess) return 3;
    return cudaMemcpyToSymbol(hepem::g_traceId, &id, sizeof(int)) == cudaSuccess ? 0 : 3;
  }
  return cudaMemcpyFromSymbol(out128, hepem::g_trace, sizeof(double) * 128) == cudaSuccess ? 0 : 3;
}
#endif
