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
#include "step_io.cuh"

namespace hepem {

// Tracks are ordered by a sort key (particle, couple bin, energy bin) with a
// counting sort, so that the warps of a stage hold tracks of one particle in
// one material at similar energies and take the same branches.
constexpr int kMaxSortEBins = 32;   // log2(E) bins over 1 keV - 100 TeV (the launch configuration picks 8..32)
constexpr int kSortCoupleBins = 64; // couples beyond 64 share bins (imc % 64)
constexpr int kMaxSortKeys = 3 * kSortCoupleBins * kMaxSortEBins;

struct Work {
  uint32_t* counts;               // [0..2] e-, e+, gamma tracks, [3..3+kNumQueues) queues
  uint32_t* hist;                 // [kMaxSortKeys] tracks per sort key
  uint32_t* cursor;               // [kMaxSortKeys] scatter cursors
  int32_t* perm;                  // [n] valid tracks in sort-key order
  int32_t* queue[kNumQueues];
  double* peXS;                   // parallel to queue[kQPhotoelectric]
  const uint64_t* seeds;          // per-track RNG keys (serving), or null: one key per call
};

__device__ __forceinline__ uint64_t key_of(const Work& w, int64_t i, uint64_t seed) {
  return w.seeds ? w.seeds[i] : seed;
}

const char* stage_name(int i) {
  static const char* names[kNumStageEvents - 1] = {
      "sort", "stage_a_charged", "stage_a_gamma", "ioni_e-", "ioni_e+", "brem_sb", "brem_rb",
      "annihilation_in_flight", "annihilation_at_rest", "conversion", "compton", "photoelectric"};
  return (i >= 0 && i < kNumStageEvents - 1) ? names[i] : "";
}

static size_t rnd(size_t b) { return (b + 255) / 256 * 256; }

size_t batched_workspace_bytes(int64_t n) {
  return rnd(64 * sizeof(uint32_t)) + 2 * rnd(kMaxSortKeys * sizeof(uint32_t)) +
         (1 + kNumQueues) * rnd(sizeof(int32_t) * (size_t)n) + rnd(sizeof(double) * (size_t)n);
}

static Work carve(void* ws, int64_t n) {
  uint8_t* p = static_cast<uint8_t*>(ws);
  Work w;
  w.counts = reinterpret_cast<uint32_t*>(p);
  p += rnd(64 * sizeof(uint32_t));
  w.hist = reinterpret_cast<uint32_t*>(p);
  p += rnd(kMaxSortKeys * sizeof(uint32_t));
  w.cursor = reinterpret_cast<uint32_t*>(p);
  p += rnd(kMaxSortKeys * sizeof(uint32_t));
  w.perm = reinterpret_cast<int32_t*>(p);
  p += rnd(sizeof(int32_t) * (size_t)n);
  for (int k = 0; k < kNumQueues; ++k) {
    w.queue[k] = reinterpret_cast<int32_t*>(p);
    p += rnd(sizeof(int32_t) * (size_t)n);
  }
  w.peXS = reinterpret_cast<double*>(p);
  return w;
}

__device__ __forceinline__ int sort_key(int type, int imc, double e, int ncb, int neb) {
  // Gammas keep their batch order (one key): their stage is light on FP64 and
  // latency bound, so coalesced loads matter more there than branch coherence.
  if (type == 2) return 2 * ncb * neb;
  // log2(1 keV / MeV) = -9.9658, log2(100 TeV / 1 keV) = 36.5412
  int eb = (int)((__log2f((float)e) + 9.965784f) * ((float)neb / 36.541209f));
  eb = eb < 0 ? 0 : (eb >= neb ? neb - 1 : eb);
  return ((type * ncb) + (imc % ncb)) * neb + eb;
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
  StepCount cnt = {};
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = active ? (int64_t)active[j] : j;
    const int type = in.type[i];
    const int imc = in.imc[i];
    const double e = in.ekin[i];
    if (track_input_bad(T, type, imc, e)) {
      // pass the track through unchanged, flagged
      Track t;
      Rng rng;
      load_track(in, i, t, rng, nullptr, 0, 0, 2);
      t.flags = kFlagBadInput;
      store_track(in, out, res, i, t, rng, 2, true);
      res.n_sec[i] = 0;
      cnt.steps += 1;
    } else {
      atomicAdd(&sh[sort_key(type, imc, e, ncb, neb)], 1u);
    }
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

__global__ void __launch_bounds__(256) sort_scatter_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                           const int32_t* __restrict__ active,
                                                           const hepem_track_state in, const Work w, int ncb,
                                                           int neb) {
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    const int64_t i = (active && j < n) ? (int64_t)active[j] : j;
    int key = -1;
    if (j < n) {
      const int type = in.type[i];
      const int imc = in.imc[i];
      const double e = in.ekin[i];
      if (!track_input_bad(T, type, imc, e)) key = sort_key(type, imc, e, ncb, neb);
    }
    // warp-aggregated: one atomic per distinct key in the warp
    const unsigned same = __match_any_sync(0xFFFFFFFFu, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(same) - 1;
    uint32_t base2 = 0;
    if (key >= 0 && lane == leader) base2 = atomicAdd(&w.cursor[key], (uint32_t)__popc(same));
    base2 = __shfl_sync(0xFFFFFFFFu, base2, leader);
    if (key >= 0) w.perm[base2 + __popc(same & ((1u << lane) - 1u))] = (int32_t)i;
  }
}

// ---- 2. stage A -----------------------------------------------------------------------
template <int BS>
__global__ void __launch_bounds__(BS) stage_a_charged_kernel(const __grid_constant__ DevTables T,
                                                              const hepem_track_state in, const hepem_track_state out,
                                                              const double* __restrict__ uniforms, int nu,
                                                              uint64_t seed, const hepem_step_out res, const Work w,
                                                              hepem_step_counters* counters) {
  const uint32_t nEm = w.counts[0], nEp = w.counts[1];
  const int64_t total = (int64_t)nEm + nEp;
  StepCount cnt = {};
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < total; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = base + threadIdx.x;
    int key = -1;
    int32_t idx = 0;
    if (j < total) {
      idx = w.perm[j];
      const int type = j < nEm ? 0 : 1;
      Track t;
      Rng rng;
      load_track(in, idx, t, rng, uniforms, nu, key_of(w, idx, seed), type);
      const int32_t c0 = rng.cursor;
      Physics P{T, rng, t};
      P.el_howfar();
      key = P.el_perform_until_discrete();
      store_track(in, out, res, idx, t, rng, type, false);
      res.n_sec[idx] = 0;
      cnt.steps += 1;
      cnt.uniforms += (uint32_t)(rng.cursor - c0);
      cnt.overflow += rng.overflow;
      if (t.winner >= 0 && t.winner < 4) cnt.inter[t.winner] += 1;
    }
    warp_push(key, idx, w.queue, w.counts + 3);
  }
  add_counters(cnt, counters);
}

template <int BS>
__global__ void __launch_bounds__(BS) stage_a_gamma_kernel(const __grid_constant__ DevTables T,
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
    if (j < total) {
      idx = w.perm[w.counts[0] + w.counts[1] + j];
      Track t;
      Rng rng;
      load_track(in, idx, t, rng, uniforms, nu, key_of(w, idx, seed), 2);
      const int32_t c0 = rng.cursor;
      Physics P{T, rng, t};
      t.isEl = false;
      P.gamma_howfar();
      if (t.onBoundary) {
        t.nia[0] -= t.gstep / t.mfp[0];
      } else {
        P.gamma_select();
        key = P.gamma_perform_until_interaction();
        if (key == -2) {
          P.gamma_tracking_cut();
          key = -1;
        }
      }
      t.pstep = t.gstep;
      pe = t.peXS;
      store_track(in, out, res, idx, t, rng, 2, false);
      res.n_sec[idx] = 0;
      cnt.steps += 1;
      cnt.uniforms += (uint32_t)(rng.cursor - c0);
      cnt.overflow += rng.overflow;
      if (t.winner >= 0 && t.winner < 4) cnt.inter[4 + t.winner] += 1;
    }
    warp_push(key, idx, w.queue, w.counts + 3, pe, w.peXS, kQPhotoelectric);
  }
  add_counters(cnt, counters);
}

// ---- 3. stage B: one interaction model per kernel ------------------------------------------
template <int Q, int BS>
__global__ void __launch_bounds__(BS) stage_b_kernel(const __grid_constant__ DevTables T,
                                                      const hepem_track_state in, const hepem_track_state out,
                                                      const double* __restrict__ uniforms, int nu, uint64_t seed,
                                                      const hepem_step_out res, const Work w,
                                                      hepem_step_counters* counters) {
  const int64_t total = w.counts[3 + Q];
  const int32_t* q = w.queue[Q];
  StepCount cnt = {};
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < total; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = q[j];
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
    rng.cursor = out.rng_cursor[i];
    rng.id = in.id[i];
    rng.overflow = 0u;
    rng.seed = key_of(w, i, seed);
    rng.gaussValid = out.gauss_valid[i] != 0;
    rng.gaussValue = out.gauss_value[i];
    const int32_t c0 = rng.cursor;
    Physics P{T, rng, t};
    if (Q == kQIoniEm || Q == kQIoniEp) P.ioni();
    if (Q == kQBremSB) P.brem(true);
    if (Q == kQBremRB) P.brem(false);
    if (Q == kQAnnihFlight) P.annihilate_in_flight();
    if (Q == kQAnnihRest) P.annihilate_at_rest();
    if (Q >= kQConversion) {
      t.edep = 0.0;
      t.peXS = (Q == kQPhotoelectric) ? w.peXS[j] : 0.0;
      if (Q == kQConversion) P.conversion();
      if (Q == kQCompton) P.compton();
      if (Q == kQPhotoelectric) P.photoelectric();
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
  }
  add_counters(cnt, counters);
}

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
  f[0] = stage_a_charged_kernel<BS>;
  f[1] = stage_a_gamma_kernel<BS>;
  f[2] = stage_b_kernel<0, BS>;
  f[3] = stage_b_kernel<1, BS>;
  f[4] = stage_b_kernel<2, BS>;
  f[5] = stage_b_kernel<3, BS>;
  f[6] = stage_b_kernel<4, BS>;
  f[7] = stage_b_kernel<5, BS>;
  f[8] = stage_b_kernel<6, BS>;
  f[9] = stage_b_kernel<7, BS>;
  f[10] = stage_b_kernel<8, BS>;
}

struct StageKernels {
  StageFn fn[3][kNumStageKernels];
  int occ[3][kNumStageKernels];  // resident CTAs per SM
};

// kernel table and occupancies (thread-safe one-time initialisation)
static const StageKernels& stage_kernels() {
  static const StageKernels K = [] {
    StageKernels r;
    stage_table<128>(r.fn[0]);
    stage_table<256>(r.fn[1]);
    stage_table<512>(r.fn[2]);
    for (int b = 0; b < 3; ++b)
      for (int k = 0; k < kNumStageKernels; ++k) {
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, r.fn[b][k], kBlockSizes[b], 0) != cudaSuccess ||
            per < 1)
          per = 1;
        r.occ[b][k] = per;
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
  const int ncb = T.nCouples < kSortCoupleBins ? T.nCouples : kSortCoupleBins;
  const int neb = cfg.sortEBins;
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
  mark();
  sort_hist_kernel<<<gC, 256, nkeys * sizeof(uint32_t), s>>>(T, n, o.active, in, out, res, w, ncb, neb, counters);
  sort_scan_kernel<<<1, 1024, 0, s>>>(w, ncb, neb);
  sort_scatter_kernel<<<gC, 256, 0, s>>>(T, n, o.active, in, w, ncb, neb);
  mark();
  for (int q = 0; q < kNumStageKernels; ++q) {
    const int b = bs_index(cfg.block[q]);
    const int occ = K.occ[b][q];
    const int per = cfg.ctasPerSM[q] > 0 && cfg.ctasPerSM[q] < occ ? cfg.ctasPerSM[q] : occ;
    K.fn[b][q]<<<sms * per, kBlockSizes[b], 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
    mark();
  }
  return cudaGetLastError();
}

}  // namespace hepem
