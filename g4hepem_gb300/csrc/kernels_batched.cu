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
constexpr int kSortEBins = 32;      // log2(E) bins over 1 keV - 100 TeV
constexpr int kSortCoupleBins = 64; // couples beyond 64 share bins (imc % 64)
constexpr int kMaxSortKeys = 3 * kSortCoupleBins * kSortEBins;

struct Work {
  uint32_t* counts;               // [0..2] e-, e+, gamma tracks, [3..3+kNumQueues) queues
  uint32_t* hist;                 // [kMaxSortKeys] tracks per sort key
  uint32_t* cursor;               // [kMaxSortKeys] scatter cursors
  int32_t* perm;                  // [n] valid tracks in sort-key order
  int32_t* queue[kNumQueues];
  double* peXS;                   // parallel to queue[kQPhotoelectric]
};

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

__device__ __forceinline__ int sort_key(int type, int imc, double e, int ncb) {
  // Gammas keep their batch order (one key): their stage is light on FP64 and
  // latency bound, so coalesced loads matter more there than branch coherence.
  if (type == 2) return 2 * ncb * kSortEBins;
  // log2(1 keV / MeV) = -9.9658, log2(100 TeV / 1 keV) = 36.5412
  int eb = (int)((__log2f((float)e) + 9.965784f) * (kSortEBins / 36.541209f));
  eb = eb < 0 ? 0 : (eb >= kSortEBins ? kSortEBins - 1 : eb);
  return ((type * ncb) + (imc % ncb)) * kSortEBins + eb;
}

// ---- 1. sort: histogram, scan, scatter ----------------------------------------------
__global__ void __launch_bounds__(256) sort_hist_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                        const hepem_track_state in, const hepem_track_state out,
                                                        const hepem_step_out res, const Work w, int ncb,
                                                        hepem_step_counters* counters) {
  extern __shared__ uint32_t sh[];
  const int nkeys = 3 * ncb * kSortEBins;
  for (int k = threadIdx.x; k < nkeys; k += blockDim.x) sh[k] = 0;
  __syncthreads();
  StepCount cnt = {};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
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
      atomicAdd(&sh[sort_key(type, imc, e, ncb)], 1u);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nkeys; k += blockDim.x)
    if (sh[k]) atomicAdd(&w.hist[k], sh[k]);
  add_counters(cnt, counters);
}

// one block: exclusive scan of the histogram into the scatter cursors, and
// the number of tracks of each particle type
__global__ void __launch_bounds__(1024) sort_scan_kernel(const Work w, int ncb) {
  __shared__ uint32_t partial[1024];
  const int nkeys = 3 * ncb * kSortEBins;
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
    for (int k = threadIdx.x * ncb * kSortEBins; k < (threadIdx.x + 1) * ncb * kSortEBins; ++k) c += w.hist[k];
    w.counts[threadIdx.x] = c;
  }
}

__global__ void __launch_bounds__(256) sort_scatter_kernel(const __grid_constant__ DevTables T, int64_t n,
                                                           const hepem_track_state in, const Work w, int ncb) {
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int key = -1;
    if (i < n) {
      const int type = in.type[i];
      const int imc = in.imc[i];
      const double e = in.ekin[i];
      if (!track_input_bad(T, type, imc, e)) key = sort_key(type, imc, e, ncb);
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
__global__ void __launch_bounds__(256) stage_a_charged_kernel(const __grid_constant__ DevTables T,
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
      load_track(in, idx, t, rng, uniforms, nu, seed, type);
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

__global__ void __launch_bounds__(256) stage_a_gamma_kernel(const __grid_constant__ DevTables T,
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
      load_track(in, idx, t, rng, uniforms, nu, seed, 2);
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
template <int Q>
__global__ void __launch_bounds__(256) stage_b_kernel(const __grid_constant__ DevTables T,
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
    rng.seed = seed;
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
template <class K>
static int grid_of(K kernel, int sms) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, 0) != cudaSuccess || per < 1) per = 1;
  return sms * per;
}

cudaError_t launch_step_batched(const DevTables& T, int64_t n, const hepem_track_state& in,
                                const hepem_track_state& out, const double* uniforms, int nu, uint64_t seed,
                                const hepem_step_out& res, hepem_step_counters* counters, void* workspace,
                                cudaStream_t s, int sms, cudaEvent_t* ev) {
  if (n <= 0) return cudaSuccess;
  static int gA = 0, gG = 0, gB[kNumQueues] = {};
  if (!gA) {
    gA = grid_of(stage_a_charged_kernel, sms);
    gG = grid_of(stage_a_gamma_kernel, sms);
    gB[0] = grid_of(stage_b_kernel<0>, sms);
    gB[1] = grid_of(stage_b_kernel<1>, sms);
    gB[2] = grid_of(stage_b_kernel<2>, sms);
    gB[3] = grid_of(stage_b_kernel<3>, sms);
    gB[4] = grid_of(stage_b_kernel<4>, sms);
    gB[5] = grid_of(stage_b_kernel<5>, sms);
    gB[6] = grid_of(stage_b_kernel<6>, sms);
    gB[7] = grid_of(stage_b_kernel<7>, sms);
    gB[8] = grid_of(stage_b_kernel<8>, sms);
  }
  const Work w = carve(workspace, n);
  const int ncb = T.nCouples < kSortCoupleBins ? T.nCouples : kSortCoupleBins;
  const int nkeys = 3 * ncb * kSortEBins;
  cudaError_t e = cudaMemsetAsync(w.counts, 0, 64 * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.hist, 0, nkeys * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  int k = 0;
  auto mark = [&]() {
    if (ev) cudaEventRecord(ev[k++], s);
  };
  const int64_t blocks = (n + 255) / 256;
  const int gC = (int)(blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8);
  mark();
  sort_hist_kernel<<<gC, 256, nkeys * sizeof(uint32_t), s>>>(T, n, in, out, res, w, ncb, counters);
  sort_scan_kernel<<<1, 1024, 0, s>>>(w, ncb);
  sort_scatter_kernel<<<gC, 256, 0, s>>>(T, n, in, w, ncb);
  mark();
  stage_a_charged_kernel<<<gA, 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_a_gamma_kernel<<<gG, 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<0><<<gB[0], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<1><<<gB[1], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<2><<<gB[2], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<3><<<gB[3], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<4><<<gB[4], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<5><<<gB[5], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<6><<<gB[6], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<7><<<gB[7], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  stage_b_kernel<8><<<gB[8], 256, 0, s>>>(T, in, out, uniforms, nu, seed, res, w, counters);
  mark();
  return cudaGetLastError();
}

}  // namespace hepem
