// tune.cu -- launch configuration of the batched form and its autotuner.
//
// The stage kernels of the batched step (kernels_batched.cu) exist for 128,
// 256 and 512 threads per block; each kernel's grid holds 1..occupancy CTAs
// per SM, and the counting sort groups e+- tracks into 8, 16 or 32 energy
// bins per couple (the tiling of the stage-A queues).  hepem_autotune times
// the caller's own batch under every candidate and keeps, per kernel, the
// fastest (block, CTAs per SM), then the fastest sort granularity.  Every
// configuration gives bit-identical results: the work of a track does not
// depend on where or with whom it runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "g4hepem_gb300.h"
#include "kernels.h"

namespace {

const size_t kStateSizes[20] = {1, 4, 4, 8, 8, 8, 8, 8, 8, 8, 8, 8, 1, 8, 8, 8, 1, 1, 8, 4};
const size_t kOutSizes[14] = {8, 8, 8, 1, 8, 8, 8, 1, 1, 2, 16, 16, 16, 16};

void to_public(const hepem::LaunchCfg& c, const float* ms, hepem_launch_config* o) {
  memset(o, 0, sizeof(*o));
  for (int k = 0; k < hepem::kNumStageKernels; ++k) {
    o->block[k] = c.block[k];
    o->ctas_per_sm[k] = c.ctasPerSM[k];
    o->ms[k] = ms ? ms[k] : 0.0f;
  }
  o->sort_energy_bins = c.sortEBins;
}

hepem::LaunchCfg from_public(const hepem_launch_config* o) {
  hepem::LaunchCfg c;
  for (int k = 0; k < hepem::kNumStageKernels; ++k) {
    c.block[k] = o->block[k];
    c.ctasPerSM[k] = o->ctas_per_sm[k];
  }
  c.sortEBins = o->sort_energy_bins;
  return c;
}

struct Scratch {
  void* mem = nullptr;
  hepem_track_state st{};
  hepem_step_out res{};
  void* work = nullptr;
  cudaEvent_t ev[hepem::kNumStageEvents] = {};
  int nev = 0;
  ~Scratch() {
    for (int k = 0; k < nev; ++k) cudaEventDestroy(ev[k]);
    if (mem) cudaFree(mem);
  }
};

}  // namespace

namespace hepem {
int set_table_window(hepem_ctx* c, int enable) {
  c->tableWindow = 0;
  c->tableHitRatio = 0.0f;
  if (!enable) return HEPEM_OK;
  int maxPersist = 0, maxWindow = 0;
  if (cudaDeviceGetAttribute(&maxPersist, cudaDevAttrMaxPersistingL2CacheSize, c->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&maxWindow, cudaDevAttrMaxAccessPolicyWindowSize, c->device) != cudaSuccess) {
    cudaGetLastError();
    return HEPEM_OK;  // no window on this device
  }
  if (maxPersist <= 0 || maxWindow <= 0) return HEPEM_OK;
  const size_t window = std::min(c->arenaBytes, (size_t)maxWindow);
  const size_t want = std::min(window, (size_t)maxPersist);
  // the persisting set-aside is a limit of this process's context: raise it
  // (never lower what another context of the process asked for)
  size_t have = 0;
  if (cudaDeviceGetLimit(&have, cudaLimitPersistingL2CacheSize) != cudaSuccess) {
    cudaGetLastError();
    return HEPEM_OK;
  }
  if (have < want) {
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) {
      cudaGetLastError();
      return HEPEM_OK;
    }
    have = want;
  }
  c->tableWindow = window;
  c->tableHitRatio = window > 0 ? (float)std::min(1.0, (double)have / (double)window) : 0.0f;
  return HEPEM_OK;
}
}  // namespace hepem

extern "C" {

int hepem_get_launch_config(const hepem_ctx* c, hepem_launch_config* out) {
  if (!c || !out) return hepem::set_error(HEPEM_BAD_ARG, "null argument");
  to_public(c->launch, nullptr, out);
  return HEPEM_OK;
}

int hepem_set_table_l2_window(hepem_ctx* c, int enable, int64_t* window_bytes) {
  if (!c) return hepem::set_error(HEPEM_BAD_ARG, "null context");
  const int rc = hepem::set_table_window(c, enable);
  if (window_bytes) *window_bytes = (int64_t)c->tableWindow;
  return rc;
}

int hepem_set_launch_config(hepem_ctx* c, const hepem_launch_config* cfg) {
  if (!c) return hepem::set_error(HEPEM_BAD_ARG, "null context");
  if (!cfg) {
    c->launch = hepem::default_launch_cfg();
    return HEPEM_OK;
  }
  const hepem::LaunchCfg l = from_public(cfg);
  if (!hepem::valid_launch_cfg(l))
    return hepem::set_error(HEPEM_BAD_ARG, "launch configuration: block 128/256/512, ctas_per_sm 0..64, "
                                           "sort_energy_bins 8/16/32");
  c->launch = l;
  return HEPEM_OK;
}

int hepem_autotune(hepem_ctx* c, int64_t n, const hepem_track_state* in, const double* uniforms, int32_t nu,
                   uint64_t seed, int apply, hepem_launch_config* out, void* stream) {
  if (!c || n <= 0 || nu < 0 || !hepem::valid_state(in) || (nu > 0 && !uniforms))
    return hepem::set_error(HEPEM_BAD_ARG, "bad autotune arguments");
  if (n > (int64_t)INT32_MAX) return hepem::set_error(HEPEM_BAD_ARG, "batch too large");
  cudaStream_t s = (cudaStream_t)stream;
  Scratch sc;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t bytes = 0;
  for (size_t b : kStateSizes) bytes += al(b * n);
  for (size_t b : kOutSizes) bytes += al(b * n);
  bytes += al(hepem::batched_workspace_bytes(n));
  cudaError_t e = cudaMalloc(&sc.mem, bytes);
  for (int k = 0; e == cudaSuccess && k < hepem::kNumStageEvents; ++k) {
    e = cudaEventCreate(&sc.ev[k]);
    if (e == cudaSuccess) sc.nev = k + 1;
  }
  if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, std::string("autotune: ") + cudaGetErrorString(e));
  uint8_t* p = (uint8_t*)sc.mem;
  void** sp = reinterpret_cast<void**>(&sc.st);
  for (int k = 0; k < 20; ++k) { sp[k] = p; p += al(kStateSizes[k] * n); }
  void** rp = reinterpret_cast<void**>(&sc.res);
  for (int k = 0; k < 14; ++k) { rp[k] = p; p += al(kOutSizes[k] * n); }
  sc.work = p;

  // one step of the caller's batch (input untouched, output to scratch); the
  // stage times of the fastest of `reps` runs, and the whole-step time
  auto run = [&](const hepem::LaunchCfg& cfg, int reps, float* stage, float* total) -> cudaError_t {
    hepem::BatchOpts o;
    o.ev = sc.ev;
    o.cfg = &cfg;
    hepem::apply_table_window(c, o);
    for (int k = 0; k < hepem::kNumStageKernels; ++k) stage[k] = 1e30f;
    *total = 1e30f;
    for (int r = 0; r < reps; ++r) {
      cudaError_t x = hepem::launch_step_batched(c->tables, n, *in, sc.st, uniforms, nu, seed, sc.res, nullptr,
                                                 sc.work, s, c->sms, o);
      if (x == cudaSuccess) x = cudaEventSynchronize(sc.ev[hepem::kNumStageEvents - 1]);
      if (x != cudaSuccess) return x;
      float t = 0.0f;
      cudaEventElapsedTime(&t, sc.ev[0], sc.ev[hepem::kNumStageEvents - 1]);
      *total = std::min(*total, t);
      for (int k = 0; k < hepem::kNumStageKernels; ++k) {
        cudaEventElapsedTime(&t, sc.ev[k + 1], sc.ev[k + 2]);
        stage[k] = std::min(stage[k], t);
      }
    }
    return cudaSuccess;
  };

  hepem::LaunchCfg best = hepem::default_launch_cfg();
  float bestMs[hepem::kNumStageKernels];
  float stage[hepem::kNumStageKernels], total = 0.0f;
  e = run(best, 2, bestMs, &total);  // warm-up and the default's times
  if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, std::string("autotune: ") + cudaGetErrorString(e));
  // 1. per kernel: threads per block and CTAs per SM (all kernels move together;
  //    kernels run one after another, so each one's time is its own)
  const int blocks[3] = {128, 256, 512};
  for (int b : blocks) {
    int maxOcc = 1;
    for (int k = 0; k < hepem::kNumStageKernels; ++k) maxOcc = std::max(maxOcc, hepem::stage_occupancy(k, b));
    for (int m = 1; m <= maxOcc; ++m) {
      hepem::LaunchCfg cand = best;
      bool any = false;
      for (int k = 0; k < hepem::kNumStageKernels; ++k) {
        const int occ = hepem::stage_occupancy(k, b);
        cand.block[k] = b;
        cand.ctasPerSM[k] = std::min(m, occ);
        any = any || m <= occ;
      }
      if (!any) continue;
      e = run(cand, 2, stage, &total);
      if (e != cudaSuccess)
        return hepem::set_error(HEPEM_CUDA_ERROR, std::string("autotune: ") + cudaGetErrorString(e));
      for (int k = 0; k < hepem::kNumStageKernels; ++k) {
        if (m > hepem::stage_occupancy(k, b)) continue;
        if (stage[k] < bestMs[k]) {
          bestMs[k] = stage[k];
          best.block[k] = cand.block[k];
          best.ctasPerSM[k] = cand.ctasPerSM[k];
        }
      }
    }
  }
  // 2. sort granularity, with the chosen kernels: the whole step decides
  float bestTotal = 1e30f;
  int bestBins = best.sortEBins;
  for (int bins : {8, 16, 32}) {
    hepem::LaunchCfg cand = best;
    cand.sortEBins = bins;
    e = run(cand, 2, stage, &total);
    if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, std::string("autotune: ") + cudaGetErrorString(e));
    if (total < bestTotal) {
      bestTotal = total;
      bestBins = bins;
      std::copy(stage, stage + hepem::kNumStageKernels, bestMs);
    }
  }
  best.sortEBins = bestBins;
  // 3. the choice against the default on the whole step as it runs outside
  //    the tuner (no stage events: independent stages overlap on the side
  //    streams, which the per-stage times above cannot see): the faster of the two
  auto whole = [&](const hepem::LaunchCfg& cfg, int reps, float* ms) -> cudaError_t {
    hepem::BatchOpts o;
    o.cfg = &cfg;
    hepem::apply_table_window(c, o);
    *ms = 1e30f;
    for (int r = 0; r < reps; ++r) {
      cudaError_t x = cudaEventRecord(sc.ev[0], s);
      if (x == cudaSuccess)
        x = hepem::launch_step_batched(c->tables, n, *in, sc.st, uniforms, nu, seed, sc.res, nullptr, sc.work, s,
                                       c->sms, o);
      if (x == cudaSuccess) x = cudaEventRecord(sc.ev[1], s);
      if (x == cudaSuccess) x = cudaEventSynchronize(sc.ev[1]);
      if (x != cudaSuccess) return x;
      float t = 0.0f;
      cudaEventElapsedTime(&t, sc.ev[0], sc.ev[1]);
      *ms = std::min(*ms, t);
    }
    return cudaSuccess;
  };
  const hepem::LaunchCfg def = hepem::default_launch_cfg();
  float msBest = 0.0f, msDef = 0.0f;
  e = whole(best, 3, &msBest);
  if (e == cudaSuccess) e = whole(def, 3, &msDef);
  if (e == cudaSuccess && msBest > msDef) {
    best = def;
    e = run(best, 2, bestMs, &total);
  }
  if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, std::string("autotune: ") + cudaGetErrorString(e));
  if (out) to_public(best, bestMs, out);
  if (apply) c->launch = best;
  return HEPEM_OK;
}

}  // extern "C"
