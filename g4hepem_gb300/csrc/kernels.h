// kernels.h -- host launchers of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "g4hepem_gb300.h"
#include "tables.h"

namespace hepem {

cudaError_t launch_lookup(const DevTables& T, int64_t n, int pos, const double* ekin, const int32_t* imc, double* xi,
                          double* xb, double* dedx, double* range, double* invr, cudaStream_t s, int sms);

cudaError_t launch_lookup_mixed(const DevTables& T, int64_t n, int pos, const double* ekin, const int32_t* imc,
                                double* xi, double* xb, double* dedx, double* range, double* invr, cudaStream_t s,
                                int sms);

cudaError_t launch_step(const DevTables& T, int64_t n, const hepem_track_state& in, const hepem_track_state& out,
                        const double* uniforms, int nu, uint64_t seed, const hepem_step_out& res,
                        hepem_step_counters* counters, cudaStream_t s, int sms);

// batched form (kernels_batched.cu): workspace of batched_workspace_bytes(n).
size_t batched_workspace_bytes(int64_t n);
// the eleven stage kernels: e+- stage A, gamma stage A, nine interaction kernels
constexpr int kNumStageKernels = 11;
// launch configuration of the stage kernels (chosen by hepem_autotune)
struct LaunchCfg {
  int block[kNumStageKernels];      // threads per block: 128, 256 or 512
  int ctasPerSM[kNumStageKernels];  // 0 (or above the occupancy) = as many as fit
  int sortEBins;                    // energy bins of the sort key: 8, 16 or 32
};
LaunchCfg default_launch_cfg();
bool valid_launch_cfg(const LaunchCfg& c);
int stage_occupancy(int kernel, int block);
// optional inputs of a batched step
struct BatchOpts {
  cudaEvent_t* ev = nullptr;         // stage timing: kNumStageEvents events
  const int32_t* active = nullptr;   // step tracks active[0..n) of larger arrays (serving pool)
  const uint64_t* seeds = nullptr;   // per-track RNG keys instead of one seed
  const LaunchCfg* cfg = nullptr;    // null: the default configuration
  bool mixed = false;                // precision form: e+- stage A in FP32 with FP64 fallback
  // precision form, in-place steps (in == out): arrays for the pre-step state
  // of the mutable fields (immutable fields pointing to the input), see
  // mixed_pre_state_bytes; null for out-of-place steps
  const hepem_track_state* preState = nullptr;
  // L2 access-policy window over the table arena (tableBytes 0: none): the
  // stage kernels mark that fraction of their table gathers persisting, so the
  // streamed track state does not evict the tables from L2
  const void* tableBase = nullptr;
  size_t tableBytes = 0;
  float tableHitRatio = 0.0f;
};
// bytes of the pre-step copy of an in-place precision-form step (n tracks)
size_t mixed_pre_state_bytes(int64_t n);
// carve the copy from `mem` (mixed_pre_state_bytes(n) bytes) around the batch `in`
hepem_track_state carve_pre_state(void* mem, int64_t n, const hepem_track_state& in);
cudaError_t launch_step_batched(const DevTables& T, int64_t n, const hepem_track_state& in,
                                const hepem_track_state& out, const double* uniforms, int nu, uint64_t seed,
                                const hepem_step_out& res, hepem_step_counters* counters, void* workspace,
                                cudaStream_t s, int sms, const BatchOpts& opts);
// per-model sampling (hepem_sample_model): models
enum { kSampleSB = 0, kSampleRB = 1, kSampleMoller = 2, kSampleBhabha = 3, kSampleCompton = 4, kSampleConversion = 5 };
cudaError_t launch_sample(const DevTables& T, int model, int mixed, int64_t n, double ekin, int imc, uint64_t seed,
                          double* out, unsigned long long* nFallback, cudaStream_t s, int sms);
// stage timing: events recorded before the first and after every stage kernel
constexpr int kNumStageEvents = 13;
const char* stage_name(int i);

cudaError_t launch_woodcock(const DevTables& T, int64_t n, const hepem_track_state& in,
                            const hepem_track_state& out, double* px, double* py, double* pz,
                            const hepem_layered_box& box, const double* uniforms, int nu, uint64_t seed,
                            const hepem_step_out& res, uint8_t* reached, cudaStream_t s, int sms);

cudaError_t launch_fill_uniforms(int64_t n, const int32_t* id, int nu, uint64_t seed, double* u, cudaStream_t s,
                                 int sms);

}  // namespace hepem
