// kernels.h -- host launchers of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "g4hepem_gb300.h"
#include "tables.h"

namespace hepem {

// ---- the step-limit record between hepem_howfar and hepem_perform -------------------
// What the reference keeps in the thread-local primary track between
// G4HepEm{Electron,Gamma}Manager::HowFar and ::Perform (G4HepEmTrack,
// G4HepEmElectronTrack, G4HepEmMSCTrackData, G4HepEmGammaTrack fields and the
// RNG state after HowFar), SoA over n tracks in one caller buffer of
// limits_bytes(n) bytes.  HowFar leaves the caller's track state unchanged and
// writes everything it changed here; Perform reads the state (with the
// direction and boundary status transport left) and this record.
enum {
  kLProposed = 0,  // the geometrical step HowFar proposed
  kLPstep,         // e+-: the proposed true step length
  kLRange,         // e+-: range at the pre-step energy
  kLMfp0,          // mean free paths [4] (gamma: total, in [0])
  kLNia0 = kLMfp0 + 4,  // numbers of interaction lengths left after HowFar [4]
  kLPeXS = kLNia0 + 4,  // gamma: photoelectric macroscopic cross section
  kLLambtr1,            // e+- MSC: transport mean free path, true and geometrical
  kLTrueStep,           //   lengths, conversion parameters, and the persistent
  kLZPath,              //   step-limit state after HowFar
  kLPar1,
  kLPar2,
  kLPar3,
  kLInitRange,
  kLDynFactor,
  kLTlimitMin,
  kLDelta,              // precision form: trueStep - zPath without cancellation
  kLGauss,              // the cached Gaussian after HowFar
  kLimDoubles
};
constexpr uint32_t kLimMscActive = 1u << 0, kLimMscDisplace = 1u << 1, kLimFirstStep = 1u << 2,
                   kLimGaussValid = 1u << 3, kLimFp32 = 1u << 4, kLimPreBoundary = 1u << 5;
constexpr int kLimProvShift = 8;    // bits 8..15: provenance bits of an FP32 record (physics_mixed.cuh)
constexpr int kLimFlagsShift = 16;  // bits 16..23: the track flags HowFar raised (kFlag*)
struct Limits {
  double* d[kLimDoubles];
  int32_t* cursor;  // RNG cursor after HowFar
  int8_t* winner;   // process that limited the proposed step
  uint32_t* bits;
};
inline size_t limits_align(size_t b) { return (b + 255) / 256 * 256; }
inline size_t limits_bytes(int64_t n) {
  const size_t m = n > 0 ? (size_t)n : 0;
  return kLimDoubles * limits_align(8 * m) + limits_align(4 * m) + limits_align(m) + limits_align(4 * m);
}
inline Limits carve_limits(void* base, int64_t n) {
  const size_t m = n > 0 ? (size_t)n : 0;
  uint8_t* p = static_cast<uint8_t*>(base);
  Limits L;
  for (int k = 0; k < kLimDoubles; ++k) {
    L.d[k] = reinterpret_cast<double*>(p);
    p += limits_align(8 * m);
  }
  L.cursor = reinterpret_cast<int32_t*>(p);
  p += limits_align(4 * m);
  L.winner = reinterpret_cast<int8_t*>(p);
  p += limits_align(m);
  L.bits = reinterpret_cast<uint32_t*>(p);
  return L;
}

// the split of the step: phase of a launch (kPhaseStep: HowFar + Perform)
enum { kPhaseStep = 0, kPhaseHowFar = 1, kPhasePerform = 2 };

cudaError_t launch_howfar(const DevTables& T, int64_t n, const hepem_track_state& in, const double* uniforms, int nu,
                          uint64_t seed, double* gstep, const Limits& L, hepem_step_counters* counters,
                          cudaStream_t s, int sms);
cudaError_t launch_perform(const DevTables& T, int64_t n, const hepem_track_state& in, const hepem_track_state& out,
                           const double* gstep, const Limits& L, const double* uniforms, int nu, uint64_t seed,
                           const hepem_step_out& res, hepem_step_counters* counters, cudaStream_t s, int sms);

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
// side streams of a context and the events that fork and join them (the
// batched step overlaps independent stage kernels on them); mu serialises
// the enqueue of one step's forks and joins against another thread's
constexpr int kSideStreams = 3;
struct SideStreams {
  cudaStream_t st[kSideStreams] = {};
  cudaEvent_t ev[kSideStreams + 2] = {};
  std::mutex mu;
};
// optional inputs of a batched step
struct BatchOpts {
  cudaEvent_t* ev = nullptr;         // stage timing: kNumStageEvents events
  const int32_t* active = nullptr;   // step tracks active[0..n) of larger arrays (serving pool)
  const uint32_t* nDev = nullptr;    // with active: the device holds the count, n is an upper bound
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
  // split step: kPhaseHowFar writes the proposed steps to gstep and the step
  // limits to limits (out unused); kPhasePerform reads them (gstep: the
  // steps transport made)
  int phase = kPhaseStep;
  double* gstep = nullptr;
  Limits limits = {};
  // side streams for independent stages (null, or with stage timing: one stream)
  SideStreams* side = nullptr;
  // with no caller uniforms (nu == 0): room for the first kPrefill values of
  // every stepped track's stream, drawn by one kernel before the stages
  // (prefill_bytes); null: each draw computes its Philox block in place
  void* prefill = nullptr;
};
// the stream values drawn ahead per track when the caller passes no uniforms,
// for batches of at least kPrefillMinTracks (below that the extra kernel costs
// more than the draws in place: 0.50 against 0.46 ms per 256k-track
// precision step; 3.59 against 5.59 ms at 4M tracks)
constexpr int kPrefill = 32;
constexpr int64_t kPrefillMinTracks = 1 << 20;
inline bool wants_prefill(int64_t n, int nu) { return nu == 0 && n >= kPrefillMinTracks; }
// bytes of BatchOpts::prefill for `rows` stepped tracks whose indices are
// below `slots` (the track -> row map of an active list)
inline size_t prefill_bytes(int64_t rows, int64_t slots) {
  return ((size_t)rows * kPrefill * 8 + 255) / 256 * 256 + ((size_t)slots * 4 + 255) / 256 * 256;
}
// the index list and per-track RNG keys of a sub-batch step: active[p] =
// offset_b + (p - prefix[b]) and keys[that index] = seed_b for the
// sub-batch b holding position p (prefix: exclusive sums of the sizes,
// nb + 1 entries; batches and prefix in device memory)
cudaError_t launch_subbatch_index(const hepem_subbatch* batches, const int64_t* prefix, int nb, int64_t total,
                                  int32_t* active, uint64_t* keys, cudaStream_t s, int sms);
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
// the quantities of the reference's device tests, function by function
// (hepem_electron_xs_stepping, hepem_brem_select_target,
// hepem_conv_select_target, hepem_gamma_xs)
enum { kProbeElXs = 0, kProbeBremTarget = 1, kProbeConvTarget = 2, kProbeGammaXs = 3 };
struct ProbeArgs {
  int64_t n;
  int kind, positron, sb;
  const double* ekin;
  const int32_t* imc;
  const double* urnd;
  double* out[5];
  int32_t* iout;
};
cudaError_t launch_probe(const DevTables& T, const ProbeArgs& a, int mixed, cudaStream_t s, int sms);
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
