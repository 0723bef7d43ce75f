// kernels.h -- host launchers of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "g4hepem_gb300.h"
#include "tables.h"

namespace hepem {

cudaError_t launch_lookup(const DevTables& T, int64_t n, int pos, const double* ekin, const int32_t* imc, double* xi,
                          double* xb, double* dedx, double* range, double* invr, cudaStream_t s, int sms);

cudaError_t launch_step(const DevTables& T, int64_t n, const hepem_track_state& in, const hepem_track_state& out,
                        const double* uniforms, int nu, uint64_t seed, const hepem_step_out& res,
                        hepem_step_counters* counters, cudaStream_t s, int sms);

// batched form (kernels_batched.cu): workspace of batched_workspace_bytes(n)
size_t batched_workspace_bytes(int64_t n);
cudaError_t launch_step_batched(const DevTables& T, int64_t n, const hepem_track_state& in,
                                const hepem_track_state& out, const double* uniforms, int nu, uint64_t seed,
                                const hepem_step_out& res, hepem_step_counters* counters, void* workspace,
                                cudaStream_t s, int sms, cudaEvent_t* stage_events);
// stage timing: events recorded before the first and after every stage kernel
constexpr int kNumStageEvents = 13;
const char* stage_name(int i);

cudaError_t launch_fill_uniforms(int64_t n, const int32_t* id, int nu, uint64_t seed, double* u, cudaStream_t s,
                                 int sms);

}  // namespace hepem
