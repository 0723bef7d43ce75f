// ctx.h -- the context behind the opaque hepem_ctx handle of the C-ABI.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "g4hepem_gb300.h"
#include "kernels.h"
#include "tables.h"

struct hepem_ctx {
  int device = -1;
  int sms = 0;
  void* arena = nullptr;
  size_t arenaBytes = 0;
  hepem::DevTables tables;
  // L2 access-policy window over the arena for the batched forms' stage
  // kernels (hepem_set_table_l2_window); tableWindow 0: none
  size_t tableWindow = 0;
  float tableHitRatio = 0.0f;
  // launch configuration of the batched form (hepem_set_launch_config / hepem_autotune)
  hepem::LaunchCfg launch = hepem::default_launch_cfg();
  // copy/compute pipeline of hepem_step_host: one stream for the copies in,
  // one for the steps, one for the copies out, and a device buffer per chunk
  // (grow-only, serialised by mu)
  static constexpr int kMaxChunks = 8;
  std::mutex mu;
  cudaStream_t pipe[3] = {};  // copies in, steps, copies out
  cudaEvent_t chunkIn[kMaxChunks] = {}, chunkStepped[kMaxChunks] = {};
  cudaEvent_t start = nullptr, finished = nullptr;
  void* pipeBuf = nullptr;
  size_t pipeBytes = 0;
  bool pipeReady = false;
  // device buffer of the host-buffer split step (hepem_howfar_host /
  // hepem_perform_host; grow-only, serialised by mu)
  void* splitBuf = nullptr;
  size_t splitBytes = 0;
  // side streams of the batched steps (created with the context)
  hepem::SideStreams side;
  bool sideReady = false;
  // per-stage timing of the batched form (hepem_profile_stages)
  bool profile = false;
  bool stageEvReady = false;
  cudaEvent_t stageEv[hepem::kNumStageEvents] = {};
};

namespace hepem {
// record the calling thread's last error message (hepem_last_error) and return code
int set_error(int code, const std::string& msg);
bool valid_state(const hepem_track_state* s);
bool valid_out(const hepem_step_out* r);
// the context's table window, as options of a batched step
inline void apply_table_window(const hepem_ctx* c, BatchOpts& o) {
  o.tableBase = c->arena;
  o.tableBytes = c->tableWindow;
  o.tableHitRatio = c->tableHitRatio;
  o.side = c->sideReady ? const_cast<SideStreams*>(&c->side) : nullptr;
}
// set (enable != 0) or clear the window; see hepem_set_table_l2_window
int set_table_window(hepem_ctx* c, int enable);
}  // namespace hepem
