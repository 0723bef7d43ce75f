// trace.h -- NVTX ranges around the C-ABI entry points and around the stage
// launches of the batched forms, in the NVTX domain "g4hepem_gb300".
//
// A range opened by an entry point carries the batch size as its int64
// payload; inside a batched step the stage ranges ("sort", "stage_a_charged",
// ..., "fp64_fallback") nest in it, so a timeline tool shows the launch
// sequence of each step on the host thread beside the kernels on the stream.
// Without a tool attached (no NVTX injection library in the environment) each
// push or pop is one call through a null function pointer check.
#pragma once

#include <cstdint>

#include <nvtx3/nvToolsExt.h>

namespace hepem {

inline nvtxDomainHandle_t trace_domain() {
  static const nvtxDomainHandle_t d = nvtxDomainCreateA("g4hepem_gb300");
  return d;
}

inline void trace_push(const char* name, int64_t n) {
  nvtxEventAttributes_t a = {};
  a.version = NVTX_VERSION;
  a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
  a.messageType = NVTX_MESSAGE_TYPE_ASCII;
  a.message.ascii = name;
  a.payloadType = NVTX_PAYLOAD_TYPE_INT64;
  a.payload.llValue = (long long)n;
  nvtxDomainRangePushEx(trace_domain(), &a);
}

inline void trace_pop() { nvtxDomainRangePop(trace_domain()); }

// One range for the lifetime of the object (an entry point's call).
struct TraceRange {
  TraceRange(const char* name, int64_t n) { trace_push(name, n); }
  ~TraceRange() { trace_pop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

// Consecutive ranges inside one call: next() closes the open one, if any,
// and opens the next; the destructor closes the last.
struct TraceStages {
  bool open = false;
  int64_t n;
  explicit TraceStages(int64_t n_) : n(n_) {}
  void next(const char* name) {
    if (open) trace_pop();
    trace_push(name, n);
    open = true;
  }
  ~TraceStages() {
    if (open) trace_pop();
  }
  TraceStages(const TraceStages&) = delete;
  TraceStages& operator=(const TraceStages&) = delete;
};

}  // namespace hepem
