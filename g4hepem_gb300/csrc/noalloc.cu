// noalloc.cu -- hepem_step_batched_noalloc: the batched step for callers that
// cannot let a library allocate device memory.
//
// Some callers of this path cannot allocate: applications that hand all device
// memory to their own pool allocator at start-up (a cudaMalloc or
// cudaMallocAsync inside a library then fails or fragments that pool), serving
// loops that must never enter an allocator on their latency path, and
// integrations whose rules forbid hidden allocations inside third-party
// libraries.  For them the workspace of the batched form (particle sort,
// interaction queues) lives in the fixed array below instead of a
// stream-ordered allocation.
//
// The array is part of the library's device image: every GPU that loads the
// library holds its 32 MiB until the process exits.  Host code cannot use the
// name of a __device__ array as a device address (in host code it names a
// host-side stand-in), so the address is looked up with cudaGetSymbolAddress,
// once per device, with that device current, by the first call on that device.
// That first call should therefore come before any stream capture.  The
// address stays valid for the life of the device's primary context: a
// cudaDeviceReset (or anything else that tears the context down) may move the
// array, so no call may follow such a reset in the same process.  All calls
// share the one array and it keeps the contents of the last call: the counters
// and histograms that must start at zero are cleared on the stream at the start
// of every call (launch_step_batched), and calls whose work overlaps on the GPU
// (different streams, or different host threads) race on the array.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "ctx.h"
#include "g4hepem_gb300.h"
#include "kernels.h"
#include "trace.h"

namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;   // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return hepem::set_error(HEPEM_BAD_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return hepem::set_error(HEPEM_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return HEPEM_OK;
}

}  // namespace

extern "C" int hepem_step_batched_noalloc(const hepem_ctx* c, int64_t n, const hepem_track_state* in,
                                          hepem_track_state* out, const double* uniforms, int32_t nu,
                                          uint64_t seed, hepem_step_out* res, hepem_step_counters* counters,
                                          void* stream) {
  if (!c || n < 0 || nu < 0) return hepem::set_error(HEPEM_BAD_ARG, "bad context or size");
  if (n == 0) return HEPEM_OK;
  if (n > HEPEM_NOALLOC_MAX_TRACKS || hepem::batched_workspace_bytes(n) > kScratchBytes) {
    char msg[160];
    snprintf(msg, sizeof(msg), "hepem_step_batched_noalloc: batch of %lld tracks exceeds the maximum of %d",
             (long long)n, HEPEM_NOALLOC_MAX_TRACKS);
    return hepem::set_error(HEPEM_BAD_ARG, msg);
  }
  if (!hepem::valid_state(in) || !hepem::valid_state(out) || !hepem::valid_out(res) || (nu > 0 && !uniforms))
    return hepem::set_error(HEPEM_BAD_ARG, "null array in track batch");
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != c->device)
    return hepem::set_error(HEPEM_BAD_ARG, "the current device is not the context's device");
  void* ws = nullptr;
  const int rc = scratch_address(&ws);
  if (rc != HEPEM_OK) return rc;
  hepem::TraceRange trace("hepem_step_batched_noalloc", n);
  hepem::BatchOpts o;
  o.cfg = &c->launch;
  hepem::apply_table_window(c, o);
  const cudaError_t e = hepem::launch_step_batched(c->tables, n, *in, *out, uniforms, nu, seed, *res, counters, ws,
                                                   (cudaStream_t)stream, c->sms, o);
  if (e != cudaSuccess)
    return hepem::set_error(HEPEM_CUDA_ERROR, std::string("batched step launch: ") + cudaGetErrorString(e));
  return HEPEM_OK;
}
