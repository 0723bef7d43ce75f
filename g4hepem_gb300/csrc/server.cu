// server.cu -- the serving form: continuous batching of event requests.
//
// A request is one event's batch of tracks.  The server keeps the tracks of
// admitted requests resident in a device slot pool sized from a memory budget
// and runs one loop on its own host thread and stream:
//   admit   : waiting requests (FIFO) get a contiguous slot range if one is
//             free (admission by memory budget), their tracks are copied in;
//   collect : one kernel compacts the alive tracks (E >= min_energy) of all
//             active requests into an index list and counts them per request;
//   step    : one batched step (kernels_batched.cu) over that list: requests
//             that arrived while others were running join the same launch;
//   account : per-track sums of deposited energy and secondaries;
//   retire  : requests with no alive track or at their step budget are
//             reduced (one block per request, fixed order), copied out, and
//             their slots are freed.
// Each track's uniform stream is Philox keyed by its request's seed and
// counted by its index in the request, and every per-request sum is reduced in
// a fixed order, so a request's result is the same alone and in any mix.
// Waits are bounded: hepem_server_wait gives up with HEPEM_TIMEOUT.
//
// Snapshot and resume: between two iterations (the loop holds iterMu for a
// whole iteration) the unfinished requests -- their track state as of the
// last completed step, their per-track sums and step counts -- are written to
// a host buffer; another server (same tables) resumes them, and each then ends
// with the result it would have had without the interruption, bit for bit:
// the state carries each track's id, RNG cursor and Gauss cache, the sums are
// per track, and the reductions have a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ctx.h"
#include "g4hepem_gb300.h"
#include "kernels.h"
#include "state_image.h"
#include "trace.h"

namespace {

using Clock = std::chrono::steady_clock;
double now_s() { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); }

const size_t kStateSizes[20] = {1, 4, 4, 8, 8, 8, 8, 8, 8, 8, 8, 8, 1, 8, 8, 8, 1, 1, 8, 4};
const size_t kOutSizes[14] = {8, 8, 8, 1, 8, 8, 8, 1, 1, 2, 16, 16, 16, 16};

// bytes of pool memory per resident track: state, results, RNG key, owner,
// accumulators, active index and the batched-step workspace share
size_t bytes_per_slot(bool mixed) {
  size_t b = 0;
  for (size_t x : kStateSizes) b += x;
  for (size_t x : kOutSizes) b += x;
  // + RNG key, owner-free accumulators, active index, workspace, and for the
  // precision form the pre-step copy of the in-place step
  return b + 8 + 4 + 8 + 8 + 4 + 4 + 52 + (mixed ? 102 : 0);
}

struct Request {
  int64_t id = 0;
  int64_t n = 0;
  uint64_t seed = 0;
  int64_t slot0 = -1;
  int32_t steps = 0;
  int32_t status = HEPEM_OK;
  bool done = false;
  std::atomic<bool> cancelled{false};
  double tSubmit = 0, tAdmit = 0, tDone = 0;
  std::vector<uint8_t> host;       // 20 state arrays back to back (input, then final state)
  std::vector<uint8_t> sums;       // resumed request: per-track sums so far (edep, e_sec, n_sec, steps)
  hepem_request_result result{};
};

// ---- kernels -----------------------------------------------------------------------
// alive tracks of active requests -> index list; per-request alive counts
__global__ void collect_kernel(int64_t nreq, const int64_t* __restrict__ slot0, const int64_t* __restrict__ off, int64_t total, const double* __restrict__ ekin,
                               double minE, int32_t* __restrict__ active, uint32_t* __restrict__ nActive,
                               uint32_t* __restrict__ aliveReq) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    // request r owns flat positions [off[r], off[r+1])
    int64_t lo = 0, hi = nreq - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) / 2;
      if (off[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const int64_t slot = slot0[lo] + (g - off[lo]);
    if (ekin[slot] > minE) {
      const uint32_t p = atomicAdd(nActive, 1u);
      active[p] = (int32_t)slot;
      atomicAdd(&aliveReq[lo], 1u);
    }
  }
}

// per-track sums of the step just taken
__global__ void account_kernel(const int32_t* __restrict__ active, const uint32_t* __restrict__ nActive,
                               const hepem_step_out res, double* __restrict__ edepSum,
                               double* __restrict__ eSecSum, int32_t* __restrict__ nSecSum,
                               int32_t* __restrict__ stepSum) {
  const uint32_t n = *nActive;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int32_t i = active[j];
    edepSum[i] += res.edep[i];
    const int ns = res.n_sec[i];
    double es = 0.0;
    for (int k = 0; k < ns && k < 2; ++k) es += res.sec_ekin[2 * (int64_t)i + k];
    eSecSum[i] += es;
    nSecSum[i] += ns;
    stepSum[i] += 1;
  }
}

// fixed-order reduction of one request's slot range (one block per request)
__global__ void reduce_kernel(const int64_t* __restrict__ slot0, const int64_t* __restrict__ cnt,
                              const double* __restrict__ edepSum, const double* __restrict__ eSecSum,
                              const int32_t* __restrict__ nSecSum, const int32_t* __restrict__ stepSum,
                              double* __restrict__ outD, int64_t* __restrict__ outI) {
  __shared__ double sd[256], se[256];
  __shared__ long long sn[256], ss[256];
  const int64_t a = slot0[blockIdx.x], m = cnt[blockIdx.x];
  double d = 0.0, e = 0.0;
  long long ns = 0, st = 0;
  for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
    d += edepSum[a + k];
    e += eSecSum[a + k];
    ns += nSecSum[a + k];
    st += stepSum[a + k];
  }
  sd[threadIdx.x] = d; se[threadIdx.x] = e; sn[threadIdx.x] = ns; ss[threadIdx.x] = st;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sd[threadIdx.x] += sd[threadIdx.x + w];
      se[threadIdx.x] += se[threadIdx.x + w];
      sn[threadIdx.x] += sn[threadIdx.x + w];
      ss[threadIdx.x] += ss[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    outD[2 * blockIdx.x] = sd[0];
    outD[2 * blockIdx.x + 1] = se[0];
    outI[2 * blockIdx.x] = sn[0];
    outI[2 * blockIdx.x + 1] = ss[0];
  }
}

// Staged state of whole requests (admission and retirement): per request,
// the 20 state arrays of its n tracks one after the other, each starting on
// a 16-byte boundary, at the request's offset in the staging buffer.
__host__ __device__ constexpr size_t stage_field_size(int k) {
  return k == 0 || k == 12 || k == 16 || k == 17 ? 1 : (k == 1 || k == 2 || k == 19) ? 4 : 8;
}
__host__ __device__ inline size_t stage_span(size_t bytes) { return (bytes + 15) & ~size_t(15); }
inline size_t staged_bytes(int64_t n) {
  size_t b = 0;
  for (int k = 0; k < 20; ++k) b += stage_span(stage_field_size(k) * (size_t)n);
  return b;
}
__device__ __forceinline__ void copy_elem(uint8_t* d, const uint8_t* s, size_t size) {
  if (size == 8) *reinterpret_cast<uint64_t*>(d) = *reinterpret_cast<const uint64_t*>(s);
  else if (size == 4) *reinterpret_cast<uint32_t*>(d) = *reinterpret_cast<const uint32_t*>(s);
  else *d = *s;
}
// request r = blockIdx.y: its staged state to (ADMIT) or from (!ADMIT) its
// pool slots [slot0[r], slot0[r] + cnt[r]); on admission also its RNG key and
// zero per-track sums
template <bool ADMIT>
__global__ void stage_kernel(const int64_t* __restrict__ slot0, const int64_t* __restrict__ cnt,
                             const int64_t* __restrict__ off, const uint64_t* __restrict__ reqSeed,
                             uint8_t* __restrict__ stage, const hepem_track_state st, uint64_t* __restrict__ seeds,
                             double* __restrict__ d0, double* __restrict__ d1, int32_t* __restrict__ i0,
                             int32_t* __restrict__ i1) {
  const int r = blockIdx.y;
  const int64_t a = slot0[r], m = cnt[r];
  void* const* pool = reinterpret_cast<void* const*>(&st);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    size_t o = (size_t)off[r];
#pragma unroll
    for (int f = 0; f < 20; ++f) {
      const size_t sz = stage_field_size(f);
      uint8_t* pp = static_cast<uint8_t*>(pool[f]) + sz * (size_t)(a + k);
      uint8_t* sp = stage + o + sz * (size_t)k;
      if (ADMIT) copy_elem(pp, sp, sz);
      else copy_elem(sp, pp, sz);
      o += stage_span(sz * (size_t)m);
    }
    if (ADMIT) {
      seeds[a + k] = reqSeed[r];
      d0[a + k] = 0.0;
      d1[a + k] = 0.0;
      i0[a + k] = 0;
      i1[a + k] = 0;
    }
  }
}

__global__ void fill_seed_kernel(uint64_t* __restrict__ seeds, int64_t a, int64_t m, uint64_t seed,
                                 double* __restrict__ d0, double* __restrict__ d1, int32_t* __restrict__ i0,
                                 int32_t* __restrict__ i1) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    seeds[a + k] = seed;
    d0[a + k] = 0.0;
    d1[a + k] = 0.0;
    i0[a + k] = 0;
    i1[a + k] = 0;
  }
}

// snapshot format (hepem_server_snapshot)
const char kSnapMagic[8] = {'H', 'E', 'P', 'E', 'M', 'S', 'N', 'P'};
constexpr uint32_t kSnapVersion = 1;
constexpr size_t kSnapHeader = 32;    // magic, version, 0, requests, tracks
constexpr size_t kSnapRecord = 32;    // id, n, seed, steps, admitted, cancelled, 0
constexpr size_t kSnapSumBytes = 24;  // per track: edep, e_sec (f64), n_sec, steps (i32)

struct SnapRec {
  int64_t id, n;
  uint64_t seed;
  int32_t steps;
  bool admitted, cancelled;
  const uint8_t* state;  // 20 state arrays, then the sums
};

// Checks a snapshot (magic, version, sizes, checksum) and lists its requests.
int parse_snapshot(const void* buf, size_t size, std::vector<SnapRec>& out) {
  out.clear();
  if (!buf) return hepem::set_error(HEPEM_BAD_ARG, "null snapshot");
  const uint8_t* p = static_cast<const uint8_t*>(buf);
  if (size < kSnapHeader + 8 || memcmp(p, kSnapMagic, 8) != 0)
    return hepem::set_error(HEPEM_PARSE_ERROR, "not a server snapshot");
  uint32_t ver[2];
  uint64_t counts[2], stored;
  memcpy(ver, p + 8, 8);
  memcpy(counts, p + 16, 16);
  if (ver[0] != kSnapVersion) return hepem::set_error(HEPEM_PARSE_ERROR, "snapshot: unknown version");
  memcpy(&stored, p + size - 8, 8);
  if (hepem::fnv1a(p, size - 8) != stored) return hepem::set_error(HEPEM_PARSE_ERROR, "snapshot: checksum mismatch");
  size_t per = kSnapSumBytes;
  for (size_t b : kStateSizes) per += b;
  size_t off = kSnapHeader;
  uint64_t tracks = 0;
  for (uint64_t k = 0; k < counts[0]; ++k) {
    if (off + kSnapRecord > size - 8) return hepem::set_error(HEPEM_PARSE_ERROR, "snapshot: truncated");
    SnapRec r;
    uint8_t flags[4];
    memcpy(&r.id, p + off, 8);
    memcpy(&r.n, p + off + 8, 8);
    memcpy(&r.seed, p + off + 16, 8);
    memcpy(&r.steps, p + off + 24, 4);
    memcpy(flags, p + off + 28, 4);
    r.admitted = flags[0] != 0;
    r.cancelled = flags[1] != 0;
    off += kSnapRecord;
    if (r.n <= 0 || r.steps < 0 || flags[0] > 1 || flags[1] > 1 || (uint64_t)r.n > (size - 8 - off) / per)
      return hepem::set_error(HEPEM_PARSE_ERROR, "snapshot: bad request record");
    r.state = p + off;
    off += per * (size_t)r.n;
    tracks += (uint64_t)r.n;
    out.push_back(r);
  }
  if (off != size - 8 || tracks != counts[1])
    return hepem::set_error(HEPEM_PARSE_ERROR, "snapshot: sizes do not add up");
  return HEPEM_OK;
}

}  // namespace

struct hepem_server {
  const hepem_ctx* ctx = nullptr;
  hepem_server_config cfg{};
  int64_t capacity = 0;
  cudaStream_t stream = nullptr;
  // pool
  void* pool = nullptr;
  hepem_track_state st{};
  hepem_step_out res{};
  uint64_t* seeds = nullptr;
  double* edepSum = nullptr;
  double* eSecSum = nullptr;
  int32_t* nSecSum = nullptr;
  int32_t* stepSum = nullptr;
  int32_t* active = nullptr;
  void* work = nullptr;
  void* pre = nullptr;                 // precision form: pre-step copy (mixed_pre_state_bytes)
  // per-iteration request tables, the same layout on the device and in pinned
  // host memory, each table group packed so that it moves in one copy:
  //   req:   slot0[m] cnt[m] off[m + 1]  (m = the iteration's requests)
  //   alive: nActive, alive[m]
  //   out:   outD[2m] outI[2m]           (sums of the retired requests)
  //   st:    slot0[m] n[m] off[m] seed[m] (staged admission / retirement)
  // and the staging buffer of the admitted and retired requests' state
  int64_t maxReq = 0;
  size_t tableBytes = 0;
  int64_t *dReq = nullptr, *hReq = nullptr;
  uint32_t *dAliveT = nullptr, *hAliveT = nullptr;
  int64_t *dOutT = nullptr, *hOutT = nullptr;
  int64_t *dStT = nullptr, *hStT = nullptr;
  size_t stageBytes = 0;
  uint8_t *hStage = nullptr, *dStage = nullptr;
  // free slot ranges: start -> length
  std::map<int64_t, int64_t> freeRanges;
  // requests
  std::mutex mu;
  std::condition_variable cv, cvDone;
  std::mutex iterMu;                   // held by the loop for a whole iteration (snapshots wait for it)
  int snapWaiters = 0;                 // snapshots waiting for iterMu (under mu): the loop lets them in first
  std::condition_variable cvSnap;
  std::deque<int64_t> waiting;
  std::vector<int64_t> activeReq;
  std::unordered_map<int64_t, std::unique_ptr<Request>> reqs;
  int64_t nextId = 1;
  std::atomic<bool> stop{false};
  std::thread loop;
  int32_t loopError = HEPEM_OK;
  std::string loopErrorMsg;
  // statistics
  std::vector<double> batchMs;
  int64_t iterations = 0, trackSteps = 0, completed = 0;

  int64_t alloc_slots(int64_t n) {
    for (auto it = freeRanges.begin(); it != freeRanges.end(); ++it) {
      if (it->second >= n) {
        const int64_t a = it->first, len = it->second;
        freeRanges.erase(it);
        if (len > n) freeRanges[a + n] = len - n;
        return a;
      }
    }
    return -1;
  }
  void free_slots(int64_t a, int64_t n) {
    auto it = freeRanges.emplace(a, n).first;
    auto nx = std::next(it);
    if (nx != freeRanges.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      freeRanges.erase(nx);
    }
    if (it != freeRanges.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        freeRanges.erase(it);
      }
    }
  }
  void* state_ptr(int k, int64_t slot) const {
    return (uint8_t*)(reinterpret_cast<void* const*>(&st)[k]) + kStateSizes[k] * slot;
  }
  void run();
  cudaError_t iterate();
};

#define SRV_CUDA(call)                  \
  do {                                  \
    cudaError_t e_ = (call);            \
    if (e_ != cudaSuccess) return e_;   \
  } while (0)

cudaError_t hepem_server::iterate() {
  // ranges: admission, the collection of the live tracks, the step, retirement
  // (payload: the iteration's index)
  hepem::TraceStages trace(iterations);
  trace.next("server_admit");
  std::vector<Request*> admitted;
  {
    std::lock_guard<std::mutex> lock(mu);
    while (!waiting.empty() && (int64_t)activeReq.size() < maxReq) {
      Request* r = reqs[waiting.front()].get();
      const int64_t a = alloc_slots(r->n);
      if (a < 0) break;                        // wait for memory (FIFO: no overtaking)
      waiting.pop_front();
      r->slot0 = a;
      r->tAdmit = now_s();
      admitted.push_back(r);
      activeReq.push_back(r->id);
    }
  }
  // admission through the staging buffers: the admitted requests' state
  // packed into pinned memory, one copy, one kernel to the pool slots
  {
    size_t used = 0;
    int64_t ns = 0, maxN = 0;
    std::vector<Request*> direct, adm;
    std::vector<int64_t> offs;
    for (Request* r : admitted) {
      const size_t need = staged_bytes(r->n);
      if (!r->sums.empty() || need > stageBytes - used || ns == 65535) {
        direct.push_back(r);
        continue;
      }
      size_t o = used, t = 0;
      for (int k = 0; k < 20; ++k) {
        const size_t b = kStateSizes[k] * (size_t)r->n;
        memcpy(hStage + o, r->host.data() + t, b);
        o += stage_span(b);
        t += b;
      }
      adm.push_back(r);
      offs.push_back((int64_t)used);
      ns += 1;
      maxN = std::max(maxN, r->n);
      used += need;
    }
    if (ns > 0) {
      for (int64_t q = 0; q < ns; ++q) {
        hStT[q] = adm[q]->slot0;
        hStT[ns + q] = adm[q]->n;
        hStT[2 * ns + q] = offs[q];
        hStT[3 * ns + q] = (int64_t)adm[q]->seed;
      }
      SRV_CUDA(cudaMemcpyAsync(dStage, hStage, used, cudaMemcpyHostToDevice, stream));
      SRV_CUDA(cudaMemcpyAsync(dStT, hStT, 32 * ns, cudaMemcpyHostToDevice, stream));
      const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>((maxN + 255) / 256, 64));
      stage_kernel<true><<<dim3(gx, (unsigned)ns), 256, 0, stream>>>(
          dStT, dStT + ns, dStT + 2 * ns, reinterpret_cast<const uint64_t*>(dStT + 3 * ns), dStage, st, seeds,
          edepSum, eSecSum, nSecSum, stepSum);
      SRV_CUDA(cudaGetLastError());
    }
    admitted.swap(direct);
  }
  // the rest (larger than the staging space left, or resumed with sums): array by array
  for (Request* r : admitted) {
    size_t o = 0;
    for (int k = 0; k < 20; ++k) {
      SRV_CUDA(cudaMemcpyAsync(state_ptr(k, r->slot0), r->host.data() + o, kStateSizes[k] * r->n,
                               cudaMemcpyHostToDevice, stream));
      o += kStateSizes[k] * r->n;
    }
    fill_seed_kernel<<<std::max<int64_t>(1, std::min<int64_t>((r->n + 255) / 256, 1024)), 256, 0, stream>>>(
        seeds, r->slot0, r->n, r->seed, edepSum, eSecSum, nSecSum, stepSum);
    SRV_CUDA(cudaGetLastError());
    if (!r->sums.empty()) {
      // a resumed request: its per-track sums so far (pageable source: staged before the call returns)
      const uint8_t* q = r->sums.data();
      SRV_CUDA(cudaMemcpyAsync(edepSum + r->slot0, q, 8 * r->n, cudaMemcpyHostToDevice, stream));
      SRV_CUDA(cudaMemcpyAsync(eSecSum + r->slot0, q + 8 * r->n, 8 * r->n, cudaMemcpyHostToDevice, stream));
      SRV_CUDA(cudaMemcpyAsync(nSecSum + r->slot0, q + 16 * r->n, 4 * r->n, cudaMemcpyHostToDevice, stream));
      SRV_CUDA(cudaMemcpyAsync(stepSum + r->slot0, q + 20 * r->n, 4 * r->n, cudaMemcpyHostToDevice, stream));
      std::vector<uint8_t>().swap(r->sums);
    }
  }
  std::vector<Request*> act;
  {
    std::lock_guard<std::mutex> lock(mu);
    for (int64_t id : activeReq) act.push_back(reqs[id].get());
  }
  if (act.empty()) return cudaSuccess;
  const double t0 = now_s();
  const int64_t nr = (int64_t)act.size();
  int64_t total = 0;
  int64_t* hSlot0 = hReq;
  int64_t* hOff = hReq + nr;
  for (int64_t k = 0; k < nr; ++k) {
    hSlot0[k] = act[k]->slot0;
    hOff[k] = total;
    total += act[k]->n;
  }
  hOff[nr] = total;
  trace.next("server_collect");
  SRV_CUDA(cudaMemcpyAsync(dReq, hReq, sizeof(int64_t) * (2 * nr + 1), cudaMemcpyHostToDevice, stream));
  SRV_CUDA(cudaMemsetAsync(dAliveT, 0, sizeof(uint32_t) * (nr + 1), stream));
  const int64_t* dSlot0 = dReq;
  const int64_t* dOff = dReq + nr;
  uint32_t* dNActive = dAliveT;
  uint32_t* dAlive = dAliveT + 1;
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)ctx->sms * 16));
  collect_kernel<<<g, 256, 0, stream>>>(nr, dSlot0, dOff, total, st.ekin, cfg.min_energy, active, dNActive,
                                        dAlive);
  SRV_CUDA(cudaGetLastError());
  // the step over the collected tracks: the kernels read their number from
  // the device (total is its upper bound), so the host does not wait here
  trace.next("server_step");
  {
    hepem::BatchOpts o;
    o.active = active;
    o.nDev = dNActive;
    o.seeds = seeds;
    o.cfg = &ctx->launch;
    hepem::apply_table_window(ctx, o);
    hepem_track_state preState;
    if (cfg.precision) {
      o.mixed = true;
      preState = hepem::carve_pre_state(pre, capacity, st);
      o.preState = &preState;
    }
    SRV_CUDA(hepem::launch_step_batched(ctx->tables, total, st, st, nullptr, 0, 0, res, nullptr, work, stream,
                                        ctx->sms, o));
    account_kernel<<<g, 256, 0, stream>>>(active, dNActive, res, edepSum, eSecSum, nSecSum, stepSum);
    SRV_CUDA(cudaGetLastError());
  }
  SRV_CUDA(cudaMemcpyAsync(hAliveT, dAliveT, sizeof(uint32_t) * (nr + 1), cudaMemcpyDeviceToHost, stream));
  const uint32_t* hAlive = hAliveT + 1;
  SRV_CUDA(cudaStreamSynchronize(stream));
  const int64_t nAct = hAliveT[0];
  trace.next("server_retire");
  // retire: nothing alive before this step, or the step budget is used up
  std::vector<int64_t> fin;
  for (int64_t k = 0; k < nr; ++k) {
    Request* r = act[k];
    if (hAlive[k] > 0) r->steps += 1;
    if (hAlive[k] == 0 || r->steps >= cfg.max_steps || r->cancelled) fin.push_back(k);
  }
  if (!fin.empty()) {
    const int64_t nf = (int64_t)fin.size();
    for (int64_t q = 0; q < nf; ++q) {
      hReq[q] = act[fin[q]]->slot0;
      hReq[nf + q] = act[fin[q]]->n;
    }
    SRV_CUDA(cudaMemcpyAsync(dReq, hReq, sizeof(int64_t) * 2 * nf, cudaMemcpyHostToDevice, stream));
    reduce_kernel<<<(unsigned)nf, 256, 0, stream>>>(dReq, dReq + nf, edepSum, eSecSum, nSecSum, stepSum,
                                                    reinterpret_cast<double*>(dOutT), dOutT + 2 * nf);
    SRV_CUDA(cudaGetLastError());
    SRV_CUDA(cudaMemcpyAsync(hOutT, dOutT, sizeof(int64_t) * 4 * nf, cudaMemcpyDeviceToHost, stream));
    const double* hOutD = reinterpret_cast<const double*>(hOutT);
    const int64_t* hOutI = hOutT + 2 * nf;
    // final states: packed on the device into the staging buffer, one copy
    // out (requests beyond its space: array by array)
    size_t used = 0;
    int64_t ns = 0, maxN = 0;
    std::vector<char> staged(nf, 0);
    std::vector<Request*> ret;
    std::vector<int64_t> offs;
    for (int64_t q = 0; q < nf; ++q) {
      Request* r = act[fin[q]];
      const size_t need = staged_bytes(r->n);
      if (need <= stageBytes - used && ns < 65535) {
        ret.push_back(r);
        offs.push_back((int64_t)used);
        ns += 1;
        maxN = std::max(maxN, r->n);
        used += need;
        staged[q] = 1;
        continue;
      }
      size_t o = 0;
      for (int k = 0; k < 20; ++k) {
        SRV_CUDA(cudaMemcpyAsync(r->host.data() + o, state_ptr(k, r->slot0), kStateSizes[k] * r->n,
                                 cudaMemcpyDeviceToHost, stream));
        o += kStateSizes[k] * r->n;
      }
    }
    if (ns > 0) {
      for (int64_t q = 0; q < ns; ++q) {
        hStT[q] = ret[q]->slot0;
        hStT[ns + q] = ret[q]->n;
        hStT[2 * ns + q] = offs[q];
      }
      SRV_CUDA(cudaMemcpyAsync(dStT, hStT, 24 * ns, cudaMemcpyHostToDevice, stream));
      const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>((maxN + 255) / 256, 64));
      stage_kernel<false><<<dim3(gx, (unsigned)ns), 256, 0, stream>>>(dStT, dStT + ns, dStT + 2 * ns, nullptr,
                                                                      dStage, st, nullptr, nullptr, nullptr,
                                                                      nullptr, nullptr);
      SRV_CUDA(cudaGetLastError());
      SRV_CUDA(cudaMemcpyAsync(hStage, dStage, used, cudaMemcpyDeviceToHost, stream));
    }
    SRV_CUDA(cudaStreamSynchronize(stream));
    {
      int64_t j = 0;
      for (int64_t q = 0; q < nf; ++q) {
        if (!staged[q]) continue;
        Request* r = act[fin[q]];
        size_t o = (size_t)offs[j++], t = 0;
        for (int k = 0; k < 20; ++k) {
          const size_t b = kStateSizes[k] * (size_t)r->n;
          memcpy(r->host.data() + t, hStage + o, b);
          o += stage_span(b);
          t += b;
        }
      }
    }
    const double t = now_s();
    std::lock_guard<std::mutex> lock(mu);
    for (int64_t q = 0; q < nf; ++q) {
      Request* r = act[fin[q]];
      r->result.n_tracks = r->n;
      r->result.steps = r->steps;
      r->result.status = r->cancelled ? HEPEM_CANCELLED : HEPEM_OK;
      r->result.edep = hOutD[2 * q];
      r->result.e_secondaries = hOutD[2 * q + 1];
      r->result.n_secondaries = hOutI[2 * q];
      r->result.track_steps = hOutI[2 * q + 1];
      r->result.t_submit = r->tSubmit;
      r->result.t_admit = r->tAdmit;
      r->result.t_done = t;
      r->done = true;
      free_slots(r->slot0, r->n);
      activeReq.erase(std::find(activeReq.begin(), activeReq.end(), r->id));
      completed += 1;
    }
    cvDone.notify_all();
  }
  {
    std::lock_guard<std::mutex> lock(mu);
    if (batchMs.size() >= (size_t)1 << 20) batchMs.erase(batchMs.begin(), batchMs.begin() + (1 << 19));
    batchMs.push_back(1e3 * (now_s() - t0));
    iterations += 1;
    trackSteps += nAct;
  }
  return cudaSuccess;
}

void hepem_server::run() {
  cudaSetDevice(ctx->device);
  while (!stop.load()) {
    bool idle;
    {
      std::unique_lock<std::mutex> lock(mu);
      cv.wait_for(lock, std::chrono::milliseconds(5),
                  [&] { return stop.load() || !waiting.empty() || !activeReq.empty(); });
      idle = waiting.empty() && activeReq.empty();
    }
    if (idle) continue;
    {
      // a waiting snapshot goes before the next iteration (the mutex alone is not fair)
      std::unique_lock<std::mutex> lock(mu);
      cvSnap.wait_for(lock, std::chrono::seconds(1), [&] { return snapWaiters == 0 || stop.load(); });
    }
    cudaError_t e;
    {
      std::lock_guard<std::mutex> g(iterMu);
      e = iterate();
    }
    if (e != cudaSuccess) {
      std::lock_guard<std::mutex> lock(mu);
      loopError = HEPEM_CUDA_ERROR;
      loopErrorMsg = cudaGetErrorString(e);
      for (auto& kv : reqs) {
        if (!kv.second->done) {
          kv.second->done = true;
          kv.second->result.status = HEPEM_CUDA_ERROR;
        }
      }
      cvDone.notify_all();
      return;
    }
  }
}

extern "C" {

int hepem_server_create(const hepem_ctx* ctx, const hepem_server_config* cfg, hepem_server** out) {
  if (!ctx || !cfg || !out || cfg->memory_budget_bytes <= 0 || cfg->max_steps <= 0 || cfg->max_requests <= 0)
    return hepem::set_error(HEPEM_BAD_ARG, "bad server configuration");
  *out = nullptr;
  std::unique_ptr<hepem_server> s(new hepem_server());
  s->ctx = ctx;
  s->cfg = *cfg;
  s->maxReq = cfg->max_requests;
  if (cfg->precision != 0 && cfg->precision != 1) return hepem::set_error(HEPEM_BAD_ARG, "precision must be 0 or 1");
  const size_t per = bytes_per_slot(cfg->precision == 1);
  const size_t fixed = hepem::batched_workspace_bytes(0) + 64 * 256;  // + rounding of ~45 arrays
  if ((size_t)cfg->memory_budget_bytes <= fixed + per) return hepem::set_error(HEPEM_BAD_ARG, "budget too small");
  s->capacity = (int64_t)(((size_t)cfg->memory_budget_bytes - fixed) / per);
  if (s->capacity > (int64_t)INT32_MAX / 2) s->capacity = INT32_MAX / 2;
  const int64_t C = s->capacity;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t bytes = 0;
  for (size_t b : kStateSizes) bytes += al(b * C);
  for (size_t b : kOutSizes) bytes += al(b * C);
  bytes += al(8 * C) * 3 + al(4 * C) * 3 + al(hepem::batched_workspace_bytes(C));
  if (cfg->precision) bytes += al(hepem::mixed_pre_state_bytes(C));
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&s->pool, bytes);
  if (e != cudaSuccess) {
    if (s->stream) cudaStreamDestroy(s->stream);
    return hepem::set_error(HEPEM_OOM_ADMISSION, std::string("server pool: ") + cudaGetErrorString(e));
  }
  uint8_t* p = (uint8_t*)s->pool;
  void** sp = reinterpret_cast<void**>(&s->st);
  for (int k = 0; k < 20; ++k) { sp[k] = p; p += al(kStateSizes[k] * C); }
  void** rp = reinterpret_cast<void**>(&s->res);
  for (int k = 0; k < 14; ++k) { rp[k] = p; p += al(kOutSizes[k] * C); }
  s->seeds = (uint64_t*)p; p += al(8 * C);
  s->edepSum = (double*)p; p += al(8 * C);
  s->eSecSum = (double*)p; p += al(8 * C);
  s->nSecSum = (int32_t*)p; p += al(4 * C);
  s->stepSum = (int32_t*)p; p += al(4 * C);
  s->active = (int32_t*)p; p += al(4 * C);
  s->work = p;
  p += al(hepem::batched_workspace_bytes(C));
  if (cfg->precision) s->pre = p;
  // request tables, same layout on the device and in pinned host memory:
  // slot0[R] cnt[R] off[R+1] outI[2R] outD[2R] nActive[1] alive[R], then the
  // staged requests' stSlot0[R] stN[R] stOff[R] stSeed[R], then the staging
  // buffer (the state of up to 1M tracks of admitted or retired requests per
  // iteration, at least the largest request the pool holds)
  const int64_t R = s->maxReq;
  const int64_t stageTracks = std::min<int64_t>(C, 1 << 20);
  s->stageBytes = staged_bytes(stageTracks) + 16 * 20;
  size_t tabOff[5];
  {
    const size_t sz[5] = {8 * (size_t)(2 * R + 1), 4 * (size_t)(R + 1), 32 * (size_t)R, 32 * (size_t)R,
                          s->stageBytes};
    size_t o = 0;
    for (int k = 0; k < 5; ++k) {
      tabOff[k] = o;
      o += al(sz[k]);
    }
    s->tableBytes = o;
  }
  uint8_t *dTab = nullptr, *hTab = nullptr;
  e = cudaMalloc((void**)&dTab, s->tableBytes);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&hTab, s->tableBytes);
  if (e != cudaSuccess) {
    cudaFree(s->pool);
    if (dTab) cudaFree(dTab);
    cudaStreamDestroy(s->stream);
    return hepem::set_error(HEPEM_CUDA_ERROR, std::string("server tables: ") + cudaGetErrorString(e));
  }
  s->dReq = (int64_t*)(dTab + tabOff[0]);
  s->dAliveT = (uint32_t*)(dTab + tabOff[1]);
  s->dOutT = (int64_t*)(dTab + tabOff[2]);
  s->dStT = (int64_t*)(dTab + tabOff[3]);
  s->dStage = dTab + tabOff[4];
  s->hReq = (int64_t*)(hTab + tabOff[0]);
  s->hAliveT = (uint32_t*)(hTab + tabOff[1]);
  s->hOutT = (int64_t*)(hTab + tabOff[2]);
  s->hStT = (int64_t*)(hTab + tabOff[3]);
  s->hStage = hTab + tabOff[4];
  s->freeRanges[0] = C;
  hepem_server* raw = s.release();
  raw->loop = std::thread([raw] { raw->run(); });
  *out = raw;
  return HEPEM_OK;
}

int hepem_server_capacity(const hepem_server* s, int64_t* tracks) {
  if (!s || !tracks) return hepem::set_error(HEPEM_BAD_ARG, "null argument");
  *tracks = s->capacity;
  return HEPEM_OK;
}

int hepem_server_submit(hepem_server* s, int64_t n, const hepem_track_state* tracks, uint64_t seed,
                        int64_t* request_id) {
  if (!s || !tracks || !request_id || n <= 0) return hepem::set_error(HEPEM_BAD_ARG, "bad request");
  if (n > s->capacity)
    return hepem::set_error(HEPEM_OOM_ADMISSION, "request larger than the server's memory budget");
  if (!hepem::valid_state(tracks)) return hepem::set_error(HEPEM_BAD_ARG, "null array in track batch");
  std::unique_ptr<Request> r(new Request());
  r->n = n;
  r->seed = seed;
  size_t tot = 0;
  for (size_t b : kStateSizes) tot += b * n;
  r->host.resize(tot);
  void* const* src = reinterpret_cast<void* const*>(tracks);
  size_t o = 0;
  for (int k = 0; k < 20; ++k) {
    memcpy(r->host.data() + o, src[k], kStateSizes[k] * n);
    o += kStateSizes[k] * n;
  }
  r->tSubmit = now_s();
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->loopError != HEPEM_OK) return hepem::set_error(s->loopError, "server loop stopped: " + s->loopErrorMsg);
  r->id = s->nextId++;
  *request_id = r->id;
  s->waiting.push_back(r->id);
  s->reqs[r->id] = std::move(r);
  s->cv.notify_all();
  return HEPEM_OK;
}

static int take_result(hepem_server* s, Request* r, hepem_request_result* result, hepem_track_state* final_tracks) {
  if (result) *result = r->result;
  if (final_tracks) {
    void* const* dst = reinterpret_cast<void* const*>(final_tracks);
    size_t o = 0;
    for (int k = 0; k < 20; ++k) {
      if (dst[k]) memcpy(dst[k], r->host.data() + o, kStateSizes[k] * r->n);
      o += kStateSizes[k] * r->n;
    }
  }
  const int st = r->result.status;
  s->reqs.erase(r->id);
  return st;
}

int hepem_server_poll(hepem_server* s, int64_t request_id, int32_t* done, hepem_request_result* result,
                      hepem_track_state* final_tracks) {
  if (!s || !done) return hepem::set_error(HEPEM_BAD_ARG, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return hepem::set_error(HEPEM_BAD_ARG, "unknown request id");
  *done = it->second->done ? 1 : 0;
  if (!it->second->done) return HEPEM_OK;
  const int st = take_result(s, it->second.get(), result, final_tracks);
  return st == HEPEM_OK ? HEPEM_OK : hepem::set_error(st, "request did not complete");
}

int hepem_server_wait(hepem_server* s, int64_t request_id, double timeout_s, hepem_request_result* result,
                      hepem_track_state* final_tracks) {
  if (!s) return hepem::set_error(HEPEM_BAD_ARG, "null server");
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return hepem::set_error(HEPEM_BAD_ARG, "unknown request id");
  Request* r = it->second.get();
  const bool ok = s->cvDone.wait_for(lock, std::chrono::duration<double>(timeout_s), [&] { return r->done; });
  if (!ok) return hepem::set_error(HEPEM_TIMEOUT, "request not finished within the timeout");
  const int st = take_result(s, r, result, final_tracks);
  return st == HEPEM_OK ? HEPEM_OK : hepem::set_error(st, "request did not complete");
}

int hepem_server_cancel(hepem_server* s, int64_t request_id) {
  if (!s) return hepem::set_error(HEPEM_BAD_ARG, "null server");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return hepem::set_error(HEPEM_BAD_ARG, "unknown request id");
  Request* r = it->second.get();
  r->cancelled = true;
  if (r->slot0 < 0 && !r->done) {          // still waiting: finish it now
    s->waiting.erase(std::find(s->waiting.begin(), s->waiting.end(), request_id));
    r->done = true;
    r->result.n_tracks = r->n;
    r->result.status = HEPEM_CANCELLED;
    r->result.t_submit = r->tSubmit;
    r->result.t_done = now_s();
    s->cvDone.notify_all();
  }
  return HEPEM_OK;
}

int hepem_server_get_stats(hepem_server* s, hepem_server_stats* out) {
  if (!s || !out) return hepem::set_error(HEPEM_BAD_ARG, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  memset(out, 0, sizeof(*out));
  out->iterations = s->iterations;
  out->track_steps = s->trackSteps;
  out->completed = s->completed;
  out->waiting = (int64_t)s->waiting.size();
  out->active = (int64_t)s->activeReq.size();
  std::vector<double> b = s->batchMs;
  if (!b.empty()) {
    std::sort(b.begin(), b.end());
    out->batch_ms_p50 = b[b.size() / 2];
    out->batch_ms_p99 = b[std::min(b.size() - 1, (size_t)(0.99 * b.size()))];
  }
  int64_t freeSlots = 0;
  for (auto& kv : s->freeRanges) freeSlots += kv.second;
  out->free_slots = freeSlots;
  return HEPEM_OK;
}

int hepem_server_reset_stats(hepem_server* s) {
  if (!s) return hepem::set_error(HEPEM_BAD_ARG, "null server");
  std::lock_guard<std::mutex> lock(s->mu);
  s->batchMs.clear();
  s->iterations = 0;
  s->trackSteps = 0;
  s->completed = 0;
  return HEPEM_OK;
}

// ---- snapshot / resume -----------------------------------------------------------------
// Layout (host byte order):
//   "HEPEMSNP" | u32 version | u32 0 | u64 requests | u64 tracks |
//   per request, in id order: i64 id | i64 n | u64 seed | i32 steps |
//     u8 admitted | u8 cancelled | u16 0 | the 20 state arrays (hepem_track_state
//     order, n elements each) | f64 edep[n] | f64 e_sec[n] | i32 n_sec[n] | i32 steps[n] |
//   u64 FNV-1a checksum of everything before it.
int hepem_server_snapshot(hepem_server* s, void* buf, size_t capacity, size_t* size) {
  if (!s || !size) return hepem::set_error(HEPEM_BAD_ARG, "null argument");
  hepem::TraceRange trace("hepem_server_snapshot", 0);
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->snapWaiters += 1;
  }
  struct Leave {
    hepem_server* s;
    ~Leave() {
      {
        std::lock_guard<std::mutex> lock(s->mu);
        s->snapWaiters -= 1;
      }
      s->cvSnap.notify_all();
    }
  } leave{s};
  std::lock_guard<std::mutex> iter(s->iterMu);
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->loopError != HEPEM_OK) return hepem::set_error(s->loopError, "server loop stopped: " + s->loopErrorMsg);
  std::vector<Request*> list;
  for (auto& kv : s->reqs)
    if (!kv.second->done) list.push_back(kv.second.get());
  std::sort(list.begin(), list.end(), [](const Request* a, const Request* b) { return a->id < b->id; });
  size_t per = 0;
  for (size_t b : kStateSizes) per += b;
  per += kSnapSumBytes;
  size_t need = kSnapHeader + 8;
  int64_t tracks = 0;
  for (const Request* r : list) {
    need += kSnapRecord + per * (size_t)r->n;
    tracks += r->n;
  }
  *size = need;
  if (!buf) return HEPEM_OK;
  if (capacity < need) return hepem::set_error(HEPEM_BAD_ARG, "snapshot buffer too small");
  uint8_t* p = static_cast<uint8_t*>(buf);
  memcpy(p, kSnapMagic, 8);
  const uint32_t ver[2] = {kSnapVersion, 0};
  memcpy(p + 8, ver, 8);
  const uint64_t counts[2] = {(uint64_t)list.size(), (uint64_t)tracks};
  memcpy(p + 16, counts, 16);
  p += kSnapHeader;
  for (const Request* r : list) {
    const int64_t n = r->n;
    const int32_t steps = r->steps;
    const uint8_t flags[4] = {(uint8_t)(r->slot0 >= 0), (uint8_t)r->cancelled.load(), 0, 0};
    memcpy(p, &r->id, 8);
    memcpy(p + 8, &n, 8);
    memcpy(p + 16, &r->seed, 8);
    memcpy(p + 24, &steps, 4);
    memcpy(p + 28, flags, 4);
    p += kSnapRecord;
    if (r->slot0 >= 0) {
      // resident: the state and sums as of the last completed iteration
      for (int k = 0; k < 20; ++k) {
        const cudaError_t e = cudaMemcpyAsync(p, s->state_ptr(k, r->slot0), kStateSizes[k] * n,
                                              cudaMemcpyDeviceToHost, s->stream);
        if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, cudaGetErrorString(e));
        p += kStateSizes[k] * n;
      }
      const void* src[4] = {s->edepSum + r->slot0, s->eSecSum + r->slot0, s->nSecSum + r->slot0,
                            s->stepSum + r->slot0};
      const size_t sz[4] = {8, 8, 4, 4};
      for (int k = 0; k < 4; ++k) {
        const cudaError_t e = cudaMemcpyAsync(p, src[k], sz[k] * n, cudaMemcpyDeviceToHost, s->stream);
        if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, cudaGetErrorString(e));
        p += sz[k] * n;
      }
    } else {
      memcpy(p, r->host.data(), r->host.size());
      p += r->host.size();
      memset(p, 0, kSnapSumBytes * n);
      p += kSnapSumBytes * n;
    }
  }
  const cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return hepem::set_error(HEPEM_CUDA_ERROR, cudaGetErrorString(e));
  const uint64_t sum = hepem::fnv1a(static_cast<const uint8_t*>(buf), need - 8);
  memcpy(p, &sum, 8);
  return HEPEM_OK;
}

int hepem_server_snapshot_check(const void* buf, size_t size, int64_t* n_requests, int64_t* n_tracks) {
  std::vector<SnapRec> recs;
  const int rc = parse_snapshot(buf, size, recs);
  if (rc != HEPEM_OK) return rc;
  int64_t t = 0;
  for (const SnapRec& r : recs) t += r.n;
  if (n_requests) *n_requests = (int64_t)recs.size();
  if (n_tracks) *n_tracks = t;
  return HEPEM_OK;
}

int hepem_server_resume(hepem_server* s, const void* buf, size_t size, int64_t max_ids, int64_t* old_ids,
                        int64_t* new_ids, int64_t* n_requests) {
  if (!s || !n_requests) return hepem::set_error(HEPEM_BAD_ARG, "null argument");
  hepem::TraceRange trace("hepem_server_resume", (int64_t)size);
  std::vector<SnapRec> recs;
  const int rc = parse_snapshot(buf, size, recs);
  if (rc != HEPEM_OK) return rc;
  *n_requests = (int64_t)recs.size();
  if ((int64_t)recs.size() > max_ids || (!recs.empty() && (!old_ids || !new_ids)))
    return hepem::set_error(HEPEM_BAD_ARG, "id arrays smaller than the snapshot's request count");
  for (const SnapRec& r : recs)
    if (r.n > s->capacity)
      return hepem::set_error(HEPEM_OOM_ADMISSION, "snapshot request larger than the server's memory budget");
  std::vector<std::unique_ptr<Request>> made;
  size_t per = 0;
  for (size_t b : kStateSizes) per += b;
  for (const SnapRec& q : recs) {
    std::unique_ptr<Request> r(new Request());
    r->n = q.n;
    r->seed = q.seed;
    r->steps = q.steps;
    r->cancelled = q.cancelled;
    r->host.assign(q.state, q.state + per * (size_t)q.n);
    if (q.admitted) r->sums.assign(q.state + per * (size_t)q.n, q.state + (per + kSnapSumBytes) * (size_t)q.n);
    r->tSubmit = now_s();
    made.push_back(std::move(r));
  }
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->loopError != HEPEM_OK) return hepem::set_error(s->loopError, "server loop stopped: " + s->loopErrorMsg);
  for (size_t k = 0; k < made.size(); ++k) {
    made[k]->id = s->nextId++;
    old_ids[k] = recs[k].id;
    new_ids[k] = made[k]->id;
    s->waiting.push_back(made[k]->id);
    s->reqs[made[k]->id] = std::move(made[k]);
  }
  s->cv.notify_all();
  return HEPEM_OK;
}

int hepem_server_destroy(hepem_server* s) {
  if (!s) return HEPEM_OK;
  s->stop.store(true);
  s->cv.notify_all();
  if (s->loop.joinable()) s->loop.join();
  cudaStreamSynchronize(s->stream);
  cudaFree(s->pool);
  cudaFree(s->dReq);
  cudaFreeHost(s->hReq);
  cudaStreamDestroy(s->stream);
  delete s;
  return HEPEM_OK;
}

}  // extern "C"
