// api.cu -- the extern "C" boundary declared in include/g4hepem_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <stdexcept>
#include <string>
#include <vector>

#include "g4hepem_gb300.h"
#include "ctx.h"
#include "kernels.h"
#include "rng.cuh"
#include "state_image.h"
#include "trace.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(HEPEM_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
}

#define HEPEM_CUDA(call)                              \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// contexts start without the L2 table window: with it, the precision-form
// step of 4,194,304 mixed tracks took 4-5% longer on a GB300 (three and
// sixteen couples; the FP64 batched step unchanged) -- the tables already
// stay in L1/L2 under ordinary caching
constexpr bool kTableWindowByDefault = false;

int create_from_image(hepem::StateImage& img, hepem_ctx** out) {
  int dev = 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(HEPEM_NO_DEVICE, "no CUDA device");
  HEPEM_CUDA(cudaGetDevice(&dev));
  hepem_ctx* c = new hepem_ctx();
  c->device = dev;
  cudaError_t e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMalloc(&c->arena, img.bytes.size());
  if (e == cudaSuccess) e = cudaMemcpy(c->arena, img.bytes.data(), img.bytes.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (c->arena) cudaFree(c->arena);
    delete c;
    return cuda_fail(e, "arena upload");
  }
  c->arenaBytes = img.bytes.size();
  hepem::relocate(img, c->tables, c->arena);
  // side streams of the batched steps; without them a step runs on one stream
  bool sideOk = true;
  for (cudaStream_t& st : c->side.st)
    sideOk = sideOk && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
  for (cudaEvent_t& ev : c->side.ev)
    sideOk = sideOk && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
  c->sideReady = sideOk;
  if (kTableWindowByDefault) hepem::set_table_window(c, 1);
  *out = c;
  return HEPEM_OK;
}

bool state_ok(const hepem_track_state* s) {
  return s && s->type && s->imc && s->id && s->ekin && s->dir_x && s->dir_y && s->dir_z && s->nia0 && s->nia1 &&
         s->nia2 && s->nia3 && s->safety && s->on_boundary && s->msc_init_range && s->msc_dyn_factor &&
         s->msc_tlimit_min && s->msc_first_step && s->gauss_valid && s->gauss_value && s->rng_cursor;
}

bool out_ok(const hepem_step_out* r) {
  return r && r->edep && r->gstep && r->pstep && r->winner && r->disp_x && r->disp_y && r->disp_z && r->flags &&
         r->n_sec && r->sec_type && r->sec_ekin && r->sec_dir_x && r->sec_dir_y && r->sec_dir_z;
}

// Byte size of each per-track array, in the field order of the structs.
const size_t kStateSizes[20] = {1, 4, 4, 8, 8, 8, 8, 8, 8, 8, 8, 8, 1, 8, 8, 8, 1, 1, 8, 4};
const size_t kOutSizes[14] = {8, 8, 8, 1, 8, 8, 8, 1, 1, 2, 16, 16, 16, 16};  // secondaries: 2 slots

}  // namespace

namespace hepem {
int set_error(int code, const std::string& msg) { return fail(code, msg); }
bool valid_state(const hepem_track_state* s) { return state_ok(s); }
bool valid_out(const hepem_step_out* r) { return out_ok(r); }
}  // namespace hepem

extern "C" {

const char* hepem_status_string(int s) {
  switch (s) {
    case HEPEM_OK: return "ok";
    case HEPEM_BAD_ARG: return "bad argument";
    case HEPEM_PARSE_ERROR: return "state JSON does not follow the G4HepEmState schema";
    case HEPEM_CUDA_ERROR: return "CUDA error";
    case HEPEM_RNG_EXHAUSTED: return "a track read past its buffered uniforms";
    case HEPEM_TIMEOUT: return "bounded wait gave up";
    case HEPEM_OOM_ADMISSION: return "request exceeds the memory budget";
    case HEPEM_NO_DEVICE: return "no CUDA device";
    case HEPEM_CANCELLED: return "request cancelled";
    default: return "unknown status";
  }
}

const char* hepem_last_error(void) { return g_last_error.c_str(); }

int hepem_create(const char* json, size_t len, hepem_ctx** out) {
  hepem::TraceRange trace("hepem_create", (int64_t)len);
  if (!json || !out) return fail(HEPEM_BAD_ARG, "null argument");
  *out = nullptr;
  try {
    hepem::StateImage img = hepem::build_state_image(json, len);
    return create_from_image(img, out);
  } catch (const std::exception& e) {
    return fail(HEPEM_PARSE_ERROR, e.what());
  }
}

int hepem_create_from_file(const char* path, hepem_ctx** out) {
  hepem::TraceRange trace("hepem_create_from_file", 0);
  if (!path || !out) return fail(HEPEM_BAD_ARG, "null argument");
  *out = nullptr;
  try {
    hepem::StateImage img = hepem::build_state_image_file(path);
    return create_from_image(img, out);
  } catch (const std::exception& e) {
    return fail(HEPEM_PARSE_ERROR, e.what());
  }
}

int hepem_image_from_json(const char* json, size_t len, void* out, size_t capacity, size_t* size) {
  hepem::TraceRange trace("hepem_image_from_json", (int64_t)len);
  if (!json || !size) return fail(HEPEM_BAD_ARG, "null argument");
  try {
    const std::vector<uint8_t> img = hepem::serialize_image(hepem::build_state_image(json, len));
    *size = img.size();
    if (!out) return HEPEM_OK;
    if (capacity < img.size()) return fail(HEPEM_BAD_ARG, "image buffer too small");
    memcpy(out, img.data(), img.size());
    return HEPEM_OK;
  } catch (const std::exception& e) {
    return fail(HEPEM_PARSE_ERROR, e.what());
  }
}

int hepem_image_check(const void* image, size_t size, int64_t* arena_bytes) {
  hepem::TraceRange trace("hepem_image_check", (int64_t)size);
  try {
    hepem::StateImage img = hepem::deserialize_image(image, size);
    if (arena_bytes) *arena_bytes = (int64_t)img.bytes.size();
    return HEPEM_OK;
  } catch (const std::exception& e) {
    return fail(HEPEM_PARSE_ERROR, e.what());
  }
}

int hepem_create_from_image(const void* image, size_t size, hepem_ctx** out) {
  hepem::TraceRange trace("hepem_create_from_image", (int64_t)size);
  if (!image || !out) return fail(HEPEM_BAD_ARG, "null argument");
  *out = nullptr;
  try {
    hepem::StateImage img = hepem::deserialize_image(image, size);
    return create_from_image(img, out);
  } catch (const std::exception& e) {
    return fail(HEPEM_PARSE_ERROR, e.what());
  }
}

int hepem_destroy(hepem_ctx* c) {
  if (!c) return HEPEM_OK;
  // the context's own streams finish before the tables they read go away
  for (cudaStream_t ps : c->pipe)
    if (ps) cudaStreamSynchronize(ps);
  for (cudaStream_t st : c->side.st)
    if (st) cudaStreamSynchronize(st);
  cudaError_t e = cudaSuccess;
  if (c->arena) e = cudaFree(c->arena);
  for (cudaStream_t st : c->side.st)
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t ev : c->side.ev)
    if (ev) cudaEventDestroy(ev);
  if (c->pipeBuf) cudaFree(c->pipeBuf);
  for (int k = 0; k < hepem_ctx::kMaxChunks; ++k) {
    if (c->chunkIn[k]) cudaEventDestroy(c->chunkIn[k]);
    if (c->chunkStepped[k]) cudaEventDestroy(c->chunkStepped[k]);
  }
  for (cudaStream_t ps : c->pipe)
    if (ps) cudaStreamDestroy(ps);
  if (c->start) cudaEventDestroy(c->start);
  if (c->finished) cudaEventDestroy(c->finished);
  if (c->splitBuf) cudaFree(c->splitBuf);
  if (c->stageEvReady)
    for (auto& e2 : c->stageEv) cudaEventDestroy(e2);
  delete c;
  return e == cudaSuccess ? HEPEM_OK : cuda_fail(e, "cudaFree");
}

int hepem_info(const hepem_ctx* c, int32_t* nc, int32_t* nm, int32_t* nr, int64_t* bytes) {
  if (!c) return fail(HEPEM_BAD_ARG, "null context");
  if (nc) *nc = c->tables.nCouples;
  if (nm) *nm = c->tables.nMats;
  if (nr) *nr = c->tables.nRegions;
  if (bytes) *bytes = (int64_t)c->arenaBytes;
  return HEPEM_OK;
}

int hepem_electron_lookup(const hepem_ctx* c, int64_t n, int is_positron, const double* ekin, const int32_t* imc,
                          double* xi, double* xb, double* dedx, double* range, double* invr, void* stream) {
  if (!c || n < 0) return fail(HEPEM_BAD_ARG, "bad context or size");
  if (n == 0) return HEPEM_OK;
  if (!ekin || !imc || !xi || !xb || !dedx || !range || !invr) return fail(HEPEM_BAD_ARG, "null array");
  HEPEM_CUDA(hepem::launch_lookup(c->tables, n, is_positron ? 1 : 0, ekin, imc, xi, xb, dedx, range, invr,
                                  (cudaStream_t)stream, c->sms));
  return HEPEM_OK;
}

int hepem_electron_lookup_mixed(const hepem_ctx* c, int64_t n, int is_positron, const double* ekin,
                                const int32_t* imc, double* xi, double* xb, double* dedx, double* range,
                                double* invr, void* stream) {
  if (!c || n < 0) return fail(HEPEM_BAD_ARG, "bad context or size");
  if (n == 0) return HEPEM_OK;
  if (!ekin || !imc || !xi || !xb || !dedx || !range || !invr) return fail(HEPEM_BAD_ARG, "null array");
  HEPEM_CUDA(hepem::launch_lookup_mixed(c->tables, n, is_positron ? 1 : 0, ekin, imc, xi, xb, dedx, range, invr,
                                        (cudaStream_t)stream, c->sms));
  return HEPEM_OK;
}

int hepem_sample_model(const hepem_ctx* c, int model, int precision, int64_t n, double ekin, int32_t imc,
                       uint64_t seed, double* out, uint64_t* n_fallback, void* stream) {
  if (!c || n < 0 || model < 0 || model > 5 || !(precision == 0 || precision == 1))
    return fail(HEPEM_BAD_ARG, "bad context, size, model or precision");
  if (!(imc >= 0 && imc < c->tables.nCouples) || !(ekin > 0.0 && ekin < 1.0e300))
    return fail(HEPEM_BAD_ARG, "bad couple index or energy");
  if (n == 0) return HEPEM_OK;
  if (!out) return fail(HEPEM_BAD_ARG, "null output");
  HEPEM_CUDA(hepem::launch_sample(c->tables, model, precision, n, ekin, imc, seed, out,
                                  reinterpret_cast<unsigned long long*>(n_fallback), (cudaStream_t)stream, c->sms));
  return HEPEM_OK;
}

int hepem_woodcock_gamma(const hepem_ctx* c, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                         double* px, double* py, double* pz, const hepem_layered_box* box, const double* uniforms,
                         int32_t nu, uint64_t seed, hepem_step_out* res, uint8_t* reached, void* stream) {
  if (!c || n < 0 || nu < 0 || !box) return fail(HEPEM_BAD_ARG, "bad context, size or box");
  if (n == 0) return HEPEM_OK;
  if (!state_ok(in) || !state_ok(out) || !out_ok(res) || (nu > 0 && !uniforms) || !px || !py || !pz)
    return fail(HEPEM_BAD_ARG, "null array in track batch");
  if (box->n_layers < 1 || !box->z_bounds || !box->layer_imc || !(box->half_x > 0.0) || !(box->half_y > 0.0) ||
      box->wdt_imc < 0 || box->wdt_imc >= c->tables.nCouples)
    return fail(HEPEM_BAD_ARG, "bad layered box");
  // the layer arrays are device arrays: check them on the host once (small)
  std::vector<double> zb(box->n_layers + 1);
  std::vector<int32_t> li(box->n_layers);
  HEPEM_CUDA(cudaMemcpy(zb.data(), box->z_bounds, sizeof(double) * zb.size(), cudaMemcpyDeviceToHost));
  HEPEM_CUDA(cudaMemcpy(li.data(), box->layer_imc, sizeof(int32_t) * li.size(), cudaMemcpyDeviceToHost));
  for (int32_t k = 0; k < box->n_layers; ++k)
    if (!(zb[k] < zb[k + 1]) || li[k] < 0 || li[k] >= c->tables.nCouples)
      return fail(HEPEM_BAD_ARG, "layer bounds must increase and layer couples must exist");
  hepem::TraceRange trace("hepem_woodcock_gamma", n);
  HEPEM_CUDA(hepem::launch_woodcock(c->tables, n, *in, *out, px, py, pz, *box, uniforms, nu, seed, *res, reached,
                                    (cudaStream_t)stream, c->sms));
  return HEPEM_OK;
}

int hepem_step(const hepem_ctx* c, int64_t n, const hepem_track_state* in, hepem_track_state* out,
               const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res,
               hepem_step_counters* counters, void* stream) {
  if (!c || n < 0 || nu < 0) return fail(HEPEM_BAD_ARG, "bad context or size");
  if (n == 0) return HEPEM_OK;
  if (!state_ok(in) || !state_ok(out) || !out_ok(res) || (nu > 0 && !uniforms))
    return fail(HEPEM_BAD_ARG, "null array in track batch");
  if (n > (int64_t)INT32_MAX * 2 / 3) return fail(HEPEM_BAD_ARG, "batch too large");
  hepem::TraceRange trace("hepem_step", n);
  HEPEM_CUDA(hepem::launch_step(c->tables, n, *in, *out, uniforms, nu, seed, *res, counters, (cudaStream_t)stream,
                                c->sms));
  return HEPEM_OK;
}

namespace {
int step_batched(const hepem_ctx* c, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                 const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res,
                 hepem_step_counters* counters, void* stream, bool mixed) {
  if (!c || n < 0 || nu < 0) return fail(HEPEM_BAD_ARG, "bad context or size");
  if (n == 0) return HEPEM_OK;
  if (!state_ok(in) || !state_ok(out) || !out_ok(res) || (nu > 0 && !uniforms))
    return fail(HEPEM_BAD_ARG, "null array in track batch");
  if (n > (int64_t)INT32_MAX) return fail(HEPEM_BAD_ARG, "batch too large");
  hepem::TraceRange trace(mixed ? "hepem_step_mixed" : "hepem_step_batched", n);
  cudaStream_t s = (cudaStream_t)stream;
  // an in-place precision-form step keeps a copy of the pre-step state of the
  // e+- tracks that reach an FP32 interaction (their FP64 fallback restarts there)
  const bool preCopy = mixed && in->ekin == out->ekin;
  const size_t wsBytes = hepem::batched_workspace_bytes(n);
  const size_t preBytes = preCopy ? hepem::mixed_pre_state_bytes(n) : 0;
  // no caller uniforms: room to draw the streams' first values ahead
  const size_t fillBytes = hepem::wants_prefill(n, nu) ? hepem::prefill_bytes(n, 0) : 0;
  void* ws = nullptr;
  HEPEM_CUDA(cudaMallocAsync(&ws, wsBytes + preBytes + fillBytes, s));
  hepem::BatchOpts o;
  o.ev = c->profile ? const_cast<cudaEvent_t*>(c->stageEv) : nullptr;
  o.cfg = &c->launch;
  o.mixed = mixed;
  hepem::apply_table_window(c, o);
  hepem_track_state pre;
  if (preCopy) {
    pre = hepem::carve_pre_state(static_cast<uint8_t*>(ws) + wsBytes, n, *in);
    o.preState = &pre;
  }
  if (fillBytes) o.prefill = static_cast<uint8_t*>(ws) + wsBytes + preBytes;
  cudaError_t e = hepem::launch_step_batched(c->tables, n, *in, *out, uniforms, nu, seed, *res, counters, ws, s,
                                             c->sms, o);
  cudaError_t f = cudaFreeAsync(ws, s);
  if (e != cudaSuccess) return cuda_fail(e, "batched step launch");
  if (f != cudaSuccess) return cuda_fail(f, "cudaFreeAsync");
  return HEPEM_OK;
}
}  // namespace

int hepem_step_batched(const hepem_ctx* c, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                       const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res,
                       hepem_step_counters* counters, void* stream) {
  return step_batched(c, n, in, out, uniforms, nu, seed, res, counters, stream, false);
}

int hepem_step_mixed(const hepem_ctx* c, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                     const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res,
                     hepem_step_counters* counters, void* stream) {
  return step_batched(c, n, in, out, uniforms, nu, seed, res, counters, stream, true);
}

int hepem_step_subbatches(const hepem_ctx* c, int form, int32_t nb, const hepem_subbatch* batches,
                          const hepem_track_state* in, hepem_track_state* out, const double* uniforms, int32_t nu,
                          hepem_step_out* res, hepem_step_counters* counters, void* stream) {
  if (!c || nb < 0 || nu < 0) return fail(HEPEM_BAD_ARG, "bad context, sub-batch count or size");
  if (form != HEPEM_FORM_BATCHED && form != HEPEM_FORM_MIXED)
    return fail(HEPEM_BAD_ARG, "form must be HEPEM_FORM_BATCHED or HEPEM_FORM_MIXED");
  if (nb == 0) return HEPEM_OK;
  if (!batches) return fail(HEPEM_BAD_ARG, "null sub-batch array");
  std::vector<hepem_subbatch> b(batches, batches + nb);
  std::stable_sort(b.begin(), b.end(), [](const hepem_subbatch& x, const hepem_subbatch& y) {
    return x.offset < y.offset;
  });
  std::vector<int64_t> prefix(nb + 1, 0);
  int64_t end = 0, maxIdx = 0;
  for (int k = 0; k < nb; ++k) {
    if (b[k].offset < 0 || b[k].n < 0) return fail(HEPEM_BAD_ARG, "negative sub-batch offset or size");
    if (b[k].n > 0 && b[k].offset < end) return fail(HEPEM_BAD_ARG, "sub-batches overlap");
    if (b[k].n > 0) end = b[k].offset + b[k].n;
    prefix[k + 1] = prefix[k] + b[k].n;
    if (end > maxIdx) maxIdx = end;
  }
  const int64_t total = prefix[nb];
  if (total == 0) return HEPEM_OK;
  hepem::TraceRange trace("hepem_step_subbatches", total);
  if (maxIdx > (int64_t)INT32_MAX) return fail(HEPEM_BAD_ARG, "batch too large");
  if (!state_ok(in) || !state_ok(out) || !out_ok(res) || (nu > 0 && !uniforms))
    return fail(HEPEM_BAD_ARG, "null array in track batch");
  cudaStream_t s = (cudaStream_t)stream;
  const bool mixed = form == HEPEM_FORM_MIXED;
  const bool preCopy = mixed && in->ekin == out->ekin;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t wsBytes = al(hepem::batched_workspace_bytes(total));
  const size_t preBytes = preCopy ? al(hepem::mixed_pre_state_bytes(maxIdx)) : 0;
  // no caller uniforms: room to draw the streams' first values ahead
  const size_t fillBytes = hepem::wants_prefill(total, nu) ? hepem::prefill_bytes(total, maxIdx) : 0;
  const size_t need = wsBytes + al(4 * (size_t)total) + al(8 * (size_t)maxIdx) + al(sizeof(hepem_subbatch) * nb) +
                      al(8 * (size_t)(nb + 1)) + preBytes + fillBytes;
  void* ws = nullptr;
  HEPEM_CUDA(cudaMallocAsync(&ws, need, s));
  uint8_t* p = static_cast<uint8_t*>(ws) + wsBytes;
  int32_t* active = reinterpret_cast<int32_t*>(p);
  p += al(4 * (size_t)total);
  uint64_t* keys = reinterpret_cast<uint64_t*>(p);
  p += al(8 * (size_t)maxIdx);
  hepem_subbatch* dB = reinterpret_cast<hepem_subbatch*>(p);
  p += al(sizeof(hepem_subbatch) * nb);
  int64_t* dPrefix = reinterpret_cast<int64_t*>(p);
  p += al(8 * (size_t)(nb + 1));
  // pageable host -> device copies return once the host arrays have been read
  cudaError_t e = cudaMemcpyAsync(dB, b.data(), sizeof(hepem_subbatch) * nb, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dPrefix, prefix.data(), 8 * (size_t)(nb + 1), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = hepem::launch_subbatch_index(dB, dPrefix, nb, total, active, keys, s, c->sms);
  if (e == cudaSuccess) {
    hepem::BatchOpts o;
    o.ev = c->profile ? const_cast<cudaEvent_t*>(c->stageEv) : nullptr;
    o.cfg = &c->launch;
    o.mixed = mixed;
    o.active = active;
    o.seeds = keys;
    hepem::apply_table_window(c, o);
    hepem_track_state pre;
    if (preCopy) {
      pre = hepem::carve_pre_state(p, maxIdx, *in);
      o.preState = &pre;
    }
    if (fillBytes) o.prefill = p + preBytes;
    e = hepem::launch_step_batched(c->tables, total, *in, *out, uniforms, nu, 0, *res, counters, ws, s, c->sms, o);
  }
  const cudaError_t f = cudaFreeAsync(ws, s);
  if (e != cudaSuccess) return cuda_fail(e, "sub-batch step launch");
  if (f != cudaSuccess) return cuda_fail(f, "cudaFreeAsync");
  return HEPEM_OK;
}

namespace {
int step_host(const hepem_ctx* cc, int64_t n, const hepem_track_state* in, hepem_track_state* out,
              const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res, hepem_step_counters* counters,
              void* stream, bool mixed) {
  hepem_ctx* c = const_cast<hepem_ctx*>(cc);
  if (!c || n < 0 || nu < 0) return fail(HEPEM_BAD_ARG, "bad context or size");
  if (n == 0) return HEPEM_OK;
  if (!state_ok(in) || !state_ok(out) || !out_ok(res) || (nu > 0 && !uniforms))
    return fail(HEPEM_BAD_ARG, "null array in track batch");
  if (n > (int64_t)INT32_MAX) return fail(HEPEM_BAD_ARG, "batch too large");
  hepem::TraceRange trace(mixed ? "hepem_step_host_mixed" : "hepem_step_host", n);
  std::lock_guard<std::mutex> lock(c->mu);
  cudaStream_t s = (cudaStream_t)stream;
  // The batch is cut into up to kMaxChunks chunks, each with a device buffer
  // of its own, and the work goes to three streams: the copies in (one chunk
  // after the other, as fast as the link takes them), the steps (each chunk
  // once its copy is in, alone on the GPU) and the copies out (each chunk
  // once stepped).  The link towards the host is the slowest of the three:
  // it stays busy from the end of the first chunk's step to the end.
  const int kc = hepem_ctx::kMaxChunks;
  const int64_t m = std::min<int64_t>(n, std::max<int64_t>(1 << 16, ((n + kc - 1) / kc + 255) / 256 * 256));
  const int nChunks = (int)((n + m - 1) / m);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t need = 0;
  for (size_t b : kStateSizes) need += al(b * m);
  for (size_t b : kOutSizes) need += al(b * m);
  need += al(sizeof(double) * (size_t)m * nu) + al(hepem::batched_workspace_bytes(m));
  // the precision form steps the chunk in place: room for its pre-step copy
  const size_t preBytes = mixed ? al(hepem::mixed_pre_state_bytes(m)) : 0;
  need += preBytes;
  // no caller uniforms: room to draw the streams' first values ahead
  const bool fill = hepem::wants_prefill(m, nu);
  if (fill) need += hepem::prefill_bytes(m, 0);
  const size_t total = need * (size_t)nChunks + al(sizeof(hepem_step_counters));
  if (!c->pipeReady) {
    for (cudaStream_t& ps : c->pipe) HEPEM_CUDA(cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking));
    for (int k = 0; k < kc; ++k) {
      HEPEM_CUDA(cudaEventCreateWithFlags(&c->chunkIn[k], cudaEventDisableTiming));
      HEPEM_CUDA(cudaEventCreateWithFlags(&c->chunkStepped[k], cudaEventDisableTiming));
    }
    HEPEM_CUDA(cudaEventCreateWithFlags(&c->start, cudaEventDisableTiming));
    HEPEM_CUDA(cudaEventCreateWithFlags(&c->finished, cudaEventDisableTiming));
    c->pipeReady = true;
  }
  if (total > c->pipeBytes) {
    for (cudaStream_t ps : c->pipe) HEPEM_CUDA(cudaStreamSynchronize(ps));
    if (c->pipeBuf) HEPEM_CUDA(cudaFree(c->pipeBuf));
    c->pipeBuf = nullptr;
    c->pipeBytes = 0;
    HEPEM_CUDA(cudaMalloc(&c->pipeBuf, total));
    c->pipeBytes = total;
  }
  const cudaStream_t sIn = c->pipe[0], sStep = c->pipe[1], sOut = c->pipe[2];
  HEPEM_CUDA(cudaEventRecord(c->start, s));
  for (cudaStream_t ps : c->pipe) HEPEM_CUDA(cudaStreamWaitEvent(ps, c->start, 0));
  hepem_step_counters* cnt =
      reinterpret_cast<hepem_step_counters*>(static_cast<uint8_t*>(c->pipeBuf) + need * (size_t)nChunks);
  if (counters) HEPEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(*cnt), sStep));
  void* const* hin = reinterpret_cast<void* const*>(in);
  void* const* hout = reinterpret_cast<void* const*>(out);
  void* const* hres = reinterpret_cast<void* const*>(res);
  static_assert(sizeof(hepem_track_state) == 20 * sizeof(void*), "state struct layout");
  static_assert(sizeof(hepem_step_out) == 14 * sizeof(void*), "out struct layout");
  for (int ch = 0; ch < nChunks; ++ch) {
    const int64_t off = (int64_t)ch * m;
    const int64_t mc = std::min<int64_t>(m, n - off);
    uint8_t* p = static_cast<uint8_t*>(c->pipeBuf) + need * (size_t)ch;
    void* dstate[20];
    void* dout[14];
    for (int k = 0; k < 20; ++k) { dstate[k] = p; p += al(kStateSizes[k] * m); }
    for (int k = 0; k < 14; ++k) { dout[k] = p; p += al(kOutSizes[k] * m); }
    double* du = (double*)p;
    p += al(sizeof(double) * (size_t)m * nu);
    void* dwork = p;
    p += al(hepem::batched_workspace_bytes(m));
    void* dpre = p;
    hepem_track_state ds;
    hepem_step_out dr;
    memcpy(&ds, dstate, sizeof(ds));
    memcpy(&dr, dout, sizeof(dr));
    for (int k = 0; k < 20; ++k)
      HEPEM_CUDA(cudaMemcpyAsync(dstate[k], (const uint8_t*)hin[k] + kStateSizes[k] * off, kStateSizes[k] * mc,
                                 cudaMemcpyHostToDevice, sIn));
    if (nu > 0)
      HEPEM_CUDA(cudaMemcpyAsync(du, uniforms + off * nu, sizeof(double) * (size_t)mc * nu, cudaMemcpyHostToDevice,
                                 sIn));
    HEPEM_CUDA(cudaEventRecord(c->chunkIn[ch], sIn));
    HEPEM_CUDA(cudaStreamWaitEvent(sStep, c->chunkIn[ch], 0));
    hepem::BatchOpts o;
    o.cfg = &c->launch;
    o.mixed = mixed;
    hepem::apply_table_window(c, o);
    hepem_track_state pre;
    if (mixed) {
      pre = hepem::carve_pre_state(dpre, m, ds);
      o.preState = &pre;
    }
    if (fill) o.prefill = static_cast<uint8_t*>(dpre) + preBytes;
    HEPEM_CUDA(hepem::launch_step_batched(c->tables, mc, ds, ds, du, nu, seed, dr, counters ? cnt : nullptr, dwork,
                                          sStep, c->sms, o));
    HEPEM_CUDA(cudaEventRecord(c->chunkStepped[ch], sStep));
    HEPEM_CUDA(cudaStreamWaitEvent(sOut, c->chunkStepped[ch], 0));
    // persistent per-track fields come back (type/imc/id/safety/boundary are inputs only)
    for (int k = 3; k < 20; ++k) {
      if (k == 11 || k == 12) continue;
      HEPEM_CUDA(cudaMemcpyAsync((uint8_t*)hout[k] + kStateSizes[k] * off, dstate[k], kStateSizes[k] * mc,
                                 cudaMemcpyDeviceToHost, sOut));
    }
    for (int k = 0; k < 14; ++k)
      HEPEM_CUDA(cudaMemcpyAsync((uint8_t*)hres[k] + kOutSizes[k] * off, dout[k], kOutSizes[k] * mc,
                                 cudaMemcpyDeviceToHost, sOut));
  }
  if (hout[0] != hin[0]) {
    // the fields a step does not change (type, couple, id, safety, boundary
    // status: 18 B per track), copied on the host while the device works, in
    // four threads (one thread copies ~15 GB/s: 5 ms for 4M tracks, as long
    // as the device pipeline itself)
    const int kPass[5] = {0, 1, 2, 11, 12};
    auto part = [&](int j, int parts) {
      for (int k : kPass) {
        const size_t b = kStateSizes[k] * (size_t)n;
        const size_t lo = b * j / parts, hi = b * (j + 1) / parts;
        memcpy(static_cast<uint8_t*>(hout[k]) + lo, static_cast<const uint8_t*>(hin[k]) + lo, hi - lo);
      }
    };
    const int parts = n >= (1 << 18) ? 4 : 1;
    std::vector<std::thread> th;
    for (int j = 1; j < parts; ++j) th.emplace_back(part, j, parts);
    part(0, parts);
    for (std::thread& x : th) x.join();
  }
  // every chunk's step precedes the last chunk's copies out on sOut
  hepem_step_counters hc;
  if (counters) HEPEM_CUDA(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, sOut));
  HEPEM_CUDA(cudaEventRecord(c->finished, sOut));
  HEPEM_CUDA(cudaStreamWaitEvent(s, c->finished, 0));
  HEPEM_CUDA(cudaStreamSynchronize(s));
  if (counters) *counters = hc;
  return HEPEM_OK;
}
}  // namespace

int hepem_step_host(const hepem_ctx* c, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                    const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res,
                    hepem_step_counters* counters, void* stream) {
  return step_host(c, n, in, out, uniforms, nu, seed, res, counters, stream, false);
}

int hepem_step_host_mixed(const hepem_ctx* c, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                          const double* uniforms, int32_t nu, uint64_t seed, hepem_step_out* res,
                          hepem_step_counters* counters, void* stream) {
  return step_host(c, n, in, out, uniforms, nu, seed, res, counters, stream, true);
}

// ---- single functions of the path (the reference's device-test quantities) -------------
namespace {
int probe(const hepem_ctx* c, hepem::ProbeArgs& a, int precision, void* stream) {
  if (!c || a.n < 0 || !(precision == 0 || precision == 1)) return fail(HEPEM_BAD_ARG, "bad context, size or precision");
  if (a.n == 0) return HEPEM_OK;
  if (!a.ekin || !a.imc) return fail(HEPEM_BAD_ARG, "null array");
  HEPEM_CUDA(hepem::launch_probe(c->tables, a, precision, (cudaStream_t)stream, c->sms));
  return HEPEM_OK;
}
}  // namespace

int hepem_electron_xs_stepping(const hepem_ctx* c, int64_t n, int is_positron, int precision, const double* ekin,
                               const int32_t* imc, double* xi, double* xb, double* xa, double* xn, double* tr,
                               void* stream) {
  if (n > 0 && (!xi || !xb || !xa || !xn || !tr)) return fail(HEPEM_BAD_ARG, "null output");
  hepem::ProbeArgs a{n, hepem::kProbeElXs, is_positron ? 1 : 0, 0, ekin, imc, nullptr, {xi, xb, xa, xn, tr}, nullptr};
  return probe(c, a, precision, stream);
}

int hepem_brem_select_target(const hepem_ctx* c, int64_t n, int is_positron, int is_sb, int precision,
                             const double* ekin, const int32_t* imc, const double* urnd, int32_t* elem,
                             void* stream) {
  if (n > 0 && (!urnd || !elem)) return fail(HEPEM_BAD_ARG, "null array");
  hepem::ProbeArgs a{n, hepem::kProbeBremTarget, is_positron ? 1 : 0, is_sb ? 1 : 0, ekin, imc, urnd, {}, elem};
  return probe(c, a, precision, stream);
}

int hepem_conv_select_target(const hepem_ctx* c, int64_t n, int precision, const double* ekin, const int32_t* imc,
                             const double* urnd, int32_t* elem, void* stream) {
  if (n > 0 && (!urnd || !elem)) return fail(HEPEM_BAD_ARG, "null array");
  hepem::ProbeArgs a{n, hepem::kProbeConvTarget, 0, 0, ekin, imc, urnd, {}, elem};
  return probe(c, a, precision, stream);
}

int hepem_gamma_xs(const hepem_ctx* c, int64_t n, int precision, const double* ekin, const int32_t* imc,
                   const double* urnd, double* xs_tot, double* xs_pe, int32_t* winner, void* stream) {
  if (n > 0 && (!urnd || !xs_tot || !xs_pe || !winner)) return fail(HEPEM_BAD_ARG, "null array");
  hepem::ProbeArgs a{n, hepem::kProbeGammaXs, 0, 0, ekin, imc, urnd, {xs_tot, xs_pe, nullptr, nullptr, nullptr},
                     winner};
  return probe(c, a, precision, stream);
}

// ---- HowFar and Perform as two calls ----------------------------------------------------
int64_t hepem_step_limit_bytes(int64_t n) { return n < 0 ? 0 : (int64_t)hepem::limits_bytes(n); }

namespace {
// one phase of the split step over device buffers (in == out for an in-place Perform)
int split_device(const hepem_ctx* c, int form, int phase, int64_t n, const hepem_track_state* in,
                 hepem_track_state* out, double* gstep, void* limits, const double* uniforms, int32_t nu,
                 uint64_t seed, hepem_step_out* res, hepem_step_counters* counters, cudaStream_t s) {
  const hepem::Limits L = hepem::carve_limits(limits, n);
  if (form == HEPEM_FORM_PLAIN) {
    if (phase == hepem::kPhaseHowFar)
      HEPEM_CUDA(hepem::launch_howfar(c->tables, n, *in, uniforms, nu, seed, gstep, L, counters, s, c->sms));
    else
      HEPEM_CUDA(hepem::launch_perform(c->tables, n, *in, *out, gstep, L, uniforms, nu, seed, *res, counters, s,
                                       c->sms));
    return HEPEM_OK;
  }
  const bool mixed = form == HEPEM_FORM_MIXED;
  const bool preCopy = mixed && phase == hepem::kPhasePerform && in->ekin == out->ekin;
  const size_t wsBytes = hepem::batched_workspace_bytes(n);
  void* ws = nullptr;
  HEPEM_CUDA(cudaMallocAsync(&ws, wsBytes + (preCopy ? hepem::mixed_pre_state_bytes(n) : 0), s));
  hepem::BatchOpts o;
  o.ev = c->profile ? const_cast<cudaEvent_t*>(c->stageEv) : nullptr;
  o.cfg = &c->launch;
  o.mixed = mixed;
  o.phase = phase;
  o.gstep = gstep;
  o.limits = L;
  hepem::apply_table_window(c, o);
  hepem_track_state pre;
  if (preCopy) {
    pre = hepem::carve_pre_state(static_cast<uint8_t*>(ws) + wsBytes, n, *in);
    o.preState = &pre;
  }
  // HowFar writes no track state and no results: `out` and `res` are not used
  hepem_step_out none;
  memset(&none, 0, sizeof(none));
  cudaError_t e = hepem::launch_step_batched(c->tables, n, *in, out ? *out : *in, uniforms, nu, seed,
                                             res ? *res : none, counters, ws, s, c->sms, o);
  cudaError_t f = cudaFreeAsync(ws, s);
  if (e != cudaSuccess) return cuda_fail(e, "split step launch");
  if (f != cudaSuccess) return cuda_fail(f, "cudaFreeAsync");
  return HEPEM_OK;
}

int split_check(const hepem_ctx* c, int form, int64_t n, int32_t nu, const hepem_track_state* in,
                const hepem_track_state* out, const void* gstep, const void* limits, const double* uniforms,
                const hepem_step_out* res, bool perform) {
  if (!c || n < 0 || nu < 0) return fail(HEPEM_BAD_ARG, "bad context or size");
  if (form != HEPEM_FORM_PLAIN && form != HEPEM_FORM_BATCHED && form != HEPEM_FORM_MIXED)
    return fail(HEPEM_BAD_ARG, "form must be HEPEM_FORM_PLAIN, HEPEM_FORM_BATCHED or HEPEM_FORM_MIXED");
  if (n == 0) return HEPEM_OK;
  if (!state_ok(in) || (perform && (!state_ok(out) || !out_ok(res))) || !gstep || !limits ||
      (nu > 0 && !uniforms))
    return fail(HEPEM_BAD_ARG, "null array in track batch");
  if (n > (int64_t)INT32_MAX * 2 / 3) return fail(HEPEM_BAD_ARG, "batch too large");
  return HEPEM_OK;
}

// host-buffer split step: inputs to one device buffer, the phase, outputs back
int split_host(const hepem_ctx* cc, int form, int phase, int64_t n, const hepem_track_state* in,
               hepem_track_state* out, double* gstep, void* limits, const double* uniforms, int32_t nu,
               uint64_t seed, hepem_step_out* res, hepem_step_counters* counters, cudaStream_t s) {
  hepem_ctx* c = const_cast<hepem_ctx*>(cc);
  std::lock_guard<std::mutex> lock(c->mu);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t m = (size_t)n;
  const size_t limBytes = hepem::limits_bytes(n);
  size_t need = al(sizeof(double) * m) + al(limBytes) + al(sizeof(double) * m * nu) + al(sizeof(hepem_step_counters));
  for (size_t b : kStateSizes) need += al(b * m);
  if (phase == hepem::kPhasePerform)
    for (size_t b : kOutSizes) need += al(b * m);
  if (need > c->splitBytes) {
    if (c->splitBuf) HEPEM_CUDA(cudaFree(c->splitBuf));
    c->splitBuf = nullptr;
    c->splitBytes = 0;
    HEPEM_CUDA(cudaMalloc(&c->splitBuf, need));
    c->splitBytes = need;
  }
  uint8_t* p = static_cast<uint8_t*>(c->splitBuf);
  double* dg = reinterpret_cast<double*>(p);
  p += al(sizeof(double) * m);
  void* dlim = p;
  p += al(limBytes);
  double* du = reinterpret_cast<double*>(p);
  p += al(sizeof(double) * m * nu);
  hepem_step_counters* dcnt = reinterpret_cast<hepem_step_counters*>(p);
  p += al(sizeof(hepem_step_counters));
  void* dstate[20];
  void* dout[14] = {};
  for (int k = 0; k < 20; ++k) { dstate[k] = p; p += al(kStateSizes[k] * m); }
  if (phase == hepem::kPhasePerform)
    for (int k = 0; k < 14; ++k) { dout[k] = p; p += al(kOutSizes[k] * m); }
  void* const* hin = reinterpret_cast<void* const*>(in);
  for (int k = 0; k < 20; ++k)
    HEPEM_CUDA(cudaMemcpyAsync(dstate[k], hin[k], kStateSizes[k] * m, cudaMemcpyHostToDevice, s));
  if (nu > 0) HEPEM_CUDA(cudaMemcpyAsync(du, uniforms, sizeof(double) * m * nu, cudaMemcpyHostToDevice, s));
  if (counters) HEPEM_CUDA(cudaMemsetAsync(dcnt, 0, sizeof(*dcnt), s));
  hepem_track_state ds;
  hepem_step_out dr;
  memcpy(&ds, dstate, sizeof(ds));
  memcpy(&dr, dout, sizeof(dr));
  if (phase == hepem::kPhasePerform) {
    HEPEM_CUDA(cudaMemcpyAsync(dg, gstep, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    HEPEM_CUDA(cudaMemcpyAsync(dlim, limits, limBytes, cudaMemcpyHostToDevice, s));
  }
  const int rc = split_device(c, form, phase, n, &ds, phase == hepem::kPhasePerform ? &ds : nullptr, dg, dlim,
                              nu > 0 ? du : nullptr, nu, seed, phase == hepem::kPhasePerform ? &dr : nullptr,
                              counters ? dcnt : nullptr, s);
  if (rc != HEPEM_OK) return rc;
  if (phase == hepem::kPhaseHowFar) {
    HEPEM_CUDA(cudaMemcpyAsync(gstep, dg, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
    HEPEM_CUDA(cudaMemcpyAsync(limits, dlim, limBytes, cudaMemcpyDeviceToHost, s));
  } else {
    void* const* hout = reinterpret_cast<void* const*>(out);
    void* const* hres = reinterpret_cast<void* const*>(res);
    for (int k = 0; k < 20; ++k)
      HEPEM_CUDA(cudaMemcpyAsync(hout[k], dstate[k], kStateSizes[k] * m, cudaMemcpyDeviceToHost, s));
    for (int k = 0; k < 14; ++k)
      HEPEM_CUDA(cudaMemcpyAsync(hres[k], dout[k], kOutSizes[k] * m, cudaMemcpyDeviceToHost, s));
  }
  if (counters) HEPEM_CUDA(cudaMemcpyAsync(counters, dcnt, sizeof(*counters), cudaMemcpyDeviceToHost, s));
  HEPEM_CUDA(cudaStreamSynchronize(s));
  return HEPEM_OK;
}
}  // namespace

int hepem_howfar(const hepem_ctx* c, int form, int64_t n, const hepem_track_state* tracks, const double* uniforms,
                 int32_t nu, uint64_t seed, double* gstep, void* limits, hepem_step_counters* counters,
                 void* stream) {
  const int rc = split_check(c, form, n, nu, tracks, nullptr, gstep, limits, uniforms, nullptr, false);
  if (rc != HEPEM_OK || n == 0) return rc;
  hepem::TraceRange trace("hepem_howfar", n);
  return split_device(c, form, hepem::kPhaseHowFar, n, tracks, nullptr, gstep, limits, uniforms, nu, seed, nullptr,
                      counters, (cudaStream_t)stream);
}

int hepem_perform(const hepem_ctx* c, int form, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                  const double* gstep, const void* limits, const double* uniforms, int32_t nu, uint64_t seed,
                  hepem_step_out* res, hepem_step_counters* counters, void* stream) {
  const int rc = split_check(c, form, n, nu, in, out, gstep, limits, uniforms, res, true);
  if (rc != HEPEM_OK || n == 0) return rc;
  hepem::TraceRange trace("hepem_perform", n);
  return split_device(c, form, hepem::kPhasePerform, n, in, out, const_cast<double*>(gstep),
                      const_cast<void*>(limits), uniforms, nu, seed, res, counters, (cudaStream_t)stream);
}

int hepem_howfar_host(const hepem_ctx* c, int form, int64_t n, const hepem_track_state* tracks,
                      const double* uniforms, int32_t nu, uint64_t seed, double* gstep, void* limits,
                      hepem_step_counters* counters, void* stream) {
  const int rc = split_check(c, form, n, nu, tracks, nullptr, gstep, limits, uniforms, nullptr, false);
  if (rc != HEPEM_OK || n == 0) return rc;
  hepem::TraceRange trace("hepem_howfar_host", n);
  return split_host(c, form, hepem::kPhaseHowFar, n, tracks, nullptr, gstep, limits, uniforms, nu, seed, nullptr,
                    counters, (cudaStream_t)stream);
}

int hepem_perform_host(const hepem_ctx* c, int form, int64_t n, const hepem_track_state* in,
                       hepem_track_state* out, const double* gstep, const void* limits, const double* uniforms,
                       int32_t nu, uint64_t seed, hepem_step_out* res, hepem_step_counters* counters,
                       void* stream) {
  const int rc = split_check(c, form, n, nu, in, out, gstep, limits, uniforms, res, true);
  if (rc != HEPEM_OK || n == 0) return rc;
  hepem::TraceRange trace("hepem_perform_host", n);
  return split_host(c, form, hepem::kPhasePerform, n, in, out, const_cast<double*>(gstep),
                    const_cast<void*>(limits), uniforms, nu, seed, res, counters, (cudaStream_t)stream);
}

int hepem_profile_stages(hepem_ctx* c, int enable) {
  if (!c) return fail(HEPEM_BAD_ARG, "null context");
  if (enable && !c->stageEvReady) {
    for (int k = 0; k < hepem::kNumStageEvents; ++k) HEPEM_CUDA(cudaEventCreate(&c->stageEv[k]));
    c->stageEvReady = true;
  }
  c->profile = enable != 0;
  return HEPEM_OK;
}

int hepem_stage_times(hepem_ctx* c, float* ms, const char** names, int32_t max, int32_t* count) {
  if (!c || !ms || max < 0) return fail(HEPEM_BAD_ARG, "bad argument");
  if (!c->stageEvReady) return fail(HEPEM_BAD_ARG, "stage profiling was never enabled");
  const int ns = hepem::kNumStageEvents - 1;
  HEPEM_CUDA(cudaEventSynchronize(c->stageEv[ns]));
  const int k = max < ns ? max : ns;
  for (int i = 0; i < k; ++i) {
    HEPEM_CUDA(cudaEventElapsedTime(&ms[i], c->stageEv[i], c->stageEv[i + 1]));
    if (names) names[i] = hepem::stage_name(i);
  }
  if (count) *count = k;
  return HEPEM_OK;
}

double hepem_philox_uniform(uint64_t seed, int32_t id, int32_t k) { return hepem::philox_uniform(seed, id, k); }

int hepem_fill_uniforms(int64_t n, const int32_t* id, int32_t nu, uint64_t seed, double* u, void* stream) {
  if (n < 0 || nu < 0 || (n > 0 && nu > 0 && (!id || !u))) return fail(HEPEM_BAD_ARG, "bad argument");
  int dev = 0, sms = 0;
  HEPEM_CUDA(cudaGetDevice(&dev));
  HEPEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  HEPEM_CUDA(hepem::launch_fill_uniforms(n, id, nu, seed, u, (cudaStream_t)stream, sms));
  return HEPEM_OK;
}

}  // extern "C"
