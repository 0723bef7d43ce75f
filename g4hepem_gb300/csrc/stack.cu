// stack.cu -- secondary stacking with production cuts on the device.
//
// The reference stacks the secondaries of a step into Geant4 tracks in
// G4HepEmTrackingManager::StackSecondaries (G4HepEm/G4HepEm/src/
// G4HepEmTrackingManager.cc:1254-1330): with "apply cuts" an e- below the
// electron production cut, an e+ below the positron cut (when m_e c^2 is
// below the gamma cut) and a gamma below the gamma cut are not stacked; their
// energy (for the e+: E + 2 m_e c^2) is deposited instead.  Here the stacked
// secondaries become fresh tracks of the SoA batch format, in parent order
// (parent i, slot 0 then slot 1), so the next step can take them directly.
// Two passes give the order without atomics: a per-block count, a scan of the
// block counts, and a write pass with a block-local scan.
#include <cuda_runtime.h>

#include <cstdint>

#include "ctx.h"
#include "g4hepem_gb300.h"
#include "tables.h"
#include "trace.h"

namespace {

constexpr int kBlock = 256;
constexpr double kMec2 = 5.1099890999999997e-01;

struct StackArgs {
  int64_t n;
  hepem_track_state par;
  hepem_step_out res;
  int applyCuts;
  int32_t idBase;
  hepem_track_state out;
  int64_t capacity;
  double* edepCut;
};

// survivors of parent i: bit k set if secondary slot k is stacked; the
// deposit of the cut secondaries in *dep
__device__ __forceinline__ unsigned survivors(const hepem::DevTables& T, const StackArgs& a, int64_t i,
                                              double* dep) {
  const int ns = a.res.n_sec[i];
  const int imc = a.par.imc[i];
  const bool okImc = imc >= 0 && imc < T.nCouples;
  unsigned m = 0;
  double d = 0.0;
  for (int k = 0; k < 2 && k < ns; ++k) {
    const int type = a.res.sec_type[2 * i + k];
    const double e = a.res.sec_ekin[2 * i + k];
    bool keep = true;
    if (a.applyCuts && okImc) {
      const hepem::DevCouple& c = T.couples[imc];
      if (type == 0 && e < c.elCut) {
        keep = false;
        d += e;
      } else if (type == 1 && kMec2 < c.gamCut && e < c.posCut) {
        keep = false;
        d += e + 2.0 * kMec2;
      } else if (type == 2 && e < c.gamCut) {
        keep = false;
        d += e;
      }
    }
    if (keep) m |= 1u << k;
  }
  *dep = d;
  return m;
}

__global__ void __launch_bounds__(kBlock) count_kernel(const __grid_constant__ hepem::DevTables T, const StackArgs a,
                                                       uint32_t* __restrict__ blockCount) {
  __shared__ uint32_t s[kBlock / 32];
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  uint32_t c = 0;
  if (i < a.n) {
    double dep;
    const unsigned m = survivors(T, a, i, &dep);
    c = __popc(m);
    if (a.edepCut) a.edepCut[i] = dep;
  }
  c = __reduce_add_sync(0xFFFFFFFFu, c);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kBlock / 32; ++w) t += s[w];
    blockCount[blockIdx.x] = t;
  }
}

// exclusive scan of nb block counts in one block; total to *total
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t* __restrict__ v, int64_t nb,
                                                    unsigned long long* __restrict__ total) {
  __shared__ unsigned long long part[1024];
  const int64_t per = (nb + 1023) / 1024;
  const int64_t b = threadIdx.x * per;
  unsigned long long s = 0;
  for (int64_t k = b; k < b + per && k < nb; ++k) s += v[k];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const unsigned long long x = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0ull;
    __syncthreads();
    part[threadIdx.x] += x;
    __syncthreads();
  }
  unsigned long long run = part[threadIdx.x] - s;
  for (int64_t k = b; k < b + per && k < nb; ++k) {
    const uint32_t c = v[k];
    v[k] = (uint32_t)run;  // block offsets fit 32 bits: at most 2 per track of an int32-indexed batch
    run += c;
  }
  if (threadIdx.x == 1023) *total = part[1023];
}

__device__ __forceinline__ void write_track(const StackArgs& a, int64_t i, int k, int64_t pos) {
  if (pos >= a.capacity) return;
  const hepem_track_state& o = a.out;
  o.type[pos] = a.res.sec_type[2 * i + k];
  o.imc[pos] = a.par.imc[i];
  o.id[pos] = (int32_t)(a.idBase + pos);
  o.ekin[pos] = a.res.sec_ekin[2 * i + k];
  o.dir_x[pos] = a.res.sec_dir_x[2 * i + k];
  o.dir_y[pos] = a.res.sec_dir_y[2 * i + k];
  o.dir_z[pos] = a.res.sec_dir_z[2 * i + k];
  o.nia0[pos] = -1.0;
  o.nia1[pos] = -1.0;
  o.nia2[pos] = -1.0;
  o.nia3[pos] = -1.0;
  o.safety[pos] = a.par.safety[i];
  o.on_boundary[pos] = 0;
  o.msc_init_range[pos] = 1.0e21;
  o.msc_dyn_factor[pos] = 0.04;
  o.msc_tlimit_min[pos] = 1.0e-7;
  o.msc_first_step[pos] = 1;
  o.gauss_valid[pos] = 0;
  o.gauss_value[pos] = 0.0;
  o.rng_cursor[pos] = 0;
}

__global__ void __launch_bounds__(kBlock) write_kernel(const __grid_constant__ hepem::DevTables T, const StackArgs a,
                                                       const uint32_t* __restrict__ blockOffset) {
  __shared__ uint32_t warpSum[kBlock / 32];
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  unsigned m = 0;
  if (i < a.n) {
    double dep;
    m = survivors(T, a, i, &dep);
  }
  const uint32_t c = __popc(m);
  // block-local exclusive scan: warp scan, then scan of the warp sums
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = c;
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) warpSum[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t r = 0;
    for (int w = 0; w < kBlock / 32; ++w) {
      const uint32_t t = warpSum[w];
      warpSum[w] = r;
      r += t;
    }
  }
  __syncthreads();
  const int64_t base = (int64_t)blockOffset[blockIdx.x] + warpSum[warp] + (incl - c);
  if (i < a.n) {
    int64_t pos = base;
    for (int k = 0; k < 2; ++k)
      if (m & (1u << k)) write_track(a, i, k, pos++);
  }
}

bool state_complete(const hepem_track_state* s) { return hepem::valid_state(s); }

}  // namespace

extern "C" int hepem_stack_secondaries(const hepem_ctx* c, int64_t n, const hepem_track_state* parents,
                                       const hepem_step_out* res, int apply_cuts, int32_t id_base,
                                       hepem_track_state* out, int64_t capacity, int64_t* n_out,
                                       double* edep_cut, void* stream) {
  if (!c || n < 0 || capacity < 0 || !parents || !res || !out || !n_out)
    return hepem::set_error(HEPEM_BAD_ARG, "null argument or negative size");
  if (!res->n_sec || !res->sec_type || !res->sec_ekin || !res->sec_dir_x || !res->sec_dir_y || !res->sec_dir_z ||
      !parents->imc || !parents->safety || !state_complete(out))
    return hepem::set_error(HEPEM_BAD_ARG, "null array in track batch");
  if (n > (int64_t)INT32_MAX) return hepem::set_error(HEPEM_BAD_ARG, "batch too large");
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    const cudaError_t e = cudaMemsetAsync(n_out, 0, sizeof(int64_t), s);
    return e == cudaSuccess ? HEPEM_OK : hepem::set_error(HEPEM_CUDA_ERROR, cudaGetErrorString(e));
  }
  hepem::TraceRange trace("hepem_stack_secondaries", n);
  StackArgs a;
  a.n = n;
  a.par = *parents;
  a.res = *res;
  a.applyCuts = apply_cuts;
  a.idBase = id_base;
  a.out = *out;
  a.capacity = capacity;
  a.edepCut = edep_cut;
  const int64_t nb = (n + kBlock - 1) / kBlock;
  uint32_t* counts = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&counts, sizeof(uint32_t) * nb, s);
  if (e == cudaSuccess) {
    count_kernel<<<(unsigned)nb, kBlock, 0, s>>>(c->tables, a, counts);
    scan_kernel<<<1, 1024, 0, s>>>(counts, nb, reinterpret_cast<unsigned long long*>(n_out));
    write_kernel<<<(unsigned)nb, kBlock, 0, s>>>(c->tables, a, counts);
    e = cudaGetLastError();
    const cudaError_t f = cudaFreeAsync(counts, s);
    if (e == cudaSuccess) e = f;
  }
  return e == cudaSuccess ? HEPEM_OK : hepem::set_error(HEPEM_CUDA_ERROR, cudaGetErrorString(e));
}
