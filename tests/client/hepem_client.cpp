// hepem_client.cpp -- a C++ client of the library, written as a G4HepEm
// client would be, through include/g4hepem_gb300.hh (compiled and run by
// tests/test_client_cpu.py and tests/test_gpu_client.py).
//
//   hepem_client info <table.json>
//       what needs no GPU: status strings, the binary table image of the
//       document, its round trip check, the step-limit record size; then
//       the tables on the device, or "no-device" when there is none.
//   hepem_client step <table.json> <dir> <form> <seed>
//       reads a track batch from <dir>/in_<field>.bin (raw arrays of the
//       hepem_track_state fields) and a transport from gfrac.bin,
//       ndir_{x,y,z}.bin, post_bnd.bin; runs HowFar, the transport (step
//       gfrac * proposed, direction, post-step boundary status) and Perform,
//       with 64 uniforms per track of the Philox stream of `seed`; writes
//       proposed.bin, out_<field>.bin and res_<field>.bin.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "g4hepem_gb300.hh"

namespace {

namespace G = g4hepem_gb300;

struct Field {
  const char* name;
  size_t size;  // bytes per track
};
// the order of hepem_track_state / hepem_step_out
const Field kState[20] = {{"type", 1}, {"imc", 4}, {"id", 4}, {"ekin", 8}, {"dir_x", 8}, {"dir_y", 8}, {"dir_z", 8},
                          {"nia0", 8}, {"nia1", 8}, {"nia2", 8}, {"nia3", 8}, {"safety", 8}, {"on_boundary", 1},
                          {"msc_init_range", 8}, {"msc_dyn_factor", 8}, {"msc_tlimit_min", 8},
                          {"msc_first_step", 1}, {"gauss_valid", 1}, {"gauss_value", 8}, {"rng_cursor", 4}};
const Field kOut[14] = {{"edep", 8}, {"gstep", 8}, {"pstep", 8}, {"winner", 1}, {"disp_x", 8}, {"disp_y", 8},
                        {"disp_z", 8}, {"flags", 1}, {"n_sec", 1}, {"sec_type", 2}, {"sec_ekin", 16},
                        {"sec_dir_x", 16}, {"sec_dir_y", 16}, {"sec_dir_z", 16}};

std::vector<char> read_all(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw G::Error(HEPEM_BAD_ARG, "cannot open " + path);
  std::vector<char> b;
  char buf[1 << 16];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) b.insert(b.end(), buf, buf + k);
  std::fclose(f);
  return b;
}

void write_all(const std::string& path, const void* p, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(p, 1, bytes, f) != bytes) throw G::Error(HEPEM_BAD_ARG, "cannot write " + path);
  std::fclose(f);
}

void cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw G::Error(HEPEM_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

// device copy of a host array (freed by the caller)
void* to_device(const void* p, size_t bytes) {
  void* d = nullptr;
  cuda(cudaMalloc(&d, bytes > 0 ? bytes : 1), "cudaMalloc");
  cuda(cudaMemcpy(d, p, bytes, cudaMemcpyHostToDevice), "cudaMemcpy");
  return d;
}

int info(const std::string& table) {
  const std::string json = G::Data::ReadFile(table);
  const std::vector<uint8_t> img = G::Data::ImageFromJson(json);
  int64_t arena = 0;
  G::check(hepem_image_check(img.data(), img.size(), &arena), "hepem_image_check");
  std::vector<uint8_t> bad = img;
  bad[bad.size() / 2] ^= 0x5A;
  const int badStatus = hepem_image_check(bad.data(), bad.size(), nullptr);
  std::printf("image_bytes %zu arena_bytes %lld damaged_image_status %d (%s)\n", img.size(), (long long)arena,
              badStatus, hepem_status_string(badStatus));
  std::printf("limit_bytes_1000 %lld\n", (long long)G::StepLimits::Bytes(1000));
  for (int s = HEPEM_OK; s <= HEPEM_CANCELLED; ++s) std::printf("status %d %s\n", s, hepem_status_string(s));
  try {
    G::Data d = G::Data::FromImage(img);
    G::Data j = G::Data::FromJson(json);
    std::printf("device couples %d %d\n", d.NumCouples(), j.NumCouples());
  } catch (const G::Error& e) {
    if (e.status() != HEPEM_NO_DEVICE && e.status() != HEPEM_CUDA_ERROR) throw;
    std::printf("no-device %d\n", e.status());
  }
  return 0;
}

int step(const std::string& table, const std::string& dir, const std::string& form, uint64_t seed) {
  const G::Form f = form == "plain" ? G::Form::Plain : form == "mixed" ? G::Form::Mixed : G::Form::Batched;
  G::Data data = G::Data::FromJsonFile(table);
  const int64_t n = (int64_t)(read_all(dir + "/in_ekin.bin").size() / 8);
  void* dstate[20];
  for (int k = 0; k < 20; ++k) {
    const std::vector<char> h = read_all(dir + "/in_" + kState[k].name + ".bin");
    if ((int64_t)h.size() != n * (int64_t)kState[k].size) throw G::Error(HEPEM_BAD_ARG, "bad size of in_" +
                                                                            std::string(kState[k].name));
    dstate[k] = to_device(h.data(), h.size());
  }
  G::Batch b;
  b.n = n;
  std::memcpy(&b.state, dstate, sizeof(b.state));
  const int32_t nu = 64;
  double* du = nullptr;
  cuda(cudaMalloc(&du, sizeof(double) * (size_t)n * nu + 8), "cudaMalloc");
  G::check(hepem_fill_uniforms(n, b.state.id, nu, seed, du, nullptr), "hepem_fill_uniforms");
  b.uniforms = du;
  b.n_uniform = nu;
  b.seed = seed;
  // HowFar
  G::StepLimits lim;
  cuda(cudaMalloc(reinterpret_cast<void**>(&lim.gstep), sizeof(double) * (size_t)n + 8), "cudaMalloc");
  cuda(cudaMalloc(&lim.limits, (size_t)G::StepLimits::Bytes(n) + 8), "cudaMalloc");
  G::ElectronManager::HowFar(data, b, lim, f);
  // the transport: the step it makes, the direction and the boundary status it leaves
  std::vector<double> g((size_t)n);
  cuda(cudaMemcpy(g.data(), lim.gstep, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost), "cudaMemcpy");
  write_all(dir + "/proposed.bin", g.data(), sizeof(double) * (size_t)n);
  const std::vector<char> fr = read_all(dir + "/gfrac.bin");
  const double* frac = reinterpret_cast<const double*>(fr.data());
  for (int64_t i = 0; i < n; ++i) g[i] = frac[i] * g[i];
  cuda(cudaMemcpy(lim.gstep, g.data(), sizeof(double) * (size_t)n, cudaMemcpyHostToDevice), "cudaMemcpy");
  const char* nd[3] = {"ndir_x", "ndir_y", "ndir_z"};
  for (int c = 0; c < 3; ++c) {
    const std::vector<char> h = read_all(dir + "/" + nd[c] + ".bin");
    cuda(cudaMemcpy(dstate[4 + c], h.data(), h.size(), cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  const std::vector<char> post = read_all(dir + "/post_bnd.bin");
  cuda(cudaMemcpy(dstate[12], post.data(), post.size(), cudaMemcpyHostToDevice), "cudaMemcpy");
  // Perform
  void* dout[14];
  for (int k = 0; k < 14; ++k) {
    cuda(cudaMalloc(&dout[k], kOut[k].size * (size_t)n + 8), "cudaMalloc");
    cuda(cudaMemset(dout[k], 0, kOut[k].size * (size_t)n + 8), "cudaMemset");
  }
  hepem_step_out res;
  std::memcpy(&res, dout, sizeof(res));
  G::GammaManager::Perform(data, b, lim, res, f);
  cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  std::vector<char> h;
  for (int k = 0; k < 20; ++k) {
    h.resize(kState[k].size * (size_t)n);
    cuda(cudaMemcpy(h.data(), dstate[k], h.size(), cudaMemcpyDeviceToHost), "cudaMemcpy");
    write_all(dir + "/out_" + kState[k].name + ".bin", h.data(), h.size());
    cudaFree(dstate[k]);
  }
  for (int k = 0; k < 14; ++k) {
    h.resize(kOut[k].size * (size_t)n);
    cuda(cudaMemcpy(h.data(), dout[k], h.size(), cudaMemcpyDeviceToHost), "cudaMemcpy");
    write_all(dir + "/res_" + kOut[k].name + ".bin", h.data(), h.size());
    cudaFree(dout[k]);
  }
  cudaFree(du);
  cudaFree(lim.gstep);
  cudaFree(lim.limits);
  std::printf("stepped %lld tracks\n", (long long)n);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    if (argc >= 3 && std::string(argv[1]) == "info") return info(argv[2]);
    if (argc >= 6 && std::string(argv[1]) == "step") return step(argv[2], argv[3], argv[4], std::strtoull(argv[5], nullptr, 10));
    std::fprintf(stderr, "usage: hepem_client info <table.json> | step <table.json> <dir> <form> <seed>\n");
    return 2;
  } catch (const G::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.status(), e.what());
    return 1;
  }
}
