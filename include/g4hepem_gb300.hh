/*
 * g4hepem_gb300.hh -- header-only C++ front end of the C-ABI (g4hepem_gb300.h)
 * with the names of the reference's interface, so that a client written
 * against G4HepEm reads the same over batches:
 *
 *   reference (one track, thread-local data)          here (a batch in device memory)
 *   G4HepEmStateFromJson(std::istream&)               Data::FromJsonFile / FromJson / FromImage
 *     (G4HepEmDataJsonIO.hh:84)
 *   G4HepEmElectronManager::HowFar / Perform          ElectronManager::HowFar / Perform
 *     (G4HepEmElectronManager.hh:71,222)
 *   G4HepEmGammaManager::HowFar / SelectInteraction   GammaManager::HowFar / Perform
 *     + Perform (G4HepEmGammaManager.hh:32,39,51)       (Perform selects the interaction first,
 *                                                        as the client calls the two back to back,
 *                                                        apps/examples/TestEm3/src/G4HepEmProcess.cc:187-188)
 *   G4HepEmTLData (primary track between HowFar       StepLimits (the proposed geometrical steps
 *     and Perform, G4HepEmTLData.hh:36-92)              and the step-limit record)
 *
 * A batch may hold e-, e+ and gammas: every track is handled by the physics
 * of its own type, whichever manager's function is called (ElectronManager
 * and GammaManager name the same batch calls).  Errors throw g4hepem_gb300::Error
 * (the reference exit()s on CUDA errors, G4HepEmCuUtils.hh:19-26).
 */
#ifndef G4HEPEM_GB300_HH
#define G4HEPEM_GB300_HH

#include <cstdint>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "g4hepem_gb300.h"

namespace g4hepem_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* where) {
  if (status != HEPEM_OK)
    throw Error(status, std::string(where) + ": " + hepem_status_string(status) + ": " + hepem_last_error());
}

// The tables (G4HepEmData + G4HepEmParameters of a G4HepEmState) on the
// current CUDA device; move-only, released with the object
// (FreeG4HepEmData, G4HepEmData.hh:80).
class Data {
 public:
  static Data FromJson(const std::string& text) {
    hepem_ctx* c = nullptr;
    check(hepem_create(text.data(), text.size(), &c), "hepem_create");
    return Data(c);
  }
  static Data FromJsonFile(const std::string& path) {
    hepem_ctx* c = nullptr;
    check(hepem_create_from_file(path.c_str(), &c), "hepem_create_from_file");
    return Data(c);
  }
  static Data FromImage(const std::vector<uint8_t>& image) {
    hepem_ctx* c = nullptr;
    check(hepem_create_from_image(image.data(), image.size(), &c), "hepem_create_from_image");
    return Data(c);
  }
  // the binary image of the tables of a JSON document (needs no GPU)
  static std::vector<uint8_t> ImageFromJson(const std::string& text) {
    size_t size = 0;
    check(hepem_image_from_json(text.data(), text.size(), nullptr, 0, &size), "hepem_image_from_json");
    std::vector<uint8_t> img(size);
    check(hepem_image_from_json(text.data(), text.size(), img.data(), img.size(), &size), "hepem_image_from_json");
    return img;
  }
  static std::string ReadFile(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw Error(HEPEM_BAD_ARG, "cannot read " + path);
    std::ostringstream s;
    s << in.rdbuf();
    return s.str();
  }

  Data(Data&& o) noexcept : c_(o.c_) { o.c_ = nullptr; }
  Data& operator=(Data&& o) noexcept {
    std::swap(c_, o.c_);
    return *this;
  }
  Data(const Data&) = delete;
  Data& operator=(const Data&) = delete;
  ~Data() {
    if (c_) hepem_destroy(c_);
  }
  const hepem_ctx* get() const { return c_; }
  hepem_ctx* get() { return c_; }
  int32_t NumCouples() const {
    int32_t nc = 0;
    check(hepem_info(c_, &nc, nullptr, nullptr, nullptr), "hepem_info");
    return nc;
  }

 private:
  explicit Data(hepem_ctx* c) : c_(c) {}
  hepem_ctx* c_;
};

enum class Form { Plain = HEPEM_FORM_PLAIN, Batched = HEPEM_FORM_BATCHED, Mixed = HEPEM_FORM_MIXED };

// A batch of n tracks (SoA device arrays, caller-owned) with its uniform
// streams (replaces the RNG of G4HepEmTLData) and the stream it runs on.
struct Batch {
  int64_t n = 0;
  hepem_track_state state{};
  const double* uniforms = nullptr;
  int32_t n_uniform = 0;
  uint64_t seed = 0;
  void* stream = nullptr;
};

// What HowFar leaves for Perform: gstep (device, n doubles: the proposed
// geometrical step; transport lowers it to the step made) and the step-limit
// record (device, Bytes(n) bytes).  Caller-owned.
struct StepLimits {
  double* gstep = nullptr;
  void* limits = nullptr;
  static int64_t Bytes(int64_t n) { return hepem_step_limit_bytes(n); }
};

struct Manager {
  // G4HepEm{Electron,Gamma}Manager::HowFar over the batch
  static void HowFar(const Data& d, const Batch& b, StepLimits& lim, Form form = Form::Batched,
                     hepem_step_counters* counters = nullptr) {
    check(hepem_howfar(d.get(), static_cast<int>(form), b.n, &b.state, b.uniforms, b.n_uniform, b.seed, lim.gstep,
                       lim.limits, counters, b.stream),
          "hepem_howfar");
  }
  // ::Perform (gammas: ::SelectInteraction first, or on a boundary only the
  // interaction-length update), in place: the batch state carries the
  // direction and boundary status transport left, and receives the
  // post-step state
  static void Perform(const Data& d, Batch& b, const StepLimits& lim, hepem_step_out& res,
                      Form form = Form::Batched, hepem_step_counters* counters = nullptr) {
    check(hepem_perform(d.get(), static_cast<int>(form), b.n, &b.state, &b.state, lim.gstep, lim.limits, b.uniforms,
                        b.n_uniform, b.seed, &res, counters, b.stream),
          "hepem_perform");
  }
  // HowFar and Perform with no geometry between them (hepem_step*)
  static void Step(const Data& d, Batch& b, hepem_step_out& res, Form form = Form::Batched,
                   hepem_step_counters* counters = nullptr) {
    int rc = HEPEM_OK;
    switch (form) {
      case Form::Plain:
        rc = hepem_step(d.get(), b.n, &b.state, &b.state, b.uniforms, b.n_uniform, b.seed, &res, counters, b.stream);
        break;
      case Form::Batched:
        rc = hepem_step_batched(d.get(), b.n, &b.state, &b.state, b.uniforms, b.n_uniform, b.seed, &res, counters,
                                b.stream);
        break;
      case Form::Mixed:
        rc = hepem_step_mixed(d.get(), b.n, &b.state, &b.state, b.uniforms, b.n_uniform, b.seed, &res, counters,
                              b.stream);
        break;
    }
    check(rc, "hepem_step");
  }
};

using ElectronManager = Manager;
using GammaManager = Manager;

}  // namespace g4hepem_gb300

#endif  // G4HEPEM_GB300_HH
