// gpu_euler.hpp — reference-side plug-in for libcilgpu.so (header-only C++).
//
// The reference selects its integrator through a function pointer,
//   typedef void(*MDIntegrator)(int& ts); extern MDIntegrator mdStep;   (MD.cuh:450-452)
// and calls it GTS times per frame (CIL.cu:1106); between frames only checkPositions and
// outputFrame read the colony arrays. GpuEuler keeps the colony on the GPU, performs one
// Euler step per call through cil_step(), and copies the colony back into the reference's
// CellColony arrays every `steps_per_frame` calls, so the host sees current arrays exactly
// where it reads them. `gpuEuler` is a free function with the MDIntegrator signature that
// dispatches to the bound plug-in.
//
// GpuGsdOutput replaces the reference's GSD output of that colony (initGSDOutput,
// outputGSDFrame and gsd_close, OutputWriter.cpp:619-644 and 726-735) with the device-fed
// frame writer of cil_gsd.h: a frame is packed on the GPU and written by a host thread while
// the next mdStep calls run.
//
// Errors follow the reference's run_assert (Utils.hpp:99-109): any status other than
// CIL_OK throws std::runtime_error carrying cil_last_error().
#pragma once

#include <functional>
#include <stdexcept>
#include <string>

#include "cil_gpu.h"
#include "cil_gsd.h"

namespace cilgpu {

// Views into one species of the reference's CellColony (Colony.hpp:88-123): pos/vel
// [cell][2][dim], sigmaCore [cell][2], cellT0 / cellTSwitch [cell].
struct SpeciesArrays {
  int ncells = 0;
  int capacity = 0;
  double *pos = nullptr;
  double *sigma = nullptr;
  double *vel = nullptr;
  int *t0 = nullptr;
  int *tswitch = nullptr;
};

class GpuEuler {
 public:
  // grow(need) must make room for `need` cells (the reference's reserveNumCells,
  // Colony.cpp:193-273) and return the new views.
  GpuEuler(const cil_config &cfg, const cil_colony_params &params, int device_capacity,
           SpeciesArrays host, int steps_per_frame,
           std::function<SpeciesArrays(int)> grow = nullptr)
      : host_(host), steps_per_frame_(steps_per_frame > 0 ? steps_per_frame : 1), grow_(grow) {
    int32_t cap = device_capacity;
    check(cil_create(&cfg, &params, &cap, &h_), "cil_create");
  }
  ~GpuEuler() { cil_destroy(h_); }
  GpuEuler(const GpuEuler &) = delete;
  GpuEuler &operator=(const GpuEuler &) = delete;

  // One Euler step (Euler, CIL.cu:1013-1020) with the MDIntegrator calling convention.
  void operator()(int &ts) {
    if (!uploaded_) upload(ts);
    int64_t t = 0;
    check(cil_step(h_, 1, &t), "cil_step");
    ts = static_cast<int>(t);
    if (++calls_ % steps_per_frame_ == 0) sync_to_host();
  }

  // Copies the colony to the host arrays now (frame boundary).
  void sync_to_host() {
    cil_colony_view v = view();
    cil_status s = cil_download(h_, 0, &v);
    if (s == CIL_ERR_CAPACITY && grow_) {
      host_ = grow_(v.ncells);
      v = view();
      s = cil_download(h_, 0, &v);
    }
    check(s, "cil_download");
    host_.ncells = v.ncells;
  }

  // Forces of the current state (calculForcesPressure), [cell][2][dim].
  void forces(double *frc) { check(cil_forces(h_, 0, frc), "cil_forces"); }

  const SpeciesArrays &host() const { return host_; }
  cil_handle *handle() { return h_; }
  // Uploads the host colony if no step has run yet (frame output before the first step).
  void ensure_uploaded(int ts = 0) {
    if (!uploaded_) upload(ts);
  }

 private:
  cil_colony_view view() const {
    cil_colony_view v{};
    v.ncells = host_.ncells;
    v.capacity = host_.capacity;
    v.pos = host_.pos;
    v.sigma = host_.sigma;
    v.vel = host_.vel;
    v.t0 = host_.t0;
    v.tswitch = host_.tswitch;
    return v;
  }
  void upload(int ts) {
    cil_colony_view v = view();
    v.ts = ts;
    check(cil_upload(h_, 0, &v), "cil_upload");
    uploaded_ = true;
  }
  void check(cil_status s, const char *what) {
    if (s == CIL_OK) return;
    char buf[512];
    cil_last_error(h_, buf, sizeof buf);
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(static_cast<int>(s)) +
                             "): " + buf);
  }

  cil_handle *h_ = nullptr;
  SpeciesArrays host_;
  int steps_per_frame_;
  std::function<SpeciesArrays(int)> grow_;
  bool uploaded_ = false;
  long long calls_ = 0;
};

// GSD frames of the plug-in's colony. frame(ts) is outputGSDFrame(fp, id, ts): the caller
// passes the step label (the final-state file passes 0). Destruction flushes and closes.
class GpuGsdOutput {
 public:
  GpuGsdOutput(GpuEuler &g, const std::string &path, const cil_frame_options *opt = nullptr) : g_(g) {
    g_.ensure_uploaded();
    const cil_status s = cil_frame_open(g_.handle(), 0, path.c_str(), opt, &w_);
    if (s != CIL_OK) {
      char buf[512];
      cil_last_error(g_.handle(), buf, sizeof buf);
      throw std::runtime_error("cil_frame_open(" + path + ") failed (" + std::to_string(static_cast<int>(s)) +
                               "): " + buf);
    }
  }
  ~GpuGsdOutput() { cil_frame_close(w_); }
  GpuGsdOutput(const GpuGsdOutput &) = delete;
  GpuGsdOutput &operator=(const GpuGsdOutput &) = delete;

  void frame(int ts) { check(cil_frame_write(w_, ts, nullptr), "cil_frame_write"); }
  void flush() { check(cil_frame_flush(w_), "cil_frame_flush"); }
  cil_frame_stats stats() const {
    cil_frame_stats s{};
    cil_frame_get_stats(w_, &s);
    return s;
  }

 private:
  void check(cil_status s, const char *what) {
    if (s == CIL_OK) return;
    char buf[512];
    cil_frame_last_error(w_, buf, sizeof buf);
    if (!buf[0]) cil_last_error(g_.handle(), buf, sizeof buf);
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(static_cast<int>(s)) + "): " + buf);
  }
  GpuEuler &g_;
  cil_frame_writer *w_ = nullptr;
};

// The MDIntegrator-compatible entry point (assign `mdStep = cilgpu::gpuEuler;`).
inline GpuEuler *&bound_plugin() {
  static GpuEuler *p = nullptr;
  return p;
}
inline void bindGpuEuler(GpuEuler *p) { bound_plugin() = p; }
inline void gpuEuler(int &ts) {
  GpuEuler *p = bound_plugin();
  if (!p) throw std::runtime_error("gpuEuler: no GpuEuler bound");
  (*p)(ts);
}

}  // namespace cilgpu
