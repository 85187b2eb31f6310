// cil_gpu_run: the reference's main loop (CIL.cu:1072-1127) on the GPU step, driven by the
// reference's JSON run description.
//
//   cil_gpu_run input.json
//
// Reads the run with cil_input (include/cil_input.h), builds INIT on the host, uploads it,
// writes frame 0, then FRAMES times: GTS steps (one cil_step call), a progress line in the
// reference's format, a GSD frame when OUTPUT.FORMAT lists GSD (device-fed writer,
// include/cil_gsd.h). At the end the final state goes to <DIR>/Last/<NAME>.Last.gsd as one
// frame labelled step 0 (finalizeOutput, OutputWriter.cpp:724-745). Failures print the
// library's message and exit 1, as run_assert does (Utils.hpp:99-109).
#include <sys/stat.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "cil_gpu.h"
#include "cil_gsd.h"
#include "cil_input.h"

namespace {

void check(cil_status s, const char *what, cil_handle *h = nullptr, cil_input *in = nullptr) {
  if (s == CIL_OK) return;
  char buf[1024] = {0};
  if (h) cil_last_error(h, buf, sizeof buf);
  if (!buf[0] && in) cil_input_last_error(in, buf, sizeof buf);
  throw std::runtime_error(std::string(what) + " failed (" + std::to_string(static_cast<int>(s)) + "): " + buf);
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s input.json\n", argv[0]);
    return 2;
  }
  cil_input *in = nullptr;
  cil_handle *h = nullptr;
  cil_frame_writer *w = nullptr;
  try {
    check(cil_input_load(argv[1], 1, &in), "reading the run description", nullptr, in);
    cil_config cfg{};
    cil_colony_params p{};
    cil_run_info run{};
    check(cil_input_config(in, &cfg, &p, &run), "cil_input_config", nullptr, in);
    if (run.output_h5) std::fprintf(stderr, "# H5 output is not served by this build (no libhdf5); GSD only\n");
    const int D = cfg.dim, cap = run.capacity > run.ncells ? run.capacity : run.ncells;
    std::vector<double> pos(static_cast<size_t>(cap) * 2 * D), sig(static_cast<size_t>(cap) * 2);
    std::vector<int> t0(cap), tsw(cap);
    cil_colony_view v{};
    v.capacity = cap;
    v.pos = pos.data();
    v.sigma = sig.data();
    v.t0 = t0.data();
    v.tswitch = tsw.data();
    check(cil_input_initial_state(in, &v), "INIT", nullptr, in);
    int32_t capacity = cap;
    check(cil_create(&cfg, &p, &capacity, &h), "cil_create");
    check(cil_upload(h, 0, &v), "cil_upload", h);

    cil_frame_options fo{};
    fo.cell_name = run.cell_name;
    fo.elem_names[0] = run.elem_names[0];
    fo.elem_names[1] = run.elem_names[1];
    const std::string dir = run.output_dir, name = run.output_name;
    if (run.output_gsd) {
      mkdir(dir.c_str(), 0755);
      check(cil_frame_open(h, 0, (dir + "/" + name + ".gsd").c_str(), &fo, &w), "cil_frame_open", h);
      check(cil_frame_write(w, 0, nullptr), "cil_frame_write", h);  // outputFrame(0, 0)
    }
    int64_t ts = 0;
    for (int iframe = 1; iframe <= run.frames; ++iframe) {
      check(cil_step(h, run.gts, &ts), "cil_step", h);  // GTS x mdStep(ts)
      cil_obs o{};
      check(cil_observables(h, 0, &o), "cil_observables", h);
      std::fprintf(stderr, "# ts = %8lld time = %12.3e \t cells = %8d elements = %8d\n", static_cast<long long>(ts),
                   static_cast<double>(ts) * p.dt, o.ncells, 2 * o.ncells);
      if (w) check(cil_frame_write(w, ts, nullptr), "cil_frame_write", h);
    }
    if (w) {
      check(cil_frame_close(w), "cil_frame_close", h);
      w = nullptr;
      mkdir((dir + "/Last").c_str(), 0733);
      check(cil_frame_open(h, 0, (dir + "/Last/" + name + ".Last.gsd").c_str(), &fo, &w), "cil_frame_open", h);
      check(cil_frame_write(w, 0, nullptr), "cil_frame_write", h);
      check(cil_frame_close(w), "cil_frame_close", h);
      w = nullptr;
    }
    cil_destroy(h);
    cil_input_free(in);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    if (w) cil_frame_close(w);
    if (h) cil_destroy(h);
    cil_input_free(in);
    return 1;
  }
  return 0;
}
