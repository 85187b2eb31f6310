// cil_gpu_run: the reference's main loop (CIL.cu:1072-1127) on the GPU step, driven by the
// reference's JSON run description.
//
//   cil_gpu_run input.json [frames [gts]]
//
// Reads the run with cil_input (include/cil_input.h), builds INIT on the host, uploads it,
// writes frame 0, then FRAMES times: GTS steps (one step call), checkPositions (with DRAIN),
// a progress line in the reference's format, a GSD frame when OUTPUT.FORMAT lists GSD. At the
// end the final state goes to <DIR>/Last/<NAME>.Last.gsd as one frame labelled step 0
// (finalizeOutput, OutputWriter.cpp:724-745). Two-element species run the two-element step
// with the device-fed frame writer (include/cil_gsd.h); single-element species, the shipped
// runs, run the cell-cycle model (include/cil_cycle.h), whose frames are downloaded and
// written with the GSD file layer (charge: the cycle activity rho, mass: the pressure, as
// outputGSDParticles writes them, OutputWriter.cpp:522-615). The optional arguments replace
// MD.FRAMES and MD.GTS. Failures print the library's message and exit 1, as run_assert does
// (Utils.hpp:99-109).
#include <sys/stat.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include <cstdlib>

#include "cil_cycle.h"
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

// One GSD frame of the cell-cycle model (outputGSDFrame with one element per cell).
void cycle_frame(cil_gsd_file *f, const cil_cycle_params &p, const cil_run_info &run, cil_cycle *h, int64_t step) {
  const int cap = 0;
  (void)cap;
  cil_cycle_view v{};
  v.capacity = 0;
  cil_cycle_download(h, &v);  // cell count (fails with CIL_ERR_CAPACITY on purpose)
  const int n = v.ncells, D = p.dim;
  std::vector<double> pos(static_cast<size_t>(n) * D), vel(static_cast<size_t>(n) * D), sig(n), rho(n), pres(n);
  v = cil_cycle_view{};
  v.capacity = n;
  v.pos = pos.data();
  v.vel = vel.data();
  v.sigma = sig.data();
  v.rho = rho.data();
  v.pressure = pres.data();
  if (cil_cycle_download(h, &v) != CIL_OK) throw std::runtime_error("cil_cycle_download failed");
  const uint64_t st = static_cast<uint64_t>(step);
  const uint8_t dims = 3;
  const float box[6] = {static_cast<float>(p.box[0]), static_cast<float>(p.box[1]),
                        static_cast<float>(D == 3 ? p.box[2] : p.sigma_core), 0, 0, 0};
  const uint32_t N = static_cast<uint32_t>(n);
  auto chunk = [&](const char *name, int type, uint64_t rows, uint32_t cols, const void *data) {
    if (rows == 0) return;
    if (cil_gsd_write_chunk(f, name, type, rows, cols, data) != CIL_OK) throw std::runtime_error("GSD write failed");
  };
  chunk("configuration/step", CIL_GSD_UINT64, 1, 1, &st);
  chunk("configuration/dimensions", CIL_GSD_UINT8, 1, 1, &dims);
  chunk("configuration/box", CIL_GSD_FLOAT, 6, 1, box);
  chunk("particles/N", CIL_GSD_UINT32, 1, 1, &N);
  if (step == 0) {
    std::vector<char> types(63, 0);
    snprintf(types.data(), 63, "%s", run.cell_name);
    chunk("particles/types", CIL_GSD_INT8, 1, 63, types.data());
  }
  std::vector<float> fs(n), fr(n), fp(n), xp(static_cast<size_t>(n) * 3, 0.0f), vp(static_cast<size_t>(n) * 3, 0.0f);
  std::vector<uint32_t> tid(n, 0);
  for (int i = 0; i < n; ++i) {
    fs[i] = static_cast<float>(sig[i]);
    fr[i] = static_cast<float>(rho[i]);
    fp[i] = static_cast<float>(pres[i]);
    for (int d = 0; d < D; ++d) {
      xp[3 * i + d] = static_cast<float>(pos[static_cast<size_t>(i) * D + d] - 0.5 * p.box[d]);
      vp[3 * i + d] = static_cast<float>(vel[static_cast<size_t>(i) * D + d]);
    }
    if (D == 2) xp[3 * i + 2] = static_cast<float>(0.0 * (-0.01 * 1.0));  // zhack[0]
  }
  if (p.divide || p.apoptosis || step == 0) {
    chunk("particles/Z", CIL_GSD_FLOAT, n, 1, fs.data());
    chunk("particles/diameter", CIL_GSD_FLOAT, n, 1, fs.data());
    chunk("particles/typeid", CIL_GSD_UINT32, n, 1, tid.data());
  }
  if (p.divide) chunk("particles/charge", CIL_GSD_FLOAT, n, 1, fr.data());
  chunk("particles/position", CIL_GSD_FLOAT, n, 3, xp.data());
  chunk("particles/velocity", CIL_GSD_FLOAT, n, 3, vp.data());
  chunk("particles/mass", CIL_GSD_FLOAT, n, 1, fp.data());
  if (cil_gsd_end_frame(f) != CIL_OK) throw std::runtime_error("GSD write failed");
}

void cycle_check(cil_status s, const char *what, cil_cycle *h) {
  if (s == CIL_OK) return;
  char buf[1024] = {0};
  if (h) cil_cycle_last_error(h, buf, sizeof buf);
  throw std::runtime_error(std::string(what) + " failed (" + std::to_string(static_cast<int>(s)) + "): " + buf);
}

// The single-element run: the cell-cycle model
int run_cycle(cil_input *in, int frames_arg, int gts_arg) {
  cil_cycle_params p{};
  cil_run_info run{};
  check(cil_input_cycle_config(in, &p, &run), "cil_input_cycle_config", nullptr, in);
  if (frames_arg > 0) run.frames = frames_arg;
  if (gts_arg > 0) run.gts = gts_arg;
  if (run.output_h5) std::fprintf(stderr, "# H5 output is not served by this build (no libhdf5); GSD only\n");
  const int n = run.ncells, D = p.dim;
  std::vector<double> pos(static_cast<size_t>(n) * D), sig(n), sigt(n), th(n), rho(n), om(n);
  cil_cycle_view v{};
  v.capacity = n;
  v.pos = pos.data();
  v.sigma = sig.data();
  v.sigma_t = sigt.data();
  v.theta = th.data();
  v.rho = rho.data();
  v.angvel = om.data();
  check(cil_input_cycle_initial_state(in, &v), "INIT", nullptr, in);
  cil_cycle *h = nullptr;
  cil_gsd_file *f = nullptr;
  try {
    const int cap = run.capacity > n ? run.capacity : n;
    if (cil_cycle_create(&p, cap, static_cast<uint64_t>(static_cast<uint32_t>(run.seed)), 0, &h) != CIL_OK)
      throw std::runtime_error("cil_cycle_create failed");
    cycle_check(cil_cycle_upload(h, &v), "cil_cycle_upload", h);
    const std::string dir = run.output_dir, name = run.output_name;
    if (run.output_gsd) {
      mkdir(dir.c_str(), 0755);
      if (cil_gsd_create((dir + "/" + name + ".gsd").c_str(), "CIL", "hoomd", CIL_GSD_VERSION(1, 1), &f) != CIL_OK)
        throw std::runtime_error("cannot create " + dir + "/" + name + ".gsd");
      cycle_frame(f, p, run, h, 0);
    }
    int64_t ts = 0;
    for (int iframe = 1; iframe <= run.frames; ++iframe) {
      cycle_check(cil_cycle_step(h, run.gts, &ts), "cil_cycle_step", h);
      cycle_check(cil_cycle_check_positions(h), "checkPositions", h);
      cil_cycle_view c{};
      cil_cycle_download(h, &c);
      std::fprintf(stderr, "# ts = %8lld time = %12.3e \t cells = %8d elements = %8d\n", static_cast<long long>(ts),
                   static_cast<double>(ts) * p.dt, c.ncells, c.ncells);
      if (f) cycle_frame(f, p, run, h, ts);
    }
    if (f) {
      cil_gsd_close(f);
      f = nullptr;
      mkdir((dir + "/Last").c_str(), 0733);
      if (cil_gsd_create((dir + "/Last/" + name + ".Last.gsd").c_str(), "CIL", "hoomd", CIL_GSD_VERSION(1, 1), &f) !=
          CIL_OK)
        throw std::runtime_error("cannot create the final-state file");
      cycle_frame(f, p, run, h, 0);
      cil_gsd_close(f);
      f = nullptr;
    }
    cil_cycle_destroy(h);
  } catch (...) {
    if (f) cil_gsd_close(f);
    cil_cycle_destroy(h);
    throw;
  }
  return 0;
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
    const int frames_arg = argc > 2 ? std::atoi(argv[2]) : 0, gts_arg = argc > 3 ? std::atoi(argv[3]) : 0;
    if (cil_input_elements(in) == 1) {
      const int rc = run_cycle(in, frames_arg, gts_arg);
      cil_input_free(in);
      return rc;
    }
    cil_config cfg{};
    cil_colony_params p{};
    cil_run_info run{};
    check(cil_input_config(in, &cfg, &p, &run), "cil_input_config", nullptr, in);
    if (frames_arg > 0) run.frames = frames_arg;
    if (gts_arg > 0) run.gts = gts_arg;
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
