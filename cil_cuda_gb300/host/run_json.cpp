// cil_gpu_run: the reference's main loop (CIL.cu:1072-1127) on the GPU step, driven by the
// reference's JSON run description.
//
//   cil_gpu_run input.json [frames [gts]]
//
// Reads the run with cil_input (include/cil_input.h), builds INIT on the host, uploads it,
// writes frame 0, then FRAMES times: GTS steps (one step call), checkPositions (with DRAIN),
// a progress line in the reference's format, a GSD frame when OUTPUT.FORMAT lists GSD. At the
// end the final state goes to <DIR>/Last/<NAME>.Last.gsd as one frame labelled step 0
// (finalizeOutput, OutputWriter.cpp:724-745), and with H5 in OUTPUT.FORMAT to
// <DIR>/Last/<NAME>.Last.h5, single-element runs also to the frame file <DIR>/<NAME>.h5. Two-element species run the
// two-element step with the device-fed frame writer (include/cil_gsd.h); single-element
// species, the shipped runs, run the cell-cycle model (include/cil_cycle.h), whose frames are
// downloaded and written with the GSD file layer (charge: the cycle activity rho, mass: the pressure, as
// outputGSDParticles writes them, OutputWriter.cpp:522-615). The optional arguments replace
// MD.FRAMES and MD.GTS. Failures print the library's message and exit 1, as run_assert does
// (Utils.hpp:99-109).
#include <sys/stat.h>

#include <chrono>

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

// One snapshot of the frame file (outputHDF5Frame with id >= 0) of a cell-cycle colony
void cycle_h5_frame(cil_h5_frames *hf, int32_t frame, int32_t ts, const cil_cycle_params &p, cil_cycle *h,
                    double cpu_time);

// The final-state file <DIR>/Last/<NAME>.Last.h5 (outputHDF5Frame with id -1 and the move into
// Last/, OutputWriter.cpp:388-441, 736-745) of a cell-cycle colony; with hf, a snapshot instead
void cycle_last_h5(const std::string &path, const cil_cycle_params &p, cil_cycle *h, double cpu_time,
                   cil_h5_frames *hf = nullptr, int32_t frame = 0, int32_t ts = 0) {
  cil_cycle_view v{};
  cil_cycle_download(h, &v);  // cell count
  const int n = v.ncells, D = p.dim;
  std::vector<double> pos(static_cast<size_t>(n) * D), vel(pos.size()), fc(pos.size()), fd(pos.size()), fr(pos.size()),
      sig(n), rho(n), th(n), pres(n);
  std::vector<int32_t> t0(n), state(n, 0);  // every cell of the single-element cycle is dividing (0)
  v = cil_cycle_view{};
  v.capacity = n;
  v.pos = pos.data();
  v.vel = vel.data();
  v.force = fc.data();
  v.force_dis = fd.data();
  v.force_ran = fr.data();
  v.sigma = sig.data();
  v.rho = rho.data();
  v.theta = th.data();
  v.pressure = pres.data();
  v.t0 = t0.data();
  if (cil_cycle_download(h, &v) != CIL_OK) throw std::runtime_error("cil_cycle_download failed");
  cil_h5_state s{};
  s.ncells = n;
  s.nelem = 1;
  s.dim = D;
  s.pos = pos.data();
  s.vel = vel.data();
  s.force = fc.data();
  s.force_dis = fd.data();
  s.force_ran = fr.data();
  s.sigma = sig.data();
  s.rho = rho.data();
  s.theta = th.data();
  s.pressure = pres.data();
  s.state = state.data();
  s.t0 = t0.data();
  s.cpu_time = cpu_time;
  const cil_status st = hf ? cil_h5_frames_write(hf, frame, ts, &s) : cil_h5_write_state(path.c_str(), &s);
  if (st != CIL_OK) {
    char buf[512] = {0};
    cil_h5_last_error(buf, sizeof buf);
    throw std::runtime_error(std::string("writing ") + (hf ? std::string("an H5 frame") : path) + ": " + buf);
  }
}

void cycle_h5_frame(cil_h5_frames *hf, int32_t frame, int32_t ts, const cil_cycle_params &p, cil_cycle *h,
                    double cpu_time) {
  cycle_last_h5(std::string(), p, h, cpu_time, hf, frame, ts);
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
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
  const int n = run.ncells, D = p.dim;
  std::vector<double> pos(static_cast<size_t>(n) * D), vel(pos.size(), 0.0), sig(n), sigt(n), th(n), rho(n), om(n);
  cil_cycle_view v{};
  v.capacity = n;
  v.pos = pos.data();
  v.vel = vel.data();  // INIT H5 ALL restarts the velocities
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
    cil_h5_frames *hf = nullptr;  // the H5 frame file (outputHDF5Frame)
    if (run.output_h5) {
      mkdir(dir.c_str(), 0755);
      if (cil_h5_frames_create((dir + "/" + name + ".h5").c_str(), p.dim, p.box, p.dt, run.gts, &hf) != CIL_OK)
        throw std::runtime_error("cannot create " + dir + "/" + name + ".h5");
      cycle_h5_frame(hf, 0, 0, p, h, 0.0);
    }
    int64_t ts = 0;
    double cpu_time = 0.0;
    for (int iframe = 1; iframe <= run.frames; ++iframe) {
      const auto t_frame = std::chrono::steady_clock::now();
      cycle_check(cil_cycle_step(h, run.gts, &ts), "cil_cycle_step", h);
      cycle_check(cil_cycle_check_positions(h), "checkPositions", h);
      cil_cycle_view c{};
      cil_cycle_download(h, &c);
      std::fprintf(stderr, "# ts = %8lld time = %12.3e \t cells = %8d elements = %8d\n", static_cast<long long>(ts),
                   static_cast<double>(ts) * p.dt, c.ncells, c.ncells);
      if (f) cycle_frame(f, p, run, h, ts);
      cpu_time = seconds_since(t_frame);
      if (hf) cycle_h5_frame(hf, iframe, static_cast<int32_t>(ts), p, h, cpu_time);
    }
    if (hf && cil_h5_frames_close(hf) != CIL_OK) throw std::runtime_error("writing " + dir + "/" + name + ".h5");
    if (run.output_h5) {
      mkdir((dir + "/Last").c_str(), 0733);
      cycle_last_h5(dir + "/Last/" + name + ".Last.h5", p, h, cpu_time);
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
    const int D = cfg.dim, cap = run.capacity > run.ncells ? run.capacity : run.ncells;
    std::vector<double> pos(static_cast<size_t>(cap) * 2 * D), sig(static_cast<size_t>(cap) * 2);
    std::vector<int> t0(cap), tsw(cap), cst(cap, 2);
    cil_colony_view v{};
    v.capacity = cap;
    v.pos = pos.data();
    v.sigma = sig.data();
    v.t0 = t0.data();
    v.tswitch = tsw.data();
    v.cell_state = cst.data();  // initializeCellStatus's states (the crawling/dividing cells use them)
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
    // the state of the colony as outputHDF5Frame writes it: a snapshot of the frame file (hf) or
    // the final-state file (path)
    auto two_element_h5 = [&](cil_handle *hh, const char *path, cil_h5_frames *f5, int32_t frame, int32_t ts5,
                              double cpu) {
      std::vector<double> p5(static_cast<size_t>(cap) * 2 * D), s5(static_cast<size_t>(cap) * 2), v5(p5.size()),
          f5f(p5.size());
      std::vector<int> t05(cap), tw5(cap), cs5(cap, 0);
      cil_colony_view w5{};
      w5.capacity = cap;
      w5.pos = p5.data();
      w5.sigma = s5.data();
      w5.vel = v5.data();
      w5.t0 = t05.data();
      w5.tswitch = tw5.data();
      w5.cell_state = cs5.data();
      check(cil_download(hh, 0, &w5), "cil_download", hh);
      check(cil_forces(hh, 0, f5f.data()), "cil_forces", hh);
      const int n5 = w5.ncells;
      std::vector<double> rho(n5, 1.0);  // initializeCellStatus's activity, which the step never changes
      std::vector<int32_t> state(cs5.begin(), cs5.begin() + n5);  // the cells' states
      cil_h5_state st5{};
      st5.ncells = n5;
      st5.nelem = 2;
      st5.dim = D;
      st5.pos = p5.data();
      st5.vel = v5.data();
      st5.force = f5f.data();
      st5.sigma = s5.data();
      st5.rho = rho.data();
      st5.state = state.data();
      st5.t0 = t05.data();
      st5.cpu_time = cpu;
      const cil_status r5 = f5 ? cil_h5_frames_write(f5, frame, ts5, &st5) : cil_h5_write_state(path, &st5);
      if (r5 != CIL_OK) {
        char buf[512] = {0};
        cil_h5_last_error(buf, sizeof buf);
        throw std::runtime_error(std::string("writing H5 output: ") + buf);
      }
    };
    cil_h5_frames *hf = nullptr;
    if (run.output_h5) {
      mkdir(dir.c_str(), 0755);
      if (cil_h5_frames_create((dir + "/" + name + ".h5").c_str(), D, p.box, p.dt, run.gts, &hf) != CIL_OK)
        throw std::runtime_error("cannot create " + dir + "/" + name + ".h5");
      two_element_h5(h, nullptr, hf, 0, 0, 0.0);
    }
    int64_t ts = 0;
    double cpu_time = 0.0;
    for (int iframe = 1; iframe <= run.frames; ++iframe) {
      const auto t_frame = std::chrono::steady_clock::now();
      check(cil_step(h, run.gts, &ts), "cil_step", h);  // GTS x mdStep(ts)
      cil_obs o{};
      check(cil_observables(h, 0, &o), "cil_observables", h);
      std::fprintf(stderr, "# ts = %8lld time = %12.3e \t cells = %8d elements = %8d\n", static_cast<long long>(ts),
                   static_cast<double>(ts) * p.dt, o.ncells, 2 * o.ncells);
      if (w) check(cil_frame_write(w, ts, nullptr), "cil_frame_write", h);
      cpu_time = seconds_since(t_frame);
      if (hf) two_element_h5(h, nullptr, hf, iframe, static_cast<int32_t>(ts), cpu_time);
    }
    if (hf && cil_h5_frames_close(hf) != CIL_OK) throw std::runtime_error("writing " + dir + "/" + name + ".h5");
    hf = nullptr;
    if (run.output_h5) {  // the final state of the two-element colony
      mkdir((dir + "/Last").c_str(), 0733);
      two_element_h5(h, (dir + "/Last/" + name + ".Last.h5").c_str(), nullptr, 0, 0, cpu_time);
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
