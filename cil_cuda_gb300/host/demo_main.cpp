// A reference-style main loop driving the GPU step through the MDIntegrator plug-in
// (CIL.cu:1072-1127 shape: frames of GTS mdStep calls, host arrays read at frames).
// Reads a colony from a binary file, runs `frames` x `gts` steps in oracle mode, writes
// the final colony; with a sixth argument, also a GSD frame at step 0 and after every frame
// of steps through the device-fed frame writer (outputFrame's GSD branch,
// OutputWriter.cpp:708-712). Used by tests/test_cpp_host.py; not part of the library.
//
// input:  int32 ncells, int32 dim, int32 capacity, double[17] params (see below),
//         pos[n*2*dim], sigma[n*2], int32 t0[n], int32 tswitch[n]
// output: int32 ncells, int32 ts, pos, sigma, vel, t0, tswitch
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "gpu_euler.hpp"

typedef void (*MDIntegrator)(int &ts);

int main(int argc, char **argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s in.bin out.bin frames gts seed [frames.gsd]\n", argv[0]);
    return 2;
  }
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t n, dim, cap;
  double q[17];
  if (std::fread(&n, 4, 1, f) != 1 || std::fread(&dim, 4, 1, f) != 1 || std::fread(&cap, 4, 1, f) != 1 ||
      std::fread(q, 8, 17, f) != 17)
    return 2;
  std::vector<double> pos(static_cast<size_t>(cap) * 2 * dim), sig(static_cast<size_t>(cap) * 2),
      vel(static_cast<size_t>(cap) * 2 * dim);
  std::vector<int> t0(cap), tsw(cap);
  size_t ok = std::fread(pos.data(), 8, static_cast<size_t>(n) * 2 * dim, f);
  ok += std::fread(sig.data(), 8, static_cast<size_t>(n) * 2, f);
  ok += std::fread(t0.data(), 4, n, f);
  ok += std::fread(tsw.data(), 4, n, f);
  std::fclose(f);
  if (ok != static_cast<size_t>(n) * (2 * dim + 2 + 2)) return 2;

  cil_colony_params p{};
  p.dim = dim;
  p.force_law = static_cast<int>(q[0]);
  p.divide = static_cast<int>(q[1]);
  for (int d = 0; d < dim; ++d) {
    p.box[d] = q[2 + d];
    p.periodic[d] = 1;
  }
  p.epsilon = q[5];
  p.rcut_scale = q[6];
  p.zeta[0] = p.zeta[1] = 1.0;
  p.motility[0] = q[7];
  p.motility[1] = q[8];
  p.kappa = q[9];
  p.rest0 = q[10];
  p.rest1 = q[11];
  p.noise_D = q[12];
  p.dt = q[13];
  p.div_tau_mu = q[14];
  p.div_tau_sigma = q[15];
  p.apop_rate = q[16];
  cil_config cfg{};
  cfg.dim = dim;
  cfg.force_law = p.force_law;
  cfg.precision = CIL_PREC_FP64;
  cfg.rng_mode = CIL_RNG_DSFMT;
  cfg.seed = static_cast<uint64_t>(std::atoll(argv[5]));
  cfg.num_colonies = 1;
  const int frames = std::atoi(argv[3]), gts = std::atoi(argv[4]);

  cilgpu::SpeciesArrays host;
  host.ncells = n;
  host.capacity = cap;
  host.pos = pos.data();
  host.sigma = sig.data();
  host.vel = vel.data();
  host.t0 = t0.data();
  host.tswitch = tsw.data();
  int ts = 0;
  try {
    cilgpu::GpuEuler plugin(cfg, p, cap, host, gts);
    cilgpu::bindGpuEuler(&plugin);
    MDIntegrator mdStep = cilgpu::gpuEuler;  // readMD's selection (Input.cpp:524-546)
    std::unique_ptr<cilgpu::GpuGsdOutput> gsd;
    if (argc > 6) {
      gsd.reset(new cilgpu::GpuGsdOutput(plugin, argv[6]));  // initializeOutput (OutputWriter.cpp:714-721)
      gsd->frame(ts);
    }
    for (int frame = 1; frame <= frames; ++frame) {
      for (int its = 0; its < gts; ++its) mdStep(ts);  // CIL.cu:1106
      if (gsd) gsd->frame(ts);
    }
    gsd.reset();  // finalizeOutput: flush and close
    n = plugin.host().ncells;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  FILE *o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  std::fwrite(&n, 4, 1, o);
  std::fwrite(&ts, 4, 1, o);
  std::fwrite(pos.data(), 8, static_cast<size_t>(n) * 2 * dim, o);
  std::fwrite(sig.data(), 8, static_cast<size_t>(n) * 2, o);
  std::fwrite(vel.data(), 8, static_cast<size_t>(n) * 2 * dim, o);
  std::fwrite(t0.data(), 4, n, o);
  std::fwrite(tsw.data(), 4, n, o);
  std::fclose(o);
  return 0;
}
