// Host side of libcilgpu.so: the C ABI declared in include/cil_gpu.h.
//
// A handle owns every device array of its colonies (layout in cil_internal.cuh), one CUDA
// stream, and, in oracle mode (CIL_RNG_DSFMT), a host mirror of the integer cell state
// (cycle start / end per cell and the cell count) so that the host can draw the
// reference's random numbers in the reference's order without reading the device back:
// division is decided by the cycle clock alone and apoptosis tests every slot, so the
// draw sequence depends only on integers the host already knows.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cil_gpu.h"
#include "cil_internal.cuh"
#include "host_rng.h"

using namespace cil;

namespace {

constexpr int kSlotAlign = 1024;

template <typename T>
T *dalloc(size_t n) {
  void *p = nullptr;
  if (n == 0) n = 1;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
  return static_cast<T *>(p);
}

struct HostColony {
  cil_colony_params p{};
  int cap = 0;
  bool uploaded = false;
  double sigma_max = 0.0;
  // oracle-mode mirror
  int n = 0;
  std::vector<int> t0, tsw;
  std::vector<int> cst;  // cell states (crawling/dividing cells)
};

}  // namespace

struct GraphSlot {
  int key;                 // cur | meta << 1 | pu << 2 at the first step, | two steps << 3, | last << 4
  uint64_t gen;
  cudaGraphExec_t exec;
  int64_t launches;        // kernels in the graph
};

struct cil_handle {
  cil_config cfg{};
  ColonyCounters *h_cnt = nullptr;  // pinned host copies of d_cnt (cil_step's status read), 2 x B
  cudaEvent_t cnt_ev[2] = {nullptr, nullptr};  // deferred status: copy of each half done
  int cnt_slot = 0;                  // deferred status: half the next copy goes to
  int cnt_pending = -1;              // deferred status: half holding the previous call's copy
  int B = 0, D = 2;
  std::vector<HostColony> hc;
  std::vector<ColonyConst> cc;
  int CC = 0;          // total cell capacity
  size_t SS = 0;       // total slots
  int NBpad = 0;       // total padded bins
  int nscan = 0;       // scan blocks
  int ctiles = 0;      // max cell tiles
  int grid_slots = 0;  // persistent grid for slot kernels
  int grid_cells = 0;
  int grid_force = 0;
  int stiles = 0;      // tiles over the slot capacity
  int ptiles = 0;      // tiles over the slot pairs of the capacity (grid of the list force kernel)
  int cell_block = 256;  // threads (cells) per block of the list force kernel
  int list_variant = 0;  // list force kernel: staging depth and CTAs per SM (cil_config.staging/occupancy)
  int nsm = 0;
  bool geometry_ready = false;
  int64_t ts = 0;
  std::string err;
  cudaStream_t stream = nullptr;

  // device arrays
  ColonyConst *d_col = nullptr;
  ColonyCounters *d_cnt = nullptr;
  double *d_x[2] = {nullptr, nullptr};
  double *d_sig[2] = {nullptr, nullptr};
  int *d_eid[2] = {nullptr, nullptr};
  int cur = 0, meta = 0;
  float4 *d_pk[2] = {nullptr, nullptr};  // mixed: packed elements (coordinates + diameter)
  int *d_sbin[2] = {nullptr, nullptr};
  int2 *d_cyc[2] = {nullptr, nullptr};
  double *d_sigma_c = nullptr;  // canonical diameters [2 * CC]
  bool need_exact = true;       // next rebuild takes the FP64 reference path
  int pu = 1;                   // which d_pk holds the current packed elements
  // skin mode
  bool skin_mode = false;
  unsigned char *d_state[2] = {nullptr, nullptr};
  int *d_nbr = nullptr, *d_ncnt = nullptr, *d_fresh = nullptr;
  int *d_lflat = nullptr, *d_lwarp = nullptr;  // the lists flattened per warp of 32 cells
  StatPart *d_spart = nullptr;                 // displacement statistics slots [B][kStatSlots]
  unsigned char *d_oflat = nullptr;
  unsigned short *d_lstart = nullptr;
  unsigned long long *d_fhead = nullptr, *d_fnext = nullptr;  // per-bin fresh lists
  float *d_uref = nullptr, *d_facc = nullptr;
  unsigned *d_ftouch = nullptr;  // one bit per slot: facc holds a fresh-pair contribution
  ColonySkin *d_skin = nullptr;
  int *d_ts = nullptr;           // device step counter (kernels read the step from here)
  int *d_anyreb = nullptr;       // skin mode: [4] some colony rebuilds at step ts ([ts & 1]),
                                 // colonies decided ([2]), rebuild nodes run ([3])
  cudaStream_t side = nullptr;   // skin mode: captures the bodies of the rebuild nodes
  bool cond_capture = false;     // a steady-step capture: rebuild kernels in a conditional node
  // CUDA graphs of two steady steps, one per buffer parity (graph_gen: invalidation)
  std::vector<GraphSlot> graphs;
  uint64_t graph_gen = 0;
  bool graphs_off = false;
  int64_t graph_steps = 0, graphs_captured = 0;
  SchedState *d_sched = nullptr;
  float *d_mlp = nullptr;        // scheduler network parameters (null: fixed skin and cadence)
  float sched_skin_min = 0.0f, sched_interval_scale = 0.0f;
  int sched_use_interval = 0;
  int permute_period = 250;      // steps between slot re-sorts (locality, compaction)
  bool lists_stale = true;       // slots were re-sorted outside a step: rebuild the lists
  double *d_vel = nullptr, *d_frc = nullptr;
  double *d_vel2 = nullptr;  // second velocity buffer for rebuilds outside a step
  int *d_key = nullptr;
  unsigned long long *d_perm = nullptr;
  int *d_bcount = nullptr;
  int2 *d_range = nullptr;
  int *d_scan_sum = nullptr, *d_scan_off = nullptr, *d_scan_col = nullptr;
  int *d_slot_of = nullptr;
  int *d_t0 = nullptr, *d_tsw = nullptr;
  int *d_cst = nullptr;     // cell states [CC] (crawling/dividing cells)
  bool any_cell_sm = false, any_swell = false;  // some colony has crawling/dividing cells (with swelling)
  unsigned char *d_smflag = nullptr;  // per cell: division criterion met (oracle mode, state machine)
  int *d_tiles_used = nullptr, *d_tiles_live = nullptr, *d_tiles_cell = nullptr;
  int *d_tiles_pairs = nullptr;  // skin mode: tiles over slot pairs (the cell-major force kernel)
  int *d_tile_count = nullptr, *d_tile_off = nullptr;
  int *d_upchk = nullptr;     // upload checks: bad-value bits, largest diameter (double bits)
  int *d_dueq = nullptr;      // skin mode, Philox: cells due to divide, per colony (due_base)
  size_t due_total = 0;
  int *d_evdone = nullptr;    // skin mode, Philox: colonies whose events are done this step
  int *d_dead = nullptr;
  int *d_divq = nullptr;  // division queue [CC]
  double *d_obs = nullptr;  // com_prev, disp, vref: 3 * D * CC
  bool obs_ready_any = false;
  std::vector<char> obs_ready;
  double *d_partials = nullptr;
  int partials_cap = 0;
  double *d_stage = nullptr;  // staging for upload/download, sized for the largest colony
  size_t stage_cap = 0;
  // oracle mode
  HostRng rng;
  double *d_noise = nullptr;
  double *h_noise = nullptr;  // pinned
  int *d_oracle_i = nullptr;  // mothers, cycle ends, removal ops
  double *d_oracle_d = nullptr;
  size_t oracle_cap = 0;
  // timings
  std::vector<cudaEvent_t> evpool;
  double t_rebuild = 0, t_force = 0, t_events = 0, t_total = 0;
  int64_t launches = 0;
};

namespace {

cil_status fail(cil_handle *h, cil_status s, const std::string &m) {
  if (h) h->err = m;
  return s;
}

#define CUDA_TRY(h, call)                                                              \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail((h), CIL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void free_all(cil_handle *h) {
  void *ptrs[] = {h->d_col, h->d_cnt, h->d_x[0], h->d_x[1], h->d_sig[0], h->d_sig[1], h->d_eid[0],
                  h->d_eid[1], h->d_pk[0], h->d_pk[1], h->d_sbin[0], h->d_sbin[1],
                  h->d_cyc[0], h->d_cyc[1], h->d_sigma_c, h->d_state[0], h->d_state[1], h->d_nbr,
                  h->d_ncnt, h->d_fresh, h->d_spart, h->d_lflat, h->d_lwarp, h->d_oflat, h->d_lstart, h->d_uref, h->d_facc, h->d_ftouch, h->d_skin, h->d_sched, h->d_mlp, h->d_fhead, h->d_fnext, h->d_ts, h->d_anyreb, h->d_vel, h->d_vel2, h->d_frc, h->d_key, h->d_perm,
                  h->d_bcount, h->d_range, h->d_scan_sum, h->d_scan_off, h->d_scan_col,
                  h->d_slot_of, h->d_t0, h->d_tsw, h->d_tiles_used, h->d_tiles_live, h->d_tiles_pairs,
                  h->d_tiles_cell, h->d_tile_count, h->d_tile_off, h->d_upchk, h->d_dueq, h->d_evdone, h->d_dead, h->d_divq, h->d_obs,
                  h->d_partials, h->d_stage, h->d_noise, h->d_oracle_i, h->d_oracle_d};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (auto &gs : h->graphs)
    if (gs.exec) cudaGraphExecDestroy(gs.exec);
  h->graphs.clear();
  if (h->h_noise) cudaFreeHost(h->h_noise);
  if (h->h_cnt) cudaFreeHost(h->h_cnt);
  for (auto e : h->cnt_ev)
    if (e) cudaEventDestroy(e);
  for (auto e : h->evpool) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->side) cudaStreamDestroy(h->side);
}

// bins per axis as LinkListOrtho::get_opt_size + reset (Utils.hpp:872-908)
void grid_geometry(const cil_colony_params &p, double width, int *ns, bool *single) {
  const int D = p.dim;
  double mn = p.box[0];
  for (int d = 1; d < D; ++d) mn = std::min(mn, p.box[d]);
  const double ir = 1.0 / (width + mn * 1.0e-8);
  bool overkill = false;
  for (int d = 0; d < 3; ++d) ns[d] = 1;
  for (int d = 0; d < D; ++d) {
    ns[d] = static_cast<int>(p.box[d] * ir);
    overkill = overkill || ns[d] < 3;
  }
  if (overkill)
    for (int d = 0; d < D; ++d) ns[d] = 1;
  *single = overkill;
}

// Steady-state length of the reference's bond (Input.cpp:139-144): sqrt(r2max (1 - alpha / beta
// kappa)) with alpha = 1/zeta0 + 1/zeta1, beta = m0/zeta0 + m1/zeta1, r2max = RMAX^2.
double fene_rss(const cil_colony_params &p) {
  const double zi0 = 1.0 / p.zeta[0], zi1 = 1.0 / p.zeta[1];
  const double alpha = zi0 + zi1;
  const double beta = p.motility[0] * zi0 + p.motility[1] * zi1;
  return std::sqrt(p.fene_rmax * p.fene_rmax * (1.0 - alpha / beta * p.fene_kappa));
}

double bin_width_for(const cil_handle *h, const HostColony &c) {
  // a colony without cells stays without (nothing divides): one bin
  if (!(c.sigma_max > 0.0)) return std::max(c.p.box[0], std::max(c.p.box[1], c.p.box[2]));
  // the law's reach for the largest diameter (the soft-core well reaches xi past contact)
  // crawling/dividing cells take SIGMA_CORE at a division and may swell up to its larger value
  double smax = c.sigma_max;
  if (c.p.intra_law == CIL_INTRA_FENE && c.p.divide) smax = std::max(smax, std::max(c.p.sigma_core[0], c.p.sigma_core[1]));
  const double reach = c.p.force_law == CIL_FORCE_SC ? smax + c.p.well_sigma : smax;
  const double need = c.p.rcut_scale * reach + h->cfg.skin;
  return h->cfg.bin_width > need ? h->cfg.bin_width : need;
}

cil_status setup_geometry(cil_handle *h) {
  int bin_base = 0;
  for (int c = 0; c < h->B; ++c) {
    HostColony &hc = h->hc[c];
    ColonyConst &C = h->cc[c];
    if (!hc.uploaded) return fail(h, CIL_ERR_STATE, "colony " + std::to_string(c) + " not uploaded");
    const double width = bin_width_for(h, hc);
    bool single;
    grid_geometry(hc.p, width, C.ns, &single);
    C.single_bin = single ? 1 : 0;
    long long nb = 1;
    for (int d = 0; d < h->D; ++d) nb *= C.ns[d];
    if (nb > (1ll << 30)) return fail(h, CIL_ERR_CONFIG, "bin grid too large");
    C.nbins = static_cast<int>(nb);
    {
      const uint32_t d0 = h->D == 2 ? static_cast<uint32_t>(C.ns[1]) : static_cast<uint32_t>(C.ns[1] * C.ns[2]);
      const uint32_t d1 = static_cast<uint32_t>(C.ns[2] > 0 ? C.ns[2] : 1);
      div_invariant_setup(d0, &C.div_m[0], &C.div_s1[0], &C.div_s2[0]);
      div_invariant_setup(d1, &C.div_m[1], &C.div_s1[1], &C.div_s2[1]);
    }
    C.nbins_pad = ((C.nbins + kScanItems - 1) / kScanItems) * kScanItems;
    C.bin_base = bin_base;
    C.scan_base = bin_base / kScanItems;
    bin_base += C.nbins_pad;
    for (int d = 0; d < 3; ++d) {
      C.bw[d] = d < h->D ? hc.p.box[d] / C.ns[d] : 0.0;
      C.bwf[d] = static_cast<float>(C.bw[d]);
      C.inv_bwf[d] = d < h->D ? static_cast<float>(1.0 / C.bw[d]) : 0.0f;
      if (d < 2) {
        C.uq_scale[d] = static_cast<float>(65535.0 / C.bw[d]);
        C.uq_inv[d] = static_cast<float>(C.bw[d] / 65535.0);
      }
    }
  }
  if (bin_base != h->NBpad) {
    cudaFree(h->d_bcount);
    cudaFree(h->d_range);
    cudaFree(h->d_scan_sum);
    cudaFree(h->d_scan_off);
    cudaFree(h->d_scan_col);
    cudaFree(h->d_fhead);
    h->d_fhead = nullptr;
    h->NBpad = bin_base;
    h->nscan = bin_base / kScanItems;
    h->d_bcount = dalloc<int>(h->NBpad);
    h->d_range = dalloc<int2>(h->NBpad);
    h->d_scan_sum = dalloc<int>(h->nscan);
    h->d_scan_off = dalloc<int>(h->nscan);
    h->d_scan_col = dalloc<int>(h->nscan);
    if (!h->d_bcount || !h->d_range || !h->d_scan_sum || !h->d_scan_off || !h->d_scan_col)
      return fail(h, CIL_ERR_CUDA, "out of device memory for bins");
    if (h->skin_mode) {
      h->d_fhead = dalloc<unsigned long long>(h->NBpad);
      if (!h->d_fhead) return fail(h, CIL_ERR_CUDA, "out of device memory for bins");
      // epoch 0xffffffff: matches no rebuild count, so every list starts empty
      CUDA_TRY(h, cudaMemsetAsync(h->d_fhead, 0xff, sizeof(unsigned long long) * h->NBpad, h->stream));
    }
  }
  std::vector<int> scol(h->nscan);
  for (int c = 0; c < h->B; ++c)
    for (int i = 0; i < h->cc[c].nbins_pad / kScanItems; ++i) scol[h->cc[c].scan_base + i] = c;
  CUDA_TRY(h, cudaMemsetAsync(h->d_bcount, 0, sizeof(int) * h->NBpad, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(h->d_range, 0, sizeof(int2) * h->NBpad, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(h->d_scan_col, scol.data(), sizeof(int) * h->nscan, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(h->d_col, h->cc.data(), sizeof(ColonyConst) * h->B, cudaMemcpyHostToDevice, h->stream));
  h->geometry_ready = true;
  h->graph_gen += 1;  // captured graphs hold the old bin arrays
  return CIL_OK;
}

cil_status ensure_ready(cil_handle *h) {
  CUDA_TRY(h, cudaSetDevice(h->cfg.device));
  if (!h->geometry_ready) return setup_geometry(h);
  return CIL_OK;
}

RebuildArgs rebuild_args(cil_handle *h) {
  RebuildArgs a{};
  a.col = h->d_col;
  a.cnt = h->d_cnt;
  a.B = h->B;
  a.SS = h->SS;
  a.tiles_used = h->d_tiles_used;
  a.tiles_live = h->d_tiles_live;
  a.tiles_cell = h->d_tiles_cell;
  a.scan_col = h->d_scan_col;
  a.nscan = h->nscan;
  const bool mixed = h->cfg.precision == CIL_PREC_MIXED;
  a.x_in = h->d_x[h->cur];
  a.sig_in = h->d_sig[h->meta];
  a.eid_in = h->d_eid[h->meta];
  a.x_out = h->d_x[1 - h->cur];
  a.sig_out = h->d_sig[1 - h->meta];
  a.eid_out = h->d_eid[1 - h->meta];
  a.pk_out = mixed ? h->d_pk[1 - h->pu] : nullptr;
  a.pk_in = mixed ? h->d_pk[h->pu] : nullptr;
  a.skin = nullptr;  // a permuting rebuild re-sorts every colony
  a.permute = 1;
  a.state_out = h->skin_mode ? h->d_state[1 - h->meta] : nullptr;
  a.sbin_in = h->d_sbin[h->meta];
  a.sbin_out = h->d_sbin[1 - h->meta];
  a.cyc_in = h->d_cyc[h->meta];
  a.cyc_out = h->d_cyc[1 - h->meta];
  a.sigma_c = h->d_sigma_c;
  a.t0c = h->d_t0;
  a.tswc = h->d_tsw;
  // the FP64 form always takes the reference path; the mixed form re-anchors its FP32
  // local coordinates on the FP64 positions after an upload and every 32 steps
  a.exact = (!mixed || h->need_exact || (h->ts % 32) == 0) ? 1 : 0;
  a.key = h->d_key;
  a.bcount = h->d_bcount;
  a.range = h->d_range;
  a.perm = h->d_perm;
  a.scan_sum = h->d_scan_sum;
  a.scan_off = h->d_scan_off;
  a.slot_of = h->d_slot_of;
  a.dim = h->D;
  return a;
}

// A rebuild inside a step needs no velocities (the force pass rewrites them); a rebuild
// outside a step (cil_forces, cil_bins) carries them through the permutation so that a
// later download still pairs each element with its own velocity.
// vel_to: carry the velocities through the permutation into this buffer instead (the first
// half step's velocities of a Heun step, read by the second half step; no buffer swap).
cil_status do_rebuild(cil_handle *h, bool carry_vel = false, bool exact = false, double *vel_to = nullptr) {
  if (exact) h->need_exact = true;
  RebuildArgs a = rebuild_args(h);
  if (vel_to) {
    a.vel_in = h->d_vel;
    a.vel_out = vel_to;
  } else if (carry_vel) {
    if (!h->d_vel2) {
      h->d_vel2 = dalloc<double>(static_cast<size_t>(h->D) * h->SS);
      if (!h->d_vel2) return fail(h, CIL_ERR_CUDA, "out of device memory (velocities)");
    }
    a.vel_in = h->d_vel;
    a.vel_out = h->d_vel2;
  }
  launch_tiles(h->d_col, h->d_cnt, h->B, 0, h->d_tiles_used, h->stream);
  launch_rebuild(a, h->grid_slots, h->stream);
  h->cur = 1 - h->cur;
  h->meta = 1 - h->meta;
  if (h->cfg.precision == CIL_PREC_MIXED) h->pu = 1 - h->pu;
  h->need_exact = false;
  h->lists_stale = true;
  if (carry_vel) {
    std::swap(h->d_vel, h->d_vel2);
    h->graph_gen += 1;  // captured steps hold the old velocity buffer
  }
  return CIL_OK;
}

// Skin mode's slot re-sort: cells ranked by the bin of their back element, each cell's
// elements moved into a slot pair (cell-major slots, the layout k_force_cells reads), tombstones
// dropped. Re-anchors the FP32 records on the FP64 positions after an upload and every 32 steps,
// like the permuting rebuild.
cil_status do_cell_resort(cil_handle *h) {
  RebuildArgs a = rebuild_args(h);
  a.skin = nullptr;
  a.any_rebuild = nullptr;
  a.permute = 0;
  launch_tiles(h->d_col, h->d_cnt, h->B, 2, h->d_tiles_cell, h->stream);
  launch_cell_resort(a, h->grid_cells, h->stream);
  h->cur = 1 - h->cur;
  h->meta = 1 - h->meta;
  h->pu = 1 - h->pu;
  h->need_exact = false;
  h->lists_stale = true;
  return CIL_OK;
}

ForceArgs force_args(cil_handle *h, int noise_mode, int integrate, double *vel, double *frc) {
  ForceArgs a{};
  a.col = h->d_col;
  a.cnt = h->d_cnt;
  a.B = h->B;
  a.SS = h->SS;
  a.cst = h->d_cst;
  a.tiles_live = h->d_tiles_live;
  a.x_in = h->d_x[h->cur];
  a.x_out = h->d_x[1 - h->cur];
  a.sig = h->d_sig[h->meta];
  a.eid = h->d_eid[h->meta];
  a.pk = h->d_pk[h->pu];
  a.pk_next = h->d_pk[1 - h->pu];
  a.dueq = h->d_dueq;
  if (h->skin_mode) {
    a.tiles = h->d_tiles_pairs;
    a.skin = h->d_skin;
    a.nbr = h->d_nbr;
    a.ncnt = h->d_ncnt;
    a.lflat = h->d_lflat;
    a.oflat = h->d_oflat;
    a.lstart = h->d_lstart;
    a.lwarp = h->d_lwarp;
    a.spart = h->d_spart;
    a.uref = h->d_uref;
    a.facc = h->d_facc;
    a.ftouch = h->d_ftouch;
    a.sched = h->d_sched;
  }
  a.sbin = h->d_sbin[h->meta];
  a.cyc = h->d_cyc[h->meta];
  a.range = h->d_range;
  a.slot_of = h->d_slot_of;
  a.noise = h->d_noise;
  a.noise_act = h->d_noise ? h->d_noise + 2 * static_cast<size_t>(h->CC) * h->D : nullptr;
  a.noise_act_t = a.noise_act ? a.noise_act + h->CC : nullptr;
  a.vel = vel;
  a.frc = frc;
  a.ts_dev = h->d_ts;
  a.seed_lo = static_cast<uint32_t>(h->cfg.seed);
  a.seed_hi = static_cast<uint32_t>(h->cfg.seed >> 32);
  a.noise_mode = noise_mode;
  a.integrate = integrate;
  return a;
}

EventArgs event_args(cil_handle *h) {
  EventArgs a{};
  a.col = h->d_col;
  a.cnt = h->d_cnt;
  a.B = h->B;
  a.SS = h->SS;
  a.tiles_cell = h->d_tiles_cell;
  a.x = h->d_x[h->cur];
  a.sig = h->d_sig[h->meta];
  a.pk = h->cfg.precision == CIL_PREC_MIXED ? h->d_pk[h->pu] : nullptr;
  a.sbin = h->d_sbin[h->meta];
  if (h->skin_mode) {
    a.skin = h->d_skin;
    a.state = h->d_state[h->meta];
    a.uref = h->d_uref;
    a.ncnt = h->d_ncnt;
    a.fresh = h->d_fresh;
    a.fhead = h->d_fhead;
    a.fnext = h->d_fnext;
  }
  a.cyc = h->d_cyc[h->meta];
  a.sigma_c = h->d_sigma_c;
  a.eid = h->d_eid[h->meta];
  a.vel = h->d_vel;
  a.slot_of = h->d_slot_of;
  a.t0 = h->d_t0;
  a.tsw = h->d_tsw;
  a.cst = h->d_cst;
  a.smflag = h->d_smflag;
  a.tile_count = h->d_tile_count;
  a.tile_off = h->d_tile_off;
  a.dueq = h->d_dueq;
  a.ev_done = h->d_evdone;
  a.any_rebuild = h->d_anyreb;
  a.dead = h->d_dead;
  a.divq = h->d_divq;
  if (h->d_obs) {
    a.obs_com_prev = h->d_obs;
    a.obs_disp = h->d_obs + static_cast<size_t>(h->D) * h->CC;
    a.obs_vref = h->d_obs + 2 * static_cast<size_t>(h->D) * h->CC;
  }
  a.CC = h->CC;
  a.ts_dev = h->d_ts;
  a.seed_lo = static_cast<uint32_t>(h->cfg.seed);
  a.seed_hi = static_cast<uint32_t>(h->cfg.seed >> 32);
  return a;
}

SkinArgs skin_args(cil_handle *h, int force_rebuild) {
  SkinArgs a{};
  a.col = h->d_col;
  a.cnt = h->d_cnt;
  a.skin = h->d_skin;
  a.sched = h->d_sched;
  a.B = h->B;
  a.SS = h->SS;
  a.tiles = h->d_tiles_used;
  a.eid = h->d_eid[h->meta];
  a.state = h->d_state[h->meta];
  a.pk = h->d_pk[h->pu];
  a.uref = h->d_uref;
  a.sbin = h->d_sbin[h->meta];
  a.range = h->d_range;
  a.perm = h->d_perm;
  a.nbr = h->d_nbr;
  a.ncnt = h->d_ncnt;
  a.lflat = h->d_lflat;
  a.oflat = h->d_oflat;
  a.lstart = h->d_lstart;
  a.lwarp = h->d_lwarp;
  a.spart = h->d_spart;
  a.fresh = h->d_fresh;
  a.fhead = h->d_fhead;
  a.fnext = h->d_fnext;
  a.facc = h->d_facc;
  a.ftouch = h->d_ftouch;
  a.key = h->d_key;
  a.bcount = h->d_bcount;
  a.force_rebuild = force_rebuild;
  a.ts_dev = h->d_ts;
  a.any_rebuild = h->d_anyreb;
  a.mlp = h->d_mlp;
  a.use_interval = h->sched_use_interval;
  a.skin_min = h->sched_skin_min;
  a.skin_max = static_cast<float>(h->cfg.skin);
  a.interval_scale = h->sched_interval_scale;
  a.grid = h->nsm * 16;  // fresh-pair kernel: 64 warps per SM over all colonies' fresh elements
  return a;
}

// oracle mode: the passive noise of the coming force evaluation, drawn exactly as
// updateWienerProcess does (CIL.cu:793-818), in canonical [cell][elem][dim] order
cil_status draw_oracle_noise(cil_handle *h, bool *any) {
  *any = false;
  // the pinned buffer may still be the source of the previous step's copy
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  size_t total = 0;
  bool active = false;
  const size_t act_off = 2 * static_cast<size_t>(h->CC) * h->D;  // the bond's active noise: radial, angular [CC]
  for (int c = 0; c < h->B; ++c) {
    const HostColony &hc = h->hc[c];
    const bool act = h->cc[c].act_noise != 0;
    if (!(hc.p.noise_D > 0.0) && !act) continue;
    *any = true;
    const int per = hc.p.noise_per_cell ? 1 : 2;
    const size_t base = static_cast<size_t>(h->cc[c].cell_base) * per * h->D;
    const size_t m = static_cast<size_t>(hc.n) * per * h->D;
    if (hc.p.noise_D > 0.0) {
      const double amp = std::sqrt(2.0 * hc.p.noise_D) * (1.0 / std::sqrt(hc.p.dt));
      for (size_t i = 0; i < m; ++i) h->h_noise[base + i] = amp * h->rng.normal();
    } else {
      std::fill(h->h_noise + base, h->h_noise + base + m, 0.0);
    }
    total = std::max(total, base + m);
    if (act) {
      // CIL.cu:803-815: radial for every cell, then angular; a zero amplitude draws nothing
      active = true;
      double *wr = h->h_noise + act_off + h->cc[c].cell_base, *wt = wr + h->CC;
      const double ar = std::sqrt(2.0 * hc.p.noise_radial) * (1.0 / std::sqrt(hc.p.dt));
      const double at = std::sqrt(2.0 * hc.p.noise_angular) * (1.0 / std::sqrt(hc.p.dt));
      for (int i = 0; i < hc.n; ++i) wr[i] = hc.p.noise_radial > 0.0 ? ar * h->rng.normal() : 0.0;
      for (int i = 0; i < hc.n; ++i) wt[i] = hc.p.noise_angular > 0.0 ? at * h->rng.normal() : 0.0;
    }
  }
  if (*any && total > 0)
    CUDA_TRY(h, cudaMemcpyAsync(h->d_noise, h->h_noise, sizeof(double) * total, cudaMemcpyHostToDevice, h->stream));
  if (active)
    CUDA_TRY(h, cudaMemcpyAsync(h->d_noise + act_off, h->h_noise + act_off, sizeof(double) * 2 * h->CC,
                                cudaMemcpyHostToDevice, h->stream));
  return CIL_OK;
}

cil_status ensure_oracle_buffers(cil_handle *h, size_t need_i, size_t need_d) {
  const size_t need = std::max(need_i, need_d);
  if (need <= h->oracle_cap) return CIL_OK;
  cudaFree(h->d_oracle_i);
  cudaFree(h->d_oracle_d);
  h->oracle_cap = std::max(need, h->oracle_cap * 2);
  h->d_oracle_i = dalloc<int>(h->oracle_cap);
  h->d_oracle_d = dalloc<double>(h->oracle_cap);
  if (!h->d_oracle_i || !h->d_oracle_d) return fail(h, CIL_ERR_CUDA, "out of device memory (oracle lists)");
  return CIL_OK;
}

// oracle mode: division and apoptosis draws on the host mirror, replayed on the device
cil_status oracle_events(cil_handle *h) {
  const int ts = static_cast<int>(h->ts);
  int cap_hit = -1;
  for (int c = 0; c < h->B; ++c) {
    HostColony &hc = h->hc[c];
    const int D = h->D;
    std::vector<int> mothers, tsws;
    std::vector<double> dirs;
    std::vector<int> smops;      // crawling/dividing cells: cell, kind (1 start, 2 failed), new time
    std::vector<double> smdirs;  // the failed divisions' axes
    const int n0 = hc.n;
    const bool sm = hc.p.divide && hc.p.intra_law == CIL_INTRA_FENE;
    if (sm) {
      // calculDivisions (CIL.cu:369-455) on the host mirror, in cell order; which dividing
      // cells have their elements Rmin apart is read from the device (this step's positions)
      std::vector<unsigned char> flags(static_cast<size_t>(n0));
      if (n0 > 0) {
        launch_sm_flags(event_args(h), c, n0, D, h->stream);
        CUDA_TRY(h, cudaMemcpyAsync(flags.data(), h->d_smflag + h->cc[c].cell_base, static_cast<size_t>(n0),
                                    cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        h->launches += 1;
      }
      auto span = [&](double mu, double sd) {
        const int s = nint(h->rng.normal(mu, sd) / hc.p.dt);
        return s >= 1 ? s : 1;
      };
      for (int i = 0; i < n0; ++i) {
        if (hc.cst[i] == 0) {  // dividing
          if (flags[i]) {
            if (hc.n >= hc.cap) {
              cap_hit = c;
              continue;
            }
            const int k = hc.n++;
            double dm[3] = {0, 0, 0}, dd[3] = {0, 0, 0};
            h->rng.on_dsphere(D, dm);
            h->rng.on_dsphere(D, dd);
            const int td = ts + span(hc.p.mig_tau_mu, hc.p.mig_tau_sigma);
            const int tm = hc.tsw[i] + span(hc.p.mig_tau_mu, hc.p.mig_tau_sigma);
            hc.t0[k] = ts;
            hc.tsw[k] = td;
            hc.cst[k] = 1;
            hc.t0[i] = ts;
            hc.tsw[i] = tm;
            hc.cst[i] = 1;
            mothers.push_back(i);
            tsws.push_back(td);
            tsws.push_back(tm);
            for (int d = 0; d < D; ++d) dirs.push_back(dm[d]);
            for (int d = 0; d < D; ++d) dirs.push_back(dd[d]);
          } else if (hc.tsw[i] == ts) {  // failed division
            double df[3] = {0, 0, 0};
            h->rng.on_dsphere(D, df);
            hc.tsw[i] += span(hc.p.mig_tau_mu, hc.p.mig_tau_sigma);
            hc.cst[i] = 1;
            smops.insert(smops.end(), {i, 2, hc.tsw[i]});
            for (int d = 0; d < D; ++d) smdirs.push_back(df[d]);
          }
        } else if (hc.tsw[i] == ts) {  // starts dividing
          hc.tsw[i] += span(hc.p.div_tau_mu, hc.p.div_tau_sigma);
          hc.cst[i] = 0;
          smops.insert(smops.end(), {i, 1, hc.tsw[i]});
          for (int d = 0; d < D; ++d) smdirs.push_back(0.0);
        }
      }
    } else if (hc.p.divide) {
      for (int i = 0; i < n0; ++i) {
        if (hc.tsw[i] != ts) continue;
        if (hc.n >= hc.cap) {  // skipped, as the oracle does, and reported after the step
          cap_hit = c;
          continue;
        }
        const int k = hc.n++;
        double dm[3] = {0, 0, 0}, dd[3] = {0, 0, 0};
        h->rng.on_dsphere(D, dm);
        h->rng.on_dsphere(D, dd);
        auto span = [&]() {
          const int s = nint(h->rng.normal(hc.p.div_tau_mu, hc.p.div_tau_sigma) / hc.p.dt);
          return s >= 1 ? s : 1;
        };
        const int td = ts + span();
        const int tm = ts + span();
        hc.t0[k] = ts;
        hc.tsw[k] = td;
        hc.t0[i] = ts;
        hc.tsw[i] = tm;
        mothers.push_back(i);
        tsws.push_back(td);
        tsws.push_back(tm);
        for (int d = 0; d < D; ++d) dirs.push_back(dm[d]);
        for (int d = 0; d < D; ++d) dirs.push_back(dd[d]);
      }
    }
    std::vector<int> ops;
    if (hc.p.apop_rate > 0.0) {
      const double prob = hc.p.apop_rate * hc.p.dt;
      int i = 0;
      while (i < hc.n) {
        if (h->rng.uniform0x(1.0) <= prob) {
          const int last = hc.n - 1;
          hc.t0[i] = hc.t0[last];
          hc.tsw[i] = hc.tsw[last];
          if (sm) hc.cst[i] = hc.cst[last];
          hc.n -= 1;
          ops.push_back(i);
        } else {
          ++i;
        }
      }
    }
    const int ndiv = static_cast<int>(mothers.size());
    const int nsm = static_cast<int>(smops.size() / 3);
    if (ndiv == 0 && ops.empty() && nsm == 0) continue;
    const size_t ni = mothers.size() + tsws.size() + ops.size() + smops.size();
    cil_status st = ensure_oracle_buffers(h, ni, dirs.size() + smdirs.size());
    if (st != CIL_OK) return st;
    std::vector<int> packed;
    packed.insert(packed.end(), mothers.begin(), mothers.end());
    packed.insert(packed.end(), tsws.begin(), tsws.end());
    packed.insert(packed.end(), ops.begin(), ops.end());
    packed.insert(packed.end(), smops.begin(), smops.end());
    dirs.insert(dirs.end(), smdirs.begin(), smdirs.end());
    CUDA_TRY(h, cudaMemcpyAsync(h->d_oracle_i, packed.data(), sizeof(int) * packed.size(), cudaMemcpyHostToDevice, h->stream));
    if (!dirs.empty())
      CUDA_TRY(h, cudaMemcpyAsync(h->d_oracle_d, dirs.data(), sizeof(double) * dirs.size(), cudaMemcpyHostToDevice, h->stream));
    // the staged host vectors must stay alive until the copies ran
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    EventArgs a = event_args(h);
    launch_sm_ops(a, c, nsm, h->d_oracle_i + 3 * ndiv + ops.size(), h->d_oracle_d + static_cast<size_t>(ndiv) * 2 * D,
                  D, h->stream);
    launch_divisions_list(a, c, n0, ndiv, h->d_oracle_i, h->d_oracle_d, h->d_oracle_i + ndiv, D, h->stream);
    launch_apo_ops_with_div(a, c, ndiv, static_cast<int>(ops.size()), h->d_oracle_i + 3 * ndiv, D, h->stream);
    h->launches += (ndiv > 0 ? 1 : 0) + (nsm > 0 ? 1 : 0) + 1;
  }
  // updateDiameters (CIL.cu:970-991) after the events: swelling of dividing cells
  for (int c = 0; c < h->B; ++c) {
    const HostColony &hc = h->hc[c];
    if (hc.p.divide && hc.p.intra_law == CIL_INTRA_FENE && hc.p.div_swelling && hc.n > 0) {
      launch_sm_swell(event_args(h), c, hc.n, ts, h->stream);
      h->launches += 1;
    }
  }
  if (cap_hit >= 0) return fail(h, CIL_ERR_CAPACITY, "cell capacity exceeded in colony " + std::to_string(cap_hit));
  return CIL_OK;
}

cil_status ensure_stage(cil_handle *h, size_t need) {
  if (need <= h->stage_cap) return CIL_OK;
  cudaFree(h->d_stage);
  h->stage_cap = std::max(need, static_cast<size_t>(1024));
  h->d_stage = dalloc<double>(h->stage_cap);
  if (!h->d_stage) {
    h->stage_cap = 0;
    return fail(h, CIL_ERR_CUDA, "out of device memory (staging)");
  }
  return CIL_OK;
}

cudaEvent_t pool_event(cil_handle *h, size_t i) {
  while (h->evpool.size() <= i) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    h->evpool.push_back(e);
  }
  return h->evpool[i];
}

// Error bits of the colonies' counters as a status (and the handle's message).
cil_status counter_status(cil_handle *h, const ColonyCounters *k) {
  for (int c = 0; c < h->B; ++c) {
    if (k[c].err & kErrNan) return fail(h, CIL_ERR_NAN, "non-finite force in colony " + std::to_string(c));
    if (k[c].err & kErrBox) return fail(h, CIL_ERR_OUT_OF_BOX, "element left the box in colony " + std::to_string(c));
    if (k[c].err & kErrCap) return fail(h, CIL_ERR_CAPACITY, "cell capacity exceeded in colony " + std::to_string(c));
  }
  return CIL_OK;
}

cil_status check_counters(cil_handle *h, std::vector<ColonyCounters> *out = nullptr) {
  std::vector<ColonyCounters> k(h->B);
  CUDA_TRY(h, cudaMemcpyAsync(k.data(), h->d_cnt, sizeof(ColonyCounters) * h->B, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (out) *out = k;
  return counter_status(h, k.data());
}

// One step's launches on the handle's stream (oracle mode: with its host draws). When timed,
// four events bracket the phases; a step being captured into a graph records none.
cil_status enqueue_force_pass(cil_handle *h, bool last, int heun, bool first, cudaEvent_t before_force);

// One Euler step, or the two half steps of a Heun step (each: noise draw, bins or lists,
// force pass with its position update), then the step counter and the events. Timed phases:
// rebuild = the first pass's bins / lists; force = the rest up to the last force pass.
cil_status enqueue_step(cil_handle *h, bool last, bool timed, size_t e0) {
  const bool heun = h->cfg.integrator == CIL_INTEGRATOR_HEUN;
  const int passes = heun ? 2 : 1;
  if (timed) CUDA_TRY(h, cudaEventRecord(pool_event(h, e0), h->stream));
  for (int pass = 0; pass < passes; ++pass) {
    const cil_status st = enqueue_force_pass(h, last, heun ? pass + 1 : 0, pass == 0,
                                             timed && pass == 0 ? pool_event(h, e0 + 1) : nullptr);
    if (st != CIL_OK) return st;
  }
  const bool philox = h->cfg.rng_mode != CIL_RNG_DSFMT;
  // skin mode, Philox: one event kernel over the force kernel's due-cell queues, which also
  // moves the step counter; otherwise a step-end launch (the step counter and, in Philox mode,
  // the cell tile table) and the tile-wise event kernels
  const bool due_events = philox && h->skin_mode;
  if (!due_events) {
    launch_advance_ts(h->d_ts, h->d_anyreb, h->stream, h->d_cnt, h->B, philox ? h->d_tiles_cell : nullptr);
    h->launches += 1;
  }
  if (timed) CUDA_TRY(h, cudaEventRecord(pool_event(h, e0 + 2), h->stream));
  h->ts += 1;
  if (h->cfg.rng_mode == CIL_RNG_DSFMT) {
    const cil_status st = oracle_events(h);
    if (st != CIL_OK) return st;
    h->launches += 2;
  } else if (due_events) {
    launch_events_due(event_args(h), h->D, h->stream);
    h->launches += 1;
  } else {
    launch_events_fast(event_args(h), h->grid_cells, h->D, h->stream, h->any_cell_sm);
    h->launches += h->any_cell_sm ? 4 : 3;
    if (h->any_swell) {
      launch_sm_swell_all(event_args(h), h->grid_cells, h->stream);
      h->launches += 1;
    }
  }
  if (timed) CUDA_TRY(h, cudaEventRecord(pool_event(h, e0 + 3), h->stream));
  CUDA_TRY(h, cudaGetLastError());
  return CIL_OK;
}

// Noise draw (oracle mode), bins or Verlet lists, and one force pass with its position
// update. heun: 0 for an Euler step, 1 / 2 for the half steps of a Heun step. first: the
// first pass of the step (the slot re-sort of skin mode happens there only).
cil_status enqueue_force_pass(cil_handle *h, bool last, int heun, bool first, cudaEvent_t before_force) {
  const bool oracle = h->cfg.rng_mode == CIL_RNG_DSFMT;
  cil_status st = CIL_OK;
  bool noise = false;
  if (oracle) {
    st = draw_oracle_noise(h, &noise);
    if (st != CIL_OK) return st;
  } else {
    for (int c = 0; c < h->B; ++c) noise = noise || h->hc[c].p.noise_D > 0.0;
  }
  if (h->skin_mode) {
    // list rebuilds are decided on the device (guard, cadence, fresh overflow); the host
    // re-sorts the slots on a fixed schedule and after uploads
    const bool permute =
        h->need_exact || h->lists_stale || (first && (h->ts % h->permute_period) == 0);
    // the rebuild decision; without a re-sort the same launch writes the tile tables over the
    // slots (list build) and the slot pairs (force kernel)
    SkinArgs sb = skin_args(h, permute ? 1 : 0);
    if (!permute) {
      sb.tiles_used_out = h->d_tiles_used;
      sb.tiles_pairs_out = h->d_tiles_pairs;
      sb.pair_tile = 2 * h->cell_block;
    }
    // with CIL_FLAG_REBUILD_NODE, a steady-step capture puts the rebuild kernels into a
    // conditional (IF) node that k_skin_begin sets: steps on which no colony rebuilds launch
    // none of them (the kernels still check the rebuild flags themselves, so the node only
    // saves launches)
    const bool use_cond = h->cond_capture && !permute;
    cudaGraph_t cg = nullptr;
    if (use_cond) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      CUDA_TRY(h, cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, &cg));
      if (cs != cudaStreamCaptureStatusActive || !cg) return fail(h, CIL_ERR_CUDA, "rebuild node: stream not capturing");
      CUDA_TRY(h, cudaGraphConditionalHandleCreate(&sb.cond, cg, 1, cudaGraphCondAssignDefault));
      sb.use_cond = 1;
    }
    launch_skin_begin(sb, h->stream);
    if (permute) {
      // cell-major re-sort; every colony then rebuilds its bin index and lists (host request)
      st = do_cell_resort(h);
      if (st != CIL_OK) return st;
      launch_tiles(h->d_col, h->d_cnt, h->B, 0, h->d_tiles_used, h->stream, 3, h->d_tiles_pairs, 2 * h->cell_block);
    }
    cudaStream_t rs = h->stream;
    if (use_cond) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      const cudaGraphNode_t *deps = nullptr;
      const cudaGraphEdgeData *edges = nullptr;
      size_t ndeps = 0;
      CUDA_TRY(h, cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, nullptr, &deps, &edges, &ndeps));
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = sb.cond;
      cp.conditional.type = cudaGraphCondTypeIf;
      cp.conditional.size = 1;
      cudaGraphNode_t node = nullptr;
      CUDA_TRY(h, cudaGraphAddNode(&node, cg, deps, edges, ndeps, &cp));
      CUDA_TRY(h, cudaStreamUpdateCaptureDependencies(h->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
      CUDA_TRY(h, cudaStreamBeginCaptureToGraph(h->side, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal));
      rs = h->side;
    }
    launch_skin_rebin(skin_args(h, 0), h->D, h->grid_slots, rs);
    RebuildArgs ra = rebuild_args(h);
    ra.permute = 0;
    ra.skin = h->d_skin;  // only colonies with rebuild_now
    ra.any_rebuild = h->d_anyreb;
    ra.ts_dev = h->d_ts;
    ra.state_out = nullptr;
    launch_rebuild(ra, h->grid_slots, rs);  // slot count unchanged: tile tables stay
    launch_skin_lists(skin_args(h, 0), h->D, h->cfg.force_law, h->grid_slots, rs);
    launch_list_flatten(skin_args(h, 0), h->grid_slots, rs);
    if (use_cond) {
      cudaGraph_t body = nullptr;
      CUDA_TRY(h, cudaStreamEndCapture(h->side, &body));
    }
    launch_fresh_pairs(skin_args(h, 0), h->D, h->cfg.force_law, h->stream);
    h->lists_stale = false;
    // kernels of the rebuild node: counted when the node runs (cil_timings)
    h->launches += permute ? 18 : (use_cond ? 2 : 9);
  } else {
    // the second half step of a Heun step reads the first half's velocities: carried through
    // the re-sort (only when velocities are written, i.e. the last step of a cil_step call)
    double *vel_prev = nullptr;
    if (heun == 2 && last) {
      if (!h->d_vel2) {
        h->d_vel2 = dalloc<double>(static_cast<size_t>(h->D) * h->SS);
        if (!h->d_vel2) return fail(h, CIL_ERR_CUDA, "out of device memory (velocities)");
      }
      vel_prev = h->d_vel2;
    }
    st = do_rebuild(h, false, false, vel_prev);
    if (st != CIL_OK) return st;
    h->launches += 10;
    if (before_force) CUDA_TRY(h, cudaEventRecord(before_force, h->stream));
    ForceArgs fa = force_args(h, noise ? (oracle ? 2 : 1) : 0, 1, last ? h->d_vel : nullptr, nullptr);
    fa.heun = heun;
    fa.vel_prev = vel_prev;
    launch_force(fa, h->D, h->cfg.force_law, h->cfg.precision, h->grid_force, kTile, h->stream);
    h->launches += 1;
    h->cur = 1 - h->cur;
    if (h->cfg.precision == CIL_PREC_MIXED) h->pu = 1 - h->pu;
    return CIL_OK;
  }
  if (before_force) CUDA_TRY(h, cudaEventRecord(before_force, h->stream));
  ForceArgs fa = force_args(h, noise ? (oracle ? 2 : 1) : 0, 1, last ? h->d_vel : nullptr, nullptr);
  fa.heun = heun;
  fa.collect_due = (!oracle && heun != 1) ? 1 : 0;  // the step's events read the due-cell queue
  launch_force_list(fa, h->D, h->cfg.force_law, h->ptiles, h->list_variant, h->cell_block, h->stream);  // skin mode
  h->launches += 1;
  h->cur = 1 - h->cur;
  if (h->cfg.precision == CIL_PREC_MIXED) h->pu = 1 - h->pu;
  return CIL_OK;
}

// A step whose launches and arguments depend only on the buffer parities: Philox noise, no
// slot re-sort (skin mode), no FP64 re-anchoring (mixed form without skin).
bool steady_step(const cil_handle *h, int64_t ts) {
  if (h->cfg.rng_mode != CIL_RNG_PHILOX || (h->cfg.flags & CIL_FLAG_NO_GRAPH) || h->need_exact) return false;
  if (h->skin_mode) return !h->lists_stale && (ts % h->permute_period) != 0;
  if (h->cfg.precision == CIL_PREC_MIXED) return (ts % 32) != 0;
  return true;
}

struct HostStepState {
  int cur, meta, pu;
  bool need_exact, lists_stale;
  int64_t ts;
};

HostStepState host_state(const cil_handle *h) {
  return HostStepState{h->cur, h->meta, h->pu, h->need_exact, h->lists_stale, h->ts};
}

// What one steady step does to the host-side state (mirrors enqueue_step)
void advance_host_state(const cil_handle *h, HostStepState *s) {
  const bool mixed = h->cfg.precision == CIL_PREC_MIXED;
  const int passes = h->cfg.integrator == CIL_INTEGRATOR_HEUN ? 2 : 1;
  for (int pass = 0; pass < passes; ++pass) {
    if (h->skin_mode) {
      s->lists_stale = false;
    } else {  // do_rebuild
      s->cur ^= 1;
      s->meta ^= 1;
      if (mixed) s->pu ^= 1;
      s->need_exact = false;
      s->lists_stale = true;
    }
    s->cur ^= 1;  // force pass
    if (mixed) s->pu ^= 1;
  }
  s->ts += 1;
}

bool same_state(const HostStepState &a, const HostStepState &b) {
  return a.cur == b.cur && a.meta == b.meta && a.pu == b.pu && a.need_exact == b.need_exact &&
         a.lists_stale == b.lists_stale && a.ts == b.ts;
}

void restore_host_state(cil_handle *h, const HostStepState &s) {
  h->cur = s.cur;
  h->meta = s.meta;
  h->pu = s.pu;
  h->need_exact = s.need_exact;
  h->lists_stale = s.lists_stale;
  h->ts = s.ts;
}

// The executable graph of `nsteps` (1 or 2) steady steps starting from the current
// parities, the last of them writing the velocities when `last` (the final step of a cil_step
// call), captured on first use (the capture advances the host state as the steps would; the
// caller then replays the graph). On a capture failure the host state is put back, graphs are
// switched off for the handle and null is returned.
cudaGraphExec_t steady_graph(cil_handle *h, int nsteps, bool last, int64_t *launches_per_graph) {
  const int key = h->cur | (h->meta << 1) | (h->pu << 2) | ((nsteps == 2 ? 1 : 0) << 3) | ((last ? 1 : 0) << 4);
  for (auto &gs : h->graphs)
    if (gs.key == key && gs.gen == h->graph_gen) {
      HostStepState s = host_state(h);
      for (int i = 0; i < nsteps; ++i) advance_host_state(h, &s);
      restore_host_state(h, s);
      *launches_per_graph = gs.launches;
      return gs.exec;
    }
  const HostStepState before = host_state(h);
  const int64_t launches0 = h->launches;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    h->graphs_off = true;
    return nullptr;
  }
  cil_status sc = CIL_OK;
  h->cond_capture = h->skin_mode && h->side != nullptr && (h->cfg.flags & CIL_FLAG_REBUILD_NODE) != 0;
  for (int i = 0; i < nsteps && sc == CIL_OK; ++i) sc = enqueue_step(h, last && i == nsteps - 1, false, 0);
  h->cond_capture = false;
  {
    // a failure inside a rebuild node's body leaves the side stream capturing: end it
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (h->side && cudaStreamIsCapturing(h->side, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t body = nullptr;
      cudaStreamEndCapture(h->side, &body);
    }
  }
  const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
  HostStepState expect = before;
  for (int i = 0; i < nsteps; ++i) advance_host_state(h, &expect);
  cudaGraphExec_t exec = nullptr;
  const bool ok = sc == CIL_OK && ec == cudaSuccess && g != nullptr && same_state(host_state(h), expect) &&
                  cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    restore_host_state(h, before);
    h->launches = launches0;
    h->graphs_off = true;
    return nullptr;
  }
  *launches_per_graph = h->launches - launches0;
  h->launches = launches0;
  h->graphs.push_back(GraphSlot{key, h->graph_gen, exec, *launches_per_graph});
  h->graphs_captured += 1;
  return exec;
}

}  // namespace

extern "C" {

const char *cil_version(void) { return "cil-gb300 0.1 (sm_103a)"; }

cil_status cil_host_register(void *ptr, size_t bytes) {
  if (!ptr || bytes == 0) return CIL_ERR_CONFIG;
  return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? CIL_OK : CIL_ERR_CUDA;
}

cil_status cil_host_unregister(void *ptr) {
  if (!ptr) return CIL_ERR_CONFIG;
  return cudaHostUnregister(ptr) == cudaSuccess ? CIL_OK : CIL_ERR_CUDA;
}

cil_status cil_host_rng_draw(uint32_t seed, int32_t kind, int64_t n, double *out) {
  if (!out || n < 0 || kind < 0 || kind > 5) return CIL_ERR_CONFIG;
  HostRng r;
  r.seed(seed);
  for (int64_t i = 0; i < n; ++i) {
    switch (kind) {
      case 0: out[i] = r.close_open(); break;
      case 1: out[i] = r.open_open(); break;
      case 2: out[i] = r.uniform(); break;
      case 3: out[i] = r.normal(); break;
      case 4: r.on_dsphere(2, out + 2 * i); break;
      default: r.on_dsphere(3, out + 3 * i); break;
    }
  }
  return CIL_OK;
}

void cil_last_error(const cil_handle *h, char *buf, size_t len) {
  if (!buf || len == 0) return;
  const std::string &m = h ? h->err : std::string("null handle");
  std::snprintf(buf, len, "%s", m.c_str());
}

cil_status cil_create(const cil_config *cfg, const cil_colony_params *params, const int32_t *cap_cells,
                      cil_handle **out) {
  if (!out) return CIL_ERR_CONFIG;
  *out = nullptr;
  if (!cfg || !params || !cap_cells) return CIL_ERR_CONFIG;
  if (cfg->dim != 2 && cfg->dim != 3) return CIL_ERR_CONFIG;
  if (cfg->num_colonies <= 0) return CIL_ERR_CONFIG;
  if (cfg->force_law < 0 || cfg->force_law > 3) return CIL_ERR_CONFIG;
  if (cfg->precision != CIL_PREC_FP64 && cfg->precision != CIL_PREC_MIXED) return CIL_ERR_CONFIG;
  if (cfg->rng_mode != CIL_RNG_PHILOX && cfg->rng_mode != CIL_RNG_DSFMT) return CIL_ERR_CONFIG;
  if (cfg->skin < 0.0 || (cfg->skin > 0.0 && cfg->precision != CIL_PREC_MIXED)) return CIL_ERR_CONFIG;
  if (cfg->skin > 0.0 && cfg->num_colonies > kMaxSkinColonies) return CIL_ERR_CONFIG;
  // block size: the list force kernel of skin mode takes 128, 256 or 512 threads; the other
  // kernels run 256
  if (cfg->block_size != 0 && cfg->block_size != kTile &&
      !(cfg->skin > 0.0 && (cfg->block_size == 128 || cfg->block_size == 512)))
    return CIL_ERR_CONFIG;
  if (cfg->integrator != CIL_INTEGRATOR_EULER && cfg->integrator != CIL_INTEGRATOR_HEUN) return CIL_ERR_CONFIG;
  int list_variant = -1;
  {
    const int st = cfg->staging == 0 ? 4 : cfg->staging, oc = cfg->occupancy == 0 ? 3 : cfg->occupancy;
    if (st == 4 && oc == 3) list_variant = 0;
    if (st == 2 && oc == 3) list_variant = 1;
    if (st == 1 && oc == 3) list_variant = 2;
    if (st == 1 && oc == 4) list_variant = 3;
    if (list_variant < 0) return CIL_ERR_CONFIG;
  }
  auto *h = new cil_handle();
  h->cfg = *cfg;
  h->list_variant = list_variant;
  h->B = cfg->num_colonies;
  h->D = cfg->dim;
  h->hc.resize(h->B);
  h->cc.resize(h->B);
  long long cells = 0, slots = 0;
  long long due_acc = 0;  // the due-cell queue: a power of two >= the cell capacity per colony
  for (int c = 0; c < h->B; ++c) {
    const cil_colony_params &p = params[c];
    if (p.dim != cfg->dim || p.force_law != cfg->force_law || cap_cells[c] <= 0 || !(p.dt > 0.0) ||
        !(p.zeta[0] > 0.0) || !(p.zeta[1] > 0.0) || p.nwalls < 0 || p.nwalls > 2 ||
        !(p.rcut_scale > 0.0) ||
        (p.force_law == CIL_FORCE_SC && (!(p.well_sigma > 0.0) || !(p.well_epsilon >= 0.0))) ||
        (p.intra_law != CIL_INTRA_SPRING && p.intra_law != CIL_INTRA_FENE) ||
        (p.intra_law == CIL_INTRA_FENE &&
         (!(p.fene_rmax > 0.0) || !(p.fene_spring_ratio >= 0.0 && p.fene_spring_ratio < 1.0) ||
          !(p.fene_kappa >= 0.0) || !(p.fene_kappa_push >= 0.0) || (!p.cil && !(fene_rss(p) > 0.0)))) ||
        // the crawling/dividing cells: oracle-mode draws (their outcomes are read back each step),
        // bins rebuilt every step (no Verlet skin), positive spans and radius
        (p.intra_law == CIL_INTRA_FENE && p.divide &&
         (cfg->skin > 0.0 || !(p.dt > 0.0) || !(p.div_r0 >= 0.0) ||
          !(p.div_rmin >= 0.0) || !(p.mig_tau_mu > 0.0) || !(p.mig_tau_sigma >= 0.0) ||
          !(p.sigma_core[0] > 0.0) || !(p.sigma_core[1] > 0.0) || !(p.fene_rmax_division >= 0.0))) ||
        // the bond's active noise: 2D, the reference's bond, oracle-mode draws, no Verlet skin
        ((p.noise_radial != 0.0 || p.noise_angular != 0.0) &&
         (!(p.noise_radial >= 0.0) || !(p.noise_angular >= 0.0) || p.intra_law != CIL_INTRA_FENE || cfg->dim != 2 ||
          cfg->rng_mode != CIL_RNG_DSFMT || cfg->skin > 0.0))) {
      delete h;
      return CIL_ERR_CONFIG;
    }
    for (int d = 0; d < cfg->dim; ++d)
      if (!(p.box[d] > 0.0)) {
        delete h;
        return CIL_ERR_CONFIG;
      }
    if (p.apop_rate * p.dt >= 1.0) {  // CIL.cuh:235
      delete h;
      return CIL_ERR_CONFIG;
    }
    HostColony &hc = h->hc[c];
    hc.p = p;
    hc.cap = cap_cells[c];
    ColonyConst &C = h->cc[c];
    std::memset(&C, 0, sizeof C);
    for (int d = 0; d < 3; ++d) {
      C.box[d] = d < cfg->dim ? p.box[d] : 1.0;
      C.ih[d] = 1.0 / C.box[d];
      C.periodic[d] = d < cfg->dim ? (p.periodic[d] != 0) : 0;
      C.ns[d] = 1;
    }
    C.cell_base = static_cast<int>(cells);
    C.cell_cap = cap_cells[c];
    C.slot_base = static_cast<int>(slots);
    // skin mode appends daughters between slot re-sorts: keep an eighth more slots
    const long long want = 2ll * cap_cells[c] + (cfg->skin > 0.0 ? (2ll * cap_cells[c]) / 8 + 4096 : 0);
    C.slot_cap = static_cast<int>(((want + kSlotAlign - 1) / kSlotAlign) * kSlotAlign);
    C.force_law = p.force_law;
    C.noise_per_cell = p.noise_per_cell;
    C.rng_stream = static_cast<uint32_t>(cfg->rng_stream_base + c);
    C.divide = p.divide;
    C.nwalls = p.nwalls;
    for (int w = 0; w < 2; ++w) {
      C.wall_dir[w] = p.wall_dir[w];
      C.wall_pos[w] = p.wall_pos[w];
    }
    C.wall_E = p.wall_E;
    C.epsilon = p.epsilon;
    C.rcut_scale = p.rcut_scale;
    for (int j = 0; j < 2; ++j) {
      C.zeta[j] = p.zeta[j];
      C.temp[j] = p.dt * (1.0 / p.zeta[j]);
      C.mu_eff[j] = C.temp[j] / p.dt;
      C.motility[j] = p.motility[j];
    }
    C.kappa = p.kappa;
    C.rest0 = p.rest0;
    C.rest1 = p.rest1;
    C.intra_fene = p.intra_law == CIL_INTRA_FENE ? 1 : 0;
    C.cil = p.cil ? 1 : 0;
    C.fene_kappa = p.fene_kappa;
    C.fene_kappa_push = p.fene_kappa_push;
    C.fene_ratio = p.fene_spring_ratio;
    C.fene_r2max = p.fene_rmax * p.fene_rmax;
    C.fene_rss = C.intra_fene ? fene_rss(p) : 0.0;
    C.fene_kappa_f = static_cast<float>(C.fene_kappa);
    C.fene_kappa_push_f = static_cast<float>(C.fene_kappa_push);
    C.fene_ratio_f = static_cast<float>(C.fene_ratio);
    C.fene_r2max_f = static_cast<float>(C.fene_r2max);
    C.fene_rss_f = static_cast<float>(C.fene_rss);
    C.cell_sm = C.intra_fene && p.divide ? 1 : 0;
    C.fene_r2max_div = p.fene_rmax_division > 0.0 ? p.fene_rmax_division * p.fene_rmax_division : C.fene_r2max;
    C.fene_r2max_div_f = static_cast<float>(C.fene_r2max_div);
    for (int j = 0; j < 2; ++j) {
      C.growth_k0[j] = p.growth_k0[j];
      C.growth_k1[j] = p.growth_k1[j];
      C.growth_k2[j] = p.growth_k2[j];
      C.growth_k0_f[j] = static_cast<float>(p.growth_k0[j]);
      C.growth_k1_f[j] = static_cast<float>(p.growth_k1[j]);
      C.growth_k2_f[j] = static_cast<float>(p.growth_k2[j]);
      C.sigma_core[j] = p.sigma_core[j];
    }
    C.div_r2min = p.div_rmin * p.div_rmin;
    C.div_r2min_f = static_cast<float>(C.div_r2min);
    C.div_rmin_ratio = p.div_rmin_ratio;
    C.div_radius = C.cell_sm ? p.div_r0 : 0.5 * p.rest0;
    C.act_noise = p.intra_law == CIL_INTRA_FENE && (p.noise_radial > 0.0 || p.noise_angular > 0.0) ? 1 : 0;
    C.dim = p.dim;
    C.swelling = C.cell_sm && p.div_swelling ? 1 : 0;
    if (C.cell_sm) h->any_cell_sm = true;
    if (C.swelling) h->any_swell = true;
    C.mig_mu_steps_f = static_cast<float>(p.mig_tau_mu / p.dt);
    C.mig_sd_steps_f = static_cast<float>(p.mig_tau_sigma / p.dt);
    C.noise_amp = p.noise_D > 0.0 ? std::sqrt(2.0 * p.noise_D) * (1.0 / std::sqrt(p.dt)) : 0.0;
    C.dt = p.dt;
    C.div_tau_mu = p.div_tau_mu;
    C.div_tau_sigma = p.div_tau_sigma;
    C.apop_p = p.apop_rate * p.dt;
    C.apop_log1m_p = static_cast<float>(std::log1p(-C.apop_p));
    C.tau_mu_steps_f = static_cast<float>(p.div_tau_mu / p.dt);
    C.tau_sd_steps_f = static_cast<float>(p.div_tau_sigma / p.dt);
    for (int j = 0; j < 2; ++j) {
      C.zeta_f[j] = static_cast<float>(C.zeta[j]);
      C.temp_f[j] = static_cast<float>(C.temp[j]);
      C.mu_f[j] = static_cast<float>(C.mu_eff[j]);
      C.motility_f[j] = static_cast<float>(C.motility[j]);
      C.wall_pos_f[j] = static_cast<float>(C.wall_pos[j]);
    }
    C.kappa_f = static_cast<float>(C.kappa);
    C.rest0_f = static_cast<float>(C.rest0);
    C.rest1_f = static_cast<float>(C.rest1);
    C.amp_f = static_cast<float>(C.noise_amp);
    C.eps_f = static_cast<float>(C.epsilon);
    C.rcs_f = static_cast<float>(C.rcut_scale);
    C.well_eps = p.force_law == CIL_FORCE_SC ? p.well_epsilon : 0.0;
    C.well_sigma = p.force_law == CIL_FORCE_SC ? p.well_sigma : 0.0;
    C.well_eps_f = static_cast<float>(C.well_eps);
    C.well_sigma_f = static_cast<float>(C.well_sigma);
    C.force_shifted = (p.force_law == CIL_FORCE_SC || p.force_law == CIL_FORCE_LJ_WCA) && p.force_shifted ? 1 : 0;
    C.wall_E_f = static_cast<float>(C.wall_E);
    C.due_base = static_cast<int>(due_acc);
    {
      long long p2 = 1;
      while (p2 < cap_cells[c]) p2 <<= 1;
      due_acc += p2;
    }
    cells += cap_cells[c];
    slots += C.slot_cap;
    if (cells > (1ll << 29) || slots > (1ll << 30)) {
      delete h;
      return CIL_ERR_CONFIG;
    }
  }
  if (cfg->skin > 0.0 && slots >= (1ll << kListSlotBits)) {
    // Verlet-list entries hold a slot index in kListSlotBits bits
    delete h;
    return CIL_ERR_CONFIG;
  }
  h->CC = static_cast<int>(cells);
  h->SS = static_cast<size_t>(slots);
  h->due_total = static_cast<size_t>(due_acc);
  h->obs_ready.assign(h->B, 0);

  cudaError_t e = cudaSetDevice(cfg->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess && cfg->skin > 0.0) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, cfg->device);
  if (e != cudaSuccess) {
    h->err = cudaGetErrorString(e);
    free_all(h);
    delete h;
    return CIL_ERR_CUDA;
  }
  const size_t SS = h->SS, D = h->D;
  h->d_col = dalloc<ColonyConst>(h->B);
  h->d_cnt = dalloc<ColonyCounters>(h->B);
  // pinned copy of the counters: the status read that ends every cil_step call
  if (!h->h_cnt && cudaHostAlloc(&h->h_cnt, 2 * sizeof(ColonyCounters) * h->B, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    h->h_cnt = nullptr;
  }
  const bool mixed = cfg->precision == CIL_PREC_MIXED;
  for (int b = 0; b < 2; ++b) {
    h->d_x[b] = dalloc<double>(D * SS);
    if (!mixed) h->d_sig[b] = dalloc<double>(SS);
    h->d_eid[b] = dalloc<int>(SS);
    h->d_sbin[b] = dalloc<int>(SS);
    h->d_cyc[b] = dalloc<int2>(SS);
    if (mixed) h->d_pk[b] = dalloc<float4>(SS);
  }
  h->d_sigma_c = dalloc<double>(2 * static_cast<size_t>(h->CC));
  h->d_ts = dalloc<int>(1);
  h->skin_mode = cfg->skin > 0.0;
  bool skin_ok = true;
  if (h->skin_mode) {
    for (int b = 0; b < 2; ++b) h->d_state[b] = dalloc<unsigned char>(SS);
    h->d_nbr = dalloc<int>(static_cast<size_t>(kListCap) * SS);
    h->d_ncnt = dalloc<int>(SS);
    h->d_lflat = dalloc<int>(static_cast<size_t>(kListCap) * SS);
    h->d_oflat = dalloc<unsigned char>(static_cast<size_t>(kListCap) * SS);
    h->d_lstart = dalloc<unsigned short>(SS);
    h->d_lwarp = dalloc<int>(SS / 64 + 1);
    h->d_spart = dalloc<StatPart>(static_cast<size_t>(h->B) * kStatSlots);
    h->d_uref = dalloc<float>(D * SS);
    h->d_facc = dalloc<float>(D * SS);
    h->d_ftouch = dalloc<unsigned>((SS + 31) / 32);
    h->d_fresh = dalloc<int>(static_cast<size_t>(h->B) * kFreshCap);
    h->d_fnext = dalloc<unsigned long long>(SS);
    h->d_anyreb = dalloc<int>(4);
    h->d_dueq = dalloc<int>(h->due_total);
    h->d_skin = dalloc<ColonySkin>(h->B);
    h->d_sched = dalloc<SchedState>(h->B);
    skin_ok = h->d_state[0] && h->d_state[1] && h->d_nbr && h->d_ncnt && h->d_uref && h->d_facc && h->d_ftouch &&
              h->d_dueq && h->d_spart && h->d_lflat && h->d_oflat && h->d_lstart && h->d_lwarp &&
              h->d_fresh &&
              h->d_fnext && h->d_anyreb && h->d_skin && h->d_sched;
  }
  h->d_vel = dalloc<double>(D * SS);
  // Heun without lists carries the first half step's velocities through the second re-sort;
  // allocated here so that a captured step never allocates
  if (h->cfg.integrator == CIL_INTEGRATOR_HEUN && !h->skin_mode && !h->d_vel2) h->d_vel2 = dalloc<double>(D * SS);
  h->d_key = dalloc<int>(SS);
  h->d_perm = dalloc<unsigned long long>(SS);
  h->d_slot_of = dalloc<int>(2 * static_cast<size_t>(h->CC));
  h->d_t0 = dalloc<int>(h->CC);
  h->d_tsw = dalloc<int>(h->CC);
  h->d_cst = dalloc<int>(h->CC);
  h->d_smflag = dalloc<unsigned char>(h->CC);
  h->d_tiles_used = dalloc<int>(h->B + 1);
  h->d_tiles_live = dalloc<int>(h->B + 1);
  h->d_tiles_cell = dalloc<int>(h->B + 1);
  h->d_tiles_pairs = dalloc<int>(h->B + 1);
  h->ctiles = 0;
  for (int c = 0; c < h->B; ++c) h->ctiles += (h->hc[c].cap + kTile - 1) / kTile;
  h->stiles = 0;
  for (int c = 0; c < h->B; ++c) h->stiles += (h->cc[c].slot_cap + kTile - 1) / kTile;
  // the list force kernel runs 128 threads per block unless asked otherwise (measured fastest
  // on the 2D growth colony and the 3D channel)
  h->cell_block = cfg->block_size ? cfg->block_size : 128;
  h->ptiles = 0;
  for (int c = 0; c < h->B; ++c) h->ptiles += (h->cc[c].slot_cap + 2 * h->cell_block - 1) / (2 * h->cell_block);
  h->d_tile_count = dalloc<int>(h->ctiles + 1);
  h->d_tile_off = dalloc<int>(h->ctiles + 1);
  h->d_upchk = dalloc<int>(4);
  h->d_evdone = dalloc<int>(1);
  h->d_dead = dalloc<int>(static_cast<size_t>(h->B) * kDeadCap);
  h->d_divq = dalloc<int>(static_cast<size_t>(h->CC));
  bool ok = h->d_col && h->d_cnt && h->d_x[0] && h->d_x[1] && h->d_eid[0] && h->d_eid[1] && h->d_sbin[0] &&
            h->d_sbin[1] && h->d_cyc[0] && h->d_cyc[1] && h->d_sigma_c && h->d_vel && h->d_key && h->d_perm &&
            h->d_slot_of && h->d_t0 && h->d_tsw && h->d_cst && h->d_smflag && h->d_tiles_used && h->d_tiles_live && h->d_tiles_cell &&
            h->d_tiles_pairs &&
            h->d_tile_count && h->d_tile_off && h->d_upchk && h->d_evdone && h->d_dead && h->d_divq && h->d_ts &&
            (mixed ? (h->d_pk[0] && h->d_pk[1]) : (h->d_sig[0] && h->d_sig[1])) &&
            skin_ok;
  if (ok && cfg->rng_mode == CIL_RNG_DSFMT) {
    const size_t nn = 2 * static_cast<size_t>(h->CC) * D + 2 * static_cast<size_t>(h->CC);  // passive, active
    h->d_noise = dalloc<double>(nn);
    ok = h->d_noise && cudaMallocHost(&h->h_noise, sizeof(double) * nn) == cudaSuccess;
    h->rng.seed(static_cast<uint32_t>(cfg->seed));
  }
  if (!ok) {
    h->err = "out of device memory";
    free_all(h);
    delete h;
    return CIL_ERR_CUDA;
  }
  cudaMemsetAsync(h->d_evdone, 0, sizeof(int), h->stream);
  // static parts of the colony table (bases, capacities, physics); the bin geometry is
  // filled in once every colony has been uploaded
  cudaMemcpyAsync(h->d_col, h->cc.data(), sizeof(ColonyConst) * h->B, cudaMemcpyHostToDevice, h->stream);
  cudaMemsetAsync(h->d_cnt, 0, sizeof(ColonyCounters) * h->B, h->stream);
  cudaMemsetAsync(h->d_ts, 0, sizeof(int), h->stream);
  cudaMemsetAsync(h->d_vel, 0, sizeof(double) * D * SS, h->stream);
  cudaMemsetAsync(h->d_eid[0], 0xff, sizeof(int) * SS, h->stream);
  cudaMemsetAsync(h->d_eid[1], 0xff, sizeof(int) * SS, h->stream);
  cudaMemsetAsync(h->d_key, 0xff, sizeof(int) * SS, h->stream);
  if (h->skin_mode) {
    std::vector<ColonySkin> sk(h->B);
    for (auto &k : sk) {
      std::memset(&k, 0, sizeof k);
      k.skin = static_cast<float>(cfg->skin);
      k.half2 = static_cast<float>(0.25 * cfg->skin * cfg->skin);
      k.need = 8;
    }
    cudaMemcpy(h->d_skin, sk.data(), sizeof(ColonySkin) * h->B, cudaMemcpyHostToDevice);
    cudaMemsetAsync(h->d_sched, 0, sizeof(SchedState) * h->B, h->stream);
    cudaMemsetAsync(h->d_anyreb, 0, 4 * sizeof(int), h->stream);
    cudaMemsetAsync(h->d_facc, 0, sizeof(float) * D * SS, h->stream);
    cudaMemsetAsync(h->d_ftouch, 0, sizeof(unsigned) * ((SS + 31) / 32), h->stream);
    cudaMemsetAsync(h->d_ncnt, 0, sizeof(int) * SS, h->stream);
    // flattened lists: every entry a valid slot and every count 0 before the first build
    cudaMemsetAsync(h->d_lflat, 0, sizeof(int) * kListCap * SS, h->stream);
    cudaMemsetAsync(h->d_oflat, 0, static_cast<size_t>(kListCap) * SS, h->stream);
    cudaMemsetAsync(h->d_lstart, 0, sizeof(unsigned short) * SS, h->stream);
    cudaMemsetAsync(h->d_lwarp, 0, sizeof(int) * (SS / 64 + 1), h->stream);
    cudaMemsetAsync(h->d_spart, 0, sizeof(StatPart) * h->B * kStatSlots, h->stream);
    cudaMemsetAsync(h->d_state[0], kSlotDead, SS, h->stream);
    cudaMemsetAsync(h->d_state[1], kSlotDead, SS, h->stream);
  }
  h->grid_slots = std::max(1, std::min(h->nsm * 8, static_cast<int>((SS + kTile - 1) / kTile)));
  h->grid_cells = std::max(1, std::min(h->nsm * 8, h->ctiles));
  h->grid_force = h->grid_slots;
  {
    // the upload and download staging, sized for the largest colony here rather than at the
    // first upload (an allocation would otherwise sit inside the first cil_upload)
    size_t need = 0;
    for (int c = 0; c < h->B; ++c) {
      const size_t ne = 2 * static_cast<size_t>(h->hc[c].cap);
      need = std::max(need, std::max(ne * D + ne + ne / 2 + 1, ne * 2 * D));
    }
    if (ensure_stage(h, need) != CIL_OK) {
      h->err = "out of device memory (staging)";
      free_all(h);
      delete h;
      return CIL_ERR_CUDA;
    }
  }
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    h->err = "initialisation failed";
    free_all(h);
    delete h;
    return CIL_ERR_CUDA;
  }
  *out = h;
  return CIL_OK;
}

void cil_destroy(cil_handle *h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
}

cil_status cil_upload(cil_handle *h, int32_t colony, const cil_colony_view *v) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !v || !v->pos || !v->sigma || !v->t0 || !v->tswitch)
    return fail(h, CIL_ERR_CONFIG, "cil_upload: bad arguments");
  HostColony &hc = h->hc[colony];
  const int n = v->ncells;
  if (n < 0 || n > hc.cap) return fail(h, CIL_ERR_CAPACITY, "cil_upload: more cells than the capacity");
  CUDA_TRY(h, cudaSetDevice(h->cfg.device));
  const int D = h->D;
  const ColonyConst &C = h->cc[colony];
  // everything is staged and checked on the device (diameters positive and finite, positions
  // finite and inside the box, CIL.cuh:54-66) before any of the colony's arrays is written, so a
  // refused upload changes nothing
  const size_t ne = 2 * static_cast<size_t>(n);
  const cil_status sst = ensure_stage(h, ne * D + ne + static_cast<size_t>(n) + 1);
  if (sst != CIL_OK) return sst;
  double *st_pos = h->d_stage, *st_sig = h->d_stage + ne * D;
  int *st_t0 = reinterpret_cast<int *>(st_sig + ne), *st_tsw = st_t0 + n;
  CUDA_TRY(h, cudaMemcpyAsync(st_pos, v->pos, sizeof(double) * ne * D, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(st_sig, v->sigma, sizeof(double) * ne, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(st_t0, v->t0, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(st_tsw, v->tswitch, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemsetAsync(h->d_upchk, 0, 4 * sizeof(int), h->stream));
  launch_upload(h->d_col, colony, n, D, h->SS, h->d_stage, h->d_x[h->cur], h->d_sigma_c, h->d_t0, h->d_tsw,
                h->d_vel, h->d_eid[h->meta], h->d_slot_of, h->d_cnt, h->d_upchk, h->stream);
  CUDA_TRY(h, cudaGetLastError());
  int chk[4] = {0, 0, 0, 0};
  CUDA_TRY(h, cudaMemcpyAsync(chk, h->d_upchk, sizeof chk, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (chk[0] & 1) return fail(h, CIL_ERR_CONFIG, "cil_upload: diameters must be positive");
  if (chk[0] & 2) return fail(h, CIL_ERR_OUT_OF_BOX, "cil_upload: position outside the box (CIL.cuh:54-66)");
  double smax = 0.0;
  std::memcpy(&smax, chk + 2, sizeof smax);
  hc.uploaded = true;
  hc.sigma_max = smax;
  hc.n = n;
  if (h->cfg.rng_mode == CIL_RNG_DSFMT) {  // the oracle mode's host mirror of the cycles
    hc.t0.assign(v->t0, v->t0 + n);
    hc.tsw.assign(v->tswitch, v->tswitch + n);
    hc.t0.resize(hc.cap);
    hc.tsw.resize(hc.cap);
    if (v->cell_state)
      hc.cst.assign(v->cell_state, v->cell_state + n);
    else
      hc.cst.assign(n, 2);
    hc.cst.resize(hc.cap, 2);
  }
  // cell states: given, or every cell undefined (CellState::Undefined, Colony.cpp:248)
  if (v->cell_state) {
    CUDA_TRY(h, cudaMemcpyAsync(h->d_cst + C.cell_base, v->cell_state, sizeof(int) * n, cudaMemcpyHostToDevice,
                                h->stream));
  } else if (n > 0) {
    launch_fill_int(h->d_cst + C.cell_base, n, 2, h->stream);
  }
  h->ts = v->ts;
  const int tsi = static_cast<int>(v->ts);
  CUDA_TRY(h, cudaMemcpyAsync(h->d_ts, &tsi, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  h->obs_ready[colony] = 0;
  h->geometry_ready = false;
  h->need_exact = true;
  // the scheduler's statistics restart with the new state
  if (h->skin_mode) CUDA_TRY(h, cudaMemsetAsync(h->d_sched + colony, 0, sizeof(SchedState), h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return CIL_OK;
}

cil_status cil_step(cil_handle *h, int32_t nsteps, int64_t *ts_out) {
  if (!h) return CIL_ERR_CONFIG;
  if (nsteps < 0) return fail(h, CIL_ERR_CONFIG, "cil_step: negative step count");
  cil_status st = ensure_ready(h);
  if (st != CIL_OK) return st;
  h->t_rebuild = h->t_force = h->t_events = 0.0;
  h->launches = 0;
  h->graph_steps = 0;
  if (h->skin_mode) CUDA_TRY(h, cudaMemsetAsync(h->d_anyreb + 3, 0, sizeof(int), h->stream));
  std::vector<char> seg_graph;  // per segment of 4 events: 1 = a graph of two steps
  int k = 0;
  while (k < nsteps) {
    const size_t e0 = 4 * seg_graph.size();
    // steady steps replay a captured graph: two at a time, or one (the call's last step,
    // which writes the velocities, or a step followed by a re-sort)
    if (!h->graphs_off && steady_step(h, h->ts)) {
      const int n = (k + 2 <= nsteps && steady_step(h, h->ts + 1)) ? 2 : 1;
      int64_t nl = 0;
      cudaGraphExec_t ex = steady_graph(h, n, k + n == nsteps, &nl);
      if (ex) {
        CUDA_TRY(h, cudaEventRecord(pool_event(h, e0), h->stream));
        CUDA_TRY(h, cudaGraphLaunch(ex, h->stream));
        CUDA_TRY(h, cudaEventRecord(pool_event(h, e0 + 3), h->stream));
        seg_graph.push_back(1);
        h->launches += nl;
        h->graph_steps += n;
        k += n;
        continue;
      }
    }
    st = enqueue_step(h, k == nsteps - 1, true, e0);
    if (st != CIL_OK) return st;
    seg_graph.push_back(0);
    k += 1;
  }
  if ((h->cfg.flags & CIL_FLAG_DEFERRED_STATUS) && h->h_cnt) {
    // the previous call's status; this call's counters are copied behind its launches
    for (auto &e : h->cnt_ev)
      if (!e) CUDA_TRY(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const int slot = h->cnt_slot;
    ColonyCounters *dst = h->h_cnt + static_cast<size_t>(slot) * h->B;
    CUDA_TRY(h, cudaMemcpyAsync(dst, h->d_cnt, sizeof(ColonyCounters) * h->B, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaEventRecord(h->cnt_ev[slot], h->stream));
    cil_status prev = CIL_OK;
    if (h->cnt_pending >= 0) {
      CUDA_TRY(h, cudaEventSynchronize(h->cnt_ev[h->cnt_pending]));
      prev = counter_status(h, h->h_cnt + static_cast<size_t>(h->cnt_pending) * h->B);
    }
    h->cnt_pending = slot;
    h->cnt_slot = 1 - slot;
    if (ts_out) *ts_out = h->ts;
    return prev;
  }
  if (h->h_cnt)
    CUDA_TRY(h, cudaMemcpyAsync(h->h_cnt, h->d_cnt, sizeof(ColonyCounters) * h->B, cudaMemcpyDeviceToHost,
                                h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  h->t_total = 0.0;
  const size_t nseg = seg_graph.size();
  if (nseg > 0) {
    float t = 0;
    cudaEventElapsedTime(&t, h->evpool[0], h->evpool[4 * (nseg - 1) + 3]);
    h->t_total = t;
  }
  for (size_t q = 0; q < nseg; ++q) {
    if (seg_graph[q]) continue;
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, h->evpool[4 * q], h->evpool[4 * q + 1]);
    cudaEventElapsedTime(&b, h->evpool[4 * q + 1], h->evpool[4 * q + 2]);
    cudaEventElapsedTime(&c, h->evpool[4 * q + 2], h->evpool[4 * q + 3]);
    h->t_rebuild += a;
    h->t_force += b;
    h->t_events += c;
  }
  if (ts_out) *ts_out = h->ts;
  return h->h_cnt ? counter_status(h, h->h_cnt) : check_counters(h);
}

cil_status cil_forces(cil_handle *h, int32_t colony, double *frc) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !frc) return fail(h, CIL_ERR_CONFIG, "cil_forces: bad arguments");
  cil_status st = ensure_ready(h);
  if (st != CIL_OK) return st;
  const bool oracle = h->cfg.rng_mode == CIL_RNG_DSFMT;
  bool noise = false;
  if (oracle) {
    // the noise the next step will draw: the host stream is put back after the draw, so that
    // reading the forces leaves the run unchanged
    const HostRng saved = h->rng;
    st = draw_oracle_noise(h, &noise);
    h->rng = saved;
    if (st != CIL_OK) return st;
  } else {
    for (int c = 0; c < h->B; ++c) noise = noise || h->hc[c].p.noise_D > 0.0;
  }
  if (!h->d_frc) {
    h->d_frc = dalloc<double>(h->D * h->SS);
    if (!h->d_frc) return fail(h, CIL_ERR_CUDA, "out of device memory (forces)");
  }
  st = do_rebuild(h, true, true);
  if (st != CIL_OK) return st;
  ForceArgs fa = force_args(h, noise ? (oracle ? 2 : 1) : 0, 0, nullptr, h->d_frc);
  launch_force(fa, h->D, h->cfg.force_law, h->cfg.precision, h->grid_force, kTile, h->stream);
  std::vector<ColonyCounters> k;
  st = check_counters(h, &k);
  if (st != CIL_OK && st != CIL_ERR_NAN) return st;
  const int n = k[colony].ncell;
  const ColonyConst &C = h->cc[colony];
  const cil_status sst = ensure_stage(h, static_cast<size_t>(2 * n) * h->D);
  if (sst != CIL_OK) return sst;
  launch_gather_canonical(n, h->D, h->SS, C.cell_base, h->d_slot_of, h->d_frc, h->D, h->d_stage, h->stream);
  CUDA_TRY(h, cudaMemcpyAsync(frc, h->d_stage, sizeof(double) * 2 * n * h->D, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return st;
}

cil_status cil_bins(cil_handle *h, int32_t colony, int32_t *ns, int32_t *bin_start, int32_t *elems,
                    int32_t max_bins) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !ns || !bin_start || !elems)
    return fail(h, CIL_ERR_CONFIG, "cil_bins: bad arguments");
  cil_status st = ensure_ready(h);
  if (st != CIL_OK) return st;
  const ColonyConst &C = h->cc[colony];
  for (int d = 0; d < 3; ++d) ns[d] = C.ns[d];
  if (C.nbins > max_bins) return fail(h, CIL_ERR_CAPACITY, "cil_bins: max_bins too small");
  st = do_rebuild(h, true, true);
  if (st != CIL_OK) return st;
  std::vector<ColonyCounters> k;
  st = check_counters(h, &k);
  if (st != CIL_OK) return st;
  std::vector<int2> r(C.nbins);
  const int nlive = k[colony].nlive;
  std::vector<int> e(std::max(nlive, 1));
  CUDA_TRY(h, cudaMemcpyAsync(r.data(), h->d_range + C.bin_base, sizeof(int2) * C.nbins, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(e.data(), h->d_eid[h->meta] + C.slot_base, sizeof(int) * nlive, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  for (int b = 0; b < C.nbins; ++b) bin_start[b] = r[b].x - C.slot_base;
  bin_start[C.nbins] = nlive;
  for (int i = 0; i < nlive; ++i) elems[i] = e[i] - 2 * C.cell_base;
  return CIL_OK;
}

cil_status cil_download(cil_handle *h, int32_t colony, cil_colony_view *v) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !v) return fail(h, CIL_ERR_CONFIG, "cil_download: bad arguments");
  cil_status st = ensure_ready(h);
  if (st != CIL_OK) return st;
  std::vector<ColonyCounters> k;
  st = check_counters(h, &k);
  const int n = k[colony].ncell;
  v->ts = static_cast<int32_t>(h->ts);
  if (n > v->capacity) {
    v->ncells = n;
    return fail(h, CIL_ERR_CAPACITY, "cil_download: host arrays too small");
  }
  v->ncells = n;
  const ColonyConst &C = h->cc[colony];
  const int D = h->D;
  const cil_status sst = ensure_stage(h, static_cast<size_t>(2 * n) * (2 * D));
  if (sst != CIL_OK) return sst;
  double *sp = h->d_stage, *sv = h->d_stage + 2 * n * D;
  launch_gather_canonical(n, D, h->SS, C.cell_base, h->d_slot_of, h->d_x[h->cur], D, sp, h->stream);
  launch_gather_canonical(n, D, h->SS, C.cell_base, h->d_slot_of, h->d_vel, D, sv, h->stream);
  if (v->pos) CUDA_TRY(h, cudaMemcpyAsync(v->pos, sp, sizeof(double) * 2 * n * D, cudaMemcpyDeviceToHost, h->stream));
  if (v->sigma)
    CUDA_TRY(h, cudaMemcpyAsync(v->sigma, h->d_sigma_c + 2 * static_cast<size_t>(C.cell_base), sizeof(double) * 2 * n,
                                cudaMemcpyDeviceToHost, h->stream));
  if (v->vel) CUDA_TRY(h, cudaMemcpyAsync(v->vel, sv, sizeof(double) * 2 * n * D, cudaMemcpyDeviceToHost, h->stream));
  if (v->t0) CUDA_TRY(h, cudaMemcpyAsync(v->t0, h->d_t0 + C.cell_base, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  if (v->tswitch) CUDA_TRY(h, cudaMemcpyAsync(v->tswitch, h->d_tsw + C.cell_base, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  if (v->cell_state)
    CUDA_TRY(h, cudaMemcpyAsync(v->cell_state, h->d_cst + C.cell_base, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return st;
}

}  // extern "C"

cil_status cil::frame_source(cil_handle *h, int colony, FrameSource *out) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !out) return fail(h, CIL_ERR_CONFIG, "frame_source: bad arguments");
  cil_status st = ensure_ready(h);
  if (st != CIL_OK) return st;
  std::vector<ColonyCounters> k;
  st = check_counters(h, &k);
  if (st != CIL_OK) return st;
  const ColonyConst &C = h->cc[colony];
  const HostColony &hc = h->hc[colony];
  FrameSource s{};
  s.x = h->d_x[h->cur];
  s.vel = h->d_vel;
  s.slot_of = h->d_slot_of;
  s.sigma_c = h->d_sigma_c;
  s.SS = h->SS;
  s.cell_base = C.cell_base;
  s.ncells = k[colony].ncell;
  s.dim = h->D;
  s.divide = hc.p.divide;
  s.dying = hc.p.apop_rate > 0.0;
  for (int d = 0; d < 3; ++d) s.box[d] = hc.p.box[d];
  s.sigma_max = hc.sigma_max;
  s.ts = h->ts;
  s.device = h->cfg.device;
  s.capacity = hc.cap;
  s.stream = h->stream;
  *out = s;
  return CIL_OK;
}

cil_status cil::frame_layout(cil_handle *h, int colony, FrameSource *out) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !out) return fail(h, CIL_ERR_CONFIG, "frame_layout: bad arguments");
  const HostColony &hc = h->hc[colony];
  FrameSource s{};
  s.dim = h->D;
  s.divide = hc.p.divide;
  s.dying = hc.p.apop_rate > 0.0;
  for (int d = 0; d < 3; ++d) s.box[d] = hc.p.box[d];
  s.device = h->cfg.device;
  s.capacity = hc.cap;
  s.stream = h->stream;
  *out = s;
  return CIL_OK;
}

extern "C" {

static cil_status run_obs(cil_handle *h, int32_t colony, int reset, cil_obs *out) {
  cil_status st = ensure_ready(h);
  if (st != CIL_OK) return st;
  if (!h->d_obs) {
    h->d_obs = dalloc<double>(3 * static_cast<size_t>(h->D) * h->CC);
    if (!h->d_obs) return fail(h, CIL_ERR_CUDA, "out of device memory (observables)");
    CUDA_TRY(h, cudaMemsetAsync(h->d_obs, 0, sizeof(double) * 3 * h->D * h->CC, h->stream));
    h->graph_gen += 1;  // captured steps hold the event arguments without the observable arrays
  }
  std::vector<ColonyCounters> k;
  st = check_counters(h, &k);
  const int n = k[colony].ncell;
  const int nblocks = std::max(1, (n + kTile - 1) / kTile);
  if (nblocks * 4 > h->partials_cap) {
    cudaFree(h->d_partials);
    h->partials_cap = nblocks * 4;
    h->d_partials = dalloc<double>(h->partials_cap);
    if (!h->d_partials) return fail(h, CIL_ERR_CUDA, "out of device memory (partials)");
  }
  if (!reset && !h->obs_ready[colony]) {
    EventArgs a = event_args(h);
    launch_observables(a, colony, n, h->D, 1, h->d_partials, nblocks, h->stream);
  }
  EventArgs a = event_args(h);
  launch_observables(a, colony, n, h->D, reset, h->d_partials, nblocks, h->stream);
  h->obs_ready[colony] = 1;
  std::vector<double> part(static_cast<size_t>(nblocks) * 4);
  CUDA_TRY(h, cudaMemcpyAsync(part.data(), h->d_partials, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (out) {
    double s[4] = {0, 0, 0, 0};
    for (int b = 0; b < nblocks; ++b)
      for (int q = 0; q < 4; ++q) s[q] += part[static_cast<size_t>(b) * 4 + q];
    out->ncells = n;
    out->pad = 0;
    out->mean_area = n ? s[0] / n : 0.0;
    out->msd = n ? s[1] / n : 0.0;
    out->vacf = s[3] > 0.0 ? s[2] / s[3] : 0.0;
    out->ndiv_total = k[colony].ndiv_total;
    out->napo_total = k[colony].napo_total;
  }
  return st;
}

cil_status cil_obs_reset(cil_handle *h, int32_t colony) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B) return fail(h, CIL_ERR_CONFIG, "cil_obs_reset: bad colony");
  return run_obs(h, colony, 1, nullptr);
}

cil_status cil_observables(cil_handle *h, int32_t colony, cil_obs *out) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !out) return fail(h, CIL_ERR_CONFIG, "cil_observables: bad arguments");
  return run_obs(h, colony, 0, out);
}

cil_status cil_skin_stats(cil_handle *h, int32_t colony, cil_skin_info *out) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !out) return fail(h, CIL_ERR_CONFIG, "cil_skin_stats: bad arguments");
  if (!h->skin_mode) return fail(h, CIL_ERR_CONFIG, "cil_skin_stats: the handle has no skin");
  ColonySkin k;
  StatPart part[kStatSlots];
  CUDA_TRY(h, cudaMemcpyAsync(&k, h->d_skin + colony, sizeof k, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(part, h->d_spart + static_cast<size_t>(colony) * kStatSlots, sizeof part,
                              cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  // the largest displacement of the last force pass: its statistics slots (folded and cleared
  // at the start of the next step)
  unsigned bits = k.maxdisp2;
  for (const StatPart &q : part) bits = q.dmax > bits ? q.dmax : bits;
  float md2;
  std::memcpy(&md2, &bits, sizeof md2);
  out->skin = k.skin;
  out->interval = k.interval;
  out->nrebuild = k.nrebuild;
  out->ntrip = k.ntrip;
  out->last_interval = k.last_interval;
  out->nfresh = k.nfresh;
  out->list_overflow = k.list_overflow;
  out->npairs = k.npairs;
  out->max_disp = std::sqrt(static_cast<double>(md2));
  return CIL_OK;
}

cil_status cil_set_skin(cil_handle *h, int32_t colony, double skin, int32_t interval) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !h->skin_mode || !(skin > 0.0) || skin > h->cfg.skin || interval < 0)
    return fail(h, CIL_ERR_CONFIG, "cil_set_skin: bad arguments");
  CUDA_TRY(h, cudaSetDevice(h->cfg.device));
  ColonySkin k;
  CUDA_TRY(h, cudaMemcpyAsync(&k, h->d_skin + colony, sizeof k, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  k.skin = static_cast<float>(skin);
  k.half2 = static_cast<float>(0.25 * skin * skin);
  k.interval = interval;
  k.need |= 8;
  CUDA_TRY(h, cudaMemcpyAsync(h->d_skin + colony, &k, sizeof k, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return CIL_OK;
}

cil_status cil_set_scheduler(cil_handle *h, const float *params, double skin_min, double interval_scale,
                             int32_t use_interval) {
  if (!h) return CIL_ERR_CONFIG;
  if (!h->skin_mode) return fail(h, CIL_ERR_CONFIG, "cil_set_scheduler: the handle has no skin");
  CUDA_TRY(h, cudaSetDevice(h->cfg.device));
  if (!params) {
    if (h->d_mlp) cudaFree(h->d_mlp);
    h->d_mlp = nullptr;
    h->graph_gen += 1;
    return CIL_OK;
  }
  if (!(skin_min > 0.0) || skin_min > h->cfg.skin || !(interval_scale >= 1.0) || !std::isfinite(interval_scale))
    return fail(h, CIL_ERR_CONFIG, "cil_set_scheduler: need 0 < skin_min <= skin and interval_scale >= 1");
  const int np = mlp_param_count();
  for (int i = 0; i < np; ++i)
    if (!std::isfinite(params[i])) return fail(h, CIL_ERR_CONFIG, "cil_set_scheduler: non-finite parameter");
  if (!h->d_mlp) {
    h->d_mlp = dalloc<float>(np);
    if (!h->d_mlp) return fail(h, CIL_ERR_CUDA, "cil_set_scheduler: out of device memory");
  }
  CUDA_TRY(h, cudaMemcpyAsync(h->d_mlp, params, sizeof(float) * np, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  h->graph_gen += 1;  // the scheduler launch is part of a captured step
  h->sched_skin_min = static_cast<float>(skin_min);
  h->sched_interval_scale = static_cast<float>(interval_scale);
  h->sched_use_interval = use_interval ? 1 : 0;
  return CIL_OK;
}

cil_status cil_sched_state(cil_handle *h, int32_t colony, cil_sched_info *out) {
  if (!h) return CIL_ERR_CONFIG;
  if (colony < 0 || colony >= h->B || !out) return fail(h, CIL_ERR_CONFIG, "cil_sched_state: bad arguments");
  if (!h->skin_mode) return fail(h, CIL_ERR_CONFIG, "cil_sched_state: the handle has no skin");
  CUDA_TRY(h, cudaSetDevice(h->cfg.device));
  SchedState q;
  CUDA_TRY(h, cudaMemcpyAsync(&q, h->d_sched + colony, sizeof q, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  static_assert(kSchedFeatures == CIL_SCHED_FEATURES, "feature count");
  for (int k = 0; k < kSchedFeatures; ++k) out->features[k] = q.features[k];
  out->div_rate = q.div_rate;
  out->apo_rate = q.apo_rate;
  out->trip_share = q.trip_share;
  out->nsched = q.nsched;
  return CIL_OK;
}

cil_status cil_graph_info(cil_handle *h, int64_t *graph_steps, int64_t *graphs_captured) {
  if (!h) return CIL_ERR_CONFIG;
  if (graph_steps) *graph_steps = h->graph_steps;
  if (graphs_captured) *graphs_captured = h->graphs_captured;
  return CIL_OK;
}

cil_status cil_timings(cil_handle *h, double *rebuild_ms, double *force_ms, double *events_ms,
                       double *total_ms, int64_t *launches) {
  if (!h) return CIL_ERR_CONFIG;
  if (rebuild_ms) *rebuild_ms = h->t_rebuild;
  if (force_ms) *force_ms = h->t_force;
  if (events_ms) *events_ms = h->t_events;
  if (total_ms) *total_ms = h->t_total;
  if (launches) {
    // plus the seven kernels of every rebuild node that ran in the last cil_step call
    int runs = 0;
    if (h->skin_mode) {
      CUDA_TRY(h, cudaMemcpyAsync(&runs, h->d_anyreb + 3, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
      CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    }
    *launches = h->launches + 7 * static_cast<int64_t>(runs);
  }
  return CIL_OK;
}

}  // extern "C"
