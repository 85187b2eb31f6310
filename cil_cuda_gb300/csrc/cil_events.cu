// Division, apoptosis, state transfer and observables on the device.
//
// Division (calculDivisions, CIL.cu:369-455, with the linear-growth model: a cell
// divides when its cycle ends, ts == tswitch): due cells are ranked by a deterministic
// per-colony scan in slot order, the daughter takes cell index ncell + rank (addCell
// appends, Colony.cpp:355-359) and both cells are re-placed as binaryCellDivision does
// (MD.cu:721-731): mother centred on her old front element, daughter on the old back
// element, each with half-separation rest0/2 along a random axis.
//
// Apoptosis (calculApoptosis, CIL.cu:627-649): Philox mode draws one uniform per cell per
// step; removals are applied as swap-with-last (removeCell, Colony.cpp:365-399), pairing
// the holes below the new count with the surviving tail cells in ascending order. Oracle
// mode replays the host's sequential removal list exactly.
//
// Element storage is binned: a removed cell's element slots become tombstones (eid -1)
// until the next rebuild; a moved cell keeps its slots and only its ids change.
#include "cil_internal.cuh"

namespace cil {

namespace {

__device__ __forceinline__ int block_excl_scan_ev(int v, int *total) {
  __shared__ int ws[kTile / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kTile / 32 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < kTile / 32) ws[lane] = w;
  }
  __syncthreads();
  const int base = wid > 0 ? ws[wid - 1] : 0;
  *total = ws[kTile / 32 - 1];
  __syncthreads();
  return base + inc - v;
}

template <int D>
__device__ __forceinline__ void place(const ColonyConst &C, const double *master, const double *dir,
                                      double radius, double *m_out, double *s_out) {
  // binaryRandomReorientation (MD.cu:650-656): slave = master; master += r dir;
  // slave -= r dir; both through BoundingBox::updatePos(r, v, dt) (Utils.hpp:561-566)
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double a = __dadd_rn(master[d], __dmul_rn(radius, dir[d]));
    const double b = __dadd_rn(master[d], __dmul_rn(-radius, dir[d]));
    m_out[d] = C.periodic[d] ? wrap_like_fmod(a, C.box[d]) : a;
    s_out[d] = C.periodic[d] ? wrap_like_fmod(b, C.box[d]) : b;
  }
}

// Division of cell i into i (mother, its slots sb, sf) and k (daughter, new slots s0, s0+1):
// binaryCellDivision (MD.cu:721-731) placement in FP64, then every output of the four
// elements written once. All loads are issued before the first store, and each record is
// formed in registers (no store-then-reload), so the per-division chain of memory round trips
// stays short. In skin mode the four slots become fresh: one atomic reserves their entries
// in the colony's fresh set, and each joins the fresh list of its bin. The lists carry the
// colony's rebuild count as an epoch, so a list rebuild empties them without touching
// memory; a slot that was already fresh (moved twice before a rebuild) would sit in the list
// of its old bin, so the colony rebuilds at the next step instead.
template <int D>
__device__ void divide_cell(const EventArgs &a, const ColonyConst &C, int c, int i, int k,
                            const double *dir_m, const double *dir_d, int tsw_d, int tsw_m,
                            int nslot0, int rank) {
  const size_t SS = a.SS;
  const int g = C.cell_base + i, gk = C.cell_base + k;
  const int sb = a.slot_of[2 * g], sf = a.slot_of[2 * g + 1];
  const int s0 = C.slot_base + nslot0 + 2 * rank;
  const int slots[4] = {sb, sf, s0, s0 + 1};
  // ---- loads
  double xb[D], xf[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    xb[d] = a.x[d * SS + sb];
    xf[d] = a.x[d * SS + sf];
  }
  double sgb = a.sigma_c[2 * g], sgf = a.sigma_c[2 * g + 1];
  double sigb = 0.0, sigf = 0.0;
  if (a.sig) {
    sigb = a.sig[sb];
    sigf = a.sig[sf];
  }
  float wb = 0.0f, wf = 0.0f;
  if (a.pk) {
    wb = fabsf(a.pk[sb].w);
    wf = fabsf(a.pk[sf].w);
  }
  if (C.cell_sm) {  // crawling/dividing cells: both cells' diameters return to SIGMA_CORE (CIL.cu:408, 427)
    sgb = sigb = C.sigma_core[0];
    sgf = sigf = C.sigma_core[1];
    wb = static_cast<float>(sgb);
    wf = static_cast<float>(sgf);
  }
  const bool skin = a.state != nullptr;
  bool was_fresh_b = false, was_fresh_f = false;
  if (skin) {
    was_fresh_b = a.state[sb] == kSlotFresh;
    was_fresh_f = a.state[sf] == kSlotFresh;
  }
  double ocp[D], odi[D], ovr[D];
  if (a.obs_disp) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      ocp[d] = a.obs_com_prev[d * a.CC + g];
      odi[d] = a.obs_disp[d * a.CC + g];
      ovr[d] = a.obs_vref[d * a.CC + g];
    }
  }
  // ---- placement (FP64), bins and records
  const double radius = C.div_radius;  // half the birth rest length, or the reference's R0
  double xs[4][D];
  place<D>(C, xf, dir_m, radius, xs[1], xs[0]);  // mother: master = front element
  place<D>(C, xb, dir_d, radius, xs[2], xs[3]);  // daughter: master = back element
  int bins[4];
  float4 rec[4];
  const float wsign = skin ? -1.0f : 1.0f;  // fresh elements are skipped by the lists
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int b[D];
    bin_coords<D>(C, xs[q], b);
    bins[q] = bin_id<D>(C, b);
    rec[q] = make_float4(0.0f, 0.0f, 0.0f, wsign * ((q & 1) ? wf : wb));
#pragma unroll
    for (int d = 0; d < D; ++d) pk_set(rec[q], d, static_cast<float>(xs[q][d] - static_cast<double>(b[d]) * C.bw[d]));
  }
  // ---- fresh-set entries and per-bin fresh lists (skin mode)
  if (skin) {
    ColonySkin &S = a.skin[c];
    const bool push[4] = {!was_fresh_b, !was_fresh_f, true, true};
    const int npush = 2 + (was_fresh_b ? 0 : 1) + (was_fresh_f ? 0 : 1);
    if (was_fresh_b || was_fresh_f) atomicOr(&S.need, 2);
    const int idx0 = atomicAdd(&S.nfresh, npush);
    const unsigned epoch = static_cast<unsigned>(S.nrebuild);
    unsigned long long prev[4];
    bool listed[4];
    int idx = idx0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      listed[q] = push[q] && idx < kFreshCap;
      if (push[q]) {
        if (listed[q]) {
          a.fresh[c * kFreshCap + idx] = slots[q];
          const unsigned long long ent =
              (static_cast<unsigned long long>(epoch) << 32) | static_cast<unsigned>(slots[q]);
          prev[q] = atomicExch(&a.fhead[C.bin_base + bins[q]], ent);
        }
        ++idx;
      }
    }
    if (idx > kFreshCap) atomicOr(&S.need, 2);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (listed[q]) a.fnext[slots[q]] = prev[q];
      a.state[slots[q]] = kSlotFresh;
      a.ncnt[slots[q]] = 0;
      if (D == 2) {
        rec[q].z = uref_pack2(C.uq_scale, rec[q].x, rec[q].y);  // list reference in the record
      } else {
#pragma unroll
        for (int d = 0; d < D; ++d) a.uref[d * SS + slots[q]] = pk_c(rec[q], d);
      }
    }
  }
  // ---- stores
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int d = 0; d < D; ++d) a.x[d * SS + slots[q]] = xs[q][d];
    a.sbin[slots[q]] = bins[q];
    if (a.pk) a.pk[slots[q]] = rec[q];
    a.cyc[slots[q]] = make_int2(a.ts, q < 2 ? tsw_m : tsw_d);
    if (a.vel) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.vel[d * SS + slots[q]] = 0.0;
    }
  }
  // daughter diameters copied from the mother (canonical and binned copies)
  a.sigma_c[2 * gk] = sgb;
  a.sigma_c[2 * gk + 1] = sgf;
  if (a.sig) {
    a.sig[s0] = sigb;
    a.sig[s0 + 1] = sigf;
  }
  if (C.cell_sm) {  // the mother's reset diameters
    a.sigma_c[2 * g] = sgb;
    a.sigma_c[2 * g + 1] = sgf;
    if (a.sig) {
      a.sig[sb] = sigb;
      a.sig[sf] = sigf;
    }
  }
  // both cells crawl after a division (CIL.cu:403, 425)
  a.cst[g] = kCellCrawling;
  a.cst[gk] = kCellCrawling;
  a.eid[s0] = 2 * gk;
  a.eid[s0 + 1] = 2 * gk + 1;
  a.slot_of[2 * gk] = s0;
  a.slot_of[2 * gk + 1] = s0 + 1;
  a.t0[g] = a.ts;
  a.t0[gk] = a.ts;
  a.tsw[gk] = tsw_d;
  a.tsw[g] = tsw_m;
  if (a.obs_disp) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      a.obs_com_prev[d * a.CC + gk] = ocp[d];
      a.obs_disp[d * a.CC + gk] = odi[d];
      a.obs_vref[d * a.CC + gk] = ovr[d];
    }
  }
}

// random axis and cycle length of a division in Philox mode (i: the mother's colony-local index;
// the colony's stream in the fourth counter word)
template <int D>
__device__ void division_draws(const EventArgs &a, int i, double *dir_m, double *dir_d,
                               int &span_d, int &span_m, const ColonyConst &C) {
  // fast mode: FP32 draws (the FP64 placement arithmetic stays in place / divide_cell); the
  // axes are FP32 unit vectors widened exactly to FP64
  const u32x4 r1 = philox4x32_10(static_cast<uint32_t>(i), static_cast<uint32_t>(a.ts), kRngDiv, C.rng_stream,
                                 a.seed_lo, a.seed_hi);
  const u32x4 r2 = philox4x32_10(static_cast<uint32_t>(i), static_cast<uint32_t>(a.ts), kRngDiv2, C.rng_stream,
                                 a.seed_lo, a.seed_hi);
  const float k24 = 5.9604644775390625e-08f;  // 2^-24
  if (D == 2) {
    float s, c;
    sincospif(2.0f * static_cast<float>(r1.v[0] >> 8) * k24, &s, &c);
    dir_m[0] = c;
    dir_m[1] = s;
    sincospif(2.0f * static_cast<float>(r1.v[1] >> 8) * k24, &s, &c);
    dir_d[0] = c;
    dir_d[1] = s;
  } else {
    const float z1 = 2.0f * static_cast<float>(r1.v[0] >> 8) * k24 - 1.0f;
    const float z2 = 2.0f * static_cast<float>(r1.v[1] >> 8) * k24 - 1.0f;
    const float q1 = sqrtf(fmaxf(0.0f, 1.0f - z1 * z1)), q2 = sqrtf(fmaxf(0.0f, 1.0f - z2 * z2));
    float s, c;
    sincospif(2.0f * static_cast<float>(r1.v[2] >> 8) * k24, &s, &c);
    dir_m[0] = q1 * c;
    dir_m[1] = q1 * s;
    dir_m[2] = z1;
    sincospif(2.0f * static_cast<float>(r1.v[3] >> 8) * k24, &s, &c);
    dir_d[0] = q2 * c;
    dir_d[1] = q2 * s;
    dir_d[2] = z2;
  }
  float n0, n1;
  box_muller(r2.v[0], r2.v[1], n0, n1);
  const float mu = C.cell_sm ? C.mig_mu_steps_f : C.tau_mu_steps_f;
  const float sdv = C.cell_sm ? C.mig_sd_steps_f : C.tau_sd_steps_f;
  const int sd = __float2int_rn(mu + sdv * n0);
  const int sm = __float2int_rn(mu + sdv * n1);
  span_d = sd >= 1 ? sd : 1;  // randomTimeSpan, MD.cuh:434-436
  span_m = sm >= 1 ? sm : 1;
}

// The crawling/dividing cells: whether dividing cell g has its elements Rmin apart
// (binaryCellDivisionCriteria, MD.cuh:426-433; BoundingBox::distance, Utils.hpp:536-544, without
// fused arithmetic, as the restatement computes it).
__device__ __forceinline__ bool sm_ready(const EventArgs &a, const ColonyConst &C, int g) {
  const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
  double r2 = 0.0;
  for (int d = 0; d < C.dim; ++d) {
    double v = __dsub_rn(a.x[d * a.SS + s0], a.x[d * a.SS + s1]);  // r0 - r1
    if (C.periodic[d]) v = __dsub_rn(v, __dmul_rn(static_cast<double>(nint(v / C.box[d])), C.box[d]));
    r2 = __dadd_rn(r2, __dmul_rn(v, v));
  }
  return C.div_rmin_ratio != 0.0 ? r2 >= __dmul_rn(C.div_rmin_ratio, a.sigma_c[2 * g]) : r2 >= C.div_r2min;
}

// A division at this step: the cycle ends (linear growth), or a dividing cell is ready
// (crawling/dividing cells).
__device__ __forceinline__ bool division_due(const EventArgs &a, const ColonyConst &C, int i, int ts) {
  const int g = C.cell_base + i;
  if (C.cell_sm) return a.cst[g] == kCellDividing && sm_ready(a, C, g);
  return a.tsw[g] == ts;
}

// division detection: kCellItems consecutive cells per thread
__global__ void __launch_bounds__(kTile) k_div_count(EventArgs a_) {
  EventArgs a = a_;
  a.ts = *a_.ts_dev;
  const int total = a.tiles_cell[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_cell, a.B, t);
    const ColonyConst &C = a.col[c];
    const int n = a.cnt[c].ncell;
    const int i0 = (t - a.tiles_cell[c]) * kCellTile + threadIdx.x * kCellItems;
    int due = 0;
    if (C.divide) {
#pragma unroll
      for (int q = 0; q < kCellItems; ++q)
        due += (i0 + q < n && division_due(a, C, i0 + q, a.ts)) ? 1 : 0;
    }
    int tot;
    block_excl_scan_ev(due, &tot);
    if (threadIdx.x == 0) a.tile_count[t] = tot;
  }
}

// due cells of the step, ranked in cell order: the first ndiv_allowed go to the colony's
// division queue. Each block sums its colony's tile counts itself (those before its tile give
// its offset, all of them the colony's total for the capacity check), so no scan pass runs in
// between; the block of the colony's first tile records the step's counts.
__global__ void __launch_bounds__(kTile) k_div_rank(EventArgs a_) {
  const EventArgs &a = a_;
  const int ts = *a.ts_dev;
  const int total = a.tiles_cell[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_cell, a.B, t);
    const ColonyConst &C = a.col[c];
    ColonyCounters &K = a.cnt[c];
    const int n = K.ncell;
    const int tc0 = a.tiles_cell[c], tc1 = a.tiles_cell[c + 1];
    int before = 0, all = 0;
    for (int u = tc0 + static_cast<int>(threadIdx.x); u < tc1; u += kTile) {
      const int v = a.tile_count[u];
      all += v;
      before += u < t ? v : 0;
    }
    int off, cnt_all;
    block_excl_scan_ev(before, &off);
    block_excl_scan_ev(all, &cnt_all);
    // room for the cells and for their two element slots each (skin mode appends daughters
    // behind removed elements until the next slot re-sort)
    const int room_cells = C.cell_cap - n;
    const int room_slots = (C.slot_cap - K.nslot) / 2;
    const int room = room_cells < room_slots ? room_cells : room_slots;
    int allowed = cnt_all < room ? cnt_all : room;
    if (allowed < 0) allowed = 0;
    if (t == tc0 && threadIdx.x == 0) {
      if (allowed < cnt_all) K.err |= kErrCap;
      K.ndiv_step = cnt_all;
      K.ndiv_allowed = allowed;
      K.ndead = 0;
    }
    const int i0 = (t - tc0) * kCellTile + threadIdx.x * kCellItems;
    bool due[kCellItems];
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < kCellItems; ++q) {
      due[q] = C.divide && i0 + q < n && division_due(a, C, i0 + q, ts);
      cnt += due[q] ? 1 : 0;
    }
    int tot;
    int rank = off + block_excl_scan_ev(cnt, &tot);
#pragma unroll
    for (int q = 0; q < kCellItems; ++q) {
      if (!due[q]) continue;
      if (rank < allowed) a.divq[C.cell_base + rank] = i0 + q;
      ++rank;
    }
  }
}

__device__ void move_cell(const EventArgs &a, const ColonyConst &C, int dst, int src, int D) {
  const int gd = C.cell_base + dst, gs = C.cell_base + src;
  a.t0[gd] = a.t0[gs];
  a.tsw[gd] = a.tsw[gs];
  a.cst[gd] = a.cst[gs];
  a.sigma_c[2 * gd] = a.sigma_c[2 * gs];
  a.sigma_c[2 * gd + 1] = a.sigma_c[2 * gs + 1];
  for (int j = 0; j < 2; ++j) {
    const int sl = a.slot_of[2 * gs + j];
    a.eid[sl] = 2 * gd + j;
    a.slot_of[2 * gd + j] = sl;
  }
  if (a.obs_disp) {
    for (int d = 0; d < D; ++d) {
      a.obs_com_prev[d * a.CC + gd] = a.obs_com_prev[d * a.CC + gs];
      a.obs_disp[d * a.CC + gd] = a.obs_disp[d * a.CC + gs];
      a.obs_vref[d * a.CC + gd] = a.obs_vref[d * a.CC + gs];
    }
  }
}

// warp-level path of apo_colony for k <= 32 deaths among n1 cells. apo_small_pick: distinct
// uniform picks (redrawn while duplicated, at most 16 rounds), ascending in lanes 0..kk-1 (the
// return value kk; duplicates left after 16 rounds, practically impossible, are dropped).
// apo_small_apply: tombstones, then the live cells of the tail [n1 - kk, n1) move into the holes
// below it in ascending order (removeCell's swap-with-last, Colony.cpp:365-399, for a sorted
// set of victims). The picks depend only on n1, so they can be drawn before the divisions are
// placed; the apply reads the victims' slots, so it comes after.
__device__ int apo_small_pick(const EventArgs &a, const ColonyConst &C, int k, int n1, int *sdv_out) {
  const int lane = threadIdx.x & 31;
  int v = 0x7fffffff;
  bool need = lane < k;
  for (int attempt = 0; attempt < 16; ++attempt) {
    if (need) {
      const u32x4 r = philox4x32_10(static_cast<uint32_t>(lane) | (static_cast<uint32_t>(attempt) << 24),
                                    static_cast<uint32_t>(a.ts), kRngApoPick, C.rng_stream, a.seed_lo,
                                    a.seed_hi);
      const int x = static_cast<int>(uniform53(r.v[0], r.v[1]) * n1);
      v = x < n1 ? x : n1 - 1;
    }
    // bitonic sort of the 32 lanes, ascending
    for (int size = 2; size <= 32; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        const int o = __shfl_xor_sync(0xffffffffu, v, stride);
        const bool up = (lane & size) == 0 || size == 32;
        const bool low = (lane & stride) == 0;
        v = (low == up) ? min(v, o) : max(v, o);
      }
    const int prev = __shfl_up_sync(0xffffffffu, v, 1);
    need = lane > 0 && lane < k && v == prev;  // a duplicate: redraw it
    if (!__any_sync(0xffffffffu, need)) break;
    if (need) v = 0x7fffffff;  // sorts to the end, redrawn in the next round
  }
  // duplicates left after 16 rounds (practically impossible) are dropped
  const int prev_v = __shfl_up_sync(0xffffffffu, v, 1);  // every lane takes part in a shuffle
  const bool dup = lane > 0 && lane < k && v == prev_v;
  const bool keep = lane < k && v < n1 && !dup;
  const unsigned km = __ballot_sync(0xffffffffu, keep);
  const int kk = __popc(km);
  // the kept victims, ascending, to lanes 0..kk-1
  int sdv = 0x7fffffff;
  for (int src = 0; src < 32; ++src) {
    const int val = __shfl_sync(0xffffffffu, v, src);
    if (((km >> src) & 1u) && __popc(km & ((1u << src) - 1u)) == lane) sdv = val;
  }
  *sdv_out = sdv;
  return kk;
}

__device__ void apo_small_apply(const EventArgs &a, const ColonyConst &C, ColonyCounters &K, int sdv, int kk,
                                int n1, int D) {
  const int lane = threadIdx.x & 31;
  if (lane < kk) {
    const int g = C.cell_base + sdv;
    const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
    a.eid[s0] = -1;
    a.eid[s1] = -1;
    if (a.state) {
      a.state[s0] = kSlotDead;
      a.state[s1] = kSlotDead;
      a.pk[s0].w = -fabsf(a.pk[s0].w);
      a.pk[s1].w = -fabsf(a.pk[s1].w);
    }
  }
  __syncwarp();
  const int n2 = n1 - kk;
  const int q = n2 + lane;
  bool victim = false;
  for (int src = 0; src < kk; ++src) {
    const int vs = __shfl_sync(0xffffffffu, sdv, src);  // unconditional: every lane shuffles
    victim = victim || vs == q;
  }
  const bool live = lane < kk && !victim;
  const unsigned lm = __ballot_sync(0xffffffffu, live);
  const int rank = __popc(lm & ((1u << lane) - 1u));
  const int hole = __shfl_sync(0xffffffffu, sdv, rank & 31);
  if (live) move_cell(a, C, hole, q, D);
  __syncwarp();
  if (lane == 0) {
    K.ncell = n2;
    K.napo_total += kk;
  }
}

// The number of deaths among n1 cells this step (thread-level). Philox mode: every cell
// (daughters included) dies with probability p this step (CIL.cu:627-649); drawn as
// k ~ Binomial(n1, p) by inversion and a uniformly random k-subset, the same distribution
// without a draw per cell.
__device__ int apo_count(const EventArgs &a, const ColonyConst &C, ColonyCounters &K, int n1) {
  int k = 0;
  if (C.apop_p > 0.0 && n1 > 0) {
    const u32x4 r = philox4x32_10(C.rng_stream, static_cast<uint32_t>(a.ts), kRngApo, 0u, a.seed_lo, a.seed_hi);
    const float nn = static_cast<float>(n1), p = static_cast<float>(C.apop_p);
    const float mean = nn * p;
    if (mean < 30.0f) {
      // inversion of the binomial CDF from k = 0 (FP32: P(0) = exp(n log(1 - p)) >= e^-30);
      // at most 200 terms (P(k > 200) is below FP32 resolution for a mean under 30)
      const float u = static_cast<float>(r.v[0] >> 8) * 5.9604644775390625e-08f;
      const float ratio = p / (1.0f - p);
      float pk = __expf(nn * C.apop_log1m_p), cdf = pk;
      while (u > cdf && k < n1 && k < kDeadCap && k < 200) {
        pk *= (nn - static_cast<float>(k)) / static_cast<float>(k + 1) * ratio;
        cdf += pk;
        ++k;
      }
    } else {
      // large means: normal approximation with continuity rounding
      float z0, z1;
      box_muller(r.v[0], r.v[1], z0, z1);
      const float kf = rintf(mean + sqrtf(mean * (1.0f - p)) * z0);
      k = kf < 0.0f ? 0 : static_cast<int>(fminf(kf, nn));
    }
    if (k >= kDeadCap) {
      K.err |= kErrCap;
      k = kDeadCap - 1;
    }
  }
  return k;
}

// The step's apoptoses of colony c by one block (any multiple of 32 threads), after its
// divisions: commits the divisions' counts, draws the number of deaths, picks distinct victims,
// leaves tombstones and moves tail cells into the holes. With planned (k_events_due), the
// counts are committed and k (and, for k <= 32, warp 0's victims sdv / kk) were drawn already.
__device__ void apo_colony(const EventArgs &a, int c, int D, bool planned = false, int k_planned = 0,
                           int sdv_planned = 0, int kk_planned = 0) {
  __shared__ int sd[kDeadCap];
  __shared__ int s_n1, s_k;
  const ColonyConst &C = a.col[c];
  ColonyCounters &K = a.cnt[c];
  if (threadIdx.x == 0) {
    if (!planned) {
      const int add = K.ndiv_allowed;
      K.ncell += add;
      K.nslot += 2 * add;
      K.ndiv_total += add;
    }
    s_n1 = K.ncell;
    s_k = planned ? k_planned : apo_count(a, C, K, K.ncell);
  }
  __syncthreads();
  const int k = s_k, n1 = s_n1;
  if (k == 0) return;
  if (k <= 32) {
    // few deaths (the usual case): one warp, no block barriers
    if (threadIdx.x >= 32) return;
    int sdv = sdv_planned, kk = kk_planned;
    if (!planned) kk = apo_small_pick(a, C, k, n1, &sdv);
    apo_small_apply(a, C, K, sdv, kk, n1, D);
    return;
  }
  int P = 1;
  while (P < k) P <<= 1;
  // distinct uniform picks: draw, sort, redraw the duplicates (rare: about k^2 / 2n)
  __shared__ int s_dup;
  for (int i = threadIdx.x; i < P; i += blockDim.x) sd[i] = i < k ? -1 : 0x7fffffff;
  __syncthreads();
  for (int attempt = 0; attempt < 16; ++attempt) {
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
      if (sd[i] == -1) {
        const u32x4 r = philox4x32_10(static_cast<uint32_t>(i) | (static_cast<uint32_t>(attempt) << 24),
                                      static_cast<uint32_t>(a.ts), kRngApoPick, C.rng_stream, a.seed_lo,
                                      a.seed_hi);
        const int v = static_cast<int>(uniform53(r.v[0], r.v[1]) * n1);
        sd[i] = v < n1 ? v : n1 - 1;
      }
    }
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
          const int l = i ^ stride;
          if (l > i) {
            const bool up = (i & size) == 0;
            const int x = sd[i], y = sd[l];
            if ((x > y) == up) {
              sd[i] = y;
              sd[l] = x;
            }
          }
        }
        __syncthreads();
      }
    if (threadIdx.x == 0) {
      int dup = 0, last = sd[0];
      for (int i = 1; i < k; ++i) {
        if (sd[i] == last) {
          sd[i] = -1;  // redraw this copy
          dup = 1;
        } else {
          last = sd[i];
        }
      }
      s_dup = dup;
    }
    __syncthreads();
    if (!s_dup) break;
  }
  if (s_dup) {
    // still duplicated after 16 rounds (practically impossible): keep the distinct ones
    if (threadIdx.x == 0) {
      int w = 0;
      for (int i = 0; i < k; ++i)
        if (sd[i] >= 0) sd[w++] = sd[i];
      for (int i = w; i < P; ++i) sd[i] = 0x7fffffff;
      s_k = w;
    }
    __syncthreads();
    // the -1 holes were dropped; the survivors stay ascending
  }
  const int kk = s_k;
  // tombstones
  for (int r = threadIdx.x; r < kk; r += blockDim.x) {
    const int g = C.cell_base + sd[r];
    const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
    a.eid[s0] = -1;
    a.eid[s1] = -1;
    if (a.state) {
      a.state[s0] = kSlotDead;
      a.state[s1] = kSlotDead;
      a.pk[s0].w = -fabsf(a.pk[s0].w);
      a.pk[s1].w = -fabsf(a.pk[s1].w);
    }
  }
  __syncthreads();
  const int n2 = n1 - kk;
  // movers: live cells of [n2, n1) in ascending order, paired with holes sd[0..h)
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = n2; base < n1; base += blockDim.x) {
    const int q = base + threadIdx.x;
    bool live = false;
    if (q < n1) {
      int lo = 0, hi = kk - 1;
      bool found = false;
      while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (sd[mid] == q) {
          found = true;
          break;
        }
        if (sd[mid] < q)
          lo = mid + 1;
        else
          hi = mid - 1;
      }
      live = !found;
    }
    // rank among live tail cells (block-wide, 1024 threads: serial over warps)
    const unsigned m = __ballot_sync(0xffffffffu, live);
    __shared__ int wcount[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wcount[wid] = __popc(m);
    __syncthreads();
    int before = s_carry;
    for (int w = 0; w < wid; ++w) before += wcount[w];
    const int rank = before + __popc(m & ((1u << lane) - 1u));
    if (live) move_cell(a, C, sd[rank], q, D);
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += wcount[w];
      s_carry += tot;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    K.ncell = n2;
    K.napo_total += kk;
  }
}

// One block per colony: the divisions of the queue, one thread each (draws, FP64 placement of
// the four elements, new cycles; daughters take cells n + rank and slots nslot + 2 rank), then
// the colony's apoptoses (apo_colony) once every division is placed.
template <int D>
__global__ void __launch_bounds__(kTile) k_events_exec(EventArgs a_) {
  EventArgs a = a_;
  a.ts = *a_.ts_dev;
  const int c = blockIdx.x;
  const ColonyConst &C = a.col[c];
  const ColonyCounters &K = a.cnt[c];
  const int nd = K.ndiv_allowed, n = K.ncell, nslot = K.nslot;
  for (int r = threadIdx.x; r < nd; r += blockDim.x) {
    const int i = a.divq[C.cell_base + r];
    double dm[D], dd[D];
    int span_d, span_m;
    division_draws<D>(a, i, dm, dd, span_d, span_m, C);
    // crawling/dividing cells: migration spans, the mother's added to her own time (CIL.cu:403, 424)
    const int tm = C.cell_sm ? a.tsw[C.cell_base + i] + span_m : a.ts + span_m;
    divide_cell<D>(a, C, c, i, n + r, dm, dd, a.ts + span_d, tm, nslot, r);
  }
  __syncthreads();  // every division is placed, and visible to the whole block
  apo_colony(a, c, D);
}

// Ascending bitonic sort of v[0, P) (P a power of two) by the whole block; v in shared or
// global memory (a block barrier orders both within the block).
__device__ void block_bitonic_sort(int *v, int P) {
  for (int size = 2; size <= P; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ stride;
        if (l > i) {
          const bool up = (i & size) == 0;
          const int x = v[i], y = v[l];
          if ((x > y) == up) {
            v[i] = y;
            v[l] = x;
          }
        }
      }
      __syncthreads();
    }
}

constexpr int kDueSort = 2048;  // due cells sorted in shared memory (more: in the queue itself)
constexpr int kDueRank = 512;   // up to this many: sorted by ranks instead of a sorting network

// Skin mode, Philox: the step's events from the due-cell queues, one block per colony. The
// force pass appended the cells whose cycle ends at this step (in no particular order); the
// block sorts them by cell index, so the first ndiv_allowed in cell order divide (within the
// colony's cell and slot room; the ranking of the tile-wise kernels), places the divisions
// (one thread each: draws, FP64 placement of the four elements, new cycles; daughters take
// cells n + rank and slots nslot + 2 rank), then the colony's apoptoses (apo_colony). The
// kernel reads the step as *ts_dev + 1; the block that finishes last writes it back and
// clears the next step's any-rebuild flag (in place of a step-counter launch).
template <int D>
__global__ void __launch_bounds__(kTile) k_events_due(EventArgs a_) {
  EventArgs a = a_;
  a.ts = *a_.ts_dev + 1;
  const int c = blockIdx.x;
  const ColonyConst &C = a.col[c];
  ColonyCounters &K = a.cnt[c];
  __shared__ int s_key[kDueSort], s_sorted[kDueRank];
  __shared__ int s_allowed;
  const int n = K.ncell;
  const int nd = min(K.ndue, n);
  int *q = a.dueq + C.due_base;  // capacity: a power of two >= cell_cap
  int *keys = s_key;
  if (nd <= kDueRank) {
    // the keys are distinct cell indices: each one's rank is the number of smaller keys, so
    // one pass over the shared keys (and two barriers) sorts them
    for (int i = threadIdx.x; i < nd; i += blockDim.x) s_key[i] = q[i];
    __syncthreads();
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
      const int v = s_key[i];
      int r = 0;
      for (int j = 0; j < nd; ++j) r += s_key[j] < v ? 1 : 0;
      s_sorted[r] = v;
    }
    keys = s_sorted;
  } else {
    int P = 1;
    while (P < nd) P <<= 1;
    if (P <= kDueSort) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) s_key[i] = i < nd ? q[i] : 0x7fffffff;
    } else {
      for (int i = nd + static_cast<int>(threadIdx.x); i < P; i += blockDim.x) q[i] = 0x7fffffff;
      keys = q;
    }
    __syncthreads();
    block_bitonic_sort(keys, P);
  }
  if (threadIdx.x == 0) {
    // room for the cells and for their two element slots each (skin mode appends daughters
    // behind removed elements until the next slot re-sort)
    const int room_cells = C.cell_cap - n;
    const int room_slots = (C.slot_cap - K.nslot) / 2;
    const int room = room_cells < room_slots ? room_cells : room_slots;
    int allowed = nd < room ? nd : room;
    if (allowed < 0) allowed = 0;
    if (allowed < nd) K.err |= kErrCap;
    K.ndiv_step = nd;
    K.ndiv_allowed = allowed;
    K.ndead = 0;
    K.ndue = 0;  // for the next step's force pass
    s_allowed = allowed;
  }
  __syncthreads();
  const int allowed = s_allowed, nslot = K.nslot;
  // the apoptosis draws depend only on the cell count after the divisions: the last warp draws
  // them (and, for k <= 32, picks the victims) while the other warps place the divisions
  __shared__ int s_k, s_kk, s_vic[32];
  if (threadIdx.x >= kTile - 32) {
    const int lane = threadIdx.x & 31;
    int k = 0;
    if (lane == 0) k = apo_count(a, C, K, n + allowed);
    k = __shfl_sync(0xffffffffu, k, 0);
    int sdv = 0, kk = 0;
    if (k > 0 && k <= 32) kk = apo_small_pick(a, C, k, n + allowed, &sdv);
    s_vic[lane] = sdv;
    if (lane == 0) {
      s_k = k;
      s_kk = kk;
    }
  }
  for (int r = threadIdx.x; r < allowed; r += blockDim.x) {
    const int i = keys[r];
    double dm[D], dd[D];
    int span_d, span_m;
    division_draws<D>(a, i, dm, dd, span_d, span_m, C);
    divide_cell<D>(a, C, c, i, n + r, dm, dd, a.ts + span_d, a.ts + span_m, nslot, r);
  }
  __syncthreads();  // every division is placed, and visible to the whole block
  if (threadIdx.x == 0) {
    K.ncell = n + allowed;
    K.nslot = nslot + 2 * allowed;
    K.ndiv_total += allowed;
  }
  __syncthreads();
  apo_colony(a, c, D, true, s_k, s_vic[threadIdx.x & 31], s_kk);
  __syncthreads();
  if (threadIdx.x == 0) {
    // the last colony's block moves the step counter (every block has read it by then)
    __threadfence();
    if (atomicAdd(a.ev_done, 1) == a.B - 1) {
      a.any_rebuild[a.ts & 1] = 0;
      *a.ts_dev = a.ts;
      *a.ev_done = 0;
    }
  }
}

// oracle mode: divisions in the host's order with host-drawn axes and cycle lengths
template <int D>
__global__ void k_div_list(EventArgs a_, int c, int n0, int ndiv, const int *mothers, const double *dirs,
                           const int *tsws) {
  EventArgs a = a_;
  a.ts = *a_.ts_dev;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ndiv) return;
  const ColonyConst &C = a.col[c];
  if (a.cnt[c].nslot + 2 * (r + 1) > C.slot_cap) {  // no slot left for the daughter
    atomicOr(&a.cnt[c].err, kErrCap);
    return;
  }
  divide_cell<D>(a, C, c, mothers[r], n0 + r, dirs + (2 * r) * D, dirs + (2 * r + 1) * D, tsws[2 * r],
                 tsws[2 * r + 1], a.cnt[c].nslot, r);
}

// oracle mode: commit divisions, then the sequential removals removeCell(i) in order
__global__ void k_apo_ops(EventArgs a, int c, int ndiv, int nops, const int *ops, int D) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const ColonyConst &C = a.col[c];
  ColonyCounters &K = a.cnt[c];
  K.ncell += ndiv;
  K.nslot += 2 * ndiv;
  K.ndiv_total += ndiv;
  for (int q = 0; q < nops; ++q) {
    const int i = ops[q];
    const int last = K.ncell - 1;
    if (i < 0 || i > last) {
      K.err |= kErrCap;
      return;
    }
    const int g = C.cell_base + i;
    const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
    a.eid[s0] = -1;
    a.eid[s1] = -1;
    if (a.state) {
      a.state[s0] = kSlotDead;
      a.state[s1] = kSlotDead;
      a.pk[s0].w = -fabsf(a.pk[s0].w);
      a.pk[s1].w = -fabsf(a.pk[s1].w);
    }
    if (i != last) move_cell(a, C, i, last, D);
    K.ncell -= 1;
    K.napo_total += 1;
  }
}

// Upload, step 1: every staged diameter positive and finite (bit 1 of chk[0] otherwise) and
// every staged position finite and in [0, L) on its axis (bit 2, CIL.cuh:54-66); the largest
// diameter (positive doubles order like their bit patterns) into chk[1..2].
template <int D>
__global__ void k_upload_check(const ColonyConst *col, int c, int ncells, const double *pos, const double *sig,
                               int *chk) {
  const ColonyConst &C = col[c];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // the grid is whole warps
  unsigned long long smax = 0ull;  // bits of the largest valid diameter (positive doubles order as integers)
  if (e < 2 * ncells) {
    const double s = sig[e];
    int bad = (s > 0.0 && isfinite(s)) ? 0 : 1;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double x = pos[static_cast<size_t>(e) * D + d];
      if (!(isfinite(x) && x >= 0.0 && x < C.box[d])) bad |= 2;
    }
    if (bad) atomicOr(chk, bad);
    if (!(bad & 1)) smax = static_cast<unsigned long long>(__double_as_longlong(s));
  }
  // one atomic per warp: the warp's largest diameter first
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_down_sync(0xffffffffu, smax, o);
    smax = v > smax ? v : smax;
  }
  if ((threadIdx.x & 31) == 0 && smax) atomicMax(reinterpret_cast<unsigned long long *>(chk + 2), smax);
}

// Upload, step 2 (nothing happens when step 1 found a bad value): the staged positions into the
// colony's first slots, the staged diameters and cycles into the cell arrays, element ids and
// slots, zero velocities, every other slot of the colony empty, the counters.
template <int D>
__global__ void k_upload(const ColonyConst *col, int c, int ncells, size_t SS, const double *pos, const double *sig,
                         const int *t0s, const int *tsws, double *x, double *sig_c, int *t0, int *tsw, double *vel,
                         int *eid, int *slot_of, ColonyCounters *cnt, const int *chk) {
  if (*chk != 0) return;  // uniform
  const ColonyConst &C = col[c];
  for (int slot = C.slot_base + blockIdx.x * blockDim.x + threadIdx.x; slot < C.slot_base + C.slot_cap;
       slot += gridDim.x * blockDim.x) {
    const int e = slot - C.slot_base;
    if (e < 2 * ncells) {
#pragma unroll
      for (int d = 0; d < D; ++d) x[d * SS + slot] = pos[static_cast<size_t>(e) * D + d];
      eid[slot] = 2 * C.cell_base + e;
      slot_of[2 * C.cell_base + e] = slot;
      sig_c[2 * static_cast<size_t>(C.cell_base) + e] = sig[e];
      if (e < ncells) {
        t0[C.cell_base + e] = t0s[e];
        tsw[C.cell_base + e] = tsws[e];
      }
    } else {
      eid[slot] = -1;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) vel[d * SS + slot] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt[c].ncell = ncells;
    cnt[c].nslot = 2 * ncells;
    cnt[c].nlive = 0;
    cnt[c].err = 0;
    cnt[c].ndead = 0;
    cnt[c].ndiv_step = 0;
    cnt[c].ndiv_allowed = 0;
    cnt[c].ndue = 0;
  }
}

__global__ void k_gather_canonical(int ncells, int dim, size_t SS, int cell_base, const int *slot_of,
                                   const double *src, int width, double *dst) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 2 * ncells) return;
  const int slot = slot_of[2 * cell_base + e];
  for (int d = 0; d < width; ++d) dst[static_cast<size_t>(e) * width + d] = src[d * SS + slot];
  (void)dim;
}

// nint(t / L) (Utils.hpp:173-175): 0 without a division when |t| < L / 4 (t / L then lies in
// (-0.25, 0.25) whatever its rounding), the division otherwise (a minimum image across the box)
__device__ __forceinline__ int nint_small(double t, double L) { return fabs(t) < 0.25 * L ? 0 : nint(t / L); }

template <int D>
__global__ void __launch_bounds__(kTile) k_obs(EventArgs a, int c, int ncells, int reset, double *partials) {
  const ColonyConst &C = a.col[c];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double area = 0.0, msd = 0.0, vv = 0.0, v0 = 0.0;
  if (i < ncells) {
    const int g = C.cell_base + i;
    const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
    double com[D], v[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double r0 = a.x[d * a.SS + s0], r1 = a.x[d * a.SS + s1];
      double rel = r1 - r0;
      if (C.periodic[d]) rel -= static_cast<double>(nint_small(rel, C.box[d])) * C.box[d];
      const double m = (0.0 + rel) / 2.0;  // calculComs, Colony.cpp:409-432
      // fmod(m + r0 + L, L) with m + r0 in [-L, 2L): the exact division-free form
      com[d] = C.periodic[d] ? wrap_like_fmod(m + r0, C.box[d]) : m + r0;
      v[d] = a.vel ? 0.5 * (a.vel[d * a.SS + s0] + a.vel[d * a.SS + s1]) : 0.0;
    }
    const double q0 = a.sigma_c[2 * g] * 0.5, q1 = a.sigma_c[2 * g + 1] * 0.5;
    area = 3.14159265358979323846 * q0 * q0 + 3.14159265358979323846 * q1 * q1;
    if (reset) {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        a.obs_com_prev[d * a.CC + g] = com[d];
        a.obs_disp[d * a.CC + g] = 0.0;
        a.obs_vref[d * a.CC + g] = v[d];
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        double dr = com[d] - a.obs_com_prev[d * a.CC + g];
        if (C.periodic[d]) dr -= static_cast<double>(nint_small(dr, C.box[d])) * C.box[d];
        const double acc = a.obs_disp[d * a.CC + g] + dr;
        a.obs_disp[d * a.CC + g] = acc;
        a.obs_com_prev[d * a.CC + g] = com[d];
        msd += acc * acc;
        const double vr = a.obs_vref[d * a.CC + g];
        vv += v[d] * vr;
        v0 += vr * vr;
      }
    }
  }
  // deterministic block reduction
  __shared__ double red[4][kTile];
  red[0][threadIdx.x] = area;
  red[1][threadIdx.x] = msd;
  red[2][threadIdx.x] = vv;
  red[3][threadIdx.x] = v0;
  __syncthreads();
  for (int s = kTile / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) partials[blockIdx.x * 4 + q] = red[q][0];
}

// the device step counter moves past the force step (before the events read it); skin mode
// also clears the next step's any-rebuild flag. With tiles_cell, the same block writes the tile
// table over the cells that the event kernels of the step read (the cell counts do not change
// between the force pass and the events).
__global__ void __launch_bounds__(kTile) k_step_end(int *ts, int *any_rebuild, const ColonyCounters *cnt, int B,
                                                    int *tiles_cell) {
  if (threadIdx.x == 0) {
    if (any_rebuild) any_rebuild[(*ts + 1) & 1] = 0;
    *ts += 1;
  }
  if (!tiles_cell) return;  // uniform
  int carry = 0;
  for (int base = 0; base < B; base += kTile) {
    const int c = base + static_cast<int>(threadIdx.x);
    const int v = c < B ? (cnt[c].ncell + kCellTile - 1) / kCellTile : 0;
    int total;
    const int ex = block_excl_scan_ev(v, &total);
    if (c < B) tiles_cell[c] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) tiles_cell[B] = carry;
}

}  // namespace

void launch_advance_ts(int *ts_dev, int *any_rebuild, cudaStream_t s, const ColonyCounters *cnt, int B,
                       int *tiles_cell) {
  k_step_end<<<1, kTile, 0, s>>>(ts_dev, any_rebuild, cnt, B, tiles_cell);
}

void launch_events_fast(const EventArgs &a, int grid_cells, int dim, cudaStream_t s, bool cell_states) {
  k_div_count<<<grid_cells, kTile, 0, s>>>(a);
  k_div_rank<<<grid_cells, kTile, 0, s>>>(a);
  if (cell_states) launch_sm_philox(a, grid_cells, s);
  if (dim == 2)
    k_events_exec<2><<<a.B, kTile, 0, s>>>(a);
  else
    k_events_exec<3><<<a.B, kTile, 0, s>>>(a);
}

void launch_events_due(const EventArgs &a, int dim, cudaStream_t s) {
  if (dim == 2)
    k_events_due<2><<<a.B, kTile, 0, s>>>(a);
  else
    k_events_due<3><<<a.B, kTile, 0, s>>>(a);
}

// The crawling/dividing cells, oracle mode: per cell of the colony, whether a dividing cell's
// elements are far enough apart to divide (binaryCellDivisionCriteria, MD.cuh:426-433; the
// squared separation of BoundingBox::distance, Utils.hpp:536-544, without fused arithmetic, as
// the restatement computes it). The host reads the flags and decides the step's events.
template <int D>
__global__ void k_sm_flags(EventArgs a, int c, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ColonyConst &C = a.col[c];
  const int g = C.cell_base + i;
  unsigned char f = 0;
  if (a.cst[g] == kCellDividing) {
    const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
    double r2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double v = __dsub_rn(a.x[d * a.SS + s0], a.x[d * a.SS + s1]);  // r0 - r1
      if (C.periodic[d]) v = __dsub_rn(v, __dmul_rn(static_cast<double>(nint(v / C.box[d])), C.box[d]));
      r2 = __dadd_rn(r2, __dmul_rn(v, v));
    }
    const bool ok = C.div_rmin_ratio != 0.0 ? r2 >= __dmul_rn(C.div_rmin_ratio, a.sigma_c[2 * g]) : r2 >= C.div_r2min;
    f = ok ? 1 : 0;
  }
  a.smflag[g] = f;
}

// The crawling/dividing cells, oracle mode: the step's non-dividing transitions in the host's
// order, ops[3 r] = cell, kind, new time; kind 1: the cell starts dividing; kind 2: a failed
// division (binaryCellDivisionFail, MD.cu:736-752: the back element moved half the bond
// towards the front, a plain add, then both reoriented about it at R0 along dirs[r]), the cell
// crawls again with its diameters reset. Velocities of the cell are zeroed (CIL.cu:432, 444).
template <int D>
__global__ void k_sm_ops(EventArgs a, int c, int nops, const int *ops, const double *dirs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nops) return;
  const ColonyConst &C = a.col[c];
  const int i = ops[3 * r], kind = ops[3 * r + 1], tsw_new = ops[3 * r + 2];
  const int g = C.cell_base + i;
  const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
  const size_t SS = a.SS;
  if (kind == 2) {
    double x0[D], x1[D], m[D], sl[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      x0[d] = a.x[d * SS + s0];
      x1[d] = a.x[d * SS + s1];
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double v = __dsub_rn(x1[d], x0[d]);  // r1 - r0
      if (C.periodic[d]) v = __dsub_rn(v, __dmul_rn(static_cast<double>(nint(v / C.box[d])), C.box[d]));
      x0[d] = __dadd_rn(x0[d], __dmul_rn(v, 0.5));
    }
    place<D>(C, x0, dirs + static_cast<size_t>(r) * D, C.div_radius, m, sl);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      a.x[d * SS + s0] = m[d];
      a.x[d * SS + s1] = sl[d];
    }
    a.sigma_c[2 * g] = C.sigma_core[0];
    a.sigma_c[2 * g + 1] = C.sigma_core[1];
    if (a.sig) {
      a.sig[s0] = C.sigma_core[0];
      a.sig[s1] = C.sigma_core[1];
    }
    a.cst[g] = kCellCrawling;
  } else {
    a.cst[g] = kCellDividing;
  }
  a.tsw[g] = tsw_new;
  if (a.vel) {
#pragma unroll
    for (int d = 0; d < D; ++d) a.vel[d * SS + s0] = a.vel[d * SS + s1] = 0.0;
  }
}

// updateDiameters (CIL.cu:970-991) with SWELLING: a dividing cell's diameters below the larger
// SIGMA_CORE grow by (max - sigma) / (tswitch - ts); canonical and binned copies.
__device__ __forceinline__ void swell_cell(const EventArgs &a, const ColonyConst &C, int g, int ts);

__global__ void k_sm_swell(EventArgs a, int c, int n, int ts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  swell_cell(a, a.col[c], a.col[c].cell_base + i, ts);
}

__device__ __forceinline__ void swell_cell(const EventArgs &a, const ColonyConst &C, int g, int ts) {
  if (a.cst[g] != kCellDividing) return;
  const double smax = C.sigma_core[0] > C.sigma_core[1] ? C.sigma_core[0] : C.sigma_core[1];
  const double span = static_cast<double>(a.tsw[g] - ts);
  for (int j = 0; j < 2; ++j) {
    double s = a.sigma_c[2 * g + j];
    if (s < smax) {
      s = __dadd_rn(s, (smax - s) / span);
      a.sigma_c[2 * g + j] = s;
      const int sl = a.slot_of[2 * g + j];
      if (a.sig) a.sig[sl] = s;
      if (a.pk) a.pk[sl].w = copysignf(static_cast<float>(s), a.pk[sl].w);
    }
  }
}

void launch_sm_swell(const EventArgs &a, int colony, int n, int ts, cudaStream_t s) {
  if (n > 0) k_sm_swell<<<(n + 255) / 256, 256, 0, s>>>(a, colony, n, ts);
}

// Philox mode, crawling/dividing cells, before the divisions are placed: a crawling (or
// undefined) cell whose time ends starts dividing (time += a division span); a dividing cell
// short of Rmin whose time ends fails (binaryCellDivisionFail at R0 along a random axis; crawling;
// time += a migration span). Draws keyed by (cell, step, purpose, colony stream).
__global__ void __launch_bounds__(kTile) k_sm_philox(EventArgs a_) {
  EventArgs a = a_;
  a.ts = *a_.ts_dev;
  const int total = a.tiles_cell[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_cell, a.B, t);
    const ColonyConst &C = a.col[c];
    if (!C.cell_sm) continue;
    const int n = a.cnt[c].ncell;
    const int i0 = (t - a.tiles_cell[c]) * kCellTile + threadIdx.x * kCellItems;
    for (int q = 0; q < kCellItems; ++q) {
      const int i = i0 + q;
      if (i >= n) break;
      const int g = C.cell_base + i;
      if (a.tsw[g] != a.ts) continue;
      const bool dividing = a.cst[g] == kCellDividing;
      if (dividing && sm_ready(a, C, g)) continue;  // divides (k_events_exec)
      const u32x4 r = philox4x32_10(static_cast<uint32_t>(i), static_cast<uint32_t>(a.ts), kRngCellState,
                                    C.rng_stream, a.seed_lo, a.seed_hi);
      float n0, n1;
      box_muller(r.v[0], r.v[1], n0, n1);
      const float mu = dividing ? C.mig_mu_steps_f : C.tau_mu_steps_f;
      const float sd = dividing ? C.mig_sd_steps_f : C.tau_sd_steps_f;
      const int span = max(__float2int_rn(mu + sd * n0), 1);
      const int s0 = a.slot_of[2 * g], s1 = a.slot_of[2 * g + 1];
      if (dividing) {  // failed division
        const float k24 = 5.9604644775390625e-08f;  // 2^-24
        double dir[3] = {0.0, 0.0, 0.0};
        if (C.dim == 2) {
          float sn, cs;
          sincospif(2.0f * static_cast<float>(r.v[2] >> 8) * k24, &sn, &cs);
          dir[0] = cs;
          dir[1] = sn;
        } else {
          const float z = 2.0f * static_cast<float>(r.v[2] >> 8) * k24 - 1.0f;
          const float qz = sqrtf(fmaxf(0.0f, 1.0f - z * z));
          float sn, cs;
          sincospif(2.0f * static_cast<float>(r.v[3] >> 8) * k24, &sn, &cs);
          dir[0] = qz * cs;
          dir[1] = qz * sn;
          dir[2] = z;
        }
        double x0[3], x1[3];
        for (int d = 0; d < C.dim; ++d) {
          x0[d] = a.x[d * a.SS + s0];
          x1[d] = a.x[d * a.SS + s1];
          double v = __dsub_rn(x1[d], x0[d]);
          if (C.periodic[d]) v = __dsub_rn(v, __dmul_rn(static_cast<double>(nint(v / C.box[d])), C.box[d]));
          x0[d] = __dadd_rn(x0[d], __dmul_rn(v, 0.5));
        }
        for (int d = 0; d < C.dim; ++d) {
          const double m = __dadd_rn(x0[d], __dmul_rn(C.div_radius, dir[d]));
          const double sl = __dadd_rn(x0[d], __dmul_rn(-C.div_radius, dir[d]));
          a.x[d * a.SS + s0] = C.periodic[d] ? wrap_like_fmod(m, C.box[d]) : m;
          a.x[d * a.SS + s1] = C.periodic[d] ? wrap_like_fmod(sl, C.box[d]) : sl;
        }
        a.sigma_c[2 * g] = C.sigma_core[0];
        a.sigma_c[2 * g + 1] = C.sigma_core[1];
        if (a.sig) {
          a.sig[s0] = C.sigma_core[0];
          a.sig[s1] = C.sigma_core[1];
        }
        a.cst[g] = kCellCrawling;
      } else {
        a.cst[g] = kCellDividing;
      }
      a.tsw[g] += span;
      if (a.vel)
        for (int d = 0; d < C.dim; ++d) a.vel[d * a.SS + s0] = a.vel[d * a.SS + s1] = 0.0;
    }
  }
}

// Philox mode: swelling of every colony's dividing cells after the events (the step from the
// device counter, so that a captured step replays correctly)
__global__ void __launch_bounds__(kTile) k_sm_swell_all(EventArgs a_) {
  const EventArgs &a = a_;
  const int ts = *a.ts_dev;
  const int total = a.tiles_cell[a.B];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int c = colony_of_tile(a.tiles_cell, a.B, t);
    const ColonyConst &C = a.col[c];
    if (!C.cell_sm || !C.swelling) continue;
    const int n = a.cnt[c].ncell;
    const int i0 = (t - a.tiles_cell[c]) * kCellTile + threadIdx.x * kCellItems;
    for (int q = 0; q < kCellItems && i0 + q < n; ++q) swell_cell(a, C, C.cell_base + i0 + q, ts);
  }
}

void launch_sm_philox(const EventArgs &a, int grid_cells, cudaStream_t s) {
  k_sm_philox<<<grid_cells, kTile, 0, s>>>(a);
}

void launch_sm_swell_all(const EventArgs &a, int grid_cells, cudaStream_t s) {
  k_sm_swell_all<<<grid_cells, kTile, 0, s>>>(a);
}

__global__ void k_fill_int(int *dst, int n, int value) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = value;
}

void launch_fill_int(int *dst, int n, int value, cudaStream_t s) {
  if (n > 0) k_fill_int<<<(n + 255) / 256, 256, 0, s>>>(dst, n, value);
}

void launch_sm_flags(const EventArgs &a, int colony, int n, int dim, cudaStream_t s) {
  if (n <= 0) return;
  if (dim == 2)
    k_sm_flags<2><<<(n + 255) / 256, 256, 0, s>>>(a, colony, n);
  else
    k_sm_flags<3><<<(n + 255) / 256, 256, 0, s>>>(a, colony, n);
}

void launch_sm_ops(const EventArgs &a, int colony, int nops, const int *ops, const double *dirs, int dim,
                   cudaStream_t s) {
  if (nops <= 0) return;
  if (dim == 2)
    k_sm_ops<2><<<(nops + 127) / 128, 128, 0, s>>>(a, colony, nops, ops, dirs);
  else
    k_sm_ops<3><<<(nops + 127) / 128, 128, 0, s>>>(a, colony, nops, ops, dirs);
}

void launch_divisions_list(const EventArgs &a, int colony, int n0, int ndiv, const int *mothers,
                           const double *dirs, const int *spans, int dim, cudaStream_t s) {
  if (ndiv <= 0) return;
  const int blocks = (ndiv + 127) / 128;
  if (dim == 2)
    k_div_list<2><<<blocks, 128, 0, s>>>(a, colony, n0, ndiv, mothers, dirs, spans);
  else
    k_div_list<3><<<blocks, 128, 0, s>>>(a, colony, n0, ndiv, mothers, dirs, spans);
}

void launch_apo_ops_with_div(const EventArgs &a, int colony, int ndiv, int nops, const int *ops, int dim,
                             cudaStream_t s) {
  k_apo_ops<<<1, 32, 0, s>>>(a, colony, ndiv, nops, ops, dim);
}

void launch_upload(const ColonyConst *col, int colony, int ncells, int dim, size_t SS, const double *stage,
                   double *x, double *sig_c, int *t0, int *tsw, double *vel, int *eid, int *slot_of,
                   ColonyCounters *cnt, int *chk, cudaStream_t s) {
  // stage: positions [2n][dim], diameters [2n], then t0 and tswitch [n] each as int
  const size_t ne = 2 * static_cast<size_t>(ncells);
  const double *pos = stage, *sig = stage + ne * dim;
  const int *t0s = reinterpret_cast<const int *>(sig + ne), *tsws = t0s + ncells;
  const int blocks = static_cast<int>((ne + kTile - 1) / kTile);
  if (dim == 2) {
    if (ne) k_upload_check<2><<<blocks, kTile, 0, s>>>(col, colony, ncells, pos, sig, chk);
    k_upload<2><<<1024, kTile, 0, s>>>(col, colony, ncells, SS, pos, sig, t0s, tsws, x, sig_c, t0, tsw, vel, eid,
                                       slot_of, cnt, chk);
  } else {
    if (ne) k_upload_check<3><<<blocks, kTile, 0, s>>>(col, colony, ncells, pos, sig, chk);
    k_upload<3><<<1024, kTile, 0, s>>>(col, colony, ncells, SS, pos, sig, t0s, tsws, x, sig_c, t0, tsw, vel, eid,
                                       slot_of, cnt, chk);
  }
}

void launch_gather_canonical(int ncells, int dim, size_t SS, int cell_base, const int *slot_of,
                             const double *src, int width, double *dst, cudaStream_t s) {
  if (ncells <= 0) return;
  const int blocks = (2 * ncells + kTile - 1) / kTile;
  k_gather_canonical<<<blocks, kTile, 0, s>>>(ncells, dim, SS, cell_base, slot_of, src, width, dst);
}

void launch_observables(const EventArgs &a, int colony, int ncells, int dim, int reset,
                        double *partials, int nblocks, cudaStream_t s) {
  if (dim == 2)
    k_obs<2><<<nblocks, kTile, 0, s>>>(a, colony, ncells, reset, partials);
  else
    k_obs<3><<<nblocks, kTile, 0, s>>>(a, colony, ncells, reset, partials);
}

}  // namespace cil
