// Internal declarations shared by the translation units of libcilgpu.so.
//
// Device data layout (one handle holds B colonies; every array is concatenated by colony):
//   cells    global cell id   g = cell_base[c] + i           (i < ncell[c] <= cell_cap[c])
//   elements global element id e = 2 g + j (j = 0 back, 1 front; the reference's
//            [cell][elem] order, Colony.cpp:204-237)
//   slots    binned element storage, colony c owns [slot_base[c], slot_base[c] + slot_cap[c]).
//            After a rebuild, slots [slot_base, slot_base + nlive) are sorted by bin and,
//            within a bin, by element id. Positions are SoA: x[d * SS + slot].
//   bins     colony c owns [bin_base[c], bin_base[c] + nbins_pad[c]); range[b] = (first, end)
//            slot of bin b. Bin ids follow the reference's link-list numbering
//            ls0*Ns1 + ls1 (2D) / (ls0*Ns1 + ls1)*Ns2 + ls2 (3D), Utils.hpp:1020-1048.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cil_gpu.h"

namespace cil {

constexpr int kTile = 256;        // threads per block of every slot/cell-parallel kernel
constexpr int kScanItems = 1024;  // bins per scan block (256 threads x 4)
constexpr int kDeadCap = 8192;    // apoptoses per colony per step handled on the device
constexpr int kListCap = 64;      // Verlet list entries per element (skin mode)
constexpr int kFreshCap = 16384;  // elements created or moved by division between list rebuilds
constexpr int kMaxSkinColonies = 4096;  // colonies per handle in skin mode (fresh-pair prefix in shared memory)
constexpr int kListSlotBits = 26; // list entry = slot | (bin offset code << 26)
// bin offset code of a list entry: (dx + 1) | (dy + 1) << 2 | (dz + 1) << 4, d* in {-1, 0, 1}
__host__ __device__ __forceinline__ unsigned list_offset_code(int o, int D) {
  return D == 2 ? static_cast<unsigned>((o / 3) | ((o % 3) << 2))
                : static_cast<unsigned>((o / 9) | (((o / 3) % 3) << 2) | ((o % 3) << 4));
}
constexpr int kCellItems = 4;     // cells per thread in the event kernels
constexpr int kCellTile = kTile * kCellItems;

// error bits in ColonyCounters::err
constexpr int kErrNan = 1 << CIL_ERR_NAN;
constexpr int kErrBox = 1 << CIL_ERR_OUT_OF_BOX;
constexpr int kErrCap = 1 << CIL_ERR_CAPACITY;

// Philox purposes (third counter word)
constexpr uint32_t kRngNoise = 1, kRngDiv = 2, kRngDiv2 = 3, kRngApo = 4, kRngApoPick = 5;
constexpr uint32_t kRngCellState = 6;  // the crawling/dividing cells' start and failed-division draws

// per-slot state in skin mode
constexpr unsigned char kSlotNormal = 0;  // in the bins and Verlet lists of the last rebuild
constexpr unsigned char kSlotFresh = 1;   // created or moved by a division since then
constexpr unsigned char kSlotDead = 2;    // removed by apoptosis

// Verlet-skin control of one colony (device resident; written by the kernels)
struct ColonySkin {
  float skin;          // skin of the current lists
  float half2;         // (skin / 2)^2, the displacement guard
  int need;            // rebuild requests: 1 guard, 2 fresh overflow, 4 cadence, 8 host
  int rebuild_now;     // this step rebuilds the lists
  int steps_since;     // steps since the last list rebuild
  int interval;        // cadence in steps (0: guard only)
  int nfresh;          // entries in the fresh list
  int nrebuild;        // list rebuilds so far
  int ntrip;           // rebuilds requested by the guard
  unsigned maxdisp2;   // largest |u - uref|^2 of the last step (float bits)
  int list_overflow;   // elements whose list was truncated at the last build
  int last_interval;   // steps between the last two rebuilds
  long long npairs;    // list entries at the last build
  int nslot_built;     // used slots at the last build (the flattened lists cover these)
};

// The force pass's displacement statistics of a colony, spread over kStatSlots slots (slot =
// block index mod kStatSlots) so that the blocks' closing atomics do not all meet on one
// address; k_skin_begin folds and clears them at the next step.
constexpr int kStatSlots = 32;
struct StatPart {
  unsigned dmax;  // largest |u - uref|^2 (float bits)
  unsigned smax;  // largest |step displacement| (float bits)
  float ssum;     // sum of |step displacement|
  int pad;
};

// Inputs of the learned skin scheduler, maintained on the device per colony in skin mode.
// The 12 features are formed by k_skin_begin at every list rebuild (before the statistics
// of the new build are reset); the scheduler network (k_skin_begin) turns them into the colony's next skin and
// rebuild cadence.
constexpr int kSchedFeatures = 12;
struct SchedState {
  float occ_sum;          // sum over elements of their home-bin occupancy at the last list build
  int occ_count;          // elements counted into occ_sum
  float occ_max;          // largest bin occupancy at the last list build (float bits, atomicMax)
  float step_sum;         // sum over elements of |displacement| in the last step
  float step_max;         // largest |displacement| in the last step (float bits, atomicMax)
  float div_rate;         // divisions per cell per step, moving average over ~100 steps
  float apo_rate;         // apoptoses per cell per step, moving average over ~100 steps
  float trip_share;       // share of guard-triggered rebuilds, moving average over ~10 rebuilds
  long long ndiv_prev, napo_prev;
  int nsched;             // scheduler decisions taken
  int pad;
  float features[kSchedFeatures];  // input of the last decision
};

// 2D skin mode: an element's list reference rides in the record's unused z word as two 16-bit
// fixed-point fractions of the bin width (resolution bw / 65535; list references lie in the
// home bin, [0, bw)). The displacement guard allows for the rounding (uref_margin).
struct ColonyConst;
__device__ __forceinline__ float uref_pack2(const float *scale, float u0, float u1) {
  const float a = fminf(fmaxf(rintf(u0 * scale[0]), 0.0f), 65535.0f);
  const float b = fminf(fmaxf(rintf(u1 * scale[1]), 0.0f), 65535.0f);
  return __uint_as_float(static_cast<unsigned>(a) | (static_cast<unsigned>(b) << 16));
}
__device__ __forceinline__ void uref_unpack2(const float *inv, float z, float *r) {
  const unsigned v = __float_as_uint(z);
  r[0] = static_cast<float>(v & 0xffffu) * inv[0];
  r[1] = static_cast<float>(v >> 16) * inv[1];
}

// Mixed precision keeps each element as one 16-byte record, so a pair costs one load:
//   xyz  FP32 coordinates relative to the origin of the element's home bin (sbin)
//   w    FP32 diameter; in skin mode negative for elements the Verlet lists must skip
//        (fresh: moved or created by a division since the last build; dead: tombstone)
__device__ __forceinline__ float pk_c(const float4 &p, int d) { return d == 0 ? p.x : (d == 1 ? p.y : p.z); }
__device__ __forceinline__ void pk_set(float4 &p, int d, float v) {
  if (d == 0)
    p.x = v;
  else if (d == 1)
    p.y = v;
  else
    p.z = v;
}

struct ColonyConst {
  double box[3];
  double ih[3];      // 1/L, as the reference binning formula uses (Utils.hpp:990)
  double bw[3];      // bin width L/Ns
  int ns[3];         // bins per axis (1 on unused axes)
  // bin-id decoding without hardware division: q = n / div_d[k] for the two divisors
  // (2D: ns1; 3D: ns1*ns2 and ns2) by multiply-high with an invariant (Granlund and
  // Montgomery, "Division by invariant integers using multiplication", PLDI 1994, fig. 4.1)
  uint32_t div_m[2], div_s1[2], div_s2[2];
  // 2D skin mode: 16-bit fixed-point list reference (fraction of the bin width per axis)
  float uq_scale[2], uq_inv[2];
  int periodic[3];
  int single_bin;    // grid collapsed to one bin (some Ns < 3, Utils.hpp:897-901)
  int bin_base;      // first global bin
  int nbins;         // real bins
  int nbins_pad;     // bins rounded up to kScanItems
  int scan_base;     // first scan block
  int slot_base, slot_cap;
  int cell_base, cell_cap;
  int due_base;      // the colony's part of the due-cell queue (a power of two >= cell_cap)
  int force_law;
  int noise_per_cell;
  uint32_t rng_stream;  // the colony's Philox stream (cil_config.rng_stream_base + colony index)
  int divide;
  int nwalls;
  int wall_dir[2];
  double wall_pos[2];
  double wall_E;
  double epsilon;
  double rcut_scale;
  double zeta[2];
  double temp[2];    // dt / zeta, the integrator's `temp` (CIL.cu:864)
  double mu_eff[2];  // temp / dt, the velocity factor (CIL.cu:935)
  double motility[2];
  double kappa;
  double rest0, rest1;
  double noise_amp;  // sqrt(2 D) / sqrt(dt)
  double dt;
  double div_tau_mu, div_tau_sigma;
  double apop_p;     // apoptosis probability per step
  float apop_log1m_p;  // log(1 - apop_p) (FP32 binomial draw of the fast mode)
  float tau_mu_steps_f, tau_sd_steps_f;  // division time mean and sd in steps (FP32 draws)
  // FP32 copies for the mixed-precision kernel (GB300 runs FP64 at ~1/64 of FP32, so the
  // mixed kernel keeps every per-element operation but the position update in FP32)
  float bwf[3];      // bin widths
  float inv_bwf[3];  // 1 / bin width
  float zeta_f[2], temp_f[2], mu_f[2], motility_f[2];
  float kappa_f, rest0_f, rest1_f, amp_f, eps_f, rcs_f, wall_E_f;
  // CIL_FORCE_SC: well depth and width, shifted force (FP64 and FP32 copies)
  double well_eps, well_sigma;
  float well_eps_f, well_sigma_f;
  int force_shifted;
  float wall_pos_f[2];
  // CIL_INTRA_FENE: the reference's bond of a crawling cell (FP64 and FP32 copies); rss is the
  // steady-state length of Input.cpp:139-144
  int intra_fene, cil;
  double fene_kappa, fene_kappa_push, fene_ratio, fene_r2max, fene_rss;
  float fene_kappa_f, fene_kappa_push_f, fene_ratio_f, fene_r2max_f, fene_rss_f;
  // the reference's crawling/dividing cells (CIL_INTRA_FENE with divide): RMAX_DIVISION^2,
  // growth activities, Rmin^2 and its ratio form, the reorientation radius of a division
  // (R0; half the birth rest length otherwise) and the diameters a division resets to
  int cell_sm;
  double fene_r2max_div, growth_k0[2], growth_k1[2], growth_k2[2], div_r2min, div_rmin_ratio;
  float fene_r2max_div_f, growth_k0_f[2], growth_k1_f[2], growth_k2_f[2], div_r2min_f;
  double div_radius, sigma_core[2];
  int act_noise;  // the bond's active noise (2D, uploaded with the passive noise)
  int dim;
  float mig_mu_steps_f, mig_sd_steps_f;  // migration time mean and sd in steps (Philox draws)
  int swelling;  // crawling/dividing cells with SWELLING
};

// Cell states of the reference's two-element cells (CellState, Cell.cuh:26-30)
constexpr int kCellDividing = 0, kCellCrawling = 1, kCellUndefined = 2;

// The bond's active noise (binaryCellForce, MD.cu:573-579; 2D): rnd = (Wr r_x / r - Wt r_y,
// Wr r_y / r + Wt r_x) / 2, which the bond term adds as rnd_d r_ij,d.
template <int D, typename R>
__device__ __forceinline__ void bond_noise(R wr, R wt, const R *rij, R r, R *rnd) {
  if (D != 2) return;
  rnd[0] = R(0.5) * (wr * rij[0] / r - wt * rij[1]);
  rnd[1] = R(0.5) * (wr * rij[1] / r + wt * rij[0]);
}

// The bond of a dividing cell (binaryCellForce, MD.cu:545-567): r2max from RMAX_DIVISION, the
// growth activities act_j = -k0_j feneDivMax + k1_j + k2_j r^4 with feneDivMax = FENE(r2max,
// Rmin^2), the bond acting once: F_back = -(act_0 + spring) rij, F_front = (act_1 + spring) rij.
template <typename R>
__device__ __forceinline__ void fene_bond_dividing(R r2, R smax, R r2max_div, R kappa, R kpush, R ratio, R r2min,
                                                   const R *k0, const R *k1, const R *k2, R &spring, R *act) {
  const R r2max = r2max_div > smax ? r2max_div : smax;
  const R lim = r2max * ratio;
  if (r2 <= lim) {
    spring = kpush * fabs(r2 - lim);
  } else {
    const R q = (r2 - lim) / (r2max * (R(1) - ratio));
    spring = -kappa / (R(1) - q * q);
  }
  const R qd = r2min / r2max;
  const R fdm = -kappa / (R(1) - qd * qd);
  act[0] = -k0[0] * fdm + k1[0] + k2[0] * (r2 * r2);
  act[1] = -k0[1] * fdm + k1[1] + k2[1] * (r2 * r2);
}

// The reference's bond of a crawling two-element cell (binaryCellForce, MD.cu:525-598): the
// magnitude `spring` of the bond term spring * rij * 2 (rij = r_front - r_back, strongContract
// = 2) and the scale s of the motility direction nij = rij * s. r2max = max(RMAX^2, the larger
// element diameter) (MD.cu:547-548); below spring_ratio * r2max the push spring
// kappa_push |r2 - r2max ratio| (Spring, MD.cu:263-265), above it FENE(kappa, r2max (1 - ratio),
// r2 - r2max ratio) = -kappa / (1 - q^2) (MD.cu:255-257, 553-558); s = 1 with contact inhibition,
// rss / r without (MD.cu:568-571). The forces are F_back = -(m0 nij + spring rij 2) and
// F_front = m1 nij + spring rij 2.
template <typename R>
__device__ __forceinline__ void fene_bond(R r2, R r, R smax, R r2max0, R kappa, R kpush, R ratio, R rss, int cil,
                                          R &spring, R &s) {
  const R r2max = r2max0 > smax ? r2max0 : smax;
  const R lim = r2max * ratio;
  if (r2 <= lim) {
    spring = kpush * fabs(r2 - lim);
  } else {
    const R q = (r2 - lim) / (r2max * (R(1) - ratio));
    spring = -kappa / (R(1) - q * q);
  }
  s = cil ? R(1) : rss / r;
}

struct ColonyCounters {
  int ncell;          // live cells
  int nslot;          // used slots (live + tombstones + appended daughters)
  int nlive;          // elements sorted into bins by the last rebuild
  int err;            // error bits
  int ndiv_step;      // divisions this step
  int ndead;          // apoptoses recorded this step (list length, may exceed kDeadCap)
  int ndiv_allowed;   // divisions that fit the capacity this step
  int ndue;           // skin mode, Philox: cells due to divide at the coming events (force kernel)
  long long ndiv_total;
  long long napo_total;
};

// ---------------------------------------------------------------- small device helpers

// Utils.hpp:173-175
__host__ __device__ __forceinline__ int nint(double a) {
  return a >= 0.0 ? static_cast<int>(a + 0.5) : static_cast<int>(a - 0.5);
}

// fmod(t + L, L) for t in [-L, 2L) without a division: every branch is an exact
// subtraction (Sterbenz), so the result equals the reference's updatePos wrap
// (Utils.hpp:561-566) bit for bit.
__device__ __forceinline__ double wrap_like_fmod(double t, double L) {
  const double t2 = __dadd_rn(t, L);
  if (t2 >= L + L) return t2 - (L + L);
  if (t2 >= L) return t2 - L;
  if (t2 >= 0.0) return t2;
  return fmod(t2, L);
}

// Colony of a tile: tile_base[c] <= t < tile_base[c+1]
__device__ __forceinline__ int colony_of_tile(const int *__restrict__ tile_base, int B, int t) {
  int lo = 0, hi = B - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(tile_base + mid) <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Coordinates of a colony-local bin id (LinkListOrtho2D/3D::get_cellCoord,
// Utils.hpp:1029-1061)
__host__ __device__ __forceinline__ uint32_t div_invariant(uint32_t n, uint32_t m, uint32_t s1, uint32_t s2) {
#ifdef __CUDA_ARCH__
  const uint32_t t1 = __umulhi(m, n);
#else
  const uint32_t t1 = static_cast<uint32_t>((static_cast<uint64_t>(m) * n) >> 32);
#endif
  return (t1 + ((n - t1) >> s1)) >> s2;
}

// host: the invariant (m, s1, s2) of divisor d >= 1
inline void div_invariant_setup(uint32_t d, uint32_t *m, uint32_t *s1, uint32_t *s2) {
  uint32_t l = 0;
  while (l < 32 && (1ull << l) < d) ++l;  // ceil(log2 d)
  *m = static_cast<uint32_t>(((1ull << 32) * ((1ull << l) - d)) / d + 1);
  *s1 = l < 1 ? l : 1;
  *s2 = l > 0 ? l - 1 : 0;
}

template <int D>
__device__ __forceinline__ void bin_decode(const ColonyConst &C, int id, int *b) {
  const uint32_t u = static_cast<uint32_t>(id);
  if (D == 2) {
    b[0] = static_cast<int>(div_invariant(u, C.div_m[0], C.div_s1[0], C.div_s2[0]));
    b[1] = id - b[0] * C.ns[1];
  } else {
    b[0] = static_cast<int>(div_invariant(u, C.div_m[0], C.div_s1[0], C.div_s2[0]));
    const int r = id - b[0] * (C.ns[1] * C.ns[2]);
    b[1] = static_cast<int>(div_invariant(static_cast<uint32_t>(r), C.div_m[1], C.div_s1[1], C.div_s2[1]));
    b[2] = r - b[1] * C.ns[2];
  }
}

// Exact float -> double conversion with integer operations only (no FP64 pipe): finite
// normal values are re-biased bit for bit; zeros and subnormals give a signed zero (a
// displacement below 1.2e-38 leaves any position unchanged); inf and NaN keep their class.
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t ex = (b >> 23) & 0xffu;
  const uint64_t sign = static_cast<uint64_t>(b & 0x80000000u) << 32;
  const uint64_t mant = static_cast<uint64_t>(b & 0x7fffffu) << 29;
  const uint64_t e64 = ex == 0u ? 0u : (ex == 0xffu ? 0x7ffu : ex - 127u + 1023u);
  const uint64_t d = sign | (e64 << 52) | (ex == 0u ? 0u : mant);
  return __longlong_as_double(static_cast<long long>(d));
}

// Bin coordinates of a position (LinkListOrtho::populate_list, Utils.hpp:990), clamped
// to the grid along non-periodic axes.
template <int D>
__device__ __forceinline__ void bin_coords(const ColonyConst &C, const double *x, int *b) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    int v = static_cast<int>(__dmul_rn(__dmul_rn(x[d], C.ih[d]), static_cast<double>(C.ns[d])));
    v = v < C.ns[d] - 1 ? v : C.ns[d] - 1;
    b[d] = v > 0 ? v : 0;
  }
}

template <int D>
__device__ __forceinline__ int bin_id(const ColonyConst &C, const int *b) {
  return D == 2 ? b[0] * C.ns[1] + b[1] : (b[0] * C.ns[1] + b[1]) * C.ns[2] + b[2];
}

// ---------------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3" (SC'11): 10 rounds of the 4x32 Philox S-box with the published
// multipliers and Weyl key increments.
struct u32x4 {
  uint32_t v[4];
};

__host__ __device__ __forceinline__ u32x4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                         uint32_t c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = static_cast<uint64_t>(M0) * c0;
    const uint64_t p1 = static_cast<uint64_t>(M1) * c2;
    const uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
    const uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  u32x4 o;
  o.v[0] = c0;
  o.v[1] = c1;
  o.v[2] = c2;
  o.v[3] = c3;
  return o;
}

// two standard normals from two 32-bit words (Box-Muller), FP32
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float &n0, float &n1) {
  const float u1 = static_cast<float>((a >> 8) + 1u) * 5.9604644775390625e-08f;  // (0, 1]
  const float u2 = static_cast<float>(b >> 8) * 5.9604644775390625e-08f;         // [0, 1)
  const float r = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  n0 = r * c;
  n1 = r * s;
}

// Philox words of the passive noise of element e = 2 g + j (colony-local ids) at step ts; the
// fourth counter word carries the colony's random stream (stream << 1, plus 1 for the 2D
// per-element blocks), so a colony draws the same numbers whether it runs alone or in a batch.
//   per element (noise_per_cell 0): in 2D one block keyed by the cell, (g, ts, noise, 2 stream + 1),
//     serves both of its elements: element j takes words 2j and 2j + 1 (one Box-Muller pair);
//     in 3D each element takes a block of its own, (e, ts, noise, 2 stream) (two pairs).
//   per cell (noise_per_cell 1, the reference's passiveWiener[cell][dim]): in 2D one block
//     (g, ts / 2, noise, 2 stream) serves two consecutive steps (the even step takes words 0-1,
//     the odd one 2-3); in 3D each step takes the block (g, ts, noise, 2 stream).
// Every force kernel draws through these two functions, so the forms agree on the noise.
template <int D>
__device__ __forceinline__ void noise_words(int e, int per_cell, int ts, uint32_t stream, uint32_t klo, uint32_t khi,
                                            uint32_t *w) {
  const uint32_t g = static_cast<uint32_t>(e) >> 1;
  if (D == 2) {
    const bool sel = per_cell ? (ts & 1) != 0 : (e & 1) != 0;
    const u32x4 r = per_cell ? philox4x32_10(g, static_cast<uint32_t>(ts) >> 1, kRngNoise, stream << 1, klo, khi)
                             : philox4x32_10(g, static_cast<uint32_t>(ts), kRngNoise, (stream << 1) | 1u, klo, khi);
    w[0] = sel ? r.v[2] : r.v[0];
    w[1] = sel ? r.v[3] : r.v[1];
  } else {
    const u32x4 r = philox4x32_10(per_cell ? g : static_cast<uint32_t>(e), static_cast<uint32_t>(ts), kRngNoise,
                                  stream << 1, klo, khi);
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = r.v[q];
  }
}

// The words of both elements of cell g (colony-local) at once (w0: back element, w1: front
// element), one Philox block per cell and step in 2D; the same values noise_words gives each
// element.
template <int D>
__device__ __forceinline__ void noise_words_cell(int g, int per_cell, int ts, uint32_t stream, uint32_t klo,
                                                 uint32_t khi, uint32_t *w0, uint32_t *w1) {
  if (D == 2) {
    if (per_cell) {
      const u32x4 r = philox4x32_10(static_cast<uint32_t>(g), static_cast<uint32_t>(ts) >> 1, kRngNoise, stream << 1,
                                    klo, khi);
      const bool odd = (ts & 1) != 0;
      w0[0] = w1[0] = odd ? r.v[2] : r.v[0];
      w0[1] = w1[1] = odd ? r.v[3] : r.v[1];
    } else {
      const u32x4 r = philox4x32_10(static_cast<uint32_t>(g), static_cast<uint32_t>(ts), kRngNoise,
                                    (stream << 1) | 1u, klo, khi);
      w0[0] = r.v[0];
      w0[1] = r.v[1];
      w1[0] = r.v[2];
      w1[1] = r.v[3];
    }
  } else if (per_cell) {
    noise_words<D>(2 * g, 1, ts, stream, klo, khi, w0);
#pragma unroll
    for (int q = 0; q < 4; ++q) w1[q] = w0[q];
  } else {
    noise_words<D>(2 * g, 0, ts, stream, klo, khi, w0);
    noise_words<D>(2 * g + 1, 0, ts, stream, klo, khi, w1);
  }
}

// [0, 1) with 53 random bits
__device__ __forceinline__ double uniform53(uint32_t a, uint32_t b) {
  const uint64_t m = (static_cast<uint64_t>(a) << 21) ^ (static_cast<uint64_t>(b) >> 11);
  return static_cast<double>(m & ((1ull << 53) - 1)) * 1.1102230246251565e-16;
}

// ---------------------------------------------------------------- pair force laws
// Force modulus f0 with F_i += f0 * (r_j - r_i); returns false outside the cutoff.
// LJ-WCA is the reference's LJParams::elemForce0 form (MD.cuh:50-56, 98-113).
// The reference soft-core cubic well's elemForce0 (MD.cuh:144-162): y = r - sigma_ij,
// t'(y, xi) = 6 y (xi - y) / xi^3.
template <typename R>
__device__ __forceinline__ R sc_force0(R r, R sij, R e0, R em, R xi) {
  const R y = r - sij;
  if (y <= -xi) return R(0);
  if (y < R(0)) return -(e0 + em) * (R(6) * (-y) * (y + xi) / (xi * xi * xi)) / r;
  if (y < xi) return em * (R(6) * y * (-y + xi) / (xi * xi * xi)) / r;
  return R(0);
}

// The bare Lennard-Jones modulus (s^6 - 2 s^12) / r^2 with s^2 = sij2 / r2 (MD.cuh:50-56).
template <typename R>
__device__ __forceinline__ R lj_force0(R sij2, R r2) {
  const R ir2 = R(1) / r2;
  R sr2n = sij2 * ir2;
  const R srn = sr2n * sr2n * sr2n;
  sr2n = srn * srn;
  return (srn - R(2) * sr2n) * ir2;
}

template <int LAW, typename R>
__device__ __forceinline__ bool pair_force(R r2, R si, R sj, R eps, R rcs, R &f0, R em = R(0), R xi = R(0),
                                           int shifted = 0) {
  const R sij = R(0.5) * (si + sj);
  if (LAW == CIL_FORCE_SC) {
    // SCParams::elemForce (MD.cuh:199-214): rcut2 (sigma_ij -+ xi)^2 bound the force
    const R rc2 = rcs * rcs * ((sij + xi) * (sij + xi));
    if (r2 > rcs * rcs * ((sij - xi) * (sij - xi)) && r2 <= rc2) {
      f0 = sc_force0(sqrt(r2), sij, eps, em, xi) - (shifted ? sc_force0(sqrt(rc2), sij, eps, em, xi) * sqrt(rc2 / r2) : R(0));
      return true;
    }
    return false;
  }
  if (LAW == CIL_FORCE_LJ_WCA) {
    // LJParams::elemForce (MD.cuh:72-92): (f(r2) - [shifted] f(rc2) sqrt(rc2 / r2)) 24 eps
    const R sij2 = sij * sij;
    const R rc2 = sij2 * (rcs * rcs);
    if (r2 <= rc2) {
      f0 = (lj_force0(sij2, r2) - (shifted ? lj_force0(sij2, rc2) * sqrt(rc2 / r2) : R(0))) * (R(24) * eps);
      return true;
    }
    return false;
  } else {
    const R rc = rcs * sij;
    if (r2 < rc * rc && r2 > R(0)) {
      const R r = sqrt(r2);
      if (LAW == CIL_FORCE_SOFTCORE) {
        const R w = R(1) - r / rc;
        f0 = -eps * w * w / r;
      } else {
        const R delta = sij - r;
        f0 = -eps * delta * sqrt(delta) / r;
      }
      return true;
    }
    return false;
  }
}

// The range test of pair_force alone (the same expressions, so the same answer).
template <int LAW, typename R>
__device__ __forceinline__ bool pair_in_range(R r2, R si, R sj, R rcs, R xi) {
  const R sij = R(0.5) * (si + sj);
  if (LAW == CIL_FORCE_SC)
    return r2 > rcs * rcs * ((sij - xi) * (sij - xi)) && r2 <= rcs * rcs * ((sij + xi) * (sij + xi));
  if (LAW == CIL_FORCE_LJ_WCA) return r2 <= (sij * sij) * (rcs * rcs);
  const R rc = rcs * sij;
  return r2 < rc * rc && r2 > R(0);
}

// A superset of pair_in_range in FP32, for a squared separation r2f within a relative 1e-6 of
// the FP64 one: the bounds are widened by 1e-5, so every pair that pair_force accepts passes.
template <int LAW>
__device__ __forceinline__ bool pair_maybe_in_range(float r2f, float si, float sj, float rcs, float xi) {
  const float sij = 0.5f * (si + sj);
  constexpr float up = 1.00001f, dn = 0.99999f;
  if (LAW == CIL_FORCE_SC)
    return r2f >= dn * (rcs * rcs * ((sij - xi) * (sij - xi))) && r2f <= up * (rcs * rcs * ((sij + xi) * (sij + xi)));
  const float rc = rcs * sij;
  return r2f <= up * (rc * rc);
}

// FP32 pair force, branch-free: the law is evaluated for every candidate and masked
// (fast reciprocal / reciprocal square root; the mixed form's tolerance is FP32-level)
template <int LAW>
__device__ __forceinline__ float pair_f0_fast(float r2, float si, float sj, float eps, float rcs, bool ok,
                                              float em = 0.0f, float xi = 0.0f, int shifted = 0) {
  const float sij = 0.5f * (si + sj);
  const float rc = rcs * sij;
  if (LAW == CIL_FORCE_SC) {
    const float rc2 = rcs * rcs * ((sij + xi) * (sij + xi));
    const bool in = ok && r2 > rcs * rcs * ((sij - xi) * (sij - xi)) && r2 <= rc2 && r2 > 0.0f;
    const float rinv = rsqrtf(r2);
    float f = sc_force0(r2 * rinv, sij, eps, em, xi);
    if (shifted) f -= sc_force0(sqrtf(rc2), sij, eps, em, xi) * sqrtf(rc2) * rinv;
    return in ? f : 0.0f;
  }
  if (LAW == CIL_FORCE_LJ_WCA) {
    const bool in = ok && r2 <= rc * rc;
    const float ir2 = __fdividef(1.0f, r2);  // fast reciprocal (about 2 ulp)
    const float sr2 = sij * sij * ir2;
    const float sr6 = sr2 * sr2 * sr2;
    float f = sr6 - 2.0f * sr6 * sr6;
    if (shifted) {
      // f(rc) sqrt(rc^2 / r^2) / r^2 with (sigma / rc)^2 = 1 / rcs^2:
      // (c6 - 2 c6^2) / (rc r^3), the r^-2 factor taken out below
      const float c2 = __fdividef(1.0f, rcs * rcs);
      const float c6 = c2 * c2 * c2;
      f -= (c6 - 2.0f * c6 * c6) * sqrtf(r2) * __fdividef(1.0f, rc);
    }
    return in ? f * ir2 * (24.0f * eps) : 0.0f;
  } else if (LAW == CIL_FORCE_SOFTCORE) {
    // -eps (1 - r/rc)^2 / r from one reciprocal square root: q = 1 / (r rc) gives
    // r / rc = r2 q and 1 / r = rc q
    const float rc2 = rc * rc;
    const bool in = ok && r2 < rc2 && r2 > 0.0f;
    const float q = rsqrtf(r2 * rc2);
    const float w = 1.0f - r2 * q;
    return in ? -eps * w * w * (rc * q) : 0.0f;
  } else {
    const bool in = ok && r2 < rc * rc && r2 > 0.0f;
    const float rinv = rsqrtf(r2);
    const float r = r2 * rinv;
    const float delta = fmaxf(sij - r, 0.0f);
    const float sq = delta * rsqrtf(fmaxf(delta, 1e-30f));
    return in ? -eps * delta * sq * rinv : 0.0f;
  }
}

// The largest distance at which the law acts between elements of diameters si, sj (the Verlet
// lists add the skin to it).
template <int LAW>
__device__ __forceinline__ float law_cutoff_f(const ColonyConst &C, float si, float sj) {
  const float sij = 0.5f * (si + sj);
  return LAW == CIL_FORCE_SC ? C.rcs_f * (sij + C.well_sigma_f) : C.rcs_f * sij;
}

// ---------------------------------------------------------------- kernel argument packs

struct RebuildArgs {
  const ColonyConst *col;
  ColonyCounters *cnt;
  int B;
  size_t SS;               // slot stride of SoA arrays
  const int *tiles_used;   // [B+1] tiles over nslot (before the rebuild)
  const int *tiles_live;   // [B+1] tiles over nlive (after the scan)
  const int *tiles_cell;   // [B+1] tiles over ncell (cell re-sort of skin mode)
  const int *scan_col;     // scan block -> colony
  int nscan;               // scan blocks
  const double *x_in;
  const double *sig_in;    // binned FP64 diameters (FP64 form), may be null
  const int *eid_in;
  double *x_out;
  double *sig_out;
  int *eid_out;
  float4 *pk_out;          // mixed: packed elements of the new order, may be null
  const float4 *pk_in;     // mixed: packed elements after the last update (relative to sbin_in)
  const int *sbin_in;      // home bin (colony-local id) of each slot
  int *sbin_out;
  const int2 *cyc_in;      // (birth step, division step) of each slot's cell
  int2 *cyc_out;
  const double *sigma_c;   // canonical diameters [2 * CC]
  const int *t0c;          // canonical cycle arrays [CC]
  const int *tswc;
  int exact;               // 1: reference FP64 bin formula and canonical gathers
  const ColonySkin *skin;  // skin mode: colonies without rebuild_now are skipped; else null
  const int *any_rebuild;  // skin mode: [2] per step parity, 0 = no colony rebuilds (kernels return); else null
  const int *ts_dev;
  int permute;             // 1: slots are re-sorted (data moves); 0: only the bin index is rebuilt
  unsigned char *state_out;// skin mode, permuting: slot states of the new order
  int *key;
  int *bcount;
  int2 *range;
  unsigned long long *perm;
  int *scan_sum;
  int *scan_off;
  int *slot_of;
  const double *vel_in;    // optional: carry velocities through the permutation
  double *vel_out;
  int dim;
};

struct ForceArgs {
  const ColonyConst *col;
  ColonyCounters *cnt;
  int B;
  size_t SS;
  const int *cst;          // cell states (the crawling/dividing cells' bond)
  const int *tiles_live;
  const double *x_in;      // sorted positions
  double *x_out;           // integrated positions (same slots)
  const double *sig;       // FP64 form
  const int *eid;
  const float4 *pk;        // mixed: packed elements of this step
  float4 *pk_next;         // mixed: packed elements after the update (same slots)
  const int *sbin;         // home bin of each slot
  const int2 *cyc;         // cycle of each slot's cell
  const int2 *range;
  const int *slot_of;
  // skin mode (null otherwise)
  const int *tiles;        // skin mode: tiles over slot pairs (k_force_cells)
  ColonySkin *skin;
  const int *nbr;          // Verlet lists [kListCap][SS]
  const int *ncnt;
  // the lists per warp of 32 cells (64 slots from w0), flattened: entries and their owners
  // (element of the warp) at w0 * kListCap, element starts per slot, entries per warp
  const int *lflat;
  const unsigned char *oflat;
  const unsigned short *lstart;
  const int *lwarp;
  const float *uref;       // 3D only (2D: packed in the record's z word)
  float *facc;             // pair forces of fresh elements / reactions [D][SS], consumed and zeroed
  unsigned *ftouch;        // one bit per slot: facc holds a contribution
  SchedState *sched;       // speed statistics for the scheduler
  StatPart *spart;         // [B][kStatSlots] displacement statistics of this pass
  const double *noise;     // oracle mode: uploaded normals (already scaled), canonical order
  const double *noise_act; // oracle mode: the bond's active noise per cell, radial
  const double *noise_act_t;  //   and angular
  double *vel;             // slot order, may be null
  const double *vel_prev;  // Heun second half step: the first half's velocities (null: vel itself)
  double *frc;             // slot order, may be null
  const int *ts_dev;       // device step counter: the step being computed
  int ts;                  // filled from *ts_dev at kernel entry
  uint32_t seed_lo, seed_hi;
  int noise_mode;          // 0 none, 1 philox, 2 uploaded
  int integrate;
  int heun;                // 0 Euler step; 1, 2: first, second half step of a Heun step
  // skin mode, Philox, the step's last force pass: cells due to divide at step ts + 1 are
  // appended to the colony's due-cell queue (dueq + col[c].due_base, count cnt[c].ndue)
  int collect_due;
  int *dueq;
};

// Half-step helpers of the Heun integrator (CIL_INTEGRATOR_HEUN): the Philox noise index of
// a force pass (the two passes of step ts take 2 ts and 2 ts + 1, one Philox block per step
// in 2D), and the step fraction of its position update.
__device__ __forceinline__ int noise_index(int ts, int heun) { return heun ? 2 * ts + (heun - 1) : ts; }

struct EventArgs {
  const ColonyConst *col;
  ColonyCounters *cnt;
  int B;
  size_t SS;
  const int *tiles_cell;   // [B+1] tiles over ncell
  double *x;               // current positions
  double *sig;             // binned FP64 diameters (FP64 form) or null
  float4 *pk;              // mixed: packed elements (after this step's update), or null
  int *sbin;
  int2 *cyc;
  double *sigma_c;         // canonical diameters
  // skin mode (null otherwise)
  ColonySkin *skin;
  unsigned char *state;
  float *uref;
  int *ncnt;
  int *fresh;              // [B][kFreshCap]
  unsigned long long *fhead;  // per bin: newest fresh slot of the current list epoch (epoch << 32 | slot)
  unsigned long long *fnext;  // per slot: the entry it displaced (a linked list per bin)
  int *eid;
  double *vel;             // may be null
  int *slot_of;
  int *t0;
  int *tsw;
  int *cst;                // cell states (crawling/dividing cells)
  unsigned char *smflag;   // per cell: the division criterion is met (oracle mode, state machine)
  int *tile_count;
  int *tile_off;
  // skin mode, Philox: the cells due to divide, appended by the force kernel (colony c's at
  // dueq + col[c].due_base, count cnt[c].ndue), and the event kernel's finished-colony count
  int *dueq;
  int *ev_done;
  int *any_rebuild;        // the any-rebuild flags (the next step's is cleared)
  int *dead;               // [B * kDeadCap]
  int *divq;               // [CC] per colony: the cells dividing this step, in rank order
  double *obs_com_prev;    // [D * CC] or null
  double *obs_disp;
  double *obs_vref;
  size_t CC;
  int *ts_dev;             // device step counter (advanced past the force step, or by k_events_due)
  int ts;                  // filled from *ts_dev at kernel entry
  uint32_t seed_lo, seed_hi;
};

struct SkinArgs {
  const ColonyConst *col;
  ColonyCounters *cnt;
  ColonySkin *skin;
  SchedState *sched;       // scheduler inputs (always maintained in skin mode)
  StatPart *spart;         // [B][kStatSlots] the last force pass's displacement statistics
  int B;
  size_t SS;
  const int *tiles;        // tiles over nslot
  const int *eid;
  unsigned char *state;
  float4 *pk;              // current packed elements (rebinned in place)
  float *uref;
  int *sbin;
  const int2 *range;
  const unsigned long long *perm;
  int *nbr;
  int *ncnt;
  int *lflat;              // flattened lists per warp of 32 cells (see ForceArgs)
  unsigned char *oflat;
  unsigned short *lstart;
  int *lwarp;
  const int *fresh;
  const unsigned long long *fhead;
  const unsigned long long *fnext;
  float *facc;
  unsigned *ftouch;        // one bit per slot: facc holds a contribution
  int *key;
  int *bcount;
  int force_rebuild;       // host request for every colony this step
  int grid;                // blocks of the fresh-pair kernel
  const int *ts_dev;       // device step counter
  int *any_rebuild;        // [4]: [ts & 1] some colony rebuilds at step ts; [2] colonies decided
                           // this step; [3] steps whose rebuild node ran (or null)
  // graph replay: the conditional (IF) node around the rebuild kernels of the step; the
  // colony that decides last sets it to "some colony rebuilds" (use_cond 0: no node)
  int use_cond;
  cudaGraphConditionalHandle cond;
  // k_skin_begin also writes the step's tile tables over the slots and the slot pairs when these
  // are set (pair tiles of pair_tile slots), or null
  int *tiles_used_out;
  int *tiles_pairs_out;
  int pair_tile;
  // learned scheduler (null: skin and cadence stay as set)
  const float *mlp;
  int use_interval;
  float skin_min, skin_max, interval_scale;
};

// ---------------------------------------------------------------- scheduler network
// 12 -> 64 -> 64 -> 2 multilayer perceptron, SiLU, FP32; one flat parameter vector
//   W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
constexpr int kMlpIn = 12, kMlpH = 64, kMlpOut = 2;
constexpr int kMlpW1 = 0, kMlpB1 = kMlpW1 + kMlpH * kMlpIn, kMlpW2 = kMlpB1 + kMlpH,
              kMlpB2 = kMlpW2 + kMlpH * kMlpH, kMlpW3 = kMlpB2 + kMlpH, kMlpB3 = kMlpW3 + kMlpOut * kMlpH,
              kMlpParams = kMlpB3 + kMlpOut;

__device__ __forceinline__ float mlp_silu(float z) { return z / (1.0f + expf(-z)); }

// The network on one input, evaluated by one whole warp (every lane calls it): lane l owns
// hidden units l and l + 32; every lane holds x; both outputs are returned to all lanes.
// Weights are read from global memory (they stay in L2).
__device__ __forceinline__ void mlp_forward_warp(const float *__restrict__ w, const float *x, float *y) {
  const int lane = threadIdx.x & 31;
  float h1[2], h2[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int u = lane + 32 * q;
    float z = __ldg(w + kMlpB1 + u);
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) z += __ldg(w + kMlpW1 + u * kMlpIn + k) * x[k];
    h1[q] = mlp_silu(z);
  }
  float z2[2] = {__ldg(w + kMlpB2 + lane), __ldg(w + kMlpB2 + lane + 32)};
  for (int v = 0; v < kMlpH; ++v) {
    const float hv = __shfl_sync(0xffffffffu, v < 32 ? h1[0] : h1[1], v & 31);
#pragma unroll
    for (int q = 0; q < 2; ++q) z2[q] += __ldg(w + kMlpW2 + (lane + 32 * q) * kMlpH + v) * hv;
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) h2[q] = mlp_silu(z2[q]);
#pragma unroll
  for (int o = 0; o < kMlpOut; ++o) {
    float part = __ldg(w + kMlpW3 + o * kMlpH + lane) * h2[0] + __ldg(w + kMlpW3 + o * kMlpH + lane + 32) * h2[1];
#pragma unroll
    for (int q = 16; q > 0; q >>= 1) part += __shfl_xor_sync(0xffffffffu, part, q);
    y[o] = part + __ldg(w + kMlpB3 + o);
  }
}



// ---------------------------------------------------------------- launchers (host side)
// which2 / tiles2: a second table in the same launch; per2: slots per tile of a which2 = 3 table
void launch_tiles(const ColonyConst *col, ColonyCounters *cnt, int B, int which, int *tiles,
                  cudaStream_t s, int which2 = 0, int *tiles2 = nullptr, int per2 = 2 * kTile);
void launch_rebuild(const RebuildArgs &a, int grid_slots, cudaStream_t s);
// skin mode: slots re-sorted by cell (cells ranked by the bin of their back element, a cell's
// elements in the slot pair slot_base + 2 rank, + 1; tombstones dropped); a.tiles_cell must be
// current; leaves bcount at zero and nslot = 2 ncell
void launch_cell_resort(const RebuildArgs &a, int grid_cells, cudaStream_t s);
void launch_force(const ForceArgs &a, int dim, int law, int prec, int grid, int block,
                  cudaStream_t s);
// skin mode: the cell kernel (one thread per slot pair); block = cells per block (128, 256, 512);
// a.tiles must be the pair tiles of that block size
void launch_force_list(const ForceArgs &a, int dim, int law, int grid, int variant, int block, cudaStream_t s);
void launch_skin_begin(const SkinArgs &a, cudaStream_t s);
void launch_skin_rebin(const SkinArgs &a, int dim, int grid, cudaStream_t s);
void launch_skin_lists(const SkinArgs &a, int dim, int law, int grid, cudaStream_t s);
void launch_list_flatten(const SkinArgs &a, int grid, cudaStream_t s);
void launch_fresh_pairs(const SkinArgs &a, int dim, int law, cudaStream_t s);
// the device step counter advance; with tiles_cell also the tile table over the cells of the
// step's events
void launch_advance_ts(int *ts_dev, int *any_rebuild, cudaStream_t s, const ColonyCounters *cnt = nullptr, int B = 0,
                       int *tiles_cell = nullptr);
int mlp_param_count();
void launch_events_fast(const EventArgs &a, int grid_cells, int dim, cudaStream_t s, bool cell_states);
void launch_events_due(const EventArgs &a, int dim, cudaStream_t s);
void launch_divisions_list(const EventArgs &a, int colony, int n0, int ndiv, const int *mothers,
                           const double *dirs, const int *spans, int dim, cudaStream_t s);
void launch_apo_ops_with_div(const EventArgs &a, int colony, int ndiv, int nops, const int *ops, int dim,
                             cudaStream_t s);
void launch_fill_int(int *dst, int n, int value, cudaStream_t s);
void launch_sm_flags(const EventArgs &a, int colony, int n, int dim, cudaStream_t s);
void launch_sm_swell(const EventArgs &a, int colony, int n, int ts, cudaStream_t s);
void launch_sm_philox(const EventArgs &a, int grid_cells, cudaStream_t s);
void launch_sm_swell_all(const EventArgs &a, int grid_cells, cudaStream_t s);
void launch_sm_ops(const EventArgs &a, int colony, int nops, const int *ops, const double *dirs, int dim,
                   cudaStream_t s);
void launch_upload(const ColonyConst *col, int colony, int ncells, int dim, size_t SS, const double *stage,
                   double *x, double *sig_c, int *t0, int *tsw, double *vel, int *eid, int *slot_of,
                   ColonyCounters *cnt, int *chk, cudaStream_t s);
void launch_gather_canonical(int ncells, int dim, size_t SS, int cell_base, const int *slot_of,
                             const double *src, int width, double *dst, cudaStream_t s);
void launch_observables(const EventArgs &a, int colony, int ncells, int dim, int reset,
                        double *partials, int nblocks, cudaStream_t s);

// ---------------------------------------------------------------- frame output
// The device state of one colony as the frame writer reads it: SoA FP64 positions and
// velocities by slot (x[d * SS + slot]), the canonical element -> slot map and the canonical
// diameters [cell][2]; valid on `stream` until the caller's next cil_step.
struct FrameSource {
  const double *x;
  const double *vel;
  const int *slot_of;
  const double *sigma_c;
  size_t SS;
  int cell_base;
  int ncells;
  int dim;
  int divide;
  int dying;
  double box[3];
  double sigma_max;
  int64_t ts;
  int device;
  int capacity;  // cells the colony can hold
  cudaStream_t stream;
};
// Waits for the handle's queued work and fills *out (cil_api.cu).
cil_status frame_source(cil_handle *h, int colony, FrameSource *out);
// The colony's static layout only (dim, box, flags, capacity, device), without waiting and
// before any upload; the device pointers, cell count, sigma_max and ts are left empty.
cil_status frame_layout(cil_handle *h, int colony, FrameSource *out);
// Packs a colony's elements in canonical order into FP32 frame arrays: position [E][3]
// (shifted by -half, 2D z from zj[j]), velocity [E][3], diameter [E] (cil_frame.cu).
void launch_frame_pack(const FrameSource &s, const double half[3], const float zj[2], float *out,
                       cudaStream_t st);

}  // namespace cil
