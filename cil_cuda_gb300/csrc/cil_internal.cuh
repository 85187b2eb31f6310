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

// error bits in ColonyCounters::err
constexpr int kErrNan = 1 << CIL_ERR_NAN;
constexpr int kErrBox = 1 << CIL_ERR_OUT_OF_BOX;
constexpr int kErrCap = 1 << CIL_ERR_CAPACITY;

// Philox purposes (third counter word)
constexpr uint32_t kRngNoise = 1, kRngDiv = 2, kRngDiv2 = 3, kRngApo = 4;

struct ColonyConst {
  double box[3];
  double ih[3];      // 1/L, as the reference binning formula uses (Utils.hpp:990)
  double bw[3];      // bin width L/Ns
  int ns[3];         // bins per axis (1 on unused axes)
  int periodic[3];
  int single_bin;    // grid collapsed to one bin (some Ns < 3, Utils.hpp:897-901)
  int bin_base;      // first global bin
  int nbins;         // real bins
  int nbins_pad;     // bins rounded up to kScanItems
  int scan_base;     // first scan block
  int slot_base, slot_cap;
  int cell_base, cell_cap;
  int ctile_base;    // first cell tile (static, from capacity)
  int ctile_cap;     // cell tiles reserved
  int force_law;
  int noise_per_cell;
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
  float bwf[3];      // bin widths in FP32 (mixed precision)
};

struct ColonyCounters {
  int ncell;          // live cells
  int nslot;          // used slots (live + tombstones + appended daughters)
  int nlive;          // elements sorted into bins by the last rebuild
  int err;            // error bits
  int ndiv_step;      // divisions this step
  int ndead;          // apoptoses recorded this step (list length, may exceed kDeadCap)
  int ndiv_allowed;   // divisions that fit the capacity this step
  int pad;
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

// [0, 1) with 53 random bits
__device__ __forceinline__ double uniform53(uint32_t a, uint32_t b) {
  const uint64_t m = (static_cast<uint64_t>(a) << 21) ^ (static_cast<uint64_t>(b) >> 11);
  return static_cast<double>(m & ((1ull << 53) - 1)) * 1.1102230246251565e-16;
}

// ---------------------------------------------------------------- pair force laws
// Force modulus f0 with F_i += f0 * (r_j - r_i); returns false outside the cutoff.
// LJ-WCA is the reference's LJParams::elemForce0 form (MD.cuh:50-56, 98-113).
template <int LAW, typename R>
__device__ __forceinline__ bool pair_force(R r2, R si, R sj, R eps, R rcs, R &f0) {
  const R sij = R(0.5) * (si + sj);
  if (LAW == CIL_FORCE_LJ_WCA) {
    const R sij2 = sij * sij;
    const R rc2 = sij2 * (rcs * rcs);
    if (r2 <= rc2) {
      const R ir2 = R(1) / r2;
      R sr2n = sij2 * ir2;
      const R srn = sr2n * sr2n * sr2n;
      sr2n = srn * srn;
      f0 = (srn - R(2) * sr2n) * ir2 * (R(24) * eps);
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

// ---------------------------------------------------------------- kernel argument packs

struct RebuildArgs {
  const ColonyConst *col;
  ColonyCounters *cnt;
  int B;
  size_t SS;               // slot stride of SoA arrays
  const int *tiles_used;   // [B+1] tiles over nslot (before the rebuild)
  const int *tiles_live;   // [B+1] tiles over nlive (after the scan)
  const int *scan_col;     // scan block -> colony
  int nscan;               // scan blocks
  const double *x_in;
  const double *sig_in;
  const int *eid_in;
  double *x_out;
  double *sig_out;
  int *eid_out;
  float *u_out;            // FP32 bin-local coordinates (mixed precision), may be null
  float *sigf_out;         // FP32 diameters (mixed precision), may be null
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
  const int *tiles_live;
  const double *x_in;      // sorted positions
  double *x_out;           // integrated positions (same slots)
  const double *sig;
  const int *eid;
  const float *u;          // mixed precision
  const float *sigf;
  const int2 *range;
  const int *slot_of;
  const int *t0;
  const int *tsw;
  const double *noise;     // oracle mode: uploaded normals (already scaled), canonical order
  double *vel;             // slot order, may be null
  double *frc;             // slot order, may be null
  int ts;
  uint32_t seed_lo, seed_hi;
  int noise_mode;          // 0 none, 1 philox, 2 uploaded
  int integrate;
};

struct EventArgs {
  const ColonyConst *col;
  ColonyCounters *cnt;
  int B;
  size_t SS;
  const int *tiles_cell;   // [B+1] tiles over ncell
  double *x;               // current positions
  double *sig;
  int *eid;
  double *vel;             // may be null
  int *slot_of;
  int *t0;
  int *tsw;
  int *tile_count;
  int *tile_off;
  int *dead;               // [B * kDeadCap]
  double *obs_com_prev;    // [D * CC] or null
  double *obs_disp;
  double *obs_vref;
  size_t CC;
  int ts;                  // step after the increment
  uint32_t seed_lo, seed_hi;
};

// ---------------------------------------------------------------- launchers (host side)
void launch_tiles(const ColonyConst *col, ColonyCounters *cnt, int B, int which, int *tiles,
                  cudaStream_t s);
void launch_rebuild(const RebuildArgs &a, int grid_slots, cudaStream_t s);
void launch_force(const ForceArgs &a, int dim, int law, int prec, int grid, int block,
                  cudaStream_t s);
void launch_events_fast(const EventArgs &a, int grid_cells, int dim, cudaStream_t s);
void launch_divisions_list(const EventArgs &a, int colony, int n0, int ndiv, const int *mothers,
                           const double *dirs, const int *spans, int dim, cudaStream_t s);
void launch_apo_ops_with_div(const EventArgs &a, int colony, int ndiv, int nops, const int *ops, int dim,
                             cudaStream_t s);
void launch_upload_scatter(const ColonyConst *col, int colony, int ncells, int dim, size_t SS,
                           const double *pos, const double *sigma, double *x, double *sig,
                           int *eid, int *slot_of, ColonyCounters *cnt, cudaStream_t s);
void launch_gather_canonical(int ncells, int dim, size_t SS, int cell_base, const int *slot_of,
                             const double *src, int width, double *dst, cudaStream_t s);
void launch_observables(const EventArgs &a, int colony, int ncells, int dim, int reset,
                        double *partials, int nblocks, cudaStream_t s);

}  // namespace cil
