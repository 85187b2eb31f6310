// The single-element cell-cycle model on the GPU (include/cil_cycle.h).
//
// Layout: structure of arrays in index order (cell i at i), FP64. Two complete state sets;
// a removal (apoptosis, drain) compacts the survivors stably into the other set and the host
// flips the set index. Positions are double-buffered within a step (the force pass reads one
// buffer and writes the other).
//
// A step (no host synchronisation; the cell count lives on the device):
//   bins       k_cy_keys / scan / k_cy_scatter / k_cy_sort: a counting sort of the cells into
//              bins (width set per call from the largest diameter), ascending cell index
//              inside a bin; the pair search walks +-k bins with k from the colony's largest
//              diameter of the previous step, so growing cells never outgrow the search; with
//              FP32 pair arithmetic (precision 1), k_cy_pack writes the FP32 records of the bin
//              order that the pair loops read instead of the FP64 positions;
//   forces     k_cy_force: motility along the velocity, passive noise, Hertz contacts with
//              adhesion and the pressure sum, then the position update with the pressure-
//              dependent friction, in one thread per cell;
//   cycle      k_cy_cycle (ODEs, division flag, per-block count) / k_cy_scan_blocks /
//              k_cy_divide (daughters appended in mother order);
//   apoptosis  k_cy_apo_mark / scan / k_cy_compact (only with apoptosis on).
// The DPD integrator: k_dpd_kick_drift (first half kick and the drift), the bins, k_cy_force in
// its forces-only mode (Fc and the pressure), k_dpd_pair (the pair dissipative and random
// forces and the second half kick, into the spare velocity buffer), k_dpd_dis (background and
// pair dissipation at the new velocities), then the same cycle and apoptosis kernels.
// The file is compiled without FMA contraction, so that the arithmetic is that of the host
// restatement the tests compare with.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cil_cycle.h"
#include "cil_internal.cuh"

// Axis loops: unrolled to three with a guard, so that per-axis arrays stay in registers (the
// dimension is a run-time value)
#define CY_AXES(d, D) _Pragma("unroll") for (int d = 0; d < 3; ++d) if (d < (D))

namespace {

using cil::kTile;
using cil::philox4x32_10;
using cil::u32x4;

constexpr double kPi = 3.14159265358979323846;
constexpr double kLn2 = 0.69314718055994530942;
constexpr int kScanTile = 1024;  // elements per block of the scans

// Philox purposes (third counter word)
constexpr uint32_t kCyNoise = 11, kCyDir = 12, kCyDiv = 13, kCyApo = 14, kCyInit = 15;
// DPD pair normals: counter (lower cell index, step, purpose, higher cell index)
constexpr uint32_t kCyDpd0 = 16, kCyDpd1 = 17;

struct CyConst {
  int D;
  int periodic[3];
  double box[3];
  double dt;
  int ns[3];
  double bw[3];       // bin width per axis
  float bwf[3], boxf[3], halff[3];  // FP32 copies for the packed pair arithmetic
  double half[3];     // box / 2
  double inv_bw[3];
  double sigma_core;
  double hz_c;        // (1 - nu^2) / E
  double adhesion;
  double motility, zeta, zeta_p, zeta_p_beta;
  double noise_amp;   // sqrt(2 D) / sqrt(dt)
  int divide;
  int apoptosis;
  double tau_div_mu, tau_div_sigma, tau_mig_mu, tau_mig_sigma;
  double v1, tau_r, tau_v, tau_p;   // tau_* in steps
  double v_s;
  double p0, beta_vs, rho_ratio, r_maxed_inv, p_shift, p_shift_tau_inv, osm;
  double apop_pressure, apop_duration, apop_rate_step, extr_gamma;
  double apop_steps;  // apop_duration / dt
  double extr_rate;
  // DPD
  int dpd;
  double kick_div;    // 2 (2 m): updateVel's divisor with the mass argument 2 m
  double sqrt_dt;
  double gamma_d, gamma_b, sigma_r;  // DISDIFCEL, DISBG, sqrt(2 DISDIFCEL kT)
  uint32_t seed_lo, seed_hi;
  int capacity;
};

struct CySet {
  double *x;      // [D][cap]
  double *v;      // [D][cap]
  double *sig, *sigt, *theta, *rho, *om, *p;
  int *tp, *t0, *tsw;
  double *fc, *fd, *fr;  // [D][cap], DPD only (conservative, dissipative, random forces)
};

// FP32 records of the cells in bin order, for the FP32 pair arithmetic (precision 1): the
// position relative to the origin of the cell's bin with the diameter, the velocity (DPD), and
// each cell's place in the bin order. Displacements are then formed in FP32 from bin offsets,
// with no FP64 operation per candidate.
struct CyPacked {
  float4 *pk;  // [q]: x - bin origin per axis (z 0 in 2D), diameter
  float4 *vk;  // [q]: velocity (DPD)
  int *qpos;   // [cell]: its place q
};

struct CyCounters {
  int n;
  int err;
  long long ndiv_total;
  long long napo_total;
  unsigned long long sigma_max_bits;  // largest diameter (non-negative doubles order like their bits)
  int ndiv_step;
  int nrem_step;
};

constexpr int kErrCapacity = 1;
constexpr int kErrNonFinite = 2;
constexpr int kErrOutOfBox = 4;
constexpr int kErrCrowded = 8;     // a bin holds more than kBinSortMax cells
constexpr int kBinSortMax = 256;   // cells a bin may hold (about 1 at the bin width used)

// ---------------------------------------------------------------- draws
__host__ __device__ inline double u53(uint32_t a, uint32_t b) {
  const uint64_t m = (static_cast<uint64_t>(a) << 21) ^ (static_cast<uint64_t>(b) >> 11);
  return static_cast<double>(m & ((1ull << 53) - 1)) * 1.1102230246251565e-16;
}

// Two standard normals (Box-Muller, FP64) from the four words of one Philox block.
__device__ inline void normal2(const u32x4 &r, double *n0, double *n1) {
  const double a = 1.0 - u53(r.v[0], r.v[1]);  // (0, 1]
  const double b = u53(r.v[2], r.v[3]);
  const double rad = sqrt(-2.0 * log(a));
  const double ang = 6.283185307179586 * b;
  *n0 = rad * cos(ang);
  *n1 = rad * sin(ang);
}

__device__ inline u32x4 draw(const CyConst &C, uint32_t cell, int ts, uint32_t purpose, uint32_t sub) {
  return philox4x32_10(cell, static_cast<uint32_t>(ts), purpose, sub, C.seed_lo, C.seed_hi);
}

__device__ inline int nint(double a) { return a >= 0.0 ? static_cast<int>(a + 0.5) : static_cast<int>(a - 0.5); }

// max(Nint(x / dt), 1) (randomTimeSpan, MD.cuh:434-436)
__device__ inline int span_steps(double x, double dt) {
  const int s = nint(x / dt);
  return s > 1 ? s : 1;
}

// exp(mu2 + s2 Z), mu2 = log(mu^2 / sqrt(mu^2 + s^2)), s2 = sqrt(log(1 + s^2/mu^2)) (Random.hpp:55-60)
__device__ inline double lognormal(double mu, double s, double z) {
  const double mu2 = log((mu * mu) / (sqrt(mu * mu + s * s)));
  const double s2 = sqrt(log(1 + (s * s) / (mu * mu)));
  return exp(mu2 + s2 * z);
}

// ---------------------------------------------------------------- geometry (Utils.hpp:223-256)
__device__ inline double area_of(double s) { return kPi * ((s / 2) * (s / 2)); }
__device__ inline double volume_of(double s) { return 4 * kPi * ((s / 2) * (s / 2) * (s / 2)) / 3; }
__device__ inline double sigma_of_area(double a) { return 2 * sqrt(a / kPi); }
__device__ inline double sigma_of_volume(double v) { return 2 * cbrt(3 * v / (4 * kPi)); }

__device__ inline double contact_length(double a, double b, double h) {
  const double ra = a / 2, rb = b / 2;
  const double q = ra - (2 * rb * h - h * h) / (2 * (ra + rb - h));
  double t = 2 * sqrt(ra * ra - q * q);
  const double small_r = (a <= b) ? a : b;
  return isnan(t) ? small_r : t;
}

__device__ inline double contact_area(double r, double a, double b) {
  const double ra = a / 2, rb = b / 2;
  const double u = r * r - rb * rb + ra * ra;
  const double t = sqrt(4 * (r * r) * (ra * ra) - u * u) / (2 * r);
  return t > 0 ? kPi * (t * t) : 0.0;
}

__device__ inline double wrap(double t, double L) {  // fmod(t + L, L)
  return fmod(t + L, L);
}

__device__ inline int bin_of(const CyConst &C, const double *xd) {
  int b = 0;
  CY_AXES(d, C.D) {
    int v = static_cast<int>(xd[d] * C.inv_bw[d]);
    v = v < 0 ? 0 : (v >= C.ns[d] ? C.ns[d] - 1 : v);
    b = b * C.ns[d] + v;
  }
  return b;
}

// The bins around a cell that hold every cell within `radius` of it: k = ceil(radius / bin
// width) bins on each side, the whole axis (each bin once) when 2k + 1 covers it, clipped at
// non-periodic walls.
struct Stencil {
  int bi[3], lo[3], hi[3];
};

__device__ inline void stencil_of(const CyConst &C, const double *xi, double radius, Stencil &s) {
  for (int d = 0; d < 3; ++d) s.bi[d] = s.lo[d] = s.hi[d] = 0;
  CY_AXES(d, C.D) {
    int v = static_cast<int>(xi[d] * C.inv_bw[d]);
    v = v < 0 ? 0 : (v >= C.ns[d] ? C.ns[d] - 1 : v);
    s.bi[d] = v;
    const double kk = ceil(radius * C.inv_bw[d]);
    const int k = (kk >= 0.0 && kk < C.ns[d]) ? static_cast<int>(kk) : C.ns[d];
    if (2 * k + 1 >= C.ns[d]) {
      s.lo[d] = -s.bi[d];
      s.hi[d] = C.ns[d] - 1 - s.bi[d];
    } else if (C.periodic[d]) {
      s.lo[d] = -k;
      s.hi[d] = k;
    } else {
      s.lo[d] = s.bi[d] - k < 0 ? -s.bi[d] : -k;
      s.hi[d] = s.bi[d] + k >= C.ns[d] ? C.ns[d] - 1 - s.bi[d] : k;
    }
  }
}

__device__ inline int stencil_bin(const CyConst &C, const Stencil &s, int o0, int o1, int o2) {
  const int oo[3] = {o0, o1, o2};
  int b = 0;
  CY_AXES(d, C.D) {
    int v = s.bi[d] + oo[d];
    if (v < 0) v += C.ns[d];
    if (v >= C.ns[d]) v -= C.ns[d];
    b = b * C.ns[d] + v;
  }
  return b;
}

// r_j - r_i at the nearest image (|dd| < L, so Nint(dd / L) is -1, 0 or 1; the two forms differ
// only at |dd| = L/2, far beyond any contact); returns |r_j - r_i|^2
__device__ inline double separation(const CyConst &C, const CySet &S, const double *xi, int j, double *rij) {
  const size_t cap = C.capacity;
  double r2 = 0.0;
  CY_AXES(d, C.D) {
    double dd = S.x[d * cap + j] - xi[d];
    if (C.periodic[d]) {
      if (dd > C.half[d])
        dd -= C.box[d];
      else if (dd < -C.half[d])
        dd += C.box[d];
    }
    rij[d] = dd;
    r2 += dd * dd;
  }
  return r2;
}

__device__ inline float f4c(const float4 &v, int d) { return d == 0 ? v.x : (d == 1 ? v.y : v.z); }

// FP32 displacement from the packed record pi to pj, whose bin lies at offset o from pi's, at
// the nearest image on periodic axes; returns its square length
__device__ inline float packed_sep(const CyConst &C, const float4 &pi, const float4 &pj, int o0, int o1, int o2,
                                   float *df) {
  const int o[3] = {o0, o1, o2};
  float r2 = 0.0f;
  CY_AXES(d, C.D) {
    float v = f4c(pj, d) + static_cast<float>(o[d]) * C.bwf[d] - f4c(pi, d);
    if (C.periodic[d]) {
      if (v > C.halff[d])
        v -= C.boxf[d];
      else if (v < -C.halff[d])
        v += C.boxf[d];
    }
    df[d] = v;
    r2 += v * v;
  }
  return r2;
}

// The squared minimum-image separation in FP32 from the FP64 difference, for the walks' range
// tests: within a relative 1e-6 of separation()'s (a pair near half a box may wrap the other
// way, and is out of range either way), so bounds widened by 1e-5 let every pair in range pass
// to the exact FP64 test.
__device__ inline float separation_f(const CyConst &C, const CySet &S, const double *xi, int j) {
  const size_t cap = C.capacity;
  float r2 = 0.0f;
  CY_AXES(d, C.D) {
    float v = static_cast<float>(S.x[d * cap + j] - xi[d]);
    if (C.periodic[d]) {
      if (v > C.halff[d])
        v -= C.boxf[d];
      else if (v < -C.halff[d])
        v += C.boxf[d];
    }
    r2 += v * v;
  }
  return r2;
}

// ---------------------------------------------------------------- block scan
// Exclusive scan over the block (any multiple of 32 threads up to kTile)
__device__ inline int block_excl_scan(int v, int *total) {
  __shared__ int ws[kTile / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < nw) ws[lane] = w;
  }
  __syncthreads();
  const int base = wid > 0 ? ws[wid - 1] : 0;
  *total = ws[nw - 1];
  __syncthreads();
  return base + inc - v;
}

// Exclusive scan of `count[0..m)` in place by one block; count[m] receives the total.
__global__ void k_cy_scan_small(int *count, int m) {
  int carry = 0;
  for (int base = 0; base < m; base += kTile) {
    const int i = base + threadIdx.x;
    const int v = i < m ? count[i] : 0;
    int tot;
    const int ex = block_excl_scan(v, &tot);
    if (i < m) count[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) count[m] = carry;
}

// Block sums of kScanTile-sized chunks (4 per thread)
__global__ void k_cy_chunk_sums(const int *count, int m, int *part) {
  const int b0 = blockIdx.x * kScanTile + threadIdx.x * 4;
  int s = 0;
  for (int q = 0; q < 4; ++q) s += (b0 + q < m) ? count[b0 + q] : 0;
  int tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Exclusive scan of count[0..m) using the scanned chunk sums, into start[0..m] (start[m] =
// total; the chunks cover index m, count[m] reads as 0)
__global__ void k_cy_chunk_apply(const int *count, int m, const int *part, int *start) {
  const int b0 = blockIdx.x * kScanTile + threadIdx.x * 4;
  int c[4], s = 0;
  for (int q = 0; q < 4; ++q) {
    c[q] = (b0 + q < m) ? count[b0 + q] : 0;
    s += c[q];
  }
  int tot;
  int e = part[blockIdx.x] + block_excl_scan(s, &tot);
  for (int q = 0; q < 4; ++q) {
    if (b0 + q <= m) start[b0 + q] = e;
    e += c[q];
  }
}

// ---------------------------------------------------------------- bins
__global__ void k_cy_clear(int *a, int m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) a[i] = 0;
}

// the bin of every cell, and 1 / (sigma / 2) for the contact pass (the same value it would
// compute per contact)
__global__ void k_cy_keys(CyConst C, CySet S, const CyCounters *cnt, int *key, int *count, double *inv_r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt->n) return;
  inv_r[i] = 1.0 / (S.sig[i] / 2);
  double xd[3];
  CY_AXES(d, C.D) xd[d] = S.x[static_cast<size_t>(d) * C.capacity + i];
  const int b = bin_of(C, xd);
  key[i] = b;
  atomicAdd(count + b, 1);
}

__global__ void k_cy_scatter(const CyCounters *cnt, const int *key, const int *start, int *cursor, int *list) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt->n) return;
  const int b = key[i];
  const int pos = start[b] + atomicAdd(cursor + b, 1);
  list[pos] = i;
}

// ascending cell index inside every bin (insertion sort: bins hold a few cells; a bin with
// more than kBinSortMax cells means overlapping cells and is reported instead of sorted)
__global__ void k_cy_sort(const int *start, int nbins, int *list, CyCounters *cnt) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const int lo = start[b], hi = start[b + 1];
  if (hi - lo > kBinSortMax) {
    atomicOr(&cnt->err, kErrCrowded);
    return;
  }
  for (int i = lo + 1; i < hi; ++i) {
    const int v = list[i];
    int j = i - 1;
    while (j >= lo && list[j] > v) {
      list[j + 1] = list[j];
      --j;
    }
    list[j + 1] = v;
  }
}

// The packed records of the bin order (CyPacked); vk only when velocities are wanted
__global__ void k_cy_pack(CyConst C, CySet S, const CyCounters *cnt, const int *list, CyPacked P, int with_vel) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= cnt->n) return;
  const int i = list[q];
  const size_t cap = C.capacity;
  float rel[3] = {0.0f, 0.0f, 0.0f}, vf[3] = {0.0f, 0.0f, 0.0f};
  CY_AXES(d, C.D) {
    const double x = S.x[d * cap + i];
    int v = static_cast<int>(x * C.inv_bw[d]);
    v = v < 0 ? 0 : (v >= C.ns[d] ? C.ns[d] - 1 : v);
    rel[d] = static_cast<float>(x - v * C.bw[d]);
    if (with_vel) vf[d] = static_cast<float>(S.v[d * cap + i]);
  }
  P.pk[q] = make_float4(rel[0], rel[1], rel[2], static_cast<float>(S.sig[i]));
  if (with_vel) P.vk[q] = make_float4(vf[0], vf[1], vf[2], 0.0f);
  P.qpos[i] = q;
}

__global__ void k_cy_pack_vel(CyConst C, CySet S, const CyCounters *cnt, const int *list, CyPacked P) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= cnt->n) return;
  const int i = list[q];
  const size_t cap = C.capacity;
  float vf[3] = {0.0f, 0.0f, 0.0f};
  CY_AXES(d, C.D) vf[d] = static_cast<float>(S.v[d * cap + i]);
  P.vk[q] = make_float4(vf[0], vf[1], vf[2], 0.0f);
}

// ---------------------------------------------------------------- forces + update
// MIXED: the candidate test and the contact arithmetic in FP32 on the FP64 separation (GB300
// runs FP64 at a small fraction of its FP32 rate); the forces and the pressure are summed in
// FP32 over the contacts and added to the FP64 motility and noise; the position update and
// the cell state stay FP64.
// mode 0 (Euler): the position update with the pressure-dependent friction follows, into x_out,
// and the velocity; mode 1 (DPD): the force goes to frc and nothing moves. Draws are keyed by
// the device step counter + key_off.
template <bool MIXED>
// lane_bits: 2^lane_bits threads share a cell (small colonies): lane l takes the l-th of every
// 2^lane_bits candidates of the flattened bin walk, and the lanes' contact sums are combined by
// a fixed xor tree (the restatement combines them the same way); lane 0 writes.
__global__ void __launch_bounds__(kTile) k_cy_force(CyConst C, CySet S, double *x_out, double *frc,
                                                    CyCounters *cnt, const int *start, const int *list,
                                                    const int *ts_dev, int mode, int key_off, CyPacked P,
                                                    int lane_bits, const double *inv_r) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = 1 << lane_bits;
  const int i = t >> lane_bits, lane = t & (L - 1);
  const int n = cnt->n;
  if (i >= n) return;  // a cell's lanes leave together (they share a warp)
  const int ts = *ts_dev + key_off;
  const size_t cap = C.capacity;
  const int D = C.D;
  double xi[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, F[3] = {0, 0, 0};
  CY_AXES(d, D) {
    xi[d] = S.x[d * cap + i];
    vi[d] = S.v[d * cap + i];
  }
  const double si = S.sig[i];
  // ---- motility along the velocity (singleCellForce, MD.cu:600-646)
  {
    double v2 = 0.0;
    CY_AXES(d, D) v2 += vi[d] * vi[d];
    double vl = sqrt(v2);
    if (vl == 0.0) {  // a direction at random, length 1e-11 (BIG_TOL_MP)
      const u32x4 r = draw(C, i, ts, kCyDir, 0);
      if (D == 2) {
        const double ang = 6.283185307179586 * u53(r.v[0], r.v[1]);
        vi[0] = 1e-11 * cos(ang);
        vi[1] = 1e-11 * sin(ang);
      } else {
        const double z = 2.0 * u53(r.v[0], r.v[1]) - 1.0;
        const double ang = 6.283185307179586 * u53(r.v[2], r.v[3]);
        const double s = sqrt(1.0 - z * z);
        vi[0] = 1e-11 * (s * cos(ang));
        vi[1] = 1e-11 * (s * sin(ang));
        vi[2] = 1e-11 * z;
      }
      v2 = 0.0;
      CY_AXES(d, D) v2 += vi[d] * vi[d];
      vl = sqrt(v2);
    }
    CY_AXES(d, D) F[d] = C.motility * (vi[d] / vl);
  }
  // ---- passive noise (CIL.cu:84-97)
  if (C.noise_amp > 0.0) {
    double nz[4];
    normal2(draw(C, i, ts, kCyNoise, 0), &nz[0], &nz[1]);
    if (D == 3) normal2(draw(C, i, ts, kCyNoise, 1), &nz[2], &nz[3]);
    CY_AXES(d, D) F[d] += C.zeta * (C.noise_amp * nz[d]);
  }
  // ---- Hertz contacts with adhesion and the pressure (device draft, MD.cu:302-366)
  double pres = 0.0;
  double Fc[3] = {0.0, 0.0, 0.0};  // the contacts' share of the force
  {
    // bins to search on each side: the largest diameter of the colony over the bin width
    Stencil st;
    stencil_of(C, xi, __longlong_as_double(static_cast<long long>(cnt->sigma_max_bits)), st);
    int kflat = 0;  // candidates of the bins walked so far
    const double c2 = C.hz_c + C.hz_c;
    const double inv_hz = 1.0 / (0.75 * c2);
    const double inv_ri = 1.0 / (si / 2);
    const float sif = static_cast<float>(si), c2f = static_cast<float>(c2), adhf = static_cast<float>(C.adhesion);
    const float inv_rif = 2.0f / sif;
    float Ff[3] = {0.0f, 0.0f, 0.0f}, presf = 0.0f;
    const int qi = MIXED ? P.qpos[i] : 0;
    const float4 pi4 = MIXED ? P.pk[qi] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    // FP64: the candidates that pass the cheap distance test, in walk order (kNear at a time)
    constexpr int kNear = 16;
    int near[kNear];
    int nnear = 0;
    auto contacts = [&]() {
      for (int k = 0; k < nnear; ++k) {
        const int j = near[k];
        double rij[3] = {0, 0, 0};
        const double r2 = separation(C, S, xi, j, rij);
        const double sj = S.sig[j];
        const double cut = (si + sj) / 2;
        const double r = sqrt(r2);
        if (!(r <= cut) || r == 0.0) continue;
        // the pair's first cell is the one of lower index (the contact length is not
        // symmetric in the two diameters)
        const double sa = i < j ? si : sj, sb = i < j ? sj : si;
        const double h = fmax((si + sj) / 2 - r, 0.0);
        const double Sr = inv_ri + inv_r[j];
        // h^1.5 / (0.75 c2 sqrt(S)) as h sqrt(h / S) / (0.75 c2): one square root fewer
        double fel, f0;
        if (D == 3) {
          fel = h * sqrt(h / Sr) * inv_hz;
          const double A = contact_area(r, sa, sb);
          const double vol = (A == 0 ? 0 : (4 * kPi * ((sa / 2) * (sa / 2)) / 3));
          f0 = -fel + C.adhesion * A;
          if (vol != 0.0) pres -= f0 / vol;
        } else {
          const double A = contact_length(sa, sb, h);  // also the contact's volume in 2D
          if (A != 0.0) {
            // one reciprocal u = 1 / (S A) gives both h / S = h A u and f0 / A = f0 S u
            const double u = 1.0 / (Sr * A);
            fel = h * sqrt(h * (A * u)) * inv_hz;
            f0 = -fel + C.adhesion * A;
            pres -= f0 * (Sr * u);
          } else {
            fel = h * sqrt(h / Sr) * inv_hz;
            f0 = -fel;
          }
        }
        CY_AXES(d, D) Fc[d] += f0 * rij[d];
      }
      nnear = 0;
    };
    for (int o0 = st.lo[0]; o0 <= st.hi[0]; ++o0)
      for (int o1 = (D > 1 ? st.lo[1] : 0); o1 <= (D > 1 ? st.hi[1] : 0); ++o1)
        for (int o2 = (D > 2 ? st.lo[2] : 0); o2 <= (D > 2 ? st.hi[2] : 0); ++o2) {
          const int b = stencil_bin(C, st, o0, o1, o2);
          const int e0 = start[b], e1 = start[b + 1];
          const int first = e0 + ((lane - kflat) & (L - 1));
          kflat += e1 - e0;
          for (int q = first; q < e1; q += L) {
            if (MIXED) {
              if (q == qi) continue;
              const float4 pj = P.pk[q];
              float df[3] = {0.0f, 0.0f, 0.0f};
              const float r2f = packed_sep(C, pi4, pj, o0, o1, o2, df);
              const float sjf = pj.w;
              const float cut = 0.5f * (sif + sjf);
              if (!(r2f <= cut * cut) || r2f == 0.0f) continue;
              const int j = list[q];
              const float r = sqrtf(r2f);
              const float sa = i < j ? sif : sjf, sb = i < j ? sjf : sif;
              const float h = fmaxf(cut - r, 0.0f);
              const float fel = (h * sqrtf(h)) / (0.75f * c2f * sqrtf(inv_rif + 2.0f / sjf));
              float A, vol;
              if (D == 3) {
                const float ra = 0.5f * sa, rb = 0.5f * sb;
                const float u = r2f - rb * rb + ra * ra;
                const float t = sqrtf(4.0f * r2f * (ra * ra) - u * u) / (2.0f * r);
                A = t > 0.0f ? static_cast<float>(kPi) * (t * t) : 0.0f;
                vol = A == 0.0f ? 0.0f : (4.0f * static_cast<float>(kPi) * (ra * ra) / 3.0f);
              } else {
                const float ra = 0.5f * sa, rb = 0.5f * sb;
                const float qq = ra - (2.0f * rb * h - h * h) / (2.0f * (ra + rb - h));
                const float t = 2.0f * sqrtf(ra * ra - qq * qq);
                A = isnan(t) ? fminf(sa, sb) : t;
                vol = A;
              }
              const float f0 = -fel + adhf * A;
              if (vol != 0.0f) presf -= f0 / vol;
              CY_AXES(d, D) Ff[d] += f0 * df[d];
              continue;
            }
            const int j = list[q];
            if (j == i) continue;
            const float cutf = 0.5f * (sif + static_cast<float>(S.sig[j]));
            if (separation_f(C, S, xi, j) > 1.00001f * (cutf * cutf)) continue;  // out of contact (exact test in contacts())
            // near candidates are evaluated together after the walk (contacts), so the warp runs
            // the FP64 contact arithmetic with its lanes converged instead of once per candidate
            near[nnear++] = j;
            if (nnear == kNear) contacts();
          }
        }
    if (!MIXED) contacts();
    if (L > 1) {  // lanes l and l ^ 2^k combine, k from the highest: a fixed tree
      const unsigned gm = (L == 32 ? 0xffffffffu : ((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
      for (int off = L >> 1; off > 0; off >>= 1) {
        if (MIXED) {
          presf += __shfl_xor_sync(gm, presf, off, L);
          CY_AXES(d, D) Ff[d] += __shfl_xor_sync(gm, Ff[d], off, L);
        } else {
          pres += __shfl_xor_sync(gm, pres, off, L);
          CY_AXES(d, D) Fc[d] += __shfl_xor_sync(gm, Fc[d], off, L);
        }
      }
    }
    CY_AXES(d, D) F[d] += Fc[d];
    if (MIXED) {
      pres += static_cast<double>(presf);
      CY_AXES(d, D) F[d] += static_cast<double>(Ff[d]);
    }
  }
  if (lane != 0) return;
  bool finite = true;
  CY_AXES(d, D) finite = finite && isfinite(F[d]);
  S.p[i] = pres;
  if (!finite) atomicOr(&cnt->err, kErrNonFinite);
  if (mode == 1) {
    CY_AXES(d, D) frc[d * cap + i] = F[d];
    return;
  }
  // ---- position update with the pressure-dependent friction (CIL.cu:902-939)
  const double pnd = pres / C.p0;
  // pow(x, 0) is 1 for every x
  const double pw = C.zeta_p_beta == 0.0 ? 1.0 : pow(pnd, C.zeta_p_beta);
  const double temp = C.dt * 1 / ((C.zeta + C.zeta_p * pw) * area_of(si));
  CY_AXES(d, D) {
    const double t = xi[d] + temp * F[d];
    x_out[d * cap + i] = C.periodic[d] ? wrap(t, C.box[d]) : t;
    S.v[d * cap + i] = F[d] * (temp / C.dt);
    if (frc) frc[d * cap + i] = F[d];
  }
}

// ---------------------------------------------------------------- DPD
__device__ inline double kick(const CyConst &C, double v, double fc, double fd, double fr) {
  return v + (fc * C.dt + fd * C.dt + fr * C.sqrt_dt) / C.kick_div;  // updateVel (Utils.hpp:568-571)
}

// updateVelocities then updatePositions (CIL.cu:871-897, 849-866; DPD step, CIL.cu:1055-1056)
__global__ void __launch_bounds__(kTile) k_dpd_kick_drift(CyConst C, CySet S, const CyCounters *cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt->n) return;
  const size_t cap = C.capacity;
  CY_AXES(d, C.D) {
    const size_t k = d * cap + i;
    const double v = kick(C, S.v[k], S.fc[k], S.fd[k], S.fr[k]);
    S.v[k] = v;
    const double x = S.x[k];
    S.x[k] = C.periodic[d] ? wrap(x + C.dt * v, C.box[d]) : x + v * C.dt;  // BoundingBox::updatePos
  }
}

// Two standard normals in FP32 (Box-Muller on 24-bit uniforms) from the four words of one
// Philox block, the FP32 counterpart of normal2: its uniforms are normal2's rounded to 24 bits
// (1 - u from the first word, u from the third), so the two agree to FP32 rounding.
__device__ inline void normal2f(const u32x4 &r, float *n0, float *n1) {
  const float u1 = static_cast<float>((1u << 24) - (r.v[0] >> 8)) * 5.9604644775390625e-08f;  // (0, 1]
  const float u2 = static_cast<float>(r.v[2] >> 8) * 5.9604644775390625e-08f;
  const float rad = sqrtf(-2.0f * __logf(u1));
  float sn, cs;
  __sincosf(6.2831853071795865f * u2, &sn, &cs);
  *n0 = rad * cs;
  *n1 = rad * sn;
}

// Pair dissipative and random forces (cellCellDisRanForce, MD.cu:861-905) over the pairs closer
// than the lower-index cell's diameter; then, with `kick`, the second half kick into v_out.
// MIXED: the pair terms in FP32 on the FP64 separation and velocity difference, FP32 normals,
// summed in FP32 per cell; the kick stays FP64.
template <bool MIXED>
__global__ void __launch_bounds__(kTile) k_dpd_pair(CyConst C, CySet S, double *v_out, CyCounters *cnt,
                                                    const int *start, const int *list, const int *ts_dev,
                                                    int key_off, int kick_on, CyPacked P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = cnt->n;
  if (i >= n) return;
  const uint32_t ts = static_cast<uint32_t>(*ts_dev + key_off);
  const size_t cap = C.capacity;
  const int D = C.D;
  double xi[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, Fd[3] = {0, 0, 0}, Fr[3] = {0, 0, 0};
  CY_AXES(d, D) {
    xi[d] = S.x[d * cap + i];
    vi[d] = S.v[d * cap + i];
  }
  const double si = S.sig[i];
  const float gdf = static_cast<float>(C.gamma_d), srf = static_cast<float>(C.sigma_r);
  float Fdf[3] = {0.0f, 0.0f, 0.0f}, Frf[3] = {0.0f, 0.0f, 0.0f};
  const int qi = MIXED ? P.qpos[i] : 0;
  const float4 pi4 = MIXED ? P.pk[qi] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float4 vi4 = MIXED ? P.vk[qi] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  // FP64: the candidates in range, in walk order, evaluated kNear at a time after the cheap
  // distance test, so the warp runs the pair terms (draws, normals, square roots) converged
  constexpr int kNear = 16;
  int near[kNear];
  int nnear = 0;
  auto pairs = [&]() {
    for (int k = 0; k < nnear; ++k) {
      const int j = near[k];
      double rij[3] = {0, 0, 0};
      const double r = sqrt(separation(C, S, xi, j, rij));
      const double rc = i < j ? si : S.sig[j];
      if (!(r < rc) || r == 0.0) continue;
      const double ir = 1.0 / r;  // one division for the weight and the unit vector
      const double w = 1 - r / rc;
      const uint32_t a = static_cast<uint32_t>(i < j ? i : j), z = static_cast<uint32_t>(i < j ? j : i);
      double xi_n[4];
      normal2(philox4x32_10(a, ts, kCyDpd0, z, C.seed_lo, C.seed_hi), &xi_n[0], &xi_n[1]);
      if (D == 3) normal2(philox4x32_10(a, ts, kCyDpd1, z, C.seed_lo, C.seed_hi), &xi_n[2], &xi_n[3]);
      const double sw = sqrt(w);
      CY_AXES(d, D) {
        const double nd = rij[d] * ir;
        const double vj = S.v[d * cap + j];
        Fd[d] -= C.gamma_d * w * ((vi[d] - vj) * nd) * nd;
        Fr[d] += C.sigma_r * sw * nd * xi_n[d];
      }
    }
    nnear = 0;
  };
  Stencil st;
  stencil_of(C, xi, __longlong_as_double(static_cast<long long>(cnt->sigma_max_bits)), st);
  for (int o0 = st.lo[0]; o0 <= st.hi[0]; ++o0)
    for (int o1 = (D > 1 ? st.lo[1] : 0); o1 <= (D > 1 ? st.hi[1] : 0); ++o1)
      for (int o2 = (D > 2 ? st.lo[2] : 0); o2 <= (D > 2 ? st.hi[2] : 0); ++o2) {
        const int b = stencil_bin(C, st, o0, o1, o2);
        for (int q = start[b]; q < start[b + 1]; ++q) {
          const int j = list[q];
          if (j == i) continue;
          if (MIXED) {
            const float4 pj = P.pk[q];
            float df[3] = {0.0f, 0.0f, 0.0f};
            const float r2 = packed_sep(C, pi4, pj, o0, o1, o2, df);
            const float rc = i < j ? pi4.w : pj.w;
            if (!(r2 < rc * rc) || r2 == 0.0f) continue;
            const float4 vj4 = P.vk[q];
            const float rinv = rsqrtf(r2);
            const float w = 1.0f - r2 * rinv / rc;
            const uint32_t a = static_cast<uint32_t>(i < j ? i : j), z = static_cast<uint32_t>(i < j ? j : i);
            float xf[4];
            normal2f(philox4x32_10(a, ts, kCyDpd0, z, C.seed_lo, C.seed_hi), &xf[0], &xf[1]);
            if (D == 3) normal2f(philox4x32_10(a, ts, kCyDpd1, z, C.seed_lo, C.seed_hi), &xf[2], &xf[3]);
            const float sw = sqrtf(w);
            CY_AXES(d, D) {
              const float nd = df[d] * rinv;
              const float dv = f4c(vi4, d) - f4c(vj4, d);
              Fdf[d] -= gdf * w * (dv * nd) * nd;
              Frf[d] += srf * sw * nd * xf[d];
            }
            continue;
          }
          const float rcf = static_cast<float>(i < j ? si : S.sig[j]);
          if (separation_f(C, S, xi, j) > 1.00001f * (rcf * rcf)) continue;  // out of range (exact test in pairs())
          near[nnear++] = j;
          if (nnear == kNear) pairs();
        }
      }
  if (!MIXED) pairs();
  if (MIXED)
    CY_AXES(d, D) {
      Fd[d] = static_cast<double>(Fdf[d]);
      Fr[d] = static_cast<double>(Frf[d]);
    }
  bool finite = true;
  CY_AXES(d, D) {
    const size_t k = d * cap + i;
    S.fd[k] = Fd[d];
    S.fr[k] = Fr[d];
    if (kick_on) {
      const double v = kick(C, vi[d], S.fc[k], Fd[d], Fr[d]);
      v_out[k] = v;
      finite = finite && isfinite(v);
    }
  }
  if (!finite) atomicOr(&cnt->err, kErrNonFinite);
}

// Background and pair dissipation at the new velocities (calculDisForces, CIL.cu:294-364:
// sameCellDisForce zeroes a single-element cell's Fd, cellBackDisForce subtracts gamma_bg v,
// cellCellDisForce, MD.cu:951-985, with w = 1 - r^2 / sigma_core for r < sigma_core)
template <bool MIXED>
__global__ void __launch_bounds__(kTile) k_dpd_dis(CyConst C, CySet S, const CyCounters *cnt, const int *start,
                                                   const int *list, CyPacked P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = cnt->n;
  if (i >= n) return;
  const size_t cap = C.capacity;
  const int D = C.D;
  double xi[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, Fd[3] = {0, 0, 0};
  CY_AXES(d, D) {
    xi[d] = S.x[d * cap + i];
    vi[d] = S.v[d * cap + i];
    Fd[d] = 0;
    Fd[d] -= C.gamma_b * vi[d];
  }
  const double rc = C.sigma_core;
  const float rcf = static_cast<float>(rc), gdf = static_cast<float>(C.gamma_d);
  float Fdf[3] = {0.0f, 0.0f, 0.0f};
  const int qi = MIXED ? P.qpos[i] : 0;
  const float4 pi4 = MIXED ? P.pk[qi] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float4 vi4 = MIXED ? P.vk[qi] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const double smax = __longlong_as_double(static_cast<long long>(cnt->sigma_max_bits));
  // FP64: the candidates in range, in walk order, evaluated kNear at a time after the walk with
  // the warp's lanes converged (same terms in the same order)
  constexpr int kNear = 16;
  int near[kNear];
  int nnear = 0;
  auto pairs = [&]() {
    for (int k = 0; k < nnear; ++k) {
      const int j = near[k];
      double rij[3] = {0, 0, 0};
      const double r = sqrt(separation(C, S, xi, j, rij));
      if (!(r < rc) || r == 0.0) continue;
      const double w = 1 - ((r * r) / rc);
      CY_AXES(d, D) {
        const double nd = -rij[d] / r;
        Fd[d] -= C.gamma_d * w * ((vi[d] - S.v[d * cap + j]) * nd) * nd;
      }
    }
    nnear = 0;
  };
  Stencil st;
  stencil_of(C, xi, smax > rc ? smax : rc, st);
  for (int o0 = st.lo[0]; o0 <= st.hi[0]; ++o0)
    for (int o1 = (D > 1 ? st.lo[1] : 0); o1 <= (D > 1 ? st.hi[1] : 0); ++o1)
      for (int o2 = (D > 2 ? st.lo[2] : 0); o2 <= (D > 2 ? st.hi[2] : 0); ++o2) {
        const int b = stencil_bin(C, st, o0, o1, o2);
        for (int q = start[b]; q < start[b + 1]; ++q) {
          if (MIXED) {
            if (q == qi) continue;
            const float4 pj = P.pk[q];
            float df[3] = {0.0f, 0.0f, 0.0f};
            const float r2 = packed_sep(C, pi4, pj, o0, o1, o2, df);
            if (!(r2 < rcf * rcf) || r2 == 0.0f) continue;
            const float4 vj4 = P.vk[q];
            const float rinv = rsqrtf(r2);
            const float w = 1.0f - r2 / rcf;
            CY_AXES(d, D) {
              const float nd = -df[d] * rinv;
              const float dv = f4c(vi4, d) - f4c(vj4, d);
              Fdf[d] -= gdf * w * (dv * nd) * nd;
            }
            continue;
          }
          const int j = list[q];
          if (j == i) continue;
          if (separation_f(C, S, xi, j) > 1.00001f * (rcf * rcf)) continue;  // out of range (exact test in pairs())
          near[nnear++] = j;
          if (nnear == kNear) pairs();
        }
      }
  if (!MIXED) pairs();
  CY_AXES(d, D) S.fd[d * cap + i] = MIXED ? Fd[d] + static_cast<double>(Fdf[d]) : Fd[d];
}

// ---------------------------------------------------------------- cell cycle and divisions
__global__ void __launch_bounds__(kTile) k_cy_cycle(CyConst C, CySet S, CyCounters *cnt, const int *ts_dev,
                                                    int *flag, int *block_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = cnt->n;
  const int ts = *ts_dev;
  int div = 0;
  if (i < n) {
    // cellTPressure (CIL.cu:493-494): every cell is in the dividing state when the species divides
    if (!C.divide || S.p[i] < C.apop_pressure)
      S.tp[i] = 0;
    else
      S.tp[i] += 1;
    if (C.divide) {
      const double shift = C.p_shift != 0.0 ? C.p_shift * exp(-ts * C.p_shift_tau_inv) : 0.0;
      const double pnd = fmax(0., S.p[i] + shift) / C.p0;
      const double om = S.om[i];
      double rho = S.rho[i];
      S.theta[i] += om * fmin(C.r_maxed_inv * rho, 1.0);
      const bool d3 = C.D == 3;
      double vt = d3 ? volume_of(S.sigt[i]) : area_of(S.sigt[i]);
      double v = d3 ? volume_of(S.sig[i]) : area_of(S.sig[i]);
      const double c0 = om * kLn2 + (C.v1 - 1) / C.tau_v;
      const double vt_prime = c0 * rho - (((vt - C.v_s) / C.v_s) / C.tau_v);
      vt += vt_prime * vt;
      const double v_prime = -(v - (vt / (1 + C.beta_vs * (C.osm + pnd)))) / C.tau_p;
      v += v_prime;
      v = C.tau_p == 0 ? vt : v;
      S.sigt[i] = d3 ? sigma_of_volume(vt) : sigma_of_area(vt);
      S.sig[i] = d3 ? sigma_of_volume(v) : sigma_of_area(v);
      const double r_np = (1 - rho - pnd);
      const double tau_r_pre = r_np > 0 ? 1 : C.rho_ratio;
      const double r_prime = r_np / (C.tau_r * tau_r_pre);
      rho += r_prime * rho;
      S.rho[i] = rho;
      div = S.theta[i] >= 1 ? 1 : 0;
    }
    flag[i] = div;
  }
  int tot;
  block_excl_scan(div, &tot);
  if (threadIdx.x == 0) block_count[blockIdx.x] = tot;
}

__device__ inline void put_sigma_max(CyCounters *cnt, double s) {
  atomicMax(&cnt->sigma_max_bits, static_cast<unsigned long long>(__double_as_longlong(s)));
}

// Divisions in mother order: daughter of the k-th dividing cell at n + k (calculDivisionsSingle,
// CIL.cu:527-600; singleCellDivision, MD.cu:664-718).
__global__ void __launch_bounds__(kTile) k_cy_divide(CyConst C, CySet S, CyCounters *cnt, const int *ts_dev,
                                                     const int *flag, const int *block_start, int n_blocks) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = cnt->n;
  const int ts = *ts_dev;
  const int f = (i < n) ? flag[i] : 0;
  int tot;
  const int rank = block_start[blockIdx.x] + block_excl_scan(f, &tot);
  const size_t cap = C.capacity;
  {  // the block's largest diameter, one atomic per block
    __shared__ unsigned long long smax;
    if (threadIdx.x == 0) smax = 0ull;
    __syncthreads();
    if (i < n) atomicMax(&smax, static_cast<unsigned long long>(__double_as_longlong(S.sig[i])));
    __syncthreads();
    if (threadIdx.x == 0 && smax) atomicMax(&cnt->sigma_max_bits, smax);
  }
  if (f) {
    const int inew = n + rank;
    if (inew >= C.capacity) {
      atomicOr(&cnt->err, kErrCapacity);
    } else {
      const int D = C.D;
      const double lmom = S.sig[i];
      double ldau, newsig;
      double dr[3] = {0, 0, 0};
      const u32x4 r0 = draw(C, i, ts, kCyDiv, 0);
      if (D == 2) {
        ldau = lmom / sqrt(2.0);
        newsig = ldau;
        const double rr = (lmom - ldau) / 2;
        const double alpha = u53(r0.v[0], r0.v[1]) * 6.283185307179586;
        dr[0] = rr * sin(alpha);
        dr[1] = rr * cos(alpha);
      } else {
        const double rmom = lmom / 2;
        const double vmom = 4 * kPi * rmom * rmom * rmom / 3;
        const double a = 9 * lmom / 4;
        const double b = -(3 * (lmom * lmom) / 2);
        const double c = lmom * lmom * lmom / 4 - 3 * vmom / (kPi);
        ldau = (-b + sqrt(b * b - 4 * a * c)) / (2 * a);
        newsig = ldau;
        const double rr = (lmom - ldau) / 2;
        const double alpha = u53(r0.v[0], r0.v[1]) * 6.283185307179586;
        const double beta = u53(r0.v[2], r0.v[3]) * 6.283185307179586;
        dr[0] = rr * sin(alpha) * cos(beta);
        dr[1] = rr * sin(alpha) * sin(beta);
        dr[2] = rr * cos(alpha);
      }
      CY_AXES(d, D) {
        const double m = S.x[d * cap + i];
        double xd = m + dr[d], xm = m + (-dr[d]);
        if (C.periodic[d]) {
          xd = wrap(xd, C.box[d]);
          xm = wrap(xm, C.box[d]);
        }
        S.x[d * cap + inew] = xd;
        S.x[d * cap + i] = xm;
        S.v[d * cap + inew] = 0.0;
        S.v[d * cap + i] = 0.0;
        if (S.fc) {  // resetFrc (CIL.cu:597-598)
          S.fc[d * cap + inew] = S.fd[d * cap + inew] = S.fr[d * cap + inew] = 0.0;
          S.fc[d * cap + i] = S.fd[d * cap + i] = S.fr[d * cap + i] = 0.0;
        }
      }
      // cycle times: migration spans (daughter, then mother), log-normal cycle speeds (mother,
      // then daughter), as the reference draws them
      double z0, z1, z2, z3;
      normal2(draw(C, i, ts, kCyDiv, 1), &z0, &z1);
      normal2(draw(C, i, ts, kCyDiv, 2), &z2, &z3);
      S.tsw[inew] = ts + span_steps(C.tau_mig_mu + C.tau_mig_sigma * z0, C.dt);
      S.tsw[i] = ts + span_steps(C.tau_mig_mu + C.tau_mig_sigma * z1, C.dt);
      S.om[i] = 1.0 / span_steps(lognormal(C.tau_div_mu, C.tau_div_sigma, z2), C.dt);
      S.om[inew] = 1.0 / span_steps(lognormal(C.tau_div_mu, C.tau_div_sigma, z3), C.dt);
      S.sig[inew] = newsig;
      S.sig[i] = newsig;
      S.sigt[inew] = newsig;
      S.sigt[i] = newsig;
      S.t0[inew] = ts;
      S.t0[i] = ts;
      S.theta[i] = 0;
      S.theta[inew] = 0;
      S.p[inew] = S.p[i];
      S.rho[inew] = S.rho[i];
      S.tp[inew] = -1;  // an unused slot of the reference's arrays (Colony.cpp:253)
    }
  }
}

__global__ void k_cy_commit_divisions(CyCounters *cnt, const int *block_start, int n_blocks, int capacity) {
  const int nd = block_start[n_blocks];
  const int room = capacity - cnt->n;
  const int add = nd < room ? nd : (room > 0 ? room : 0);
  cnt->n += add;
  cnt->ndiv_total += add;
  cnt->ndiv_step = add;
}

__global__ void k_cy_reset_smax(CyCounters *cnt) { cnt->sigma_max_bits = 0ull; }

__global__ void k_cy_advance(int *ts) { *ts += 1; }

// ---------------------------------------------------------------- removals
// mode 1: apoptosis (the law of C.apoptosis, one Philox block per cell and step); mode 2:
// outside the box (drain)
__global__ void __launch_bounds__(kTile) k_cy_mark(CyConst C, CySet S, CyCounters *cnt, const int *ts_dev,
                                                   int mode, int *keep, int *block_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = cnt->n;
  int k = 0;
  if (i < n) {
    k = 1;
    if (mode == 1) {
      const int ts = *ts_dev;
      const u32x4 r = draw(C, i, ts, kCyApo, 0);
      const double u = u53(r.v[0], r.v[1]);
      const double rho = S.rho[i];
      if (C.apoptosis == CIL_APOP_CYCLE_PRESSURE) {
        const double p = S.p[i];
        const double rate = C.apop_rate_step * pow((1 - (rho / C.apop_pressure)), C.apop_duration) *
                            pow(p / (p + C.p0), C.extr_gamma);
        if (u <= rate) k = 0;
      } else if (C.apoptosis == CIL_APOP_PRESSURE_TIME) {
        if (((C.apop_duration > 0) && (S.tp[i] >= C.apop_steps)) || ((C.apop_rate_step > 0) && (u <= C.apop_rate_step)))
          k = 0;
      } else if (C.apoptosis == CIL_APOP_RATE) {
        if (u <= C.apop_rate_step) k = 0;
      } else if (C.apoptosis == CIL_APOP_CYCLE) {
        if (rho < 1 && u <= C.apop_rate_step * pow((1 - (rho / C.apop_pressure)), C.apop_duration)) k = 0;
      } else {  // CIL_APOP_CYCLE_EXTRUDE
        if (rho < 1 && u <= C.apop_rate_step) k = 0;
        const double u2 = u53(r.v[2], r.v[3]);
        if (rho <= 0.1 &&
            u2 <= C.extr_rate * pow(((S.p[i] - C.apop_pressure) / C.apop_pressure), C.extr_gamma))
          k = 0;
      }
    } else {
      CY_AXES(d, C.D) {
        const double x = S.x[static_cast<size_t>(d) * C.capacity + i];
        if (!(x >= 0.0 && x < C.box[d])) k = 0;
      }
    }
    keep[i] = k;
  }
  int tot;
  block_excl_scan(k, &tot);
  if (threadIdx.x == 0) block_count[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kTile) k_cy_compact(CyConst C, CySet A, CySet B, const CyCounters *cnt,
                                                      const int *keep, const int *block_start) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = cnt->n;
  const int k = (i < n) ? keep[i] : 0;
  int tot;
  const int dst = block_start[blockIdx.x] + block_excl_scan(k, &tot);
  if (!k) return;
  const size_t cap = C.capacity;
  CY_AXES(d, C.D) {
    B.x[d * cap + dst] = A.x[d * cap + i];
    B.v[d * cap + dst] = A.v[d * cap + i];
    if (A.fc) {
      B.fc[d * cap + dst] = A.fc[d * cap + i];
      B.fd[d * cap + dst] = A.fd[d * cap + i];
      B.fr[d * cap + dst] = A.fr[d * cap + i];
    }
  }
  B.sig[dst] = A.sig[i];
  B.sigt[dst] = A.sigt[i];
  B.theta[dst] = A.theta[i];
  B.rho[dst] = A.rho[i];
  B.om[dst] = A.om[i];
  B.p[dst] = A.p[i];
  B.tp[dst] = A.tp[i];
  B.t0[dst] = A.t0[i];
  B.tsw[dst] = A.tsw[i];
}

__global__ void k_cy_commit_removals(CyCounters *cnt, const int *block_start, int n_blocks, int mode) {
  const int kept = block_start[n_blocks];
  const int removed = cnt->n - kept;
  cnt->n = kept;
  cnt->nrem_step = removed;
  if (mode == 1) cnt->napo_total += removed;
}

// ---------------------------------------------------------------- initial cell status
// initializeCellStatus (CIL.cuh:253-330) for single-element cells, counter-based draws
__global__ void k_cy_init_status(CyConst C, CySet S, const CyCounters *cnt, int ts, int fill_sigma, int fill_cycle) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt->n) return;
  if (fill_sigma) {
    S.sig[i] = C.sigma_core;
    S.sigt[i] = C.sigma_core;
  }
  S.tp[i] = 0;
  S.t0[i] = 0;
  if (!fill_cycle) return;
  S.tsw[i] = -1;
  S.rho[i] = 1;
  if (!C.divide) {
    S.theta[i] = 0;
    S.om[i] = 0;
    return;
  }
  // every cell starts in the dividing state (the migration probability is 0): a cycle length
  // max(Nint(N(tau_div) / dt), 1), the phase U[0, 1), and the elapsed part of the span
  const u32x4 r0 = draw(C, i, ts, kCyInit, 0);
  double z0, z1;
  normal2(draw(C, i, ts, kCyInit, 1), &z0, &z1);
  int span = span_steps(C.tau_div_mu + C.tau_div_sigma * z0, C.dt);
  S.om[i] = 1.0 / span;
  S.theta[i] = u53(r0.v[2], r0.v[3]);
  const u32x4 r2 = draw(C, i, ts, kCyInit, 2);
  span -= nint(u53(r2.v[0], r2.v[1]) * static_cast<double>(span)) - 1;
  S.tsw[i] = S.t0[i] + span;
}

__global__ void k_cy_sigma_max(CyConst C, CySet S, CyCounters *cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ unsigned long long smax;
  if (threadIdx.x == 0) smax = 0ull;
  __syncthreads();
  if (i < cnt->n) atomicMax(&smax, static_cast<unsigned long long>(__double_as_longlong(S.sig[i])));
  __syncthreads();
  if (threadIdx.x == 0 && smax) put_sigma_max(cnt, __longlong_as_double(static_cast<long long>(smax)));
}

}  // namespace

// ================================================================ host side
struct cil_cycle {
  cil_cycle_params p{};
  CyConst C{};
  int device = 0;
  int cap = 0;
  cudaStream_t stream = nullptr;
  CySet set[2] = {};
  int cur = 0;
  double *xs = nullptr;   // position output buffer of the force pass
  double *vs = nullptr;   // velocity output buffer of the DPD pair pass
  CyPacked P{};           // FP32 records of the bin order (precision 1)
  double *frc = nullptr;  // last forces (output only)
  double *inv_r = nullptr;  // 1 / (sigma / 2) per cell, written with the bin keys
  // captured steps: keyed by the buffer configuration before the step and the bin grid, each
  // records the configuration after it (a step rotates x / xs, v / vs and the state sets)
  struct Buffers {
    CySet set[2];
    double *xs, *vs;
    int cur;
  };
  struct StepGraph {
    Buffers before, after;
    uint64_t grid;
    cudaGraphExec_t exec;
    int64_t nodes;
  };
  std::vector<StepGraph> graphs;
  uint64_t grid_gen = 0;
  int pair_bs = kTile;  // threads per block of the per-cell pair kernels (set per call)
  int lane_bits = 0;    // log2 of the threads per cell of the contact pass (set per call)
  CyCounters *cnt = nullptr;
  CyCounters *h_cnt = nullptr;  // pinned
  int *ts_dev = nullptr;
  int *key = nullptr, *bcount = nullptr, *bstart = nullptr, *cursor = nullptr, *list = nullptr, *part = nullptr;
  int *flag = nullptr, *blk = nullptr;
  int nbins = 0, nparts = 0, nblocks = 0;
  long long nbins_cap = 0;  // bins the arrays hold
  int64_t ts = 0;
  bool uploaded = false;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double t_total = 0.0;
  int64_t launches = 0;
  std::string err;
  std::vector<void *> allocs;

  template <typename T>
  T *alloc(size_t n) {
    void *q = nullptr;
    if (cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    allocs.push_back(q);
    return static_cast<T *>(q);
  }
  cil_status fail(cil_status s, const std::string &m) {
    err = m;
    return s;
  }
};

#define CY_TRY(h, call)                                                                      \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return (h)->fail(CIL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

namespace {

cil_status check_params(const cil_cycle_params *p) {
  if (p->dim != 2 && p->dim != 3) return CIL_ERR_CONFIG;
  if (!(p->dt > 0.0) || !(p->sigma_core > 0.0) || !(p->E > 0.0)) return CIL_ERR_CONFIG;
  for (int d = 0; d < p->dim; ++d)
    if (!(p->box[d] > 0.0)) return CIL_ERR_CONFIG;
  if (p->integrator == CIL_CYCLE_EULER) {
    if (!(p->zeta > 0.0)) return CIL_ERR_CONFIG;  // "In Euler, zeta should > 0!!!" (CIL.cu:924)
  } else if (p->integrator == CIL_CYCLE_DPD) {
    // the reference's DPD step draws no passive noise (NOISE_ON is set by the stochastic
    // integrators only, Input.cpp:527-535)
    if (!(p->mass > 0.0) || !(p->kbt >= 0.0) || !(p->dis_diff >= 0.0) || !(p->dis_bg >= 0.0) || p->noise_D != 0.0)
      return CIL_ERR_CONFIG;
  } else {
    return CIL_ERR_CONFIG;
  }
  if (p->apoptosis < CIL_APOP_NONE || p->apoptosis > CIL_APOP_CYCLE_EXTRUDE) return CIL_ERR_CONFIG;
  if (p->precision != 0 && p->precision != 1) return CIL_ERR_CONFIG;
  if (p->divide && (!(p->tau_div_mu > 0.0) || !(p->cycle_p0 != 0.0) || !(p->cycle_sigma_min > 0.0) ||
                    !(p->cycle_tau_r > 0.0) || !(p->cycle_tau_v > 0.0)))
    return CIL_ERR_CONFIG;
  // a migration time (crawling state) takes cells out of the single-element cycle for good in
  // the reference (initializeCellStatus with calculDivisionsSingle); the shipped runs use 0
  if (p->divide && p->tau_mig_mu != 0.0) return CIL_ERR_CONFIG;
  return CIL_OK;
}

int blocks_for(int n) { return n > 0 ? (n + kTile - 1) / kTile : 1; }

constexpr int kNumSMs = 152;  // GB300

// grid of a per-cell pair kernel at h->pair_bs threads per block
int pair_grid(const cil_cycle *h) { return (h->cap + h->pair_bs - 1) / h->pair_bs; }

// Threads per cell of the contact pass: up to 8, while the colony gives fewer than two warps
// per scheduler of every SM (152 SMs x 4 x 2 x 32 threads), and while the grid over the
// capacity stays within 2^24 threads. The restatement uses the same rule.
int contact_lane_bits(long long ncells, long long capacity) {
  int b = 0;
  while (b < 3 && ncells * (2LL << b) <= 2LL * kNumSMs * 4 * 32 && (capacity << (b + 1)) <= (1LL << 24)) ++b;
  return b;
}

int bins_along(double box, double width) {
  const int ns = static_cast<int>(box / width);
  return ns < 1 ? 1 : (ns > 4096 ? 4096 : ns);
}

// The bin grid of a step call: bins at least 1.05 x max(SIGMA_CORE, the colony's largest
// diameter) wide, so that the pair search spans one bin on each side (3^D bins) unless cells
// grow by more than 5 % within the call (the search then widens by itself). Narrower bins than
// the diameter would make every search span two bins on each side (5^D bins). The host
// restatement picks its grid by the same rule at the start of each call.
void set_bins(cil_cycle *h, double smax, int ncells) {
  CyConst &C = h->C;
  const double w = (smax > h->p.sigma_core ? smax : h->p.sigma_core) * 1.05;
  const int before[3] = {C.ns[0], C.ns[1], C.ns[2]};
  // blocks of the per-cell pair kernels (FP64-heavy, no block cooperation): small enough that
  // a small colony still spreads over every SM (two blocks per SM), 32 to kTile threads
  const int bs_before = h->pair_bs, lb_before = h->lane_bits;
  h->lane_bits = contact_lane_bits(ncells, h->cap);
  if (h->lane_bits != lb_before) h->grid_gen += 1;
  h->pair_bs = 32;
  while (h->pair_bs < kTile && static_cast<long long>(h->pair_bs) * 2 * kNumSMs < ncells) h->pair_bs *= 2;
  // the grids cover the capacity: keep them at most 65536 blocks (a large capacity, few cells)
  while (h->pair_bs < kTile && (h->cap + h->pair_bs - 1) / h->pair_bs > 65536) h->pair_bs *= 2;
  if (h->pair_bs != bs_before) h->grid_gen += 1;
  h->nbins = 1;
  for (int d = 0; d < 3; ++d) {
    if (d < h->p.dim) {
      const int ns = bins_along(C.box[d], w);
      C.ns[d] = ns;
      C.bw[d] = C.box[d] / ns;
      C.inv_bw[d] = ns / C.box[d];
    } else {
      C.ns[d] = 1;
      C.bw[d] = 1.0;
      C.inv_bw[d] = 1.0;
    }
    C.bwf[d] = static_cast<float>(C.bw[d]);
    h->nbins *= C.ns[d];
  }
  if (C.ns[0] != before[0] || C.ns[1] != before[1] || C.ns[2] != before[2]) h->grid_gen += 1;
}

double host_sigma_max(const cil_cycle *h) {
  double s;
  const unsigned long long b = h->h_cnt->sigma_max_bits;
  std::memcpy(&s, &b, sizeof s);
  return s;
}

// scan of count[0..m) into start[0..m] (start[m] = total)
void scan_into(cil_cycle *h, const int *count, int m, int *start) {
  const int nchunks = m / kScanTile + 1;  // covers index m
  k_cy_chunk_sums<<<nchunks, kTile, 0, h->stream>>>(count, m, h->part);
  k_cy_scan_small<<<1, kTile, 0, h->stream>>>(h->part, nchunks);
  k_cy_chunk_apply<<<nchunks, kTile, 0, h->stream>>>(count, m, h->part, start);
  h->launches += 3;
}

cil_status bin_cells(cil_cycle *h) {
  const CySet &S = h->set[h->cur];
  const int g = blocks_for(h->cap);
  k_cy_clear<<<256, kTile, 0, h->stream>>>(h->bcount, h->nbins);
  k_cy_keys<<<g, kTile, 0, h->stream>>>(h->C, S, h->cnt, h->key, h->bcount, h->inv_r);
  scan_into(h, h->bcount, h->nbins, h->bstart);
  k_cy_clear<<<256, kTile, 0, h->stream>>>(h->cursor, h->nbins);
  k_cy_scatter<<<g, kTile, 0, h->stream>>>(h->cnt, h->key, h->bstart, h->cursor, h->list);
  k_cy_sort<<<blocks_for(h->nbins), kTile, 0, h->stream>>>(h->bstart, h->nbins, h->list, h->cnt);
  h->launches += 5;
  if (h->p.precision == 1) {
    k_cy_pack<<<g, kTile, 0, h->stream>>>(h->C, S, h->cnt, h->list, h->P, h->C.dpd);
    h->launches += 1;
  }
  return CIL_OK;
}

cil_status removals(cil_cycle *h, int mode) {
  const int g = pair_grid(h), bs = h->pair_bs;
  CySet &A = h->set[h->cur];
  CySet &B = h->set[1 - h->cur];
  k_cy_mark<<<g, bs, 0, h->stream>>>(h->C, A, h->cnt, h->ts_dev, mode, h->flag, h->blk);
  k_cy_scan_small<<<1, kTile, 0, h->stream>>>(h->blk, g);
  k_cy_compact<<<g, bs, 0, h->stream>>>(h->C, A, B, h->cnt, h->flag, h->blk);
  k_cy_commit_removals<<<1, 1, 0, h->stream>>>(h->cnt, h->blk, g, mode);
  h->launches += 4;
  h->cur = 1 - h->cur;
  return CIL_OK;
}

void launch_force(cil_cycle *h, CySet &S, double *x_out, double *frc, int mode, int key_off) {
  const int bs = h->pair_bs;
  const long long threads = static_cast<long long>(h->cap) << h->lane_bits;
  const int g = static_cast<int>((threads + bs - 1) / bs);
  if (h->p.precision == 1)
    k_cy_force<true><<<g, bs, 0, h->stream>>>(h->C, S, x_out, frc, h->cnt, h->bstart, h->list, h->ts_dev, mode,
                                                 key_off, h->P, h->lane_bits, h->inv_r);
  else
    k_cy_force<false><<<g, bs, 0, h->stream>>>(h->C, S, x_out, frc, h->cnt, h->bstart, h->list, h->ts_dev, mode,
                                                  key_off, h->P, h->lane_bits, h->inv_r);
  h->launches += 1;
}

void launch_dpd_pair(cil_cycle *h, CySet &S, int key_off, int kick_on) {
  const int g = pair_grid(h), bs = h->pair_bs;
  if (h->p.precision == 1)
    k_dpd_pair<true><<<g, bs, 0, h->stream>>>(h->C, S, h->vs, h->cnt, h->bstart, h->list, h->ts_dev, key_off,
                                                 kick_on, h->P);
  else
    k_dpd_pair<false><<<g, bs, 0, h->stream>>>(h->C, S, h->vs, h->cnt, h->bstart, h->list, h->ts_dev, key_off,
                                                  kick_on, h->P);
}

// Fc, pressure, Fd and Fr at the current positions and velocities (the forces the reference
// evaluates before its first step, CIL.cu:1096), draws keyed by the current step counter
void dpd_initial_forces(cil_cycle *h) {
  CySet &S = h->set[h->cur];
  bin_cells(h);
  launch_force(h, S, nullptr, S.fc, 1, 0);
  launch_dpd_pair(h, S, 0, 0);
  h->launches += 1;
}

cil_status enqueue_step(cil_cycle *h) {
  const int g = blocks_for(h->cap);
  CySet &S = h->set[h->cur];
  if (h->C.dpd) {  // DPD (CIL.cu:1054-1066); this step's draws are keyed by ts + 1
    k_dpd_kick_drift<<<g, kTile, 0, h->stream>>>(h->C, S, h->cnt);
    bin_cells(h);
    launch_force(h, S, nullptr, S.fc, 1, 1);
    launch_dpd_pair(h, S, 1, 1);
    std::swap(S.v, h->vs);
    if (h->p.precision == 1) {  // the records take the new velocities
      k_cy_pack_vel<<<g, kTile, 0, h->stream>>>(h->C, S, h->cnt, h->list, h->P);
      k_dpd_dis<true><<<pair_grid(h), h->pair_bs, 0, h->stream>>>(h->C, S, h->cnt, h->bstart, h->list, h->P);
      h->launches += 1;
    } else {
      k_dpd_dis<false><<<pair_grid(h), h->pair_bs, 0, h->stream>>>(h->C, S, h->cnt, h->bstart, h->list, h->P);
    }
    h->launches += 3;
  } else {
    bin_cells(h);
    launch_force(h, S, h->xs, h->frc, 0, 0);
    std::swap(S.x, h->xs);
  }
  k_cy_advance<<<1, 1, 0, h->stream>>>(h->ts_dev);
  h->ts += 1;
  h->launches += 1;
  if (h->C.divide) {
    const int ge = pair_grid(h), bs = h->pair_bs;  // per-cell event kernels: the pair kernels' blocks
    k_cy_cycle<<<ge, bs, 0, h->stream>>>(h->C, S, h->cnt, h->ts_dev, h->flag, h->blk);
    k_cy_scan_small<<<1, kTile, 0, h->stream>>>(h->blk, ge);
    k_cy_reset_smax<<<1, 1, 0, h->stream>>>(h->cnt);
    k_cy_divide<<<ge, bs, 0, h->stream>>>(h->C, S, h->cnt, h->ts_dev, h->flag, h->blk, ge);
    k_cy_commit_divisions<<<1, 1, 0, h->stream>>>(h->cnt, h->blk, ge, h->cap);
    h->launches += 5;
  }
  if (h->C.apoptosis != CIL_APOP_NONE) removals(h, 1);
  CY_TRY(h, cudaGetLastError());
  return CIL_OK;
}

constexpr size_t kMaxStepGraphs = 16;

cil_cycle::Buffers buffers_of(const cil_cycle *h) {
  cil_cycle::Buffers b{};
  b.set[0] = h->set[0];
  b.set[1] = h->set[1];
  b.xs = h->xs;
  b.vs = h->vs;
  b.cur = h->cur;
  return b;
}

bool same_buffers(const cil_cycle::Buffers &a, const cil_cycle::Buffers &b) {
  return std::memcmp(&a.set[0], &b.set[0], sizeof(CySet)) == 0 &&
         std::memcmp(&a.set[1], &b.set[1], sizeof(CySet)) == 0 && a.xs == b.xs && a.vs == b.vs && a.cur == b.cur;
}

// One step through the graph of its buffer configuration: captured from enqueue_step the first
// time (the capture leaves the host state as the step leaves it), replayed afterwards
cil_status graph_step(cil_cycle *h) {
  const cil_cycle::Buffers b = buffers_of(h);
  for (const auto &g : h->graphs)
    if (g.grid == h->grid_gen && same_buffers(g.before, b)) {
      CY_TRY(h, cudaGraphLaunch(g.exec, h->stream));
      h->set[0] = g.after.set[0];
      h->set[1] = g.after.set[1];
      h->xs = g.after.xs;
      h->vs = g.after.vs;
      h->cur = g.after.cur;
      h->ts += 1;
      h->launches += g.nodes;
      return CIL_OK;
    }
  if (h->graphs.size() >= kMaxStepGraphs) return enqueue_step(h);
  const int64_t l0 = h->launches, ts0 = h->ts;
  if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return enqueue_step(h);
  }
  const cil_status st = enqueue_step(h);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
  cudaGraphExec_t exec = nullptr;
  cudaError_t ie = cudaErrorUnknown;
  if (st == CIL_OK && ce == cudaSuccess && graph) ie = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    // nothing ran: put the host state back as it was before the capture and launch the step
    cudaGetLastError();
    h->set[0] = b.set[0];
    h->set[1] = b.set[1];
    h->xs = b.xs;
    h->vs = b.vs;
    h->cur = b.cur;
    h->ts = ts0;
    h->launches = l0;
    return enqueue_step(h);
  }
  h->graphs.push_back({b, buffers_of(h), h->grid_gen, exec, h->launches - l0});
  CY_TRY(h, cudaGraphLaunch(exec, h->stream));
  return CIL_OK;
}

cil_status read_counters(cil_cycle *h) {
  CY_TRY(h, cudaMemcpyAsync(h->h_cnt, h->cnt, sizeof(CyCounters), cudaMemcpyDeviceToHost, h->stream));
  CY_TRY(h, cudaStreamSynchronize(h->stream));
  if (h->h_cnt->err & kErrNonFinite) return h->fail(CIL_ERR_NAN, "non-finite force");
  if (h->h_cnt->err & kErrCapacity) return h->fail(CIL_ERR_CAPACITY, "cell capacity exceeded");
  if (h->h_cnt->err & kErrOutOfBox) return h->fail(CIL_ERR_OUT_OF_BOX, "Particle outside domain!");
  if (h->h_cnt->err & kErrCrowded) return h->fail(CIL_ERR_CAPACITY, "more than 256 cells in one bin (overlapping cells)");
  return CIL_OK;
}

}  // namespace

extern "C" {

cil_status cil_cycle_create(const cil_cycle_params *p, int32_t capacity, uint64_t seed, int32_t device,
                            cil_cycle **out) {
  if (!p || !out || capacity <= 0) return CIL_ERR_CONFIG;
  *out = nullptr;
  if (check_params(p) != CIL_OK) return CIL_ERR_CONFIG;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return CIL_ERR_CUDA;
  }
  cil_cycle *h = new cil_cycle();
  h->p = *p;
  h->device = device;
  h->cap = capacity;
  CyConst &C = h->C;
  C.D = p->dim;
  C.capacity = capacity;
  C.dt = p->dt;
  for (int d = 0; d < 3; ++d) {
    C.periodic[d] = d < p->dim ? p->periodic[d] : 0;
    C.box[d] = d < p->dim ? p->box[d] : 1.0;
    C.half[d] = 0.5 * C.box[d];
    C.boxf[d] = static_cast<float>(C.box[d]);
    C.halff[d] = static_cast<float>(C.half[d]);
  }
  // bin arrays for the finest grid the colony can use (width SIGMA_CORE); set_bins picks the
  // grid of each call
  h->nbins_cap = 1;
  for (int d = 0; d < p->dim; ++d) h->nbins_cap *= bins_along(C.box[d], p->sigma_core);
  C.sigma_core = p->sigma_core;
  set_bins(h, p->sigma_core, capacity);
  C.hz_c = (1 - p->nu * p->nu) / p->E;
  C.adhesion = p->adhesion;
  C.motility = p->motility;
  C.zeta = p->zeta;
  C.zeta_p = p->zeta_p;
  C.zeta_p_beta = p->zeta_p_beta;
  C.noise_amp = p->noise_D > 0.0 ? std::sqrt(2.0 * p->noise_D) * (1.0 / std::sqrt(p->dt)) : 0.0;
  C.divide = p->divide;
  C.apoptosis = p->apoptosis;
  C.tau_div_mu = p->tau_div_mu;
  C.tau_div_sigma = p->tau_div_sigma;
  C.tau_mig_mu = p->tau_mig_mu;
  C.tau_mig_sigma = p->tau_mig_sigma;
  // cycle times in steps (Input.cpp:176-178, CIL.cuh:225-233)
  C.v1 = p->v1;
  C.tau_r = p->cycle_tau_r * p->tau_div_mu / p->dt;
  C.tau_v = p->cycle_tau_v * p->tau_div_mu / p->dt;
  C.tau_p = p->cycle_tau_p * p->tau_div_mu / p->dt;
  {
    const double r = p->cycle_sigma_min / 2;
    C.v_s = p->dim == 3 ? 4 * kPi * (r * r * r) / 3 : kPi * (r * r);  // Sigma2Volume / Sigma2Area
  }
  C.p0 = p->cycle_p0;
  C.beta_vs = p->cycle_beta_vs;
  C.rho_ratio = p->cycle_rho_ratio;
  C.r_maxed_inv = p->cycle_r_maxed > 0.0 ? 1.0 / p->cycle_r_maxed : 1.0;
  C.p_shift = p->cycle_p_shift * p->cycle_p0;
  C.p_shift_tau_inv = p->cycle_p_shift_tau > 0.0 ? 1.0 / (p->cycle_p_shift_tau * p->tau_div_mu) * p->dt : 0.0;
  C.osm = p->osmotic_pressure;
  C.apop_pressure = p->apop_pressure;
  C.apop_duration = p->apop_duration;
  C.apop_rate_step = p->apop_rate * p->dt;
  C.extr_gamma = p->extr_gamma;
  C.apop_steps = p->apop_duration / p->dt;
  C.extr_rate = p->extr_rate;
  C.dpd = p->integrator == CIL_CYCLE_DPD ? 1 : 0;
  C.kick_div = 2 * (2 * p->mass);
  C.sqrt_dt = std::sqrt(p->dt);
  C.gamma_d = p->dis_diff;
  C.gamma_b = p->dis_bg;
  C.sigma_r = std::sqrt(2 * p->dis_diff * p->kbt);  // Sigma (MD.cu:872)
  C.seed_lo = static_cast<uint32_t>(seed);
  C.seed_hi = static_cast<uint32_t>(seed >> 32);

  const size_t cap = capacity, D = p->dim;
  bool ok = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreate(&h->ev[0]) == cudaSuccess && cudaEventCreate(&h->ev[1]) == cudaSuccess;
  for (int s = 0; ok && s < 2; ++s) {
    CySet &S = h->set[s];
    S.x = h->alloc<double>(D * cap);
    S.v = h->alloc<double>(D * cap);
    S.sig = h->alloc<double>(cap);
    S.sigt = h->alloc<double>(cap);
    S.theta = h->alloc<double>(cap);
    S.rho = h->alloc<double>(cap);
    S.om = h->alloc<double>(cap);
    S.p = h->alloc<double>(cap);
    S.tp = h->alloc<int>(cap);
    S.t0 = h->alloc<int>(cap);
    S.tsw = h->alloc<int>(cap);
    ok = S.x && S.v && S.sig && S.sigt && S.theta && S.rho && S.om && S.p && S.tp && S.t0 && S.tsw;
    if (ok && C.dpd) {
      S.fc = h->alloc<double>(D * cap);
      S.fd = h->alloc<double>(D * cap);
      S.fr = h->alloc<double>(D * cap);
      ok = S.fc && S.fd && S.fr;
    }
  }
  if (ok && C.dpd) {
    h->vs = h->alloc<double>(D * cap);
    ok = h->vs != nullptr;
  }
  if (ok && p->precision == 1) {
    h->P.pk = h->alloc<float4>(cap);
    h->P.qpos = h->alloc<int>(cap);
    h->P.vk = C.dpd ? h->alloc<float4>(cap) : nullptr;
    ok = h->P.pk && h->P.qpos && (!C.dpd || h->P.vk);
  }
  h->nblocks = (capacity + 31) / 32;  // blocks of the per-cell event kernels at their smallest (32 threads)
  h->nparts = (h->nbins_cap + kScanTile - 1) / kScanTile + 1;
  if (ok) {
    h->xs = h->alloc<double>(D * cap);
    h->frc = h->alloc<double>(D * cap);
    h->inv_r = h->alloc<double>(cap);
    h->cnt = h->alloc<CyCounters>(1);
    h->ts_dev = h->alloc<int>(1);
    h->key = h->alloc<int>(cap);
    h->bcount = h->alloc<int>(h->nbins_cap + 1);
    h->bstart = h->alloc<int>(h->nbins_cap + 1);
    h->cursor = h->alloc<int>(h->nbins_cap + 1);
    h->list = h->alloc<int>(cap);
    h->part = h->alloc<int>(h->nparts + 1);
    h->flag = h->alloc<int>(cap);
    h->blk = h->alloc<int>(h->nblocks + 1);
    ok = h->xs && h->frc && h->inv_r && h->cnt && h->ts_dev && h->key && h->bcount && h->bstart && h->cursor && h->list &&
         h->part && h->flag && h->blk &&
         cudaHostAlloc(&h->h_cnt, sizeof(CyCounters), cudaHostAllocDefault) == cudaSuccess;
  }
  if (ok) ok = cudaMemsetAsync(h->cnt, 0, sizeof(CyCounters), h->stream) == cudaSuccess &&
               cudaMemsetAsync(h->ts_dev, 0, sizeof(int), h->stream) == cudaSuccess &&
               cudaStreamSynchronize(h->stream) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    cil_cycle_destroy(h);
    return CIL_ERR_CUDA;
  }
  *out = h;
  return CIL_OK;
}

void cil_cycle_destroy(cil_cycle *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto &g : h->graphs) cudaGraphExecDestroy(g.exec);
  for (void *q : h->allocs) cudaFree(q);
  if (h->h_cnt) cudaFreeHost(h->h_cnt);
  for (auto e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

cil_status cil_cycle_upload(cil_cycle *h, const cil_cycle_view *v) {
  if (!h || !v || !v->pos) return CIL_ERR_CONFIG;
  if (v->ncells < 0 || v->ncells > h->cap) return h->fail(CIL_ERR_CAPACITY, "cil_cycle_upload: more cells than the capacity");
  CY_TRY(h, cudaSetDevice(h->device));
  const int n = v->ncells, D = h->C.D;
  const size_t cap = h->cap;
  h->cur = 0;
  CySet &S = h->set[0];
  std::vector<double> t(static_cast<size_t>(n));
  for (int d = 0; d < D; ++d) {
    for (int i = 0; i < n; ++i) {
      const double x = v->pos[static_cast<size_t>(i) * D + d];
      if (!(x >= 0.0 && x < h->C.box[d])) return h->fail(CIL_ERR_OUT_OF_BOX, "Input Positions Out of Bounds!");
      t[i] = x;
    }
    CY_TRY(h, cudaMemcpy(S.x + d * cap, t.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CY_TRY(h, cudaMemset(S.v + d * cap, 0, sizeof(double) * cap));
    if (v->vel) {
      for (int i = 0; i < n; ++i) t[i] = v->vel[static_cast<size_t>(i) * D + d];
      CY_TRY(h, cudaMemcpy(S.v + d * cap, t.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    }
  }
  auto up = [&](double *dst, const double *src) -> cudaError_t {
    return src ? cudaMemcpy(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  CY_TRY(h, up(S.sig, v->sigma));
  CY_TRY(h, up(S.sigt, v->sigma_t ? v->sigma_t : v->sigma));
  CY_TRY(h, up(S.theta, v->theta));
  CY_TRY(h, up(S.rho, v->rho));
  CY_TRY(h, up(S.om, v->angvel));
  CY_TRY(h, cudaMemset(S.p, 0, sizeof(double) * cap));
  if (v->pressure) CY_TRY(h, up(S.p, v->pressure));
  CyCounters c{};
  c.n = n;
  CY_TRY(h, cudaMemcpy(h->cnt, &c, sizeof(c), cudaMemcpyHostToDevice));
  const int ts = v->ts;
  CY_TRY(h, cudaMemcpy(h->ts_dev, &ts, sizeof(int), cudaMemcpyHostToDevice));
  h->ts = ts;
  const int fill_sigma = v->sigma ? 0 : 1;
  const int fill_cycle = (v->theta && v->rho && v->angvel) ? 0 : 1;
  k_cy_init_status<<<blocks_for(h->cap), kTile, 0, h->stream>>>(h->C, S, h->cnt, ts, fill_sigma, fill_cycle);
  if (v->tpressure) {
    CY_TRY(h, cudaStreamSynchronize(h->stream));
    CY_TRY(h, cudaMemcpy(S.tp, v->tpressure, sizeof(int) * n, cudaMemcpyHostToDevice));
  }
  k_cy_sigma_max<<<blocks_for(h->cap), kTile, 0, h->stream>>>(h->C, S, h->cnt);
  CY_TRY(h, cudaGetLastError());
  const cil_status st = read_counters(h);
  if (st != CIL_OK) return st;
  set_bins(h, host_sigma_max(h), h->h_cnt->n);
  h->uploaded = true;
  if (!h->C.dpd) return CIL_OK;
  dpd_initial_forces(h);
  CY_TRY(h, cudaGetLastError());
  return read_counters(h);
}

cil_status cil_cycle_step(cil_cycle *h, int32_t nsteps, int64_t *ts) {
  if (!h) return CIL_ERR_CONFIG;
  if (!h->uploaded) return h->fail(CIL_ERR_STATE, "cil_cycle_step before cil_cycle_upload");
  if (nsteps < 0) return h->fail(CIL_ERR_CONFIG, "negative step count");
  CY_TRY(h, cudaSetDevice(h->device));
  // the counters of the last call (every entry point ends by reading them)
  set_bins(h, host_sigma_max(h), h->h_cnt->n);
  h->launches = 0;
  CY_TRY(h, cudaEventRecord(h->ev[0], h->stream));
  const bool graphs = !(h->p.flags & CIL_CYCLE_NO_GRAPH);
  for (int k = 0; k < nsteps; ++k) {
    const cil_status st = graphs ? graph_step(h) : enqueue_step(h);
    if (st != CIL_OK) return st;
  }
  CY_TRY(h, cudaEventRecord(h->ev[1], h->stream));
  const cil_status st = read_counters(h);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
  h->t_total = ms;
  if (ts) *ts = h->ts;
  return st;
}

cil_status cil_cycle_check_positions(cil_cycle *h) {
  if (!h) return CIL_ERR_CONFIG;
  if (!h->uploaded) return h->fail(CIL_ERR_STATE, "not uploaded");
  CY_TRY(h, cudaSetDevice(h->device));
  if (h->p.drain) {
    removals(h, 2);
    CY_TRY(h, cudaGetLastError());
    return read_counters(h);
  }
  // without drain any cell off the box is an error (run_assert, CIL.cu:956)
  const int g = pair_grid(h);
  k_cy_mark<<<g, h->pair_bs, 0, h->stream>>>(h->C, h->set[h->cur], h->cnt, h->ts_dev, 2, h->flag, h->blk);
  k_cy_scan_small<<<1, kTile, 0, h->stream>>>(h->blk, g);
  CY_TRY(h, cudaGetLastError());
  cil_status st = read_counters(h);
  if (st != CIL_OK) return st;
  int kept = 0;
  CY_TRY(h, cudaMemcpy(&kept, h->blk + g, sizeof(int), cudaMemcpyDeviceToHost));
  if (kept != h->h_cnt->n) return h->fail(CIL_ERR_OUT_OF_BOX, "Particle outside domain!");
  return CIL_OK;
}

cil_status cil_cycle_download(cil_cycle *h, cil_cycle_view *v) {
  if (!h || !v) return CIL_ERR_CONFIG;
  CY_TRY(h, cudaSetDevice(h->device));
  if (h->uploaded && !h->C.dpd) {
    const int64_t launches = h->launches;  // cil_cycle_timings reports the last cil_cycle_step
    // the forces and pressures at the current state, which the reference's Euler step
    // evaluates at its end (CIL.cu:1019) and writes out; the next step's force pass computes
    // the same values again (same positions, velocities and step key)
    bin_cells(h);
    launch_force(h, h->set[h->cur], nullptr, h->frc, 1, 0);
    h->launches = launches;
    CY_TRY(h, cudaGetLastError());
  }
  const cil_status st = read_counters(h);
  const int n = h->h_cnt->n, D = h->C.D;
  v->ncells = n;
  v->ts = static_cast<int32_t>(h->ts);
  if (n > v->capacity) return h->fail(CIL_ERR_CAPACITY, "cil_cycle_download: host arrays too small");
  const CySet &S = h->set[h->cur];
  const size_t cap = h->cap;
  std::vector<double> t(static_cast<size_t>(n) * D);
  auto vec = [&](double *dst, const double *src) -> cudaError_t {
    if (!dst) return cudaSuccess;
    for (int d = 0; d < D; ++d) {
      const cudaError_t e = cudaMemcpy(t.data() + static_cast<size_t>(d) * n, src + d * cap, sizeof(double) * n,
                                       cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return e;
    }
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < D; ++d) dst[static_cast<size_t>(i) * D + d] = t[static_cast<size_t>(d) * n + i];
    return cudaSuccess;
  };
  auto sca = [&](void *dst, const void *src, size_t es) -> cudaError_t {
    return dst ? cudaMemcpy(dst, src, es * n, cudaMemcpyDeviceToHost) : cudaSuccess;
  };
  CY_TRY(h, vec(v->pos, S.x));
  CY_TRY(h, vec(v->vel, S.v));
  CY_TRY(h, sca(v->sigma, S.sig, sizeof(double)));
  CY_TRY(h, sca(v->sigma_t, S.sigt, sizeof(double)));
  CY_TRY(h, sca(v->theta, S.theta, sizeof(double)));
  CY_TRY(h, sca(v->rho, S.rho, sizeof(double)));
  CY_TRY(h, sca(v->angvel, S.om, sizeof(double)));
  CY_TRY(h, sca(v->pressure, S.p, sizeof(double)));
  CY_TRY(h, sca(v->tpressure, S.tp, sizeof(int)));
  CY_TRY(h, sca(v->t0, S.t0, sizeof(int)));
  if (h->C.dpd) {
    CY_TRY(h, vec(v->force, S.fc));
    CY_TRY(h, vec(v->force_dis, S.fd));
    CY_TRY(h, vec(v->force_ran, S.fr));
  } else {
    CY_TRY(h, vec(v->force, h->frc));
    for (double *f : {v->force_dis, v->force_ran})
      if (f) std::fill(f, f + static_cast<size_t>(n) * D, 0.0);
  }
  return st;
}

cil_status cil_cycle_timings(cil_cycle *h, double *total_ms, int64_t *launches) {
  if (!h) return CIL_ERR_CONFIG;
  if (total_ms) *total_ms = h->t_total;
  if (launches) *launches = h->launches;
  return CIL_OK;
}

void cil_cycle_last_error(const cil_cycle *h, char *buf, size_t len) {
  if (!buf || len == 0) return;
  snprintf(buf, len, "%s", h ? h->err.c_str() : "");
}

}  // extern "C"
