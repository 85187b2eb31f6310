// ORACLE — test infrastructure only (see cil_oracle.h for what is pinned and what is not).
//
// Restates the reference's Euler step for 2-element cells. Per step, in the reference's
// order (CIL.cu:1013-1020 with the force evaluation moved to the head of the step, which
// is the same sequence of operations since the reference evaluates forces once before the
// loop, CIL.cu:1097):
//   forces (noise draw CIL.cu:793-818, intra CIL.cu:30-100, inter CIL.cu:177-231)
//   -> integrate (CIL.cu:858-875 / Utils.hpp:561-566) -> ++ts -> division (CIL.cu:369-455)
//   -> apoptosis (CIL.cu:627-649).
// With ora_set_integrator(h, 1) a step is the reference's StochasticHeun (CIL.cu:1028-1050):
// two half steps, each a force evaluation with its own noise draw and x += (dt/2) F / zeta,
// then ++ts, division, apoptosis. The reference leaves the velocities of a Heun step stale;
// here they are the mean of the two half steps' F / zeta (the library's definition).
// Build: oracle/build.sh (gcc -O2 -ffp-contract=off -fno-fast-math, optional OpenMP).
#include "cil_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "dsfmt19937.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;

// Utils.hpp:173-175 — round half away from zero
inline int nint(double a) { return a >= 0.0 ? static_cast<int>(a + 0.5) : static_cast<int>(a - 0.5); }

// Random.hpp:9-114 on top of the restated dSFMT
struct Rng {
  ora::Dsfmt19937 g;
  void init(uint32_t s) { g.seed(s); }
  double uniform() { return (g.open_open() - 0.5) * 2.0; }          // Random.hpp:16-18
  double uniform0x(double x) { return g.close_open() * x; }          // Random.hpp:19-21
  double normal() {                                                  // Random.hpp:28-56 (Leva 1992)
    const double s = 0.449871, t = -0.386595, a = 0.19600, b = 0.25472;
    const double r1 = 0.27597, r2 = 0.27846;
    double u, v, x, y, q;
    do {
      u = 1.0 - g.close_open();
      v = 1.7156 * (g.close_open() - 0.5);
      x = u - s;
      y = std::fabs(v) - t;
      q = x * x + y * (a * y - b * x);
    } while (q >= r1 && (q > r2 || v * v > -4.0 * u * u * std::log(u)));
    return v / u;
  }
  double normal(double mu, double sigma) { return mu + sigma * normal(); }  // Random.hpp:57
  double inside_dsphere(int dim, double *ni) {                               // Random.hpp:89-102
    double r2;
    for (;;) {
      r2 = 0.0;
      for (int d = 0; d < dim; ++d) {
        ni[d] = uniform();
        r2 += ni[d] * ni[d];
      }
      if (r2 <= 1.0) return r2;
    }
  }
  void on_dsphere(int dim, double *ni) {  // Random.hpp:115-118
    double norm = 1.0 / std::sqrt(inside_dsphere(dim, ni));
    for (int d = 0; d < dim; ++d) ni[d] *= norm;
  }
};

// Orthorhombic link list geometry: Utils.hpp:872-876 (get_opt_size), 891-908 (reset),
// 922-936 (get_cellID), 982-1001 (populate_list), 1018-1069 (2D/3D ids and coordinates).
struct LinkGrid {
  int dim = 2;
  int ns[3] = {1, 1, 1};
  double ih[3] = {0, 0, 0};
  bool pbc[3] = {false, false, false};
  int ncells = 1;

  void init(int d, double rcut, const double *lbox, const int32_t *periodic) {
    dim = d;
    double mn = lbox[0];
    for (int k = 1; k < dim; ++k) mn = std::min(mn, lbox[k]);
    const double delta = mn * 1.0e-8;
    const double ir = 1.0 / (rcut + delta);
    bool overkill = false;
    for (int k = 0; k < 3; ++k) {
      ns[k] = 1;
      ih[k] = 0.0;
      pbc[k] = false;
    }
    for (int k = 0; k < dim; ++k) {
      ns[k] = static_cast<int>(lbox[k] * ir);
      ih[k] = 1.0 / lbox[k];
      pbc[k] = periodic[k] != 0;
      overkill = overkill || ns[k] < 3;
    }
    if (overkill) {
      for (int k = 0; k < dim; ++k) ns[k] = 1;
      ncells = 1;
    } else {
      ncells = 1;
      for (int k = 0; k < dim; ++k) ncells *= ns[k];
    }
  }
  int id0(const int *ls) const {
    return dim == 2 ? ls[0] * ns[1] + ls[1] : (ls[0] * ns[1] + ls[1]) * ns[2] + ls[2];
  }
  // Bin of a position. The reference indexes out of range for a coordinate outside
  // [0, L) along a non-periodic axis; the restatement clamps to the edge bin instead.
  int bin_of(const double *r) const {
    int ls[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      int v = std::min(static_cast<int>((r[d] * ih[d]) * ns[d]), ns[d] - 1);
      ls[d] = v < 0 ? 0 : v;
    }
    return id0(ls);
  }
  void coord(int i, int *c) const {
    if (dim == 2) {
      c[0] = i / ns[1];
      c[1] = i - ns[1] * c[0];
    } else {
      c[0] = i / (ns[1] * ns[2]);
      int ii = i - c[0] * ns[1] * ns[2];
      c[1] = ii / ns[2];
      c[2] = ii - c[1] * ns[2];
    }
  }
  int neighbor(const int *c, const int *dc) const {
    int ls[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      ls[d] = c[d] + dc[d];
      if (pbc[d])
        ls[d] = (ls[d] + ns[d]) % ns[d];
      else if (ls[d] < 0 || ls[d] >= ns[d])
        return -1;
    }
    return id0(ls);
  }
  // LIFO fill: the last inserted index is the head (Utils.hpp:982-1001)
  void populate(const double *r, int num, std::vector<int> &head, std::vector<int> &list) const {
    head.assign(ncells, -1);
    list.assign(num, -1);
    for (int i = 0; i < num; ++i) {
      int k = bin_of(r + static_cast<size_t>(i) * dim);
      if (head[k] == -1) {
        head[k] = i;
      } else {
        list[i] = head[k];
        head[k] = i;
      }
    }
  }
};

// BoundingBox::distance, Utils.hpp:536-544: r12 = r2 - r1, minus the nearest whole box along
// periodic axes (Nint of r12 / L); returns |r12|^2
double box_distance(int D, const double *box, const int32_t *periodic, double *r12, const double *r1,
                    const double *r2) {
  double ans = 0.0;
  for (int d = 0; d < D; ++d) {
    r12[d] = r2[d] - r1[d];
    if (periodic[d]) r12[d] -= static_cast<double>(nint(r12[d] / box[d])) * box[d];
    ans += r12[d] * r12[d];
  }
  return ans;
}
// BoundingBox::updatePos(r, v, dt), Utils.hpp:561-566
void box_update_pos(int D, const double *box, const int32_t *periodic, double *r, const double *v, double dt) {
  for (int d = 0; d < D; ++d)
    r[d] = periodic[d] ? std::fmod(r[d] + dt * v[d] + box[d], box[d]) : r[d] + v[d] * dt;
}
// BoundingBox::updatePos(r, dr), Utils.hpp:556-559
void box_update_pos(int D, const double *box, const int32_t *periodic, double *r, const double *dr) {
  for (int d = 0; d < D; ++d) r[d] = periodic[d] ? std::fmod(r[d] + dr[d] + box[d], box[d]) : r[d] + dr[d];
}

// Element pair force modulus f0 (force on i is f0 * rij with rij = rj - ri), in the
// reference's PairForceParams::elemForce shape (MD.cuh:98-113). Laws:
//  LJ-WCA: the reference LJ (MD.cuh:50-56), eps_ij = 24 sqrt(eps_i eps_j) (MD.cu:13),
//          rc^2 = 2^(1/3) sigma_ij^2 (Input.cpp:296-301), inclusive cutoff.
//  soft-core: F = eps (1 - r/rc)^2, rc = rcut_scale * sigma_ij.
//  Hertz: F = E delta^1.5, delta = sigma_ij - r.
// The reference soft-core cubic well (SCParams, MD.cuh:134-232), one species: the pair
// coefficients of SCParams::init (MD.cu:57-77) reduce to eps_core, eps_well, xi and rcut2 for a
// single element type. elemForce0 (MD.cuh:144-162) with t'(y, xi) = 6 y (-y + xi) / xi^3
// (MD.cuh:135-137), in the reference's operation order.
double sc_force0(double r2, double sig_core, double e0, double em, double xi) {
  const double r = std::sqrt(r2);
  const double y = r - sig_core;
  if (y <= -xi) return 0.0;
  if (-xi <= y && y < 0.0) {
    const double yy = -y;
    return -(e0 + em) * (6.0 * yy * (-yy + xi) / (xi * xi * xi)) / r;
  }
  if (0 <= y && y < xi) return em * (6.0 * y * (-y + xi) / (xi * xi * xi)) / r;
  return 0.0;
}

// LJParams::elemForce0 (MD.cuh:50-56): (s^6 - 2 s^12) / r2 with s^2 = sij2 / r2
static double lj_force0(double sij2, double r2) {
  const double ir2 = 1.0 / r2;
  double sr2n = sij2 * ir2;
  const double srn = sr2n * sr2n * sr2n;
  sr2n = srn * srn;
  return (srn - 2.0 * sr2n) * ir2;
}

bool pair_force_law(int law, double eps, double rcut_scale, double r2, double si, double sj, double &f0,
                    double well_eps, double well_sigma, int shifted) {
  const double sij = 0.5 * (si + sj);
  f0 = 0.0;
  if (law == ORA_FORCE_SC) {
    // SCParams::elemForce (MD.cuh:199-214): the force acts for rcut2 (sigCore - xi)^2 < r2 <=
    // rcut2 (sigCore + xi)^2, minus its value at the cutoff with OPT::FORCE_SHIFTED
    const double rcut2 = rcut_scale * rcut_scale;
    const double rc2 = rcut2 * ((sij + well_sigma) * (sij + well_sigma));
    if (r2 > rcut2 * ((sij - well_sigma) * (sij - well_sigma)) && r2 <= rc2) {
      f0 = sc_force0(r2, sij, eps, well_eps, well_sigma) -
           (shifted ? sc_force0(rc2, sij, eps, well_eps, well_sigma) * std::sqrt(rc2 / r2) : 0.0);
      return true;
    }
    return false;
  }
  if (law == ORA_FORCE_LJ_WCA) {
    // LJParams::elemForce (MD.cuh:72-92): eps_ij = 24 eps (one species), rc2 = sij2 rcut2,
    // minus the modulus at the cutoff times sqrt(rc2 / r2) with OPT::FORCE_SHIFTED
    const double sij2 = sij * sij;
    const double rc2 = sij2 * (rcut_scale * rcut_scale);
    if (r2 <= rc2) {
      f0 = (lj_force0(sij2, r2) - (shifted ? lj_force0(sij2, rc2) * std::sqrt(rc2 / r2) : 0.0)) * (24.0 * eps);
      return true;
    }
    return false;
  }
  const double rc = rcut_scale * sij;
  if (r2 < rc * rc && r2 > 0.0) {
    const double r = std::sqrt(r2);
    if (law == ORA_FORCE_SOFTCORE) {
      const double w = 1.0 - r / rc;
      f0 = -eps * w * w / r;
    } else {
      const double delta = sij - r;
      f0 = -eps * delta * std::sqrt(delta) / r;
    }
    return true;
  }
  return false;
}

// Half stencils including the own bin (Utils.hpp:700-704, DNS2D / DNS3D)
const int kDns2d[5][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {-1, 1, 0}};
const int kDns3d[14][3] = {{0, 0, 0},  {1, 0, 0},  {1, 1, 0},   {0, 1, 0},  {-1, 1, 0},
                           {0, 0, 1},  {1, 0, 1},  {1, 1, 1},   {0, 1, 1},  {-1, 1, 1},
                           {-1, 0, 1}, {-1, -1, 1}, {0, -1, 1}, {1, -1, 1}};

// CellState (Cell.cuh:26-30)
constexpr int kDividing = 0, kCrawling = 1, kUndefined = 2;

struct Oracle {
  ora_params p{};
  int D = 2;
  int cap = 0, n = 0, ts = 0;
  int nthreads = 0;
  int integrator = 0;  // 0 Euler, 1 Heun
  double fene_r2max = 0.0, fene_rss = 0.0;  // intra_law 1: RMAX^2, steady-state length
  double fene_r2max_div = 0.0;                // intra_law 1: RMAX_DIVISION^2 (RMAX^2 without it)
  std::vector<int> cst;                       // CellState per cell (Cell.cuh:26-30)
  std::vector<double> awr, awt;               // the bond's active noise per cell (radial, angular)
  std::vector<double> pos, vel, frc, sig, wiener;
  std::vector<int> t0, tsw;
  Rng rng;
  std::vector<ora_event> events;
  int64_t ndiv_total = 0, napo_total = 0;
  // observables (per cell, moved with the cell on removal, inherited on division)
  std::vector<double> com_prev, disp, vref;
  bool obs_ready = false;
  // scratch
  std::vector<double> com;
  std::vector<int> head, list;
  LinkGrid grid;

  double *P(int c, int j) { return &pos[(static_cast<size_t>(c) * 2 + j) * D]; }
  double *F(int c, int j) { return &frc[(static_cast<size_t>(c) * 2 + j) * D]; }
  double *V(int c, int j) { return &vel[(static_cast<size_t>(c) * 2 + j) * D]; }

  // BoundingBox::distance, Utils.hpp:536-544: r12 = r2 - r1 with the minimum image
  double distance(double *r12, const double *r1, const double *r2) const {
    return box_distance(D, p.box, p.periodic, r12, r1, r2);
  }
  // BoundingBox::updatePos(r, v, dt), Utils.hpp:561-566
  void update_pos(double *r, const double *v, double dt) const { box_update_pos(D, p.box, p.periodic, r, v, dt); }
  // BoundingBox::updatePos(r, dr), Utils.hpp:556-559
  void update_pos(double *r, const double *dr) const { box_update_pos(D, p.box, p.periodic, r, dr); }

  bool elem_force(double r2, double si, double sj, double &f0) const {
    return pair_force_law(p.force_law, p.epsilon, p.rcut_scale, r2, si, sj, f0, p.well_epsilon, p.well_sigma,
                          p.force_shifted);
  }

  // Rest length of the intra-cell spring at step ts (linear growth over the cell cycle).
  double rest_length(int c) const {
    if (!p.divide) return p.rest0;
    const int span = tsw[c] - t0[c];
    double frac = span > 0 ? static_cast<double>(ts - t0[c]) / static_cast<double>(span) : 1.0;
    frac = std::min(1.0, std::max(0.0, frac));
    return p.rest0 + (p.rest1 - p.rest0) * frac;
  }

  // the bond's active noise term (MD.cu:573-579, 2D): rnd = (Wr r_x / r - Wt r_y,
  // Wr r_y / r + Wt r_x) / 2, added as rnd_d r_ij,d
  void active_noise(int c, const double *rij, double r, double *rnd) const {
    if (D != 2 || awr.empty()) return;
    const double wr = awr[c], wt = awt[c];
    rnd[0] = 0.5 * (wr * rij[0] / r - wt * rij[1]);
    rnd[1] = 0.5 * (wr * rij[1] / r + wt * rij[0]);
  }

  // binaryCellForce (MD.cu:525-598) with the linear bond: spring kappa (r - l)
  // along the back->front axis, motility -m0 n on the back element and +m1 n on the front.
  // The reference's velocity-dependent friction term and FENE are not part of this model.
  // Assigns the force (the reference's migrationFunc assigns, MD.cu:595-596).
  void intra_force(int c) {
    double rij[3] = {0, 0, 0};
    const double r2 = distance(rij, P(c, 0), P(c, 1));  // rij = r1 - r0
    double *f0 = F(c, 0), *f1 = F(c, 1);
    if (r2 == 0.0) {
      for (int d = 0; d < D; ++d) f0[d] = f1[d] = 0.0;
      return;
    }
    const double r = std::sqrt(r2);
    if (p.intra_law == 1) {
      // binaryCellForce (MD.cu:525-598) for a crawling cell: r2max = max(RMAX^2, the larger
      // diameter) (MD.cu:547-548); push spring below spring_ratio r2max (MD.cu:263-265, 553-554),
      // FENE above it (MD.cu:255-257, 553-558); motility along nij = rij, or rij rss / r
      // without CIL (MD.cu:568-571); the bond acts twice (strongContract = 2). The reference's
      // velocity-squared friction (MD.cu:592-596) is left out: its two-element integrator
      // (StochasticHeun) never updates the velocities, which stay 0, and the NaN guard drops it.
      const bool dividing = cst[c] == kDividing;
      const double smax = std::max(sig[2 * c], sig[2 * c + 1]);
      const double r2max0 = dividing ? fene_r2max_div : fene_r2max;
      const double r2max = r2max0 > smax ? r2max0 : smax;
      const double lim = r2max * p.fene_spring_ratio;
      double spring;
      if (r2 <= lim) {
        spring = p.fene_kappa_push * std::fabs(r2 - lim);
      } else {
        const double q = (r2 - lim) / (r2max * (1.0 - p.fene_spring_ratio));
        spring = -p.fene_kappa / (1.0 - q * q);
      }
      if (dividing) {
        // MD.cu:559-567: the growth activity along rij against the FENE force at the division
        // length (feneDivMax, with divisionR2min = Rmin^2), the bond acting once
        const double qd = p.div_rmin * p.div_rmin / r2max;
        const double fdm = -p.fene_kappa / (1.0 - qd * qd);
        double act[2];
        for (int j = 0; j < 2; ++j) act[j] = -p.growth_k0[j] * fdm + p.growth_k1[j] + p.growth_k2[j] * (r2 * r2);
        double rnd[3] = {0, 0, 0};
        active_noise(c, rij, r, rnd);
        for (int d = 0; d < D; ++d) {
          f0[d] = -(act[0] * rij[d] + spring * rij[d] * 1.0 + rnd[d] * rij[d]);
          f1[d] = act[1] * rij[d] + spring * rij[d] * 1.0 + rnd[d] * rij[d];
        }
        return;
      }
      const double scaling = p.cil ? 1.0 : fene_rss / r;
      double rnd[3] = {0, 0, 0};
      active_noise(c, rij, r, rnd);
      for (int d = 0; d < D; ++d) {
        const double nd = p.cil ? rij[d] : rij[d] * scaling;
        f0[d] = -(p.motility[0] * nd + spring * rij[d] * 2.0 + rnd[d] * rij[d]);
        f1[d] = p.motility[1] * nd + spring * rij[d] * 2.0 + rnd[d] * rij[d];
      }
      return;
    }
    const double s = p.kappa * (r - rest_length(c));
    for (int d = 0; d < D; ++d) {
      const double nd = rij[d] / r;
      f0[d] = s * nd - p.motility[0] * nd;
      f1[d] = -s * nd + p.motility[1] * nd;
    }
  }

  // One-sided flat Hertz walls normal to the last axis (the channel workload; the reference's
  // FlatWall::addHZForce, Wall.hpp:80-91, is the unused precursor). Overlap
  // delta = sigma/2 - dir*(x - x0); force +dir * E delta^1.5.
  void wall_force(int c, int j) {
    const int ax = D - 1;
    const double x = P(c, j)[ax];
    const double rad = 0.5 * sig[static_cast<size_t>(c) * 2 + j];
    for (int w = 0; w < p.nwalls; ++w) {
      const double dir = static_cast<double>(p.wall_dir[w]);
      const double delta = rad - dir * (x - p.wall_pos[w]);
      if (delta > 0.0) F(c, j)[ax] += dir * p.wall_E * delta * std::sqrt(delta);
    }
  }

  // updateWienerProcess, CIL.cu:793-818: amplitude sqrt(2 D) (Input.cpp:112) / sqrt(dt)
  // (CIL.cuh:211-215); drawn for every entry in storage order only when D > 0.
  void draw_noise() {
    if (p.noise_D > 0.0) {
      const double amp = std::sqrt(2.0 * p.noise_D) * (1.0 / std::sqrt(p.dt));
      const size_t m = static_cast<size_t>(n) * (p.noise_per_cell ? 1 : 2) * D;
      wiener.resize(std::max(wiener.size(), m));
      for (size_t i = 0; i < m; ++i) wiener[i] = amp * rng.normal();
    }
    // the bond's active noise after the passive one (CIL.cu:803-815): radial for every cell,
    // then angular; a component whose amplitude is zero is never drawn and stays 0
    if (p.intra_law == 1 && D == 2) {
      awr.assign(static_cast<size_t>(cap), 0.0);
      awt.assign(static_cast<size_t>(cap), 0.0);
      if (p.noise_radial > 0.0) {
        const double amp = std::sqrt(2.0 * p.noise_radial) * (1.0 / std::sqrt(p.dt));
        for (int i = 0; i < n; ++i) awr[i] = amp * rng.normal();
      }
      if (p.noise_angular > 0.0) {
        const double amp = std::sqrt(2.0 * p.noise_angular) * (1.0 / std::sqrt(p.dt));
        for (int i = 0; i < n; ++i) awt[i] = amp * rng.normal();
      }
    }
  }
  void add_noise(int c, int j) {
    if (!(p.noise_D > 0.0)) return;
    const double *w = p.noise_per_cell ? &wiener[static_cast<size_t>(c) * D]
                                       : &wiener[(static_cast<size_t>(c) * 2 + j) * D];
    for (int d = 0; d < D; ++d) F(c, j)[d] += p.zeta[j] * w[d];
  }

  // calculComs, Colony.cpp:409-432
  void calc_coms() {
    com.resize(static_cast<size_t>(n) * D);
    for (int c = 0; c < n; ++c) {
      double acc[3] = {0, 0, 0}, rij[3];
      for (int j = 0; j < 2; ++j) {
        distance(rij, P(c, 0), P(c, j));
        for (int d = 0; d < D; ++d) acc[d] += rij[d];
      }
      for (int d = 0; d < D; ++d) acc[d] /= 2.0;
      update_pos(acc, P(c, 0));
      for (int d = 0; d < D; ++d) com[static_cast<size_t>(c) * D + d] = acc[d];
    }
  }

  // cellCellForce, MD.cu:757-790 (single species: no cross-adhesion branch)
  void cell_cell(int ci, int cj, bool both) {
    double rij[3];
    for (int a = 0; a < 2; ++a) {
      const double sa = sig[static_cast<size_t>(ci) * 2 + a];
      for (int b = 0; b < 2; ++b) {
        const double sb = sig[static_cast<size_t>(cj) * 2 + b];
        double f0;
        if (elem_force(distance(rij, P(ci, a), P(cj, b)), sa, sb, f0)) {
          for (int d = 0; d < D; ++d) {
            F(ci, a)[d] += f0 * rij[d];
            if (both) F(cj, b)[d] -= f0 * rij[d];
          }
        }
      }
    }
  }

  // Cell link list over cell centres of mass (CellLinkList::populate, Container.cpp:81-103).
  // The reference sizes the grid once from nominal parameters (CIL.cuh:88-136); the
  // restatement sizes it every step from the actual largest cutoff and cell extent so that
  // no interacting pair can be missed.
  void build_cell_grid() {
    double smax = 0.0, ext = 0.0, rij[3];
    for (int c = 0; c < n; ++c) {
      smax = std::max(smax, std::max(sig[static_cast<size_t>(c) * 2], sig[static_cast<size_t>(c) * 2 + 1]));
      ext = std::max(ext, std::sqrt(distance(rij, P(c, 0), P(c, 1))));
    }
    const double reach = p.force_law == ORA_FORCE_SC ? smax + p.well_sigma : smax;  // the well reaches xi further
    const double width = p.rcut_scale * reach + ext;
    grid.init(D, width, p.box, p.periodic);
    calc_coms();
    grid.populate(com.data(), n, head, list);
  }

  // calculInterForces LINKLIST_ON branch, CIL.cu:177-231 (half stencil, LIFO lists,
  // Newton's third law); the all-pairs branch CIL.cu:232-262 when the grid collapses.
  void inter_forces_reference() {
    build_cell_grid();
    if (grid.ncells == 1) {
      for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) cell_cell(i, j, true);
      return;
    }
    const int nn = D == 2 ? 5 : 14;
    for (int ic = 0; ic < grid.ncells; ++ic) {
      int icell[3] = {0, 0, 0};
      grid.coord(ic, icell);
      for (int dc = 0; dc < nn; ++dc) {
        const int jc = grid.neighbor(icell, D == 2 ? kDns2d[dc] : kDns3d[dc]);
        if (jc == -1) continue;
        for (int ii = head[ic]; ii >= 0; ii = list[ii]) {
          for (int jj = head[jc]; jj >= 0; jj = list[jj]) {
            if ((ic != jc || jj > ii) && ii != jj) cell_cell(ii, jj, true);
          }
        }
      }
    }
  }

  // Race-free variant for timing on many threads: full 3^d stencil, each thread writes
  // only its own cell's forces (the reference's OpenMP loop races on fj, CIL.cu:183-230).
  void inter_forces_parallel() {
    build_cell_grid();
    if (grid.ncells == 1) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          if (j != i) cell_cell(i, j, false);
      return;
    }
    std::vector<int> bin_of_cell(n);
    for (int ic = 0; ic < grid.ncells; ++ic)
      for (int ii = head[ic]; ii >= 0; ii = list[ii]) bin_of_cell[ii] = ic;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int i = 0; i < n; ++i) {
      int icell[3] = {0, 0, 0};
      grid.coord(bin_of_cell[i], icell);
      int dc[3] = {0, 0, 0};
      const int zr = D == 3 ? 1 : 0;
      for (dc[0] = -1; dc[0] <= 1; ++dc[0])
        for (dc[1] = -1; dc[1] <= 1; ++dc[1])
          for (dc[2] = -zr; dc[2] <= zr; ++dc[2]) {
            const int jc = grid.neighbor(icell, dc);
            if (jc == -1) continue;
            for (int jj = head[jc]; jj >= 0; jj = list[jj])
              if (jj != i) cell_cell(i, jj, false);
          }
    }
  }

  // calculForcesPressure, CIL.cu:999-1007
  void compute_forces() {
    draw_noise();
    for (int c = 0; c < n; ++c) {
      intra_force(c);
      for (int j = 0; j < 2; ++j) wall_force(c, j);
      for (int j = 0; j < 2; ++j) add_noise(c, j);
    }
    if (nthreads > 0)
      inter_forces_parallel();
    else
      inter_forces_reference();
  }

  // updatePositions (CIL.cu:858-875) with mobility 1/zeta; velocity v = F * (temp/dt) as
  // updateVelocityPositions does (CIL.cu:923-935).
  // heun: 0 a full Euler step; 1, 2 the first and second half step of a Heun step
  // (temp = (dt/2) / zeta, CIL.cu:1037-1042; velocity: F/zeta, then the mean of both halves).
  void integrate(int heun = 0) {
    for (int c = 0; c < n; ++c)
      for (int j = 0; j < 2; ++j) {
        const double temp = p.dt * (1.0 / p.zeta[j]);
        update_pos(P(c, j), F(c, j), heun ? 0.5 * temp : temp);
        const double mu = temp / p.dt;
        for (int d = 0; d < D; ++d) {
          const double v = F(c, j)[d] * mu;
          V(c, j)[d] = heun == 2 ? 0.5 * (V(c, j)[d] + v) : v;
        }
      }
  }

  // randomTimeSpan, MD.cuh:434-436
  int time_span() {
    const int s = nint(rng.normal(p.div_tau_mu, p.div_tau_sigma) / p.dt);
    return s >= 1 ? s : 1;
  }

  // binaryRandomReorientation, MD.cu:650-656
  void reorient(double *slave, double *master, double radius) {
    for (int d = 0; d < D; ++d) slave[d] = master[d];
    double dr[3] = {0, 0, 0};
    rng.on_dsphere(D, dr);
    update_pos(master, dr, radius);
    update_pos(slave, dr, -radius);
  }

  void copy_cell(int dst, int src) {
    for (int j = 0; j < 2; ++j) {
      std::memcpy(P(dst, j), P(src, j), sizeof(double) * D);
      std::memcpy(V(dst, j), V(src, j), sizeof(double) * D);
      std::memcpy(F(dst, j), F(src, j), sizeof(double) * D);
      sig[static_cast<size_t>(dst) * 2 + j] = sig[static_cast<size_t>(src) * 2 + j];
    }
    t0[dst] = t0[src];
    tsw[dst] = tsw[src];
    cst[dst] = cst[src];
    for (int d = 0; d < D; ++d) {
      com_prev[static_cast<size_t>(dst) * D + d] = com_prev[static_cast<size_t>(src) * D + d];
      disp[static_cast<size_t>(dst) * D + d] = disp[static_cast<size_t>(src) * D + d];
      vref[static_cast<size_t>(dst) * D + d] = vref[static_cast<size_t>(src) * D + d];
    }
  }

  // calculDivisions (CIL.cu:369-455) for the linear-growth model: a cell divides when its
  // cycle ends (ts == tswitch); binaryCellDivision (MD.cu:721-731) places both daughters
  // with half-separation rest0/2; random draws in the reference order: mother axis,
  // daughter axis, daughter cycle, mother cycle.
  // randomTimeSpan (MD.cuh:434-436) of the migration time
  int mig_span() {
    const int s = nint(rng.normal(p.mig_tau_mu, p.mig_tau_sigma) / p.dt);
    return s >= 1 ? s : 1;
  }

  void reset_motion(int c) {
    for (int j = 0; j < 2; ++j)
      for (int d = 0; d < D; ++d) V(c, j)[d] = F(c, j)[d] = 0.0;
  }

  // calculDivisions (CIL.cu:369-455) for the reference's two-element cells with the FENE bond:
  // a crawling cell whose time ends starts dividing (time += span(TAU_DIVISION)); a dividing
  // cell whose elements are Rmin apart (binaryCellDivisionCriteria, MD.cuh:426-433) divides
  // (binaryCellDivision with radius R0, MD.cu:721-731; both cells crawl, their times from
  // TAU_MIGRATION, the mother's added to her own), and one whose time ends without that fails
  // (binaryCellDivisionFail, MD.cu:736-752). Diameters return to SIGMA_CORE.
  int state_divisions() {
    const int n0 = n;
    int err = 0;
    for (int i = 0; i < n0; ++i) {
      if (cst[i] == kDividing) {
        double rij[3] = {0, 0, 0};
        const double r2 = distance(rij, P(i, 1), P(i, 0));
        const bool ok = p.div_rmin_ratio != 0.0 ? r2 >= p.div_rmin_ratio * sig[2 * static_cast<size_t>(i)]
                                                : r2 >= p.div_rmin * p.div_rmin;
        if (ok) {
          if (n >= cap) {
            err = -2;
            continue;
          }
          const int k = n++;
          copy_cell(k, i);
          for (int d = 0; d < D; ++d) P(k, 0)[d] = P(i, 0)[d];
          reorient(P(i, 0), P(i, 1), p.div_r0);
          reorient(P(k, 1), P(k, 0), p.div_r0);
          t0[k] = ts;
          t0[i] = ts;
          tsw[k] = ts + mig_span();
          cst[k] = kCrawling;
          sig[2 * static_cast<size_t>(k)] = p.sigma_core[0];
          sig[2 * static_cast<size_t>(k) + 1] = p.sigma_core[1];
          reset_motion(k);
          reset_motion(i);
          tsw[i] += mig_span();
          cst[i] = kCrawling;
          sig[2 * static_cast<size_t>(i)] = p.sigma_core[0];
          sig[2 * static_cast<size_t>(i) + 1] = p.sigma_core[1];
          events.push_back({ts, 0, i, k});
          ++ndiv_total;
        } else if (tsw[i] == ts) {
          // back element to the centre (a plain add, MD.cu:744-746), then both reoriented
          double dr[3] = {0, 0, 0};
          distance(dr, P(i, 0), P(i, 1));
          for (int d = 0; d < D; ++d) P(i, 0)[d] += dr[d] * 0.5;
          reorient(P(i, 1), P(i, 0), p.div_r0);
          reset_motion(i);
          tsw[i] += mig_span();
          cst[i] = kCrawling;
          sig[2 * static_cast<size_t>(i)] = p.sigma_core[0];
          sig[2 * static_cast<size_t>(i) + 1] = p.sigma_core[1];
          events.push_back({ts, 2, i, i});
        }
      } else if (tsw[i] == ts) {
        cst[i] = kDividing;
        tsw[i] += time_span();
        reset_motion(i);
        events.push_back({ts, 3, i, i});
      }
    }
    return err;
  }

  int divisions() {
    if (!p.divide) return 0;
    if (p.intra_law == 1) return state_divisions();
    const int n0 = n;
    const double radius = 0.5 * p.rest0;
    int err = 0;
    for (int i = 0; i < n0; ++i) {
      if (tsw[i] != ts) continue;
      if (n >= cap) {
        err = -2;
        continue;
      }
      const int k = n++;
      copy_cell(k, i);
      for (int d = 0; d < D; ++d) P(k, 0)[d] = P(i, 0)[d];
      reorient(P(i, 0), P(i, 1), radius);
      reorient(P(k, 1), P(k, 0), radius);
      t0[k] = ts;
      t0[i] = ts;
      cst[k] = kCrawling;  // both cells crawl after a division (CIL.cu:403, 425)
      cst[i] = kCrawling;
      tsw[k] = ts + time_span();
      for (int j = 0; j < 2; ++j)
        for (int d = 0; d < D; ++d) V(k, j)[d] = V(i, j)[d] = F(k, j)[d] = F(i, j)[d] = 0.0;
      tsw[i] = ts + time_span();
      events.push_back({ts, 0, i, k});
      ++ndiv_total;
    }
    return err;
  }

  // updateDiameters (CIL.cu:970-991): with SWELLING a dividing cell's diameters below the larger
  // SIGMA_CORE grow by (max - sigma) / (tswitch - ts) each step
  void swell() {
    if (!(p.divide && p.intra_law == 1 && p.div_swelling)) return;
    const double smax = std::max(p.sigma_core[0], p.sigma_core[1]);
    for (int i = 0; i < n; ++i) {
      if (cst[i] != kDividing) continue;
      for (int j = 0; j < 2; ++j) {
        double &s = sig[2 * static_cast<size_t>(i) + j];
        if (s < smax) s += (smax - s) / (tsw[i] - ts);
      }
    }
  }

  // calculApoptosis, CIL.cu:627-649: sequential test of every slot, swap-with-last removal
  // (removeCell, Colony.cpp:365-399) and a re-test of the same slot.
  void apoptosis() {
    if (!(p.apop_rate > 0.0)) return;
    const double prob = p.apop_rate * p.dt;  // CIL.cuh:233
    int i = 0;
    while (i < n) {
      if (rng.uniform0x(1.0) <= prob) {
        const int last = n - 1;
        if (i != last) copy_cell(i, last);
        --n;
        events.push_back({ts, 1, i, last});
        ++napo_total;
      } else {
        ++i;
      }
    }
  }

  int step() {
    if (integrator == 1) {
      compute_forces();
      integrate(1);
      compute_forces();
      integrate(2);
    } else {
      compute_forces();
      integrate();
    }
    ++ts;
    const int err = divisions();
    apoptosis();
    swell();
    // checkPositions (CIL.cu:945-966): every coordinate inside the box
    for (int c = 0; c < n; ++c)
      for (int j = 0; j < 2; ++j)
        for (int d = 0; d < D; ++d) {
          const double x = P(c, j)[d];
          if (!(x >= 0.0 && x < p.box[d])) return -3;
        }
    return err;
  }

  void cell_velocity(int c, double *v) {
    for (int d = 0; d < D; ++d) v[d] = 0.5 * (V(c, 0)[d] + V(c, 1)[d]);
  }
};

inline Oracle *H(void *h) { return static_cast<Oracle *>(h); }
inline const Oracle *H(const void *h) { return static_cast<const Oracle *>(h); }

}  // namespace

extern "C" {

void *ora_create(const ora_params *p, int32_t cap_cells, uint32_t seed) {
  if (!p || cap_cells <= 0 || (p->dim != 2 && p->dim != 3)) return nullptr;
  auto *o = new Oracle();
  o->p = *p;
  o->D = p->dim;
  o->cap = cap_cells;
  const size_t ne = static_cast<size_t>(cap_cells) * 2;
  o->pos.assign(ne * o->D, 0.0);
  o->vel.assign(ne * o->D, 0.0);
  o->frc.assign(ne * o->D, 0.0);
  o->sig.assign(ne, 0.0);
  o->t0.assign(cap_cells, 0);
  o->tsw.assign(cap_cells, 0);
  o->com_prev.assign(static_cast<size_t>(cap_cells) * o->D, 0.0);
  o->disp.assign(static_cast<size_t>(cap_cells) * o->D, 0.0);
  o->vref.assign(static_cast<size_t>(cap_cells) * o->D, 0.0);
  o->rng.init(seed);  // Random::init, Random.hpp:12-14
  if (p->intra_law == 1) {
    // params.r2max and the steady-state length rss of Input.cpp:123-144
    o->fene_r2max = p->fene_rmax * p->fene_rmax;
    const double zi0 = 1.0 / p->zeta[0], zi1 = 1.0 / p->zeta[1];
    const double alpha = zi0 + zi1, beta = p->motility[0] * zi0 + p->motility[1] * zi1;
    o->fene_rss = std::sqrt(o->fene_r2max * (1.0 - alpha / beta * p->fene_kappa));
    o->fene_r2max_div = p->fene_rmax_division > 0.0 ? p->fene_rmax_division * p->fene_rmax_division : o->fene_r2max;
  }
  o->cst.assign(cap_cells, kUndefined);
  return o;
}

void ora_destroy(void *h) { delete H(h); }

void ora_set_threads(void *h, int32_t nthreads) { H(h)->nthreads = nthreads < 0 ? 0 : nthreads; }

void ora_set_integrator(void *h, int32_t integrator) { H(h)->integrator = integrator == 1 ? 1 : 0; }

int32_t ora_set_state(void *h, int32_t ncells, const double *pos, const double *sigma,
                      const int32_t *t0, const int32_t *tswitch, int32_t ts) {
  Oracle *o = H(h);
  if (ncells < 0 || ncells > o->cap) return -2;
  o->n = ncells;
  o->ts = ts;
  const size_t ne = static_cast<size_t>(ncells) * 2;
  std::memcpy(o->pos.data(), pos, sizeof(double) * ne * o->D);
  std::memcpy(o->sig.data(), sigma, sizeof(double) * ne);
  std::memcpy(o->t0.data(), t0, sizeof(int32_t) * ncells);
  std::memcpy(o->tsw.data(), tswitch, sizeof(int32_t) * ncells);
  std::fill(o->vel.begin(), o->vel.end(), 0.0);
  std::fill(o->frc.begin(), o->frc.end(), 0.0);
  std::fill(o->cst.begin(), o->cst.end(), kUndefined);
  o->obs_ready = false;
  return 0;
}

void ora_set_cell_states(void *h, int32_t n, const int32_t *states) {
  Oracle *o = H(h);
  for (int i = 0; i < n && i < o->cap; ++i) o->cst[i] = states[i];
}

void ora_get_cell_states(const void *h, int32_t *states) {
  const Oracle *o = H(h);
  for (int i = 0; i < o->n; ++i) states[i] = o->cst[i];
}

int32_t ora_num_cells(const void *h) { return H(h)->n; }
int32_t ora_timestep(const void *h) { return H(h)->ts; }

void ora_get_state(const void *h, double *pos, double *sigma, double *vel, double *frc,
                   int32_t *t0, int32_t *tswitch) {
  const Oracle *o = H(h);
  const size_t ne = static_cast<size_t>(o->n) * 2;
  if (pos) std::memcpy(pos, o->pos.data(), sizeof(double) * ne * o->D);
  if (sigma) std::memcpy(sigma, o->sig.data(), sizeof(double) * ne);
  if (vel) std::memcpy(vel, o->vel.data(), sizeof(double) * ne * o->D);
  if (frc) std::memcpy(frc, o->frc.data(), sizeof(double) * ne * o->D);
  if (t0) std::memcpy(t0, o->t0.data(), sizeof(int32_t) * o->n);
  if (tswitch) std::memcpy(tswitch, o->tsw.data(), sizeof(int32_t) * o->n);
}

// The forces of the current state with the noise the next step will draw; the random stream
// is put back, as cil_forces does, so that reading them leaves the run unchanged.
void ora_compute_forces(void *h) {
  const Rng saved = H(h)->rng;
  H(h)->compute_forces();
  H(h)->rng = saved;
}

int32_t ora_step(void *h, int32_t nsteps) {
  Oracle *o = H(h);
  int32_t err = 0;
  for (int s = 0; s < nsteps; ++s) {
    const int e = o->step();
    if (e < 0 && err == 0) err = e;
  }
  return err;
}

int32_t ora_bin_elements(const void *h, double width, int32_t *ns, int32_t *head, int32_t *list,
                         int32_t max_bins) {
  const Oracle *o = H(h);
  LinkGrid g;
  g.init(o->D, width, o->p.box, o->p.periodic);
  for (int d = 0; d < 3; ++d) ns[d] = g.ns[d];
  if (g.ncells > max_bins) return -g.ncells;
  std::vector<int> hd, ls;
  g.populate(o->pos.data(), o->n * 2, hd, ls);
  std::memcpy(head, hd.data(), sizeof(int32_t) * g.ncells);
  std::memcpy(list, ls.data(), sizeof(int32_t) * ls.size());
  return g.ncells;
}

int32_t ora_num_events(const void *h) { return static_cast<int32_t>(H(h)->events.size()); }
void ora_get_events(const void *h, ora_event *out) {
  const auto &e = H(h)->events;
  if (!e.empty()) std::memcpy(out, e.data(), sizeof(ora_event) * e.size());
}
void ora_clear_events(void *h) { H(h)->events.clear(); }

// Observable definitions: cell count; mean cell area sum_j pi (sigma_j/2)^2
// (cilJintaoTools.py:112-115); MSD of the unwrapped cell centre of mass since the last
// reset, accumulated by minimum-image displacement between calls
// (simulationtools.py:602-607); VACF <v_c(t).v_c(0)>/<|v_c(0)|^2> of the cell velocity.
// Daughters inherit the mother's track.
void ora_obs_reset(void *h) {
  Oracle *o = H(h);
  o->calc_coms();
  for (int c = 0; c < o->n; ++c) {
    double v[3];
    o->cell_velocity(c, v);
    for (int d = 0; d < o->D; ++d) {
      o->com_prev[static_cast<size_t>(c) * o->D + d] = o->com[static_cast<size_t>(c) * o->D + d];
      o->disp[static_cast<size_t>(c) * o->D + d] = 0.0;
      o->vref[static_cast<size_t>(c) * o->D + d] = v[d];
    }
  }
  o->obs_ready = true;
}

void ora_observables(void *h, ora_obs *out) {
  Oracle *o = H(h);
  if (!o->obs_ready) ora_obs_reset(h);
  o->calc_coms();
  const int D = o->D;
  double area = 0.0, msd = 0.0, vv = 0.0, v0 = 0.0;
  for (int c = 0; c < o->n; ++c) {
    double dr[3];
    o->distance(dr, &o->com_prev[static_cast<size_t>(c) * D], &o->com[static_cast<size_t>(c) * D]);
    double v[3];
    o->cell_velocity(c, v);
    double m2 = 0.0;
    for (int d = 0; d < D; ++d) {
      double &acc = o->disp[static_cast<size_t>(c) * D + d];
      acc += dr[d];
      m2 += acc * acc;
      o->com_prev[static_cast<size_t>(c) * D + d] = o->com[static_cast<size_t>(c) * D + d];
      vv += v[d] * o->vref[static_cast<size_t>(c) * D + d];
      v0 += o->vref[static_cast<size_t>(c) * D + d] * o->vref[static_cast<size_t>(c) * D + d];
    }
    msd += m2;
    for (int j = 0; j < 2; ++j) {
      const double s = o->sig[static_cast<size_t>(c) * 2 + j];
      area += kPi * (s * 0.5) * (s * 0.5);
    }
  }
  out->ncells = o->n;
  out->pad = 0;
  out->mean_area = o->n ? area / o->n : 0.0;
  out->msd = o->n ? msd / o->n : 0.0;
  out->vacf = v0 > 0.0 ? vv / v0 : 0.0;
  out->ndiv_total = o->ndiv_total;
  out->napo_total = o->napo_total;
}

int32_t ora_geom_nint(double a) { return nint(a); }

void ora_geom_distance(int32_t dim, const double *box, const int32_t *periodic, int64_t n, const double *r1,
                       const double *r2, double *r12, double *d2) {
  for (int64_t i = 0; i < n; ++i)
    d2[i] = box_distance(dim, box, periodic, r12 + i * dim, r1 + i * dim, r2 + i * dim);
}

void ora_geom_update_pos(int32_t dim, const double *box, const int32_t *periodic, int64_t n, double *r,
                         const double *v, double dt) {
  for (int64_t i = 0; i < n; ++i) {
    if (dt == 0.0)
      box_update_pos(dim, box, periodic, r + i * dim, v + i * dim);
    else
      box_update_pos(dim, box, periodic, r + i * dim, v + i * dim, dt);
  }
}

int32_t ora_geom_link_list(int32_t dim, double rcut, const double *box, const int32_t *periodic, int32_t n,
                           const double *r, int32_t *ns, int32_t *head, int32_t *list, int32_t *coords,
                           int32_t *neighbor_ids, int32_t max_bins) {
  LinkGrid g;
  g.init(dim, rcut, box, periodic);
  for (int d = 0; d < 3; ++d) ns[d] = g.ns[d];
  if (g.ncells > max_bins) return -g.ncells;
  std::vector<int> hd, ls;
  g.populate(r, n, hd, ls);
  std::memcpy(head, hd.data(), sizeof(int32_t) * g.ncells);
  if (n > 0) std::memcpy(list, ls.data(), sizeof(int32_t) * n);
  const int nst = dim == 2 ? 5 : 14;
  for (int b = 0; b < g.ncells; ++b) {
    int c[3] = {0, 0, 0};
    g.coord(b, c);
    for (int d = 0; d < dim; ++d) coords[b * dim + d] = c[d];
    for (int k = 0; k < nst; ++k) neighbor_ids[b * nst + k] = g.neighbor(c, dim == 2 ? kDns2d[k] : kDns3d[k]);
  }
  return g.ncells;
}

void ora_geom_pair_force(int32_t law, double eps, double rcut_scale, int64_t n, const double *r2, const double *si,
                         const double *sj, double *f0, int32_t *inside) {
  for (int64_t k = 0; k < n; ++k)
    inside[k] = pair_force_law(law, eps, rcut_scale, r2[k], si[k], sj[k], f0[k], 0.0, 0.0, 0) ? 1 : 0;
}

void ora_geom_lj_force(double eps, double rcut_scale, int32_t shifted, int64_t n, const double *r2, const double *si,
                       const double *sj, double *f0, int32_t *inside) {
  for (int64_t k = 0; k < n; ++k)
    inside[k] =
        pair_force_law(ORA_FORCE_LJ_WCA, eps, rcut_scale, r2[k], si[k], sj[k], f0[k], 0.0, 0.0, shifted) ? 1 : 0;
}

void ora_geom_sc_force(double eps_core, double eps_well, double well_sigma, double rcut_scale, int32_t shifted,
                       int64_t n, const double *r2, const double *si, const double *sj, double *f0, int32_t *inside) {
  for (int64_t k = 0; k < n; ++k)
    inside[k] = pair_force_law(ORA_FORCE_SC, eps_core, rcut_scale, r2[k], si[k], sj[k], f0[k], eps_well, well_sigma,
                               shifted)
                    ? 1
                    : 0;
}

void ora_rng_seed(void *h, uint32_t seed) { H(h)->rng.init(seed); }
double ora_rng_close_open(void *h) { return H(h)->rng.g.close_open(); }
double ora_rng_open_open(void *h) { return H(h)->rng.g.open_open(); }
double ora_rng_uniform(void *h) { return H(h)->rng.uniform(); }
double ora_rng_normal(void *h) { return H(h)->rng.normal(); }
void ora_rng_on_dsphere(void *h, int32_t dim, double *out) { H(h)->rng.on_dsphere(dim, out); }

}  // extern "C"
