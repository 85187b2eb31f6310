// ORACLE — test infrastructure only. A CPU restatement of the reference's single-element
// cell-cycle model, the oracle the tests compare the GPU model (cil_cuda_gb300/csrc/cil_cycle.cu) with.
//
// Parity of this restatement with the reference is unpinned: the reference's host pair force
// with pressure (cellCellForcePressure, declared MD.cuh:397-399, called CIL.cu:165,220,259)
// has no body, and the rest of its code does not build (Cell.hpp, MD.hpp, CIL.hpp and Units.hpp
// are missing). Each step restates, in the reference's order:
//   motility along the velocity (singleCellForce, MD.cu:600-646), passive noise
//   (CIL.cu:84-97), Hertz contacts with adhesion and pressure (the device draft of
//   cellCellForcePressure, MD.cu:302-366; HZParams::elemForce0, MD.cuh:237-251; contact
//   length / area, Utils.hpp:236-250), the position update with pressure-dependent friction
//   (updateVelocityPositions, CIL.cu:902-939), ++ts, the cycle ODEs and divisions
//   (calculDivisionsSingle, CIL.cu:469-619; singleCellDivision, MD.cu:664-718), apoptosis
//   (calculApoptosisCyclePressure, CIL.cu:711-738; calculApoptosisPressureTime, CIL.cu:653-676;
//   calculApoptosis, CIL.cu:627-649; calculApoptosisCycle, CIL.cu:681-709;
//   calculApoptosisCycleExtrude, CIL.cu:749-788), and checkPositions with DRAIN (CIL.cu:945-966).
// The DPD step (CIL.cu:1054-1066): half kick and drift (updateVelocities / updatePositions,
//   CIL.cu:871-897, 849-866), the forces with the pair dissipative and random forces
//   (cellCellDisRanForce, MD.cu:861-905), the second half kick, the background and pair
//   dissipation (calculDisForces, CIL.cu:294-364), ++ts, divisions and apoptosis; every pair is
//   visited once and the forces are reset at every evaluation, which the reference's OpenMP
//   loops do not do (include/cil_cycle.h lists the differences).
// Random numbers: Philox4x32-10 (Salmon et al., SC'11) keyed by (cell, step, purpose, sub)
// exactly as the GPU model keys them, so that both draw the same numbers; the pair search
// visits bins and cells in the GPU model's order, so that the force sums agree to the last
// bits of libm. Build: oracle/build.sh (gcc -O2 -ffp-contract=off).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {

typedef struct cyo_params {  // the layout of cil_cycle_params (include/cil_cycle.h)
  int32_t dim;
  int32_t periodic[3];
  double box[3];
  double dt;
  double sigma_core, E, nu, adhesion, motility, zeta, zeta_p, zeta_p_beta, noise_D;
  int32_t divide;
  int32_t apoptosis;
  double tau_div_mu, tau_div_sigma, tau_mig_mu, tau_mig_sigma;
  double v1, cycle_tau_r, cycle_tau_v, cycle_tau_p, cycle_sigma_min, cycle_p0, cycle_beta_vs, cycle_rho_ratio,
      cycle_r_maxed, cycle_p_shift, cycle_p_shift_tau, osmotic_pressure;
  double apop_pressure, apop_duration, apop_rate, extr_gamma;
  int32_t drain;
  int32_t precision;  // read by the GPU model only: the restatement is FP64
  int32_t integrator;  // 0 Euler, 1 DPD
  int32_t flags;       // read by the GPU model only
  double mass, kbt, dis_same, dis_diff, dis_bg, extr_rate;
} cyo_params;

}  // extern "C"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr uint32_t kNoise = 11, kDir = 12, kDiv = 13, kApo = 14, kInit = 15, kDpd0 = 16, kDpd1 = 17;

struct Block {
  uint32_t v[4];
};

// Philox4x32-10: 10 rounds with the published multipliers and key increments
Block philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c0;
    const uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c2;
    const uint32_t n0 = static_cast<uint32_t>(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n2 = static_cast<uint32_t>(p0 >> 32) ^ c3 ^ k1;
    c1 = static_cast<uint32_t>(p1);
    c3 = static_cast<uint32_t>(p0);
    c0 = n0;
    c2 = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return Block{{c0, c1, c2, c3}};
}

double u53(uint32_t a, uint32_t b) {
  const uint64_t m = (static_cast<uint64_t>(a) << 21) ^ (static_cast<uint64_t>(b) >> 11);
  return static_cast<double>(m & ((1ull << 53) - 1)) * 1.1102230246251565e-16;
}

void normal2(const Block &r, double *n0, double *n1) {
  const double a = 1.0 - u53(r.v[0], r.v[1]);
  const double b = u53(r.v[2], r.v[3]);
  const double rad = std::sqrt(-2.0 * std::log(a));
  const double ang = 6.283185307179586 * b;
  *n0 = rad * std::cos(ang);
  *n1 = rad * std::sin(ang);
}

int nint(double a) { return a >= 0.0 ? static_cast<int>(a + 0.5) : static_cast<int>(a - 0.5); }
int span_steps(double x, double dt) {
  const int s = nint(x / dt);
  return s > 1 ? s : 1;
}
double lognormal(double mu, double s, double z) {
  const double mu2 = std::log((mu * mu) / (std::sqrt(mu * mu + s * s)));
  const double s2 = std::sqrt(std::log(1 + (s * s) / (mu * mu)));
  return std::exp(mu2 + s2 * z);
}
double area_of(double s) { return kPi * ((s / 2) * (s / 2)); }
double volume_of(double s) { return 4 * kPi * ((s / 2) * (s / 2) * (s / 2)) / 3; }
double sigma_of_area(double a) { return 2 * std::sqrt(a / kPi); }
double sigma_of_volume(double v) { return 2 * std::cbrt(3 * v / (4 * kPi)); }
double contact_length(double a, double b, double h) {
  const double ra = a / 2, rb = b / 2;
  const double q = ra - (2 * rb * h - h * h) / (2 * (ra + rb - h));
  const double t = 2 * std::sqrt(ra * ra - q * q);
  const double small_r = (a <= b) ? a : b;
  return std::isnan(t) ? small_r : t;
}
double contact_area(double r, double a, double b) {
  const double ra = a / 2, rb = b / 2;
  const double u = r * r - rb * rb + ra * ra;
  const double t = std::sqrt(4 * (r * r) * (ra * ra) - u * u) / (2 * r);
  return t > 0 ? kPi * (t * t) : 0.0;
}

struct Cell {
  double x[3], v[3];
  double sig, sigt, theta, rho, om, p;
  int tp, t0, tsw;
  double fc[3], fd[3], fr[3];  // DPD forces
};

struct Model {
  cyo_params p{};
  int D = 2;
  uint32_t k0 = 0, k1 = 0;
  int ns[3] = {1, 1, 1};
  double inv_bw[3] = {1, 1, 1};
  double tau_r = 0, tau_v = 0, tau_p = 0, v_s = 0, r_maxed_inv = 1, p_shift = 0, p_shift_tau_inv = 0;
  double noise_amp = 0, apop_rate_step = 0, apop_steps = 0;
  double smax = 0;
  int cap = 0;
  int ts = 0;
  int err = 0;  // 1 capacity, 2 non-finite, 4 out of box
  long long ndiv = 0, napo = 0;
  std::vector<Cell> c;

  Block draw(uint32_t cell, int t, uint32_t purpose, uint32_t sub) const {
    return philox(cell, static_cast<uint32_t>(t), purpose, sub, k0, k1);
  }

  void init(const cyo_params &q, int capacity, uint64_t seed) {
    p = q;
    D = q.dim;
    cap = capacity;
    k0 = static_cast<uint32_t>(seed);
    k1 = static_cast<uint32_t>(seed >> 32);
    rebin();
    tau_r = q.cycle_tau_r * q.tau_div_mu / q.dt;
    tau_v = q.cycle_tau_v * q.tau_div_mu / q.dt;
    tau_p = q.cycle_tau_p * q.tau_div_mu / q.dt;
    const double r = q.cycle_sigma_min / 2;
    v_s = D == 3 ? 4 * kPi * (r * r * r) / 3 : kPi * (r * r);
    r_maxed_inv = q.cycle_r_maxed > 0.0 ? 1.0 / q.cycle_r_maxed : 1.0;
    p_shift = q.cycle_p_shift * q.cycle_p0;
    p_shift_tau_inv = q.cycle_p_shift_tau > 0.0 ? 1.0 / (q.cycle_p_shift_tau * q.tau_div_mu) * q.dt : 0.0;
    noise_amp = q.noise_D > 0.0 ? std::sqrt(2.0 * q.noise_D) * (1.0 / std::sqrt(q.dt)) : 0.0;
    apop_rate_step = q.apop_rate * q.dt;
    apop_steps = q.apop_duration / q.dt;
    kick_div = 2 * (2 * q.mass);
    sqrt_dt = std::sqrt(q.dt);
    sigma_r = std::sqrt(2 * q.dis_diff * q.kbt);
  }

  // threads per cell of the GPU model's contact pass (2^lane_bits), whose candidate split and
  // combining tree conservative() follows; set per call by the GPU model's rule
  int lane_bits = 0;

  // the bin grid of a call: width >= 1.05 x max(SIGMA_CORE, the largest diameter), the GPU
  // model's rule
  void rebin() {
    {
      const long long n = static_cast<long long>(c.size()), capl = cap;
      int b = 0;
      while (b < 3 && n * (2LL << b) <= 2LL * 152 * 4 * 32 && (capl << (b + 1)) <= (1LL << 24)) ++b;
      lane_bits = b;
    }
    const double w = (smax > p.sigma_core ? smax : p.sigma_core) * 1.05;
    for (int d = 0; d < 3; ++d) {
      ns[d] = 1;
      inv_bw[d] = 1;
      if (d < D) {
        int n = static_cast<int>(p.box[d] / w);
        n = n < 1 ? 1 : (n > 4096 ? 4096 : n);
        ns[d] = n;
        inv_bw[d] = n / p.box[d];
      }
    }
  }

  int bin_coord(double x, int d) const {
    int v = static_cast<int>(x * inv_bw[d]);
    return v < 0 ? 0 : (v >= ns[d] ? ns[d] - 1 : v);
  }

  using Bins = std::vector<std::vector<int>>;

  // cells per bin in ascending index (the GPU model's counting sort order)
  Bins bin_cells() const {
    Bins bins(static_cast<size_t>(ns[0]) * ns[1] * ns[2]);
    for (int i = 0; i < static_cast<int>(c.size()); ++i) {
      int b = 0;
      for (int d = 0; d < D; ++d) b = b * ns[d] + bin_coord(c[i].x[d], d);
      bins[b].push_back(i);
    }
    return bins;
  }

  // every other cell in the bins within `radius` of cell i, in the GPU model's visiting order
  template <class Fn>
  void each_neighbour(int i, double radius, const Bins &bins, Fn fn, bool with_self = false) const {
    int bi[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
      bi[d] = bin_coord(c[i].x[d], d);
      const double kk = std::ceil(radius * inv_bw[d]);
      const int k = (kk >= 0.0 && kk < ns[d]) ? static_cast<int>(kk) : ns[d];
      if (2 * k + 1 >= ns[d]) {
        lo[d] = -bi[d];
        hi[d] = ns[d] - 1 - bi[d];
      } else if (p.periodic[d]) {
        lo[d] = -k;
        hi[d] = k;
      } else {
        lo[d] = bi[d] - k < 0 ? -bi[d] : -k;
        hi[d] = bi[d] + k >= ns[d] ? ns[d] - 1 - bi[d] : k;
      }
    }
    for (int o0 = lo[0]; o0 <= hi[0]; ++o0)
      for (int o1 = (D > 1 ? lo[1] : 0); o1 <= (D > 1 ? hi[1] : 0); ++o1)
        for (int o2 = (D > 2 ? lo[2] : 0); o2 <= (D > 2 ? hi[2] : 0); ++o2) {
          const int oo[3] = {o0, o1, o2};
          int b = 0;
          for (int d = 0; d < D; ++d) {
            int v = bi[d] + oo[d];
            if (v < 0) v += ns[d];
            if (v >= ns[d]) v -= ns[d];
            b = b * ns[d] + v;
          }
          for (int j : bins[b])
            if (j != i || with_self) fn(j);
        }
  }

  // every cell in the bins within `radius` of cell i, itself included, in the GPU model's order
  template <class Fn>
  void each_neighbour_all(int i, double radius, const Bins &bins, Fn fn) const {
    each_neighbour(i, radius, bins, fn, true);
  }

  // r_j - r_i at the nearest image (Box::distance's Nint, |dd| < L); returns its square length
  double separation(int i, int j, double *rij) const {
    double r2 = 0;
    for (int d = 0; d < D; ++d) {
      double dd = c[j].x[d] - c[i].x[d];
      if (p.periodic[d]) {
        if (dd > 0.5 * p.box[d])
          dd -= p.box[d];
        else if (dd < -(0.5 * p.box[d]))
          dd += p.box[d];
      }
      rij[d] = dd;
      r2 += dd * dd;
    }
    return r2;
  }

  // motility, passive noise, Hertz contacts with adhesion, and the pressure of cell i; draws
  // keyed by step `key`
  void conservative(int i, const Bins &bins, int key, double *F, double *pres_out) {
    const Cell &ci = c[i];
    const double c2 = (1 - p.nu * p.nu) / p.E + (1 - p.nu * p.nu) / p.E;
    double vi[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) F[d] = 0;
    for (int d = 0; d < D; ++d) vi[d] = ci.v[d];
    double v2 = 0;
    for (int d = 0; d < D; ++d) v2 += vi[d] * vi[d];
    double vl = std::sqrt(v2);
    if (vl == 0.0) {
      const Block r = draw(i, key, kDir, 0);
      if (D == 2) {
        const double ang = 6.283185307179586 * u53(r.v[0], r.v[1]);
        vi[0] = 1e-11 * std::cos(ang);
        vi[1] = 1e-11 * std::sin(ang);
      } else {
        const double z = 2.0 * u53(r.v[0], r.v[1]) - 1.0;
        const double ang = 6.283185307179586 * u53(r.v[2], r.v[3]);
        const double s = std::sqrt(1.0 - z * z);
        vi[0] = 1e-11 * (s * std::cos(ang));
        vi[1] = 1e-11 * (s * std::sin(ang));
        vi[2] = 1e-11 * z;
      }
      v2 = 0;
      for (int d = 0; d < D; ++d) v2 += vi[d] * vi[d];
      vl = std::sqrt(v2);
    }
    for (int d = 0; d < D; ++d) F[d] = p.motility * (vi[d] / vl);
    if (noise_amp > 0.0) {
      double nz[4];
      normal2(draw(i, key, kNoise, 0), &nz[0], &nz[1]);
      if (D == 3) normal2(draw(i, key, kNoise, 1), &nz[2], &nz[3]);
      for (int d = 0; d < D; ++d) F[d] += p.zeta * (noise_amp * nz[d]);
    }
    // the candidates of the bin walk (self included) go to 2^lane_bits partial sums in turn
    const int L = 1 << lane_bits;
    double pl[8] = {0, 0, 0, 0, 0, 0, 0, 0}, Fl[8][3] = {};
    int kflat = 0;
    each_neighbour_all(i, smax, bins, [&](int j) {
      const int lane = kflat++ & (L - 1);
      if (j == i) return;
      double *Fc = Fl[lane];
      double &pres = pl[lane];
      double rij[3] = {0, 0, 0};
      const double r2 = separation(i, j, rij);
      const double si = ci.sig, sj = c[j].sig;
      const double r = std::sqrt(r2);
      if (!(r <= (si + sj) / 2) || r == 0.0) return;
      const double sa = i < j ? si : sj, sb = i < j ? sj : si;
      const double h = std::fmax((si + sj) / 2 - r, 0.0);
      const double Sr = 1.0 / (si / 2) + 1.0 / (sj / 2);
      const double inv_hz = 1.0 / (0.75 * c2);
      // h^1.5 / (0.75 c2 sqrt(S)) as h sqrt(h / S) / (0.75 c2), the GPU model's expression;
      // in 2D one reciprocal u = 1 / (S A) gives both h / S = h A u and f0 / A = f0 S u
      double fel, f0;
      if (D == 3) {
        fel = h * std::sqrt(h / Sr) * inv_hz;
        const double A = contact_area(r, sa, sb);
        const double vol = (A == 0 ? 0 : (4 * kPi * ((sa / 2) * (sa / 2)) / 3));
        f0 = -fel + p.adhesion * A;
        if (vol != 0.0) pres -= f0 / vol;
      } else {
        const double A = contact_length(sa, sb, h);
        if (A != 0.0) {
          const double u = 1.0 / (Sr * A);
          fel = h * std::sqrt(h * (A * u)) * inv_hz;
          f0 = -fel + p.adhesion * A;
          pres -= f0 * (Sr * u);
        } else {
          fel = h * std::sqrt(h / Sr) * inv_hz;
          f0 = -fel;
        }
      }
      for (int d = 0; d < D; ++d) Fc[d] += f0 * rij[d];
    });
    // the GPU model's xor tree: lane l adds lane l ^ off, off from L / 2 down to 1
    for (int off = L >> 1; off > 0; off >>= 1)
      for (int l = 0; l < L; ++l)
        if (l < (l ^ off)) {
          const double ps = pl[l] + pl[l ^ off];
          pl[l] = pl[l ^ off] = ps;
          for (int d = 0; d < D; ++d) {
            const double fs = Fl[l][d] + Fl[l ^ off][d];
            Fl[l][d] = Fl[l ^ off][d] = fs;
          }
        }
    for (int d = 0; d < D; ++d) F[d] += Fl[0][d];
    for (int d = 0; d < D; ++d)
      if (!std::isfinite(F[d])) err |= 2;
    *pres_out = pl[0];
  }

  // Euler: forces, then the position update with pressure-dependent friction (CIL.cu:902-939)
  void forces(std::vector<double> &xn) {
    const int n = static_cast<int>(c.size());
    const Bins bins = bin_cells();
    xn.assign(static_cast<size_t>(n) * D, 0.0);
    std::vector<double> vn(static_cast<size_t>(n) * D), pn(n);
    for (int i = 0; i < n; ++i) {
      const Cell &ci = c[i];
      double F[3], pres;
      conservative(i, bins, ts, F, &pres);
      const double pnd = pres / p.cycle_p0;
      const double temp = p.dt * 1 / ((p.zeta + p.zeta_p * std::pow(pnd, p.zeta_p_beta)) * area_of(ci.sig));
      for (int d = 0; d < D; ++d) {
        const double t = ci.x[d] + temp * F[d];
        xn[static_cast<size_t>(i) * D + d] = p.periodic[d] ? std::fmod(t + p.box[d], p.box[d]) : t;
        vn[static_cast<size_t>(i) * D + d] = F[d] * (temp / p.dt);
      }
      pn[i] = pres;
    }
    for (int i = 0; i < n; ++i) {
      for (int d = 0; d < D; ++d) {
        c[i].x[d] = xn[static_cast<size_t>(i) * D + d];
        c[i].v[d] = vn[static_cast<size_t>(i) * D + d];
      }
      c[i].p = pn[i];
    }
  }

  // Euler: the forces and pressures at the current state, which the reference's step evaluates
  // at its end (CIL.cu:1019) and writes out; the next step computes the same values again
  std::vector<double> out_f;  // [cell][3]
  void refresh() {
    if (p.integrator == 1) return;
    const int n = static_cast<int>(c.size());
    const Bins bins = bin_cells();
    out_f.assign(static_cast<size_t>(n) * 3, 0.0);
    std::vector<double> pn(n);
    for (int i = 0; i < n; ++i) conservative(i, bins, ts, &out_f[static_cast<size_t>(i) * 3], &pn[i]);
    for (int i = 0; i < n; ++i) c[i].p = pn[i];
  }

  // ---- DPD (CIL.cu:1054-1066)
  double kick_div = 1, sqrt_dt = 1, sigma_r = 0;

  double kick(double v, double fc, double fd, double fr) const {  // updateVel, Utils.hpp:568-571
    return v + (fc * p.dt + fd * p.dt + fr * sqrt_dt) / kick_div;
  }

  // Fc and the pressure, then the pair dissipative and random forces (cellCellDisRanForce,
  // MD.cu:861-905) over the pairs closer than the lower-index cell's diameter, one normal per
  // pair and axis keyed (lower index, key, purpose, higher index); with `kick_on`, the second
  // half kick
  void dpd_forces(int key, bool kick_on) {
    const int n = static_cast<int>(c.size());
    const Bins bins = bin_cells();
    std::vector<double> fc(static_cast<size_t>(n) * 3), pn(n);
    for (int i = 0; i < n; ++i) conservative(i, bins, key, &fc[static_cast<size_t>(i) * 3], &pn[i]);
    std::vector<double> fd(static_cast<size_t>(n) * 3, 0.0), fr(static_cast<size_t>(n) * 3, 0.0),
        vn(static_cast<size_t>(n) * 3, 0.0);
    for (int i = 0; i < n; ++i) {
      double *Fd = &fd[static_cast<size_t>(i) * 3], *Fr = &fr[static_cast<size_t>(i) * 3];
      const double si = c[i].sig;
      each_neighbour(i, smax, bins, [&](int j) {
        double rij[3] = {0, 0, 0};
        const double r = std::sqrt(separation(i, j, rij));
        const double rc = i < j ? si : c[j].sig;
        if (!(r < rc) || r == 0.0) return;
        const double w = 1 - (r / rc);
        const uint32_t a = static_cast<uint32_t>(i < j ? i : j), z = static_cast<uint32_t>(i < j ? j : i);
        double xi[4];
        normal2(philox(a, static_cast<uint32_t>(key), kDpd0, z, k0, k1), &xi[0], &xi[1]);
        if (D == 3) normal2(philox(a, static_cast<uint32_t>(key), kDpd1, z, k0, k1), &xi[2], &xi[3]);
        const double sw = std::sqrt(w);
        const double ir = 1.0 / r;  // the GPU model's one division per pair
        for (int d = 0; d < D; ++d) {
          const double nd = rij[d] * ir;
          Fd[d] -= p.dis_diff * w * ((c[i].v[d] - c[j].v[d]) * nd) * nd;
          Fr[d] += sigma_r * sw * nd * xi[d];
        }
      });
      for (int d = 0; d < D; ++d) {
        const size_t k = static_cast<size_t>(i) * 3 + d;
        vn[k] = kick(c[i].v[d], fc[k], fd[k], fr[k]);
        if (kick_on && !std::isfinite(vn[k])) err |= 2;
      }
    }
    for (int i = 0; i < n; ++i) {
      c[i].p = pn[i];
      for (int d = 0; d < D; ++d) {
        const size_t k = static_cast<size_t>(i) * 3 + d;
        c[i].fc[d] = fc[k];
        c[i].fd[d] = fd[k];
        c[i].fr[d] = fr[k];
        if (kick_on) c[i].v[d] = vn[k];
      }
    }
  }

  // background and pair dissipation at the current velocities (calculDisForces,
  // CIL.cu:294-364; cellBackDisForce, MD.cu:846-859; cellCellDisForce, MD.cu:951-985)
  void dpd_dis() {
    const int n = static_cast<int>(c.size());
    const Bins bins = bin_cells();
    const double rc = p.sigma_core;
    std::vector<double> fd(static_cast<size_t>(n) * 3, 0.0);
    for (int i = 0; i < n; ++i) {
      double *Fd = &fd[static_cast<size_t>(i) * 3];
      for (int d = 0; d < D; ++d) {
        Fd[d] = 0;
        Fd[d] -= p.dis_bg * c[i].v[d];
      }
      each_neighbour(i, smax > rc ? smax : rc, bins, [&](int j) {
        double rij[3] = {0, 0, 0};
        const double r = std::sqrt(separation(i, j, rij));
        if (!(r < rc) || r == 0.0) return;
        const double w = 1 - ((r * r) / rc);
        for (int d = 0; d < D; ++d) {
          const double nd = -rij[d] / r;
          Fd[d] -= p.dis_diff * w * ((c[i].v[d] - c[j].v[d]) * nd) * nd;
        }
      });
    }
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < D; ++d) c[i].fd[d] = fd[static_cast<size_t>(i) * 3 + d];
  }

  void dpd_step() {
    for (Cell &ci : c)  // updateVelocities, updatePositions (CIL.cu:1055-1056)
      for (int d = 0; d < D; ++d) {
        ci.v[d] = kick(ci.v[d], ci.fc[d], ci.fd[d], ci.fr[d]);
        const double x = ci.x[d];
        ci.x[d] = p.periodic[d] ? std::fmod(x + p.dt * ci.v[d] + p.box[d], p.box[d]) : x + ci.v[d] * p.dt;
      }
    dpd_forces(ts + 1, true);
    dpd_dis();
  }

  void cycle() {
    const int n = static_cast<int>(c.size());
    std::vector<int> flag(n, 0);
    for (int i = 0; i < n; ++i) {
      Cell &ci = c[i];
      if (!p.divide || ci.p < p.apop_pressure)
        ci.tp = 0;
      else
        ci.tp += 1;
      if (!p.divide) continue;
      const double shift = p_shift != 0.0 ? p_shift * std::exp(-ts * p_shift_tau_inv) : 0.0;
      const double pnd = std::fmax(0., ci.p + shift) / p.cycle_p0;
      const double om = ci.om;
      double rho = ci.rho;
      ci.theta += om * std::fmin(r_maxed_inv * rho, 1.0);
      const bool d3 = D == 3;
      double vt = d3 ? volume_of(ci.sigt) : area_of(ci.sigt);
      double v = d3 ? volume_of(ci.sig) : area_of(ci.sig);
      const double c0 = om * std::log(2.0) + (p.v1 - 1) / tau_v;
      const double vt_prime = c0 * rho - (((vt - v_s) / v_s) / tau_v);
      vt += vt_prime * vt;
      const double v_prime = -(v - (vt / (1 + p.cycle_beta_vs * (p.osmotic_pressure + pnd)))) / tau_p;
      v += v_prime;
      v = tau_p == 0 ? vt : v;
      ci.sigt = d3 ? sigma_of_volume(vt) : sigma_of_area(vt);
      ci.sig = d3 ? sigma_of_volume(v) : sigma_of_area(v);
      const double r_np = (1 - rho - pnd);
      const double tau_r_pre = r_np > 0 ? 1 : p.cycle_rho_ratio;
      rho += r_np / (tau_r * tau_r_pre) * rho;
      ci.rho = rho;
      flag[i] = ci.theta >= 1 ? 1 : 0;
    }
    if (!p.divide) return;
    smax = 0;
    for (int i = 0; i < n; ++i) smax = std::fmax(smax, c[i].sig);
    for (int i = 0; i < n; ++i) {
      if (!flag[i]) continue;
      if (static_cast<int>(c.size()) >= cap) {
        err |= 1;
        continue;
      }
      Cell &m = c[i];
      Cell dau = m;
      const double lmom = m.sig;
      double ldau, dr[3] = {0, 0, 0};
      const Block r0 = draw(i, ts, kDiv, 0);
      if (D == 2) {
        ldau = lmom / std::sqrt(2.0);
        const double rr = (lmom - ldau) / 2;
        const double alpha = u53(r0.v[0], r0.v[1]) * 6.283185307179586;
        dr[0] = rr * std::sin(alpha);
        dr[1] = rr * std::cos(alpha);
      } else {
        const double rmom = lmom / 2;
        const double vmom = 4 * kPi * rmom * rmom * rmom / 3;
        const double a = 9 * lmom / 4, b = -(3 * (lmom * lmom) / 2), cc = lmom * lmom * lmom / 4 - 3 * vmom / (kPi);
        ldau = (-b + std::sqrt(b * b - 4 * a * cc)) / (2 * a);
        const double rr = (lmom - ldau) / 2;
        const double alpha = u53(r0.v[0], r0.v[1]) * 6.283185307179586;
        const double beta = u53(r0.v[2], r0.v[3]) * 6.283185307179586;
        dr[0] = rr * std::sin(alpha) * std::cos(beta);
        dr[1] = rr * std::sin(alpha) * std::sin(beta);
        dr[2] = rr * std::cos(alpha);
      }
      for (int d = 0; d < D; ++d) {
        const double x0 = m.x[d];
        double xd = x0 + dr[d], xm = x0 + (-dr[d]);
        if (p.periodic[d]) {
          xd = std::fmod(xd + p.box[d], p.box[d]);
          xm = std::fmod(xm + p.box[d], p.box[d]);
        }
        dau.x[d] = xd;
        m.x[d] = xm;
        dau.v[d] = 0;
        m.v[d] = 0;
        dau.fc[d] = dau.fd[d] = dau.fr[d] = 0;  // resetFrc (CIL.cu:597-598)
        m.fc[d] = m.fd[d] = m.fr[d] = 0;
      }
      double z0, z1, z2, z3;
      normal2(draw(i, ts, kDiv, 1), &z0, &z1);
      normal2(draw(i, ts, kDiv, 2), &z2, &z3);
      dau.tsw = ts + span_steps(p.tau_mig_mu + p.tau_mig_sigma * z0, p.dt);
      m.tsw = ts + span_steps(p.tau_mig_mu + p.tau_mig_sigma * z1, p.dt);
      m.om = 1.0 / span_steps(lognormal(p.tau_div_mu, p.tau_div_sigma, z2), p.dt);
      dau.om = 1.0 / span_steps(lognormal(p.tau_div_mu, p.tau_div_sigma, z3), p.dt);
      m.sig = dau.sig = ldau;
      m.sigt = dau.sigt = ldau;
      m.t0 = dau.t0 = ts;
      m.theta = dau.theta = 0;
      dau.p = m.p;
      dau.rho = m.rho;
      dau.tp = -1;
      c.push_back(dau);
      ++ndiv;
    }
  }

  void remove_if(const std::vector<char> &keep) {
    std::vector<Cell> out;
    out.reserve(c.size());
    for (size_t i = 0; i < c.size(); ++i)
      if (keep[i]) out.push_back(c[i]);
    c.swap(out);
  }

  void apoptosis() {
    if (p.apoptosis == 0) return;
    const int n = static_cast<int>(c.size());
    std::vector<char> keep(n, 1);
    for (int i = 0; i < n; ++i) {
      const Block r = draw(i, ts, kApo, 0);
      const double u = u53(r.v[0], r.v[1]);
      const double rho = c[i].rho;
      if (p.apoptosis == 1) {  // CyclePressure (CIL.cu:711-738)
        const double pr = c[i].p;
        const double rate = apop_rate_step * std::pow((1 - (rho / p.apop_pressure)), p.apop_duration) *
                            std::pow(pr / (pr + p.cycle_p0), p.extr_gamma);
        if (u <= rate) keep[i] = 0;
      } else if (p.apoptosis == 2) {  // PressureTime (CIL.cu:653-676)
        if (((p.apop_duration > 0) && (c[i].tp >= apop_steps)) || ((apop_rate_step > 0) && (u <= apop_rate_step)))
          keep[i] = 0;
      } else if (p.apoptosis == 3) {  // constant rate (CIL.cu:627-649)
        if (u <= apop_rate_step) keep[i] = 0;
      } else if (p.apoptosis == 4) {  // Cycle (CIL.cu:681-709); cells with rho >= 1 stay
        if (rho < 1 && u <= apop_rate_step * std::pow((1 - (rho / p.apop_pressure)), p.apop_duration)) keep[i] = 0;
      } else {  // CycleExtrude (CIL.cu:749-788)
        if (rho < 1 && u <= apop_rate_step) keep[i] = 0;
        const double u2 = u53(r.v[2], r.v[3]);
        if (rho <= 0.1 && u2 <= p.extr_rate * std::pow(((c[i].p - p.apop_pressure) / p.apop_pressure), p.extr_gamma))
          keep[i] = 0;
      }
    }
    const size_t before = c.size();
    remove_if(keep);
    napo += static_cast<long long>(before - c.size());
  }

  void step() {
    if (p.integrator == 1) {
      dpd_step();
    } else {
      std::vector<double> xn;
      forces(xn);
    }
    ++ts;
    cycle();
    apoptosis();
  }

  int check_positions() {
    const int n = static_cast<int>(c.size());
    std::vector<char> keep(n, 1);
    int out = 0;
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < D; ++d)
        if (!(c[i].x[d] >= 0.0 && c[i].x[d] < p.box[d])) keep[i] = 0;
    for (char k : keep) out += !k;
    if (!p.drain) return out ? -1 : 0;
    remove_if(keep);
    return out;
  }
};

}  // namespace

extern "C" {

void *cyo_create(const cyo_params *p, int32_t capacity, uint64_t seed) {
  Model *m = new Model();
  m->init(*p, capacity, seed);
  return m;
}

void cyo_destroy(void *h) { delete static_cast<Model *>(h); }

// Sets the colony; theta/rho/angvel may be NULL only together with sigma NULL handled by the
// caller: this restatement takes the full state (the initial-status draws are checked on the
// GPU side against the reference's formulas separately).
void cyo_set_state(void *h, int32_t n, int32_t ts, const double *pos, const double *vel, const double *sigma,
                   const double *sigma_t, const double *theta, const double *rho, const double *angvel,
                   const double *pressure, const int32_t *tpressure) {
  Model *m = static_cast<Model *>(h);
  m->c.assign(n, Cell{});
  m->ts = ts;
  m->smax = 0;
  for (int i = 0; i < n; ++i) {
    Cell &c = m->c[i];
    for (int d = 0; d < m->D; ++d) {
      c.x[d] = pos[static_cast<size_t>(i) * m->D + d];
      c.v[d] = vel ? vel[static_cast<size_t>(i) * m->D + d] : 0.0;
    }
    c.sig = sigma[i];
    c.sigt = sigma_t ? sigma_t[i] : sigma[i];
    c.theta = theta[i];
    c.rho = rho[i];
    c.om = angvel[i];
    c.p = pressure ? pressure[i] : 0.0;
    c.tp = tpressure ? tpressure[i] : 0;
    c.t0 = 0;
    c.tsw = -1;
    m->smax = std::fmax(m->smax, c.sig);
  }
  m->rebin();
  if (m->p.integrator == 1) m->dpd_forces(ts, false);  // the forces before the first step (CIL.cu:1096)
}

int32_t cyo_step(void *h, int32_t nsteps) {
  Model *m = static_cast<Model *>(h);
  m->rebin();
  for (int s = 0; s < nsteps; ++s) m->step();
  return m->err;
}

int32_t cyo_check_positions(void *h) { return static_cast<Model *>(h)->check_positions(); }

int32_t cyo_num_cells(const void *h) { return static_cast<int32_t>(static_cast<const Model *>(h)->c.size()); }

void cyo_get_state(void *h, double *pos, double *vel, double *sigma, double *sigma_t, double *theta,
                   double *rho, double *angvel, double *pressure, int32_t *tpressure, int64_t *counts) {
  Model *m = static_cast<Model *>(h);
  m->refresh();
  const int n = static_cast<int>(m->c.size());
  for (int i = 0; i < n; ++i) {
    const Cell &c = m->c[i];
    for (int d = 0; d < m->D; ++d) {
      pos[static_cast<size_t>(i) * m->D + d] = c.x[d];
      vel[static_cast<size_t>(i) * m->D + d] = c.v[d];
    }
    sigma[i] = c.sig;
    sigma_t[i] = c.sigt;
    theta[i] = c.theta;
    rho[i] = c.rho;
    angvel[i] = c.om;
    pressure[i] = c.p;
    tpressure[i] = c.tp;
  }
  counts[0] = m->ts;
  counts[1] = m->ndiv;
  counts[2] = m->napo;
}

// The forces a final-state file holds: Euler, the force at the current state (Fd, Fr zero);
// DPD, Fc, Fd and Fr. Arrays [cell][dim].
void cyo_get_forces(void *h, double *fc, double *fd, double *fr) {
  Model *m = static_cast<Model *>(h);
  m->refresh();
  const int n = static_cast<int>(m->c.size());
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < m->D; ++d) {
      const size_t k = static_cast<size_t>(i) * m->D + d;
      const bool dpd = m->p.integrator == 1;
      fc[k] = dpd ? m->c[i].fc[d] : m->out_f[static_cast<size_t>(i) * 3 + d];
      fd[k] = dpd ? m->c[i].fd[d] : 0.0;
      fr[k] = dpd ? m->c[i].fr[d] : 0.0;
    }
}

}  // extern "C"
