// Test infrastructure only: the reference's Lennard-Jones element force (LJParams::elemForce,
// MD.cuh:98-113, with elemForce0 MD.cuh:50-56) and soft-core cubic well (SCParams::elemForce,
// MD.cuh:199-214, with elemForce0 MD.cuh:144-162) called from C, compiled from the reference tree
// by oracle/ref_build.sh into oracle/_ref/libref_force.so. MD.cuh is compiled as host C++
// (__host__/__device__ defined empty) with the stand-ins of oracle/ref_stubs for the headers
// its tree lacks, and with the HDF5 header SimIO.hpp skipped (-DSIMIO_HPP; nothing compiled
// here uses it). The force golden vectors (tests/golden/make_geometry_golden.py) come from these
// calls.
#include <cmath>
#include <cstdint>
#include <vector>
using std::isnan;  // Utils.hpp calls isnan unqualified
#include "MD.cuh"

// globals the reference's headers declare extern (Common.hpp:19-20, 61)
int DIM = 2;
int ACTIVE_NOISE_DIM = 2;
enum_set<OPT::OPT> SWITCH;

// LJParams::init and SCParams::init are defined in MD.cu, whose CUDA draft does not compile;
// these stand-ins (never called) are the classes' key functions, so that their vtables and type
// information are emitted here
void LJParams::init(const vector<ElemParams> &, const array2<double> &) {
  throw std::runtime_error("LJParams::init is not part of what is compiled here");
}
void SCParams::init(const vector<ElemParams> &, const array2<double> &) {
  throw std::runtime_error("SCParams::init is not part of what is compiled here");
}

namespace {

// LJParams with its two coefficient tables set directly for one element type: epsilon(0, 0) as
// LJParams::init forms it (24 sqrt(eps_i eps_j), MD.cu:13) and rcut2(0, 0) as readInteractionsLJ
// sets it without attraction (pow(2, 1/3), Input.cpp:296-301). LJParams::init itself lives in
// MD.cu, whose CUDA draft does not compile.
class PinnedLJ : public LJParams {
 public:
  PinnedLJ(double eps, double rc2) {
    epsilon.Allocate(1, 1);
    rcut2.Allocate(1, 1);
    epsilon(0, 0) = 24.0 * std::sqrt(eps * eps);
    rcut2(0, 0) = rc2;
  }
};

// SCParams with its coefficient tables set directly for one element type, as SCParams::init
// forms them (MD.cu:57-77): sqrt(eps0 eps0), sqrt(eps1 eps1), (xi + xi) / 2 and rcut2.
class PinnedSC : public SCParams {
 public:
  PinnedSC(double eps_core, double eps_well, double xi, double rc2) {
    epsilonCore.Allocate(1, 1);
    epsilonWell.Allocate(1, 1);
    sigmaWell.Allocate(1, 1);
    rcut2.Allocate(1, 1);
    epsilonCore(0, 0) = std::sqrt(eps_core * eps_core);
    epsilonWell(0, 0) = std::sqrt(eps_well * eps_well);
    sigmaWell(0, 0) = 0.5 * (xi + xi);
    rcut2(0, 0) = rc2;
  }
  // SCParams leaves the diameter-taking elemForce of PairForceParams pure (the reference never
  // instantiates it through this path); a stand-in makes the class concrete here
  using SCParams::elemForce;
  bool elemForce(const ElemParams &, const ElemParams &, const double &, double &, const double &,
                 const double &) const override {
    throw std::runtime_error("not part of what is compiled here");
  }
};

}  // namespace

extern "C" {

// f0[i] = SCParams::elemForce(ei, ej, r2[i], fij, phi, false, pe) for elements of diameters si[i],
// sj[i]; inside[i] = its return value; shifted sets OPT::FORCE_SHIFTED for the calls
void ref_sc_force(double eps_core, double eps_well, double xi, double rc2, int32_t shifted, int64_t n,
                  const double *r2, const double *si, const double *sj, double *f0, int32_t *inside) {
  const PinnedSC sc(eps_core, eps_well, xi, rc2);
  SWITCH.set(OPT::FORCE_SHIFTED, shifted != 0);
  ElemParams ei{}, ej{};
  ei.type = ej.type = 0;
  for (int64_t k = 0; k < n; ++k) {
    ei.sigmaCoreX = si[k];
    ej.sigmaCoreX = sj[k];
    double fij = 0.0, phi = 0.0, pe = 0.0;
    inside[k] = sc.elemForce(ei, ej, r2[k], fij, phi, false, pe) ? 1 : 0;
    f0[k] = fij;
  }
  SWITCH.set(OPT::FORCE_SHIFTED, false);
}

// WCA cutoff of the reference (its readInteractionsLJ default)
double ref_lj_wca_rc2() { return pow(2.0, 1.0 / 3.0); }

// f0[i] = LJParams::elemForce(ei, ej, r2[i], fij, ...) for elements of diameters si[i], sj[i];
// inside[i] = its return value (r2 <= rc2)
void ref_lj_force(double eps, double rc2, int64_t n, const double *r2, const double *si, const double *sj,
                  double *f0, int32_t *inside) {
  const PinnedLJ lj(eps, rc2);
  ElemParams ei{}, ej{};
  ei.type = ej.type = 0;
  for (int64_t k = 0; k < n; ++k) {
    ei.sigmaCoreX = si[k];
    ej.sigmaCoreX = sj[k];
    double fij = 0.0;
    inside[k] = lj.elemForce(ei, ej, r2[k], fij, si[k], sj[k]) ? 1 : 0;
    f0[k] = fij;
  }
}

// f0[i] = LJParams::elemForce(ei, ej, r2[i], fij, phi, false, pe) (the overload cellCellForce
// calls, MD.cu:768-769) with the attraction's cutoff, rcut2 = SQ(RCUT) as readInteractionsLJ sets
// it (Input.cpp:303-315), and OPT::FORCE_SHIFTED when shifted (its SHIFT FORCE)
void ref_lj_attr_force(double eps, double rcut, int32_t shifted, int64_t n, const double *r2, const double *si,
                       const double *sj, double *f0, int32_t *inside) {
  const PinnedLJ lj(eps, rcut * rcut);
  SWITCH.set(OPT::FORCE_SHIFTED, shifted != 0);
  ElemParams ei{}, ej{};
  ei.type = ej.type = 0;
  for (int64_t k = 0; k < n; ++k) {
    ei.sigmaCoreX = si[k];
    ej.sigmaCoreX = sj[k];
    double fij = 0.0, phi = 0.0, pe = 0.0;
    inside[k] = lj.elemForce(ei, ej, r2[k], fij, phi, false, pe) ? 1 : 0;
    f0[k] = fij;
  }
  SWITCH.set(OPT::FORCE_SHIFTED, false);
}

}  // extern "C"
