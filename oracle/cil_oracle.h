/* ORACLE — test infrastructure only.
 *
 * CPU restatement of the reference's overdamped cell-colony timestep (KokoroSinx/cil_cuda,
 * Euler integrator: CIL.cu:1013-1020 with calculForcesPressure CIL.cu:999-1007), used as
 * the oracle the tests compare the CUDA library with, and as the timed CPU baseline. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs load it; the product never does.
 *
 * Pinning: the random-number layer (dSFMT-19937, Leva normals, onDSphere, uniform
 * variants) is pinned bit-for-bit against the reference's own mt/dSFMT.c + Random.hpp
 * (golden vectors in tests/golden/dsfmt_random_golden.json). The box and link-list geometry
 * (Nint, minimum image, the fmod wrap of updatePos, grid sizing, bin ids, LIFO lists, bin
 * coordinates, half-stencil neighbours) and the Lennard-Jones law are pinned bit for bit
 * against the reference's Utils.hpp and MD.cuh compiled from its tree
 * (tests/golden/geometry_golden.json). The reference's step itself does not compile and ships
 * no fixtures, so the soft-core and Hertz laws of the benchmark workloads (which have no
 * reference counterpart), the cell-cell force assembly, division and apoptosis remain
 * restated from the reference source (cited per function in cil_oracle.cpp) without a
 * reference-produced number: "parity unpinned" for those parts.
 */
#ifndef CIL_ORACLE_H
#define CIL_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORA_FORCE_LJ_WCA = 0, ORA_FORCE_SOFTCORE = 1, ORA_FORCE_HERTZ = 2, ORA_FORCE_SC = 3 };

typedef struct ora_params {
  int32_t dim;            /* 2 or 3 */
  int32_t force_law;      /* ORA_FORCE_* */
  int32_t noise_per_cell; /* 0: one normal per element component, 1: per cell (reference) */
  int32_t divide;         /* linear growth + division on */
  double box[3];
  int32_t periodic[3];
  int32_t nwalls; /* 0..2 flat one-sided Hertz walls normal to the last axis */
  int32_t wall_dir[2];
  double wall_pos[2];
  double wall_E;
  double epsilon;    /* LJ epsilon / soft-core epsilon / Hertz modulus E */
  double rcut_scale; /* cutoff in units of sigma_ij = (sigma_i + sigma_j)/2 */
  double zeta[2];    /* friction of back/front element; mobility = 1/zeta */
  double motility[2];/* back element gets -m0*n, front +m1*n (n = back->front unit axis) */
  double kappa;      /* linear intra-cell spring */
  double rest0;      /* rest length at birth */
  double rest1;      /* rest length at division */
  double noise_D;    /* passive diffusion constant */
  double dt;
  double div_tau_mu, div_tau_sigma; /* division time ~ N(mu, sigma), time units */
  double apop_rate;                 /* per unit time */
  double well_epsilon;              /* ORA_FORCE_SC: well depth Em */
  double well_sigma;                /* ORA_FORCE_SC: well width xi (absolute) */
  int32_t force_shifted;            /* ORA_FORCE_SC: OPT::FORCE_SHIFTED */
  int32_t intra_law;                /* 0: linear spring with growth, 1: the reference's FENE / push bond */
  int32_t cil;                      /* intra_law 1: the species' CIL flag */
  double fene_kappa, fene_kappa_push, fene_spring_ratio, fene_rmax; /* intra_law 1 */
  /* intra_law 1 with divide: the reference's crawling/dividing cells (calculDivisions,
   * CIL.cu:369-455): RMAX_DIVISION (0: RMAX), GROWTHK0/1/2 per element, R0, Rmin, Rmin_RATIO,
   * TAU_MIGRATION, the diameters a division resets to (SIGMA_CORE) */
  double fene_rmax_division;
  double growth_k0[2], growth_k1[2], growth_k2[2];
  double div_r0, div_rmin, div_rmin_ratio;
  double mig_tau_mu, mig_tau_sigma;
  double sigma_core[2];
  double noise_radial, noise_angular; /* intra_law 1, 2D: the bond's active noise (NOISE_ACTIVE) */
  int32_t div_swelling;               /* intra_law 1 with divide: DIVISION.SWELLING */
  int32_t pad_swell;
} ora_params;

typedef struct ora_event {
  int32_t ts;
  int32_t kind; /* 0 = division (a = mother, b = daughter), 1 = apoptosis (a = slot, b = moved-from) */
  int32_t a, b;
} ora_event;

typedef struct ora_obs {
  int32_t ncells;
  int32_t pad;
  double mean_area;
  double msd;
  double vacf;
  int64_t ndiv_total;
  int64_t napo_total;
} ora_obs;

void *ora_create(const ora_params *p, int32_t cap_cells, uint32_t seed);
void ora_destroy(void *h);
/* 0 = single thread, reference half-stencil order; >0 = OpenMP race-free full stencil */
void ora_set_threads(void *h, int32_t nthreads);
/* 0: Euler (CIL.cu:1013-1020); 1: StochasticHeun (CIL.cu:1028-1050), two half steps. */
void ora_set_integrator(void *h, int32_t integrator);
int32_t ora_set_state(void *h, int32_t ncells, const double *pos, const double *sigma,
                      const int32_t *t0, const int32_t *tswitch, int32_t ts);
int32_t ora_num_cells(const void *h);
int32_t ora_timestep(const void *h);
/* cell states of the reference's two-element cells (CellState: 0 dividing, 1 crawling,
 * 2 undefined), [cell]; set after ora_set_state (which leaves every cell undefined) */
void ora_set_cell_states(void *h, int32_t n, const int32_t *states);
void ora_get_cell_states(const void *h, int32_t *states);
void ora_get_state(const void *h, double *pos, double *sigma, double *vel, double *frc,
                   int32_t *t0, int32_t *tswitch);
/* forces at the current state (draws the noise like calculForcesPressure) into frc */
void ora_compute_forces(void *h);
/* nsteps full Euler steps; returns 0 or a negative error */
int32_t ora_step(void *h, int32_t nsteps);
/* element link list of the current positions (Container.cpp:58-79, Utils.hpp:872-1001);
 * returns the number of bins, fills ns[3], head[nbins], list[2*ncells] */
int32_t ora_bin_elements(const void *h, double width, int32_t *ns, int32_t *head, int32_t *list,
                         int32_t max_bins);
int32_t ora_num_events(const void *h);
void ora_get_events(const void *h, ora_event *out);
void ora_clear_events(void *h);
void ora_obs_reset(void *h);
void ora_observables(void *h, ora_obs *out);

/* The restated box and link-list geometry on its own, for the checks against the reference's
 * compiled Utils.hpp (golden vectors in tests/golden/geometry_golden.json):
 *   Nint (Utils.hpp:173-175);
 *   BoundingBox::distance over n pairs (Utils.hpp:536-544): r12[n][dim], d2[n];
 *   BoundingBox::updatePos over n positions (Utils.hpp:556-566): dt == 0 takes v as the
 *     displacement dr, otherwise r += dt v, both wrapped by fmod on periodic axes;
 *   LinkListOrtho get_opt_size + init/reset + populate_list (Utils.hpp:872-1001) with
 *     get_cellCoord and get_cellID over the half stencil (Utils.hpp:922-936, 1018-1069):
 *     ns[3], head[nbins], list[n], coords[nbins][dim], neighbor_ids[nbins][5 or 14];
 *     returns nbins, or -nbins when nbins > max_bins;
 *   the element pair force modulus of a law (the one the step uses) for n (r2, si, sj):
 *     f0[n] and inside[n] (PairForceParams::elemForce's value and return, MD.cuh:98-113). */
int32_t ora_geom_nint(double a);
void ora_geom_distance(int32_t dim, const double *box, const int32_t *periodic, int64_t n, const double *r1,
                       const double *r2, double *r12, double *d2);
void ora_geom_update_pos(int32_t dim, const double *box, const int32_t *periodic, int64_t n, double *r,
                         const double *v, double dt);
int32_t ora_geom_link_list(int32_t dim, double rcut, const double *box, const int32_t *periodic, int32_t n,
                           const double *r, int32_t *ns, int32_t *head, int32_t *list, int32_t *coords,
                           int32_t *neighbor_ids, int32_t max_bins);
void ora_geom_pair_force(int32_t law, double eps, double rcut_scale, int64_t n, const double *r2, const double *si,
                         const double *sj, double *f0, int32_t *inside);
/* the Lennard-Jones law (ORA_FORCE_LJ_WCA) with any cutoff, shifted or not */
void ora_geom_lj_force(double eps, double rcut_scale, int32_t shifted, int64_t n, const double *r2, const double *si,
                       const double *sj, double *f0, int32_t *inside);
/* the soft-core cubic well (ORA_FORCE_SC) with its well parameters */
void ora_geom_sc_force(double eps_core, double eps_well, double well_sigma, double rcut_scale, int32_t shifted,
                       int64_t n, const double *r2, const double *si, const double *sj, double *f0, int32_t *inside);

/* RNG access for golden-vector checks */
void ora_rng_seed(void *h, uint32_t seed);
double ora_rng_close_open(void *h);
double ora_rng_open_open(void *h);
double ora_rng_uniform(void *h);
double ora_rng_normal(void *h);
void ora_rng_on_dsphere(void *h, int32_t dim, double *out);

#ifdef __cplusplus
}
#endif
#endif
