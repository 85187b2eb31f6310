/*
 * cil_cycle.h - the reference's single-element cell-cycle model on the GPU: what every
 * shipped configuration runs (PRX_MDCK_2D.json, Match_Puliafito_2D.json,
 * Ecoli_channel_2D.json: NELEM 1, Hertz contacts with adhesion, Euler).
 *
 * One element per cell. Per step, in the reference's order (Euler, CIL.cu:1013-1020, with the
 * force evaluation at the head of the step):
 *   forces and pressures: the cell's motility along its velocity (singleCellForce,
 *     MD.cu:600-646; a cell at rest gets a random direction of length 1e-11 first), passive
 *     noise zeta sqrt(2D/dt) N (CIL.cu:84-97), Hertz contacts with adhesion and the cell
 *     pressure (cellCellForcePressure; its host body is missing from the reference, so the
 *     arithmetic is its device draft, MD.cu:302-366: for r <= sigma_ij, h = sigma_ij - r,
 *     f0 = -h^1.5 / (0.75 ((1-nu^2)/E + (1-nu^2)/E) sqrt(2/sigma_i + 2/sigma_j)) + adhesion A,
 *     A the contact length (2D, Utils.hpp:243-250) or area (3D, Utils.hpp:236-241),
 *     F_i += f0 (r_j - r_i), p_i -= f0 / A (3D: / the element volume));
 *   positions: x += F dt / ((zeta + zeta_p (p/p0)^beta) area(sigma)), v = that / dt
 *     (updateVelocityPositions, CIL.cu:902-939);
 *   ++ts; cell cycle and divisions (calculDivisionsSingle, CIL.cu:469-619): theta, rho and the
 *     target / actual volumes advance by one explicit step, theta >= 1 divides the cell into
 *     two of volume v/2 placed +-dr around it (singleCellDivision, MD.cu:664-700), both with
 *     theta = 0 and new cycle speeds 1 / lognormal(tau_div) (randomTimeSpanLogNormal,
 *     MD.cuh:438-440);
 *   apoptosis (calculApoptosisCyclePressure, CIL.cu:711-738; the reference's other laws are
 *     selectable: PressureTime, CIL.cu:653-676, which its DPD step applies; the constant rate,
 *     CIL.cu:627-649; Cycle, CIL.cu:681-709; CycleExtrude, CIL.cu:749-788).
 *
 * The reference's DPD step (CIL.cu:1054-1066) is the other integrator (CIL_CYCLE_DPD): cells
 * carry a velocity, a mass and three forces (conservative Fc, dissipative Fd, random Fr), and a
 * step is
 *   v += (Fc dt + Fd dt + Fr sqrt(dt)) / (4m); x += v dt           (updateVelocities passes
 *     2m as the mass to updateVel, which divides by twice the mass: CIL.cu:894, Utils.hpp:568-571;
 *     updatePositions, CIL.cu:849-866)
 *   Fc, pressure: motility along v and the Hertz contacts as above; Fd, Fr over the pairs with
 *     r < sigma_a (sigma_a: the diameter of the pair's lower-index cell), w = 1 - r / sigma_a:
 *     Fd_i,d -= gamma w (v_i,d - v_j,d) n_d n_d, Fr_i,d += sqrt(2 gamma kT) sqrt(w) n_d xi_d,
 *     n the unit vector from i to j, one standard normal xi_d per pair and axis shared by the
 *     two cells (cellCellDisRanForce, MD.cu:861-905)
 *   v += (Fc dt + Fd dt + Fr sqrt(dt)) / (4m)
 *   Fd = -gamma_bg v_i - sum over r < sigma_core of gamma (1 - r^2 / sigma_core)(v_i,d - v_j,d)
 *     n_d n_d (calculDisForces, CIL.cu:294-364; cellBackDisForce, MD.cu:846-859;
 *     cellCellDisForce, MD.cu:951-985)
 *   ++ts, cell cycle and divisions (both cells of a division restart at rest with zero forces,
 *     CIL.cu:593-598), apoptosis.
 * cil_cycle_upload evaluates Fc, Fd and Fr once at the uploaded positions and velocities, as
 * the reference does before its first step (CIL.cu:1096). Where the reference's DPD loops are
 * not well defined, this is what they compute with every pair visited once: they never reset
 * the random force (it sums over all steps), apply the background term once per neighbour
 * bin, and let OpenMP threads reset and add to one cell's forces at the same time.
 *
 * Random draws are counter-based (Philox4x32-10 keyed by seed, step, cell index and purpose),
 * so runs are reproducible and independent of the launch configuration; the reference draws
 * from one dSFMT stream inside OpenMP loops, whose order is not reproducible with threads.
 * FP64 (or FP32 contacts, cil_cycle_params.precision). Cells are kept in index order; removals
 * compact stably.
 */
#ifndef CIL_CYCLE_H
#define CIL_CYCLE_H

#include <stddef.h>
#include <stdint.h>

#include "cil_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  CIL_APOP_NONE = 0,
  CIL_APOP_CYCLE_PRESSURE = 1, /* calculApoptosisCyclePressure (Euler, CIL.cu:711-738) */
  CIL_APOP_PRESSURE_TIME = 2,  /* calculApoptosisPressureTime (DPD, CIL.cu:653-676) */
  CIL_APOP_RATE = 3,           /* calculApoptosis (Heun, CIL.cu:627-649): u <= apop_rate dt */
  CIL_APOP_CYCLE = 4,          /* calculApoptosisCycle (CIL.cu:681-709): cells with rho < 1,
                                * u <= apop_rate dt (1 - rho / apop_pressure)^apop_duration
                                * (the reference's loop never advances past a cell with
                                * rho >= 1; such a cell is kept) */
  CIL_APOP_CYCLE_EXTRUDE = 5   /* calculApoptosisCycleExtrude (CIL.cu:749-788): rho < 1 and
                                * u1 <= apop_rate dt, or rho <= 0.1 and
                                * u2 <= extr_rate ((p - apop_pressure) / apop_pressure)^extr_gamma
                                * (extr_rate per step, as the reference uses it) */
};

enum { CIL_CYCLE_EULER = 0, CIL_CYCLE_DPD = 1 };

/* cil_cycle_params.flags. By default a step is captured once as a CUDA graph per
 * configuration of the device buffers it reads and writes (the buffers rotate from step to
 * step) and of the bin grid, and replayed: one launch per step, what small colonies (the
 * shipped runs start from one or two cells) are bound by. */
#define CIL_CYCLE_NO_GRAPH 1

/* Model parameters with the reference's JSON meaning (Input.cpp:6-262; Cell.cuh:236-260
 * defaults). Times in time units; cycle times in units of tau_div_mu as in the JSON. */
typedef struct cil_cycle_params {
  int32_t dim;             /* 2 or 3 */
  int32_t periodic[3];
  double box[3];
  double dt;
  /* element (PAIRFORCES.HZ, MOTILITY, FRICTION, P_FRICTION, P_FRICTION_BETA, NOISE.PASSIVE) */
  double sigma_core;       /* SIGMA_CORE: diameter of a new cell of the initial configuration */
  double E;                /* ELASTIC_MODULUS */
  double nu;               /* POISSON_RATIO */
  double adhesion;         /* ADHESION_CONSTANT */
  double motility;
  double zeta, zeta_p, zeta_p_beta;
  double noise_D;
  /* division and cell cycle (DIVISION block) */
  int32_t divide;
  int32_t apoptosis;       /* CIL_APOP_* */
  double tau_div_mu, tau_div_sigma;  /* TAU_DIVISION */
  double tau_mig_mu, tau_mig_sigma;  /* TAU_MIGRATION */
  double v1;               /* V1 */
  double cycle_tau_r, cycle_tau_v, cycle_tau_p;  /* CYCLE_TAU_R/V/P, units of tau_div_mu */
  double cycle_sigma_min;  /* CYCLE_SIGMA_MIN: v_s = its area (2D) or volume (3D) */
  double cycle_p0;         /* CYCLE_P0 */
  double cycle_beta_vs;    /* CYCLE_BETA_VS */
  double cycle_rho_ratio;  /* CYCLE_RHO_RATIO (default 1) */
  double cycle_r_maxed;    /* CYCLE_R_MAXED (default 1) */
  double cycle_p_shift;    /* CYCLE_P_SHIFT in units of CYCLE_P0 (default 0) */
  double cycle_p_shift_tau;/* CYCLE_P_SHIFT_TAU in units of tau_div_mu (0: no decay term) */
  double osmotic_pressure; /* MD.OSMOTIC_PRESSURE */
  /* apoptosis (APOPTOSIS block) */
  double apop_pressure, apop_duration, apop_rate, extr_gamma;
  int32_t drain;           /* MD.DRAIN: cil_cycle_check_positions removes cells off the box */
  int32_t precision;       /* 0: FP64 throughout (computes what the CPU restatement computes);
                            * 1: FP32 pair arithmetic on the FP64 separations (the contacts; with
                            * DPD also the dissipative and random pair terms, with FP32 normals
                            * from the same counters), FP64 positions, velocities, forces of
                            * motility and noise, and cell state */
  int32_t integrator;      /* CIL_CYCLE_EULER or CIL_CYCLE_DPD (MD.INTEGRATOR.SELECT) */
  int32_t flags;           /* CIL_CYCLE_NO_GRAPH: launch every kernel of every step */
  double mass;             /* MASS (DPD) */
  double kbt;              /* MD.KBT (DPD) */
  double dis_same;         /* DISSAMCEL: acts between the elements of one cell, none here */
  double dis_diff;         /* DISDIFCEL (DPD) */
  double dis_bg;           /* DISBG (DPD) */
  double extr_rate;        /* EXTR_RATE (CIL_APOP_CYCLE_EXTRUDE) */
} cil_cycle_params;

/* Per-cell state in index order. Arrays may be NULL where not wanted. */
typedef struct cil_cycle_view {
  int32_t ncells;    /* upload: cells given; download: cells on the device */
  int32_t capacity;  /* download: cells the arrays can hold */
  int32_t ts;
  int32_t pad;
  double *pos;       /* [cell][dim] */
  double *vel;       /* [cell][dim]; upload: NULL for cells at rest */
  double *sigma;     /* sigmaCore */
  double *sigma_t;   /* sigmaCoreT, the target diameter */
  double *theta;     /* cellTTheta, cycle phase */
  double *rho;       /* cellTRho, cycle activity */
  double *angvel;    /* cellAngVel, cycle speed per step */
  double *pressure;  /* pressure at the cells' positions (download: evaluated at the current
                      * state, as the reference's step leaves it for output) */
  int32_t *tpressure;/* cellTPressure */
  /* download only (NULL where not wanted): the forces the reference writes to its final-state
   * file (F, FD, FR): Euler, the force at the current state; DPD, Fc, Fd and Fr */
  double *force, *force_dis, *force_ran;  /* [cell][dim] */
  int32_t *t0;       /* cellT0, the step of the cell's birth (download only) */
  int32_t pad2;
} cil_cycle_view;

typedef struct cil_cycle cil_cycle;

cil_status cil_cycle_create(const cil_cycle_params *p, int32_t capacity, uint64_t seed, int32_t device,
                            cil_cycle **out);
void cil_cycle_destroy(cil_cycle *h);

/* Sets the colony. Arrays NULL take the reference's initial cell status (initializeCellStatus,
 * CIL.cuh:253-330) drawn from the counter-based stream: sigma = sigma_t = sigma_core,
 * rho = 1, theta = U[0, 1), angvel = 1 / max(Nint(N(tau_div) / dt), 1), tpressure = 0. */
cil_status cil_cycle_upload(cil_cycle *h, const cil_cycle_view *v);

/* Advances nsteps steps; *ts (may be NULL) receives the step counter. */
cil_status cil_cycle_step(cil_cycle *h, int32_t nsteps, int64_t *ts);

/* checkPositions (CIL.cu:945-966) at a frame boundary: with drain, cells outside the box along
 * a non-periodic axis are removed; without, such a cell is CIL_ERR_OUT_OF_BOX. */
cil_status cil_cycle_check_positions(cil_cycle *h);

cil_status cil_cycle_download(cil_cycle *h, cil_cycle_view *v);

/* Device time of the last cil_cycle_step call (ms) and its kernel launches. */
cil_status cil_cycle_timings(cil_cycle *h, double *total_ms, int64_t *launches);

void cil_cycle_last_error(const cil_cycle *h, char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* CIL_CYCLE_H */
