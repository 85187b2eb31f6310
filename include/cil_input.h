/*
 * cil_input.h - the reference's JSON run description (Input.cpp, CIL.cuh:332-393) read into
 * the step library's configuration, and its initial configuration (INIT, Input.cpp:591-761;
 * initializeCellStatus, CIL.cuh:253-330) built on the host for cil_upload.
 *
 * What is read, and what it becomes:
 *   UNITS       LENGTH, MOTILITY, FRICTION must be 1: the derived units need the reference's
 *               Units class, which is not part of its tree.
 *   MD          DIM, BOX, PBC, GTS, FRAMES; DT (MANUAL); INTEGRATOR EULER (no noise),
 *               STOCHASTIC_EULER (passive noise), STOCHASTIC_HEUN (CIL_INTEGRATOR_HEUN;
 *               its active RADIAL/ANGULAR noise must be 0) or DPD (single-element cells:
 *               CIL_CYCLE_DPD with INTEGRATOR.DPD DISSAMCEL / DISDIFCEL / DISBG, KBT and the
 *               species' MASS). AUTOSCALE is refused with a message.
 *   RUNTIME     RNG.SEED (<= 0: the current time, as Random::init(time(NULL))).
 *   OUTPUT      DIR, NAME, FORMAT (GSD is served by cil_gsd.h; H5 by the frame file <NAME>.h5,
 *               cil_h5_frames_* below, and the final-state file <NAME>.Last.h5,
 *               cil_h5_write_state).
 *   SPECIES     one species. Two-element cells (cil_gpu.h): NELEM, NAMES, MOTILITY, FRICTION,
 *               NOISE.PASSIVE, the element diameters of the selected pair force, FENE RMAX /
 *               KAPPA_PULL (for the steady-state length rss that INIT RANDOM uses),
 *               DIVISION (ENABLED, CONST_FORCE, TAU_DIVISION, TAU_MIGRATION), APOPTOSIS
 *               (ENABLED, APOP_RATE). Single-element cells, the shipped runs (the cell-cycle
 *               model, cil_cycle.h): PAIRFORCES.HZ (ELASTIC_MODULUS, POISSON_RATIO, SIGMA_CORE,
 *               ADHESION_CONSTANT), MOTILITY, FRICTION, P_FRICTION, P_FRICTION_BETA, NOISE,
 *               DIVISION (TAU_DIVISION, V1, CYCLE_*), APOPTOSIS (the Euler step's cycle-pressure
 *               law, or the DPD step's pressure-time law); MD.OSMOTIC_PRESSURE and MD.DRAIN;
 *               GPU.PRECISION FP64 (default) or MIXED (cil_cycle_params.precision 1).
 *   INTERACTIONS PAIRFORCES.SELECT "LJ" with ATTRACTION OFF is the reference's own law
 *               (WCA, cil_gpu.h CIL_FORCE_LJ_WCA, epsilon from the species' LJ EPSILON).
 *   GPU         (optional block, this library's own): PRECISION "FP64" | "MIXED", RNG
 *               "PHILOX" | "DSFMT", SKIN, SCHEDULER, CAPACITY, NOISE_PER_CELL, and the model
 *               parameters the reference's JSON has no key for: FORCE_LAW ("LJ_WCA",
 *               "SOFTCORE", "HERTZ") with EPSILON and RCUT_SCALE (required for SC/HZ runs,
 *               whose reference laws differ from this library's), SPRING {KAPPA, REST0, REST1}
 *               (the linear intra-cell spring; required: the reference's FENE law differs),
 *               WALLS {E, POS[], DIR[]}.
 *   INIT        per species: RANDOM (NUMBER) with the reference's draw sequence, so that the
 *               positions equal the reference's bit for bit for the same seed; JSON (element
 *               positions); H5 (Input.cpp:610-726): LOCATION [file, positions dataset] or ALL
 *               [file, R, Vel, State, Theta, RHO, SigmaCore] with an optional RANGE of cells,
 *               read from a final-state file (the reference's <NAME>.Last.h5) by this
 *               library's own HDF5 reader; ALL replaces the drawn cell status by the file's
 *               (positions, velocities, phases, activities, diameters); the file path is
 *               taken relative to the working directory, as the reference opens it.
 *
 * Errors carry the JSON key that failed, as json_parser's std::domain_error messages do
 * (JsonParser.hpp:13-135).
 */
#ifndef CIL_INPUT_H
#define CIL_INPUT_H

#include <stddef.h>
#include <stdint.h>

#include "cil_cycle.h"
#include "cil_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cil_input cil_input;

/* Run-level settings that are not part of cil_config / cil_colony_params. */
typedef struct cil_run_info {
  int32_t gts;                 /* MD.GTS: steps per frame */
  int32_t frames;              /* MD.FRAMES */
  int32_t output_gsd;          /* OUTPUT.FORMAT lists "GSD" */
  int32_t output_h5;           /* OUTPUT.FORMAT lists "H5" (not served by this library) */
  int32_t ncells;              /* cells of the initial configuration */
  int32_t capacity;            /* GPU.CAPACITY, else 4 x ncells + 64 */
  int32_t use_scheduler;       /* GPU.SCHEDULER */
  int32_t seed;                /* RUNTIME.RNG.SEED as used (time-based when <= 0 in the file) */
  char output_dir[256];        /* OUTPUT.DIR */
  char output_name[256];       /* OUTPUT.NAME */
  char cell_name[64];          /* SPECIES.DEFINE[0] */
  char elem_names[2][64];      /* SPECIES.<cell>.NAMES */
} cil_run_info;

/* Parses a JSON document (is_path != 0: `text` is a file name) and reads the run
 * description. On failure *out is still set (unless it is NULL) so that the message can be
 * read with cil_input_last_error; free it with cil_input_free. */
cil_status cil_input_load(const char *text, int32_t is_path, cil_input **out);

/* The configuration for cil_create (num_colonies = 1) and the colony's parameters. */
cil_status cil_input_config(const cil_input *in, cil_config *cfg, cil_colony_params *params, cil_run_info *run);

/* Builds the initial configuration on the host in the reference layout: pos [cell][2][dim],
 * sigma [cell][2] (the species' element diameters), t0 = 0 and tswitch from the reference's
 * cell-status draws (initializeCellStatus), ts = 0. The view's arrays must hold
 * run.ncells cells (view->capacity); view->ncells receives the count. INIT RANDOM consumes
 * the reference's Random stream in the reference's order: positions, cell status, then
 * positions again (initialize() reads INIT twice, CIL.cuh:374-378, and the second read wins). */
cil_status cil_input_initial_state(const cil_input *in, cil_colony_view *view);

/* Elements per cell of the described species: 2 (cil_input_config / cil_input_initial_state,
 * the two-element step) or 1 (cil_input_cycle_config / cil_input_cycle_initial_state, the
 * cell-cycle model); 0 if the description did not load. */
int32_t cil_input_elements(const cil_input *in);

/* The cell-cycle model's parameters of a single-element run. */
cil_status cil_input_cycle_config(const cil_input *in, cil_cycle_params *params, cil_run_info *run);

/* Initial state of a single-element run for cil_cycle_upload: positions (INIT RANDOM with the
 * reference's draws, or JSON), sigma = sigma_t = SIGMA_CORE, rho = 1, and theta and the cycle
 * speed from the reference's cell-status draws (theta = U[0, 1), angvel = 1 / max(Nint(N(tau_div)
 * / dt), 1)), all on the reference's Random stream in its order. pos, sigma, sigma_t, theta,
 * rho and angvel must be given. */
cil_status cil_input_cycle_initial_state(const cil_input *in, cil_cycle_view *view);

/* Message of the last failure (empty if none). */
void cil_input_last_error(const cil_input *in, char *buf, size_t len);

void cil_input_free(cil_input *in);

/* ---- HDF5 final-state files, without libhdf5 (the subset libhdf5 writes for the reference's
 * <NAME>.Last.h5: superblock 0, symbol-table groups, contiguous or compact numeric datasets).
 * Errors: cil_h5_last_error (per thread). */

/* Rank and dimensions (up to 8) of a dataset ("R", "/group/R"). */
cil_status cil_h5_shape(const char *path, const char *dataset, int32_t *rank, int64_t dims[8]);
/* The dataset converted to double, row-major; capacity in elements. */
cil_status cil_h5_read(const char *path, const char *dataset, double *out, int64_t capacity);
void cil_h5_last_error(char *buf, size_t len);

/* One colony's final state as outputHDF5Frame writes it with id -1 (OutputWriter.cpp:388-441):
 * datasets R, Vel, F, FD, FR [cell][elem][dim], SigmaCore [cell][elem], RHO, Theta, PR, State,
 * T0 [cell], CpuTime [1], doubles stored as FP32 (SimIO.hpp:73) and integers as int32. NULL
 * arrays are written as zeros. */
typedef struct cil_h5_state {
  int32_t ncells, nelem, dim, pad;
  const double *pos, *vel, *force, *force_dis, *force_ran; /* [cell][elem][dim] */
  const double *sigma;                                     /* [cell][elem] */
  const double *rho, *theta, *pressure;                    /* [cell] */
  const int32_t *state, *t0;                               /* [cell] */
  double cpu_time;
} cil_h5_state;
cil_status cil_h5_write_state(const char *path, const cil_h5_state *s);

/* A numeric attribute of an object ("params", "/snapshots/t_3") as doubles; *n receives its
 * length. */
cil_status cil_h5_attr(const char *path, const char *object, const char *name, double *out, int64_t capacity,
                       int64_t *n);

/* The frame file <NAME>.h5 (initHDF5Output and outputHDF5Frame, OutputWriter.cpp:240-330,
 * 388-441): /params with the attributes dt, L (the box) and Tdump (GTS), then per frame the
 * group /snapshots/t_<frame> with the datasets of cil_h5_write_state and the attribute ts.
 * Frames are appended as written; the file is complete at cil_h5_frames_close. Groups are
 * symbol tables: the reference's groups also track the creation order of their links. */
typedef struct cil_h5_frames cil_h5_frames;
cil_status cil_h5_frames_create(const char *path, int32_t dim, const double *box, double dt, int32_t gts,
                                cil_h5_frames **out);
cil_status cil_h5_frames_write(cil_h5_frames *w, int32_t frame, int32_t ts, const cil_h5_state *s);
cil_status cil_h5_frames_close(cil_h5_frames *w);

#ifdef __cplusplus
}
#endif
#endif /* CIL_INPUT_H */
