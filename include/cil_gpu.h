/* cil_gpu.h — C ABI of the GB300 (sm_103a) cell-colony step library, libcilgpu.so.
 *
 * Drop-in boundary for the reference's step loop (KokoroSinx/cil_cuda). The reference
 * plugs its integrator in through `typedef void(*MDIntegrator)(int& ts); extern
 * MDIntegrator mdStep;` (MD.cuh:450-452), chosen in readMD (Input.cpp:524-546) and called
 * GTS times per frame (CIL.cu:1106). A host wrapper `gpuEuler(int& ts)` registered there
 * calls cil_step(); frames cross to the host through cil_download() only. Host arrays keep
 * the reference CellColony layout (pos/vel/frc[cell][elem][dim], sigmaCore[cell][elem],
 * cellT0/cellTSwitch[cell]; Colony.hpp:88-123, Colony.cpp:193-313).
 *
 * Plain C types only: no exceptions, no C++ or torch types cross this boundary. One host
 * thread per handle; one CUDA stream per handle; handles are independent.
 */
#ifndef CIL_GPU_H
#define CIL_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference reports failures through run_assert -> std::runtime_error
 * -> exit(1) (Utils.hpp:99-109, CIL.cuh:365-381); a host wrapper maps any non-OK status
 * to run_assert(false, cil_last_error(...)). */
typedef enum cil_status {
  CIL_OK = 0,
  CIL_ERR_CONFIG = 1,     /* invalid parameters or call order */
  CIL_ERR_CUDA = 2,       /* a CUDA runtime call failed */
  CIL_ERR_CAPACITY = 3,   /* more cells than the reserved capacity (division) or host arrays too small */
  CIL_ERR_NAN = 4,        /* non-finite force or position */
  CIL_ERR_OUT_OF_BOX = 5, /* an element left the box along a non-periodic axis (checkPositions, CIL.cu:945-966) */
  CIL_ERR_TIMEOUT = 6,    /* a bounded device wait gave up */
  CIL_ERR_STATE = 7,      /* handle not ready (e.g. step before upload) */
  CIL_ERR_IO = 8          /* a file could not be written (frame output, cil_gsd.h) */
} cil_status;

/* Pair-force laws (the reference's PairForceParams family, MD.cuh:23-344, with the
 * benchmark workloads' forms: WCA, the (1 - r/rc)^2 soft core, E h^1.5 Hertz; and the
 * reference's own soft-core cubic well). Force on element i from j is f0(r) * (r_j - r_i). */
enum {
  CIL_FORCE_LJ_WCA = 0,   /* LJParams (MD.cuh:47-129): eps_ij = 24 eps, rc^2 = rcut_scale^2 sigma_ij^2
                             (rcut_scale 2^(1/6): WCA; larger: the attractive tail, the reference's
                             ATTRACTION ON with RCUT = rcut_scale); with force_shifted, minus
                             f0(rc) sqrt(rc^2 / r^2) (SHIFT FORCE, OPT::FORCE_SHIFTED) */
  CIL_FORCE_SOFTCORE = 1, /* F = eps (1 - r/rc)^2, rc = rcut_scale sigma_ij */
  CIL_FORCE_HERTZ = 2,    /* F = E delta^1.5, delta = sigma_ij - r */
  CIL_FORCE_SC = 3        /* SCParams (MD.cuh:134-232), one species: y = r - sigma_ij, xi = well_sigma;
                             f0 = -(E0 + Em) t'(-y, xi) / r for -xi <= y < 0, Em t'(y, xi) / r for
                             0 <= y < xi, t'(y, xi) = 6 y (xi - y) / xi^3, E0 = epsilon,
                             Em = well_epsilon; acting for rcut_scale^2 (sigma_ij - xi)^2 < r^2 <=
                             rcut_scale^2 (sigma_ij + xi)^2 (the reference's rc2 is 1); with
                             force_shifted, minus f0(rc) sqrt(rc^2 / r^2) (OPT::FORCE_SHIFTED) */
};

/* Intra-cell bond of the two-element cells (cil_colony_params.intra_law). */
enum {
  CIL_INTRA_SPRING = 0, /* linear spring kappa (r - l) with the rest length growing over the cycle */
  CIL_INTRA_FENE = 1    /* the reference's FENE / push bond, and with divide its crawling/dividing cells */
};

/* Arithmetic of the pair forces. */
enum {
  CIL_PREC_FP64 = 0, /* everything in FP64 */
  CIL_PREC_MIXED = 1 /* FP32 pair forces from bin-origin-relative displacements; FP64 positions,
                        wrap, integration and daughter placement */
};

/* Random streams. */
enum {
  CIL_RNG_PHILOX = 0, /* device Philox4x32-10 keyed by (seed, step, element/cell, purpose) */
  CIL_RNG_DSFMT = 1   /* oracle mode: host dSFMT-19937 stream in the reference's draw order
                         (Random.hpp, CIL.cu:369-455, 627-649, 793-818), uploaded each step */
};

/* Per-colony model parameters (one species of 2-element cells). Times in simulation units. */
typedef struct cil_colony_params {
  int32_t dim;            /* 2 or 3; must equal cil_config.dim */
  int32_t force_law;      /* CIL_FORCE_*; must equal cil_config.force_law */
  int32_t noise_per_cell; /* 0: independent noise per element component; 1: per cell (reference) */
  int32_t divide;         /* 1: linear growth of the rest length and division */
  double box[3];          /* box lengths */
  int32_t periodic[3];    /* 1 = periodic axis */
  int32_t nwalls;         /* 0..2 one-sided flat Hertz walls normal to the last axis */
  int32_t wall_dir[2];    /* +1 keeps elements at larger coordinates, -1 at smaller */
  double wall_pos[2];
  double wall_E;
  double epsilon;         /* LJ eps / soft-core eps / Hertz E */
  double rcut_scale;      /* cutoff / sigma_ij (WCA: 2^(1/6), soft-core and Hertz: 1) */
  double zeta[2];         /* friction of back/front element; mobility 1/zeta */
  double motility[2];     /* back element -m0 n, front +m1 n, n = back->front unit axis */
  double kappa;           /* linear intra-cell spring constant */
  double rest0;           /* spring rest length at birth */
  double rest1;           /* spring rest length at division */
  double noise_D;         /* passive diffusion constant (noise sqrt(2D/dt) zeta per component) */
  double dt;
  double div_tau_mu;      /* division time ~ N(mu, sigma) */
  double div_tau_sigma;
  double apop_rate;       /* apoptosis rate per unit time */
  double well_epsilon;    /* CIL_FORCE_SC: well depth Em (other laws: unused) */
  double well_sigma;      /* CIL_FORCE_SC: well width xi, absolute (other laws: unused) */
  int32_t force_shifted;  /* CIL_FORCE_SC and CIL_FORCE_LJ_WCA: 1 = the reference's shifted force */
  int32_t intra_law;      /* CIL_INTRA_SPRING (0) or CIL_INTRA_FENE (1) */
  /* CIL_INTRA_FENE: the reference's bond for a crawling cell (binaryCellForce, MD.cu:525-598):
   * below spring_ratio * r2max the push spring kappa_push |r^2 - r2max spring_ratio|
   * (MD.cu:263-265), above it the FENE law -kappa / (1 - ((r^2 - r2max ratio) /
   * (r2max (1 - ratio)))^2) (MD.cu:255-257), acting twice along r_front - r_back, with
   * r2max = max(fene_rmax^2, the larger element diameter) (MD.cu:547-548); motility m_j along the
   * axis, scaled by rss / r without contact inhibition (cil = 0; rss from Input.cpp:139-144).
   * kappa, rest0, rest1 are unused; with divide, the crawling/dividing cells below. */
  int32_t cil;            /* CIL_INTRA_FENE: the species' CIL flag */
  double fene_kappa;      /* KAPPA_PULL */
  double fene_kappa_push; /* KAPPA_PUSH */
  double fene_spring_ratio; /* SPRING_RATIO, in [0, 1) */
  double fene_rmax;       /* RMAX */
  /* CIL_INTRA_FENE with divide = 1: the reference's crawling/dividing cells (calculDivisions,
   * CIL.cu:369-455; oracle-mode draws, FP64 or mixed, no Verlet skin). A crawling cell whose
   * time ends starts dividing (time += N(div_tau_mu, div_tau_sigma) / dt); a dividing cell whose
   * elements are div_rmin apart (or, with div_rmin_ratio != 0, whose r^2 reaches
   * div_rmin_ratio x its back diameter) divides: binaryCellDivision at radius div_r0, both cells
   * crawling, born now, the daughter's time now + N(mig_tau_mu, mig_tau_sigma) / dt and the
   * mother's own time plus another such span, diameters reset to sigma_core; one that does
   * not get there by its time fails (binaryCellDivisionFail: the back element to the centre,
   * both reoriented at div_r0; crawling; time += a migration span). While dividing, the bond uses
   * RMAX_DIVISION and the growth activity -k0 FENE(r2max, Rmin^2) + k1 + k2 r^4 (MD.cu:545-567). */
  double fene_rmax_division; /* RMAX_DIVISION (0: RMAX) */
  double growth_k0[2], growth_k1[2], growth_k2[2]; /* GROWTHK0/1/2 of the two elements */
  double div_r0;          /* DIVISION.R0 */
  double div_rmin;        /* DIVISION.Rmin */
  double div_rmin_ratio;  /* DIVISION.Rmin_RATIO (0: Rmin decides) */
  double mig_tau_mu, mig_tau_sigma; /* TAU_MIGRATION */
  double sigma_core[2];   /* SIGMA_CORE of the two elements (what a division resets to) */
  /* CIL_INTRA_FENE in 2D: the bond's active noise (NOISE_ACTIVE of StochasticHeun, Input.cpp:99-111,
   * CIL.cu:803-815; binaryCellForce, MD.cu:573-578): per cell and force evaluation a radial and an
   * angular normal of amplitude sqrt(2 D) / sqrt(dt), drawn after the passive noise (oracle-mode
   * draws, no Verlet skin); the bond term gains rnd_d r_ij,d with rnd = (Wr r_ij,x / r - Wt r_ij,y,
   * Wr r_ij,y / r + Wt r_ij,x) / 2 */
  double noise_radial;    /* NOISE.RADIAL (D_r) */
  double noise_angular;   /* NOISE.ANGULAR (D_a) */
  /* crawling/dividing cells: DIVISION.SWELLING, each step a dividing cell's diameters below the
   * larger SIGMA_CORE grow by (max - sigma) / (tswitch - ts) (updateDiameters, CIL.cu:970-991) */
  int32_t div_swelling;
  int32_t pad_swell;
} cil_colony_params;

typedef struct cil_config {
  int32_t dim;
  int32_t force_law;
  int32_t precision;      /* CIL_PREC_* */
  int32_t rng_mode;       /* CIL_RNG_* */
  uint64_t seed;          /* dSFMT seed (low 32 bits, Random::init) or Philox key */
  int32_t num_colonies;
  int32_t device;         /* CUDA device ordinal */
  double bin_width;       /* 0: cutoff of the largest element (+ skin); else at least this */
  double skin;            /* Verlet skin of the binned structure (0 = rebuild every step) */
  int32_t block_size;     /* threads per block of the force kernels: 0 or 256; in skin mode the
                           * list force kernel takes 128 (the default there), 256 or 512
                           * (cells per block) */
  int32_t flags;          /* CIL_FLAG_* bits */
  /* Verlet-list force kernel (skin mode: one thread per cell, each warp's list entries taken as
   * one flattened range): chunks of 32 entries in flight per warp (0 = 4; 1, 2) and CTAs per SM
   * of 256 threads it is compiled for (0 = 3; 4). Supported pairs: (4, 3), (2, 3), (1, 3),
   * (1, 4). cil_cuda_gb300/autotune.py picks them. */
  int32_t staging;
  int32_t occupancy;
  int32_t integrator;     /* CIL_INTEGRATOR_*: 0 = Euler */
  /* Philox mode: colony c draws from random stream rng_stream_base + c. The draws of a colony
   * depend only on the seed, its stream and its own (colony-local) cell indices, so a colony
   * run alone with rng_stream_base = c draws what it draws as colony c of a batch. */
  int32_t rng_stream_base;
} cil_config;

/* cil_config.integrator. EULER is the reference's Euler (CIL.cu:1013-1020). HEUN is its
 * StochasticHeun (CIL.cu:1028-1050): per step, two half steps dt/2, each with a force
 * evaluation and its own noise draw (forces -> x += (dt/2) F / zeta, twice), then the step
 * counter, division and apoptosis. The reference's predictor copy (pos0) is never read and
 * its Heun never updates the velocities; here the velocity of a Heun step is the mean of the
 * two half steps' F / zeta, i.e. the step's displacement over dt. */
#define CIL_INTEGRATOR_EULER 0
#define CIL_INTEGRATOR_HEUN 1

/* cil_config.flags: run every step as individual launches (no CUDA graphs). By default, in
 * Philox mode, steps whose launches depend on nothing the host decides (no slot re-sort, no
 * FP64 re-anchoring) are captured once as CUDA graphs of two steps or of one step (per buffer
 * parity, and with or without the velocity output of a call's last step) and replayed, so a
 * one-step cil_step call (the reference's mdStep) launches one graph; the kernels read the
 * step index from device memory. cil_timings then reports phase times for the individually
 * launched steps only. */
#define CIL_FLAG_NO_GRAPH 1

/* cil_config.flags: cil_step returns once its launches and an asynchronous copy of the colony
 * counters are enqueued, and reports the status of the previous call (whose copy it waits
 * for), so that the host queues the next step while the GPU runs this one. The reference's
 * mdStep returns nothing; its run_assert stops the run. Errors surface one call late; calls
 * that read state (cil_download, cil_observables, ...) synchronise as always. cil_timings is
 * not updated by such calls. */
#define CIL_FLAG_DEFERRED_STATUS 2

/* cil_config.flags, skin mode with graphs: the list-rebuild kernels of a replayed step sit in
 * a conditional graph node that runs only on steps where some colony rebuilds, instead of being
 * launched every step and returning at once when no colony rebuilds (the default). The results
 * are the same either way; on one GB300 the node made steps 0.5-2 % slower than the early
 * returns, so it is off unless asked for. */
#define CIL_FLAG_REBUILD_NODE 4

/* Host view of one colony in the reference layout. */
typedef struct cil_colony_view {
  int32_t ncells;   /* upload: cells in the arrays; download: cells on the device */
  int32_t capacity; /* download: cells the host arrays can hold */
  int32_t ts;       /* time step of the state */
  int32_t pad;
  double *pos;      /* [cell][2][dim] */
  double *sigma;    /* [cell][2] element diameters (sigmaCore) */
  double *vel;      /* [cell][2][dim], download only, may be NULL */
  int32_t *t0;      /* [cell] birth step (cellT0) */
  int32_t *tswitch; /* [cell] division step (cellTSwitch) */
  int32_t *cell_state; /* [cell] CellState (0 dividing, 1 crawling, 2 undefined); may be NULL
                          (upload: undefined; download: not copied); used by the crawling/
                          dividing cells of CIL_INTRA_FENE with divide */
} cil_colony_view;

/* Observables reduced on the device (per colony). */
typedef struct cil_obs {
  int32_t ncells;
  int32_t pad;
  double mean_area;   /* mean over cells of sum_j pi (sigma_j/2)^2 */
  double msd;         /* mean squared unwrapped centre-of-mass displacement since cil_obs_reset */
  double vacf;        /* <v_c(t).v_c(0)> / <|v_c(0)|^2> of the cell velocity */
  int64_t ndiv_total; /* divisions since creation */
  int64_t napo_total; /* apoptoses since creation */
} cil_obs;

typedef struct cil_handle cil_handle;

/* Creates a handle for num_colonies colonies. params[c] and cap_cells[c] per colony.
 * Replaces the reference's initialize() step-loop setup (CIL.cuh:332-393) for the GPU. */
cil_status cil_create(const cil_config *cfg, const cil_colony_params *params,
                      const int32_t *cap_cells, cil_handle **out);
void cil_destroy(cil_handle *h);

/* Copies one colony to the device (all colonies must be uploaded before cil_step).
 * Replaces the host-resident colony state used by Euler (CIL.cu:1013-1020). */
cil_status cil_upload(cil_handle *h, int32_t colony, const cil_colony_view *view);

/* Copies one colony to the host at a frame boundary (outputFrame, OutputWriter.cpp:708).
 * CIL_ERR_CAPACITY if view->capacity is too small (view->ncells is set to the need). After a step
 * that failed on a colony's counters (CIL_ERR_NAN, CIL_ERR_OUT_OF_BOX, CIL_ERR_CAPACITY) the view
 * is still filled with the state that step left, which never holds more cells than the colony's
 * capacity, and the call returns that status again. */
cil_status cil_download(cil_handle *h, int32_t colony, cil_colony_view *view);

/* Advances every colony by nsteps Euler steps (MDIntegrator mdStep, MD.cuh:450-458;
 * Euler CIL.cu:1013-1020). *ts (may be NULL) receives the step counter afterwards. */
cil_status cil_step(cil_handle *h, int32_t nsteps, int64_t *ts);

/* Computes the forces of the current state without integrating (calculForcesPressure,
 * CIL.cu:999-1007), with the noise the next step will draw, and copies them to frc
 * [cell][2][dim]; the run is left unchanged (the host stream of the dSFMT mode is put back).
 * For parity checks and frame output. */
cil_status cil_forces(cil_handle *h, int32_t colony, double *frc);

/* Bin structure of the current positions (LinkList::populate, Container.cpp:58-79;
 * Utils.hpp:872-1001) for parity checks: ns[3] bins per axis, bin_start[nbins+1] offsets
 * into elems[2*ncells] (element ids 2*cell+elem, ascending within a bin). Returns
 * CIL_ERR_CAPACITY if max_bins is too small. */
cil_status cil_bins(cil_handle *h, int32_t colony, int32_t *ns, int32_t *bin_start,
                    int32_t *elems, int32_t max_bins);

/* Observables (offline analysis in the reference: cilJintaoTools.py:97-125,
 * simulationtools.py:602-607). cil_obs_reset sets the MSD/VACF origin. */
cil_status cil_obs_reset(cil_handle *h, int32_t colony);
cil_status cil_observables(cil_handle *h, int32_t colony, cil_obs *out);

/* Verlet-skin mode (cil_config.skin > 0, mixed precision only): the bins and per-element
 * Verlet lists (cutoff rc_ij + skin) are rebuilt only when an element has moved more than
 * skin/2 since the last build, when the cadence `interval` (steps, 0 = none) expires, or
 * when too many elements were created by divisions; results agree with the per-step
 * rebuild of the reference (CIL.cu:180) to FP32 summation order. No counterpart in the
 * reference, which rebuilds its link list every step. */
typedef struct cil_skin_info {
  double skin;           /* skin of the current lists */
  int32_t interval;      /* cadence in steps (0: guard only) */
  int32_t nrebuild;      /* list rebuilds so far */
  int32_t ntrip;         /* of which requested by the displacement guard */
  int32_t last_interval; /* steps between the last two rebuilds */
  int32_t nfresh;        /* elements created or moved by divisions since the last rebuild */
  int32_t list_overflow; /* elements whose list exceeded the capacity at the last build */
  int64_t npairs;        /* list entries at the last build */
  double max_disp;       /* largest displacement from the list reference in the last step */
} cil_skin_info;

cil_status cil_skin_stats(cil_handle *h, int32_t colony, cil_skin_info *out);
/* Sets the skin (<= cil_config.skin, which sizes the bins) and cadence of one colony; they
 * take effect at its next list rebuild, which this call requests. */
cil_status cil_set_skin(cil_handle *h, int32_t colony, double skin, int32_t interval);

/* Learned skin scheduler (skin mode only) — no counterpart in the reference.
 *
 * A 12 -> 64 -> 64 -> 2 SiLU multilayer perceptron (FP32) evaluated on the device at every
 * list rebuild of a colony, from 12 features the step maintains per colony (cells, bin
 * occupancy, step displacements, division/apoptosis rates, current skin, steps since the
 * last rebuild, displacement at the rebuild, guard-trip share, fresh elements; see
 * cil_sched_info). Output y0 sets the skin skin_min + (cil_config.skin - skin_min) *
 * sigmoid(y0), output y1 the cadence round(interval_scale * softplus(y1)) steps when
 * use_interval != 0. The displacement guard stays on, so the physics is unchanged: only the
 * cost of a step depends on the choice. params: host, cil_mlp_num_params() floats in the
 * layout W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]; NULL switches it off (the
 * skin and cadence then stay where they are). */
#define CIL_SCHED_FEATURES 12
cil_status cil_set_scheduler(cil_handle *h, const float *params, double skin_min, double interval_scale,
                             int32_t use_interval);

typedef struct cil_sched_info {
  /* input of the last decision: 0 log(cells)/14, 1 mean home-bin occupancy/10, 2 max bin
   * occupancy/20, 3 mean and 4 max step displacement (log10(d)/4 + 1), 5 divisions and
   * 6 apoptoses per cell per step x1e4, 7 skin, 8 log(1 + steps since the last rebuild)/5,
   * 9 largest displacement from the list reference / (skin/2), 10 share of guard-triggered
   * rebuilds, 11 fresh elements / elements x10 */
  float features[CIL_SCHED_FEATURES];
  float div_rate, apo_rate, trip_share;
  int32_t nsched; /* scheduler decisions so far */
} cil_sched_info;

cil_status cil_sched_state(cil_handle *h, int32_t colony, cil_sched_info *out);

/* Training kernels of the scheduler network (all pointers device memory, FP32, run on the
 * current device's default stream):
 *   cil_mlp_forward  Y[n][2] = net(X[n][12])
 *   cil_mlp_grad     loss = mean over samples and outputs of w[o] * (y - T)^2 and its
 *                    gradient (deterministic: block partials summed in a fixed order);
 *                    workspace of cil_mlp_workspace_floats(n) floats
 *   cil_mlp_adam     one Adam step (beta1 0.9, beta2 0.999, eps 1e-8), step count t >= 1 */
int32_t cil_mlp_num_params(void);
int64_t cil_mlp_workspace_floats(int32_t n);
cil_status cil_mlp_forward(const float *params, const float *X, int32_t n, float *Y);
cil_status cil_mlp_grad(const float *params, const float *X, const float *T, const float *out_weights,
                        int32_t n, float *workspace, float *grad, float *loss);
cil_status cil_mlp_adam(float *params, const float *grad, float *m, float *v, int32_t t, float lr);

/* Device time of the last cil_step, milliseconds, measured with CUDA events on the
 * handle's stream: per phase summed over its steps (rebuild, forces, events), the whole
 * call from the first launch to the last (total, including any idle gaps), and the number
 * of kernels it launched. Any pointer may be NULL. */
cil_status cil_timings(cil_handle *h, double *rebuild_ms, double *force_ms, double *events_ms,
                       double *total_ms, int64_t *launches);

/* Steps of the last cil_step call that ran inside CUDA graphs, and graphs captured so far. */
cil_status cil_graph_info(cil_handle *h, int64_t *graph_steps, int64_t *graphs_captured);

/* The oracle-mode host random stream on its own (no device needed): n draws of `kind`
 * from a fresh stream seeded with `seed` through the reference's Random:: functions
 * (Random.hpp:9-118): 0 dsfmt close_open, 1 open_open, 2 uniform, 3 normal (Leva),
 * 4 onDSphere in 2D (2 values per draw), 5 onDSphere in 3D (3 values per draw). */
cil_status cil_host_rng_draw(uint32_t seed, int32_t kind, int64_t n, double *out);

/* Element binning without any device allocation — no counterpart in the reference.
 *
 * For callers that cannot allocate device memory: a host framework that owns a budgeted
 * device pool and forbids outside cudaMalloc, or a real-time loop that cannot risk an
 * allocation's latency or its failure mid-run. Same result as cil_bins for the same
 * positions and width (bins numbered as the reference's link list, ascending element ids
 * inside each bin, in time linear in n_elems whatever the bins' occupancy), but the caller
 * passes every buffer:
 *   pos        device, [n_elems][dim] FP64 positions inside [0, box)
 *   box        host, dim lengths;  width: minimum bin width
 *   ns         host out, bins per axis (1 on unused axes)
 *   bin_start  device out, nbins + 1 offsets into elems
 *   elems      device out, n_elems element indices sorted by bin
 *   stream     cudaStream_t to run on (NULL = default stream)
 * Scratch lives in fixed device arrays inside the library: at most 1,048,576 elements and
 * 1,048,576 bins per call (about 14.7 MB held on every GPU that loads the library, until
 * exit). Larger inputs, more than 1,048,576 bins along one axis, or nbins > max_bins return
 * CIL_ERR_CAPACITY before any work is enqueued. The first call on a device resolves the
 * scratch addresses (cudaGetSymbolAddress with that device current); make it before any
 * stream capture. All calls share the scratch and each call overwrites what the last one
 * left: calls that overlap on the GPU race, so serialise them. */
cil_status cil_bin_elements_noalloc(const double *pos, int32_t n_elems, int32_t dim,
                                    const double *box, double width, int32_t *ns,
                                    int32_t *bin_start, int32_t *elems, int32_t max_bins,
                                    void *stream);

/* Last error message of the handle (empty if none). */
void cil_last_error(const cil_handle *h, char *buf, size_t len);

/* Pins (page-locks) a host range for DMA with the GPUs (cudaHostRegister), so that cil_upload
 * and cil_download from and into it run as direct copies instead of through a staging buffer
 * (the reference's CellColony arrays, for instance, registered once after they are sized).
 * cil_host_unregister releases it; ranges must not overlap a registered range. No counterpart in
 * the reference. */
cil_status cil_host_register(void *ptr, size_t bytes);
cil_status cil_host_unregister(void *ptr);

/* Library version string. */
const char *cil_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CIL_GPU_H */
