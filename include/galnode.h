/*
 * galnode.h -- C ABI of the GB300 node evolver.
 *
 * This library replaces the per-node ODE evolution step of Galacticus, the
 * `mergerTreeNodeEvolver` class with its default `standard` implementation
 * (source/merger_trees/node_evolver/_class.F90:41-57, method `evolve`;
 * implementation source/merger_trees/node_evolver/standard.F90:385-755).
 * The reference serialises one node's evolvable properties into an FP64
 * vector and integrates them with GSL's embedded Cash-Karp stepper through a
 * scaled error controller (source/external/gslODEInitVal2/driver2.c:148-250,
 * cscal2.c:93-169).  Here a whole batch of nodes is integrated on one GPU by
 * hand-written sm_103a kernels; the per-node semantics (tolerances, scales,
 * trial halving, step-size reuse, post-step clamps) are the reference's.
 *
 * Conventions
 *  - Plain C types only.  Every array is caller-owned.  Functions whose name
 *    contains `_device` take device pointers and a cudaStream_t passed as
 *    `void*`; all others take host pointers and copy inside the call.
 *  - Node data is structure-of-arrays: `state[v*n + i]` is property v of
 *    node i.  The property order is the GAL_Y_* enumeration below.
 *  - Return value 0 means success; a non-zero value is a GAL_ERR_* code and
 *    gal_gpu_last_error() gives the message.  The library never aborts.
 *  - Per-node status uses the reference's integer codes (errorStatus* in
 *    source/error/_module.F90:66-75).
 *  - A context is used by one host thread at a time; it owns one CUDA stream.
 */
#ifndef GALNODE_H
#define GALNODE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- evolved node properties (one FP64 value each) --------------------
 * The serialisation order of the standard hot halo, disk, spheroid and
 * black hole components for the "P-std" physics profile.  Angular momenta
 * are not evolved: the `fixed` galactic structure solver sizes galaxies from
 * the halo spin, not from their angular momentum. */
enum {
  GAL_Y_HOT_MASS = 0,          /* hotHalo%mass                         */
  GAL_Y_HOT_METALS = 1,        /* hotHalo%abundances (metals)          */
  GAL_Y_OUTFLOWED_MASS = 2,    /* hotHalo%outflowedMass                */
  GAL_Y_OUTFLOWED_METALS = 3,  /* hotHalo%outflowedAbundances          */
  GAL_Y_DISK_GAS = 4,          /* disk%massGas                         */
  GAL_Y_DISK_GAS_METALS = 5,   /* disk%abundancesGas                   */
  GAL_Y_DISK_STARS = 6,        /* disk%massStellar                     */
  GAL_Y_DISK_STARS_METALS = 7, /* disk%abundancesStellar               */
  GAL_Y_SPHEROID_GAS = 8,      /* spheroid%massGas                     */
  GAL_Y_SPHEROID_GAS_METALS = 9, /* spheroid%abundancesGas             */
  GAL_Y_SPHEROID_STARS = 10,   /* spheroid%massStellar                 */
  GAL_Y_BLACK_HOLE = 11,       /* blackHole%mass                       */
  GAL_NY = 12
};

/* ---- per-node inputs that are not evolved ------------------------------ */
enum {
  GAL_P_MASS = 0,        /* basic%mass at the start time (Msun)                 */
  GAL_P_MASS_RATE = 1,   /* basic%accretionRate (Msun/Gyr); mass is linear in t */
  GAL_P_RADIUS_VIRIAL = 2,   /* virial radius (Mpc)                             */
  GAL_P_VELOCITY_VIRIAL = 3, /* virial velocity (km/s)                          */
  GAL_P_SPIN = 4,        /* halo spin parameter lambda                          */
  GAL_NP = 5
};

/* ---- per-node status codes (reference values) --------------------------- */
enum {
  GAL_STATUS_SUCCESS = 0,     /* errorStatusSuccess                            */
  GAL_STATUS_UNDERFLOW = 15,  /* errorStatusUnderflow: all ODE trials failed   */
  GAL_STATUS_XCPU = 1025,     /* errorStatusXCPU: per-node step budget used up */
  GAL_STATUS_NOT_FINITE = 2001, /* a state value became NaN or infinite      */
  GAL_STATUS_INTERRUPTED = 9   /* odeSolverInterrupt (= GSL_EBADFUNC): the
                                  evolution stopped early for an interrupt
                                  task (gal_gpu_evolve_batch_interrupt)       */
};

/* ---- components and interrupt tasks (gal_gpu_evolve_batch_interrupt) -----
 * components[i] says which optional components node i has.  As in the
 * reference, where a rate into a component the node does not have makes
 * that component's null-class rate function interrupt the integration so
 * that the host creates it, an evaluation that gives a non-zero rate to a
 * property of a missing component interrupts; the task is the bit mask of
 * the components to create. */
enum {
  GAL_COMPONENT_DISK = 1,
  GAL_COMPONENT_SPHEROID = 2,
  GAL_COMPONENT_BLACK_HOLE = 4,
  GAL_COMPONENT_ALL = 7
};
enum {
  GAL_INTERRUPT_CREATE_DISK = 1,
  GAL_INTERRUPT_CREATE_SPHEROID = 2,
  GAL_INTERRUPT_CREATE_BLACK_HOLE = 4
};

/* ---- library error codes ------------------------------------------------- */
enum {
  GAL_OK = 0,
  GAL_ERR_ARGUMENT = 1,
  GAL_ERR_CUDA = 2,
  GAL_ERR_TABLE = 3,
  GAL_ERR_NO_DEVICE = 4,
  GAL_ERR_TOO_LARGE = 5
};

/* ---- physics switches (bit mask in gal_params.physics) -------------------
 * Each bit enables one node operator of the reference's `nodeOperatorMulti`
 * list (source/nodes/operators/multi.F90:313-332). */
enum {
  GAL_PHYS_STAR_FORMATION_DISK = 1 << 0,     /* starFormationDisks          */
  GAL_PHYS_STAR_FORMATION_SPHEROID = 1 << 1, /* starFormationSpheroids      */
  GAL_PHYS_FEEDBACK_DISK = 1 << 2,           /* stellarFeedbackDisks        */
  GAL_PHYS_FEEDBACK_SPHEROID = 1 << 3,       /* stellarFeedbackSpheroids    */
  GAL_PHYS_BLACK_HOLE_ACCRETION = 1 << 4,    /* blackHolesAccretion         */
  GAL_PHYS_CGM_ACCRETION = 1 << 5,           /* CGMAccretion                */
  GAL_PHYS_REINCORPORATION = 1 << 6,         /* CGMOutflowReincorporation   */
  GAL_PHYS_COOLING = 1 << 7,                 /* CGMCoolingHeating           */
  GAL_PHYS_ALL = 0xff
};

/* Star-formation timescale and outflow classes. */
enum {
  GAL_SF_TIMESCALE_DYNAMICAL = 0, /* starFormationTimescaleDynamicalTime */
  GAL_SF_TIMESCALE_FIXED = 1      /* starFormationTimescaleFixed         */
};
enum {
  GAL_OUTFLOW_POWER_LAW = 0, /* stellarFeedbackOutflowsPowerLaw */
  GAL_OUTFLOW_FIXED = 1      /* stellarFeedbackOutflowsFixed    */
};

/* Arithmetic of the rate functions (gal_gpu_set_rate_precision).  The state,
 * the error norm and the step-size control are FP64 in both. */
enum {
  GAL_RATES_FP64 = 0, /* the reference's arithmetic (default)          */
  GAL_RATES_FP32 = 1  /* FP32 rates and table: the fast form           */
};

/* Star-formation rate class of disks (gal_params.sf_disk_rate). */
enum {
  GAL_SF_RATE_TIMESCALE = 0,   /* starFormationRateDisksTimescale (P-std)              */
  GAL_SF_RATE_KRUMHOLZ2009 = 1 /* starFormationRateDisksIntgrtdSurfaceDensity with
                                  starFormationRateSurfaceDensityDisksKrumholz2009:
                                  the reference's default                            */
};

/* Star formation in one component (disk or spheroid).
 * Reference: source/star_formation/timescales/dynamical_time.F90:121-189,
 * source/star_formation/rates/disks/timescale.F90:109-130. */
typedef struct gal_star_formation {
  int32_t timescale_type;    /* GAL_SF_TIMESCALE_*                        */
  int32_t pad;
  double efficiency;         /* epsilon_* (dynamicalTime: 0.01)             */
  double exponent_velocity;  /* alpha_* (dynamicalTime: -1.5)              */
  double timescale_minimum;  /* Gyr (1e-3)                                  */
  double timescale_fixed;    /* Gyr, used by GAL_SF_TIMESCALE_FIXED         */
} gal_star_formation;

/* Stellar-feedback outflows from one component, wrapped by `rateLimit`.
 * Reference: source/stellar_feedback/outflows/power_law/_class.F90:118-164,
 * fixed.F90, rate_limit.F90. */
typedef struct gal_outflow {
  int32_t type;                /* GAL_OUTFLOW_*                               */
  int32_t pad;
  double velocity_characteristic; /* km/s (disk 250, spheroid 100)          */
  double exponent;             /* power-law exponent (3.5)                   */
  double fraction;             /* GAL_OUTFLOW_FIXED mass-loading fraction    */
  double timescale_fractional_minimum; /* rateLimit; <= 0 disables the limit */
} gal_outflow;

/* All parameters of one evolution context.  gal_params_default() fills the
 * values of the "P-std" profile (the reference's default classes, with the
 * documented substitutions); callers may change any field before
 * gal_gpu_init(). */
typedef struct gal_params {
  /* mergerTreeNodeEvolverStandard (standard.F90:174-181, 135) */
  double ode_tolerance_absolute;   /* odeToleranceAbsolute (0.01)            */
  double ode_tolerance_relative;   /* odeToleranceRelative (0.01)            */
  int32_t reuse_step_size;         /* reuseODEStepSize (1)                   */
  int32_t trial_count_maximum;     /* trialCountMaximum (8)                  */
  int32_t step_budget;             /* attempted steps per node before XCPU   */
  uint32_t physics;                /* GAL_PHYS_* mask                        */
  /* cosmologyParameters simple */
  double omega_matter, omega_baryon, omega_dark_energy, hubble_constant;
  /* hot halo: betaProfile with virialFraction core radius, virial T profile */
  double core_radius_fraction;     /* coreRadiusOverVirialRadius (0.3)       */
  double cooling_velocity_cutoff;  /* coolingRateWhiteFrenk1991 (1e4 km/s)   */
  double cooling_degrees_of_freedom; /* coolingTimeSimple (3)                */
  double reincorporation_multiplier; /* haloDynamicalTime multiplier (5)     */
  /* galacticStructureSolverFixed: r = f lambda r_vir, v = v_vir */
  double radius_factor_disk, radius_factor_spheroid; /* sqrt(1/2)          */
  gal_star_formation sf_disk, sf_spheroid;
  /* stellarPopulationPropertiesInstantaneous */
  double recycled_fraction;        /* 0.46                                   */
  double metal_yield;              /* 0.035                                  */
  gal_outflow outflow_disk, outflow_spheroid;
  /* blackHoleAccretionRateStandard + Shakura-Sunyaev thin disk */
  double bh_enhancement_spheroid;  /* 5                                      */
  double bh_enhancement_hot_halo;  /* 6                                      */
  double bh_temperature_spheroid;  /* K (100)                                */
  int32_t bh_hot_mode_only;        /* 1                                      */
  int32_t pad;
  double bh_efficiency_radiative;  /* 1 - E_ISCO(spin 0) = 1 - sqrt(8/9)     */
  double bh_efficiency_jet;        /* 0                                      */
  /* mergerTreeEvolveTimestepSimple (merger_trees/evolve/timesteps/simple.F90:
   * 71-80, 124-161): in a forest, one evolve call advances a node by at most
   * min(timestep_relative / H(t), timestep_absolute), H the expansion rate
   * at the call's start (timestep_relative <= 0: the absolute limit alone). */
  double timestep_relative;        /* timeStepRelative (0.1)                 */
  double timestep_absolute;        /* timeStepAbsolute, Gyr (1)              */
  /* Disk star-formation rate class.  GAL_SF_RATE_KRUMHOLZ2009 integrates the
   * Krumholz, McKee & Tumlinson (2009) surface density law over the
   * exponential gas disk (star_formation/rates/disks/
   * integrated_surface_density.F90:131-190, star_formation/
   * rate_surface_density/disks/Krumholz2009.F90:312-620); the spheroid keeps
   * the timescale rate and sf_disk is then unused. */
  int32_t sf_disk_rate;            /* GAL_SF_RATE_* (P-std: timescale)       */
  int32_t krumholz_fast;           /* molecularFractionFast (0)              */
  double krumholz_frequency;       /* frequencyStarFormation, 1/Gyr (0.385)  */
  double krumholz_clumping;        /* clumpingFactorMolecularComplex (5)     */
  /* Forests: a secondary progenitor merges into the primary at the parent's
   * time with the mass movements of mergerMassMovementsSimple
   * (satellites/merging/mass_movements/simple.F90): a merger is major when
   * the smaller galaxy has at least this fraction of the larger one's
   * disk-plus-spheroid mass. */
  double merger_mass_ratio_major;  /* massRatioMajorMerger (0.25)            */
} gal_params;

/* Cooling-function and electron-density tables in the layout of the
 * reference's CIE files (cooling_function/CIE_file.F90:535-663,
 * chemical/state/CIE_file.F90:617-760): temperatures in K, metallicities as
 * Z/Zsun (the first may be zero), cooling_rate in erg cm^3 s^-1 and
 * electron_density as n_e/n_H, both row-major [iZ][iT]. */
typedef struct gal_cie_table {
  int32_t n_temperature;
  int32_t n_metallicity;
  const double* temperature;
  const double* metallicity;
  const double* cooling_rate;
  const double* electron_density;
} gal_cie_table;

typedef struct gal_ctx gal_ctx;

/* Fill `p` with the P-std defaults. */
void gal_params_default(gal_params* p);

/* Library version string. */
const char* gal_version(void);

/* Create a context on the current CUDA device: validate the parameters,
 * take the log of the tables as the reference does, stage them in device
 * memory and pick launch shapes.  Replaces the constructor
 * mergerTreeNodeEvolverStandard (standard.F90:313-383) plus the class
 * objects it builds from the parameter file. */
int gal_gpu_init(const gal_params* p, const gal_cie_table* table, gal_ctx** out);

/* Release a context and its device memory. */
void gal_gpu_free(gal_ctx* ctx);

/* Copy the last error message of `ctx` (or of the library, if ctx is NULL)
 * into buf (at most len bytes, NUL terminated).  Returns the error code. */
int gal_gpu_last_error(const gal_ctx* ctx, char* buf, int len);

/* Evolve n independent nodes, node i from t_start[i] to t_end[i] (Gyr).
 * Batched form of mergerTreeNodeEvolver%evolve (node_evolver/_class.F90:41-57,
 * standard.F90:385-755) for nodes that are not interrupted.
 *   state     [GAL_NY][n]  in/out  evolved properties
 *   param     [GAL_NP][n]  in      GAL_P_* inputs
 *   t_start, t_end [n]     in
 *   step      [n]          in/out  node%timeStep(): the step size to try
 *                                  first (<= 0: the whole interval); on
 *                                  success the suggested next step
 *   status    [n]          out     GAL_STATUS_*
 *   counters  [3][n]       out     accepted steps, rejected steps, RHS
 *                                  evaluations (may be NULL)
 * Host pointers; the call copies inputs to the device, evolves and copies
 * the outputs back before it returns. */
int gal_gpu_evolve_batch(gal_ctx* ctx, int64_t n, double* state, const double* param,
                         const double* t_start, const double* t_end, double* step,
                         int32_t* status, uint32_t* counters);

/* As gal_gpu_evolve_batch, on device-resident arrays, enqueued on `stream`
 * (a cudaStream_t used as given; NULL is the legacy default stream).
 * Asynchronous: the results are ready when the stream reaches this point. */
int gal_gpu_evolve_batch_device(gal_ctx* ctx, int64_t n, double* state, const double* param,
                                const double* t_start, const double* t_end, double* step,
                                int32_t* status, uint32_t* counters, void* stream);

/* Evolution with interrupts: mergerTreeNodeEvolver%evolve with its
 * `interrupted` and `functionInterrupt` outputs (node_evolver/_class.F90:
 * 41-57; standard.F90:385-406, 575-578, 729-737, 895-945; the solver's
 * re-targeting numerical/ODE_solver/solver.F90:608-620).  Arrays as in
 * gal_gpu_evolve_batch, plus
 *   components [n]  in   GAL_COMPONENT_* mask of the components node i has
 *   t_reached  [n]  out  the time node i reached: t_end[i], or the time of
 *                        its earliest interrupt
 *   task       [n]  out  GAL_INTERRUPT_* mask of that interrupt (0: none)
 * An interrupted node has status GAL_STATUS_INTERRUPTED, its state at
 * t_reached[i] and step[i] = -1 (node%timeStepSet(-1)); the caller creates
 * the components named by the task and evolves it again from t_reached.
 * Every evaluation at or after an interrupt time returns zero derivatives,
 * and the step function evaluates f(t+h, y_new) on every attempt, as GSL's
 * rkck does, since that evaluation can interrupt too.  FP64 rates only
 * (GAL_ERR_ARGUMENT in the FP32-rate form or with a surrogate installed);
 * 128 threads per block. */
int gal_gpu_evolve_batch_interrupt(gal_ctx* ctx, int64_t n, double* state, const double* param, const double* t_start,
                                   const double* t_end, double* step, const int32_t* components, int32_t* status,
                                   uint32_t* counters, double* t_reached, int32_t* task);
/* As gal_gpu_evolve_batch_interrupt on device arrays, enqueued on `stream`. */
int gal_gpu_evolve_batch_interrupt_device(gal_ctx* ctx, int64_t n, double* state, const double* param,
                                          const double* t_start, const double* t_end, double* step,
                                          const int32_t* components, int32_t* status, uint32_t* counters,
                                          double* t_reached, int32_t* task, void* stream);

/* Evolution for callers that cannot let a library allocate device memory,
 * e.g. a host code whose pool allocator owns all device memory, or one that
 * must not take the device-wide synchronisation cudaMalloc/cudaFree can
 * cause.  No counterpart in the reference: it exists for such integrations.
 * Same node arrays and semantics as gal_gpu_evolve_batch_device (device
 * pointers, enqueued on `stream`, NULL = legacy default stream); `p` and
 * `table` are host structures as for gal_gpu_init.  No context is used and
 * nothing is allocated, on the device or the host: the kernel's scratch (the
 * work-queue head plus the log-converted CIE tables) is one fixed 128 KiB
 * static device array in this library, held by every GPU that loads it until
 * the process exits.  Tables needing more than that are rejected with
 * GAL_ERR_TOO_LARGE: a table takes 16 B per cell, 8 B per temperature and
 * 16 B per metallicity, plus 2,816 B that do not depend on it (the 2 KiB
 * short-log and 512 B exponential tables of the FP64 functions and the
 * 256 B queue head); the reference's 24 x 261 grid takes 105,512 B.  The
 * first call on a device looks up the array's device address; make that
 * first call before any stream capture.  Every call restages the table and
 * resets the queue head in the shared array, so calls that overlap on the
 * GPU (on different streams or from different threads) race: serialise
 * them.  Launch shape is fixed at 128 threads, one block per SM. */
int gal_gpu_evolve_batch_noalloc(const gal_params* p, const gal_cie_table* table, int64_t n, double* state,
                                 const double* param, const double* t_start, const double* t_end, double* step,
                                 int32_t* status, uint32_t* counters, void* stream);

/* Launch shape of the evolve kernel (threads per block, blocks per SM); 0
 * keeps the current value.  Used by the autotuner.  Block sizes per form:
 * FP64 rates 64-512, FP32 rates 128-512, with the surrogate 128 or 256;
 * get_launch reports the shape the current form will use. */
int gal_gpu_set_launch(gal_ctx* ctx, int32_t threads_per_block, int32_t blocks_per_sm);
int gal_gpu_get_launch(const gal_ctx* ctx, int32_t* threads_per_block, int32_t* blocks_per_sm);

/* Arithmetic of the rate functions: GAL_RATES_FP64 (default; the
 * reference's FP64 arithmetic throughout) or GAL_RATES_FP32 (rates, cooling
 * table and stage arguments in FP32; the state, the accepted-step update,
 * the error norm and the step control stay FP64).  No counterpart in the
 * reference, which evaluates every rate in FP64. */
int gal_gpu_set_rate_precision(gal_ctx* ctx, int32_t precision);
int gal_gpu_get_rate_precision(const gal_ctx* ctx);

/* Number of kernel launches this context has made since creation. */
int64_t gal_gpu_launch_count(const gal_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* GALNODE_H */
