/*
 * galnode_forest.h -- merger forests on the GB300 node evolver: a host
 * merger-tree builder and whole-forest evolution in one persistent kernel.
 *
 * Reference: the tree evolver advances each node from its own time to its
 * parent's, limited by the output times, and promotes or merges it there
 * (merger_trees/evolver/standard.F90:762-1035, threaded.F90:418-840); trees
 * come from the Cole et al. (2000) builder with the Parkinson, Cole & Helly
 * (2008) branching rates (merger_trees/construct/builder/Cole2000/
 * _class.F90:360-913, merger_trees/branching_probability/
 * Parkinson_Cole_Helly.F90:265-634).  gal_gpu_forest_evolve replaces the
 * per-node evolve calls of one forest (mergerTreeNodeEvolver%evolve, called
 * from evolver/standard.F90:452 and threaded.F90:637) with one graph launch.
 *
 * Forest layout (caller-owned host arrays, n nodes; gal_forest_build puts
 * each tree's root first): the progenitors of every node are contiguous,
 * primary (most massive) first:
 *   parent[n]       index of the parent, -1 for a root
 *   child_first[n]  index of the first progenitor (any value if none)
 *   child_count[n]  number of progenitors
 *   time[n]         cosmic time of the node (Gyr); a progenitor's time is
 *                   earlier than its parent's
 *   mass[n]         halo mass at that time (Msun)
 *   spin[n]         spin parameter
 * A node evolves from time[i] to time[parent[i]].  On reaching it, the
 * primary progenitor's state becomes the parent's initial state and the
 * other progenitors merge into it in index order as satellites, with the
 * mass movements of mergerMassMovementsSimple (satellites/merging/
 * mass_movements/simple.F90; gal_params.merger_mass_ratio_major): minor
 * mergers put the satellite's gas and stars into the host's spheroid, major
 * ones both galaxies; hot gas, outflowed gas and black holes add up (the
 * satellite's orbit until it merges is not modelled).  A primary progenitor's halo mass grows linearly to its
 * parent's over the interval; its hot halo accretes (Omega_b/Omega_m) times
 * the parent's mass not brought in by its progenitors.  The interval is cut
 * into evolve calls at every output time inside it and wherever a call would
 * be longer than the timestep limit min(timestep_relative / H(t),
 * timestep_absolute) of gal_params (merger_trees/evolve/timesteps/
 * simple.F90:124-161); each call recomputes the halo's mass, virial radius
 * and velocity at its start, carries the step size over, and the state at
 * each output time is recorded.
 */
#ifndef GALNODE_FOREST_H
#define GALNODE_FOREST_H

#include <stdint.h>
#include "galnode.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- trees */

typedef struct gal_pch_params {
  double g0, gamma1, gamma2;  /* PCH merger-rate modifier G0 (s1/s2)^g1 (d2/s2)^g2 (quickTest: 0.57, 0.38, -0.01) */
  double accuracy_first;      /* step limit on the split probability (0.1)                 */
  double accuracy_second;     /* step limit on d(delta_c) relative to sigma (0.1)          */
  double sigma8, n_s;         /* power-spectrum normalisation and slope                     */
  double temperature_cmb;     /* K (2.72548)                                               */
  int32_t transfer_function;  /* GAL_TRANSFER_* (the reference's default, Eisenstein & Hu 1999) */
  int32_t reserved;
  double neutrino_number_effective; /* Eisenstein & Hu (1999): N_eff (3.046)              */
  double neutrino_mass_summed;      /* Eisenstein & Hu (1999): sum of masses, eV (0)      */
} gal_pch_params;

/* Transfer functions of the builder's power spectrum: the reference's
 * transferFunctionEisensteinHu1999 (its default; structure_formation/
 * transfer_function/Eisenstein_Hu1999.F90) and the Eisenstein & Hu (1998)
 * zero-baryon form. */
enum { GAL_TRANSFER_EISENSTEIN_HU_1999 = 0, GAL_TRANSFER_EISENSTEIN_HU_1998 = 1 };

typedef struct gal_forest_spec {
  int64_t n_trees;
  uint64_t seed;
  double root_mass_min, root_mass_max; /* Msun                                                  */
  double root_mass_slope;              /* dN/dln M ~ M^slope for the roots (-0.9)              */
  double root_redshift;                /* 0                                                    */
  double redshift_max;                 /* branches end here (8)                                */
  double mass_resolution;              /* Msun                                                 */
  /* Satellites.  GAL_SATELLITES_NONE: a secondary progenitor merges into
   * the primary at their parent's time.  GAL_SATELLITES_JIANG2008: it
   * becomes a satellite there and merges with the central galaxy of the
   * halo that holds it after the Jiang et al. (2008) dynamical-friction
   * time on a Benson (2005) orbit (satellites/merging/timescale/
   * Jiang2008.F90, satellites/merging/virial_orbits/Benson2005.F90, the
   * reference's default classes); see gal_satellite_merging_time. */
  int32_t satellites;
  int32_t reserved;
  double satellite_timescale_multiplier; /* Jiang2008 timescaleMultiplier (quickTest: 0.75)    */
} gal_forest_spec;

enum { GAL_SATELLITES_NONE = 0, GAL_SATELLITES_JIANG2008 = 1 };

typedef struct gal_forest gal_forest;  /* host-side forest built by gal_forest_build */

void gal_pch_params_default(gal_pch_params* p);

/* Build n_trees trees with the Cole et al. (2000) algorithm and PCH
 * branching rates, in the cosmology of p (omega_*, hubble_constant),
 * OpenMP-parallel over trees; every tree is a deterministic function of
 * (seed, tree index). */
int gal_forest_build(const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec, gal_forest** out);
/* The same builder with its branches grown on the GPU of ctx: the tables
 * (sigma(M), the split and sub-resolution rates, the split's distribution
 * in ln q) and each tree's root mass are those of gal_forest_build, and
 * every branch is walked by the host builder's steps with the rates
 * evaluated in FP32 (the mass and w accumulated in FP64); each branch draws
 * from its own stream, keyed by its tree and its path from the root, so the
 * trees are a deterministic function of (seed, tree index), of the host
 * builder's distribution, but not the trees gal_forest_build makes from the
 * same seed.  Spins and
 * satellite orbits are drawn on the host as by gal_forest_build.  The
 * Cole2000 builder's per-tree build (merger_trees/construct/builder/
 * Cole2000/_class.F90:360-913), for a whole forest at once.  The node
 * arrays on the GPU are sized from the roots' masses and grown (the growth
 * repeated) when a forest outgrows them; the environment variable
 * GALNODE_BRANCH_CAPACITY sets their first size instead (for tests of that
 * path).  Errors are recorded in ctx. */
int gal_gpu_forest_build(gal_ctx* ctx, const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec,
                         gal_forest** out);
/* The inputs of the GPU branching for a forest spec (for tests of it
 * against a restatement of its walk): sizes[2] = {sigma rows, rate rows};
 * meta[10] = {ln M of the first sigma row, its spacing in ln M, the same
 * for the rate rows, mass resolution, w at the maximum redshift, gamma2,
 * accuracy_first, accuracy_second, w at the roots' redshift}; and, where
 * not NULL, ln_sigma[sizes[0]] (ln sigma(M) at z = 0), rate[sizes[1]] and
 * accretion[sizes[1]] (without their (w/sigma)^gamma2 factor),
 * ln_q[sizes[1]][96] and cdf[sizes[1]][96] (the split's cumulative
 * distribution in ln q). */
int gal_pch_branch_tables(const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec, int32_t* sizes,
                          double* meta, double* ln_sigma, double* rate, double* accretion, double* ln_q, double* cdf);
int64_t gal_forest_node_count(const gal_forest* f);
/* Where a build's time went, host clock: stats[7] = {seconds building the
 * tables, seconds of the GPU growth (its generations; 0 for
 * gal_forest_build), seconds downloading and renumbering the GPU's nodes,
 * seconds of the
 * per-tree loop (root, growth on the host, spins, satellites), seconds of
 * the assembly into the forest layout, GPU generations, total seconds}. */
int gal_forest_build_stats(const gal_forest* f, double* stats);
/* Copy the forest out in the layout above (any pointer may be NULL);
 * tree[n] receives the tree index of each node. */
int gal_forest_get(const gal_forest* f, int32_t* tree, int32_t* parent, int32_t* child_first, int32_t* child_count,
                   double* time, double* mass, double* spin);
/* With satellites: satellite_host[n] receives, for each node that is a
 * satellite's phase from its infall to its merger (or to the end), the
 * node it fell into (its host at infall), and -1 for every other node.  A
 * satellite's phase is its own node: its only progenitor is the halo that
 * fell in, its parent the piece of the host's branch that starts at the
 * merger (a node whose primary progenitor is the host's branch before the
 * merger), or none when it outlives the tree.  Its halo mass and virial
 * scales stay those at infall and it accretes nothing
 * (dmoInterpolateNodeInitialize, nodes/operators/physics/
 * dark_matter_only_mass/interpolate.F90:118-120). */
int gal_forest_get_satellite_host(const gal_forest* f, int32_t* satellite_host);
void gal_forest_free(gal_forest* f);

/* The merging time (Gyr) of a satellite of mass_satellite that falls into a
 * host halo of mass_host at time t on an orbit with radial and tangential
 * velocities velocity_radial and velocity_tangential at the host's virial
 * radius, in units of its virial velocity: Jiang et al. (2008, ApJ 675,
 * 1095) as satelliteMergingTimescalesJiang2008%timeUntilMerging
 * (satellites/merging/timescale/Jiang2008.F90),
 *   multiplier t_dyn (r_c/r_vir)^1/2 (0.94 eps^0.60 + 0.60)/(2 0.43) q/ln(1+q),
 * q = mass_host/mass_satellite, t_dyn = r_vir/V_vir of the host, r_c and
 * eps the radius and circularity of the circular orbit of the same energy
 * in a singular isothermal host truncated at r_vir (point mass outside).
 * Returns a negative value for an unbound orbit. */
double gal_satellite_merging_time(const gal_params* p, double mass_host, double mass_satellite, double t,
                                  double velocity_radial, double velocity_tangential, double multiplier);

/* n orbits from the builder's Benson (2005) sampler (satellites/merging/
 * virial_orbits/Benson2005.F90): radial and tangential velocities at the
 * host's virial radius in units of its virial velocity, bound for the
 * specific reduced mass mu = M_host/(M_host + M_sat); one stream seeded by
 * seed (for tests of the sampler against the published distribution). */
int gal_satellite_orbits(uint64_t seed, double mu, int64_t n, double* velocity_radial, double* velocity_tangential);

/* Cosmic time (Gyr) at redshift z and its inverse, in the cosmology of p. */
double gal_cosmic_time(const gal_params* p, double z);
double gal_redshift(const gal_params* p, double t);
/* sigma(M) of the builder's power spectrum at z = 0 (for tests). */
double gal_pch_sigma(const gal_params* p, const gal_pch_params* pch, double mass);
/* The builder's transfer function at wavenumber k (1/Mpc) (for tests);
 * the reference's transferFunctionClass%value. */
double gal_pch_transfer(const gal_params* p, const gal_pch_params* pch, double k);
/* The builder's branching rates, per unit of the critical overdensity w,
 * for a branch of mass_parent at w when sigma(M) is the power law
 * sigma_parent (M/mass_parent)^alpha: rate = the probability rate of a
 * split into a progenitor above mass_resolution, accretion = the rate of
 * the mass fraction lost below it.  The reference's
 * mergerTreeBranchingProbabilityParkinsonColeHelly%probability and
 * %fractionSubresolution (merger_trees/branching_probability/
 * Parkinson_Cole_Helly.F90:265-634); for tests against the reference's
 * branching-rate known answers (source/tests/merger_tree_branching.F90). */
int gal_pch_branching_rates(const gal_pch_params* pch, double alpha, double sigma_parent, double mass_parent,
                            double mass_resolution, double w, double* rate, double* accretion);

/* -------------------------------------------------------------- evolution */

typedef struct gal_forest_dev gal_forest_dev;  /* a forest resident on the GPU of a context */

/* Upload a forest and its output times (sorted, Gyr) to the context's GPU:
 * the segment table (per piece: halo mass, accretion rate, virial radius
 * and velocity, spin, start and end time) is built on the GPU, and
 * state0[GAL_NY][n] holds the initial states (only progenitor-less nodes
 * are read).  A node's halo mass grows by the mass its parent holds beyond
 * its progenitors' (the unresolved mass, over the node's interval) when it
 * is its parent's primary progenitor, and stays constant otherwise
 * (dmoInterpolateNodeInitialize, nodes/operators/physics/
 * dark_matter_only_mass/interpolate.F90:84-168).  satellite_host (may be
 * NULL: no satellites) marks the satellite phases as gal_forest_get_
 * satellite_host does: such a node keeps its halo mass and the virial
 * scales of its infall time, accretes nothing, and its mass counts as
 * brought into its host at infall.  The returned object owns every device
 * array and a CUDA graph of one evolution (reset, counters, kernel). */
int gal_gpu_forest_create(gal_ctx* ctx, int64_t n, const int32_t* parent, const int32_t* child_first,
                          const int32_t* child_count, const double* time, const double* mass, const double* spin,
                          const int32_t* satellite_host, const double* state0, int32_t n_outputs,
                          const double* output_times, gal_forest_dev** out);
/* Evolve the whole forest from state0 (one graph launch on the context
 * stream; asynchronous: gal_gpu_forest_sync waits).  Available in the FP64
 * form and the FP32-rate forms (with or without the surrogate); with a
 * surrogate and FP64 rates it returns GAL_ERR_ARGUMENT. */
int gal_gpu_forest_evolve(gal_ctx* ctx, gal_forest_dev* f);
int gal_gpu_forest_sync(gal_ctx* ctx, gal_forest_dev* f);
/* Results of the last evolution:
 *   state[GAL_NY][n]     each node's state on reaching its parent's time
 *                        (a root: its state at its own time);
 *   status[n], counters[3][n] (accepted, rejected, RHS over all pieces);
 *   snapshot[GAL_NY][m]  states at the output times, m = snapshot count;
 *   snap_node[m], snap_output[m]: node and output index of each snapshot. */
int64_t gal_gpu_forest_snapshot_count(const gal_forest_dev* f);
int gal_gpu_forest_results(gal_ctx* ctx, gal_forest_dev* f, double* state, int32_t* status, uint32_t* counters,
                           double* snapshot, int32_t* snap_node, int32_t* snap_output);
/* Node-timesteps (accepted steps) of the last evolution. */
int64_t gal_gpu_forest_accepted_steps(gal_ctx* ctx, gal_forest_dev* f);
/* Time a few evolutions at each launch shape the current form is built for
 * (threads per block x blocks per SM) and keep the fastest in the context;
 * times_ms[i] (may be NULL, length >= 8) receives the mean time of shape i
 * in the order 64x1, 128x1, 128x2, 256x1, 256x2, 512x1 (negative: not
 * available). */
int gal_gpu_forest_autotune(gal_ctx* ctx, gal_forest_dev* f, int32_t repeats, double* times_ms);
void gal_gpu_forest_free(gal_forest_dev* f);

#ifdef __cplusplus
}
#endif

#endif
