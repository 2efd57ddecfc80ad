/*
 * ocm.h - C ABI of the GB300-native force-and-integrate engine for
 * OpenCafeMol's coarse-grained protein force field.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (OCM_OK == 0) and never throws.  The text of the last error of
 * the calling thread is available from ocm_last_error().
 *
 * Units are OpenMM's: nm, ps, amu, kJ/mol, elementary charge.  Index arrays
 * are int64 and flattened (pairs: 2*n, triplets: 3*n, quadruplets: 4*n).
 *
 * Three layers, each replacing one seam of the reference:
 *   1. Topology + force-field generators + system assembly
 *      (src/Topology.hpp, src/forcefield/*ForceFieldGenerator.*,
 *       src/SystemGenerator.cpp): ocm_topology_*, ocm_add_*, ocm_system_*.
 *   2. The plain single-system path, the part of OpenMM's Context +
 *      LangevinIntegrator that src/Simulator.cpp drives: ocm_context_*.
 *   3. The batched / served multi-system path (no counterpart in the
 *      reference, which runs one system per process): ocm_batch_*.
 */
#ifndef OCM_GB300_H
#define OCM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCM_ABI_VERSION 2

enum ocm_status {
    OCM_OK = 0,
    OCM_ERR_INVALID_ARGUMENT = 1,   /* bad index, size mismatch, NaN where a value is required */
    OCM_ERR_CUDA = 2,               /* a CUDA runtime call failed */
    OCM_ERR_OUT_OF_MEMORY = 3,      /* device allocation failed or batch capacity exhausted */
    OCM_ERR_NEIGHBOR_OVERFLOW = 4,  /* tile list capacity exceeded (grown and retried internally) */
    OCM_ERR_STATE = 5,              /* call made in the wrong state (e.g. no positions set) */
    OCM_ERR_UNSUPPORTED = 6,        /* a valid reference input this engine does not handle */
    OCM_ERR_NONFINITE = 7,          /* NaN/Inf found in forces or positions */
    OCM_ERR_TIMEOUT = 8             /* reserved, never returned: no kernel of this library waits on a
                                       flag or on another block, so there is no bounded wait to give up */
};

/* Force-group limit; OpenMM allows 32 groups (Force::setForceGroup). */
#define OCM_MAX_GROUPS 32

const char* ocm_last_error(void);
int ocm_abi_version(void);
/* Number of CUDA devices visible (0 on a machine without a GPU); never fails. */
int ocm_device_count(void);

/* ---------------------------------------------------------------------------
 * Parameter tables of the flexible-local potentials.
 * Replaces the lookups into src/util/Constants.hpp:28-102
 * (Constant::fla_spline_table, fla_spline_second_derivative_table,
 *  fld_fourier_table).  Amino acids are the 20 three-letter codes; the FLD
 * keys are "R1-GLY", "R2-PRO", "<AA>-R3" and "GLY-PRO".
 * ------------------------------------------------------------------------ */
int ocm_fla_table(const char* aa_name, double* spline_table10, double* second_derivative10);
int ocm_fld_table(const char* key, double* fourier_table7);
/* Key of FLD table number idx (0..22) in the reference's std::map order. */
int ocm_fld_table_key(int idx, char* buf, int64_t cap);

/* ---------------------------------------------------------------------------
 * Topology: replaces class Topology (src/Topology.hpp:9-81, Topology.cpp).
 * ------------------------------------------------------------------------ */
typedef struct ocm_topology ocm_topology;
int ocm_topology_create(int64_t n_particles, ocm_topology** out);
void ocm_topology_destroy(ocm_topology* topo);
/* Topology::add_edges (Topology.hpp:25-38): n_edges pairs. */
int ocm_topology_add_edges(ocm_topology* topo, int64_t n_edges, const int64_t* pairs,
                           const char* edge_type);
/* Topology::make_molecule (Topology.cpp:7-48). */
int ocm_topology_make_molecule(ocm_topology* topo, const char* edge_type);
/* Topology::ignore_list_within_edge (Topology.cpp:75-110): writes sorted,
 * unique pairs (first < second) into out_pairs (2*capacity int64), count in
 * *n_out.  If capacity is too small, *n_out is the needed size and
 * OCM_ERR_INVALID_ARGUMENT is returned. */
int ocm_topology_ignore_list_within_edge(const ocm_topology* topo, int64_t dist,
                                         const char* edge_type, int64_t* out_pairs,
                                         int64_t capacity, int64_t* n_out);
/* Topology::ignore_list_within_molecule (Topology.cpp:51-73). */
int ocm_topology_ignore_list_within_molecule(const ocm_topology* topo, int64_t* out_pairs,
                                             int64_t capacity, int64_t* n_out);

/* ---------------------------------------------------------------------------
 * System assembly: replaces SystemGenerator (src/SystemGenerator.hpp:24-38,
 * SystemGenerator.cpp:4-111).  Each ocm_add_* call is one generator's
 * constructor + generate() + SystemGenerator::add_ff_generator; the force
 * group it lands in follows SystemGenerator.cpp:4-32 (one group per
 * generator name; all FlexibleLocalAngle and all FlexibleLocalDihedral
 * generators share one group each) and is returned in *group_out.
 * ------------------------------------------------------------------------ */
typedef struct ocm_system ocm_system;
/* SystemGenerator(mass_vec) + System::addParticle (SystemGenerator.cpp:39-42). */
int ocm_system_create(int64_t n_particles, const double* masses, ocm_system** out);
void ocm_system_destroy(ocm_system* sys);
/* SystemGenerator::set_pbc -> setDefaultPeriodicBoxVectors (SystemGenerator.cpp:45-56). */
int ocm_system_set_pbc(ocm_system* sys, double lx, double ly, double lz);
int64_t ocm_system_num_particles(const ocm_system* sys);
int ocm_system_num_groups(const ocm_system* sys);
/* Name of force group g ("HarmonicBond", "FlexibleLocalAngle", ...). */
int ocm_system_group_name(const ocm_system* sys, int group, char* buf, int64_t cap);
/* JSON description of every generated force: cutoffs, global parameters,
 * participant counts, exclusion counts (what generate() put into the
 * OpenMM Force objects). */
int ocm_system_describe(const ocm_system* sys, char* buf, int64_t cap, int64_t* needed);

/* HarmonicBondForceFieldGenerator(indices, v0s, ks, use_periodic)
 * (HarmonicBondForceFieldGenerator.hpp:24-41, .cpp:3-14).  ks are the
 * OpenMM 1/2 k (r-r0)^2 constants, i.e. already doubled by the reader
 * (ReadTOMLForceFieldGenerator.cpp:57-64). */
int ocm_add_harmonic_bond(ocm_system* sys, int64_t n, const int64_t* indices,
                          const double* v0s, const double* ks, int use_periodic,
                          int* group_out);
/* GoContactForceFieldGenerator(indices, ks, r0s, use_periodic)
 * (GoContactForceFieldGenerator.hpp:22-40, .cpp:3-20). */
int ocm_add_go_contact(ocm_system* sys, int64_t n, const int64_t* indices,
                       const double* ks, const double* r0s, int use_periodic,
                       int* group_out);
/* GaussianBondForceFieldGenerator(indices, ks, v0s, sigmas, use_periodic)
 * (GaussianBondForceFieldGenerator.hpp:22-48, .cpp:3-23): the AICG2+
 * k exp(-(r - v0)^2 / (2 sigma^2)); ks in kJ/mol, v0s and sigmas in nm. */
int ocm_add_gaussian_bond(ocm_system* sys, int64_t n, const int64_t* indices, const double* ks,
                          const double* v0s, const double* sigmas, int use_periodic,
                          int* group_out);
/* GaussianDihedralForceFieldGenerator(indices, ks, theta0s, sigmas, use_periodic)
 * (GaussianDihedralForceFieldGenerator.hpp:22-50, .cpp:3-27): the AICG2+
 * k exp(-dphi^2 / (2 sigma^2)), dphi = phi - theta0 wrapped to [-pi, pi);
 * theta0s and sigmas in radians. */
int ocm_add_gaussian_dihedral(ocm_system* sys, int64_t n, const int64_t* indices,
                              const double* ks, const double* theta0s, const double* sigmas,
                              int use_periodic, int* group_out);
/* FlexibleLocalAngleForceFieldGenerator(indices, ks, spline_table, aa_name,
 * use_periodic) with the default theta range
 * (FlexibleLocalAngleForceFieldGenerator.hpp:21-47, .cpp:3-68). */
int ocm_add_flexible_local_angle(ocm_system* sys, int64_t n, const int64_t* indices,
                                 const double* ks, const double* spline_table10,
                                 const char* aa_name, int use_periodic, int* group_out);
/* FlexibleLocalDihedralForceFieldGenerator(indices, ks, fourier_table,
 * aa_pair_name, use_periodic) (FlexibleLocalDihedralForceFieldGenerator.hpp:22-40,
 * .cpp:5-62). */
int ocm_add_flexible_local_dihedral(ocm_system* sys, int64_t n, const int64_t* indices,
                                    const double* ks, const double* fourier_table7,
                                    const char* aa_pair_name, int use_periodic,
                                    int* group_out);

/* Pair (CustomNonbondedForce) generators share these trailing arguments:
 *   n_ignore, ignore_pairs      : the ignore_list (exclusions)
 *   use_periodic                : CutoffPeriodic vs CutoffNonPeriodic
 *   n_ignore_groups, ignore_group_pairs, group_vec :
 *       ignore_group_pairs (2*n int32 group ids) and group_vec (per particle
 *       group id, -1 = no group; may be NULL when n_ignore_groups == 0); they
 *       feed extract_interaction_group (InteractionGroup.hpp:17-101).
 * Per-particle parameters use NaN for "no value" (std::nullopt). */

/* ExcludedVolumeForceFieldGenerator(eps, cutoff, radii, ignore_list, ...)
 * (ExcludedVolumeForceFieldGenerator.cpp:11-92); cutoff is the ratio
 * applied to (max radius + second max radius). */
int ocm_add_excluded_volume(ocm_system* sys, double eps, double cutoff_ratio,
                            const double* radii, int64_t n_ignore,
                            const int64_t* ignore_pairs, int use_periodic,
                            int64_t n_ignore_groups, const int32_t* ignore_group_pairs,
                            const int32_t* group_vec, int* group_out);
/* DebyeHuckelForceFieldGenerator(ionic_strength, temperature, cutoff_ratio,
 * charges, ignore_list, ...) (DebyeHuckelForceFieldGenerator.hpp:22-41,
 * .cpp:10-108). */
int ocm_add_debye_huckel(ocm_system* sys, double ionic_strength, double temperature,
                         double cutoff_ratio, const double* charges, int64_t n_ignore,
                         const int64_t* ignore_pairs, int use_periodic,
                         int64_t n_ignore_groups, const int32_t* ignore_group_pairs,
                         const int32_t* group_vec, int* group_out);
/* LennardJonesRepulsiveForceFieldGenerator(cutoff_ratio, epsilons, sigmas, ...)
 * (LennardJonesRepulsiveForceFieldGenerator.cpp:9-115). */
int ocm_add_lennard_jones_repulsive(ocm_system* sys, double cutoff_ratio,
                                    const double* epsilons, const double* sigmas,
                                    int64_t n_ignore, const int64_t* ignore_pairs,
                                    int use_periodic, int64_t n_ignore_groups,
                                    const int32_t* ignore_group_pairs,
                                    const int32_t* group_vec, int* group_out);
/* LennardJonesAttractiveForceFieldGenerator(cutoff_ratio, epsilons, sigmas, ...)
 * (LennardJonesAttractiveForceFieldGenerator.cpp:9-124), switching from
 * 0.9 cutoff to cutoff. */
int ocm_add_lennard_jones_attractive(ocm_system* sys, double cutoff_ratio,
                                     const double* epsilons, const double* sigmas,
                                     int64_t n_ignore, const int64_t* ignore_pairs,
                                     int use_periodic, int64_t n_ignore_groups,
                                     const int32_t* ignore_group_pairs,
                                     const int32_t* group_vec, int* group_out);

/* WeeksChandlerAndersenForceFieldGenerator(sigmas, epsilons, ignore_list,
 * use_periodic, ignore_group_pairs, group_vec)
 * (WeeksChandlerAndersenForceFieldGenerator.cpp:9-113):
 * step(2^(1/6) s - r) (4 e ((s/r)^12 - (s/r)^6) + e), s the arithmetic and e
 * the geometric mean, cutoff 2^(1/6) (s_max + s_2nd) / 2.  It shares the
 * repulsive Lennard-Jones pair slot: a system holds at most one of
 * LennardJonesRepulsive, WeeksChandlerAndersen, UniformWeeksChadlerAndersen
 * (else OCM_ERR_UNSUPPORTED).  NaN sigma and epsilon = no participation. */
int ocm_add_weeks_chandler_andersen(ocm_system* sys, const double* sigmas, const double* epsilons,
                                    int64_t n_ignore, const int64_t* ignore_pairs, int use_periodic,
                                    int64_t n_ignore_groups, const int32_t* ignore_group_pairs,
                                    const int32_t* group_vec, int* group_out);
/* UniformWeeksChandlerAndersenForceFieldGenerator(system_size, eps, sigma,
 * former_group_vec, latter_group_vec, ignore_list, use_periodic,
 * ignore_group_pairs, group_vec)
 * (UniformWeeksChandlerAndersenForceFieldGenerator.cpp:9-185):
 * 4 eps ((sigma/r)^12 - (sigma/r)^6 + 1/4) for pairs between the `former`
 * and `latter` particle lists, cutoff 2^(1/6) sigma; force group
 * "UniformWeeksChadlerAndersen" (the reference's spelling). */
int ocm_add_uniform_weeks_chandler_andersen(ocm_system* sys, double eps, double sigma,
                                            int64_t n_former, const int64_t* former,
                                            int64_t n_latter, const int64_t* latter,
                                            int64_t n_ignore, const int64_t* ignore_pairs,
                                            int use_periodic, int64_t n_ignore_groups,
                                            const int32_t* ignore_group_pairs,
                                            const int32_t* group_vec, int* group_out);
/* UniformLennardJonesAttractiveForceFieldGenerator(system_size, eps, sigma,
 * cutoff_ratio, former_group_vec, latter_group_vec, ...)
 * (UniformLennardJonesAttractiveForceFieldGenerator.cpp:11-189): the
 * attractive Lennard-Jones form with one sigma and epsilon, cutoff
 * sigma * cutoff_ratio, switched from 0.9 cutoff; shares the attractive
 * Lennard-Jones pair slot (one per system). */
int ocm_add_uniform_lennard_jones_attractive(ocm_system* sys, double eps, double sigma,
                                             double cutoff_ratio, int64_t n_former,
                                             const int64_t* former, int64_t n_latter,
                                             const int64_t* latter, int64_t n_ignore,
                                             const int64_t* ignore_pairs, int use_periodic,
                                             int64_t n_ignore_groups,
                                             const int32_t* ignore_group_pairs,
                                             const int32_t* group_vec, int* group_out);
/* CappedGoContactForceFieldGenerator(indices, ks, r0s, capping_ratio,
 * use_periodic) (CappedGoContactForceFieldGenerator.hpp:14-47, .cpp:5-31):
 * k (5 (r0/r)^12 - 6 (r0/r)^10) for r > cap r0, below it the linear
 * continuation k (slope r / r0 + intercept) with slope = -60 (cap^-13 -
 * cap^-11), intercept = 65 cap^-12 - 66 cap^-10. */
int ocm_add_capped_go_contact(ocm_system* sys, int64_t n, const int64_t* indices, const double* ks,
                              const double* r0s, double capping_ratio, int use_periodic,
                              int* group_out);

/* ---------------------------------------------------------------------------
 * Plain single-system path.  ocm_context_create replaces
 * LangevinIntegratorGenerator::generate (IntegratorGenerator.cpp:5-14:
 * LangevinIntegrator(T, friction, dt) + setRandomNumberSeed) followed by
 * OpenMM::Context(system, integrator, platform) (Simulator.cpp:17).
 * ------------------------------------------------------------------------ */
typedef struct ocm_context ocm_context;
int ocm_context_create(const ocm_system* sys, double temperature, double friction,
                       double step_size, int32_t seed, int device, ocm_context** out);
void ocm_context_destroy(ocm_context* ctx);
/* Context::setPositions (Simulator.cpp:41); xyz is 3*n doubles (nm). */
int ocm_context_set_positions(ocm_context* ctx, const double* xyz);
int ocm_context_get_positions(ocm_context* ctx, double* xyz);
int ocm_context_set_velocities(ocm_context* ctx, const double* v);
int ocm_context_get_velocities(ocm_context* ctx, double* v);
/* Context::setVelocitiesToTemperature(T, seed) (Simulator.hpp:57-58). */
int ocm_context_set_velocities_to_temperature(ocm_context* ctx, double temperature,
                                              int32_t seed);
/* Context::getState(Forces|Energy, false, groups) (Observer.cpp:339-341):
 * forces (3*n, kJ/mol/nm) and the potential energy (kJ/mol) of the force
 * groups set in the mask.  Either output may be NULL. */
int ocm_context_get_state(ocm_context* ctx, uint32_t groups, double* forces,
                          double* potential_energy);
/* One fused evaluation returning the energy of every force group
 * (energies[OCM_MAX_GROUPS]); replaces one getState call per group. */
int ocm_context_get_group_energies(ocm_context* ctx, double* energies);
/* Kinetic energy (kJ/mol) of the current (half-step) velocities. */
int ocm_context_get_kinetic_energy(ocm_context* ctx, double* kinetic_energy);
/* LangevinIntegrator::step(steps) (Simulator.cpp:60). */
int ocm_context_step(ocm_context* ctx, int64_t steps);
/* OpenMM::LocalEnergyMinimizer::minimize(context, tolerance, maxIterations)
 * as the reference's Simulator calls it (Simulator.cpp:41-46): a
 * limited-memory BFGS on the potential energy until the RMS of all force
 * components is <= tolerance (kJ/mol/nm; the reference uses OpenMM's
 * default 10) or max_iterations (0: no limit) iterations are done.  The
 * context keeps the minimised positions; velocities are untouched.
 * iterations_out may be NULL. */
int ocm_context_minimize(ocm_context* ctx, double tolerance, int64_t max_iterations,
                         int64_t* iterations_out);
/* Engine of ocm_context_step.  0 (default): a non-periodic system of at
 * most 512 beads runs as a one-system persistent launch of the batched
 * kernel (its whole chunk of steps in one SM's shared memory, no per-step
 * launches; the state moves device-to-device between the context and the
 * one-slot batch), every other system on the cluster-pair tiles; 1: always
 * the tiles; 2: always the one-system kernel (non-periodic, at most 2048
 * beads, else OCM_ERR_UNSUPPORTED).  Both engines evaluate the same force
 * field with the same Langevin noise stream; trajectories differ by FP32
 * rounding.  Evaluations (get_state, energies, minimisation) always use the
 * tiles.  OpenMM has no counterpart: a Platform picks its kernels itself. */
int ocm_context_set_engine(ocm_context* ctx, int32_t mode);
/* Why the last ocm_context_minimize stopped and the RMS force it reached
 * (kJ/mol/nm, may be NULL).  *reason: 0 the RMS force reached the
 * tolerance; 1 the iteration limit; 2 the energy stopped changing (twenty
 * accepted steps in a row below 1e-12 relative: the FP32 force noise floor,
 * so a tolerance under that floor is not reached); 3 no step along the
 * search direction lowered the energy.  OpenMM's LocalEnergyMinimizer
 * reports none of this (the reference calls it and goes on,
 * src/Simulator.cpp:41-46).  OCM_ERR_STATE before any minimisation. */
int ocm_context_minimize_report(ocm_context* ctx, int32_t* reason, double* rms_force);

typedef struct ocm_context_stats {
    int64_t steps_done;
    int64_t list_builds;
    int64_t tiles;            /* cluster-pair tiles in the current list */
    int64_t masked_tiles;     /* tiles carrying exclusion masks */
    int32_t rebuild_interval; /* steps between list builds */
    int32_t reordered;        /* 1 if beads are sorted into column clusters */
    double  skin;             /* nm */
    double  max_cutoff;       /* nm */
    double  tile_cutoff;      /* nm: largest cutoff the cluster-pair tiles serve */
    int64_t charged_pairs;    /* entries of the charged-pair list (0 without one) */
    int32_t charged_split;    /* 1 if Debye-Hueckel runs on its own charged-pair list */
    int32_t one_system;       /* 1 if the last step call ran on the one-system batched kernel */
} ocm_context_stats;
int ocm_context_get_stats(ocm_context* ctx, ocm_context_stats* out);
/* Rebuild interval / skin overrides (0 keeps the current value). */
int ocm_context_set_list_options(ocm_context* ctx, int32_t rebuild_interval, double skin);
/* Debug/verification: every pair (i<j, original indices) that the tile list
 * makes the nonbonded kernel test AND that passes the FP32 cutoff test of
 * the largest cutoff the tiles serve (stats.tile_cutoff), followed, when
 * Debye-Hueckel runs on its own charged-pair list (stats.charged_split),
 * by the listed charged pairs that pass its FP32 cutoff test; written to
 * out_pairs.  Used to prove the lists are bit-exact against brute force. */
int ocm_context_list_pairs(ocm_context* ctx, int64_t* out_pairs, int64_t capacity,
                           int64_t* n_out);
/* Debug/verification: the bead order of the cluster layout (sorted slot ->
 * original index, -1 for padding); n_out = padded bead count. */
int ocm_context_cluster_order(ocm_context* ctx, int64_t* order, int64_t capacity,
                              int64_t* n_out);

/* ---------------------------------------------------------------------------
 * Batched / served path: many independent systems (up to
 * max_beads_per_system beads each) advanced together by one persistent
 * kernel launch per chunk of steps; every system keeps its state resident
 * in device memory between chunks.  No counterpart in the reference.
 * ------------------------------------------------------------------------ */
typedef struct ocm_batch ocm_batch;
int ocm_batch_create(int device, int64_t max_systems, int64_t max_total_beads,
                     int32_t max_beads_per_system, ocm_batch** out);
void ocm_batch_destroy(ocm_batch* batch);
/* Device bytes a system of this shape occupies in a batch (admission control). */
int64_t ocm_batch_footprint(const ocm_system* sys);
/* Copy a system and its state into a free slot.  velocities may be NULL:
 * then they are drawn at `temperature` from `seed` like
 * setVelocitiesToTemperature.  n_steps is the number of steps to run.
 * Returns OCM_ERR_OUT_OF_MEMORY if no slot or bead capacity is free. */
int ocm_batch_admit(ocm_batch* batch, const ocm_system* sys, const double* positions,
                    const double* velocities, double temperature, double friction,
                    double step_size, int32_t seed, int64_t n_steps, int64_t* slot_out);
/* ocm_batch_admit for a trajectory that already ran steps_done of its
 * n_steps steps (preemption / resume): with the positions and velocities
 * read back from the slot it left (ocm_batch_get_positions /
 * ocm_batch_get_velocities) and the same seed, the Langevin noise stream
 * continues at step steps_done and the trajectory is the one it would have
 * followed without the interruption.  The reference restarts a run from the
 * TOML pos / vel keys instead (src/input/ReadTOMLInput.cpp:908-962). */
int ocm_batch_admit_resume(ocm_batch* batch, const ocm_system* sys, const double* positions,
                           const double* velocities, double temperature, double friction,
                           double step_size, int32_t seed, int64_t n_steps, int64_t steps_done,
                           int64_t* slot_out);
/* Advance every admitted, unfinished system by min(steps_per_launch,
 * remaining) steps with one persistent launch; asynchronous with respect
 * to the host unless sync != 0.  A system whose force, velocity or
 * position becomes non-finite, or whose force exceeds 1e9 kJ/mol/nm in a
 * component, stops at that step and is reported by ocm_batch_slot_status;
 * the other systems of the launch are not affected. */
int ocm_batch_run(ocm_batch* batch, int32_t steps_per_launch, int sync);
/* Wait for the last launch and list the slots whose systems have finished:
 * every step done, or stopped because the system blew up (see
 * ocm_batch_slot_status). */
int ocm_batch_finished(ocm_batch* batch, int64_t* slots, int64_t capacity, int64_t* n_out);
/* Balanced launches (on != 0; off by default): in each ocm_batch_run the
 * costliest unfinished system advances steps_per_launch steps and every
 * other one proportionally more (by its bead count, up to 64x), so that a
 * launch keeps every SM busy until its end instead of waiting for the
 * largest system.  A system's trajectory does not depend on how its steps
 * are split into launches.  Meant for a serving loop; the ensemble
 * benchmark keeps every system in step. */
int ocm_batch_set_balanced(ocm_batch* batch, int on);
/* Tuning knob of the persistent kernel (set by the autotuner; results do not
 * depend on it): when a launch has at least two systems per CTA and the
 * systems a CTA claims have at most `beads` beads, the CTA splits into two
 * groups of half its threads, each with half of its shared memory,
 * advancing two systems at a time (default 512; 0 = never split; capped so
 * that a system's state fits half of the CTA's shared memory). */
int ocm_batch_set_split(ocm_batch* batch, int32_t beads);
/* Wait for the last launch; *status = OCM_OK, or OCM_ERR_NONFINITE if the
 * slot's system blew up (it is no longer advanced; its state is the one of
 * the failing step).  The reference terminates the whole run in that case
 * (src/OpenAICG2Plus.cpp:84-93). */
int ocm_batch_slot_status(ocm_batch* batch, int64_t slot, int32_t* status);
int ocm_batch_get_positions(ocm_batch* batch, int64_t slot, double* xyz);
int ocm_batch_get_velocities(ocm_batch* batch, int64_t slot, double* v);
/* Replace the positions (and, if v is not NULL, velocities) of n slots in
 * one host->device copy; xyz (and v) hold the slots' beads back to back in
 * the order of `slots` (3 x the slots' total beads values each).  The
 * positions are checked on the device: a non-finite one returns
 * OCM_ERR_NONFINITE and no slot changes.  Returns after the copy, so the
 * host buffers may be reused at once. */
int ocm_batch_set_positions_many(ocm_batch* batch, int64_t n, const int64_t* slots,
                                 const double* xyz, const double* v);
/* Read the positions of n slots, back to back in the order of `slots`, in
 * one device->host copy. */
int ocm_batch_get_positions_many(ocm_batch* batch, int64_t n, const int64_t* slots, double* xyz);
/* Same read-out as ocm_batch_get_positions_many, without allocating device
 * memory: no counterpart in the reference.
 *
 * ocm_batch_get_positions_many grows its device staging buffers with
 * cudaMalloc/cudaFree when a call needs more than any earlier one.  Callers
 * that cannot allocate use this one instead: a serving loop that admits work
 * against a fixed device-memory budget (an allocation there can fail or
 * fragment the budget), and a host thread reading results while other
 * streams of the device run (cudaMalloc/cudaFree may synchronise the
 * device).  Its scratch is a fixed set of file-scope device arrays in the
 * library (about 3 MiB per device), so it has fixed limits: at most 131072
 * beads and 2048 slots per call; larger requests return
 * OCM_ERR_INVALID_ARGUMENT with the limit in ocm_last_error().
 *
 * The first call on each device does a one-time set-up (it looks up the
 * scratch addresses with that device current); make that first call before
 * any stream capture.  Nothing in the scratch needs to start at zero: every
 * call writes all of the scratch it reads.  The scratch is shared by every
 * batch on the device, so calls that overlap in time (from several host
 * threads) race on it and must be serialised by the caller. */
int ocm_batch_get_positions_many_noalloc(ocm_batch* batch, int64_t n, const int64_t* slots,
                                         double* xyz);
int ocm_batch_steps_done(ocm_batch* batch, int64_t slot, int64_t* steps);
/* Forces (3*n) and per-group energies (OCM_MAX_GROUPS) of one slot at its
 * current positions, evaluated by the batched kernel.  Returns
 * OCM_ERR_NONFINITE (with the outputs filled) if a force is non-finite or
 * exceeds 1e9 kJ/mol/nm in a component. */
int ocm_batch_get_state(ocm_batch* batch, int64_t slot, uint32_t groups, double* forces,
                        double* energies);
/* Free a slot (its beads' capacity is returned to the pool). */
int ocm_batch_retire(ocm_batch* batch, int64_t slot);
int ocm_batch_active(ocm_batch* batch, int64_t* n_active, int64_t* beads_active);
/* Device milliseconds of the last ocm_batch_run (CUDA events on its stream). */
int ocm_batch_last_run_ms(ocm_batch* batch, double* ms);
/* Launch shape of the persistent kernel: threads per CTA (256, 512 or
 * 1024); the number of resident CTAs per SM follows from occupancy.  Set
 * by the autotuner; results do not depend on it. */
int ocm_batch_set_threads(ocm_batch* batch, int32_t threads_per_cta);
/* Shared memory per CTA given to neighbour lists, in KiB (the rest of the
 * SM's unified memory stays L1 cache for the static parameters); -1 = all
 * that fits.  Set by the autotuner; results do not depend on it. */
int ocm_batch_set_list_smem(ocm_batch* batch, int32_t kib);
int ocm_batch_get_threads(ocm_batch* batch, int32_t* threads_per_cta);
/* Neighbour-list statistics of a slot: list builds during its last chunk
 * and the list capacity (entries per bead). */
int ocm_batch_slot_stats(ocm_batch* batch, int64_t slot, int32_t* list_builds,
                         int32_t* list_capacity);

#ifdef __cplusplus
}
#endif

#endif /* OCM_GB300_H */
