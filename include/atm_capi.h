/*
 * atm_capi.h -- C ABI of the GB300-native ATMMetaForce evaluation path.
 *
 * Plain C types only (pointers, sizes, doubles); every function returns an
 * ATM_* status code (0 = success) and atm_last_error() gives the message of the
 * most recent failure on the calling thread.  Reference citations are paths in
 * the reference plugin (Gallicchio-Lab/openmm-atmmetaforce-plugin) of the
 * interface each entry point stands in for.
 *
 * Object model (mirrors OpenMM's, which the reference plugs into):
 *   atm_force_t      ATMMetaForce                   openmmapi/include/ATMMetaForce.h:54-315
 *   atm_nonbonded_t  the inner NonbondedForce the ATM force re-evaluates
 *                    (ATMMetaForceImpl.cpp:32-67 clones it into the inner systems)
 *   atm_system_t     System: particles, default box, forces (owned, as in OpenMM)
 *   atm_context_t    one evaluation context on one GPU (ATMMetaForceImpl +
 *                    CalcATMMetaForceKernel, ATMMetaForceKernels.h:15-59)
 *   atm_batch_t      R replicas (systems of any sizes) evaluated by one CUDA graph
 */
#ifndef ATM_CAPI_H
#define ATM_CAPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define ATM_OK 0
#define ATM_ERR_INVALID_ARGUMENT 1 /* bad value or null pointer */
#define ATM_ERR_INDEX 2            /* index out of range (ASSERT_VALID_INDEX, ATMMetaForce.cpp:18,27) */
#define ATM_ERR_STATE 3            /* call not valid in the current state */
#define ATM_ERR_CUDA 4             /* CUDA runtime / cuFFT failure */
#define ATM_ERR_UNSUPPORTED 5      /* feature outside this implementation */
#define ATM_ERR_OVERFLOW 6         /* device-side capacity exceeded and not recoverable */
#define ATM_ERR_PARSE 7            /* malformed or unsupported XML (ATMMetaForceProxy.cpp:44) */
#define ATM_ERR_GROUP 8            /* ATM group among the variable groups (ATMMetaForceImpl.cpp:78-79) */
#define ATM_ERR_PARTICLES 9        /* particle count/index changed (ReferenceATMMetaForceKernels.cpp:147-154) */
#define ATM_ERR_CONSTRAINTS 10     /* constraint iterations did not converge (MD driver) */

/* ---- nonbonded methods (OpenMM NonbondedForce::NonbondedMethod numbering) -- */
#define ATM_NB_NOCUTOFF 0
#define ATM_NB_CUTOFF_NONPERIODIC 1
#define ATM_NB_CUTOFF_PERIODIC 2
#define ATM_NB_PME 4

/* ---- global parameter indices (ATMMetaForce.h:151-218) -------------------- */
#define ATM_LAMBDA1 0
#define ATM_LAMBDA2 1
#define ATM_ALPHA 2
#define ATM_U0 3
#define ATM_W0 4
#define ATM_UMAX 5
#define ATM_UBCORE 6
#define ATM_ACORE 7
#define ATM_DIRECTION 8
#define ATM_NUM_GLOBALS 9

/* ---- per-replica result record (atm_batch_get_results) -------------------- */
#define ATM_RES_ENERGY 0      /* e0 + W, the ATMMetaForce energy (ReferenceATMMetaForceKernels.cpp:98) */
#define ATM_RES_PERT 1        /* soft-cored perturbation energy usc (:86) */
#define ATM_RES_SP 2          /* dW/du (:101) */
#define ATM_RES_W 3           /* softplus bias energy W (:89-94) */
#define ATM_RES_U 4           /* raw u = U2-U1 (dir>0) or U1-U2 (:84) */
#define ATM_RES_E0 5          /* U1 (dir>0) or U2 (:85) */
#define ATM_RES_BFP 6         /* dW/dusc (:95) */
#define ATM_RES_FP 7          /* dusc/du (:35) */
#define ATM_RES_E1 8          /* U_var at x */
#define ATM_RES_E2 9          /* U_var at x + d */
#define ATM_RES_DW_DLAMBDA1 10
#define ATM_RES_DW_DLAMBDA2 11
#define ATM_RES_DW_DALPHA 12
#define ATM_RES_DW_DU0 13
#define ATM_RES_DW_DW0 14
#define ATM_RES_STATUS 15     /* device status word (0 = ok) */
#define ATM_RES_DWDU 16       /* dW/du of the W actually computed (lambda2 fp when alpha = 0) */
#define ATM_NUM_RES 17

typedef struct atm_force_s* atm_force_t;
typedef struct atm_nonbonded_s* atm_nonbonded_t;
typedef struct atm_system_s* atm_system_t;
typedef struct atm_context_s* atm_context_t;
typedef struct atm_batch_s* atm_batch_t;

/* Message of the last failure on this thread ("" if none). */
const char* atm_last_error(void);
/* ATMMetaForce::Version(), ATMMetaForce.h:223-227 / ATMMetaForceVersion.h:4. */
const char* atm_version(void);
/* ATMMetaForce::Lambda1() ... Direction(), ATMMetaForce.h:151-218; which = ATM_LAMBDA1..ATM_DIRECTION. */
const char* atm_global_name(int which);

/* ---- ATMMetaForce (ATMMetaForce.h:54-315, ATMMetaForce.cpp:12-44) --------- */
/* Constructor, ATMMetaForce.h:79-83. */
int atm_force_create(double lambda1, double lambda2, double alpha, double u0, double w0, double umax,
                     double ubcore, double acore, double direction, const int* variable_groups, int n_groups,
                     atm_force_t* out);
/* Frees a force that was never added to a system (a system owns its forces). */
int atm_force_destroy(atm_force_t force);
/* addParticle, ATMMetaForce.h:104 / ATMMetaForce.cpp:12-15. */
int atm_force_add_particle(atm_force_t force, int particle, double dx, double dy, double dz, int* index);
/* getParticleParameters, ATMMetaForce.h:113 / ATMMetaForce.cpp:17-24. */
int atm_force_get_particle_parameters(atm_force_t force, int index, int* particle, double* dx, double* dy, double* dz);
/* setParticleParameters, ATMMetaForce.h:122 / ATMMetaForce.cpp:26-32. */
int atm_force_set_particle_parameters(atm_force_t force, int index, int particle, double dx, double dy, double dz);
/* getNumParticles, ATMMetaForce.h:90-92. */
int atm_force_get_num_particles(atm_force_t force, int* n);
/* getDefaultLambda1() ... getDefaultDirection(), ATMMetaForce.h:232-290; which = ATM_LAMBDA1.. */
int atm_force_get_default(atm_force_t force, int which, double* value);
/* getVariableForceGroups, ATMMetaForce.h:295-297: writes min(cap, n) groups, n to *n. */
int atm_force_get_variable_force_groups(atm_force_t force, int* groups, int cap, int* n);
/* Force::setForceGroup / getForceGroup / setName / getName (OpenMM base class). */
int atm_force_set_force_group(atm_force_t force, int group);
int atm_force_get_force_group(atm_force_t force, int* group);
int atm_force_set_name(atm_force_t force, const char* name);
int atm_force_get_name(atm_force_t force, char* buf, size_t cap, size_t* len);
/* usesPeriodicBoundaryConditions, ATMMetaForce.h:135-137 (always 0). */
int atm_force_uses_periodic_boundary_conditions(atm_force_t force, int* uses);
/* updateParametersInContext, ATMMetaForce.h:130 / CommonATMMetaForceKernels.cpp:229-251. */
int atm_force_update_parameters_in_context(atm_force_t force, atm_context_t context);
/* getPerturbationEnergy, ATMMetaForce.h:145 / ATMMetaForceImpl.cpp:124-125. */
int atm_force_get_perturbation_energy(atm_force_t force, atm_context_t context, double* value);
/* XmlSerializer::serialize<ATMMetaForce> through ATMMetaForceProxy::serialize,
 * serialization/src/ATMMetaForceProxy.cpp:11-40.  Writes a NUL-terminated
 * document of at most cap bytes; *len = bytes needed (excluding NUL). */
int atm_force_serialize(atm_force_t force, char* buf, size_t cap, size_t* len);
/* ATMMetaForceProxy::deserialize, ATMMetaForceProxy.cpp:42-79. */
int atm_force_deserialize(const char* xml, atm_force_t* out);

/* ---- inner NonbondedForce (OpenMM NonbondedForce, cloned by ATMMetaForceImpl.cpp:58-63) --- */
int atm_nonbonded_create(atm_nonbonded_t* out);
int atm_nonbonded_destroy(atm_nonbonded_t nb);
int atm_nonbonded_add_particle(atm_nonbonded_t nb, double charge, double sigma, double epsilon, int* index);
int atm_nonbonded_set_particle_parameters(atm_nonbonded_t nb, int index, double charge, double sigma, double epsilon);
int atm_nonbonded_get_particle_parameters(atm_nonbonded_t nb, int index, double* charge, double* sigma, double* epsilon);
int atm_nonbonded_get_num_particles(atm_nonbonded_t nb, int* n);
/* An exception replaces the pair's interaction (chargeProd 0 and epsilon 0 = exclusion). */
int atm_nonbonded_add_exception(atm_nonbonded_t nb, int i, int j, double charge_prod, double sigma, double epsilon,
                                int* index);
int atm_nonbonded_get_num_exceptions(atm_nonbonded_t nb, int* n);
int atm_nonbonded_set_method(atm_nonbonded_t nb, int method);
int atm_nonbonded_set_cutoff(atm_nonbonded_t nb, double cutoff);
int atm_nonbonded_set_reaction_field_dielectric(atm_nonbonded_t nb, double eps_rf);
int atm_nonbonded_set_ewald_error_tolerance(atm_nonbonded_t nb, double tol);
/* alpha = 0 selects OpenMM's rule from the tolerance and the system's default box. */
int atm_nonbonded_set_pme_parameters(atm_nonbonded_t nb, double alpha, int nx, int ny, int nz);
int atm_nonbonded_set_use_dispersion_correction(atm_nonbonded_t nb, int use);
int atm_nonbonded_set_force_group(atm_nonbonded_t nb, int group);
int atm_nonbonded_get_force_group(atm_nonbonded_t nb, int* group);

/* ---- System --------------------------------------------------------------- */
int atm_system_create(atm_system_t* out);
int atm_system_destroy(atm_system_t sys);
int atm_system_add_particle(atm_system_t sys, double mass, int* index);
int atm_system_get_num_particles(atm_system_t sys, int* n);
/* Orthorhombic boxes: a = (ax,0,0), b = (0,by,0), c = (0,0,cz). */
int atm_system_set_default_periodic_box_vectors(atm_system_t sys, const double* a, const double* b, const double* c);
/* System::addForce: the system takes ownership of the force object. */
int atm_system_add_nonbonded(atm_system_t sys, atm_nonbonded_t nb);
int atm_system_add_atm_force(atm_system_t sys, atm_force_t force);

/* Terms the MD driver integrates alongside the ATM force (the group-0 forces of
 * python/tests/test_abfe.py:55-103).  They do not enter contexts or batches. */
/* System::addConstraint: fixed distance (nm); clusters of at most 4 particles /
 * 6 constraints (rigid water, X-H bonds). */
int atm_system_add_constraint(atm_system_t sys, int i, int j, double distance, int* index);
int atm_system_get_num_constraints(atm_system_t sys, int* n);
/* HarmonicBondForce::addBond: (k/2)(r - length)^2, kJ/mol/nm^2. */
int atm_system_add_bond(atm_system_t sys, int i, int j, double length, double k);
/* HarmonicAngleForce::addAngle: (k/2)(theta - angle)^2 at vertex j, radians, kJ/mol/rad^2. */
int atm_system_add_angle(atm_system_t sys, int i, int j, int l, double angle, double k);
/* ATMMetaForceUtils.addVsiteRestraintForceCMCM (python/ATMMetaForceUtils.py:79-138):
 * (kf/2) step(d - tol)(d - tol)^2, d = |c1 - offset - c2|, c the mass-weighted
 * centroids of g1 (ligand) and g2 (receptor), no periodic image. */
int atm_system_add_centroid_restraint(atm_system_t sys, int n1, const int* g1, int n2, const int* g2, double kf,
                                      double tol, const double* offset);
/* ATMMetaForceUtils.addPosRestraints (python/ATMMetaForceUtils.py:707-752):
 * 0.5 fc step(d - tol)(d - tol)^2, d the distance to (x0,y0,z0), periodic
 * (minimum image) unless set_position_restraints_periodic(0). */
int atm_system_add_position_restraint(atm_system_t sys, int particle, double x0, double y0, double z0, double fc,
                                      double tol);
int atm_system_set_position_restraints_periodic(atm_system_t sys, int periodic);

/* ---- Context: one replica on one GPU -------------------------------------- */
/* properties: "key=value;key=value".  Keys: DifferencePath=0|1 (default 0, two
 * full inner evaluations as in ATMMetaForceImpl.cpp:113,116); ListSkin=nm
 * (default 0: the pair lists are built at every evaluation; > 0: built at the
 * cutoff plus the skin and kept until an atom has moved more than half the skin,
 * which the GPU checks at every evaluation); FusedTiles=0|1 (default 0: the
 * pair lists and the pair tiles as two kernels; 1: one persistent kernel that
 * builds each row's lists and evaluates its tiles at once; the autotuner chooses
 * between them); SpreadByOwner=0|1 (default 1: PME charges spread once per atom,
 * by the grid brick that holds its stencil base, and the bricks summed into
 * integer grids; 0: every brick spreads each atom whose stencil touches it; the
 * grids, and so every result, are the same bits either way); SpreadBrick=n (the
 * spreading brick edge in grid points, 0: each atom's stencil added straight into
 * the integer grid by atomics; the autotuner chooses among 20, 19, 16, 12 and 0;
 * same bits in every case). */
int atm_context_create(atm_system_t sys, int device, const char* properties, atm_context_t* out);
int atm_context_destroy(atm_context_t ctx);
/* Context::setPositions (host doubles, n x 3, nm). */
int atm_context_set_positions(atm_context_t ctx, const double* pos, int n);
int atm_context_set_periodic_box_vectors(atm_context_t ctx, const double* a, const double* b, const double* c);
/* Context::setParameter / getParameter for the ATM globals, which the force
 * registers as context parameters with their defaults (ATMMetaForceImpl.cpp:130-142). */
int atm_context_set_parameter(atm_context_t ctx, const char* name, double value);
int atm_context_get_parameter(atm_context_t ctx, const char* name, double* value);
/* Context::getState(getEnergy, getForces, groups): energy and forces (n x 3,
 * host, nullable) of the forces whose group bit is set in groups_mask
 * (ATMMetaForceImpl.cpp:103: the ATM force contributes only when its group
 * is requested; :113,116,119-122: its forces are merged even if forces are not
 * requested). */
int atm_context_get_state(atm_context_t ctx, int groups_mask, double* energy, double* forces);
/* Last per-replica result record (ATM_NUM_RES doubles). */
int atm_context_get_results(atm_context_t ctx, double* results);

/* ---- Batch: R replicas in one CUDA graph ----------------------------------- */
/* systems[r] each hold one NonbondedForce and one ATMMetaForce (copied; the
 * systems stay owned by the caller).  properties as for contexts
 * (DifferencePath defaults to 1 here). */
int atm_batch_create(const atm_system_t* systems, int n_replicas, int device, const char* properties,
                     atm_batch_t* out);
int atm_batch_destroy(atm_batch_t b);
int atm_batch_get_num_replicas(atm_batch_t b, int* r);
int atm_batch_get_num_particles(atm_batch_t b, int replica, int* n);
int atm_batch_set_positions(atm_batch_t b, int replica, const double* pos);
int atm_batch_set_parameter(atm_batch_t b, int replica, const char* name, double value);
int atm_batch_set_periodic_box_vectors(atm_batch_t b, int replica, const double* a, const double* b_, const double* c);
/* One evaluation of every replica.  pos_all (nullable: keep the stored
 * positions) holds the replicas' positions back to back (host, nm); energies
 * (R), forces (sum n_r x 3, host) and results (R x ATM_NUM_RES) are nullable. */
int atm_batch_evaluate(atm_batch_t b, const double* pos_all, double* energies, double* forces, double* results);
/* Same with device pointers on the caller's CUDA stream (cudaStream_t as void*). */
int atm_batch_evaluate_device(atm_batch_t b, const double* d_pos_all, double* d_forces, double* d_results,
                              void* stream);
/* R x R matrix of beta * (e0_r + W_s(u_r)): replica r's coordinates under
 * replica s's alchemical parameters, from the last evaluation. */
int atm_batch_energy_matrix(atm_batch_t b, double beta, double* matrix);
/* No counterpart in the reference.  The list skin, and how many evaluations ran
 * and how many of them built the pair lists (nullable outputs). */
int atm_batch_get_list_info(atm_batch_t b, double* skin, long long* evaluations, long long* builds);
/* Per-replica displacement vectors (n x 3), as ATMMetaForce::setParticleParameters
 * + updateParametersInContext (ATMMetaForce.cpp:26-40) for a batch replica. */
int atm_batch_set_displacements(atm_batch_t b, int replica, const double* displ);
/* Per-replica NonbondedForce charges, sigmas, epsilons (n each). */
int atm_batch_set_nonbonded_parameters(atm_batch_t b, int replica, const double* charge, const double* sigma,
                                       const double* epsilon);
/* No counterpart in the reference (the adjoint of the ATM energy).  Gradients of
 * L = sum_r g[r] W_r, W the softplus bias energy of the last evaluation, with
 * respect to positions and displacements (sum n x 3), charges, sigmas, epsilons
 * (sum n) and the 5 parameters lambda1, lambda2, alpha, u0, w0 (R x 5).  The
 * batch must have been created with "Adjoint=1" for the charge/sigma/epsilon
 * terms.  Device pointers on the given stream; every output is nullable. */
int atm_batch_backward_device(atm_batch_t b, const double* d_g, double* d_dx, double* d_dd, double* d_dq,
                              double* d_dsig, double* d_deps, double* d_dparams, void* stream);
/* Same with host buffers. */
int atm_batch_backward(atm_batch_t b, const double* g, double* dx, double* dd, double* dq, double* dsig,
                       double* deps, double* dparams);

/* ---- MD: Langevin dynamics of R replicas ------------------------------------ */
/* OpenMM's LangevinIntegrator (leapfrog: v <- a v + (1-a)/g f/m + sqrt(kT(1-a^2)/m) N,
 * a = exp(-g dt); x' = x + dt v, constrained; v = (x' - x)/dt) stepping the ATM
 * force plus each system's bonds, angles and restraints, as the reference's
 * tests and examples do with integrator.setIntegrationForceGroups({0, ATM group})
 * (python/tests/test_abfe.py:96-103, example/abfe/abfe.py:94-101).  systems as
 * for atm_batch_create, plus masses (mass 0: the particle does not move).
 * properties: DifferencePath=0|1 (default 1), ReorderInterval=steps (default
 * 0: re-sort when the pair-tile count has grown by 20 %), ListSkin=nm|auto
 * (default 0.1, reduced to what the boxes allow; auto: chosen by
 * atm_md_autotune before the first step),
 * CheckInterval=steps (default 20: the host reads the list status every that
 * many steps instead of after every step, and redoes the steps since the last
 * check if a list build overflowed), FusedTiles=0|1, SpreadByOwner=0|1 and
 * SpreadBrick=n (as for contexts).
 * temperature K, friction 1/ps, step_size ps; seed keys the Philox4x32-10
 * thermostat noise. */
typedef struct atm_md_s* atm_md_t;
int atm_md_create(const atm_system_t* systems, int n_replicas, int device, const char* properties,
                  double temperature, double friction, double step_size, unsigned long long seed, atm_md_t* out);
int atm_md_destroy(atm_md_t md);
/* No counterpart in the reference.  Times the evaluation's launch space, then
 * `trials` steps at each pair-list skin from 0 to 0.2 nm, keeps the fastest and
 * writes a report (NUL-terminated, at most cap bytes; *len = bytes needed).  The
 * positions, velocities, step count and recording are restored afterwards. */
int atm_md_autotune(atm_md_t md, int trials, char* report, size_t cap, size_t* len);
/* No counterpart in the reference.  The list skin in use, how many evaluations
 * ran, how many of them built the pair lists, and how many list checks sent the
 * state back to their snapshot (nullable outputs). */
int atm_md_get_list_info(atm_md_t md, double* skin, long long* evaluations, long long* builds, int* redos);
int atm_md_get_num_particles(atm_md_t md, int* n_total);
/* Positions / velocities of every replica back to back (host, n_total x 3). */
int atm_md_set_positions(atm_md_t md, const double* pos);
int atm_md_set_velocities(atm_md_t md, const double* vel);
/* Maxwell-Boltzmann velocities at temperature (K) from the seed's Philox stream. */
int atm_md_set_velocities_to_temperature(atm_md_t md, double temperature, unsigned long long seed);
int atm_md_set_parameter(atm_md_t md, int replica, const char* name, double value);
int atm_md_set_integrator(atm_md_t md, double temperature, double friction, double step_size);
int atm_md_step(atm_md_t md, int steps);
/* Host outputs, each nullable: positions, velocities (v at t - dt/2), total forces
 * (n_total x 3); per replica potential energy (bonded + restraints + ATM) and
 * kinetic energy (velocities shifted by dt/2 f/m, as OpenMM's leapfrog
 * integrators report it); results (R x ATM_NUM_RES) of the ATM evaluation at
 * the current positions. */
int atm_md_get_state(atm_md_t md, double* pos, double* vel, double* forces, double* potential, double* kinetic,
                     double* results);
/* Steps taken, re-sorts made, and per replica degrees of freedom
 * (3 x particles with mass - constraints; dof nullable, R entries). */
int atm_md_get_info(atm_md_t md, long long* steps, int* reorders, int* dof);
/* No counterpart in the reference (its scripts read the perturbation energy from
 * the context after each MD cycle, example/abfe/abfe.py:108-131).  Streaming of
 * the thermodynamic data of the ATM replicas: every `interval` steps (0: off) the
 * result records (R x ATM_NUM_RES: u, W, dW/dlambda1, dW/dlambda2, ...) and the
 * R x R reduced-energy matrix at beta = 1/kT are copied on the device into a
 * ring of `capacity` records, with no host synchronisation.  get_records copies
 * the kept records oldest first (steps, results R x ATM_NUM_RES each, matrices
 * R x R each; outputs nullable, sized for max_records) and empties the ring. */
int atm_md_set_recording(atm_md_t md, int interval, int capacity);
int atm_md_get_records(atm_md_t md, long long* steps, double* results, double* matrices, int max_records,
                       int* n_records);

/* ---- allocation-free variant ------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * code whose device memory all comes from its own pool or arena, or that runs
 * where new allocations are forbidden (a budget already handed out, an
 * allocator that must not be re-entered, a step that must not pay allocation
 * latency).  Reaction-field (CutoffPeriodic) NonbondedForce energy and forces
 * of n <= 16384 particles, every pair within the cutoff except the excluded
 * ones, on the current device and the given stream.  All pointers except box
 * are device pointers the caller owns: d_pos (n x 3 nm), d_charge, d_sigma,
 * d_epsilon (n each), excluded partners as CSR (d_excl_start[n+1], d_excl,
 * both directions listed), outputs d_energy (1, kJ/mol) and d_forces (n x 3,
 * kJ/mol/nm); box = 3 host doubles (orthorhombic edges, each >= 2 cutoff).
 * It allocates nothing: its scratch (about 400 KB of fixed-point force
 * accumulators and energy partials) is a static device array that every GPU
 * loading the library holds until exit, cleared at the start of every call.
 * The first call on a device looks up that array's address; make that first
 * call before any stream capture.  Calls that overlap on the GPU (other
 * streams, other threads) share the array and race.  Larger n returns
 * ATM_ERR_INVALID_ARGUMENT. */
int atm_rf_nonbonded_noalloc(int n, const double* d_pos, const double* d_charge, const double* d_sigma,
                             const double* d_epsilon, const int* d_excl_start, const int* d_excl, const double* box,
                             double cutoff, double eps_rf, double* d_energy, double* d_forces, void* stream);

/* ---- autotuner -------------------------------------------------------------- */
/* No counterpart in the reference.  Times `trials` evaluations per configuration
 * of the launch space (pair-tile CTAs per SM and register variant, the fused
 * list + pair-tile kernel, PME spreading brick edge 12/16/19/20, PME chain on its
 * own stream or in line) on the stored positions and keeps the
 * fastest; with use_cache a choice stored for the same GPU and workload (file
 * $ATM_AUTOTUNE_CACHE, else ~/.cache/atm_gb300_autotune.txt) is reused.  The
 * report (one line per configuration) is written to report (nullable). */
int atm_batch_autotune(atm_batch_t b, int trials, int use_cache, char* report, size_t cap, size_t* len);

/* ---- diagnostics ------------------------------------------------------------ */
/* Timings (ms) of the kernels of the last evaluate() when profiling is on. */
int atm_batch_set_profiling(atm_batch_t b, int on);
int atm_batch_get_kernel_times(atm_batch_t b, char* names, size_t names_cap, double* ms, int cap, int* n);
/* Number of the library's own kernel launches per evaluation. */
int atm_batch_get_launch_count(atm_batch_t b, int* n);
/* Pair tiles of the last evaluation, tile rows, and the largest row (nullable outputs). */
int atm_batch_get_stats(atm_batch_t b, int* tiles, int* rows, int* max_row);

#ifdef __cplusplus
}
#endif
#endif
