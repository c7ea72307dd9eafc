/*
 * sdm_capi.h -- C ABI of the GB300 (sm_103a) SDM two-state force.
 *
 * One call evaluates, for every replica (lambda state) of every registered
 * system, what one step of the reference's SDM integrator computes on the
 * nonbonded force group:
 *
 *   U0, F0   at the original coordinates x
 *            (reference: calcForcesAndEnergy(true,true,4) followed by SaveState1,
 *             openmmapi/src/LangevinIntegratorSDM.cpp:159-162)
 *   U1, F1   at the displaced coordinates x+d
 *            (MakeState2 + calcForcesAndEnergy + SaveState2 + RestoreState1,
 *             LangevinIntegratorSDM.cpp:165-173; displacement
 *             platforms/reference/src/ReferenceSDMKernels.cpp:192-199)
 *   u = U1-U0, u' = SoftCoreF(u), W(u'), W'(u'), E_pot = U0 + W
 *            (LangevinIntegratorSDM.cpp:125-149; ReferenceSDMKernels.cpp:247-287)
 *   F = (1-s) F0 + s F1 with s = W' * du'/du
 *            (ReferenceSDMKernels.cpp:309-318; OpenCL sdmForce, langevin.cl:72-87)
 *   dW/dlambda of the non-equilibrium schedule
 *            (ReferenceSDMKernels.cpp:231-245,289-302)
 *
 * The Langevin update and the group-1 (bonded/restraint) forces stay with the
 * caller: the caller adds its own group-1 energy to E_pot and its group-1
 * forces to F, exactly as the reference adds them at
 * ReferenceSDMKernels.cpp:283 and :315-317.
 *
 * Nonbonded model (the part of OpenMM's NonbondedForce the reference calls
 * with CutoffPeriodic + reaction field, example/desmonddmsfile75.py:424-438):
 * Lennard-Jones (Lorentz-Berthelot mixing, truncated, unshifted) plus
 * reaction-field Coulomb, orthorhombic periodic box, excluded pairs skipped,
 * no dispersion correction.
 *
 * Conventions: nm, kJ/mol, e.  Coordinates, energies and forces are FP64 at
 * the ABI.  Pair arithmetic is FP32 on the GPU, forces accumulate in 64-bit
 * fixed point (scale 2^32, the OpenMM-CUDA convention), energies in FP64.
 * Replicas are numbered system by system: system 0's replicas first.
 * No function throws; every function returns an sdm_status.  One host
 * thread per handle at a time.
 */
#ifndef SDM_CAPI_H
#define SDM_CAPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int sdm_status;
enum {
    SDM_OK = 0,
    SDM_ERR_INVALID_ARGUMENT = 1,  /* bad pointer, size, index or parameter */
    SDM_ERR_CUDA = 2,              /* a CUDA runtime call failed; see sdm_last_error */
    SDM_ERR_NO_DEVICE = 3,         /* no usable sm_103 device */
    SDM_ERR_OVERFLOW = 4,          /* fixed-point force overflow or non-finite pair term */
    SDM_ERR_CAPACITY = 5,          /* a diagnostic buffer was too small */
    SDM_ERR_UNKNOWN_METHOD = 6,    /* bias or soft-core method id not 0,1,2 */
    SDM_ERR_TIMEOUT = 7            /* a bounded device wait expired */
};

/* Bias and soft-core method ids: the reference's integer constants
 * (openmmapi/include/LangevinIntegratorSDM.h:120-122 and :143-145). */
enum { SDM_LINEAR = 0, SDM_QUADRATIC = 1, SDM_ILOGISTIC = 2 };
enum { SDM_NO_SOFTCORE = 0, SDM_TANH_SOFTCORE = 1, SDM_RATIONAL_SOFTCORE = 2 };

/* Per-replica SDM parameters, SDM_NPARAMS doubles in this order.  Each field
 * is the value of the reference integrator setter named beside it
 * (openmmapi/include/LangevinIntegratorSDM.h). */
enum {
    SDM_P_BIAS_METHOD = 0,      /* setBiasMethod        :127 */
    SDM_P_SOFTCORE_METHOD = 1,  /* setSoftCoreMethod    :146 */
    SDM_P_LAMBDA = 2,           /* setLambda            :75  (Linear slope; t/Ntmax when non-equilibrium) */
    SDM_P_LAMBDA1 = 3,          /* setLambda1           :212 */
    SDM_P_LAMBDA2 = 4,          /* setLambda2           :218 */
    SDM_P_ALPHA = 5,            /* setAlpha             :224 (1/(kJ/mol)) */
    SDM_P_U0 = 6,               /* setU0                :230 */
    SDM_P_W0 = 7,               /* setW0coeff           :196 */
    SDM_P_GAMMA = 8,            /* setGamma             :161 */
    SDM_P_WB = 9,               /* setWBcoeff           :178 */
    SDM_P_UMAX = 10,            /* setUmax              :350 */
    SDM_P_ACORE = 11,           /* setAcore             :359 */
    SDM_P_UBCORE = 12,          /* setUbcore            :369 */
    SDM_P_NONEQ = 13,           /* setNonEquilibrium    :393 */
    SDM_P_M_LAMBDA1 = 14,       /* setlambda1Slope      :403 */
    SDM_P_M_LAMBDA2 = 15,       /* setlambda2Slope      :409 */
    SDM_P_M_U0 = 16,            /* setu0Slope           :415 */
    SDM_P_M_W0 = 17,            /* setw0Slope           :421 */
    SDM_P_B_LAMBDA1 = 18,       /* setlambda1intercept  :427 */
    SDM_P_B_LAMBDA2 = 19,       /* setlambda2intercept  :433 */
    SDM_P_B_U0 = 20,            /* setu0intercept       :439 */
    SDM_P_B_W0 = 21,            /* setw0intercept       :445 */
    SDM_NPARAMS = 22
};

/* Per-replica results, SDM_NRESULTS doubles in this order. */
enum {
    SDM_R_U0 = 0,        /* state-1 (original coordinates) nonbonded energy */
    SDM_R_U1 = 1,        /* state-2 (displaced coordinates) nonbonded energy = U0 + u */
    SDM_R_U = 2,         /* perturbation energy u = U1 - U0, accumulated directly */
    SDM_R_BINDE = 3,     /* u' = SoftCoreF(u): the reference's getBindE() */
    SDM_R_FP = 4,        /* du'/du */
    SDM_R_W = 5,         /* bias energy W(u') ("ebias") */
    SDM_R_DW = 6,        /* W'(u') ("bfp") */
    SDM_R_S = 7,         /* force mixing weight s = W' * du'/du ("sp") */
    SDM_R_EPOT = 8,      /* U0 + W: the reference's getPotEnergy() without group 1 */
    SDM_R_DWDLAMBDA = 9, /* non-equilibrium dW/dlambda (0 unless SDM_P_NONEQ == 1) */
    SDM_R_LAMBDA1 = 10,  /* parameters actually used (after the non-equilibrium schedule) */
    SDM_R_LAMBDA2 = 11,
    SDM_R_U0PARAM = 12,
    SDM_R_W0PARAM = 13,
    SDM_R_STATUS = 14,   /* device status bits of this call (0 = clean) */
    SDM_R_RESERVED = 15,
    SDM_NRESULTS = 16
};

typedef struct sdm_handle sdm_handle;

/* Topology of one system.  All arrays are read during sdm_create only. */
typedef struct {
    int num_particles;
    const double* charge;        /* [num_particles] e */
    const double* sigma;         /* [num_particles] nm */
    const double* epsilon;       /* [num_particles] kJ/mol */
    int num_exclusions;          /* excluded pairs (each unordered pair once) */
    const int* exclusions;       /* [2*num_exclusions] particle indices */
    const double* displacement;  /* [3*num_particles] nm, NULL = all zero */
    double box[3];               /* orthorhombic periodic box edges, nm */
    double cutoff;               /* nm; must satisfy cutoff < box/2 in every axis */
    double reaction_field_dielectric;
    int num_replicas;            /* coordinate sets (lambda states) per call, >= 1 */
    /* Exceptions: pairs with their own parameters (OpenMM NonbondedForce
     * exceptions, e.g. the 1-4 pairs the reference's DMS reader adds from
     * pair_12_6_es_term, example/desmonddmsfile75.py:813-848).  Each pair must
     * also be in the exclusion list.  E = K qq/r + 4 eps ((sigma/r)^12 -
     * (sigma/r)^6) on the caller's coordinates: no cutoff, no reaction field,
     * no periodic image.  Zero-initialised fields: no exceptions. */
    int num_exceptions;
    const int* exception_pairs;     /* [2*num_exceptions] particle indices */
    const double* exception_params; /* [3*num_exceptions] charge product (e^2), sigma (nm), epsilon (kJ/mol) */
    /* Electrostatics: SDM_NB_REACTION_FIELD (0, default) or SDM_NB_PME (smooth
     * particle-mesh Ewald as OpenMM's NonbondedForce.PME, the reference's
     * explicit-solvent setup, example/test_explicit.py:64).  PME: splitting
     * beta = sqrt(-ln(2 tol))/cutoff with tol = ewald_tolerance (0: 5e-4),
     * grid pme_grid (0: the smallest 2,3,5,7-smooth n >= 2 beta L/(3 tol^0.2)),
     * B-spline order 5; reaction_field_dielectric is ignored. */
    int nonbonded_method;
    double ewald_tolerance;
    int pme_grid[3];
} sdm_system_desc;

#define SDM_NB_REACTION_FIELD 0
#define SDM_NB_PME 1

/* Creates a handle for num_systems systems on CUDA device `device`, owning all
 * device memory and one CUDA stream.  Replaces the reference's kernel
 * construction and initialize(): ReferenceSDMKernelFactory.cpp:58-63,
 * ReferenceSDMKernels.cpp:144-159, OpenCLSDMKernels.cpp:73-133. */
sdm_status sdm_create(const sdm_system_desc* systems, int num_systems, int device,
                      sdm_handle** out);

/* Releases every resource of the handle.  NULL is accepted. */
sdm_status sdm_destroy(sdm_handle* h);

/* Message of the last failing call on this handle ("" if none).  With a NULL
 * handle: the message of the last failing sdm_create or sdm_evaluate_noalloc
 * on this thread. */
const char* sdm_last_error(const sdm_handle* h);

/* Number of replicas over all systems. */
sdm_status sdm_num_replicas(const sdm_handle* h, int* out);

/* Replaces the displacement map of one system ([3*num_particles] nm).
 * Reference: LangevinIntegratorSDM::setDisplacement
 * (openmmapi/include/LangevinIntegratorSDM.h:467) with the upload of
 * OpenCLSDMKernels.cpp:86-97. */
sdm_status sdm_set_displacement(sdm_handle* h, int system, const double* displacement);

/* Sets the SDM parameters of one replica (SDM_NPARAMS doubles, see above).
 * Rejects unknown bias/soft-core method ids with SDM_ERR_UNKNOWN_METHOD (the
 * reference throws "Unknown soft core method", LangevinIntegratorSDM.cpp:147). */
sdm_status sdm_set_params(sdm_handle* h, int replica, const double* params);

/* Host-buffer evaluation of all replicas.
 *   x        [sum over replicas of 3*num_particles] FP64 coordinates
 *   results  [num_replicas * SDM_NRESULTS] (may be NULL)
 *   forces   [sum over replicas of 3*num_particles] mixed force F (may be NULL)
 * Copies in, evaluates, copies out and synchronises (SDM_OPT_ZERO_COPY: read
 * page-locked coordinates in place).  Replaces one SDM step's
 * force part: LangevinIntegratorSDM.cpp:158-176 with
 * ReferenceSDMKernels.cpp:202-318 (minus the Langevin update). */
sdm_status sdm_evaluate(sdm_handle* h, const double* x, double* results, double* forces);

/* Device-buffer evaluation, asynchronous on `stream` (a cudaStream_t, NULL =
 * the handle's own stream).  x/results/forces are device pointers with the
 * sizes of sdm_evaluate.  With graph mode on (default), the launch sequence is
 * captured once per distinct (x, results, forces, stream) tuple and replayed
 * as a CUDA graph.  The default streams (cudaStreamLegacy, cudaStreamPerThread)
 * cannot be captured: given one of them, the call runs on the handle's own
 * stream, ordered after the caller's earlier work on it and before its later
 * work (two event edges); the same holds for every entry point below that
 * takes a stream and evaluates (sdm_langevin_step, sdm_evaluate_engine). */
sdm_status sdm_evaluate_device(sdm_handle* h, const double* x, double* results, double* forces,
                               void* stream);

/* Per-state forces of the last evaluation (device pointers or host pointers
 * selected by `on_device`): F0 and F1 = F0 + dF, [sum 3*num_particles] each. */
sdm_status sdm_get_state_forces(sdm_handle* h, double* F0, double* F1, int on_device);

/* The same per-state forces into device buffers, asynchronous on `stream`
 * (NULL = the handle's own stream), which must be the stream of the last
 * evaluation or ordered after it.  Either pointer may be NULL.  The
 * reference's counterparts are its saved state forces (SaveState1/SaveState2,
 * platforms/reference/src/ReferenceSDMKernels.cpp:161-190). */
sdm_status sdm_get_state_forces_device(sdm_handle* h, double* F0, double* F1, void* stream);

/* Langevin dynamics on the SDM force (the caller side of the path).  One
 * sdm_langevin_step step = the two-state evaluation of every replica, then the
 * stochastic-dynamics update of platforms/reference/src/
 * ReferenceStochasticDynamicsSDM.cpp:131-266 on the hybrid force of
 * ReferenceSDMKernels.cpp:309-318 (+ f_extra, e.g. the group-1 bonded and
 * restraint forces the reference adds, ReferenceSDMKernels.cpp:310-316):
 *   v <- vscale v + fscale F/m + noise N(0,1)/sqrt(m);  x' = x + dt v;
 *   v <- (x' - x)/dt;  x <- x'
 * vscale = exp(-dt friction), fscale = (1 - vscale)/friction, noise =
 * sqrt(2 kT friction) sqrt((1 - vscale^2)/(2 friction)).  Replaces
 * IntegrateLangevinStepSDMKernel::execute (SDMKernels.h:47-113) and
 * LangevinIntegratorSDM::step (LangevinIntegratorSDM.cpp:153-183) with one
 * CUDA graph per step and no host synchronisation.  Constraints are not
 * applied (the reference applies the context's constraint algorithm). */
typedef struct {
    double step_size;        /* ps */
    double friction;         /* 1/ps, > 0 */
    double temperature;      /* K, >= 0 (0: no noise) */
    unsigned long long seed; /* counter-based generator key */
} sdm_langevin_params;

/* Sets the integrator parameters; `step` is the generator's step counter
 * (advanced by one on the device after every step). */
sdm_status sdm_set_langevin(sdm_handle* h, const sdm_langevin_params* params, unsigned long long step);

/* nsteps steps on device buffers, asynchronous on `stream` (NULL: the
 * handle's stream):
 *   x        [3*total particles] FP64 positions, updated in place
 *   v        [3*total particles] FP64 velocities (nm/ps), updated in place
 *   inv_mass [total particles] 1/m (mol/g); 0 holds a particle fixed
 *   f_extra  [3*total particles] forces added to the SDM force (may be NULL)
 *   results  [num_replicas * SDM_NRESULTS] the last step's energies
 * No counterpart in the reference's C++ API beyond the step above. */
sdm_status sdm_langevin_step(sdm_handle* h, double* x, double* v, const double* inv_mass,
                             const double* f_extra, double* results, int nsteps, void* stream);

/* ------------------------------------------------------------------------ *
 * Group-1 restraints of the reference's SDMUtils (python/SDMUtils.py), as
 * the reference builds them for LangevinIntegratorSDM's group 1: evaluated
 * on the device in the same call, on the caller's coordinates x (no
 * periodic images, like the reference's custom forces).  Units: nm, rad,
 * kJ/mol.  Energies enter SDM_R_EPOT (and sdm_get_restraint_energies);
 * forces enter F, and the state forces F0 and F1 alike (they do not depend
 * on the SDM state).
 *
 * Centroid restraint (SDMUtils.py:32-157, CustomCentroidBondForce):
 *   lambda_r (kfcm/2) step(d - tolcm) (d - tolcm)^2,
 *   d = |c_lig - offset - c_rcpt|, c = sum w_i x_i / sum w_i (the reference
 *   weights by particle mass: pass the masses as weights; NULL = 1).
 * With use_angles, three flat-bottom terms over the reference particles
 * r0 r1 r2 (receptor) and l0 l1 l2 (ligand), each
 *   lambda_r (kf/2) (step(dm) max(0, db)^2 + step(-dm) max(0, -da)^2),
 *   da, db, dm = the variable minus lo, hi, (lo + hi)/2 wrapped to (-P/2, P/2]:
 *   theta = angle(r0, l0, l1) (P = pi), phi1 = dihedral(r1, r0, l0, l1),
 *   phi2 = dihedral(r0, l0, l1, l2) (P = 2 pi); lo/hi = center -/+ tolerance.
 * lambda_r is SDMRestraintControlParameter (per replica, default 1).
 *
 * Alignment restraint (SDMUtils.py:160-257, CustomCompoundBondForce) between
 * reference particles a0 a1 a2 (ligand A) and b0 b1 b2 (ligand B):
 *   (kf_displ/2) |b0 - offset - a0|^2
 *   + (k_theta/2) (1 - cos theta), theta between b1 - b0 and a1 - a0
 *   + (k_psi/4) (1 - cos psi_b) + (k_psi/4) (1 - cos psi_a), psi_b between the
 *     components of b2 - b0 and a2 - a0 orthogonal to b1 - b0, psi_a the same
 *     with A and B exchanged.
 * ------------------------------------------------------------------------ */
typedef struct {
    int num_lig, num_rcpt;          /* centroid groups (either 0: no centroid restraint) */
    const int* lig_particles;       /* [num_lig] */
    const int* rcpt_particles;      /* [num_rcpt] */
    const double* lig_weights;      /* [num_lig] or NULL (all 1) */
    const double* rcpt_weights;     /* [num_rcpt] or NULL (all 1) */
    double kfcm, tolcm;             /* kJ/mol/nm^2, nm */
    double offset[3];               /* nm */
    int use_angles;                 /* 1: the angle / dihedral terms */
    int rcpt_ref[3], lig_ref[3];    /* r0 r1 r2, l0 l1 l2 */
    double kf_angle, angle_center, angle_tol;          /* kJ/mol/rad^2, rad, rad */
    double kf_dihedral1, dihedral1_center, dihedral1_tol;
    double kf_dihedral2, dihedral2_center, dihedral2_tol;
    int use_alignment;              /* 1: the alignment restraint */
    int liga_ref[3], ligb_ref[3];   /* a0 a1 a2, b0 b1 b2 */
    double kf_displ, k_theta, k_psi;                   /* kJ/mol/nm^2, kJ/mol, kJ/mol */
    double align_offset[3];         /* nm */
} sdm_restraints;

/* Restraints of system `system` (NULL removes them); applies to every
 * replica of the system from the next evaluation.  Reference:
 * SDMUtils.addRestraintForce / addAlignmentForce. */
sdm_status sdm_set_restraints(sdm_handle* h, int system, const sdm_restraints* r);
/* SDMRestraintControlParameter of one replica (reference: the global
 * parameter SDMUtils.py:99, Context::setParameter). */
sdm_status sdm_set_restraint_control(sdm_handle* h, int replica, double lambda_r);
/* Restraint energy of every replica at the last evaluation ([num_replicas]).
 * Synchronises. */
sdm_status sdm_get_restraint_energies(sdm_handle* h, double* energies);

/* Rigid 3-site waters in sdm_langevin_step: the constraint step the
 * reference's integrator applies between the position update and the
 * velocity recomputation (ReferenceStochasticDynamicsSDM.cpp:131-266, with
 * the OpenMM context's constraint algorithm), solved per water in closed
 * form (SETTLE, Miyamoto and Kollman, J. Comput. Chem. 13, 952 (1992)):
 * the unconstrained positions move along the old bond vectors, mass
 * weighted, until |O-H| = d_oh and |H-H| = d_hh; then v = (x' - x)/dt.
 * waters: [3 * num_waters] (O, H, H) particle indices of `system` (each
 * particle in at most one water; the hydrogens of a water share a mass).
 * Hydrogens are taken in the minimum image of their oxygen.  A water with a
 * fixed particle (1/m = 0) is left unconstrained.  num_waters = 0 removes
 * them.  Applies to every replica of the system. */
sdm_status sdm_set_rigid_waters(sdm_handle* h, int system, int num_waters, const int* waters, double d_oh,
                                double d_hh);

/* Reads and clears the device status word (SDM_DEV_* bits).  Synchronises. */
sdm_status sdm_check_status(sdm_handle* h, int* device_status);

/* Options. */
enum {
    SDM_OPT_GRAPH = 0,        /* 1 = capture/replay CUDA graphs in sdm_evaluate_device (default 1) */
    SDM_OPT_PROFILE = 1,      /* 1 = time every kernel with CUDA events (eager launches);
                                 2 = record the same events inside the replayed graph */
    SDM_OPT_SPLIT = 2,        /* work items per i-cluster in the pair kernel (1,2,4) */
    SDM_OPT_CTAS_PER_SM = 3,  /* persistent pair-kernel CTAs per SM (1..4, default 4); the launch
                                 never exceeds the CTAs that fit (SDM_OPT_PAIR_RESIDENT) */
    SDM_OPT_VERIFY = 4,       /* 1 = sdm_evaluate checks the device status word after each call */
    SDM_OPT_PAIR_RESIDENT = 5, /* read only: pair-kernel CTAs per SM that are resident for the
                                  current SDM_OPT_CTAS_PER_SM (occupancy calculator) */
    SDM_OPT_ZERO_COPY = 6,    /* 1 = sdm_evaluate reads page-locked coordinates (cudaHostAlloc /
                                 cudaHostRegister) in place instead of staging them through a
                                 device copy; results and forces are always copied out (default 0:
                                 on GB300 the two measured on par) */
    SDM_OPT_STAGE_CHUNK = 7,  /* cluster-pair list entries the main pass stages per chunk
                                 (cp.async into shared memory, two chunks ahead): 8, 12 (default)
                                 or 16.  Same pair sets and terms; the autotuner's tile-staging axis. */
    SDM_OPT_OVERLAP = 8,      /* 2 = the perturbation pass (changed pairs of the displaced particles),
                                 the exceptions, the PME reciprocal space and the combine (u, soft
                                 core, bias, mixing weight) run on a second stream branch beside the
                                 list build and the main pass, joined before the finalize (default);
                                 1 = the branch (without the reciprocal space; the combine then
                                 follows it on the main stream when the system has PME) joins
                                 before the main pass; 0 = one stream.  Identical results. */
    SDM_OPT_LIST_GROUP = 9    /* z-consecutive i-clusters of a column whose lists one warp of the list
                                 builder builds together (column searches and candidate boxes shared):
                                 1, 2, 4, or 0 = automatic (default: 4).  Identical lists. */
};
sdm_status sdm_set_option(sdm_handle* h, int option, int value);
sdm_status sdm_get_option(const sdm_handle* h, int option, int* value);

/* Kernel timings of the last profiled evaluation: names[i] (static strings)
 * and ms[i] for i < *count (in: capacity, out: entries). */
sdm_status sdm_get_kernel_times(const sdm_handle* h, const char** names, float* ms, int* count);

/* The schedule chosen by the autotuner. */
typedef struct {
    int stage_chunk;    /* SDM_OPT_STAGE_CHUNK */
    int ctas_per_sm;    /* SDM_OPT_CTAS_PER_SM */
    int split;          /* SDM_OPT_SPLIT */
    float ms;           /* median time of one whole evaluation (graph replay) with this choice */
    int from_cache;     /* 1: read from the cache file, nothing timed */
    int list_group;     /* SDM_OPT_LIST_GROUP (1, 2 or 4) */
    int overlap;        /* SDM_OPT_OVERLAP (0, 1 or 2) */
} sdm_tune_result;

/* Autotuner (no counterpart in the reference, which has one fixed OpenCL
 * schedule).  Times every staging chunk (8, 12, 16 list entries) x CTAs per
 * SM (3, 4) x split (1, 2) on coordinates x (device pointer), then, on the
 * fastest of those, the list-building group (1, 2, 4) and the graph's second
 * branch (SDM_OPT_OVERLAP 0, 1, 2): each candidate is a whole evaluation
 * replayed as a CUDA graph, 5 timed replays after 2 warm-up ones, median.
 * The fastest becomes the handle's setting.  With cache_path, the
 * choice is stored in that text file under the workload key of
 * sdm_tune_key, and a later call with the same key (another handle, another
 * process) takes it from there without timing.  Synchronises.  Returns
 * SDM_ERR_CAPACITY if the lists overflowed on x (evaluate once, then tune). */
sdm_status sdm_autotune_cached(sdm_handle* h, const double* x_device, const char* cache_path,
                               sdm_tune_result* out);

/* The cache key of a workload: mean particles per replica, mean density
 * (1/nm^3, one decimal), cutoff, replicas, systems, electrostatics and the
 * device's SM count.  Host only (no device needed). */
sdm_status sdm_tune_key(const sdm_system_desc* systems, int num_systems, int num_sms, char* key, int capacity);

/* sdm_autotune_cached without a cache file; writes the chosen split and CTAs
 * per SM. */
sdm_status sdm_autotune(sdm_handle* h, const double* x_device, int* split, int* ctas_per_sm);

/* Interaction counts of coordinates x (host pointer) under the kernels' own
 * pair rule: counts[2*r] = P0 (pairs within the cutoff at x), counts[2*r+1] =
 * P1delta (pairs within the cutoff at x+d whose displacements differ). */
sdm_status sdm_count_pairs(sdm_handle* h, const double* x, long long* counts);

/* Cell grid of one system: M[0..2] cells per axis (columns are M[0]*M[1]). */
sdm_status sdm_get_grid(const sdm_handle* h, int system, int* M);

/* Replaces charge/sigma/epsilon of n particles of one system (indices into
 * the system; values in nm, kJ/mol, e).  The reference sets them on OpenMM's
 * NonbondedForce (example/desmonddmsfile75.py:776-808); here they feed the
 * next evaluation and the adjoint. */
sdm_status sdm_set_particle_params(sdm_handle* h, int system, int n, const int* index,
                                   const double* charge, const double* sigma,
                                   const double* epsilon);

/* Adjoint of the last evaluation with respect to the parameters of the
 * displaced particles (no counterpart in the reference, whose only
 * derivative is the non-equilibrium dW/dlambda of ReferenceSDMKernels.cpp:289-302).
 * For every replica r, every displaced particle k of its system (ascending
 * particle index) and both states s (0: original, 1: displaced coordinates)
 * writes three FP64 sums over the interacting partners j of k in state s:
 *   out[((D_r + k)*2 + s)*3 + 0] = sum_j K q_j (1/r + krf r^2 - crf)   = dU_s/dq_k
 *   out[((D_r + k)*2 + s)*3 + 1] = sum_j d e_LJ / d sigma_k             = dU_s/dsigma_k
 *   out[((D_r + k)*2 + s)*3 + 2] = sum_j e_LJ(k,j)                       (= 2 eps_k dU_s/deps_k)
 * D_r = displaced particles of the replicas before r.  Host pointer;
 * synchronises.  The parameter gradient of U_lambda = U0 + W is
 * (1-s) dU_0 + s dU_1 with s = results[SDM_R_S]; the displacement gradient
 * is -s F1 (sdm_get_state_forces).  `out` holds 6 * sdm_get_num_perturbed
 * doubles. */
sdm_status sdm_adjoint(sdm_handle* h, double* out);

/* The same sums into a device buffer of 6 * sdm_get_num_perturbed doubles,
 * asynchronous on `stream` (a cudaStream_t, NULL = the handle's own stream).
 * The stream must be the one of the last evaluation, or ordered after it.
 * No counterpart in the reference (see sdm_adjoint). */
sdm_status sdm_adjoint_device(sdm_handle* h, double* out, void* stream);

/* Backward of the differentiable potential U_r = U0 + W(u') of every replica
 * (no counterpart in the reference), one launch on `stream`, device pointers.
 * Inputs: grad_u [nrep] = dL/dU_r; results [nrep * SDM_NRESULTS], forces
 * (mixed F) and forces1 (F1, sdm_get_state_forces_device) [3 * particles of
 * all replicas] and adjoint [6 * sdm_get_num_perturbed] (sdm_adjoint_device)
 * of the evaluation being differentiated; eps_displaced [sum over systems
 * of their displaced particles] their FP64 epsilon (NULL: the third
 * parameter gradient stays 2 eps dL/deps); bias_params [4 * nrep] rows of
 * lambda1, lambda2, alpha, u0 used by that evaluation (NULL: the handle's
 * current parameters).  Outputs (any may be NULL):
 *   grad_x    [3 * particles of all replicas]  -grad_u[r] F
 *   grad_d    [3 * particles of all systems]   -sum_r grad_u[r] s_r F1 over the system's replicas
 *   grad_p    [3 * displaced of all systems]   charge, sigma, epsilon: sum_r grad_u[r]
 *                                              ((1 - s_r) dU_0 + s_r dU_1)
 *   grad_bias [5 * nrep] rows: dL/dlambda1, dL/dlambda2, dL/dalpha, dL/du0, dL/dw0
 *             (partial derivatives of W at fixed u' = results[SDM_R_BINDE])
 * Sums over replicas run in index order (deterministic).  grad_p needs
 * reaction field (sdm_adjoint). */
sdm_status sdm_backward_device(sdm_handle* h, const double* grad_u, const double* results, const double* forces,
                               const double* forces1, const double* adjoint, const double* eps_displaced,
                               const double* bias_params, double* grad_x, double* grad_d, double* grad_p,
                               double* grad_bias, void* stream);

/* Number of (replica, displaced particle) entries of the adjoint output: the
 * sum over replicas of their system's particles with a nonzero displacement
 * under the current displacement maps.  No counterpart in the reference. */
sdm_status sdm_get_num_perturbed(const sdm_handle* h, int* count);

/* Diagnostic export of the clustering and neighbour lists of replica
 * `replica` for coordinates x (host pointer, that replica's 3*num_particles):
 *   perm[cap_slots]                slot -> particle (-1 = padding)
 *   ncl                            clusters
 *   cnt[cap_clusters]              list entries per i-cluster
 *   ent_slot/ent_mask[cap_clusters*cap_per_cluster]  (j slot, allowed-i bits)
 * Returns SDM_ERR_CAPACITY if a capacity is too small. */
sdm_status sdm_export_lists(sdm_handle* h, int replica, const double* x, int cap_slots,
                            int cap_clusters, int cap_per_cluster, int* perm, int* ncl, int* cnt,
                            int* ent_slot, unsigned char* ent_mask);

/* Allocation-free evaluation of ONE system (one coordinate set).  There is
 * no counterpart in the reference.
 *
 * For callers that cannot allocate device memory at the point where they
 * need a force: code recording into a CUDA graph (cudaMalloc is not allowed
 * while a stream is being captured), hosts whose memory manager owns every
 * device byte (a simulation engine's context, a framework's caching
 * allocator: an allocation behind their back breaks their accounting or
 * fails under a fixed budget), and latency-bound loops that cannot afford
 * the implicit device synchronisation of cudaMalloc/cudaFree.  This call
 * allocates nothing, on the device or on the host, and creates no handle.
 *
 * All scratch lives in one file-scope device array of
 * SDM_NOALLOC_SCRATCH_BYTES bytes that every GPU loading the library holds
 * until the process exits.  The first call on a device, with that device
 * current, looks up the array's device address once; make that first call
 * before any stream capture.  Every call shares the array: calls whose work
 * overlaps on the GPU (other streams, other host threads) race and corrupt
 * each other's results; serialise them.  Each call clears what must start at
 * zero itself.
 *
 * Limits: 1 <= num_particles <= SDM_NOALLOC_MAX_PARTICLES (else
 * SDM_ERR_INVALID_ARGUMENT, nothing launched); 0 < cutoff < box/2.  The
 * pair work is all-pairs (N^2), with the handle path's pair terms, 2^32
 * fixed-point forces and FP64 energies; the pair rule is the FP64 minimum
 * image rounded to FP32, so pairs within ~1e-7 nm of the cutoff may differ
 * from the handle path.
 *
 * Device pointers: x [3n], charge/sigma/epsilon [n], excl_offsets [n+1] and
 * excl_indices (symmetric CSR of excluded partners), displacement [3n] or
 * NULL, results [SDM_NRESULTS], forces [3n] or NULL (mixed force F).
 * Host pointers: box [3], params [SDM_NPARAMS].  Asynchronous on `stream`
 * (NULL = the legacy default stream); errors in the arguments are reported
 * through sdm_last_error(NULL). */
#define SDM_NOALLOC_MAX_PARTICLES 8192
#define SDM_NOALLOC_SCRATCH_BYTES 727296
sdm_status sdm_evaluate_noalloc(int num_particles, const double* x, const double* charge,
                                const double* sigma, const double* epsilon,
                                const int* excl_offsets, const int* excl_indices,
                                const double* displacement, const double* box, double cutoff,
                                double reaction_field_dielectric, const double* params,
                                double* results, double* forces, void* stream);

/* Interop with an engine that keeps its particles in its own order on the
 * device (OpenMM's CUDA platform: posq, atom index and the 64-bit
 * fixed-point force buffer; the reference's CUDA/OpenCL kernels read and
 * write those arrays directly, platforms/opencl/src/OpenCLSDMKernels.cpp:86-97
 * and platforms/cuda/src/kernels/langevin.cu:10,19-21).  Both calls are
 * asynchronous on `stream` (a cudaStream_t, NULL = the legacy default
 * stream) and take device pointers; errors in the arguments are reported
 * through sdm_last_error(NULL).
 *
 * sdm_gather_positions: for k < n, x[3*index[k] + c] = posq[k].c (+
 * posq_correction[k].c when not NULL, the FP32 remainder of mixed
 * precision), c = 0..2; posq and the correction are float4, or double4 when
 * double_precision is nonzero.  x is [3n] in the ABI's particle order. */
sdm_status sdm_gather_positions(const void* posq, const void* posq_correction, int double_precision,
                                const int* index, int n, double* x, void* stream);

/* sdm_scatter_forces_fixed: for k < n and c = 0..2,
 * buffer[c*padded_n + k] += round(forces[3*index[k] + c] * 2^32), with forces
 * in kJ/mol/nm in the ABI's order and buffer the engine's component-major
 * fixed-point accumulator. */
sdm_status sdm_scatter_forces_fixed(const double* forces, const int* index, int n, int padded_n,
                                    long long* buffer, void* stream);

/* One evaluation of a handle of one replica, fed from and into an engine's
 * device arrays in the engine's particle order: the positions are gathered
 * as by sdm_gather_positions (n = the handle's particle count), the call
 * evaluates as sdm_evaluate_device does into the handle's own buffers (a
 * captured graph), and the mixed force is added into `force_buffer` as by
 * sdm_scatter_forces_fixed (skipped when it is NULL).  This replaces the
 * reference kernel's Save/Make/Restore state copies and its force mix on the
 * engine's arrays (platforms/opencl/src/OpenCLSDMKernels.cpp:104-146,
 * 271-276; platforms/cuda/src/kernels/langevin.cu:10,19-21).
 *
 * results NULL: asynchronous on `stream`; a device status error (a list
 * overflow among them) stays in the status word for the next synchronous
 * call or sdm_check_status, and the forces added since then are incomplete.
 * results given (host, SDM_NRESULTS doubles): the call synchronises, a list
 * overflow regrows the lists and evaluates again before any force is added,
 * and another status error fails the call (SDM_OPT_VERIFY) with nothing
 * added.  No counterpart in the reference as one call. */
sdm_status sdm_evaluate_engine(sdm_handle* h, const void* posq, const void* posq_correction, int double_precision,
                               const int* index, int padded_n, long long* force_buffer, double* results,
                               void* stream);

/* Results of the last evaluation (host, SDM_NRESULTS doubles per replica);
 * synchronises the device.  The reference integrator's getters read its last
 * step the same way (openmmapi/include/LangevinIntegratorSDM.h:301-324). */
sdm_status sdm_get_last_results(sdm_handle* h, double* results);

/* Device status bits (sdm_check_status, SDM_R_STATUS). */
enum {
    SDM_DEV_FORCE_OVERFLOW = 1,   /* |force term| >= 2^31 kJ/mol/nm or NaN */
    SDM_DEV_ENERGY_NONFINITE = 2, /* NaN/Inf energy */
    SDM_DEV_EXCL_OVERFLOW = 4,    /* internal exclusion table overflow (should not happen) */
    SDM_DEV_LIST_OVERFLOW = 8,    /* a cluster-pair list exceeded its capacity; sdm_evaluate
                                     regrows and repeats, device callers see SDM_ERR_CAPACITY
                                     from sdm_check_status and call sdm_evaluate once */
    SDM_DEV_COORD_NONFINITE = 16  /* a coordinate is NaN or Inf (OpenMM raises for these; the
                                     particle drops out of the pair search, results are invalid) */
};

#ifdef __cplusplus
}
#endif
#endif /* SDM_CAPI_H */
