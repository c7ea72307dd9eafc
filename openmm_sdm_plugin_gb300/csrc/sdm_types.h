// sdm_types.h -- plain-old-data tables shared by the host orchestration
// (sdm_capi.cpp) and the CUDA kernels (sdm_kernels.cu).
//
// HBM layout (all per-replica arrays are concatenated replica after replica,
// each replica owning a fixed-capacity window computed at handle creation):
//
//   topology (per particle of every system, original order)
//     topo_q   float   q * sqrt(K_coulomb)            (so qi*qj carries K)
//     topo_hs  float   sigma / 2                      (sigma_ij = hs_i + hs_j)
//     topo_se  float   2 sqrt(epsilon)                (se_i*se_j = 4 eps_ij)
//     topo_grp int     displacement group (0 = not displaced)
//     topo_d   double3 displacement
//     excl_off/excl_idx  symmetric CSR of exclusions (system-local indices)
//   per replica, particle-indexed (window = num_particles)
//     w        double3 coordinates wrapped into the box
//     cellinfo int2    (column id, z cell)
//     inv      int     particle -> slot
//   per replica, column-indexed (window = ncol+1)
//     col_cnt, col_aoff (atom prefix), col_cl (cluster prefix)
//   per replica, cell-indexed (window = ncol*Mz+1; cell = column*Mz + z cell)
//     cel_cnt, cel_fill (counters), cel_off (atom prefix; a column's cells are consecutive)
//   per replica, slot-indexed (window = slot_cap = num_particles + 8*ncol + 8)
//     perm     int     slot -> particle (-1 padding)
//     clX      float4  cluster-local x,y,z (FP32) and q*sqrt(K)
//     clP      float2  sigma/2, 2 sqrt(eps)
//     grp      int     displacement group of the slot's particle
//     excl4    int4    up to 4 exclusion partners as slots (-1 none, -2 overflow)
//     clM      int     molecule (exclusion component) id of the slot's particle
//     F0x/F0y/F0z, dFx/dFy/dFz   int64 fixed point 2^32
//   per replica, cluster-indexed (window = slot_cap/8)
//     jl       int4[jl_cap]  cluster-pair list of the i-cluster, jl_cnt entries
//     cl_grp   int2    list-building groups: SDM_JG z-consecutive clusters of a column
//     cl_ref   int4    reference cell (cx, cy, cz) and column id
//     cl_bbc   float4  bounding-box centre (cluster frame)
//     cl_bbh   float4  bounding-box half extents
//     cl_link  int4[2] up to 8 clusters holding exclusion partners of this cluster (-1 none, -2 many)
//     cl_zb    float2  absolute z of the first / last particle (outward rounded)
//     e_part   double  main-pass energy of the cluster's work items
#pragma once
#include <stdint.h>

#define SDM_CL 8                 // particles per cluster
#define SDM_FIX_SCALE 4294967296.0 // 2^32 fixed point for forces
#define SDM_LIST_MARGIN 1.0e-4   // nm added to the cutoff in the list filter
#define SDM_MAX_SPLIT 4
#define SDM_JG 4                 // largest list-building group (i-clusters of one column, z-consecutive)
#define SDM_PERT_PARTS 2         // warps per perturbation item (stencil columns split between them)
// per-replica record of the combine (perturbation energy u, soft core, bias)
#define SDM_CMB_FIELDS 10

// Langevin parameter block (doubles; seed and step are stored as integer bits)
#define SDM_LV_DT 0
#define SDM_LV_VSCALE 1
#define SDM_LV_FSCALE 2
#define SDM_LV_NOISE 3
#define SDM_LV_INVDT 4
#define SDM_LV_SEED 5
#define SDM_LV_STEP 6
#define SDM_LV_COUNT 8

struct SdmSys {
    int n;            // particles
    int atom_base;    // offset into the topology arrays
    int excl_base;    // offset into excl_idx (excl_off is indexed atom_base + i, values are absolute)
    int M[3];         // cells per axis
    int ncol;         // M[0]*M[1]
    int stlo[2], sthi[2];  // stencil column offsets per axis (x,y)
    int img_static;   // 1 if the x/y extents already force per-pair minimum image
    float tz;         // z threshold: image mode unless max cluster z extent < tz
    double box[3], invL[3], g[3], invg[3];
    long long wrap_lim[3];  // bit pattern of L(1 - 2^-40): 0 <= v below it wraps to v itself
    double rc;
    float Lf[3], invLf[3];
    float gf[3];      // (float)g, for conservative prefilters only
    float rc2f;       // (float)(rc*rc): pair rule
    float rcl, rcl2f; // list filter cutoff (rc + margin) and its square
    float krf, crf;   // reaction-field constants (FP32)
    int nD;           // displaced particles
    int D_base;       // offset into D_idx
    int shift_base;   // offset into shift_tab: 3 tables of 2*Mk+1 floats (index n+Mk)
    int org_base;     // offset into cell_org: 3 tables of Mk doubles, c * g[k]
    int cx_base;      // offset into cx_off/cx_idx (changed-pair exclusions per displaced particle)
    int rep0, nrep;   // the system's replicas: rep0 .. rep0+nrep-1 (replicas are numbered system by system)
    int half_geo;     // 1: pairs of columns are owned through the forward half stencil
                      // (offset ox>0, or ox==0 and oy>0; own column J>=I); 0: by lower column id
    int excl_clique;  // 1: every exclusion component is a clique (excluded <=> same molecule id)
    int hst_base, hst_count;  // owner stencil (int2 column offsets), own column first
    int fst_base, fst_count;  // full stencil for point queries
    int ex_base, ex_count;    // exceptions: offset into ex_pair/ex_prm, count
    // PME (pme = 1): Ewald direct space replaces the reaction field
    int pme;
    float beta_f, c2_f;       // beta, 2 beta / sqrt(pi) (FP32 pair terms)
    double beta;
    double e_const;           // self + neutralising-background energy (constant)
    int xc_base, xc_count;    // excluded-pair corrections: offset into xc_pair/xc_qq, count
    int pme_grid[3];
    int pme_base;             // offset of this system's B-spline moduli * Ewald kernel in pme_bc
    float pme_gs[3];          // K / L: grid points per nm (FP32 stencils)
    int pme_bc[3];            // cells per side of a spreading / interpolation brick
    int pme_nb[3];            // bricks per dimension
    int pme_cap;              // grid points of a brick's shared-memory sub-grid
    // group-1 restraints (SDMUtils): rs_on bit 0 centroid, 1 angles, 2 alignment
    int rs_on;
    int rs_base, rs_nlig, rs_nrcpt;   // offset into rs_idx / rs_w (ligand group, then receptor group), counts
    int rs_prm;                       // offset of the system's SDM_RS_COUNT parameters in rs_prm
    int rs_ref[12];                   // r0 r1 r2 l0 l1 l2 (centroid angles), a0 a1 a2 b0 b1 b2 (alignment)
    // rigid waters in the Langevin step (sdm_set_rigid_waters)
    int st_base, st_count;            // offset into st_idx (triples), number of waters
    double st_doh, st_dhh;            // O-H and H-H distances (nm)
};

// restraint parameters (doubles per system)
enum {
    SDM_RS_KFCM = 0, SDM_RS_TOLCM = 1, SDM_RS_OFF = 2,            // + 3
    SDM_RS_INVW_LIG = 5, SDM_RS_INVW_RCPT = 6,
    SDM_RS_KFA = 7, SDM_RS_ALO = 8, SDM_RS_AHI = 9,
    SDM_RS_KFD1 = 10, SDM_RS_D1LO = 11, SDM_RS_D1HI = 12,
    SDM_RS_KFD2 = 13, SDM_RS_D2LO = 14, SDM_RS_D2HI = 15,
    SDM_RS_KDISPL = 16, SDM_RS_KTHETA = 17, SDM_RS_KPSI = 18, SDM_RS_AOFF = 19,   // + 3
    SDM_RS_COUNT = 24
};

// per perturbation item (replica, displaced particle, state): the wrapped
// position in that state, its cell and its cell-local FP32 coordinates
struct SdmPertPos {
    double y[3];
    int cy[3];
    float o[3];
};

struct SdmRep {
    int sys;
    int n;            // particles of the system
    long long x_off;  // particle offset into the concatenated coordinates / forces
    int atom_win;     // particle-indexed window base
    int col_win;      // column-indexed window base (ncol+1 per replica)
    int cel_win;      // cell-indexed window base (ncol*M[2]+1 per replica; cell = column*M[2] + z cell)
    int slot_win;     // slot window base
    int slot_cap;     // slots in the window
    int cl_win;       // cluster window base (slot_win/8)
    int pert_win;     // perturbation partial base (2*nD per replica)
    int ex_win;       // exception item base (ex_count per replica)
    int xc_win;       // excluded-pair correction item base (xc_count per replica)
    long long pg_win; // PME: offset of this replica's state-0 grid (its dQ grid follows)
    long long pg_size;  // PME: grid points of one grid
    long long ps_win; // PME: offset of this replica's state-0 spectrum (its dQ spectrum follows)
};

// Everything a kernel needs, passed by value (fits the 32 KB parameter space).
struct SdmArgs {
    int nsys, nrep;
    const SdmSys* sys;
    const SdmRep* rep;
    // topology
    const float* topo_q;
    const float* topo_hs;
    const float* topo_se;
    const int* topo_grp;
    const int* topo_mol;  // exclusion component (molecule) id
    const int4* topo_ex4; // up to 4 exclusion partners (system-local; -1 none, -2 more than 4)
    const double* topo_d;
    const int2* ex_pair;    // exceptions (system-local particle indices)
    const double4_16a* ex_prm;  // (K qq, sigma, 4 eps, 0)
    const int2* xc_pair;    // PME: excluded pairs (i < j, system-local) ...
    const float* xc_qq;     // ... and their K q_i q_j
    const int* excl_off;
    const int* excl_idx;
    const int* D_idx;     // system-local particle indices of displaced particles
    const int* cx_off;    // per displaced particle: changed-pair exclusion partners
    const int* cx_idx;
    const float* shift_tab;
    const double* cell_org;  // cell origins c * g[k] (FP64, as the kernels would compute them)
    const double* params; // nrep * SDM_NPARAMS
    // input / output
    const double* x;      // concatenated coordinates
    double* results;      // nrep * SDM_NRESULTS (device or mapped host memory)
    double* s_rep;        // nrep: mixing weight s of the last combine (device)
    double* cmb;          // nrep * SDM_CMB_FIELDS: u and the combine terms of the last evaluation
    // Langevin step (sdm_langevin_step): positions lv_x are also the evaluation's x
    double* lv_x;         // [3 * total particles] updated in place
    double* lv_v;         // [3 * total particles] updated in place
    const double* lv_invm;  // [total particles] inverse masses (0: particle held fixed)
    const double* lv_fext;  // [3 * total particles] forces added to the SDM force (may be null)
    double* lv_prm;       // SDM_LV_* (device): dt, vscale, fscale, noise scale, 1/dt, seed, step
    double* forces;       // mixed forces (may be null)
    double* F0out;        // optional per-state forces
    double* F1out;
    // scratch
    double* w;
    int2* cellinfo;
    int* inv;
    int* col_cnt;        // particles per column (written by k_scan)
    int* cel_cnt;        // particles per cell (counter)
    int* cel_fill;       // bucket fill per cell (counter)
    int* cel_off;        // particle prefix per cell within the replica
    int* col_aoff;
    int* col_cl;
    int* bucket;
    int* perm;
    float4* clX;
    float2* clP;
    int* grp;
    int4* excl4;
    int* clM;            // per slot: molecule id (clique exclusion mode)
    unsigned long long* F0x;
    unsigned long long* F0y;
    unsigned long long* F0z;
    unsigned long long* dFx;
    unsigned long long* dFy;
    unsigned long long* dFz;
    int4* cl_ref;
    float4* cl_bbc;
    float4* cl_bbh;
    int4* cl_link;
    float2* cl_zb;       // per cluster: absolute z of its first and last particle (-/+ 1e-4 nm)
    const int2* stencil; // column offset tables (see SdmSys hst/fst)
    int4* jl;            // cluster-pair lists: cl window * jl_cap entries (J|needmask<<31, Sx, Sy, Sz)
    int* jl_cnt;         // entries per i-cluster (may exceed jl_cap: overflow)
    int jl_cap;
    double* e_part;      // cl window * SDM_MAX_SPLIT
    double* p_part;      // perturbation partials
    double* ex_e0;       // per exception item: energy at x
    double* ex_du;       // per exception item: E(x+d) - E(x) (0 when d_i = d_j)
    double* xc_e0;       // per replica x xc block (PME): sums of -K qq erf(beta r)/r at x
    double* xc_du;       // ... and of its change at x+d
    int xc_blocks;       // blocks of 256 excluded pairs per replica (largest system)
    // PME reciprocal space
    const float* pme_charge;        // q sqrt(K) per particle (the topology charges)
    unsigned long long* pme_acc;    // fixed-point spread grids (2 per replica)
    float* pme_grid;                // float grids: spread charges, then potentials
    float2* pme_spec;               // half spectra (2 per replica)
    const float* pme_theta;         // per system: Ewald kernel x B-spline moduli, half spectrum
    double* pme_epart;              // per replica x convolution block: state-0 energy partials
    double* pme_du;                 // per displaced particle: reciprocal part of u
    long long pme_total_grid;       // grid points over all grids
    int pme_conv_blocks;
    int4* pme_brick;                // per replica x brick: {sub-grid origin, state}, {extents, 0}
    int pme_max_bricks;             // bricks per replica (largest system)
    int pme_smem;                   // dynamic shared memory of the brick kernels (bytes)
    SdmPertPos* pert_pos; // per perturbation item (total_pert entries)
    double* adj;         // adjoint sums: 3 per perturbation item
    // group-1 restraints
    const int* rs_idx;      // restraint group particles of every system
    const double* rs_w;     // their centroid weights
    const double* rs_prm;   // SDM_RS_COUNT parameters per system
    const double* rs_lam;   // per replica: SDMRestraintControlParameter
    double* rs_e;           // per replica: restraint energy of the last evaluation
    int rs_any;             // 1 when some system has restraints
    // rigid waters (Langevin step)
    const int* st_idx;      // (O, H, H) system-local indices, every system's waters
    const int* st_flag;     // per topology particle: 1 in a rigid water
    double* lv_xp;          // per particle: unconstrained positions of water particles
    int st_any;             // 1 when some system has rigid waters
    int st_max;             // largest water count of a system
    int* ncl;            // clusters per replica
    int* ngrp;           // list-building groups per replica
    int jg;              // clusters per list-building group (1, 2 or SDM_JG)
    int2* cl_grp;        // per group (cluster window): first cluster, clusters (1..SDM_JG)
    unsigned* extz;      // per replica max cluster z extent (float bits)
    int* work_counter;   // [0] list build, [1] perturbation pass, [2] main pass (zeroed every call)
    int* status;         // device status word
    long long* counts;   // optional: per replica P0, P1delta (count mode)
    // list export (diagnostic)
    int* ex_cnt;
    int* ex_slot;
    unsigned char* ex_mask;
    int ex_cap;
    int ex_rep;
    // totals
    int total_atoms;     // sum of n over replicas
    int max_rep_atoms;   // largest n of a replica
    int total_cols;      // sum of ncol over replicas
    int total_cells;     // sum of ncol*M[2]+1 over replicas
    int total_slots;     // sum of slot_cap over replicas
    int total_pert;      // sum of 2*nD
    int total_ex;        // sum of ex_count over replicas
    int total_xc;        // sum of xc_count over replicas
    int split;           // work items per i-cluster
};

// Backward of the differentiable potential (k_backward): inputs of the
// forward, the upstream gradient and the outputs wanted (n_* = 0: skipped)
struct BwdArgs {
    const double* g;        // [nrep] dL/dU_r
    const double* res;      // [nrep * SDM_NRESULTS] results of the forward
    const double* F;        // mixed forces [3 * total particles]
    const double* F1;       // state-1 forces [3 * total particles]
    const double* G;        // adjoint sums [6 * perturbed]
    const double* eps;      // FP64 epsilon of the displaced particles [sum nD], or null
    const double* prm;      // [4 * nrep] lambda1, lambda2, alpha, u0 rows, or null (the handle's)
    double* gx;             // [3 * total particles]
    double* gd;             // [3 * sum of the systems' particles]
    double* gp;             // [3 * sum nD]: charge, sigma, epsilon
    double* gb;             // [5 * nrep]: lambda1, lambda2, alpha, u0, w0 rows
    long long n_x, n_d, n_p, n_b;
};
