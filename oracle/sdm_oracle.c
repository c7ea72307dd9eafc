/*
 * sdm_oracle.c -- FP64 CPU oracle for the SDM two-state force.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the test-suite, the
 * smoke entry point and the CPU-baseline leg of the benchmark load it; the
 * product library never does.
 *
 * What it restates (reference paths relative to the reference project):
 *
 *   two-state sequence   openmmapi/src/LangevinIntegratorSDM.cpp:158-176
 *                        U0 = E(x) (state 1 of the reference), U1 = E(x+d)
 *                        (state 2), both over the nonbonded force group only.
 *   displacement         platforms/reference/src/ReferenceSDMKernels.cpp:192-199
 *                        (x_i += d_i for every particle).
 *   soft core            openmmapi/src/LangevinIntegratorSDM.cpp:125-149
 *   bias / W' / E_pot    platforms/reference/src/ReferenceSDMKernels.cpp:247-287
 *   force mix            platforms/reference/src/ReferenceSDMKernels.cpp:309-318
 *   non-equilibrium      platforms/reference/src/ReferenceSDMKernels.cpp:231-245,289-302
 *
 * The pair arithmetic itself lives in OpenMM's NonbondedForce, which is a
 * third-party dependency absent from the reference tree (called at
 * LangevinIntegratorSDM.cpp:160,168 and configured by
 * example/desmonddmsfile75.py:424-438,776-808).  It is restated here from the
 * published physics: Lennard-Jones with Lorentz-Berthelot mixing, truncated
 * and unshifted at the cutoff, plus reaction-field Coulomb
 *     E = K qi qj (1/r + krf r^2 - crf),
 *     krf = (eps_rf-1)/((2 eps_rf+1) rc^3),  crf = 3 eps_rf/((2 eps_rf+1) rc),
 * minimum image in an orthorhombic box, excluded pairs contribute nothing,
 * no dispersion correction.
 *
 * PARITY UNPINNED.  The reference ships no tests, golden vectors or fixtures
 * for this path, and it cannot be built here (every source needs OpenMM).  So
 * neither the pair arithmetic nor the combine above is pinned against the
 * reference's own outputs.  The restatement is cross-checked instead against
 * an independent dense numpy implementation, analytic two-particle cases,
 * invariances and an independent Python restatement of the combine.
 *
 * Besides the FP64 physics ("fp64 rule": a pair interacts iff its FP64
 * minimum-image distance is below rc) the file restates the pair-inclusion
 * rule of the CUDA implementation bit for bit ("fp32 rule"): cluster-local
 * FP32 coordinates, per-cluster-pair FP32 shifts and an FP32 r^2 with a fixed
 * FMA order.  Under that rule the oracle's pair sets equal the GPU's exactly,
 * while every energy and force is still computed in FP64 from the FP64
 * coordinates.
 *
 * Build with -ffp-contract=off: the FP32 rule relies on unfused products.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_K_COULOMB 138.935456
#define ORC_LIST_MARGIN 1.0e-4

/* ------------------------------------------------------------------------- */
/* system description                                                        */
/* ------------------------------------------------------------------------- */
typedef struct {
    int n;
    const double* q;       /* e */
    const double* sig;     /* nm */
    const double* eps;     /* kJ/mol */
    const int* excl_off;   /* CSR offsets, n+1, symmetric, partners sorted */
    const int* excl_idx;
    const double* box;     /* 3 */
    double rc;
    double eps_rf;
} orc_sys;

static int is_excluded(const orc_sys* s, int i, int j) {
    for (int k = s->excl_off[i]; k < s->excl_off[i + 1]; ++k)
        if (s->excl_idx[k] == j) return 1;
    return 0;
}

static void rf_consts(const orc_sys* s, double* krf, double* crf) {
    double e = s->eps_rf, rc = s->rc;
    *krf = (e - 1.0) / ((2.0 * e + 1.0) * rc * rc * rc);
    *crf = 3.0 * e / ((2.0 * e + 1.0) * rc);
}

/* FP64 pair term. d = r_j - r_i; returns energy, *fscal such that
 * F_j = fscal*d and F_i = -fscal*d. */
static double pair64(const orc_sys* s, int i, int j, double r2, double krf, double crf,
                     double* fscal) {
    double r = sqrt(r2);
    double ir2 = 1.0 / r2;
    double sig = 0.5 * (s->sig[i] + s->sig[j]);
    double eps = sqrt(s->eps[i] * s->eps[j]);
    double s2 = sig * sig * ir2;
    double s6 = s2 * s2 * s2;
    double e_lj = 4.0 * eps * (s6 * s6 - s6);
    double f_lj = 4.0 * eps * (12.0 * s6 * s6 - 6.0 * s6);
    double qq = ORC_K_COULOMB * s->q[i] * s->q[j];
    double e_rf = qq * (1.0 / r + krf * r2 - crf);
    double f_rf = qq * (1.0 / r - 2.0 * krf * r2);
    *fscal = (f_lj + f_rf) * ir2;
    return e_lj + e_rf;
}

static inline double min_image(double v, double L) { return v - L * nearbyint(v / L); }

/* ------------------------------------------------------------------------- */
/* FP64 cell list over positions y (n*3, any image)                          */
/* ------------------------------------------------------------------------- */
typedef struct {
    int nc[3];
    int* head;   /* per cell first atom, -1 */
    int* next;   /* per atom */
    int brute;
} cells64;

static void cells64_build(cells64* c, const double* y, int n, const double* box, double rcut) {
    c->brute = 0;
    for (int k = 0; k < 3; ++k) {
        c->nc[k] = (int)floor(box[k] / rcut);
        if (c->nc[k] < 3) c->brute = 1;
    }
    if (c->brute) { c->head = NULL; c->next = NULL; return; }
    int ncell = c->nc[0] * c->nc[1] * c->nc[2];
    c->head = (int*)malloc(sizeof(int) * (size_t)ncell);
    c->next = (int*)malloc(sizeof(int) * (size_t)n);
    for (int i = 0; i < ncell; ++i) c->head[i] = -1;
    for (int i = n - 1; i >= 0; --i) {
        int ci[3];
        for (int k = 0; k < 3; ++k) {
            double w = y[3 * i + k] - box[k] * floor(y[3 * i + k] / box[k]);
            int v = (int)floor(w / box[k] * c->nc[k]);
            if (v < 0) v = 0;
            if (v >= c->nc[k]) v = c->nc[k] - 1;
            ci[k] = v;
        }
        int id = (ci[0] * c->nc[1] + ci[1]) * c->nc[2] + ci[2];
        c->next[i] = c->head[id];
        c->head[id] = i;
    }
}

static void cells64_free(cells64* c) { free(c->head); free(c->next); }

/* visit every unordered pair {i,j} (i<j) with min-image distance^2 < rc2 ;
 * callback-free: the caller passes what to accumulate through `mode`. */
typedef struct {
    double energy;
    long long pairs;
    double* f;       /* n*3 or NULL */
} acc64;

/* mode bits: 1 = all pairs, 2 = only pairs with d_i != d_j ("changed") */
static int changed_pair(const double* d, int i, int j) {
    return d[3 * i] != d[3 * j] || d[3 * i + 1] != d[3 * j + 1] || d[3 * i + 2] != d[3 * j + 2];
}

static void pair_loop64(const orc_sys* s, const double* y, const double* d, int only_changed,
                        acc64* out, int nthreads) {
    const int n = s->n;
    const double* box = s->box;
    double krf, crf;
    rf_consts(s, &krf, &crf);
    const double rc2 = s->rc * s->rc;
    cells64 c;
    cells64_build(&c, y, n, box, s->rc);
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#else
    nthreads = 1;
#endif
    double* fth = NULL;
    if (out->f) {
        fth = (double*)calloc((size_t)nthreads * 3 * (size_t)n, sizeof(double));
    }
    double etot = 0.0;
    long long ptot = 0;
    const int ncell = c.brute ? n : c.nc[0] * c.nc[1] * c.nc[2];
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4) reduction(+ : etot, ptot)
#endif
    for (int u = 0; u < ncell; ++u) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* ft = fth ? fth + (size_t)tid * 3 * (size_t)n : NULL;
        if (c.brute) {
            int i = u;
            for (int j = i + 1; j < n; ++j) {
                if (only_changed && !changed_pair(d, i, j)) continue;
                double dv[3], r2 = 0.0;
                for (int k = 0; k < 3; ++k) {
                    dv[k] = min_image(y[3 * j + k] - y[3 * i + k], box[k]);
                    r2 += dv[k] * dv[k];
                }
                if (r2 >= rc2 || is_excluded(s, i, j)) continue;
                double fs;
                etot += pair64(s, i, j, r2, krf, crf, &fs);
                ptot++;
                if (ft)
                    for (int k = 0; k < 3; ++k) { ft[3 * j + k] += fs * dv[k]; ft[3 * i + k] -= fs * dv[k]; }
            }
            continue;
        }
        int cz = u % c.nc[2], cy = (u / c.nc[2]) % c.nc[1], cx = u / (c.nc[1] * c.nc[2]);
        for (int i = c.head[u]; i >= 0; i = c.next[i]) {
            for (int ox = -1; ox <= 1; ++ox)
                for (int oy = -1; oy <= 1; ++oy)
                    for (int oz = -1; oz <= 1; ++oz) {
                        int nx = (cx + ox + c.nc[0]) % c.nc[0];
                        int ny = (cy + oy + c.nc[1]) % c.nc[1];
                        int nz = (cz + oz + c.nc[2]) % c.nc[2];
                        int v = (nx * c.nc[1] + ny) * c.nc[2] + nz;
                        for (int j = c.head[v]; j >= 0; j = c.next[j]) {
                            if (j <= i) continue;
                            if (only_changed && !changed_pair(d, i, j)) continue;
                            double dv[3], r2 = 0.0;
                            for (int k = 0; k < 3; ++k) {
                                dv[k] = min_image(y[3 * j + k] - y[3 * i + k], box[k]);
                                r2 += dv[k] * dv[k];
                            }
                            if (r2 >= rc2 || is_excluded(s, i, j)) continue;
                            double fs;
                            etot += pair64(s, i, j, r2, krf, crf, &fs);
                            ptot++;
                            if (ft)
                                for (int k = 0; k < 3; ++k) {
                                    ft[3 * j + k] += fs * dv[k];
                                    ft[3 * i + k] -= fs * dv[k];
                                }
                        }
                    }
        }
    }
    if (out->f) {
        for (int t = 0; t < nthreads; ++t)
            for (size_t k = 0; k < 3 * (size_t)n; ++k) out->f[k] += fth[(size_t)t * 3 * n + k];
        free(fth);
    }
    out->energy += etot;
    out->pairs += ptot;
    cells64_free(&c);
}

/* Nonbonded energy (+forces, may be NULL) at positions y. Returns energy. */
double orc_nonbonded(int n, const double* q, const double* sig, const double* eps,
                     const int* excl_off, const int* excl_idx, const double* box, double rc,
                     double eps_rf, const double* y, double* f, long long* npairs, int nthreads) {
    orc_sys s = {n, q, sig, eps, excl_off, excl_idx, box, rc, eps_rf};
    acc64 a = {0.0, 0, f};
    if (f) memset(f, 0, sizeof(double) * 3 * (size_t)n);
    pair_loop64(&s, y, NULL, 0, &a, nthreads);
    if (npairs) *npairs = a.pairs;
    return a.energy;
}

/* Two states, FP64 rule.
 *   out[0]=U0, out[1]=U1 (full evaluation at x+d), out[2]=u_direct (sum over
 *   changed pairs of e(x+d)-e(x)), F0/F1 may be NULL; counts[0]=P0,
 *   counts[1]=P1 (all pairs at x+d), counts[2]=P1delta (changed pairs at x+d),
 *   counts[3]=changed pairs at x. */
void orc_sdm_states(int n, const double* q, const double* sig, const double* eps,
                    const int* excl_off, const int* excl_idx, const double* box, double rc,
                    double eps_rf, const double* x, const double* d, double* out, double* F0,
                    double* F1, long long* counts, int nthreads) {
    orc_sys s = {n, q, sig, eps, excl_off, excl_idx, box, rc, eps_rf};
    double* y = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    for (size_t k = 0; k < 3 * (size_t)n; ++k) y[k] = x[k] + d[k];
    acc64 a0 = {0.0, 0, F0}, a1 = {0.0, 0, F1}, c0 = {0.0, 0, NULL}, c1 = {0.0, 0, NULL};
    if (F0) memset(F0, 0, sizeof(double) * 3 * (size_t)n);
    if (F1) memset(F1, 0, sizeof(double) * 3 * (size_t)n);
    pair_loop64(&s, x, d, 0, &a0, nthreads);
    pair_loop64(&s, y, d, 0, &a1, nthreads);
    pair_loop64(&s, x, d, 1, &c0, nthreads);
    pair_loop64(&s, y, d, 1, &c1, nthreads);
    out[0] = a0.energy;
    out[1] = a1.energy;
    out[2] = c1.energy - c0.energy;
    if (counts) {
        counts[0] = a0.pairs;
        counts[1] = a1.pairs;
        counts[2] = c1.pairs;
        counts[3] = c0.pairs;
    }
    free(y);
}

/* ------------------------------------------------------------------------- */
/* combine: soft core, bias, mix (restated from the reference)              */
/* ------------------------------------------------------------------------- */
/* LangevinIntegratorSDM::SoftCoreF (openmmapi/src/LangevinIntegratorSDM.cpp:125-149).
 * Returns u' and writes du'/du to *fp.  Returns NAN with *fp=NAN for an
 * unknown method (the reference throws). */
double orc_softcore(double u, int method, double umax, double a, double ub, double* fp) {
    if (u <= ub) { *fp = 1.0; return u; }
    if (method == 0) { *fp = 1.0; return u; }
    if (method == 1) {
        double t = tanh((u - ub) / umax);
        *fp = 1.0 - t * t;
        return umax * t + ub;
    }
    if (method == 2) {
        double gu = (u - ub) / (a * (umax - ub));
        double zeta = 1.0 + 2.0 * gu * (gu + 1.0);
        double za = pow(zeta, a);
        *fp = 4.0 * (2.0 * gu + 1.0) / zeta * za / ((1.0 + za) * (1.0 + za));
        return (umax - ub) * (za - 1.0) / (za + 1.0) + ub;
    }
    *fp = NAN;
    return NAN;
}

/* Parameter block, same order as sdm_params in include/sdm_capi.h. */
enum {
    P_BIAS, P_SOFT, P_LAMBDA, P_L1, P_L2, P_ALPHA, P_U0, P_W0, P_GAMMA, P_WB, P_UMAX, P_ACORE,
    P_UB, P_NONEQ, P_ML1, P_ML2, P_MU0, P_MW0, P_BL1, P_BL2, P_BU0, P_BW0, P_COUNT
};

/* Combine of ReferenceIntegrateLangevinStepSDMKernel::execute
 * (platforms/reference/src/ReferenceSDMKernels.cpp:202-318) without the
 * Langevin update and with the group-1 (restraint) energy set to zero.
 * out: [0]=u (=U1-U0) [1]=u' (BindE) [2]=fp [3]=W (ebias) [4]=W' (bfp)
 *      [5]=s=W'*fp [6]=E_pot=U0+W [7]=dW/dlambda (non-equilibrium, else 0)
 *      [8..11]=lambda1,lambda2,u0,w0 actually used */
void orc_combine(const double* p, double U0, double U1, double* out) {
    int method = (int)p[P_BIAS];
    double lambdac = p[P_LAMBDA];
    double gamma = 0.0, wb = lambdac, w0 = 0.0, l1 = lambdac, l2 = lambdac, alpha = 1.0, u0 = 0.0;
    if ((int)p[P_NONEQ] == 1) {
        /* the caller supplies lambdac = t/Ntmax; parameters follow p = m*lambda + b */
        l1 = p[P_ML1] * lambdac + p[P_BL1];
        l2 = p[P_ML2] * lambdac + p[P_BL2];
        u0 = p[P_MU0] * lambdac + p[P_BU0];
        w0 = p[P_MW0] * lambdac + p[P_BW0];
    }
    if (method == 1) {
        gamma = p[P_GAMMA];
        wb = p[P_WB];
        w0 = ((int)p[P_NONEQ] == 1) ? w0 : p[P_W0];
    } else if (method == 2) {
        if ((int)p[P_NONEQ] != 1) {
            l1 = p[P_L1];
            l2 = p[P_L2];
            u0 = p[P_U0];
            w0 = p[P_W0];
        }
        alpha = p[P_ALPHA];
    }
    double u = U1 - U0;
    double fp;
    double be = orc_softcore(u, (int)p[P_SOFT], p[P_UMAX], p[P_ACORE], p[P_UB], &fp);
    double ebias, bfp;
    if (method == 1) {
        ebias = 0.5 * gamma * be * be + wb * be + w0;
        bfp = gamma * be + wb;
    } else if (method == 2) {
        double ee = 1.0 + exp(-alpha * (be - u0));
        ebias = 0.0;
        if (alpha > 0) ebias = ((l2 - l1) / alpha) * log(ee);
        ebias += l2 * be + w0;
        bfp = (l2 - l1) / ee + l1;
    } else {
        ebias = lambdac * be;
        bfp = lambdac;
    }
    double dwdl = 0.0;
    if ((int)p[P_NONEQ] == 1) {
        /* ReferenceSDMKernels.cpp:289-297 reads the function-scope lambda1,
         * lambda2, alpha, u0 (:214-217).  The scheduled values of the
         * non-equilibrium block are block-local declarations (:236-239), and
         * only the integrated-logistic branch (:255-260) reloads the outer
         * ones.  For linear and quadratic bias the derivative therefore sees
         * lambda1 = lambda2 (the lambda before the step), alpha = 1 and
         * u0 = 0; the lambda value itself only enters as lambda2 - lambda1 = 0.
         * OpenCLSDMKernels.cpp:156-185,256-265 behaves the same. */
        double dl1 = l1, dl2 = l2, da = alpha, du0 = u0;
        if (method != 2) {
            dl1 = lambdac;
            dl2 = lambdac;
            da = 1.0;
            du0 = 0.0;
        }
        double ee = 1.0 + exp(-da * (be - du0));
        double dwdl1 = -log(ee) / da;
        double dwdl2 = be + log(ee) / da;
        double dwdu0 = (dl2 - dl1) * exp(-da * (be - du0)) / ee;
        dwdl = dwdl1 * p[P_ML1] + dwdl2 * p[P_ML2] + dwdu0 * p[P_MU0] + 1.0 * p[P_MW0];
    }
    out[0] = u;
    out[1] = be;
    out[2] = fp;
    out[3] = ebias;
    out[4] = bfp;
    out[5] = bfp * fp;
    out[6] = U0 + ebias;
    out[7] = dwdl;
    out[8] = l1;
    out[9] = l2;
    out[10] = u0;
    out[11] = w0;
}

/* Mixed force F = (1-s) F0 + s F1 (ReferenceSDMKernels.cpp:309-318). */
void orc_mix(int n, double s, const double* F0, const double* F1, double* F) {
    for (size_t k = 0; k < 3 * (size_t)n; ++k) F[k] = s * F1[k] + (1.0 - s) * F0[k];
}

/* Full FP64 evaluation of one lambda state (the CPU baseline's unit of work):
 * U0, U1, u, u', W, W' and the mixed force F (n*3). res[0..11] as orc_combine,
 * res[12]=U0, res[13]=U1.  F0/F1 scratch may be NULL (allocated inside). */
void orc_eval_state(int n, const double* q, const double* sig, const double* eps,
                    const int* excl_off, const int* excl_idx, const double* box, double rc,
                    double eps_rf, const double* x, const double* d, const double* params,
                    double* res, double* F, int nthreads) {
    double* F0 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* F1 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* y = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    for (size_t k = 0; k < 3 * (size_t)n; ++k) y[k] = x[k] + d[k];
    double U0 = orc_nonbonded(n, q, sig, eps, excl_off, excl_idx, box, rc, eps_rf, x, F0, NULL, nthreads);
    double U1 = orc_nonbonded(n, q, sig, eps, excl_off, excl_idx, box, rc, eps_rf, y, F1, NULL, nthreads);
    orc_combine(params, U0, U1, res);
    res[12] = U0;
    res[13] = U1;
    if (F) orc_mix(n, res[5], F0, F1, F);
    free(F0);
    free(F1);
    free(y);
}

/* ------------------------------------------------------------------------- */
/* FP32-rule restatement of the CUDA clustering (bit-exact index maps)       */
/* ------------------------------------------------------------------------- */
static double wrap1(double v, double L, double invL) {
    double t = floor(v * invL);
    double w = v - t * L;
    if (w >= L) w -= L;
    if (w < 0.0) w += L;
    return w;
}

static int cell_of(double w, double invg, int M) {
    int c = (int)floor(w * invg);
    if (c < 0) c = 0;
    if (c > M - 1) c = M - 1;
    return c;
}

typedef struct {
    double z;
    int idx;
} zkey;

static int zkey_cmp(const void* a, const void* b) {
    const zkey* x = (const zkey*)a;
    const zkey* y = (const zkey*)b;
    if (x->z < y->z) return -1;
    if (x->z > y->z) return 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* Clustering of one coordinate set.
 *   M[3]      grid (columns Mx*My, z cells Mz)
 *   outputs   perm[cap_slots]   slot -> original index or -1 (padding)
 *             ncl               number of clusters
 *             ref[3*cap_cl]     integer reference cell of each cluster
 *             X[4*cap_slots]    cluster-local FP32 coordinates (w unused = 0)
 *             colcl[Mx*My+1]    first cluster of each column (prefix)
 *   returns number of slots (8*ncl) or -1 if a capacity is exceeded. */
int orc_build_clusters(int n, const double* x, const double* box, const int* M, int cap_slots,
                       int* perm, int* ncl_out, int* ref, float* X, int* colcl) {
    const int ncol = M[0] * M[1];
    double g[3], invg[3], invL[3];
    for (int k = 0; k < 3; ++k) {
        g[k] = box[k] / (double)M[k];
        invg[k] = (double)M[k] / box[k];
        invL[k] = 1.0 / box[k];
    }
    double* w = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    int* col = (int*)malloc(sizeof(int) * (size_t)n);
    int* cz = (int*)malloc(sizeof(int) * (size_t)n);
    int* cnt = (int*)calloc((size_t)ncol + 1, sizeof(int));
    for (int i = 0; i < n; ++i) {
        int c[3];
        for (int k = 0; k < 3; ++k) {
            w[3 * i + k] = wrap1(x[3 * i + k], box[k], invL[k]);
            c[k] = cell_of(w[3 * i + k], invg[k], M[k]);
        }
        col[i] = c[0] * M[1] + c[1];
        cz[i] = c[2];
        cnt[col[i]]++;
    }
    int* aoff = (int*)malloc(sizeof(int) * ((size_t)ncol + 1));
    aoff[0] = 0;
    colcl[0] = 0;
    for (int c = 0; c < ncol; ++c) {
        aoff[c + 1] = aoff[c] + cnt[c];
        colcl[c + 1] = colcl[c] + (cnt[c] + 7) / 8;
    }
    const int ncl = colcl[ncol];
    if (8 * ncl > cap_slots) {
        free(w); free(col); free(cz); free(cnt); free(aoff);
        return -1;
    }
    zkey* keys = (zkey*)malloc(sizeof(zkey) * (size_t)(n > 0 ? n : 1));
    int* fill = (int*)calloc((size_t)ncol, sizeof(int));
    for (int i = 0; i < n; ++i) {
        zkey kk;
        kk.z = w[3 * i + 2];
        kk.idx = i;
        keys[aoff[col[i]] + fill[col[i]]++] = kk;
    }
    for (int s = 0; s < 8 * ncl; ++s) perm[s] = -1;
    for (int c = 0; c < ncol; ++c) {
        qsort(keys + aoff[c], (size_t)cnt[c], sizeof(zkey), zkey_cmp);
        for (int r = 0; r < cnt[c]; ++r) {
            int slot = 8 * colcl[c] + r;
            perm[slot] = keys[aoff[c] + r].idx;
        }
    }
    for (int C = 0; C < ncl; ++C) {
        int a0 = perm[8 * C];
        int cx = col[a0] / M[1], cy = col[a0] % M[1];
        ref[3 * C] = cx;
        ref[3 * C + 1] = cy;
        ref[3 * C + 2] = cz[a0];
        double R[3] = {(double)cx * g[0], (double)cy * g[1], (double)cz[a0] * g[2]};
        for (int t = 0; t < 8; ++t) {
            int s = 8 * C + t, a = perm[s];
            for (int k = 0; k < 3; ++k)
                X[4 * s + k] = (a >= 0) ? (float)(w[3 * a + k] - R[k]) : 1.0e6f;
            X[4 * s + 3] = 0.0f;
        }
    }
    *ncl_out = ncl;
    free(w); free(col); free(cz); free(cnt); free(aoff); free(keys); free(fill);
    return 8 * ncl;
}

/* single-image mode flag as decided by the CUDA code: 0 if one shift per
 * cluster pair gives the minimum image for every interacting pair. */
int orc_image_mode(const double* box, const int* M, double rc, int ncl, const int* perm,
                   const float* X) {
    /* x, y: the cell edge bounds the in-column extent; z: the cell edge, then the
     * largest cluster extent against a float threshold rounded down */
    for (int k = 0; k < 2; ++k)
        if (!(0.5 * box[k] - rc - box[k] / M[k] > 1.0e-3)) return 1;
    double tzd = 0.5 * box[2] - rc - 1.0e-3;
    if (!(box[2] / M[2] < tzd)) return 1;
    float tzf = (float)tzd;
    if ((double)tzf > tzd) tzf = nextafterf(tzf, -1.0f);
    float ext = 0.0f;
    for (int s = 0; s < 8 * ncl; ++s)
        if (perm[s] >= 0 && X[4 * s + 2] > ext) ext = X[4 * s + 2];
    return !(ext < tzf);
}

static int wrap_cell(int n, int M) {
    if (2 * n > M) n -= M;
    else if (2 * n <= -M) n += M;
    return n;
}

/* Pair ownership of the CUDA main pass (which cluster's list holds a pair).
 * When the column stencil cannot wrap onto itself (2K+1 <= M in x and y,
 * K = floor((rc+2e-4)/g)+1) a pair of different columns belongs to the
 * cluster from whose column the other lies at a forward offset
 * (ox > 0, or ox == 0 and oy > 0); otherwise to the lower column id.  In one
 * column the lower cluster owns; in one cluster the lower slot is i. */
static int half_geo(const double* box, const int* M, double rc) {
    for (int k = 0; k < 2; ++k) {
        double g = box[k] / (double)M[k];
        int K = (int)floor((rc + 2.0e-4) / g) + 1;
        if (2 * K + 1 > M[k]) return 0;
    }
    return 1;
}

static int wrap_cell(int n, int M);

static int owns(const int* ref, int A, int B, const int* M, int geo) {
    int colA = ref[3 * A] * M[1] + ref[3 * A + 1];
    int colB = ref[3 * B] * M[1] + ref[3 * B + 1];
    if (colA == colB) return A <= B;
    if (!geo) return colA < colB;
    int ox = wrap_cell(ref[3 * B] - ref[3 * A], M[0]);
    int oy = wrap_cell(ref[3 * B + 1] - ref[3 * A + 1], M[1]);
    return ox > 0 || (ox == 0 && oy > 0);
}

typedef struct {
    float Lf[3], invLf[3], g[3];
    double gd[3];
    int M[3];
    int img;
    float rc2f;
} f32rule;

static void f32rule_init(f32rule* r, const double* box, const int* M, double rc, int img) {
    for (int k = 0; k < 3; ++k) {
        r->Lf[k] = (float)box[k];
        r->invLf[k] = (float)(1.0 / box[k]);
        r->gd[k] = box[k] / (double)M[k];
        r->M[k] = M[k];
    }
    r->img = img;
    r->rc2f = (float)(rc * rc);
}

static float img32(float d, float L, float invL) {
    float t = rintf(d * invL);
    return fmaf(-L, t, d);
}

/* FP32 r^2 between slot i (cluster I) and slot j (cluster J) as the main-pass
 * kernel computes it. */
static float r2_main32(const f32rule* r, const int* ref, const float* X, int I, int si, int J,
                       int sj) {
    float dd[3];
    for (int k = 0; k < 3; ++k) {
        int nn = wrap_cell(ref[3 * J + k] - ref[3 * I + k], r->M[k]);
        float S = (float)((double)nn * r->gd[k]);
        float xs = X[4 * sj + k] + S;
        float dv = xs - X[4 * si + k];
        if (r->img) dv = img32(dv, r->Lf[k], r->invLf[k]);
        dd[k] = dv;
    }
    return fmaf(dd[2], dd[2], fmaf(dd[1], dd[1], dd[0] * dd[0]));
}

/* FP32 rule of the perturbation pass for a displaced particle at FP64 position
 * yp (wrapped) against slot sj of cluster J: the particle is expressed in the
 * frame of its own cell, o = fl32(yp - c*g), and j in that frame through the
 * same cell-pair shift table as the main pass. */
static float r2_pert32(const f32rule* r, const double* box, const int* ref, const float* X,
                       const double* yp, int J, int sj) {
    float dd[3];
    for (int k = 0; k < 3; ++k) {
        int cyk = cell_of(yp[k], (double)r->M[k] / box[k], r->M[k]);
        float o = (float)(yp[k] - (double)cyk * r->gd[k]);
        int nn = wrap_cell(ref[3 * J + k] - cyk, r->M[k]);
        float S = (float)((double)nn * r->gd[k]);
        float xs = X[4 * sj + k] + S;
        float dv = xs - o;
        if (r->img) dv = img32(dv, r->Lf[k], r->invLf[k]);
        dd[k] = dv;
    }
    return fmaf(dd[2], dd[2], fmaf(dd[1], dd[1], dd[0] * dd[0]));
}

/* FP32 rule for two displaced particles (FP64 minimum image, then FP32). */
static float r2_dd32(const double* box, const double* yp, const double* yj) {
    float dd[3];
    for (int k = 0; k < 3; ++k) {
        double v = yj[k] - yp[k];
        double t = nearbyint(v * (1.0 / box[k]));
        v = v - t * box[k];
        dd[k] = (float)v;
    }
    return fmaf(dd[2], dd[2], fmaf(dd[1], dd[1], dd[0] * dd[0]));
}

/* Two states under the FP32 rule (the CUDA pair sets), FP64 arithmetic.
 *   out[0]=U0 (main pass), out[1]=u (perturbation pass), out[2]=U1=U0+u
 *   F0 (n*3) main pass, dF (n*3) = sum over changed pairs of f(x+d)-f(x)
 *   counts[0]=P0, counts[1]=P1delta (changed pairs at x+d), counts[2]=changed at x
 *   M, and the clustering are recomputed here from x. */
int orc_sdm_f32rule(int n, const double* q, const double* sig, const double* eps,
                    const int* excl_off, const int* excl_idx, const double* box, double rc,
                    double eps_rf, const int* M, const double* x, const double* d, double* out,
                    double* F0, double* dF, long long* counts) {
    orc_sys s = {n, q, sig, eps, excl_off, excl_idx, box, rc, eps_rf};
    double krf, crf;
    rf_consts(&s, &krf, &crf);
    int ncol = M[0] * M[1];
    int cap = n + 8 * ncol + 8;
    int* perm = (int*)malloc(sizeof(int) * (size_t)cap);
    int* ref = (int*)malloc(sizeof(int) * 3 * (size_t)cap);
    float* X = (float*)malloc(sizeof(float) * 4 * (size_t)cap);
    int* colcl = (int*)malloc(sizeof(int) * ((size_t)ncol + 1));
    int ncl = 0;
    int ns = orc_build_clusters(n, x, box, M, cap, perm, &ncl, ref, X, colcl);
    if (ns < 0) { free(perm); free(ref); free(X); free(colcl); return -1; }
    int img = orc_image_mode(box, M, rc, ncl, perm, X);
    int geo = half_geo(box, M, rc);
    f32rule R;
    f32rule_init(&R, box, M, rc, img);
    int* slot_of = (int*)malloc(sizeof(int) * (size_t)n);
    for (int t = 0; t < ns; ++t)
        if (perm[t] >= 0) slot_of[perm[t]] = t;
    double invL[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
    double* w = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) w[3 * i + k] = wrap1(x[3 * i + k], box[k], invL[k]);
    if (F0) memset(F0, 0, sizeof(double) * 3 * (size_t)n);
    if (dF) memset(dF, 0, sizeof(double) * 3 * (size_t)n);
    /* candidates: FP64 cell list with a margin, then the FP32 rule decides */
    double rcand = rc + 1.0e-3;
    double U0 = 0.0;
    long long P0 = 0;
    {
        orc_sys s2 = s;
        s2.rc = rcand;
        cells64 c;
        cells64_build(&c, w, n, box, rcand);
        int ncell = c.brute ? 1 : c.nc[0] * c.nc[1] * c.nc[2];
        for (int u = 0; u < ncell; ++u) {
            int ilist_b = c.brute;
            int cx = 0, cy = 0, cz = 0;
            if (!ilist_b) { cz = u % c.nc[2]; cy = (u / c.nc[2]) % c.nc[1]; cx = u / (c.nc[1] * c.nc[2]); }
            for (int i = ilist_b ? 0 : c.head[u]; ilist_b ? (i < n) : (i >= 0); i = ilist_b ? i + 1 : c.next[i]) {
                int nb = ilist_b ? 1 : 27;
                for (int o = 0; o < nb; ++o) {
                    int jstart;
                    if (ilist_b) jstart = 0;
                    else {
                        int ox = o / 9 - 1, oy = (o / 3) % 3 - 1, oz = o % 3 - 1;
                        int nx = (cx + ox + c.nc[0]) % c.nc[0], ny = (cy + oy + c.nc[1]) % c.nc[1],
                            nz = (cz + oz + c.nc[2]) % c.nc[2];
                        jstart = c.head[(nx * c.nc[1] + ny) * c.nc[2] + nz];
                    }
                    for (int j = jstart; ilist_b ? (j < n) : (j >= 0); j = ilist_b ? j + 1 : c.next[j]) {
                        if (j == i) continue;
                        int si = slot_of[i], sj = slot_of[j];
                        if (si / 8 == sj / 8) {
                            if (si > sj) continue; /* one cluster: lower slot is "i" */
                        } else if (!owns(ref, si / 8, sj / 8, M, geo)) {
                            continue;
                        }
                        if (is_excluded(&s, i, j)) continue;
                        float r2f = r2_main32(&R, ref, X, si / 8, si, sj / 8, sj);
                        if (!(r2f < R.rc2f)) continue;
                        double dv[3], r2 = 0.0;
                        for (int k = 0; k < 3; ++k) {
                            dv[k] = min_image(w[3 * j + k] - w[3 * i + k], box[k]);
                            r2 += dv[k] * dv[k];
                        }
                        double fs;
                        U0 += pair64(&s, i, j, r2, krf, crf, &fs);
                        P0++;
                        if (F0)
                            for (int k = 0; k < 3; ++k) { F0[3 * j + k] += fs * dv[k]; F0[3 * i + k] -= fs * dv[k]; }
                    }
                }
            }
        }
        cells64_free(&c);
    }
    /* perturbation pass: displaced particles p against particles with d_j != d_p */
    double u = 0.0;
    long long P1 = 0, Pc0 = 0;
    for (int p = 0; p < n; ++p) {
        if (d[3 * p] == 0.0 && d[3 * p + 1] == 0.0 && d[3 * p + 2] == 0.0) continue;
        for (int st = 0; st < 2; ++st) {
            double yp[3];
            for (int k = 0; k < 3; ++k) yp[k] = wrap1(w[3 * p + k] + (st ? d[3 * p + k] : 0.0), box[k], invL[k]);
            double sgn = st ? 1.0 : -1.0;
            for (int j = 0; j < n; ++j) {
                if (j == p || !changed_pair(d, p, j)) continue;
                int jdisp = !(d[3 * j] == 0.0 && d[3 * j + 1] == 0.0 && d[3 * j + 2] == 0.0);
                if (jdisp && j < p) continue; /* displaced-displaced pairs once */
                /* quick FP64 reject before the FP32 rule */
                double yj[3], dv[3], r2 = 0.0;
                for (int k = 0; k < 3; ++k) {
                    yj[k] = jdisp ? wrap1(w[3 * j + k] + (st ? d[3 * j + k] : 0.0), box[k], invL[k]) : w[3 * j + k];
                    dv[k] = min_image(yj[k] - yp[k], box[k]);
                    r2 += dv[k] * dv[k];
                }
                if (r2 > rcand * rcand) continue;
                if (is_excluded(&s, p, j)) continue;
                float r2f;
                if (jdisp) r2f = r2_dd32(box, yp, yj);
                else {
                    int sj = slot_of[j];
                    r2f = r2_pert32(&R, box, ref, X, yp, sj / 8, sj);
                }
                if (!(r2f < R.rc2f)) continue;
                double fs;
                double e = pair64(&s, p, j, r2, krf, crf, &fs);
                u += sgn * e;
                if (st) P1++; else Pc0++;
                if (dF)
                    for (int k = 0; k < 3; ++k) { dF[3 * j + k] += sgn * fs * dv[k]; dF[3 * p + k] -= sgn * fs * dv[k]; }
            }
        }
    }
    out[0] = U0;
    out[1] = u;
    out[2] = U0 + u;
    if (counts) { counts[0] = P0; counts[1] = P1; counts[2] = Pc0; }
    free(perm); free(ref); free(X); free(colcl); free(slot_of); free(w);
    return img;
}

/* Emulated j-lists of the CUDA list builder for bit-exact comparison.
 * For each i-cluster I the entries are (slot j, allowed-i mask) over all
 * clusters J >= I, using the FP32 bounding-box rule with margin.  Entries are
 * written sorted by slot; cnt[I] gets the count; returns total entries or -1
 * if cap_per_cluster is exceeded. */
long long orc_emit_lists(int n, const int* excl_off, const int* excl_idx, const double* box,
                         double rc, const int* M, const double* x, int cap_per_cluster,
                         int* ncl_out, int* perm_out, int* cnt, int* ent_slot,
                         unsigned char* ent_mask) {
    int ncol = M[0] * M[1];
    int cap = n + 8 * ncol + 8;
    int* perm = perm_out;
    int* ref = (int*)malloc(sizeof(int) * 3 * (size_t)cap);
    float* X = (float*)malloc(sizeof(float) * 4 * (size_t)cap);
    int* colcl = (int*)malloc(sizeof(int) * ((size_t)ncol + 1));
    int ncl = 0;
    int ns = orc_build_clusters(n, x, box, M, cap, perm, &ncl, ref, X, colcl);
    if (ns < 0) { free(ref); free(X); free(colcl); return -1; }
    int img = orc_image_mode(box, M, rc, ncl, perm, X);
    int geo = half_geo(box, M, rc);
    f32rule R;
    f32rule_init(&R, box, M, rc, img);
    int* slot_of = (int*)malloc(sizeof(int) * (size_t)n);
    for (int t = 0; t < ns; ++t)
        if (perm[t] >= 0) slot_of[perm[t]] = t;
    float rl = (float)(rc + ORC_LIST_MARGIN);
    float rl2 = rl * rl;
    long long total = 0;
    for (int I = 0; I < ncl; ++I) {
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        for (int t = 0; t < 8; ++t) {
            int si = 8 * I + t;
            if (perm[si] < 0) continue;
            for (int k = 0; k < 3; ++k) {
                lo[k] = fminf(lo[k], X[4 * si + k]);
                hi[k] = fmaxf(hi[k], X[4 * si + k]);
            }
        }
        float c[3], h[3];
        for (int k = 0; k < 3; ++k) { c[k] = 0.5f * (lo[k] + hi[k]); h[k] = 0.5f * (hi[k] - lo[k]); }
        int k_out = 0;
        for (int sj = 0; sj < 8 * ncl; ++sj) {
            int b = perm[sj];
            if (b < 0) continue;
            int J = sj / 8;
            if (J != I && !owns(ref, I, J, M, geo)) continue;
            float e[3];
            for (int k = 0; k < 3; ++k) {
                int nn = wrap_cell(ref[3 * J + k] - ref[3 * I + k], M[k]);
                float S = (float)((double)nn * R.gd[k]);
                float xs = X[4 * sj + k] + S;
                float t = xs - c[k];
                if (img) t = img32(t, R.Lf[k], R.invLf[k]);
                e[k] = fmaxf(fabsf(t) - h[k], 0.0f);
            }
            float d2 = fmaf(e[2], e[2], fmaf(e[1], e[1], e[0] * e[0]));
            if (!(d2 < rl2)) continue;
            unsigned mask = 0;
            for (int t = 0; t < 8; ++t) {
                int si = 8 * I + t;
                int a = perm[si];
                if (a < 0) continue;
                if (J == I && !(t < sj - 8 * I)) continue;
                int ex = 0;
                for (int kk = excl_off[b]; kk < excl_off[b + 1]; ++kk)
                    if (excl_idx[kk] == a) { ex = 1; break; }
                if (!ex) mask |= 1u << t;
            }
            if (mask == 0) continue; /* no allowed i: the CUDA list drops the entry */
            if (k_out >= cap_per_cluster) { free(ref); free(X); free(colcl); free(slot_of); return -1; }
            ent_slot[(size_t)I * cap_per_cluster + k_out] = sj;
            ent_mask[(size_t)I * cap_per_cluster + k_out] = (unsigned char)mask;
            k_out++;
        }
        cnt[I] = k_out;
        total += k_out;
    }
    *ncl_out = ncl;
    free(ref); free(X); free(colcl); free(slot_of);
    return total;
}
