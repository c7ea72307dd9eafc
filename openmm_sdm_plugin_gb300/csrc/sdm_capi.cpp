// sdm_capi.cpp -- host side of the C ABI declared in include/sdm_capi.h.
//
// The handle owns one device arena (a single cudaMalloc sized at creation),
// one CUDA stream, pinned staging for parameters, and a small cache of CUDA
// graphs (one per distinct set of input/output pointers).  Nothing here throws
// across the ABI: every entry point catches and converts to an sdm_status.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/sdm_capi.h"
#include "sdm_types.h"

cudaError_t sdm_launch_prep(const SdmArgs& a, int* item_prefix, int* grp_prefix, int* done, cudaStream_t st,
                            cudaEvent_t* ev, int nev, unsigned ev_flags);
cudaError_t sdm_launch_jlist(const SdmArgs& a, const int* grp_prefix, cudaStream_t st);
cudaError_t sdm_launch_backward(const SdmArgs& a, const BwdArgs& b, cudaStream_t st);
cudaError_t sdm_pair_prepare();
#define SDM_MAX_CTAS 4  // pair-kernel CTAs per SM with a built register bound
int sdm_pair_resident(int ctas_per_sm, int chunk);
cudaError_t sdm_launch_pair(const SdmArgs& a, const int* item_prefix, int mode, int ctas_per_sm,
                            int resident, bool pme, int chunk, cudaStream_t st);
cudaError_t sdm_launch_perturb(const SdmArgs& a, int mode, cudaStream_t st);
cudaError_t sdm_launch_exceptions(const SdmArgs& a, cudaStream_t st);
cudaError_t sdm_launch_pme(const SdmArgs& a, const cufftHandle* r2c, const cufftHandle* c2r, const long long* grid_off,
                           const long long* spec_off, int nsys, int conv_blocks, cudaStream_t st);
cudaError_t sdm_pme_prepare(int smem_bytes);
cudaError_t sdm_launch_restraints(const SdmArgs& a, cudaStream_t st);
cudaError_t sdm_launch_combine(const SdmArgs& a, cudaStream_t st);
cudaError_t sdm_launch_finalize(const SdmArgs& a, cudaStream_t st);
cudaError_t sdm_launch_mix(const SdmArgs& a, cudaStream_t st);
cudaError_t sdm_launch_gather_positions(const void* posq, const void* corr, int double_precision,
                                        const int* index, int n, double* x, cudaStream_t st);
cudaError_t sdm_launch_scatter_forces(const double* f, const int* index, int n, int padded, long long* buf,
                                      cudaStream_t st);
cudaError_t sdm_launch_adjoint(const SdmArgs& a, cudaStream_t st);

namespace {

const double kCoulomb = 138.935456;  // kJ nm / (mol e^2), OpenMM's ONE_4PI_EPS0
const double kMolarGasConstant = 0.008314462618;  // kJ / (mol K), R of CODATA 2018 (k_B N_A)
const long long kPmeBrickPoints = 6144;   // preferred sub-grid size of a PME brick (48 KB of fixed point)
const long long kPmeBrickMax = 27648;     // largest sub-grid (216 KB); bricks beyond it use global atomics
thread_local std::string g_create_error;

struct SysHost {
    int n;
    std::vector<float> q, hs, se;
    std::vector<int> grp;
    std::vector<int> mol;       // exclusion component id
    std::vector<double> d;      // 3n
    std::vector<int> excl_off;  // n+1 (local)
    std::vector<int> excl_idx;
    std::vector<int> D;         // displaced particles
    std::vector<int> cx_off;    // nD+1 (local)
    std::vector<int> cx_idx;
    std::vector<int2> hst, fst;  // owner / full column stencils
    std::vector<int2> ex_pair;   // exceptions (local indices)
    std::vector<double4_16a> ex_prm; // (K qq, sigma, 4 eps, 0)
    std::vector<int2> xc_pair;   // PME: excluded pairs i < j and K q_i q_j
    std::vector<float> xc_qq;
    std::vector<float> theta;    // PME: Ewald kernel x B-spline moduli, half spectrum
    // group-1 restraints (sdm_set_restraints): particles / weights (ligand group,
    // then receptor group), parameters (SDM_RS_*), reference particles, bits
    std::vector<int> rs_idx;
    std::vector<double> rs_w;
    double rs_prm[SDM_RS_COUNT] = {};
    int rs_ref[12] = {};
    int rs_on = 0, rs_nlig = 0, rs_nrcpt = 0;
    // rigid waters (sdm_set_rigid_waters): (O, H, H) triples, distances
    std::vector<int> st_idx;
    double st_doh = 0.0, st_dhh = 0.0;
    bool clique = false;
    SdmSys dev;
    int replicas;
};

struct Arena {
    size_t off = 0;
    template <class T>
    size_t take(size_t count) {
        off = (off + 255) & ~size_t(255);
        size_t o = off;
        off += count * sizeof(T) + 16;
        return o;
    }
};

struct GraphKey {
    const void* x;
    const void* res;
    const void* f;
    const void* stream;
    int split, ctas;
    const void* v = nullptr;      // Langevin step: velocities, inverse masses, external forces
    const void* invm = nullptr;
    const void* fext = nullptr;
    bool operator<(const GraphKey& o) const {
        return std::tie(x, res, f, stream, split, ctas, v, invm, fext) <
               std::tie(o.x, o.res, o.f, o.stream, o.split, o.ctas, o.v, o.invm, o.fext);
    }
};

// device buffers of a Langevin step (positions double as the evaluation's x)
struct LvBind {
    double* x;
    double* v;
    const double* invm;
    const double* fext;
};

}  // namespace

struct sdm_handle {
    int device = 0;
    std::vector<SysHost> sys;
    std::vector<SdmRep> rep;
    int nrep = 0;
    long long total_particles = 0;  // over replicas (coordinate count / 3)
    // device
    char* arena = nullptr;
    size_t arena_bytes = 0;
    void* rs_buf = nullptr;   // restraint data of every system (sdm_set_restraints)
    void* st_buf = nullptr;   // rigid-water data and the unconstrained-position scratch
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;          // second branch of an evaluation (perturbation pass)
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    cudaEvent_t bridge_ev[2] = {};         // special caller streams: into and out of the handle's stream
    SdmArgs args{};
    int* item_prefix = nullptr;
    int* grp_prefix = nullptr;   // list-building groups over replicas (k_jlist items)
    int* done = nullptr;
    // cluster-pair lists (own allocation: regrown on overflow)
    int4* jl_buf = nullptr;
    long long jl_clusters = 0;  // cluster windows covered
    int jl_cap = 0;
    void* counters = nullptr;  // memset block
    size_t counters_bytes = 0;
    double* x_in = nullptr;
    double* res_in = nullptr;
    double* f_in = nullptr;
    double* params_dev = nullptr;
    double* lv_dev = nullptr;     // SDM_LV_COUNT doubles
    // host
    double* params_pinned = nullptr;  // params, then SDM_LV_COUNT Langevin doubles
    std::vector<double> params;
    bool params_dirty = true;
    double lv_host[SDM_LV_COUNT] = {};
    bool lv_set = false, lv_dirty = false;
    // options
    int opt_graph = 1, opt_profile = 0, opt_split = 1, opt_ctas = 4, opt_verify = 1, opt_zero_copy = 0;
    int opt_chunk = 12;                   // list entries per staged chunk of the main pass (8, 12, 16)
    int opt_overlap = 2;                  // second graph branch (SDM_OPT_OVERLAP)
    int opt_list_group = 0;               // clusters per list-building group (SDM_OPT_LIST_GROUP; 0 automatic)
    int auto_list_group = 4;              // the automatic choice, set at creation
    int pair_res[3][SDM_MAX_CTAS + 1] = {};  // resident pair-kernel CTAs per SM by chunk (8, 12, 16) and request
    // graphs
    std::map<GraphKey, cudaGraphExec_t> graphs;
    // profiling
    cudaEvent_t ev[12] = {};
    float last_ms[12] = {};
    int last_nk = 0;
    std::string err;
    // last evaluation pointers (for state forces)
    bool have_eval = false;
    bool pme = false;            // every system uses PME (no mixed batches)
    std::vector<cufftHandle> pme_r2c, pme_c2r;      // per system, batch 2 grids per replica
    std::vector<long long> pme_grid_off, pme_spec_off;
};

static sdm_status sdm_reserve_lists(sdm_handle* h, int cap);

namespace {

// index of a staging chunk size (8, 12, 16) in the per-chunk tables
inline int chunk_index(int chunk) { return chunk == 8 ? 0 : chunk == 16 ? 2 : 1; }

const char* const kKernelNames[] = {"k_cells", "k_scan", "k_bucket", "k_cellsort", "k_clusters",
                                    "k_jlist", "k_pair", "k_pert_prep+k_perturb", "k_combine+k_finalize_mix"};
const int kNumTimed = 9;

sdm_status fail(sdm_handle* h, sdm_status code, const std::string& msg) {
    if (h) h->err = msg; else g_create_error = msg;
    return code;
}

sdm_status cuda_fail(sdm_handle* h, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(h, SDM_ERR_CUDA, m);
}

#define SDM_CUDA(h, call)                                   \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
    } while (0)

void default_params(double* p) {
    // reference integrator defaults, openmmapi/src/LangevinIntegratorSDM.cpp:48-85
    for (int k = 0; k < SDM_NPARAMS; ++k) p[k] = 0.0;
    p[SDM_P_BIAS_METHOD] = SDM_LINEAR;
    p[SDM_P_SOFTCORE_METHOD] = SDM_NO_SOFTCORE;
    p[SDM_P_LAMBDA] = 1.0;
    p[SDM_P_LAMBDA1] = 1.0;
    p[SDM_P_LAMBDA2] = 1.0;
    p[SDM_P_ALPHA] = 1.0;
    p[SDM_P_U0] = 0.0;
    p[SDM_P_W0] = 0.0;
    p[SDM_P_GAMMA] = 0.0;
    p[SDM_P_WB] = 1.0;
    p[SDM_P_UMAX] = 200.0;
    p[SDM_P_ACORE] = 0.25;
    p[SDM_P_UBCORE] = 0.0;
}

int round8(long long v) { return (int)((v + 7) / 8 * 8); }

std::string setup_system(const sdm_system_desc& d, SysHost& s) {
    char buf[256];
    if (d.num_particles < 1) return "num_particles must be >= 1";
    if (!d.charge || !d.sigma || !d.epsilon) return "charge/sigma/epsilon must not be NULL";
    if (d.num_exclusions < 0 || (d.num_exclusions > 0 && !d.exclusions))
        return "invalid exclusion list";
    if (d.num_replicas < 1) return "num_replicas must be >= 1";
    if (!(d.cutoff > 0.0)) return "cutoff must be > 0";
    for (int k = 0; k < 3; ++k) {
        if (!(d.box[k] > 0.0) || !std::isfinite(d.box[k])) return "box edges must be finite and > 0";
        if (!(d.cutoff < 0.5 * d.box[k])) {
            snprintf(buf, sizeof buf, "cutoff %.6g must be below half the box edge %.6g", d.cutoff, d.box[k]);
            return buf;
        }
    }
    if (d.nonbonded_method != SDM_NB_REACTION_FIELD && d.nonbonded_method != SDM_NB_PME)
        return "unknown nonbonded_method";
    if (d.nonbonded_method == SDM_NB_REACTION_FIELD && !(d.reaction_field_dielectric > 0.0))
        return "reaction_field_dielectric must be > 0";
    const int n = d.num_particles;
    s.n = n;
    s.replicas = d.num_replicas;
    s.q.resize(n); s.hs.resize(n); s.se.resize(n); s.grp.assign(n, 0); s.d.assign(3 * (size_t)n, 0.0);
    const double sk = std::sqrt(kCoulomb);
    for (int i = 0; i < n; ++i) {
        if (!(d.sigma[i] >= 0.0) || !(d.epsilon[i] >= 0.0) || !std::isfinite(d.sigma[i]) ||
            !std::isfinite(d.epsilon[i]) || !std::isfinite(d.charge[i]))
            return "sigma/epsilon must be finite and >= 0, charges finite";
        s.q[i] = (float)(d.charge[i] * sk);
        s.hs[i] = (float)(0.5 * d.sigma[i]);
        s.se[i] = (float)(2.0 * std::sqrt(d.epsilon[i]));
    }
    // the same rule as sdm_set_displacement: a NaN would break the ordering of
    // the displacement-group map and reach the kernels as displaced coordinates
    if (d.displacement)
        for (size_t k = 0; k < 3 * (size_t)n; ++k)
            if (!std::isfinite(d.displacement[k])) return "non-finite displacement";
    // exclusions: symmetric CSR, sorted, de-duplicated
    std::vector<std::vector<int>> adj(n);
    for (int e = 0; e < d.num_exclusions; ++e) {
        const int a = d.exclusions[2 * e], b = d.exclusions[2 * e + 1];
        if (a < 0 || b < 0 || a >= n || b >= n || a == b) return "exclusion index out of range or self pair";
        adj[a].push_back(b);
        adj[b].push_back(a);
    }
    s.excl_off.assign(n + 1, 0);
    s.excl_idx.clear();
    for (int i = 0; i < n; ++i) {
        auto& v = adj[i];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        s.excl_idx.insert(s.excl_idx.end(), v.begin(), v.end());
        s.excl_off[i + 1] = (int)s.excl_idx.size();
    }
    // exclusion components: when each is a clique, "excluded" is "same component"
    s.mol.resize(n);
    {
        std::vector<int> par(n);
        for (int i = 0; i < n; ++i) par[i] = i;
        auto root = [&](int x) { while (par[x] != x) { par[x] = par[par[x]]; x = par[x]; } return x; };
        for (int i = 0; i < n; ++i)
            for (int k = s.excl_off[i]; k < s.excl_off[i + 1]; ++k) {
                const int a = root(i), b = root(s.excl_idx[k]);
                if (a != b) par[std::max(a, b)] = std::min(a, b);
            }
        std::vector<long long> size(n, 0), edges(n, 0);
        for (int i = 0; i < n; ++i) {
            s.mol[i] = root(i);
            size[s.mol[i]] += 1;
            edges[s.mol[i]] += s.excl_off[i + 1] - s.excl_off[i];  // each edge twice
        }
        bool clique = true;
        for (int i = 0; i < n && clique; ++i)
            if (size[i] > 0 && edges[i] != size[i] * (size[i] - 1)) clique = false;
        s.clique = clique;
    }
    // exceptions: every pair must be excluded from the nonbonded sum
    if (d.num_exceptions < 0 || (d.num_exceptions > 0 && (!d.exception_pairs || !d.exception_params)))
        return "invalid exception list";
    s.ex_pair.clear();
    s.ex_prm.clear();
    for (int e = 0; e < d.num_exceptions; ++e) {
        const int a = d.exception_pairs[2 * e], b = d.exception_pairs[2 * e + 1];
        if (a < 0 || b < 0 || a >= n || b >= n || a == b) return "exception index out of range or self pair";
        if (!std::binary_search(s.excl_idx.begin() + s.excl_off[a], s.excl_idx.begin() + s.excl_off[a + 1], b))
            return "exception pair " + std::to_string(a) + "-" + std::to_string(b) + " is not excluded";
        const double qq = d.exception_params[3 * e], sg = d.exception_params[3 * e + 1],
                     ep = d.exception_params[3 * e + 2];
        if (!std::isfinite(qq) || !std::isfinite(sg) || !std::isfinite(ep) || ep < 0.0)
            return "invalid exception parameters";
        s.ex_pair.push_back(make_int2(a, b));
        s.ex_prm.push_back(make_double4_16a(kCoulomb * qq, sg, 4.0 * ep, 0.0));
    }
    // grid
    SdmSys& g = s.dev;
    std::memset(&g, 0, sizeof g);
    g.n = n;
    g.excl_clique = s.clique ? 1 : 0;
    const double vol = d.box[0] * d.box[1] * d.box[2];
    const double side = std::cbrt(8.0 * vol / n);
    for (int k = 0; k < 3; ++k) {
        int M = (int)std::floor(d.box[k] / side + 0.5);
        M = std::max(1, std::min(M, 1024));
        g.M[k] = M;
        g.box[k] = d.box[k];
        g.invL[k] = 1.0 / d.box[k];
        {
            const double lim = d.box[k] * (1.0 - 9.094947017729282e-13);   // L (1 - 2^-40)
            std::memcpy(&g.wrap_lim[k], &lim, sizeof lim);
        }
        g.g[k] = d.box[k] / (double)M;
        g.invg[k] = (double)M / d.box[k];
        g.Lf[k] = (float)d.box[k];
        g.invLf[k] = (float)(1.0 / d.box[k]);
        g.gf[k] = (float)g.g[k];
    }
    g.ncol = g.M[0] * g.M[1];
    g.rc = d.cutoff;
    g.img_static = 0;
    for (int k = 0; k < 2; ++k) {
        const int K = (int)std::floor((d.cutoff + 2.0e-4) / g.g[k]) + 1;
        if (2 * K + 1 <= g.M[k]) { g.stlo[k] = -K; g.sthi[k] = K; }
        else { g.stlo[k] = -((g.M[k] - 1) / 2); g.sthi[k] = g.M[k] / 2; }
        if (!(0.5 * d.box[k] - d.cutoff - g.g[k] > 1.0e-3)) g.img_static = 1;
    }
    // z: the cell edge is a static lower bound of the cluster extent
    const double tzd = 0.5 * d.box[2] - d.cutoff - 1.0e-3;
    if (!(g.g[2] < tzd)) g.img_static = 1;
    float tzf = (float)tzd;
    if ((double)tzf > tzd) tzf = std::nextafter(tzf, -1.0f);
    g.tz = tzf;
    // owner stencil: the forward half when the stencil cannot wrap onto itself
    int Kx = (int)std::floor((d.cutoff + 2.0e-4) / g.g[0]) + 1;
    int Ky = (int)std::floor((d.cutoff + 2.0e-4) / g.g[1]) + 1;
    g.half_geo = (2 * Kx + 1 <= g.M[0] && 2 * Ky + 1 <= g.M[1]) ? 1 : 0;
    s.hst.clear();
    s.fst.clear();
    const double rcs = d.cutoff + 3.0e-4;
    auto near = [&](int ox, int oy) {
        // columns offset by (ox,oy) can hold particles closer than the cutoff
        const double gx = std::max(std::abs(ox) - 1, 0) * g.g[0];
        const double gy = std::max(std::abs(oy) - 1, 0) * g.g[1];
        return gx * gx + gy * gy < rcs * rcs;
    };
    for (int ox = g.stlo[0]; ox <= g.sthi[0]; ++ox)
        for (int oy = g.stlo[1]; oy <= g.sthi[1]; ++oy)
            if (near(ox, oy)) s.fst.push_back({ox, oy});
    if (g.half_geo) {
        s.hst.push_back({0, 0});
        for (int ox = 0; ox <= Kx; ++ox)
            for (int oy = -Ky; oy <= Ky; ++oy)
                if ((ox > 0 || oy > 0) && near(ox, oy)) s.hst.push_back({ox, oy});
    } else {
        s.hst = s.fst;
    }
    const double rc = d.cutoff;
    if (d.nonbonded_method == SDM_NB_PME) {
        const double tol = d.ewald_tolerance > 0.0 ? d.ewald_tolerance : 5e-4;
        if (!(tol < 0.5)) return "ewald_tolerance must be below 0.5";
        // the FP32 screening function of the pair kernels covers beta rc <= 4
        if (!(tol >= 5.7e-8)) return "ewald_tolerance must be at least 5.7e-8";
        const double beta = std::sqrt(-std::log(2.0 * tol)) / rc;
        g.pme = 1;
        g.beta = beta;
        g.beta_f = (float)beta;
        g.c2_f = (float)(2.0 * beta / std::sqrt(M_PI));
        g.krf = 0.0f;
        g.crf = 0.0f;
        for (int k = 0; k < 3; ++k) {
            int m = d.pme_grid[k];
            if (m <= 0) {   // smallest 2,3,5,7-smooth m >= 2 beta L / (3 tol^(1/5))
                m = std::max(6, (int)std::ceil(2.0 * beta * d.box[k] / (3.0 * std::pow(tol, 0.2))));
                for (;; ++m) {
                    int v = m;
                    for (int p : {2, 3, 5, 7})
                        while (v % p == 0) v /= p;
                    if (v == 1) break;
                }
            }
            if (m < 6 || m > 1024) return "PME grid dimensions must be in 6..1024";
            g.pme_grid[k] = m;
            g.pme_gs[k] = (float)((double)m / d.box[k]);
        }
        // spreading / interpolation bricks of bc cells per side: the stencils of
        // a brick's particles cover at most ceil(bc K / M) + 5 grid points per
        // dimension (+2 for FP32 rounding at the cell faces)
        for (int bc = 5; bc >= 1; --bc) {
            long long cap = 1;
            for (int k = 0; k < 3; ++k)
                cap *= (long long)std::ceil((double)std::min(bc, g.M[k]) * g.pme_grid[k] / g.M[k]) + 7;
            if (cap <= kPmeBrickPoints || bc == 1) {
                for (int k = 0; k < 3; ++k) {
                    g.pme_bc[k] = std::min(bc, g.M[k]);
                    g.pme_nb[k] = (g.M[k] + g.pme_bc[k] - 1) / g.pme_bc[k];
                }
                g.pme_cap = (int)std::min(cap, (long long)kPmeBrickMax);
                break;
            }
        }
        // self and neutralising-background terms (coordinate independent)
        double q2 = 0.0, qs = 0.0;
        for (int i = 0; i < n; ++i) { q2 += d.charge[i] * d.charge[i]; qs += d.charge[i]; }
        const double V = d.box[0] * d.box[1] * d.box[2];
        g.e_const = -kCoulomb * beta / std::sqrt(M_PI) * q2 - kCoulomb * M_PI * qs * qs / (2.0 * V * beta * beta);
        // Ewald kernel x B-spline moduli on the half spectrum (order 5):
        // theta(m) = |b0|^2 |b1|^2 |b2|^2 exp(-pi^2 m^2 / beta^2) / (pi V m^2)
        {
            const double m5[4] = {1.0 / 24.0, 11.0 / 24.0, 11.0 / 24.0, 1.0 / 24.0};   // M_5(1..4)
            std::vector<double> bm[3];
            for (int k = 0; k < 3; ++k) {
                const int K = g.pme_grid[k];
                std::vector<double> s2(K);
                for (int m = 0; m < K; ++m) {
                    double re = 0.0, im = 0.0;
                    for (int j = 0; j < 4; ++j) {
                        re += m5[j] * std::cos(2.0 * M_PI * m * j / K);
                        im += m5[j] * std::sin(2.0 * M_PI * m * j / K);
                    }
                    s2[m] = re * re + im * im;
                }
                for (int m = 0; m < K; ++m)   // odd order: zero at the Nyquist index, use the neighbours
                    if (s2[m] < 1e-7) s2[m] = 0.5 * (s2[(m + K - 1) % K] + s2[(m + 1) % K]);
                bm[k].resize(K);
                for (int m = 0; m < K; ++m) bm[k][m] = 1.0 / s2[m];
            }
            const int K0 = g.pme_grid[0], K1 = g.pme_grid[1], K2 = g.pme_grid[2], K2h = K2 / 2 + 1;
            const double V = d.box[0] * d.box[1] * d.box[2];
            s.theta.assign((size_t)K0 * K1 * K2h, 0.0f);
            for (int a = 0; a < K0; ++a)
                for (int b = 0; b < K1; ++b)
                    for (int c = 0; c < K2h; ++c) {
                        if (a == 0 && b == 0 && c == 0) continue;
                        const double ma = (a <= K0 / 2 ? a : a - K0) / d.box[0];
                        const double mb = (b <= K1 / 2 ? b : b - K1) / d.box[1];
                        const double mc = c / d.box[2];
                        const double m2 = ma * ma + mb * mb + mc * mc;
                        s.theta[((size_t)a * K1 + b) * K2h + c] = (float)(
                            bm[0][a] * bm[1][b] * bm[2][c] * std::exp(-M_PI * M_PI * m2 / (beta * beta)) / (M_PI * V * m2));
                    }
        }
        // excluded pairs leave the reciprocal sum
        s.xc_pair.clear();
        s.xc_qq.clear();
        for (int i = 0; i < n; ++i)
            for (int k = s.excl_off[i]; k < s.excl_off[i + 1]; ++k) {
                const int j = s.excl_idx[k];
                if (j > i) {
                    s.xc_pair.push_back(make_int2(i, j));
                    s.xc_qq.push_back((float)(kCoulomb * d.charge[i] * d.charge[j]));
                }
            }
    } else {
        const double e = d.reaction_field_dielectric;
        g.krf = (float)((e - 1.0) / ((2.0 * e + 1.0) * rc * rc * rc));
        g.crf = (float)(3.0 * e / ((2.0 * e + 1.0) * rc));
    }
    g.rc2f = (float)(rc * rc);
    g.rcl = (float)(rc + SDM_LIST_MARGIN);
    g.rcl2f = g.rcl * g.rcl;
    return "";
}

// displacement groups: distinct displacement vectors (exact), 0 = zero vector
void setup_displacement(SysHost& s, const double* disp) {
    const int n = s.n;
    s.grp.assign(n, 0);
    if (disp) std::copy(disp, disp + 3 * (size_t)n, s.d.begin());
    else std::fill(s.d.begin(), s.d.end(), 0.0);
    std::map<std::tuple<double, double, double>, int> ids;
    s.D.clear();
    for (int i = 0; i < n; ++i) {
        const double x = s.d[3 * i], y = s.d[3 * i + 1], z = s.d[3 * i + 2];
        if (x == 0.0 && y == 0.0 && z == 0.0) continue;
        auto key = std::make_tuple(x, y, z);
        auto it = ids.find(key);
        int id;
        if (it == ids.end()) { id = (int)ids.size() + 1; ids[key] = id; }
        else id = it->second;
        s.grp[i] = id;
        s.D.push_back(i);
    }
    s.cx_off.assign(s.D.size() + 1, 0);
    s.cx_idx.clear();
    for (size_t k = 0; k < s.D.size(); ++k) {
        const int p = s.D[k];
        for (int e = s.excl_off[p]; e < s.excl_off[p + 1]; ++e) {
            const int j = s.excl_idx[e];
            if (s.grp[j] != s.grp[p]) s.cx_idx.push_back(j);
        }
        s.cx_off[k + 1] = (int)s.cx_idx.size();
    }
}

template <class T>
T* at(char* base, size_t off) { return reinterpret_cast<T*>(base + off); }

sdm_status upload_topology(sdm_handle* h) {
    // rebuilds the per-particle topology arrays of every system (after a
    // displacement change) in the arena
    std::vector<float> q, hs, se;
    std::vector<int> grp, mol, eoff, eidx, D, cxo, cxi;
    std::vector<double> dd, org;
    std::vector<float> tab;
    std::vector<int4> ex4;
    std::vector<int2> sten, exp_, xcp;
    std::vector<double4_16a> exq;
    std::vector<float> xcq, th;
    std::vector<SdmSys> sd;
    int atom = 0, excl = 0, dbase = 0, cxbase = 0, tabbase = 0, orgbase = 0;
    for (auto& s : h->sys) {
        SdmSys g = s.dev;
        g.atom_base = atom;
        g.excl_base = excl;
        g.D_base = dbase;
        g.nD = (int)s.D.size();
        g.cx_base = cxbase;
        g.shift_base = tabbase;
        g.org_base = orgbase;
        g.ex_base = (int)exp_.size();
        g.ex_count = (int)s.ex_pair.size();
        exp_.insert(exp_.end(), s.ex_pair.begin(), s.ex_pair.end());
        exq.insert(exq.end(), s.ex_prm.begin(), s.ex_prm.end());
        g.pme_base = (int)th.size();
        th.insert(th.end(), s.theta.begin(), s.theta.end());
        g.xc_base = (int)xcp.size();
        g.xc_count = (int)s.xc_pair.size();
        xcp.insert(xcp.end(), s.xc_pair.begin(), s.xc_pair.end());
        xcq.insert(xcq.end(), s.xc_qq.begin(), s.xc_qq.end());
        q.insert(q.end(), s.q.begin(), s.q.end());
        hs.insert(hs.end(), s.hs.begin(), s.hs.end());
        se.insert(se.end(), s.se.begin(), s.se.end());
        grp.insert(grp.end(), s.grp.begin(), s.grp.end());
        mol.insert(mol.end(), s.mol.begin(), s.mol.end());
        dd.insert(dd.end(), s.d.begin(), s.d.end());
        for (int i = 0; i < s.n; ++i) eoff.push_back(excl + s.excl_off[i]);
        for (int i = 0; i < s.n; ++i) {
            const int b = s.excl_off[i], e = s.excl_off[i + 1];
            int v[4] = {-1, -1, -1, -1};
            if (e - b > 4) v[0] = v[1] = v[2] = v[3] = -2;
            else for (int k = b; k < e; ++k) v[k - b] = s.excl_idx[k];
            ex4.push_back(make_int4(v[0], v[1], v[2], v[3]));
        }
        eidx.insert(eidx.end(), s.excl_idx.begin(), s.excl_idx.end());
        D.insert(D.end(), s.D.begin(), s.D.end());
        for (size_t k = 0; k < s.D.size(); ++k) cxo.push_back((int)cxi.size() + s.cx_off[k]);
        const int cx_total = (int)cxi.size() + s.cx_off[s.D.size()];
        cxi.insert(cxi.end(), s.cx_idx.begin(), s.cx_idx.end());
        cxo.push_back(cx_total);
        for (int k = 0; k < 3; ++k)
            for (int m = -g.M[k]; m <= g.M[k]; ++m) tab.push_back((float)((double)m * g.g[k]));
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < g.M[k]; ++c) org.push_back((double)c * g.g[k]);
        g.hst_base = (int)sten.size();
        g.hst_count = (int)s.hst.size();
        sten.insert(sten.end(), s.hst.begin(), s.hst.end());
        g.fst_base = (int)sten.size();
        g.fst_count = (int)s.fst.size();
        sten.insert(sten.end(), s.fst.begin(), s.fst.end());
        atom += s.n;
        excl += (int)s.excl_idx.size();
        dbase += (int)s.D.size();
        cxbase += (int)s.D.size() + 1;
        tabbase += 2 * (g.M[0] + g.M[1] + g.M[2]) + 3;
        orgbase += g.M[0] + g.M[1] + g.M[2];
        s.dev = g;
        sd.push_back(g);
    }
    eoff.push_back(excl);
    if (eidx.empty()) eidx.push_back(0);
    if (D.empty()) D.push_back(0);
    if (cxi.empty()) cxi.push_back(0);
    SdmArgs& a = h->args;
    auto put = [&](const void* dst, const void* src, size_t bytes) -> sdm_status {
        SDM_CUDA(h, cudaMemcpyAsync(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice, h->stream));
        return SDM_OK;
    };
    sdm_status st;
    if ((st = put(a.sys, sd.data(), sd.size() * sizeof(SdmSys)))) return st;
    if ((st = put(a.topo_q, q.data(), q.size() * 4))) return st;
    if ((st = put(a.topo_hs, hs.data(), hs.size() * 4))) return st;
    if ((st = put(a.topo_se, se.data(), se.size() * 4))) return st;
    if ((st = put(a.topo_grp, grp.data(), grp.size() * 4))) return st;
    if ((st = put(a.topo_mol, mol.data(), mol.size() * 4))) return st;
    if ((st = put(a.topo_ex4, ex4.data(), ex4.size() * sizeof(int4)))) return st;
    if ((st = put(a.cell_org, org.data(), org.size() * sizeof(double)))) return st;
    if ((st = put(a.topo_d, dd.data(), dd.size() * 8))) return st;
    if ((st = put(a.excl_off, eoff.data(), eoff.size() * 4))) return st;
    if ((st = put(a.excl_idx, eidx.data(), eidx.size() * 4))) return st;
    if ((st = put(a.D_idx, D.data(), D.size() * 4))) return st;
    if ((st = put(a.cx_off, cxo.data(), cxo.size() * 4))) return st;
    if ((st = put(a.cx_idx, cxi.data(), cxi.size() * 4))) return st;
    if ((st = put(a.shift_tab, tab.data(), tab.size() * 4))) return st;
    if ((st = put(a.stencil, sten.data(), sten.size() * sizeof(int2)))) return st;
    if (!exp_.empty()) {
        if ((st = put(a.ex_pair, exp_.data(), exp_.size() * sizeof(int2)))) return st;
        if ((st = put(a.ex_prm, exq.data(), exq.size() * sizeof(double4_16a)))) return st;
    }
    if (!xcp.empty()) {
        if ((st = put(a.xc_pair, xcp.data(), xcp.size() * sizeof(int2)))) return st;
        if ((st = put(a.xc_qq, xcq.data(), xcq.size() * sizeof(float)))) return st;
    }
    if (!th.empty())
        if ((st = put(a.pme_theta, th.data(), th.size() * sizeof(float)))) return st;
    // perturbation windows depend on nD
    int pw = 0, ew = 0, xw = 0;
    for (auto& r : h->rep) {
        r.pert_win = pw;
        pw += 2 * h->sys[r.sys].dev.nD;
        r.ex_win = ew;
        ew += h->sys[r.sys].dev.ex_count;
        r.xc_win = xw;
        xw += h->sys[r.sys].dev.xc_count;
    }
    a.total_pert = pw;
    a.total_ex = ew;
    a.total_xc = xw;
    if ((st = put(a.rep, h->rep.data(), h->rep.size() * sizeof(SdmRep)))) return st;
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return SDM_OK;
}

// capture: event records become graph event-record nodes only with the
// External flag (otherwise they are capture-internal dependency markers)
sdm_status enqueue(sdm_handle* h, const SdmArgs& a, int mode, cudaStream_t st, bool profile,
                   bool capturing) {
    const unsigned fl = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    SDM_CUDA(h, cudaMemsetAsync(h->counters, 0, h->counters_bytes, st));
    cudaEvent_t* ev = profile ? h->ev : nullptr;
    SDM_CUDA(h, sdm_launch_prep(a, h->item_prefix, h->grp_prefix, h->done, st, ev, 6, fl));
    // The perturbation pass reads only what the preparation kernels wrote and
    // adds into its own accumulators (dF, its energy partials), and the PME
    // reciprocal space reads positions and cell data and adds forces by
    // integer atomics: they run on a second branch of the graph beside the
    // list build.  SDM_OPT_OVERLAP 1 joins it before the main pass, 2 after it
    // (with PME on the branch: the main pass takes clusters from a counter, so
    // CTAs that start late take fewer).  Timed evaluations keep one branch so
    // that the events bracket single kernels.
    //
    // The combine (u, soft core, bias, the mixing weight s) needs every part
    // of u (perturbation pass, exceptions, excluded-pair corrections,
    // reciprocal space) and nothing of the main pass, so with a branch the
    // exceptions and the combine run there too; the finalize then reads s and
    // only reduces U0.  The exceptions add forces by integer atomics, in any
    // order beside the main pass's.
    const int ov = profile || mode == 2 ? 0 : h->opt_overlap;
    const bool pme_side = ov == 2 && mode == 0 && h->pme;
    const bool fork = ov != 0 && (a.total_pert > 0 || pme_side);
    const bool ex_side = fork && mode == 0;
    const bool cmb_side = ex_side && (!h->pme || pme_side);
    if (fork) {
        SDM_CUDA(h, cudaEventRecord(h->fork_ev, st));
        SDM_CUDA(h, cudaStreamWaitEvent(h->side, h->fork_ev, 0));
        SDM_CUDA(h, sdm_launch_perturb(a, mode, h->side));
        if (ex_side) SDM_CUDA(h, sdm_launch_exceptions(a, h->side));
        if (pme_side)
            SDM_CUDA(h, sdm_launch_pme(a, h->pme_r2c.data(), h->pme_c2r.data(), h->pme_grid_off.data(),
                                       h->pme_spec_off.data(), (int)h->sys.size(), a.pme_conv_blocks, h->side));
        if (cmb_side) SDM_CUDA(h, sdm_launch_combine(a, h->side));
        SDM_CUDA(h, cudaEventRecord(h->join_ev, h->side));
    }
    SDM_CUDA(h, sdm_launch_jlist(a, h->grp_prefix, st));
    if (fork && ov == 1) SDM_CUDA(h, cudaStreamWaitEvent(st, h->join_ev, 0));
    if (profile) SDM_CUDA(h, cudaEventRecordWithFlags(h->ev[6], st, fl));
    SDM_CUDA(h, sdm_launch_pair(a, h->item_prefix, mode, h->opt_ctas, h->pair_res[chunk_index(h->opt_chunk)][h->opt_ctas],
                                h->pme, h->opt_chunk, st));
    if (profile) SDM_CUDA(h, cudaEventRecordWithFlags(h->ev[7], st, fl));
    if (fork && ov == 2) SDM_CUDA(h, cudaStreamWaitEvent(st, h->join_ev, 0));
    if (mode != 2 && !fork) SDM_CUDA(h, sdm_launch_perturb(a, mode, st));
    if (mode == 0 && !ex_side) SDM_CUDA(h, sdm_launch_exceptions(a, st));
    if (mode == 0) SDM_CUDA(h, sdm_launch_restraints(a, st));
    if (mode == 0 && h->pme && !pme_side)
        SDM_CUDA(h, sdm_launch_pme(a, h->pme_r2c.data(), h->pme_c2r.data(), h->pme_grid_off.data(),
                                   h->pme_spec_off.data(), (int)h->sys.size(), a.pme_conv_blocks, st));
    if (profile) SDM_CUDA(h, cudaEventRecordWithFlags(h->ev[8], st, fl));
    if (mode == 0 && !cmb_side) SDM_CUDA(h, sdm_launch_combine(a, st));
    if (mode == 0) SDM_CUDA(h, sdm_launch_finalize(a, st));
    if (profile) SDM_CUDA(h, cudaEventRecordWithFlags(h->ev[9], st, fl));
    return SDM_OK;
}

sdm_status flush_params(sdm_handle* h, cudaStream_t st) {
    if (!h->params_dirty) return SDM_OK;
    std::memcpy(h->params_pinned, h->params.data(), h->params.size() * sizeof(double));
    SDM_CUDA(h, cudaMemcpyAsync(h->params_dev, h->params_pinned, h->params.size() * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    // the pinned staging must not be overwritten before the copy ran
    SDM_CUDA(h, cudaStreamSynchronize(st));
    h->params_dirty = false;
    return SDM_OK;
}

sdm_status flush_langevin(sdm_handle* h, cudaStream_t st) {
    if (!h->lv_dirty) return SDM_OK;
    double* stage = h->params_pinned + h->params.size();
    std::memcpy(stage, h->lv_host, sizeof h->lv_host);
    SDM_CUDA(h, cudaMemcpyAsync(h->lv_dev, stage, sizeof h->lv_host, cudaMemcpyHostToDevice, st));
    SDM_CUDA(h, cudaStreamSynchronize(st));
    h->lv_dirty = false;
    return SDM_OK;
}

sdm_status run(sdm_handle* h, const double* x, double* res, double* f, cudaStream_t st, int mode,
               bool allow_graph, const LvBind* lv = nullptr) {
    if (st == cudaStreamLegacy || st == cudaStreamPerThread) {
        // the default streams cannot be captured into a graph: the call runs
        // on the handle's stream, after the caller's earlier work on `st` and
        // before its later work
        SDM_CUDA(h, cudaEventRecord(h->bridge_ev[0], st));
        SDM_CUDA(h, cudaStreamWaitEvent(h->stream, h->bridge_ev[0], 0));
        const sdm_status s = run(h, x, res, f, h->stream, mode, allow_graph, lv);
        SDM_CUDA(h, cudaEventRecord(h->bridge_ev[1], h->stream));
        SDM_CUDA(h, cudaStreamWaitEvent(st, h->bridge_ev[1], 0));
        return s;
    }
    if (!h->jl_buf) {   // a failed regrow left no lists: allocate the last capacity again
        sdm_status s0 = sdm_reserve_lists(h, h->jl_cap);
        if (s0) return s0;
    }
    SdmArgs a = h->args;
    a.x = x;
    a.results = res;
    a.forces = f;
    a.F0out = nullptr;
    a.jg = h->opt_list_group ? h->opt_list_group : h->auto_list_group;
    a.lv_x = lv ? lv->x : nullptr;
    a.lv_v = lv ? lv->v : nullptr;
    a.lv_invm = lv ? lv->invm : nullptr;
    a.lv_fext = lv ? lv->fext : nullptr;
    a.lv_prm = lv ? h->lv_dev : nullptr;
    if (lv) {
        sdm_status s0 = flush_langevin(h, st);
        if (s0) return s0;
    }
    a.F1out = nullptr;
    a.split = mode == 2 ? 1 : h->opt_split;
    sdm_status s = flush_params(h, st);
    if (s) return s;
    // profile 1: eager launches timed with events; profile 2: the same events
    // recorded inside the captured graph (read back by sdm_get_kernel_times)
    const bool profile = h->opt_profile == 1;
    if (profile || !h->opt_graph || !allow_graph || mode != 0) {
        s = enqueue(h, a, mode, st, profile, false);
        if (s) return s;
        if (profile) {
            SDM_CUDA(h, cudaEventSynchronize(h->ev[kNumTimed]));
            for (int k = 0; k < kNumTimed; ++k)
                SDM_CUDA(h, cudaEventElapsedTime(&h->last_ms[k], h->ev[k], h->ev[k + 1]));
            h->last_nk = kNumTimed;
        }
        h->have_eval = (mode == 0);
        return SDM_OK;
    }
    const bool gprof = h->opt_profile == 2;
    GraphKey key{x, res, f, st, a.split, h->opt_ctas + (gprof ? 100 : 0) + 1000 * h->opt_chunk + 100000 * h->opt_overlap + 1000000 * h->opt_list_group};
    if (lv) { key.v = lv->v; key.invm = lv->invm; key.fext = lv->fext; }
    auto it = h->graphs.find(key);
    if (it == h->graphs.end()) {
        cudaGraph_t g = nullptr;
        SDM_CUDA(h, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        s = enqueue(h, a, mode, st, gprof, true);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (s) { if (g) cudaGraphDestroy(g); return s; }
        if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaStreamEndCapture");
        cudaGraphExec_t ex = nullptr;
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaGraphInstantiate");
        if (h->graphs.size() > 16) {
            for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
            h->graphs.clear();
        }
        it = h->graphs.emplace(key, ex).first;
    }
    SDM_CUDA(h, cudaGraphLaunch(it->second, st));
    h->have_eval = true;
    h->last_nk = gprof ? -kNumTimed : 0;  // negative: times pending inside the last replay
    return SDM_OK;
}

sdm_status check_dev_status(sdm_handle* h, int* out, bool clear) {
    int v = 0;
    SDM_CUDA(h, cudaMemcpy(&v, h->args.status, sizeof(int), cudaMemcpyDeviceToHost));
    if (clear && v) SDM_CUDA(h, cudaMemset(h->args.status, 0, sizeof(int)));
    if (out) *out = v;
    return SDM_OK;
}

}  // namespace

// Message for sdm_last_error(NULL) from entry points that have no handle.
void sdm_set_thread_error(const char* msg) { g_create_error = msg ? msg : ""; }

// (Re)allocates the cluster-pair lists with `cap` entries per i-cluster.
static sdm_status sdm_reserve_lists(sdm_handle* h, int cap) {
    if (h->stream) SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->jl_buf) { cudaFree(h->jl_buf); h->jl_buf = nullptr; }
    const size_t bytes = (size_t)h->jl_clusters * (size_t)cap * sizeof(int4);
    cudaError_t ce = cudaMalloc(&h->jl_buf, bytes);
    if (ce != cudaSuccess) {
        // jl_cap keeps the last capacity that was allocated; run() retries it
        h->jl_buf = nullptr;
        h->args.jl = nullptr;
        return cuda_fail(h, ce, "cudaMalloc(cluster-pair lists)");
    }
    h->jl_cap = cap;
    h->args.jl = h->jl_buf;
    h->args.jl_cap = cap;
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return SDM_OK;
}

// After an overflow: double the capacity (the last results are invalid).
static sdm_status regrow_lists(sdm_handle* h) {
    return sdm_reserve_lists(h, h->jl_cap * 2);
}

// --------------------------------------------------------------------------- //
extern "C" {

sdm_status sdm_create(const sdm_system_desc* systems, int num_systems, int device, sdm_handle** out) {
    if (!out) return fail(nullptr, SDM_ERR_INVALID_ARGUMENT, "out must not be NULL");
    *out = nullptr;
    if (!systems || num_systems < 1) return fail(nullptr, SDM_ERR_INVALID_ARGUMENT, "need >= 1 system");
    sdm_handle* h = new (std::nothrow) sdm_handle();
    if (!h) return fail(nullptr, SDM_ERR_INVALID_ARGUMENT, "out of host memory");
    auto bail = [&](sdm_status s) {
        g_create_error = h->err.empty() ? g_create_error : h->err;
        sdm_destroy(h);
        return s;
    };
    // host-side setup and validation of every system first (no device call),
    // so that a bad descriptor is reported as such with or without a GPU
    h->sys.resize(num_systems);
    for (int s = 0; s < num_systems; ++s) {
        std::string e = setup_system(systems[s], h->sys[s]);
        if (!e.empty()) {
            delete h;
            return fail(nullptr, SDM_ERR_INVALID_ARGUMENT, "system " + std::to_string(s) + ": " + e);
        }
        setup_displacement(h->sys[s], systems[s].displacement);
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        delete h;
        return fail(nullptr, SDM_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev) {
        delete h;
        return fail(nullptr, SDM_ERR_INVALID_ARGUMENT, "device index out of range");
    }
    h->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete h; return fail(nullptr, SDM_ERR_CUDA, "cudaSetDevice failed"); }
    if (sdm_pair_prepare() != cudaSuccess) { delete h; return fail(nullptr, SDM_ERR_CUDA, "pair kernel setup failed"); }
    for (int k = 0; k < 3; ++k)
        for (int c = 1; c <= SDM_MAX_CTAS; ++c) h->pair_res[k][c] = sdm_pair_resident(c, 8 + 4 * k);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    if (prop.major < 10) {
        delete h;
        return fail(nullptr, SDM_ERR_NO_DEVICE, "the library is built for sm_103a (Blackwell Ultra)");
    }
    h->pme = h->sys[0].dev.pme != 0;
    for (int s = 1; s < num_systems; ++s)
        if ((h->sys[s].dev.pme != 0) != h->pme) {
            delete h;
            return fail(nullptr, SDM_ERR_INVALID_ARGUMENT, "all systems of a handle must use the same nonbonded_method");
        }
    // replica windows
    long long xo = 0, pg = 0, ps = 0;
    int aw = 0, cw = 0, sw = 0, zw = 0;
    for (int s = 0, r0 = 0; s < num_systems; r0 += h->sys[s].replicas, ++s) {
        h->sys[s].dev.rep0 = r0;
        h->sys[s].dev.nrep = h->sys[s].replicas;
    }
    for (int s = 0; s < num_systems; ++s) {
        const SysHost& S = h->sys[s];
        const long long kp = S.dev.pme ? (long long)S.dev.pme_grid[0] * S.dev.pme_grid[1] * S.dev.pme_grid[2] : 0;
        const long long kh = S.dev.pme ? (long long)S.dev.pme_grid[0] * S.dev.pme_grid[1] * (S.dev.pme_grid[2] / 2 + 1) : 0;
        h->pme_grid_off.push_back(pg);
        h->pme_spec_off.push_back(ps);
        for (int k = 0; k < S.replicas; ++k) {
            SdmRep r{};
            r.sys = s;
            r.pg_win = pg;
            r.pg_size = kp;
            r.ps_win = ps;
            pg += 2 * kp;
            ps += 2 * kh;
            r.n = S.n;
            r.x_off = xo;
            r.atom_win = aw;
            r.col_win = cw;
            r.cel_win = zw;
            r.slot_win = sw;
            r.slot_cap = round8((long long)S.n + 8LL * S.dev.ncol + 8);
            r.cl_win = sw / 8;
            h->rep.push_back(r);
            xo += S.n;
            aw += S.n;
            cw += S.dev.ncol + 1;
            zw += S.dev.ncol * S.dev.M[2] + 1;
            sw += r.slot_cap;
        }
    }
    h->nrep = (int)h->rep.size();
    h->total_particles = xo;
    if (xo > (1LL << 30) || (long long)sw > (1LL << 30) || (long long)zw > (1LL << 30)) {
        delete h;
        return fail(nullptr, SDM_ERR_INVALID_ARGUMENT, "batch too large");
    }
    // arena layout
    int tot_n = 0, tot_excl = 0, tot_D = 0, tot_cx = 0, tot_tab = 0, tot_cxidx = 0, tot_org = 0;
    int tot_expair = 0;
    long long tot_exitem = 0, tot_xcpair = 0;
    for (auto& s : h->sys) {
        tot_n += s.n;
        tot_excl += (int)s.excl_idx.size();
        tot_D += (int)s.D.size();
        tot_cx += (int)s.D.size() + 1;
        tot_tab += 2 * (s.dev.M[0] + s.dev.M[1] + s.dev.M[2]) + 3;
        tot_org += s.dev.M[0] + s.dev.M[1] + s.dev.M[2];
        tot_expair += (int)s.ex_pair.size();
        tot_exitem += (long long)s.ex_pair.size() * s.replicas;
        tot_xcpair += (long long)s.xc_pair.size();
    }
    // the displacement map may change later: reserve the worst case (every particle displaced)
    tot_D = std::max(tot_D, tot_n);
    tot_cx = tot_n + (int)h->sys.size();
    tot_cxidx = std::max(tot_excl, 1);
    const int nrep = h->nrep;
    const long long A = aw, Ccol = cw, Sl = sw, Cl = sw / 8, Ccel = zw;
    long long Pp = 0;
    for (auto& r : h->rep) Pp += 2LL * h->sys[r.sys].n;
    Arena ar;
    SdmArgs& a = h->args;
    const size_t o_sys = ar.take<SdmSys>(h->sys.size());
    const size_t o_rep = ar.take<SdmRep>(nrep);
    const size_t o_q = ar.take<float>(tot_n), o_hs = ar.take<float>(tot_n), o_se = ar.take<float>(tot_n);
    const size_t o_grp = ar.take<int>(tot_n), o_d = ar.take<double>(3LL * tot_n);
    const size_t o_mol = ar.take<int>(tot_n), o_ex4t = ar.take<int4>(tot_n);
    const size_t o_org = ar.take<double>(std::max(tot_org, 1));
    const size_t o_exp = ar.take<int2>(std::max(tot_expair, 1)), o_exq = ar.take<double4_16a>(std::max(tot_expair, 1));
    const size_t o_exe = ar.take<double>(std::max(tot_exitem, 1LL)), o_exu = ar.take<double>(std::max(tot_exitem, 1LL));
    const size_t o_xcp = ar.take<int2>(std::max(tot_xcpair, 1LL)), o_xcq = ar.take<float>(std::max(tot_xcpair, 1LL));
    int max_xc = 0;
    for (auto& s : h->sys) max_xc = std::max(max_xc, (int)s.xc_pair.size());
    const int xc_blocks = std::max(1, (max_xc + 255) / 256);
    const size_t o_xce = ar.take<double>((size_t)nrep * xc_blocks), o_xcu = ar.take<double>((size_t)nrep * xc_blocks);
    long long tot_theta = 0;
    for (auto& s : h->sys) tot_theta += (long long)s.theta.size();
    const int conv_blocks = 64;
    const size_t o_pacc = ar.take<unsigned long long>(std::max(pg, 1LL)), o_pgrid = ar.take<float>(std::max(pg, 1LL));
    const size_t o_pspec = ar.take<float2>(std::max(ps, 1LL)), o_pth = ar.take<float>(std::max(tot_theta, 1LL));
    const size_t o_pep = ar.take<double>((size_t)nrep * conv_blocks), o_pdu = ar.take<double>(std::max(Pp / 2, 1LL));
    int max_bricks = 1, pme_smem = 0;
    for (auto& s : h->sys)
        if (s.dev.pme) {
            max_bricks = std::max(max_bricks, s.dev.pme_nb[0] * s.dev.pme_nb[1] * s.dev.pme_nb[2]);
            pme_smem = std::max(pme_smem, s.dev.pme_cap * 8);
        }
    const size_t o_pbr = ar.take<int4>(2 * (size_t)nrep * max_bricks);
    const size_t o_rsl = ar.take<double>(nrep), o_rse = ar.take<double>(nrep);
    const size_t o_eoff = ar.take<int>(tot_n + 1), o_eidx = ar.take<int>(std::max(tot_excl, 1));
    const size_t o_D = ar.take<int>(std::max(tot_D, 1)), o_cxo = ar.take<int>(tot_cx + 1);
    const size_t o_cxi = ar.take<int>(tot_cxidx), o_tab = ar.take<float>(tot_tab);
    int tot_st = 0;
    for (auto& s : h->sys) tot_st += (int)(s.hst.size() + s.fst.size());
    const size_t o_st2 = ar.take<int2>(std::max(tot_st, 1));
    const size_t o_par = ar.take<double>((size_t)nrep * SDM_NPARAMS);
    const size_t o_x = ar.take<double>(3 * xo), o_res = ar.take<double>((size_t)nrep * SDM_NRESULTS);
    const size_t o_f = ar.take<double>(3 * xo);
    const size_t o_w = ar.take<double>(3 * A), o_ci = ar.take<int2>(A), o_inv = ar.take<int>(A);
    const size_t o_bk = ar.take<int>(A);
    const size_t o_cnt = ar.take<int>(2 * Ccel + nrep + 4);  // counters block: cel_cnt, cel_fill, extz, work
    const size_t o_aoff = ar.take<int>(Ccol), o_cl = ar.take<int>(Ccol), o_ccnt = ar.take<int>(Ccol);
    const size_t o_coff = ar.take<int>(Ccel);
    const size_t o_perm = ar.take<int>(Sl), o_clX = ar.take<float4>(Sl), o_clP = ar.take<float2>(Sl);
    const size_t o_sgrp = ar.take<int>(Sl), o_ex4 = ar.take<int4>(Sl);
    const size_t o_clm = ar.take<int>(Sl);
    const size_t o_F = ar.take<unsigned long long>(6 * Sl);
    const size_t o_ref = ar.take<int4>(Cl), o_bbc = ar.take<float4>(Cl), o_bbh = ar.take<float4>(Cl);
    const size_t o_lnk = ar.take<int4>(2 * Cl), o_ep = ar.take<double>(Cl * SDM_MAX_SPLIT);
    const size_t o_zb = ar.take<float2>(Cl);
    const size_t o_pp = ar.take<double>(std::max(Pp, 1LL) * SDM_PERT_PARTS);   // partials per item
    const size_t o_ppos = ar.take<SdmPertPos>(std::max(Pp, 1LL));
    const size_t o_adj = ar.take<double>(3 * std::max(Pp, 1LL));
    const size_t o_ncl = ar.take<int>(nrep), o_st = ar.take<int>(4), o_srep = ar.take<double>(nrep);
    const size_t o_cmb = ar.take<double>((size_t)nrep * SDM_CMB_FIELDS);
    const size_t o_lv = ar.take<double>(SDM_LV_COUNT);
    const size_t o_counts = ar.take<long long>(2 * nrep), o_ip = ar.take<int>(nrep + 1);
    const size_t o_cp = ar.take<int>(nrep + 1), o_jc = ar.take<int>(Cl);
    const size_t o_done = ar.take<int>(4);
    const size_t o_ngrp = ar.take<int>(nrep), o_lgrp = ar.take<int2>(Cl);
    h->arena_bytes = ar.off + 256;
    cudaError_t ce = cudaMalloc(&h->arena, h->arena_bytes);
    if (ce != cudaSuccess) { h->arena = nullptr; cuda_fail(h, ce, "cudaMalloc(arena)"); return bail(SDM_ERR_CUDA); }
    ce = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { cuda_fail(h, ce, "cudaStreamCreate"); return bail(SDM_ERR_CUDA); }
    ce = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->bridge_ev[0], cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->bridge_ev[1], cudaEventDisableTiming);
    if (ce != cudaSuccess) { cuda_fail(h, ce, "cudaStreamCreate(side)"); return bail(SDM_ERR_CUDA); }
    ce = cudaMemsetAsync(h->arena, 0, h->arena_bytes, h->stream);
    if (ce != cudaSuccess) { cuda_fail(h, ce, "cudaMemset(arena)"); return bail(SDM_ERR_CUDA); }
    for (int k = 0; k < 12; ++k) cudaEventCreate(&h->ev[k]);
    char* B = h->arena;
    a.nsys = (int)h->sys.size();
    a.nrep = nrep;
    a.sys = at<SdmSys>(B, o_sys);
    a.rep = at<SdmRep>(B, o_rep);
    a.topo_q = at<float>(B, o_q);
    a.topo_hs = at<float>(B, o_hs);
    a.topo_se = at<float>(B, o_se);
    a.topo_grp = at<int>(B, o_grp);
    a.topo_mol = at<int>(B, o_mol);
    a.topo_ex4 = at<int4>(B, o_ex4t);
    a.cell_org = at<double>(B, o_org);
    a.ex_pair = at<int2>(B, o_exp);
    a.ex_prm = at<double4_16a>(B, o_exq);
    a.ex_e0 = at<double>(B, o_exe);
    a.ex_du = at<double>(B, o_exu);
    a.xc_pair = at<int2>(B, o_xcp);
    a.xc_qq = at<float>(B, o_xcq);
    a.xc_e0 = at<double>(B, o_xce);
    a.xc_du = at<double>(B, o_xcu);
    a.xc_blocks = xc_blocks;
    a.topo_d = at<double>(B, o_d);
    a.excl_off = at<int>(B, o_eoff);
    a.excl_idx = at<int>(B, o_eidx);
    a.D_idx = at<int>(B, o_D);
    a.cx_off = at<int>(B, o_cxo);
    a.cx_idx = at<int>(B, o_cxi);
    a.shift_tab = at<float>(B, o_tab);
    a.params = at<double>(B, o_par);
    h->params_dev = at<double>(B, o_par);
    h->lv_dev = at<double>(B, o_lv);
    h->x_in = at<double>(B, o_x);
    h->res_in = at<double>(B, o_res);
    h->f_in = at<double>(B, o_f);
    a.w = at<double>(B, o_w);
    a.cellinfo = at<int2>(B, o_ci);
    a.inv = at<int>(B, o_inv);
    a.bucket = at<int>(B, o_bk);
    a.cel_cnt = at<int>(B, o_cnt);
    a.cel_fill = a.cel_cnt + Ccel;
    a.extz = reinterpret_cast<unsigned*>(a.cel_fill + Ccel);
    a.work_counter = reinterpret_cast<int*>(a.extz + nrep);
    h->counters = a.cel_cnt;
    h->counters_bytes = sizeof(int) * (size_t)(2 * Ccel + nrep + 4);
    a.col_cnt = at<int>(B, o_ccnt);
    a.cel_off = at<int>(B, o_coff);
    a.col_aoff = at<int>(B, o_aoff);
    a.col_cl = at<int>(B, o_cl);
    a.perm = at<int>(B, o_perm);
    a.clX = at<float4>(B, o_clX);
    a.clP = at<float2>(B, o_clP);
    a.grp = at<int>(B, o_sgrp);
    a.excl4 = at<int4>(B, o_ex4);
    a.clM = at<int>(B, o_clm);
    unsigned long long* F = at<unsigned long long>(B, o_F);
    a.F0x = F; a.F0y = F + Sl; a.F0z = F + 2 * Sl;
    a.dFx = F + 3 * Sl; a.dFy = F + 4 * Sl; a.dFz = F + 5 * Sl;
    a.cl_ref = at<int4>(B, o_ref);
    a.cl_bbc = at<float4>(B, o_bbc);
    a.cl_bbh = at<float4>(B, o_bbh);
    a.cl_link = at<int4>(B, o_lnk);
    a.cl_zb = at<float2>(B, o_zb);
    a.stencil = at<int2>(B, o_st2);
    a.e_part = at<double>(B, o_ep);
    a.p_part = at<double>(B, o_pp);
    a.s_rep = at<double>(B, o_srep);
    a.cmb = at<double>(B, o_cmb);
    a.pert_pos = at<SdmPertPos>(B, o_ppos);
    a.adj = at<double>(B, o_adj);
    a.ncl = at<int>(B, o_ncl);
    a.ngrp = at<int>(B, o_ngrp);
    a.cl_grp = at<int2>(B, o_lgrp);
    a.status = at<int>(B, o_st);
    a.counts = at<long long>(B, o_counts);
    h->item_prefix = at<int>(B, o_ip);
    h->grp_prefix = at<int>(B, o_cp);
    a.jl_cnt = at<int>(B, o_jc);
    h->done = at<int>(B, o_done);
    a.total_atoms = (int)A;
    a.max_rep_atoms = 0;
    for (auto& r : h->rep) a.max_rep_atoms = std::max(a.max_rep_atoms, r.n);
    a.total_cols = (int)Ccol;
    a.total_cells = (int)Ccel;
    a.pme_charge = a.topo_q;
    a.pme_acc = at<unsigned long long>(B, o_pacc);
    a.pme_grid = at<float>(B, o_pgrid);
    a.pme_spec = at<float2>(B, o_pspec);
    a.pme_theta = at<float>(B, o_pth);
    a.pme_epart = at<double>(B, o_pep);
    a.pme_du = at<double>(B, o_pdu);
    a.pme_total_grid = pg;
    a.pme_conv_blocks = conv_blocks;
    a.pme_brick = at<int4>(B, o_pbr);
    a.rs_lam = at<double>(B, o_rsl);
    a.rs_e = at<double>(B, o_rse);
    a.rs_any = 0;
    {
        std::vector<double> ones(nrep, 1.0);   // SDMRestraintControlParameter defaults to 1
        ce = cudaMemcpy(const_cast<double*>(a.rs_lam), ones.data(), nrep * sizeof(double), cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) { cuda_fail(h, ce, "cudaMemcpy"); return bail(SDM_ERR_CUDA); }
    }
    a.pme_max_bricks = max_bricks;
    a.pme_smem = pme_smem;
    if (h->pme) {   // cuFFT plans: per system, two grids (state 0, dQ) per replica
        ce = sdm_pme_prepare(pme_smem);
        if (ce != cudaSuccess) { cuda_fail(h, ce, "PME kernel setup"); return bail(SDM_ERR_CUDA); }
        for (int s = 0; s < num_systems; ++s) {
            int n[3] = {h->sys[s].dev.pme_grid[0], h->sys[s].dev.pme_grid[1], h->sys[s].dev.pme_grid[2]};
            cufftHandle p1 = 0, p2 = 0;
            if (cufftPlanMany(&p1, 3, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_R2C, 2 * h->sys[s].replicas) != CUFFT_SUCCESS ||
                cufftPlanMany(&p2, 3, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_C2R, 2 * h->sys[s].replicas) != CUFFT_SUCCESS) {
                fail(h, SDM_ERR_CUDA, "cufftPlanMany failed");
                return bail(SDM_ERR_CUDA);
            }
            h->pme_r2c.push_back(p1);
            h->pme_c2r.push_back(p2);
        }
    }
    a.total_slots = (int)Sl;
    // list-building groups of four clusters, also for a single replica: with
    // the perturbation pass running beside the list build, the fewer, longer
    // list-building warps leave it room (1-replica call 0.115 ms against
    // 0.120 ms with groups of 1 or 2)
    h->auto_list_group = SDM_JG;
    a.jg = h->auto_list_group;
    a.split = 1;
    a.ex_cap = 0;
    a.ex_rep = -1;
    // parameters
    h->params.resize((size_t)nrep * SDM_NPARAMS);
    for (int r = 0; r < nrep; ++r) default_params(&h->params[(size_t)r * SDM_NPARAMS]);
    ce = cudaMallocHost(&h->params_pinned, (h->params.size() + SDM_LV_COUNT) * sizeof(double));
    if (ce != cudaSuccess) { h->params_pinned = nullptr; cuda_fail(h, ce, "cudaMallocHost"); return bail(SDM_ERR_CUDA); }
    // cluster-pair list capacity: twice the expected count of clusters within
    // rc + 1.5 cluster edges over a half shell, at the densest system
    double need = 64.0;
    for (auto& s : h->sys) {
        const double vol = s.dev.box[0] * s.dev.box[1] * s.dev.box[2];
        const double rho = s.n / vol;
        const double edge = std::cbrt(8.0 / rho);
        const double rr = s.dev.rc + 1.5 * edge;
        need = std::max(need, 0.5 * rho / 8.0 * 4.18879 * rr * rr * rr);
    }
    h->jl_clusters = Cl;
    sdm_status st = sdm_reserve_lists(h, (int)std::min(4096.0, 2.0 * need + 64.0));
    if (st) return bail(st);
    st = upload_topology(h);
    if (st) return bail(st);
    *out = h;
    return SDM_OK;
}

sdm_status sdm_destroy(sdm_handle* h) {
    if (!h) return SDM_OK;
    if (h->jl_buf) { cudaSetDevice(h->device); cudaFree(h->jl_buf); h->jl_buf = nullptr; }
    if (h->rs_buf) { cudaSetDevice(h->device); cudaFree(h->rs_buf); h->rs_buf = nullptr; }
    if (h->st_buf) { cudaSetDevice(h->device); cudaFree(h->st_buf); h->st_buf = nullptr; }
    if (h->arena) cudaSetDevice(h->device);
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    for (int k = 0; k < 12; ++k) if (h->ev[k]) cudaEventDestroy(h->ev[k]);
    for (auto p : h->pme_r2c) cufftDestroy(p);
    for (auto p : h->pme_c2r) cufftDestroy(p);
    if (h->stream) { cudaStreamSynchronize(h->stream); cudaStreamDestroy(h->stream); }
    if (h->side) { cudaStreamSynchronize(h->side); cudaStreamDestroy(h->side); }
    if (h->fork_ev) cudaEventDestroy(h->fork_ev);
    if (h->join_ev) cudaEventDestroy(h->join_ev);
    for (cudaEvent_t e : h->bridge_ev) if (e) cudaEventDestroy(e);
    if (h->arena) cudaFree(h->arena);
    if (h->params_pinned) cudaFreeHost(h->params_pinned);
    delete h;
    return SDM_OK;
}

const char* sdm_last_error(const sdm_handle* h) {
    return h ? h->err.c_str() : g_create_error.c_str();
}

sdm_status sdm_num_replicas(const sdm_handle* h, int* out) {
    if (!h || !out) return SDM_ERR_INVALID_ARGUMENT;
    *out = h->nrep;
    return SDM_OK;
}

sdm_status sdm_set_displacement(sdm_handle* h, int system, const double* displacement) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    if (system < 0 || system >= (int)h->sys.size()) return fail(h, SDM_ERR_INVALID_ARGUMENT, "system index out of range");
    if (displacement)
        for (size_t k = 0; k < 3 * (size_t)h->sys[system].n; ++k)
            if (!std::isfinite(displacement[k])) return fail(h, SDM_ERR_INVALID_ARGUMENT, "non-finite displacement");
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    setup_displacement(h->sys[system], displacement);
    return upload_topology(h);
}

// Restraint data of every system into one device buffer (parameters,
// weights, particle indices) and the systems' offsets into the device SdmSys
// array; the cached graphs hold the previous pointers and are dropped.
static sdm_status upload_restraints(sdm_handle* h) {
    std::vector<int> idx;
    std::vector<double> w, prm;
    int any = 0;
    for (auto& s : h->sys) {
        s.dev.rs_on = s.rs_on;
        s.dev.rs_base = (int)idx.size();
        s.dev.rs_nlig = s.rs_nlig;
        s.dev.rs_nrcpt = s.rs_nrcpt;
        s.dev.rs_prm = (int)prm.size();
        std::copy(s.rs_ref, s.rs_ref + 12, s.dev.rs_ref);
        idx.insert(idx.end(), s.rs_idx.begin(), s.rs_idx.end());
        w.insert(w.end(), s.rs_w.begin(), s.rs_w.end());
        prm.insert(prm.end(), s.rs_prm, s.rs_prm + SDM_RS_COUNT);
        any |= s.rs_on ? 1 : 0;
    }
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    SDM_CUDA(h, cudaDeviceSynchronize());
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    if (h->rs_buf) { cudaFree(h->rs_buf); h->rs_buf = nullptr; }
    // no kernel may see the freed buffer if the allocation below fails
    h->args.rs_prm = h->args.rs_w = nullptr;
    h->args.rs_idx = nullptr;
    h->args.rs_any = 0;
    const size_t nd = prm.size() + w.size();
    SDM_CUDA(h, cudaMalloc(&h->rs_buf, nd * sizeof(double) + idx.size() * sizeof(int) + 16));
    double* dp = static_cast<double*>(h->rs_buf);
    SDM_CUDA(h, cudaMemcpy(dp, prm.data(), prm.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (!w.empty()) SDM_CUDA(h, cudaMemcpy(dp + prm.size(), w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice));
    int* ip = reinterpret_cast<int*>(dp + nd);
    if (!idx.empty()) SDM_CUDA(h, cudaMemcpy(ip, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice));
    h->args.rs_prm = dp;
    h->args.rs_w = dp + prm.size();
    h->args.rs_idx = ip;
    h->args.rs_any = any;
    return upload_topology(h);
}

sdm_status sdm_set_restraints(sdm_handle* h, int system, const sdm_restraints* r) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    if (system < 0 || system >= (int)h->sys.size()) return fail(h, SDM_ERR_INVALID_ARGUMENT, "system index out of range");
    cudaSetDevice(h->device);
    SysHost& s = h->sys[system];
    if (!r) {
        s.rs_on = s.rs_nlig = s.rs_nrcpt = 0;
        s.rs_idx.clear();
        s.rs_w.clear();
        return upload_restraints(h);
    }
    const int n = s.n;
    auto bad = [&](const char* m) { return fail(h, SDM_ERR_INVALID_ARGUMENT, m); };
    auto in_range = [n](int i) { return i >= 0 && i < n; };
    auto finite = [](std::initializer_list<double> v) {
        for (double x : v)
            if (!std::isfinite(x)) return false;
        return true;
    };
    if (r->num_lig < 0 || r->num_rcpt < 0) return bad("negative restraint group size");
    int on = 0;
    std::vector<int> idx;
    std::vector<double> w;
    double wsum[2] = {0.0, 0.0};
    if (r->num_lig > 0 && r->num_rcpt > 0) {
        if (!r->lig_particles || !r->rcpt_particles) return bad("restraint group particles missing");
        for (int g = 0; g < 2; ++g) {
            const int m = g ? r->num_rcpt : r->num_lig;
            const int* p = g ? r->rcpt_particles : r->lig_particles;
            const double* wt = g ? r->rcpt_weights : r->lig_weights;
            for (int k = 0; k < m; ++k) {
                if (!in_range(p[k])) return bad("restraint particle index out of range");
                const double wk = wt ? wt[k] : 1.0;
                if (!(wk > 0.0) || !std::isfinite(wk)) return bad("restraint weights must be positive");
                idx.push_back(p[k]);
                w.push_back(wk);
                wsum[g] += wk;
            }
        }
        if (!finite({r->kfcm, r->tolcm, r->offset[0], r->offset[1], r->offset[2]}) || r->tolcm < 0.0)
            return bad("invalid centroid restraint parameters");
        on |= 1;
        if (r->use_angles) {
            for (int k = 0; k < 3; ++k)
                if (!in_range(r->rcpt_ref[k]) || !in_range(r->lig_ref[k])) return bad("reference particle out of range");
            if (!finite({r->kf_angle, r->angle_center, r->angle_tol, r->kf_dihedral1, r->dihedral1_center,
                         r->dihedral1_tol, r->kf_dihedral2, r->dihedral2_center, r->dihedral2_tol}))
                return bad("invalid angle restraint parameters");
            on |= 2;
        }
    } else if (r->use_angles) {
        return bad("the angle restraint terms need both centroid groups");
    }
    if (r->use_alignment) {
        for (int k = 0; k < 3; ++k)
            if (!in_range(r->liga_ref[k]) || !in_range(r->ligb_ref[k])) return bad("alignment particle out of range");
        if (!finite({r->kf_displ, r->k_theta, r->k_psi, r->align_offset[0], r->align_offset[1], r->align_offset[2]}))
            return bad("invalid alignment restraint parameters");
        on |= 4;
    }
    s.rs_idx = idx;
    s.rs_w = w;
    s.rs_nlig = (on & 1) ? r->num_lig : 0;
    s.rs_nrcpt = (on & 1) ? r->num_rcpt : 0;
    double* P = s.rs_prm;
    std::fill(P, P + SDM_RS_COUNT, 0.0);
    P[SDM_RS_KFCM] = r->kfcm;
    P[SDM_RS_TOLCM] = r->tolcm;
    for (int k = 0; k < 3; ++k) P[SDM_RS_OFF + k] = r->offset[k];
    P[SDM_RS_INVW_LIG] = wsum[0] > 0.0 ? 1.0 / wsum[0] : 0.0;
    P[SDM_RS_INVW_RCPT] = wsum[1] > 0.0 ? 1.0 / wsum[1] : 0.0;
    // windows [center - tol, center + tol] (SDMUtils.py:140-149)
    P[SDM_RS_KFA] = r->kf_angle;
    P[SDM_RS_ALO] = r->angle_center - r->angle_tol;
    P[SDM_RS_AHI] = r->angle_center + r->angle_tol;
    P[SDM_RS_KFD1] = r->kf_dihedral1;
    P[SDM_RS_D1LO] = r->dihedral1_center - r->dihedral1_tol;
    P[SDM_RS_D1HI] = r->dihedral1_center + r->dihedral1_tol;
    P[SDM_RS_KFD2] = r->kf_dihedral2;
    P[SDM_RS_D2LO] = r->dihedral2_center - r->dihedral2_tol;
    P[SDM_RS_D2HI] = r->dihedral2_center + r->dihedral2_tol;
    P[SDM_RS_KDISPL] = r->kf_displ;
    P[SDM_RS_KTHETA] = r->k_theta;
    P[SDM_RS_KPSI] = r->k_psi;
    for (int k = 0; k < 3; ++k) P[SDM_RS_AOFF + k] = r->align_offset[k];
    for (int k = 0; k < 3; ++k) {
        s.rs_ref[k] = (on & 2) ? r->rcpt_ref[k] : 0;
        s.rs_ref[3 + k] = (on & 2) ? r->lig_ref[k] : 0;
        s.rs_ref[6 + k] = (on & 4) ? r->liga_ref[k] : 0;
        s.rs_ref[9 + k] = (on & 4) ? r->ligb_ref[k] : 0;
    }
    s.rs_on = on;
    return upload_restraints(h);
}

// Rigid-water data of every system into one device buffer (water triples,
// per-particle flags, the per-particle scratch of unconstrained positions);
// the cached graphs hold the previous pointers and are dropped.
static sdm_status upload_rigid_waters(sdm_handle* h) {
    std::vector<int> idx, flag;
    int any = 0, mx = 0;
    for (auto& s : h->sys) {
        s.dev.st_base = (int)(idx.size() / 3);
        s.dev.st_count = (int)(s.st_idx.size() / 3);
        s.dev.st_doh = s.st_doh;
        s.dev.st_dhh = s.st_dhh;
        idx.insert(idx.end(), s.st_idx.begin(), s.st_idx.end());
        std::vector<int> f(s.n, 0);
        for (int v : s.st_idx) f[v] = 1;
        flag.insert(flag.end(), f.begin(), f.end());
        any |= s.dev.st_count ? 1 : 0;
        mx = std::max(mx, s.dev.st_count);
    }
    SDM_CUDA(h, cudaDeviceSynchronize());
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    if (h->st_buf) { cudaFree(h->st_buf); h->st_buf = nullptr; }
    // no kernel may see the freed buffer if the allocation below fails
    h->args.lv_xp = nullptr;
    h->args.st_idx = h->args.st_flag = nullptr;
    h->args.st_any = h->args.st_max = 0;
    const size_t nxp = 3 * (size_t)h->total_particles;
    SDM_CUDA(h, cudaMalloc(&h->st_buf, nxp * sizeof(double) + (idx.size() + flag.size()) * sizeof(int) + 16));
    double* xp = static_cast<double*>(h->st_buf);
    int* ip = reinterpret_cast<int*>(xp + nxp);
    if (!idx.empty()) SDM_CUDA(h, cudaMemcpy(ip, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice));
    SDM_CUDA(h, cudaMemcpy(ip + idx.size(), flag.data(), flag.size() * sizeof(int), cudaMemcpyHostToDevice));
    h->args.lv_xp = xp;
    h->args.st_idx = ip;
    h->args.st_flag = ip + idx.size();
    h->args.st_any = any;
    h->args.st_max = mx;
    return upload_topology(h);
}

sdm_status sdm_set_rigid_waters(sdm_handle* h, int system, int num_waters, const int* waters, double d_oh,
                                double d_hh) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    if (system < 0 || system >= (int)h->sys.size()) return fail(h, SDM_ERR_INVALID_ARGUMENT, "system index out of range");
    if (num_waters < 0 || (num_waters > 0 && !waters)) return fail(h, SDM_ERR_INVALID_ARGUMENT, "invalid water list");
    SysHost& s = h->sys[system];
    if (num_waters > 0) {
        if (!(d_oh > 0.0) || !(d_hh > 0.0) || !(d_hh < 2.0 * d_oh) || !std::isfinite(d_oh) || !std::isfinite(d_hh))
            return fail(h, SDM_ERR_INVALID_ARGUMENT, "water distances must satisfy 0 < d_hh < 2 d_oh");
        std::vector<char> used(s.n, 0);
        for (int k = 0; k < 3 * num_waters; ++k) {
            const int i = waters[k];
            if (i < 0 || i >= s.n) return fail(h, SDM_ERR_INVALID_ARGUMENT, "water particle index out of range");
            if (used[i]) return fail(h, SDM_ERR_INVALID_ARGUMENT, "a particle belongs to two waters");
            used[i] = 1;
        }
    }
    cudaSetDevice(h->device);
    s.st_idx.assign(waters, waters + 3 * (size_t)num_waters);
    s.st_doh = num_waters ? d_oh : 0.0;
    s.st_dhh = num_waters ? d_hh : 0.0;
    return upload_rigid_waters(h);
}

sdm_status sdm_set_restraint_control(sdm_handle* h, int replica, double lambda_r) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    if (replica < 0 || replica >= h->nrep) return fail(h, SDM_ERR_INVALID_ARGUMENT, "replica index out of range");
    if (!std::isfinite(lambda_r)) return fail(h, SDM_ERR_INVALID_ARGUMENT, "non-finite restraint control parameter");
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaDeviceSynchronize());   // no evaluation in flight reads the old value
    SDM_CUDA(h, cudaMemcpy(const_cast<double*>(h->args.rs_lam) + replica, &lambda_r, sizeof(double),
                           cudaMemcpyHostToDevice));
    return SDM_OK;
}

sdm_status sdm_get_restraint_energies(sdm_handle* h, double* energies) {
    if (!h || !energies) return SDM_ERR_INVALID_ARGUMENT;
    if (!h->args.rs_any) {
        std::fill(energies, energies + h->nrep, 0.0);
        return SDM_OK;
    }
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaDeviceSynchronize());
    SDM_CUDA(h, cudaMemcpy(energies, h->args.rs_e, h->nrep * sizeof(double), cudaMemcpyDeviceToHost));
    return SDM_OK;
}

sdm_status sdm_set_params(sdm_handle* h, int replica, const double* params) {
    if (!h || !params) return SDM_ERR_INVALID_ARGUMENT;
    if (replica < 0 || replica >= h->nrep) return fail(h, SDM_ERR_INVALID_ARGUMENT, "replica index out of range");
    // compared as doubles: a cast of NaN or of a huge value to int is undefined
    const double bm = params[SDM_P_BIAS_METHOD], sm = params[SDM_P_SOFTCORE_METHOD];
    if (!(bm == 0.0 || bm == 1.0 || bm == 2.0)) return fail(h, SDM_ERR_UNKNOWN_METHOD, "Unknown bias method");
    if (!(sm == 0.0 || sm == 1.0 || sm == 2.0)) return fail(h, SDM_ERR_UNKNOWN_METHOD, "Unknown soft core method");
    std::memcpy(&h->params[(size_t)replica * SDM_NPARAMS], params, sizeof(double) * SDM_NPARAMS);
    h->params_dirty = true;
    return SDM_OK;
}

// Device address of a page-locked, mapped host buffer (a kernel then reads it
// directly over the host link), or null for any other pointer.
static void* mapped_host(const void* p) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();   // clear the lookup error
        return nullptr;
    }
    return (pa.type == cudaMemoryTypeHost) ? pa.devicePointer : nullptr;
}

sdm_status sdm_evaluate(sdm_handle* h, const double* x, double* results, double* forces) {
    if (!h || !x) return SDM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    const size_t nx = 3 * (size_t)h->total_particles;
    // optionally page-locked coordinates are read in place by k_cells (no
    // staging copy; measured on par with the copy); results and forces always
    // return through copy-engine transfers, which beat kernel stores into host
    // memory (0.98 vs 1.11 ms per 22-replica call)
    const double* xd = h->opt_zero_copy ? static_cast<const double*>(mapped_host(x)) : nullptr;
    if (!xd) {
        SDM_CUDA(h, cudaMemcpyAsync(h->x_in, x, nx * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        xd = h->x_in;
    }
    sdm_status s = run(h, xd, h->res_in, h->f_in, h->stream, 0, true);
    if (s) return s;
    if (results)
        SDM_CUDA(h, cudaMemcpyAsync(results, h->res_in, sizeof(double) * SDM_NRESULTS * h->nrep,
                                    cudaMemcpyDeviceToHost, h->stream));
    if (forces)
        SDM_CUDA(h, cudaMemcpyAsync(forces, h->f_in, nx * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    // the status word is read after every host call; it is cleared here only
    // when this call acts on it (list regrow, or verification on).  With a
    // results buffer the word comes back in it: every status source runs
    // before or inside the finalize kernel, and each replica's SDM_R_STATUS
    // holds the word as its block saw it plus its own flags, so their OR is
    // the word (a separate read only when it is nonzero)
    int v = 0;
    if (results) {
        for (int r = 0; r < h->nrep; ++r) v |= (int)results[(size_t)r * SDM_NRESULTS + SDM_R_STATUS];
        if (v) {
            s = check_dev_status(h, &v, false);
            if (s) return s;
        }
    } else {
        s = check_dev_status(h, &v, false);
        if (s) return s;
    }
    if (v & SDM_DEV_LIST_OVERFLOW) {
        SDM_CUDA(h, cudaMemset(h->args.status, 0, sizeof(int)));
        // lists too small for these coordinates: regrow and evaluate again
        if (h->jl_cap >= (1 << 16)) return fail(h, SDM_ERR_CAPACITY, "cluster-pair list capacity limit reached");
        s = regrow_lists(h);
        if (s) return s;
        return sdm_evaluate(h, x, results, forces);
    }
    if (h->opt_verify && v) {
        SDM_CUDA(h, cudaMemset(h->args.status, 0, sizeof(int)));
        return fail(h, SDM_ERR_OVERFLOW, "device status " + std::to_string(v) +
                                             ": force overflow, non-finite energy or non-finite coordinates");
    }
    return SDM_OK;
}

sdm_status sdm_evaluate_device(sdm_handle* h, const double* x, double* results, double* forces, void* stream) {
    if (!h || !x || !results) return SDM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    return run(h, x, results, forces, st, 0, true);
}

sdm_status sdm_evaluate_engine(sdm_handle* h, const void* posq, const void* posq_correction, int double_precision,
                               const int* index, int padded_n, long long* force_buffer, double* results,
                               void* stream) {
    if (!h || !posq || !index) return SDM_ERR_INVALID_ARGUMENT;
    const int n = (int)h->total_particles;
    if (padded_n < n) return fail(h, SDM_ERR_INVALID_ARGUMENT, "padded_n is below the particle count");
    cudaSetDevice(h->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    SDM_CUDA(h, sdm_launch_gather_positions(posq, posq_correction, double_precision, index, n, h->x_in, st));
    sdm_status s = run(h, h->x_in, h->res_in, force_buffer ? h->f_in : nullptr, st, 0, true);
    if (s) return s;
    if (results) {
        // the synchronous form validates before the forces go out: a list
        // overflow regrows the lists and evaluates again
        for (int attempt = 0;; ++attempt) {
            SDM_CUDA(h, cudaMemcpyAsync(results, h->res_in, sizeof(double) * SDM_NRESULTS * h->nrep,
                                        cudaMemcpyDeviceToHost, st));
            SDM_CUDA(h, cudaStreamSynchronize(st));
            int v = 0;
            for (int r = 0; r < h->nrep; ++r) v |= (int)results[(size_t)r * SDM_NRESULTS + SDM_R_STATUS];
            if (!(v & SDM_DEV_LIST_OVERFLOW)) {
                if (v) {
                    SDM_CUDA(h, cudaMemset(h->args.status, 0, sizeof(int)));
                    if (h->opt_verify) return fail(h, SDM_ERR_OVERFLOW, "device status error (see SDM_R_STATUS)");
                }
                break;
            }
            SDM_CUDA(h, cudaMemset(h->args.status, 0, sizeof(int)));
            if (attempt >= 8) return fail(h, SDM_ERR_CAPACITY, "cluster-pair lists keep overflowing");
            s = regrow_lists(h);
            if (s) return s;
            s = run(h, h->x_in, h->res_in, force_buffer ? h->f_in : nullptr, st, 0, true);
            if (s) return s;
        }
    }
    if (force_buffer) SDM_CUDA(h, sdm_launch_scatter_forces(h->f_in, index, n, padded_n, force_buffer, st));
    return SDM_OK;
}

sdm_status sdm_get_last_results(sdm_handle* h, double* results) {
    if (!h || !results) return SDM_ERR_INVALID_ARGUMENT;
    if (!h->have_eval) return fail(h, SDM_ERR_INVALID_ARGUMENT, "no evaluation yet");
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaDeviceSynchronize());
    SDM_CUDA(h, cudaMemcpy(results, h->res_in, sizeof(double) * SDM_NRESULTS * h->nrep, cudaMemcpyDeviceToHost));
    return SDM_OK;
}

sdm_status sdm_set_langevin(sdm_handle* h, const sdm_langevin_params* p, unsigned long long step) {
    if (!h || !p) return SDM_ERR_INVALID_ARGUMENT;
    if (!(p->step_size > 0.0) || !std::isfinite(p->step_size))
        return fail(h, SDM_ERR_INVALID_ARGUMENT, "step size must be positive");
    // the reference sets tau = 1/friction and 0 for zero friction, which makes
    // its noise scale sqrt(2kT/0) undefined (ReferenceSDMKernels.cpp:327)
    if (!(p->friction > 0.0) || !std::isfinite(p->friction))
        return fail(h, SDM_ERR_INVALID_ARGUMENT, "friction must be positive");
    if (!(p->temperature >= 0.0) || !std::isfinite(p->temperature))
        return fail(h, SDM_ERR_INVALID_ARGUMENT, "temperature must be non-negative");
    // ReferenceStochasticDynamicsSDM.cpp:145-148
    const double tau = 1.0 / p->friction, dt = p->step_size;
    const double vscale = std::exp(-dt / tau);
    const double fscale = (1.0 - vscale) * tau;
    const double kT = kMolarGasConstant * p->temperature;
    const double noise = std::sqrt(2.0 * kT / tau) * std::sqrt(0.5 * (1.0 - vscale * vscale) * tau);
    double* q = h->lv_host;
    q[SDM_LV_DT] = dt;
    q[SDM_LV_VSCALE] = vscale;
    q[SDM_LV_FSCALE] = fscale;
    q[SDM_LV_NOISE] = noise;
    q[SDM_LV_INVDT] = 1.0 / dt;
    std::memcpy(&q[SDM_LV_SEED], &p->seed, 8);
    std::memcpy(&q[SDM_LV_STEP], &step, 8);
    h->lv_set = true;
    h->lv_dirty = true;
    return SDM_OK;
}

sdm_status sdm_langevin_step(sdm_handle* h, double* x, double* v, const double* inv_mass, const double* f_extra,
                             double* results, int nsteps, void* stream) {
    if (!h || !x || !v || !inv_mass || !results || nsteps < 0) return SDM_ERR_INVALID_ARGUMENT;
    if (!h->lv_set) return fail(h, SDM_ERR_INVALID_ARGUMENT, "sdm_set_langevin was not called");
    cudaSetDevice(h->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    const LvBind lv{x, v, inv_mass, f_extra};
    for (int k = 0; k < nsteps; ++k) {
        sdm_status s = run(h, x, results, nullptr, st, 0, true, &lv);
        if (s) return s;
    }
    return SDM_OK;
}

sdm_status sdm_get_state_forces(sdm_handle* h, double* F0, double* F1, int on_device) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    if (!h->have_eval) return fail(h, SDM_ERR_INVALID_ARGUMENT, "no evaluation yet");
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaDeviceSynchronize());
    const size_t nx = 3 * (size_t)h->total_particles;
    SdmArgs a = h->args;
    a.forces = nullptr;
    a.results = h->res_in;
    if (on_device) {
        a.F0out = F0;
        a.F1out = F1;
        SDM_CUDA(h, sdm_launch_mix(a, h->stream));
    } else {
        // stage through the internal force buffer, one state at a time
        if (F0) {
            a.F0out = h->f_in;
            a.F1out = nullptr;
            SDM_CUDA(h, sdm_launch_mix(a, h->stream));
            SDM_CUDA(h, cudaMemcpyAsync(F0, h->f_in, nx * 8, cudaMemcpyDeviceToHost, h->stream));
        }
        if (F1) {
            a.F0out = nullptr;
            a.F1out = h->f_in;
            SDM_CUDA(h, sdm_launch_mix(a, h->stream));
            SDM_CUDA(h, cudaMemcpyAsync(F1, h->f_in, nx * 8, cudaMemcpyDeviceToHost, h->stream));
        }
    }
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    return SDM_OK;
}

sdm_status sdm_get_state_forces_device(sdm_handle* h, double* F0, double* F1, void* stream) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    if (!h->have_eval) return fail(h, SDM_ERR_INVALID_ARGUMENT, "no evaluation yet");
    if (!F0 && !F1) return SDM_OK;
    cudaSetDevice(h->device);
    SdmArgs a = h->args;
    a.forces = nullptr;
    a.F0out = F0;
    a.F1out = F1;
    SDM_CUDA(h, sdm_launch_mix(a, stream ? (cudaStream_t)stream : h->stream));
    return SDM_OK;
}

sdm_status sdm_gather_positions(const void* posq, const void* posq_correction, int double_precision,
                                const int* index, int n, double* x, void* stream) {
    if (!posq || !index || !x || n < 0) {
        sdm_set_thread_error("sdm_gather_positions: NULL array or negative count");
        return SDM_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return SDM_OK;
    const cudaError_t e = sdm_launch_gather_positions(posq, posq_correction, double_precision, index, n, x,
                                                      (cudaStream_t)stream);
    if (e != cudaSuccess) {
        sdm_set_thread_error(cudaGetErrorString(e));
        return SDM_ERR_CUDA;
    }
    return SDM_OK;
}

sdm_status sdm_scatter_forces_fixed(const double* forces, const int* index, int n, int padded_n,
                                    long long* buffer, void* stream) {
    if (!forces || !index || !buffer || n < 0 || padded_n < n) {
        sdm_set_thread_error("sdm_scatter_forces_fixed: NULL array or bad sizes");
        return SDM_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return SDM_OK;
    const cudaError_t e = sdm_launch_scatter_forces(forces, index, n, padded_n, buffer, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        sdm_set_thread_error(cudaGetErrorString(e));
        return SDM_ERR_CUDA;
    }
    return SDM_OK;
}

sdm_status sdm_set_particle_params(sdm_handle* h, int system, int n, const int* index,
                                   const double* charge, const double* sigma, const double* epsilon) {
    if (!h || n < 0 || (n > 0 && (!index || !charge || !sigma || !epsilon))) return SDM_ERR_INVALID_ARGUMENT;
    if (system < 0 || system >= (int)h->sys.size()) return fail(h, SDM_ERR_INVALID_ARGUMENT, "system index out of range");
    SysHost& S = h->sys[system];
    const double sk = std::sqrt(kCoulomb);
    for (int k = 0; k < n; ++k) {
        const int i = index[k];
        if (i < 0 || i >= S.n) return fail(h, SDM_ERR_INVALID_ARGUMENT, "particle index out of range");
        if (!(sigma[k] >= 0.0) || !(epsilon[k] >= 0.0) || !std::isfinite(sigma[k]) || !std::isfinite(epsilon[k]) ||
            !std::isfinite(charge[k]))
            return fail(h, SDM_ERR_INVALID_ARGUMENT, "sigma/epsilon must be finite and >= 0, charges finite");
    }
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < n; ++k) {
        const int i = index[k];
        S.q[i] = (float)(charge[k] * sk);
        S.hs[i] = (float)(0.5 * sigma[k]);
        S.se[i] = (float)(2.0 * std::sqrt(epsilon[k]));
    }
    h->have_eval = false;
    return upload_topology(h);
}

sdm_status sdm_adjoint(sdm_handle* h, double* out) {
    if (!h || !out) return SDM_ERR_INVALID_ARGUMENT;
    if (h->pme) return fail(h, SDM_ERR_INVALID_ARGUMENT, "parameter derivatives are reaction-field only");
    if (!h->have_eval) return fail(h, SDM_ERR_INVALID_ARGUMENT, "no evaluation yet");
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaDeviceSynchronize());
    SDM_CUDA(h, sdm_launch_adjoint(h->args, h->stream));
    const size_t n = 3 * (size_t)h->args.total_pert;
    if (n) SDM_CUDA(h, cudaMemcpyAsync(out, h->args.adj, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    return SDM_OK;
}

sdm_status sdm_backward_device(sdm_handle* h, const double* grad_u, const double* results, const double* forces,
                               const double* forces1, const double* adjoint, const double* eps_displaced,
                               const double* bias_params, double* grad_x, double* grad_d, double* grad_p,
                               double* grad_bias, void* stream) {
    if (!h || !grad_u || !results) return SDM_ERR_INVALID_ARGUMENT;
    if ((grad_x && !forces) || ((grad_d || grad_p) && !results) || (grad_d && !forces1) || (grad_p && !adjoint))
        return fail(h, SDM_ERR_INVALID_ARGUMENT, "sdm_backward_device: an output lacks its input");
    if (grad_p && h->pme) return fail(h, SDM_ERR_INVALID_ARGUMENT, "parameter derivatives are reaction-field only");
    cudaSetDevice(h->device);
    long long atoms = 0, nd = 0;
    for (const SysHost& s : h->sys) {
        atoms += s.n;
        nd += (long long)s.D.size();
    }
    BwdArgs b{};
    b.g = grad_u;
    b.res = results;
    b.F = forces;
    b.F1 = forces1;
    b.G = adjoint;
    b.eps = eps_displaced;
    b.prm = bias_params;
    b.gx = grad_x;
    b.gd = grad_d;
    b.gp = grad_p;
    b.gb = grad_bias;
    b.n_x = grad_x ? 3 * (long long)h->total_particles : 0;
    b.n_d = grad_d ? 3 * atoms : 0;
    b.n_p = grad_p ? 3 * nd : 0;
    b.n_b = grad_bias ? 5LL * h->nrep : 0;
    SDM_CUDA(h, sdm_launch_backward(h->args, b, stream ? (cudaStream_t)stream : h->stream));
    return SDM_OK;
}

sdm_status sdm_adjoint_device(sdm_handle* h, double* out, void* stream) {
    if (!h || !out) return SDM_ERR_INVALID_ARGUMENT;
    if (h->pme) return fail(h, SDM_ERR_INVALID_ARGUMENT, "parameter derivatives are reaction-field only");
    if (!h->have_eval) return fail(h, SDM_ERR_INVALID_ARGUMENT, "no evaluation yet");
    cudaSetDevice(h->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    SDM_CUDA(h, sdm_launch_adjoint(h->args, st));
    const size_t n = 3 * (size_t)h->args.total_pert;
    if (n) SDM_CUDA(h, cudaMemcpyAsync(out, h->args.adj, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    return SDM_OK;
}

sdm_status sdm_get_num_perturbed(const sdm_handle* h, int* count) {
    if (!h || !count) return SDM_ERR_INVALID_ARGUMENT;
    *count = h->args.total_pert / 2;
    return SDM_OK;
}

sdm_status sdm_check_status(sdm_handle* h, int* device_status) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    SDM_CUDA(h, cudaDeviceSynchronize());
    int v = 0;
    sdm_status s = check_dev_status(h, &v, true);
    if (s) return s;
    if (device_status) *device_status = v;
    if (v & SDM_DEV_LIST_OVERFLOW) {
        s = regrow_lists(h);
        if (s) return s;
        return fail(h, SDM_ERR_CAPACITY, "cluster-pair lists overflowed and were regrown: evaluate again");
    }
    return SDM_OK;
}

sdm_status sdm_set_option(sdm_handle* h, int option, int value) {
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    switch (option) {
        case SDM_OPT_GRAPH: h->opt_graph = value ? 1 : 0; break;
        case SDM_OPT_PROFILE:
            if (value < 0 || value > 2) return fail(h, SDM_ERR_INVALID_ARGUMENT, "profile must be 0, 1 or 2");
            h->opt_profile = value;
            break;
        case SDM_OPT_SPLIT:
            if (value != 1 && value != 2 && value != 4) return fail(h, SDM_ERR_INVALID_ARGUMENT, "split must be 1, 2 or 4");
            h->opt_split = value;
            break;
        case SDM_OPT_CTAS_PER_SM:
            if (value < 1 || value > SDM_MAX_CTAS)
                return fail(h, SDM_ERR_INVALID_ARGUMENT, "ctas per SM must be in 1..4");
            h->opt_ctas = value;
            break;
        case SDM_OPT_VERIFY: h->opt_verify = value ? 1 : 0; break;
        case SDM_OPT_ZERO_COPY: h->opt_zero_copy = value ? 1 : 0; break;
        case SDM_OPT_STAGE_CHUNK:
            if (value != 8 && value != 12 && value != 16)
                return fail(h, SDM_ERR_INVALID_ARGUMENT, "stage chunk must be 8, 12 or 16");
            h->opt_chunk = value;
            break;
        case SDM_OPT_OVERLAP:
            if (value < 0 || value > 2) return fail(h, SDM_ERR_INVALID_ARGUMENT, "overlap must be 0, 1 or 2");
            h->opt_overlap = value;
            break;
        case SDM_OPT_LIST_GROUP:
            if (value != 0 && value != 1 && value != 2 && value != SDM_JG)
                return fail(h, SDM_ERR_INVALID_ARGUMENT, "list group must be 0 (automatic), 1, 2 or 4");
            h->opt_list_group = value;
            break;
        default: return fail(h, SDM_ERR_INVALID_ARGUMENT, "unknown option");
    }
    return SDM_OK;
}

sdm_status sdm_get_option(const sdm_handle* h, int option, int* value) {
    if (!h || !value) return SDM_ERR_INVALID_ARGUMENT;
    switch (option) {
        case SDM_OPT_GRAPH: *value = h->opt_graph; break;
        case SDM_OPT_PROFILE: *value = h->opt_profile; break;
        case SDM_OPT_SPLIT: *value = h->opt_split; break;
        case SDM_OPT_CTAS_PER_SM: *value = h->opt_ctas; break;
        case SDM_OPT_VERIFY: *value = h->opt_verify; break;
        case SDM_OPT_PAIR_RESIDENT: *value = h->pair_res[chunk_index(h->opt_chunk)][h->opt_ctas]; break;
        case SDM_OPT_STAGE_CHUNK: *value = h->opt_chunk; break;
        case SDM_OPT_ZERO_COPY: *value = h->opt_zero_copy; break;
        case SDM_OPT_OVERLAP: *value = h->opt_overlap; break;
        case SDM_OPT_LIST_GROUP: *value = h->opt_list_group; break;
        default: return SDM_ERR_INVALID_ARGUMENT;
    }
    return SDM_OK;
}

sdm_status sdm_get_kernel_times(const sdm_handle* hc, const char** names, float* ms, int* count) {
    if (!hc || !count) return SDM_ERR_INVALID_ARGUMENT;
    sdm_handle* h = const_cast<sdm_handle*>(hc);
    if (h->last_nk < 0) {
        cudaSetDevice(h->device);
        SDM_CUDA(h, cudaEventSynchronize(h->ev[kNumTimed]));
        for (int k = 0; k < kNumTimed; ++k)
            SDM_CUDA(h, cudaEventElapsedTime(&h->last_ms[k], h->ev[k], h->ev[k + 1]));
        h->last_nk = kNumTimed;
    }
    const int n = std::min(*count, h->last_nk);
    for (int k = 0; k < n; ++k) {
        if (names) names[k] = kKernelNames[k];
        if (ms) ms[k] = h->last_ms[k];
    }
    *count = n;
    return SDM_OK;
}

// ---------------------------------------------------------------------------
// autotuner: main-pass implementation x CTAs per SM x split, each timed on
// the production path (the captured graph of a whole evaluation), the choice
// kept in a text cache keyed by the workload
// ---------------------------------------------------------------------------
namespace {

// workload key: mean particles per replica, mean density, cutoff, replicas,
// systems, electrostatics and the SM count of the device
std::string tune_key_of(long long particles, int replicas, double volume_weighted, double rc, int systems, bool pme,
                        int sms) {
    const double rho = volume_weighted > 0.0 ? (double)particles / volume_weighted : 0.0;
    char buf[256];
    snprintf(buf, sizeof buf, "sdm-tune-v1 n=%lld rho=%.1f rc=%.3f replicas=%d systems=%d method=%s sms=%d",
             replicas > 0 ? (particles + replicas / 2) / replicas : 0LL, rho, rc, replicas, systems,
             pme ? "pme" : "rf", sms);
    return buf;
}

bool tune_cache_read(const char* path, const std::string& key, sdm_tune_result* r) {
    if (!path) return false;
    FILE* f = fopen(path, "r");
    if (!f) return false;
    char line[512];
    bool found = false;
    while (fgets(line, sizeof line, f)) {
        const char* bar = strchr(line, '|');
        if (!bar || std::string(line, bar - line) != key) continue;
        sdm_tune_result t = {};
        t.list_group = SDM_JG;
        t.overlap = 2;
        // chunk, CTAs, split, ms [, list group, overlap]: lines without the last
        // two (an older cache) take the defaults
        if (sscanf(bar + 1, "%d %d %d %f %d %d", &t.stage_chunk, &t.ctas_per_sm, &t.split, &t.ms, &t.list_group,
                   &t.overlap) >= 4) {
            *r = t;
            found = true;   // the last line of a key wins
        }
    }
    fclose(f);
    return found;
}

bool tune_cache_write(const char* path, const std::string& key, const sdm_tune_result& r) {
    if (!path) return true;
    std::vector<std::string> keep;
    if (FILE* f = fopen(path, "r")) {
        char line[512];
        while (fgets(line, sizeof line, f)) {
            const char* bar = strchr(line, '|');
            if (bar && std::string(line, bar - line) == key) continue;
            keep.emplace_back(line);
        }
        fclose(f);
    }
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "w");
    if (!f) return false;
    for (const std::string& l : keep) fputs(l.c_str(), f);
    fprintf(f, "%s|%d %d %d %.6f %d %d\n", key.c_str(), r.stage_chunk, r.ctas_per_sm, r.split, r.ms, r.list_group,
            r.overlap);
    const bool ok = fclose(f) == 0;
    return ok && rename(tmp.c_str(), path) == 0;
}

std::string tune_key_handle(const sdm_handle* h) {
    long long particles = 0;
    double vol = 0.0, rc = 0.0;
    for (const SysHost& s : h->sys) {
        particles += (long long)s.n * s.replicas;
        vol += s.dev.box[0] * s.dev.box[1] * s.dev.box[2] * s.replicas;
        rc = std::max(rc, s.dev.rc);
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    return tune_key_of(particles, h->nrep, vol, rc, (int)h->sys.size(), h->pme, sms);
}

}  // namespace

sdm_status sdm_tune_key(const sdm_system_desc* systems, int num_systems, int num_sms, char* key, int capacity) {
    if (!systems || num_systems < 1 || !key || capacity < 1) return SDM_ERR_INVALID_ARGUMENT;
    long long particles = 0;
    int replicas = 0;
    double vol = 0.0, rc = 0.0;
    bool pme = false;
    for (int k = 0; k < num_systems; ++k) {
        const sdm_system_desc& d = systems[k];
        particles += (long long)d.num_particles * d.num_replicas;
        replicas += d.num_replicas;
        vol += d.box[0] * d.box[1] * d.box[2] * d.num_replicas;
        rc = std::max(rc, d.cutoff);
        pme = pme || d.nonbonded_method == SDM_NB_PME;
    }
    const std::string s = tune_key_of(particles, replicas, vol, rc, num_systems, pme, num_sms);
    if ((int)s.size() + 1 > capacity) return SDM_ERR_CAPACITY;
    memcpy(key, s.c_str(), s.size() + 1);
    return SDM_OK;
}

sdm_status sdm_autotune_cached(sdm_handle* h, const double* x_device, const char* cache_path,
                               sdm_tune_result* out) {
    if (!h || !x_device) return SDM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    const std::string key = tune_key_handle(h);
    sdm_tune_result best = {};
    if (tune_cache_read(cache_path, key, &best) &&
        (best.stage_chunk == 8 || best.stage_chunk == 12 || best.stage_chunk == 16) &&
        best.ctas_per_sm >= 1 && best.ctas_per_sm <= SDM_MAX_CTAS &&
        (best.split == 1 || best.split == 2 || best.split == 4) &&
        (best.list_group == 1 || best.list_group == 2 || best.list_group == SDM_JG) &&
        best.overlap >= 0 && best.overlap <= 2 &&
        h->pair_res[chunk_index(best.stage_chunk)][best.ctas_per_sm] > 0) {
        h->opt_chunk = best.stage_chunk;
        h->opt_ctas = best.ctas_per_sm;
        h->opt_split = best.split;
        h->opt_list_group = best.list_group;
        h->opt_overlap = best.overlap;
        best.from_cache = 1;
        if (out) *out = best;
        return SDM_OK;
    }
    const int ochunk = h->opt_chunk, octas = h->opt_ctas, osplit = h->opt_split, oprof = h->opt_profile;
    const int ogroup = h->opt_list_group, oover = h->opt_overlap;
    auto restore = [&]() {
        h->opt_chunk = ochunk; h->opt_ctas = octas; h->opt_split = osplit; h->opt_profile = oprof;
        h->opt_list_group = ogroup; h->opt_overlap = oover;
    };
    h->opt_profile = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        restore();
        return fail(h, SDM_ERR_CUDA, "cudaEventCreate");
    }
    best.ms = 1e30f;
    sdm_status st = SDM_OK;
    // median of 5 timed graph replays (after 2 untimed) of the current setting
    auto time_setting = [&](float* med) -> sdm_status {
        std::vector<float> ms;
        for (int rep = 0; rep < 7; ++rep) {
            if (rep >= 2) cudaEventRecord(e0, h->stream);
            sdm_status s2 = run(h, x_device, h->res_in, h->f_in, h->stream, 0, true);
            if (s2) return s2;
            if (rep >= 2) {
                cudaEventRecord(e1, h->stream);
                cudaEventSynchronize(e1);
                float t = 0.f;
                cudaEventElapsedTime(&t, e0, e1);
                ms.push_back(t);
            }
        }
        std::sort(ms.begin(), ms.end());
        *med = ms[ms.size() / 2];
        return SDM_OK;
    };
    // pass 1: staging chunk x CTAs per SM x split, with the handle's list
    // group and branch settings
    const int group0 = h->opt_list_group ? h->opt_list_group : h->auto_list_group;
    for (int ch : {8, 12, 16})
        for (int c = 3; c <= SDM_MAX_CTAS && st == SDM_OK; ++c)
            for (int sp : {1, 2}) {
                if (st != SDM_OK || h->pair_res[chunk_index(ch)][c] < 1) continue;
                h->opt_chunk = ch;
                h->opt_ctas = c;
                h->opt_split = sp;
                float med = 0.f;
                st = time_setting(&med);
                if (st) break;
                if (med < best.ms) best = sdm_tune_result{ch, c, sp, med, 0, group0, h->opt_overlap};
            }
    // pass 2: on that schedule, the list-building group, then the second branch
    if (st == SDM_OK) {
        h->opt_chunk = best.stage_chunk;
        h->opt_ctas = best.ctas_per_sm;
        h->opt_split = best.split;
        for (int g : {1, 2, SDM_JG}) {
            if (g == best.list_group) continue;
            h->opt_list_group = g;
            h->opt_overlap = best.overlap;
            float med = 0.f;
            st = time_setting(&med);
            if (st) break;
            if (med < best.ms) { best.ms = med; best.list_group = g; }
        }
        for (int ov : {0, 1, 2}) {
            if (st != SDM_OK || ov == best.overlap) continue;
            h->opt_list_group = best.list_group;
            h->opt_overlap = ov;
            float med = 0.f;
            st = time_setting(&med);
            if (st) break;
            if (med < best.ms) { best.ms = med; best.overlap = ov; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) { restore(); return st; }
    // the timed calls ran on the caller's coordinates: their lists may have
    // overflowed, which the status word reports (and the next call regrows)
    int v = 0;
    st = check_dev_status(h, &v, false);
    if (st) { restore(); return st; }
    if (v & SDM_DEV_LIST_OVERFLOW) {
        restore();
        return fail(h, SDM_ERR_CAPACITY, "lists overflowed while tuning: evaluate once, then tune again");
    }
    h->opt_chunk = best.stage_chunk;
    h->opt_ctas = best.ctas_per_sm;
    h->opt_split = best.split;
    h->opt_list_group = best.list_group;
    h->opt_overlap = best.overlap;
    h->opt_profile = oprof;
    if (!tune_cache_write(cache_path, key, best)) return fail(h, SDM_ERR_INVALID_ARGUMENT, "cannot write the tuning cache");
    if (out) *out = best;
    return SDM_OK;
}

sdm_status sdm_autotune(sdm_handle* h, const double* x_device, int* split, int* ctas_per_sm) {
    sdm_tune_result r = {};
    sdm_status s = sdm_autotune_cached(h, x_device, nullptr, &r);
    if (s) return s;
    if (split) *split = r.split;
    if (ctas_per_sm) *ctas_per_sm = r.ctas_per_sm;
    return SDM_OK;
}

sdm_status sdm_count_pairs(sdm_handle* h, const double* x, long long* counts) {
    if (!h || !x || !counts) return SDM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    const size_t nx = 3 * (size_t)h->total_particles;
    SDM_CUDA(h, cudaMemcpyAsync(h->x_in, x, nx * 8, cudaMemcpyHostToDevice, h->stream));
    SDM_CUDA(h, cudaMemsetAsync(h->args.counts, 0, sizeof(long long) * 2 * h->nrep, h->stream));
    sdm_status s = run(h, h->x_in, h->res_in, h->f_in, h->stream, 1, false);
    if (s) return s;
    SDM_CUDA(h, cudaMemcpyAsync(counts, h->args.counts, sizeof(long long) * 2 * h->nrep,
                                cudaMemcpyDeviceToHost, h->stream));
    SDM_CUDA(h, cudaStreamSynchronize(h->stream));
    return SDM_OK;
}

sdm_status sdm_get_grid(const sdm_handle* h, int system, int* M) {
    if (!h || !M || system < 0 || system >= (int)h->sys.size()) return SDM_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 3; ++k) M[k] = h->sys[system].dev.M[k];
    return SDM_OK;
}

sdm_status sdm_export_lists(sdm_handle* h, int replica, const double* x, int cap_slots, int cap_clusters,
                            int cap_per_cluster, int* perm, int* ncl, int* cnt, int* ent_slot,
                            unsigned char* ent_mask) {
    if (!h || !x || !perm || !ncl || !cnt || !ent_slot || !ent_mask) return SDM_ERR_INVALID_ARGUMENT;
    if (replica < 0 || replica >= h->nrep) return fail(h, SDM_ERR_INVALID_ARGUMENT, "replica index out of range");
    if (cap_per_cluster < 1) return fail(h, SDM_ERR_INVALID_ARGUMENT, "cap_per_cluster must be >= 1");
    cudaSetDevice(h->device);
    const SdmRep& R = h->rep[replica];
    const int n = R.n;
    SDM_CUDA(h, cudaMemcpyAsync(h->x_in + 3 * R.x_off, x, 3 * (size_t)n * 8, cudaMemcpyHostToDevice, h->stream));
    const int capcl = R.slot_cap / 8;
    void* dbuf = nullptr;
    const size_t nent = (size_t)capcl * cap_per_cluster;
    SDM_CUDA(h, cudaMalloc(&dbuf, nent * 5 + (size_t)capcl * 4 + 64));
    int* d_cnt = (int*)dbuf;
    int* d_slot = d_cnt + capcl;
    unsigned char* d_mask = (unsigned char*)(d_slot + nent);
    SdmArgs save = h->args;
    h->args.ex_cnt = d_cnt;
    h->args.ex_slot = d_slot;
    h->args.ex_mask = d_mask;
    h->args.ex_cap = cap_per_cluster;
    h->args.ex_rep = replica;
    sdm_status s = run(h, h->x_in, h->res_in, h->f_in, h->stream, 2, false);
    h->args = save;
    if (s) { cudaFree(dbuf); return s; }
    int k = 0, st = 0;
    cudaMemcpyAsync(&k, h->args.ncl + replica, 4, cudaMemcpyDeviceToHost, h->stream);
    cudaStreamSynchronize(h->stream);
    check_dev_status(h, &st, true);
    if (8 * k > cap_slots || k > cap_clusters || (st & (1 << 16))) {
        cudaFree(dbuf);
        return fail(h, SDM_ERR_CAPACITY, "export capacity too small");
    }
    *ncl = k;
    cudaError_t ce = cudaMemcpy(perm, h->args.perm + R.slot_win, 8 * (size_t)k * 4, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(cnt, d_cnt, (size_t)k * 4, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(ent_slot, d_slot, (size_t)k * cap_per_cluster * 4, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(ent_mask, d_mask, (size_t)k * cap_per_cluster, cudaMemcpyDeviceToHost);
    cudaFree(dbuf);
    if (ce != cudaSuccess) return cuda_fail(h, ce, "export copy");
    return SDM_OK;
}

}  // extern "C"
