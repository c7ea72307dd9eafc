// sdm_pme.cu -- smooth particle-mesh Ewald reciprocal space for both SDM
// states (sm_103a).
//
// Smooth PME (Essmann et al., J. Chem. Phys. 103, 8577 (1995)), B-spline
// order 5, orthorhombic boxes; the reference's explicit-solvent setup uses
// OpenMM NonbondedForce.PME (example/test_explicit.py:64).  Per replica:
//   Q      charges of state 0 spread on the grid (fixed point: order-independent)
//   dQ     state 1 minus state 0: +q at y = x + d and -q at x for every
//          displaced particle (the other charges do not move)
//   phi1 = theta * Q, phiD = theta * dQ   (theta: Ewald kernel x B-spline
//          moduli, one R2C / C2R cuFFT pair per grid)
//   E_rec(state 0)       = 1/2 sum_k theta(k) |Q(k)|^2
//   E_rec(1) - E_rec(0)  = sum_{i in D} q_i [phi1(y_i) - phi1(x_i)] + 1/2 q_i [phiD(y_i) - phiD(x_i)]
//   F0_i = -q_i grad phi1(x_i);  F1_i = -q_i grad (phi1 + phiD)(pos1_i)
// (the grid energy is quadratic in the spread charges, so these identities
// are exact on the grid).  Forces enter the same fixed-point F0 / dF slot
// accumulators as the pair kernels.
#include <cuda_runtime.h>
#include <cufft.h>

#include "../../include/sdm_capi.h"
#include "sdm_types.h"

namespace {

constexpr int kOrder = 5;
constexpr double kGridFix = 1099511627776.0;   // 2^40: fixed-point scale of the spread grids


// round(v * 2^32) via two 32-bit conversions (|v| < 2^30)
__device__ __forceinline__ unsigned long long pme_fix64(float v) {
    const float a = rintf(v);
    const int hi = __float2int_rn(a);
    const int lo = __float2int_rn(__fmul_rn(__fsub_rn(v, a), 4294967296.0f));
    return (unsigned long long)(((long long)hi << 32) + (long long)lo);
}

// round(v * 2^40): the grid scale (|v| < 2^22), FP32 and 32-bit conversions only
__device__ __forceinline__ unsigned long long grid_fix(float v) { return pme_fix64(v * 256.0f); }

__device__ __forceinline__ void pme_red(unsigned long long* p, float v, int* status) {
    if (!(fabsf(v) < 1.0e9f)) {
        atomicOr(status, SDM_DEV_FORCE_OVERFLOW);
        return;
    }
    atomicAdd(p, pme_fix64(v));
}

// B-spline weights M_5(w + j) and derivatives, j = 0..4; element j belongs to
// grid point floor(u) - j
__device__ __forceinline__ void bspline5(float w, float M[kOrder], float dM[kOrder]) {
    float P[kOrder];
    P[0] = w;
    P[1] = 1.0f - w;
#pragma unroll
    for (int k = 3; k <= kOrder; ++k) {
        if (k == kOrder) {
#pragma unroll
            for (int j = 0; j < kOrder; ++j)
                dM[j] = (j < k - 1 ? P[j] : 0.0f) - (j > 0 ? P[j - 1] : 0.0f);
        }
        float N[kOrder];
        const float inv = 1.0f / (float)(k - 1);
#pragma unroll
        for (int j = 0; j < kOrder; ++j) {
            if (j >= k) { N[j] = 0.0f; continue; }
            const float xj = w + (float)j;
            const float cur = j < k - 1 ? P[j] : 0.0f;
            const float prv = j > 0 ? P[j - 1] : 0.0f;
            N[j] = (xj * cur + ((float)k - xj) * prv) * inv;
        }
#pragma unroll
        for (int j = 0; j < kOrder; ++j) P[j] = N[j];
    }
#pragma unroll
    for (int j = 0; j < kOrder; ++j) M[j] = P[j];
}

// element j of a 5-element register array, j warp-divergent (select chain,
// no local memory)
__device__ __forceinline__ float pick5(const float v[kOrder], int j) {
    float r = v[0];
#pragma unroll
    for (int k = 1; k < kOrder; ++k) r = (j == k) ? v[k] : r;
    return r;
}

// v 2^40 (the grid's fixed point) as hi 2^20 + lo: hi = floor(v 2^20), lo =
// round(frac 2^20) in [0, 2^20].  Exact: v 2^20, its floor and its fraction
// are exact in FP32, and hi 2^20 + lo = round(v 2^40) (|v| < 2^11)
__device__ __forceinline__ void grid_split(float v, int& hi, int& lo) {
    const float s = v * 1048576.0f;
    const float f = floorf(s);
    hi = (int)f;
    lo = __float2int_rn((s - f) * 1048576.0f);
}

// scaled coordinate u = v K / L in FP32 (v already wrapped into [0, L): u in
// [0, K]; placement error ~K 2^-24 grid spacings)
struct Stencil {
    int base[3];          // floor(u) mod K
    int ub[3];            // floor(u) in [0, K]: contiguous over the box (brick sub-grids)
    float M[3][kOrder], dM[3][kOrder];
};

// floor(u) clamped to [0, K]: a non-finite coordinate gives non-finite
// weights at grid point 0 (the energies report it), never an index outside
// the grid
__device__ __forceinline__ int grid_floor(float u, int K) { return min(max((int)floorf(u), 0), K); }

__device__ __forceinline__ float grid_u(const SdmSys& S, const double p[3], int k) {
    return __fmul_rn(__double2float_rn(p[k]), S.pme_gs[k]);
}

__device__ __forceinline__ void make_stencil(const SdmSys& S, const double p[3], Stencil& st) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int K = S.pme_grid[k];
        const float u = grid_u(S, p, k);
        const int fl = grid_floor(u, K);
        const float w = u - (float)fl;
        st.ub[k] = fl;
        st.base[k] = fl == K ? 0 : fl;
        bspline5(w, st.M[k], st.dM[k]);
    }
}

__device__ __forceinline__ int wrapk(int i, int K) { return i < 0 ? i + K : (i >= K ? i - K : i); }

__device__ __forceinline__ int wrapg(int i, int K) { return i < 0 ? i + K : i; }

__device__ void spread(unsigned long long* acc, const SdmSys& S, const Stencil& st, float q) {
    const int K0 = S.pme_grid[0], K1 = S.pme_grid[1], K2 = S.pme_grid[2];
#pragma unroll
    for (int a = 0; a < kOrder; ++a) {
        const int i0 = wrapg(st.base[0] - a, K0);
        const float qa = q * st.M[0][a];
#pragma unroll
        for (int b = 0; b < kOrder; ++b) {
            const int i1 = wrapg(st.base[1] - b, K1);
            const float qab = qa * st.M[1][b];
            unsigned long long* row = acc + ((size_t)i0 * K1 + i1) * K2;
#pragma unroll
            for (int c = 0; c < kOrder; ++c) {
                const int i2 = wrapg(st.base[2] - c, K2);
                atomicAdd(row + i2, grid_fix(qab * st.M[2][c]));
            }
        }
    }
}

// potential and its gradient (grid units) interpolated from a potential grid
__device__ void interp(const float* phi, const SdmSys& S, const Stencil& st, float& v, float g[3]) {
    const int K0 = S.pme_grid[0], K1 = S.pme_grid[1], K2 = S.pme_grid[2];
    v = 0.0f;
    g[0] = g[1] = g[2] = 0.0f;
#pragma unroll
    for (int a = 0; a < kOrder; ++a) {
        const int i0 = wrapg(st.base[0] - a, K0);
#pragma unroll
        for (int b = 0; b < kOrder; ++b) {
            const int i1 = wrapg(st.base[1] - b, K1);
            const float* row = phi + ((size_t)i0 * K1 + i1) * K2;
            float s = 0.0f, sd = 0.0f;
#pragma unroll
            for (int c = 0; c < kOrder; ++c) {
                const float p = row[wrapg(st.base[2] - c, K2)];
                s = fmaf(st.M[2][c], p, s);
                sd = fmaf(st.dM[2][c], p, sd);
            }
            v = fmaf(st.M[0][a] * st.M[1][b], s, v);
            g[0] = fmaf(st.dM[0][a] * st.M[1][b], s, g[0]);
            g[1] = fmaf(st.M[0][a] * st.dM[1][b], s, g[1]);
            g[2] = fmaf(st.M[0][a] * st.M[1][b], sd, g[2]);
        }
    }
}

// ---- bricks: spreading and interpolation through shared-memory sub-grids ----
// A brick is bc^3 cells of the cell grid (fewer at the upper faces); its
// particles are the bucket ranges of its cells (contiguous per cell column).
// The sub-grid spans the bricks' stencils: origin lo = min(ub) - 4, extents
// E = max(ub) - lo + 1 per dimension, points indexed ((i0 E1) + i1) E2 + i2.
constexpr int kBrickThreads = 256;
constexpr int kMaxBrickCols = 25;   // bc <= 5
// shared-memory accumulation: a grid contribution (fixed point 2^40) goes
// into two 32-bit sums, its high part (units of 2^kLoBits) and its low part
// in [0, 2^kLoBits] (grid_split)
constexpr int kLoBits = 20;
constexpr int kBrickMaxCharged = 2047;      // low-word sums <= 2047 2^20 < 2^31
constexpr float kBrickMaxValue = 2000.0f;   // high-word sums < 2^31 (values < 2^(51-40))

struct BrickCols {
    int beg[kMaxBrickCols];        // bucket offset of the brick's first cell in each column
    int pre[kMaxBrickCols + 1];    // particle prefix over the columns
    int ncols;
};

// cells of brick b of the replica's system; false past the system's bricks
__device__ __forceinline__ bool brick_cells(const SdmSys& S, int b, int c0[3], int c1[3]) {
    const int nz = S.pme_nb[2], ny = S.pme_nb[1];
    const int bz = b % nz, by = (b / nz) % ny, bx = b / (nz * ny);
    if (bx >= S.pme_nb[0]) return false;
    const int bb[3] = {bx, by, bz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c0[k] = bb[k] * S.pme_bc[k];
        c1[k] = min(c0[k] + S.pme_bc[k], S.M[k]);
    }
    return true;
}

// column ranges and particle prefix of the brick (block-wide; ends synchronised)
__device__ void brick_columns(const SdmArgs& a, const SdmRep& R, const SdmSys& S, const int c0[3], const int c1[3],
                              BrickCols& bc) {
    const int ny = c1[1] - c0[1];
    const int ncols = (c1[0] - c0[0]) * ny;
    const int t = threadIdx.x;
    if (t < ncols) {
        const int col = (c0[0] + t / ny) * S.M[1] + c0[1] + t % ny;
        const int* off = a.cel_off + R.cel_win + col * S.M[2];
        bc.beg[t] = off[c0[2]];
        bc.pre[t + 1] = off[c1[2]] - off[c0[2]];
    }
    __syncthreads();
    if (t == 0) {
        bc.pre[0] = 0;
        for (int c = 0; c < ncols; ++c) bc.pre[c + 1] += bc.pre[c];
        bc.ncols = ncols;
    }
    __syncthreads();
}

// particle index of the brick's it-th particle
__device__ __forceinline__ int brick_atom(const SdmArgs& a, const SdmRep& R, const BrickCols& bc, int it) {
    int c = 0;
    while (bc.pre[c + 1] <= it) ++c;
    return a.bucket[R.atom_win + bc.beg[c] + (it - bc.pre[c])];
}

__device__ __forceinline__ void load_pos(const SdmArgs& a, int gi, double p[3]) {
    p[0] = a.w[3 * (size_t)gi];
    p[1] = a.w[3 * (size_t)gi + 1];
    p[2] = a.w[3 * (size_t)gi + 2];
}

// state-0 charges of every particle of every replica: one block per brick
// (blockIdx.x) of replica blockIdx.y.  Pass 1 finds the sub-grid of the
// brick's stencils, pass 2 spreads into it with shared-memory fixed-point
// atomics, the flush adds each nonzero point into the global grid.  A brick
// whose sub-grid exceeds the shared memory spreads with global atomics.
__global__ void __launch_bounds__(kBrickThreads) k_pme_spread(SdmArgs a) {
    extern __shared__ int sg[];   // sub-grid accumulators: high words [0, npts), low words [npts, 2 npts)
    __shared__ BrickCols bc;
    __shared__ int lo[3], hi[3], nq;
    __shared__ float qabs;
    const int r = blockIdx.y;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    int c0[3], c1[3];
    if (!brick_cells(S, blockIdx.x, c0, c1)) return;   // block-uniform
    const int t = threadIdx.x;
    if (t < 3) { lo[t] = 0x7fffffff; hi[t] = -0x7fffffff; }
    if (t == 0) { nq = 0; qabs = 0.0f; }
    brick_columns(a, R, S, c0, c1, bc);
    const int total = bc.pre[bc.ncols];
    float qsum = 0.0f;
    int cnt = 0;
    for (int it = t; it < total; it += kBrickThreads) {
        const int i = brick_atom(a, R, bc, it);
        const float qi = a.pme_charge[S.atom_base + i];
        if (qi == 0.0f) continue;
        qsum += fabsf(qi);
        ++cnt;
        double p[3];
        load_pos(a, R.atom_win + i, p);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int ub = grid_floor(grid_u(S, p, k), S.pme_grid[k]);   // = make_stencil's ub
            atomicMin(&lo[k], ub - (kOrder - 1));
            atomicMax(&hi[k], ub);
        }
    }
    if (cnt) { atomicAdd(&nq, cnt); atomicAdd(&qabs, qsum); }
    __syncthreads();
    int4* info = a.pme_brick + 2 * ((size_t)r * a.pme_max_bricks + blockIdx.x);
    if (hi[0] < lo[0]) {   // no charged particle in the brick
        if (t == 0) { info[0] = make_int4(0, 0, 0, -1); info[1] = make_int4(0, 0, 0, 0); }
        return;
    }
    const int L0 = lo[0], L1 = lo[1], L2 = lo[2];
    const int E0 = hi[0] - L0 + 1, E1 = hi[1] - L1 + 1, E2 = hi[2] - L2 + 1;
    const int npts = E0 * E1 * E2;
    // the split accumulators are exact while every point's sum of low words
    // stays below 2^31 (at most 2047 contributions) and every point's value
    // below 2^11 (|sum q W| <= max W sum |q|, max W = (115/192)^3 < 0.215)
    const bool fits = npts <= S.pme_cap && nq <= kBrickMaxCharged && 0.215f * qabs < kBrickMaxValue;
    const bool sub = npts <= S.pme_cap;   // the sub-grid of the interpolation fits
    if (t == 0) { info[0] = make_int4(L0, L1, L2, sub ? 1 : 0); info[1] = make_int4(E0, E1, E2, 0); }
    if (fits)
        for (int q = t; q < 2 * npts; q += kBrickThreads) sg[q] = 0;
    __syncthreads();
    unsigned long long* acc = a.pme_acc + R.pg_win;
    for (int it = t; it < total; it += kBrickThreads) {
        const int i = brick_atom(a, R, bc, it);
        const float q = a.pme_charge[S.atom_base + i];
        if (q == 0.0f) continue;
        double p[3];
        load_pos(a, R.atom_win + i, p);
        Stencil st;
        make_stencil(S, p, st);
        if (!fits) {
            spread(acc, S, st, q);
            continue;
        }
#pragma unroll
        for (int x = 0; x < kOrder; ++x) {
            const float qa = q * st.M[0][x];
            const int i0 = st.ub[0] - x - L0;
#pragma unroll
            for (int y = 0; y < kOrder; ++y) {
                const float qab = qa * st.M[1][y];
                int* row = sg + (i0 * E1 + (st.ub[1] - y - L1)) * E2 + (st.ub[2] - L2);
#pragma unroll
                for (int z = 0; z < kOrder; ++z) {
                    int hi, lo;
                    grid_split(qab * st.M[2][z], hi, lo);
                    atomicAdd(row - z, hi);
                    atomicAdd(row - z + npts, lo);
                }
            }
        }
    }
    if (!fits) return;
    __syncthreads();
    const int K0 = S.pme_grid[0], K1 = S.pme_grid[1], K2 = S.pme_grid[2];
#pragma unroll 4
    for (int q = t; q < npts; q += kBrickThreads) {
        const unsigned long long v = (unsigned long long)(((long long)sg[q] << kLoBits) + (long long)sg[npts + q]);
        if (v == 0ull) continue;
        const int i2 = q % E2, i01 = q / E2;
        const int i1 = i01 % E1, i0 = i01 / E1;
        const size_t g = ((size_t)wrapk(L0 + i0, K0) * K1 + wrapk(L1 + i1, K1)) * K2 + wrapk(L2 + i2, K2);
        atomicAdd(acc + g, v);
    }
}

// dQ: +q at y = x + d and -q at x for every displaced particle (one thread per
// (perturbation item = particle and state)): state 1 item spreads +q at y,
// state 0 item spreads -q at x
__global__ void k_pme_spread_delta(SdmArgs a) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= a.total_pert) return;
    int lo = 0, hi = a.nrep - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.rep[mid].pert_win <= item) lo = mid; else hi = mid - 1;
    }
    const SdmRep& R = a.rep[lo];
    const SdmSys& S = a.sys[R.sys];
    const int local = item - R.pert_win;
    const int st1 = local & 1;
    const int p = a.D_idx[S.D_base + (local >> 1)];
    const float q = a.pme_charge[S.atom_base + p];
    if (q == 0.0f) return;
    const SdmPertPos pp = a.pert_pos[item];   // y in state 1, x in state 0 (written by k_pert_prep)
    Stencil st;
    make_stencil(S, pp.y, st);
    spread(a.pme_acc + R.pg_win + R.pg_size, S, st, st1 ? q : -q);
}

// fixed point -> float grids (both grids of every replica).  Read only: the
// accumulators are cleared by a memset before spreading (a store of zeros
// right after the load of the same lines ran at a tenth of the bandwidth)
__global__ void k_pme_to_float(SdmArgs a) {
    const long long n = a.pme_total_grid;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long v = (long long)a.pme_acc[k];
        // hi 2^32 + lo: FP32 and 32-bit conversions only (hi exact, lo below the grid's resolution)
        const float hi = (float)(int)(v >> 32), lo = (float)(unsigned)(v & 0xffffffffll);
        a.pme_grid[k] = __fmaf_rn(hi, 1.0f / 256.0f, lo * (float)(1.0 / kGridFix));
    }
}

// spectra *= theta; state-0 energy 1/2 sum theta |Q|^2 (half spectrum weighted)
// in fixed per-replica blocks
__global__ void __launch_bounds__(256) k_pme_convolve(SdmArgs a) {
    __shared__ double red[256];
    const int r = blockIdx.y;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int K2h = S.pme_grid[2] / 2 + 1;
    const long long ns = (long long)S.pme_grid[0] * S.pme_grid[1] * K2h;
    const float* theta = a.pme_theta + S.pme_base;
    float2* spec = a.pme_spec + R.ps_win;
    double e = 0.0;
    const int nsi = (int)ns;   // < 2^31 (K <= 1024)
    int m2 = blockIdx.x * blockDim.x + threadIdx.x;
    const int step = gridDim.x * blockDim.x, step2 = step % K2h;
    m2 %= K2h;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nsi; k += step) {
        const float t = theta[k];
        const float2 z = spec[k];
        const float wgt = (m2 == 0 || (2 * m2 == S.pme_grid[2])) ? 0.5f : 1.0f;
        e += (double)(wgt * t * __fmaf_rn(z.x, z.x, z.y * z.y));
        m2 += step2;
        if (m2 >= K2h) m2 -= K2h;
        spec[k] = make_float2(z.x * t, z.y * t);
        const float2 zd = spec[ns + k];
        spec[ns + k] = make_float2(zd.x * t, zd.y * t);
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.pme_epart[(size_t)r * gridDim.x + blockIdx.x] = red[0];
}

// potentials (phi1, phiD) and their gradients (grid units) from a brick's
// shared-memory sub-grid
__device__ __forceinline__ void interp_local(const float2* sp, int L0, int L1, int L2, int E1, int E2,
                                             const Stencil& st, float v[2], float g[2][3]) {
    v[0] = v[1] = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) g[0][k] = g[1][k] = 0.0f;
#pragma unroll
    for (int x = 0; x < kOrder; ++x) {
        const int i0 = st.ub[0] - x - L0;
#pragma unroll
        for (int y = 0; y < kOrder; ++y) {
            const float2* row = sp + ((size_t)i0 * E1 + (st.ub[1] - y - L1)) * E2 + (st.ub[2] - L2);
            float s1 = 0.0f, sd1 = 0.0f, sD = 0.0f, sdD = 0.0f;
#pragma unroll
            for (int z = 0; z < kOrder; ++z) {
                const float2 pp = row[-z];
                s1 = fmaf(st.M[2][z], pp.x, s1);
                sd1 = fmaf(st.dM[2][z], pp.x, sd1);
                sD = fmaf(st.M[2][z], pp.y, sD);
                sdD = fmaf(st.dM[2][z], pp.y, sdD);
            }
            const float mm = st.M[0][x] * st.M[1][y];
            const float dm0 = st.dM[0][x] * st.M[1][y], dm1 = st.M[0][x] * st.dM[1][y];
            v[0] = fmaf(mm, s1, v[0]);
            g[0][0] = fmaf(dm0, s1, g[0][0]);
            g[0][1] = fmaf(dm1, s1, g[0][1]);
            g[0][2] = fmaf(mm, sd1, g[0][2]);
            v[1] = fmaf(mm, sD, v[1]);
            g[1][0] = fmaf(dm0, sD, g[1][0]);
            g[1][1] = fmaf(dm1, sD, g[1][1]);
            g[1][2] = fmaf(mm, sdD, g[1][2]);
        }
    }
}

// state-0 forces of every particle and the state-1 change of the forces on
// the particles that stay; one block per brick, the potentials of the brick's
// sub-grid (as recorded by k_pme_spread) staged in shared memory
__global__ void __launch_bounds__(kBrickThreads, 3) k_pme_gather(SdmArgs a) {
    extern __shared__ float2 sp[];
    __shared__ BrickCols bc;
    const int r = blockIdx.y;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    int c0[3], c1[3];
    if (!brick_cells(S, blockIdx.x, c0, c1)) return;   // block-uniform
    const int4* info = a.pme_brick + 2 * ((size_t)r * a.pme_max_bricks + blockIdx.x);
    const int4 o = info[0], e = info[1];
    if (o.w < 0) return;   // no charged particle
    const bool fits = o.w == 1;
    const int t = threadIdx.x;
    const float* phi1 = a.pme_grid + R.pg_win;
    const float* phiD = phi1 + R.pg_size;
    const int K0 = S.pme_grid[0], K1 = S.pme_grid[1], K2 = S.pme_grid[2];
    brick_columns(a, R, S, c0, c1, bc);
    if (fits) {
        const int npts = e.x * e.y * e.z;
#pragma unroll 4
        for (int q = t; q < npts; q += kBrickThreads) {
            const int i2 = q % e.z, i01 = q / e.z;
            const int i1 = i01 % e.y, i0 = i01 / e.y;
            const size_t g = ((size_t)wrapk(o.x + i0, K0) * K1 + wrapk(o.y + i1, K1)) * K2 + wrapk(o.z + i2, K2);
            sp[q] = make_float2(phi1[g], phiD[g]);
        }
        __syncthreads();
    }
    const float sc[3] = {(float)K0 * S.invLf[0], (float)K1 * S.invLf[1], (float)K2 * S.invLf[2]};
    const int total = bc.pre[bc.ncols];
    unsigned long long* F0[3] = {a.F0x, a.F0y, a.F0z};
    unsigned long long* dF[3] = {a.dFx, a.dFy, a.dFz};
    for (int it = t; it < total; it += kBrickThreads) {
        const int i = brick_atom(a, R, bc, it);
        const float q = a.pme_charge[S.atom_base + i];
        if (q == 0.0f) continue;
        const int gi = R.atom_win + i;
        double p[3];
        load_pos(a, gi, p);
        Stencil sx;
        make_stencil(S, p, sx);
        float v[2], g[2][3];
        if (fits) {
            interp_local(sp, o.x, o.y, o.z, e.y, e.z, sx, v, g);
        } else {
            interp(phi1, S, sx, v[0], g[0]);
            interp(phiD, S, sx, v[1], g[1]);
        }
        const size_t gsl = (size_t)R.slot_win + a.inv[gi];
#pragma unroll
        for (int k = 0; k < 3; ++k) pme_red(F0[k] + gsl, -q * sc[k] * g[0][k], a.status);
        if (a.topo_grp[S.atom_base + i] == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) pme_red(dF[k] + gsl, -q * sc[k] * g[1][k], a.status);
        }
    }
}

// one stencil row (a, b) of the interpolation: value and gradient parts of
// both potential grids at stencil st
__device__ __forceinline__ void interp_row(const float* phi1, const float* phiD, const SdmSys& S, const Stencil& st,
                                           int a, int b, float o1[4], float oD[4]) {
    const int K0 = S.pme_grid[0], K1 = S.pme_grid[1], K2 = S.pme_grid[2];
    const int i0 = wrapg(st.base[0] - a, K0), i1 = wrapg(st.base[1] - b, K1);
    const size_t row = ((size_t)i0 * K1 + i1) * K2;
    float s1 = 0.0f, sd1 = 0.0f, sD = 0.0f, sdD = 0.0f;
#pragma unroll
    for (int c = 0; c < kOrder; ++c) {
        const int i2 = wrapg(st.base[2] - c, K2);
        const float p1 = phi1[row + i2], pD = phiD[row + i2];
        s1 = fmaf(st.M[2][c], p1, s1);
        sd1 = fmaf(st.dM[2][c], p1, sd1);
        sD = fmaf(st.M[2][c], pD, sD);
        sdD = fmaf(st.dM[2][c], pD, sdD);
    }
    const float mx = pick5(st.M[0], a), dmx = pick5(st.dM[0], a);
    const float my = pick5(st.M[1], b), dmy = pick5(st.dM[1], b);
    o1[0] = mx * my * s1;  o1[1] = dmx * my * s1;  o1[2] = mx * dmy * s1;  o1[3] = mx * my * sd1;
    oD[0] = mx * my * sD;  oD[1] = dmx * my * sD;  oD[2] = mx * dmy * sD;  oD[3] = mx * my * sdD;
}

// displaced particles: forces at y in state 1 and the reciprocal part of u;
// one warp per displaced particle, lane l < 25 takes stencil row (l / 5, l % 5)
// of both grids at x and at y, then a fixed-order warp reduction
__global__ void __launch_bounds__(128) k_pme_gather_displaced(SdmArgs a) {
    const int item = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= a.total_pert / 2) return;   // warp-uniform
    const int pi = 2 * item;
    int lo = 0, hi = a.nrep - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.rep[mid].pert_win <= pi) lo = mid; else hi = mid - 1;
    }
    const SdmRep& R = a.rep[lo];
    const SdmSys& S = a.sys[R.sys];
    const int local = pi - R.pert_win;
    const int p = a.D_idx[S.D_base + (local >> 1)];
    const float q = a.pme_charge[S.atom_base + p];
    if (q == 0.0f) {   // warp-uniform
        if (lane == 0) a.pme_du[item] = 0.0;
        return;
    }
    const float* phi1 = a.pme_grid + R.pg_win;
    const float* phiD = phi1 + R.pg_size;
    float t[16];   // [0..3] phi1 at x, [4..7] phiD at x, [8..11] phi1 at y, [12..15] phiD at y
#pragma unroll
    for (int k = 0; k < 16; ++k) t[k] = 0.0f;
    if (lane < kOrder * kOrder) {
        Stencil sx, sy;
        make_stencil(S, a.pert_pos[pi].y, sx);        // state 0: x
        make_stencil(S, a.pert_pos[pi + 1].y, sy);    // state 1: y = x + d
        interp_row(phi1, phiD, S, sx, lane / kOrder, lane % kOrder, t, t + 4);
        interp_row(phi1, phiD, S, sy, lane / kOrder, lane % kOrder, t + 8, t + 12);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t[k] += __shfl_xor_sync(0xffffffffu, t[k], o);
    if (lane != 0) return;
    const double du = (double)q * ((double)t[8] - (double)t[0]) + 0.5 * (double)q * ((double)t[12] - (double)t[4]);
    const float sc[3] = {(float)S.pme_grid[0] * S.invLf[0], (float)S.pme_grid[1] * S.invLf[1],
                         (float)S.pme_grid[2] * S.invLf[2]};
    const size_t gsl = (size_t)R.slot_win + a.inv[R.atom_win + p];
    unsigned long long* dF[3] = {a.dFx, a.dFy, a.dFz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float f1 = -q * sc[k] * (t[9 + k] + t[13 + k]);
        const float f0 = -q * sc[k] * t[1 + k];
        pme_red(dF[k] + gsl, f1 - f0, a.status);
    }
    a.pme_du[item] = du;
}

}  // namespace

// Launch sequence of the reciprocal part (every replica of every system);
// plans[s] are the R2C / C2R plans of system s (batch: 2 grids per replica).
cudaError_t sdm_launch_pme(const SdmArgs& a, const cufftHandle* r2c, const cufftHandle* c2r, const long long* grid_off,
                           const long long* spec_off, int nsys, int conv_blocks, cudaStream_t st) {
    const int ns = 152 * 16;
    const dim3 bricks(a.pme_max_bricks, a.nrep);
    cudaError_t e0 = cudaMemsetAsync(a.pme_acc, 0, (size_t)a.pme_total_grid * sizeof(unsigned long long), st);
    if (e0 != cudaSuccess) return e0;
    k_pme_spread<<<bricks, kBrickThreads, a.pme_smem, st>>>(a);
    if (a.total_pert) k_pme_spread_delta<<<(a.total_pert + 127) / 128, 128, 0, st>>>(a);
    k_pme_to_float<<<ns, 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    for (int s = 0; s < nsys; ++s) {
        if (cufftSetStream(r2c[s], st) != CUFFT_SUCCESS) return cudaErrorUnknown;
        if (cufftExecR2C(r2c[s], a.pme_grid + grid_off[s], reinterpret_cast<cufftComplex*>(a.pme_spec + spec_off[s])) !=
            CUFFT_SUCCESS)
            return cudaErrorUnknown;
    }
    k_pme_convolve<<<dim3(conv_blocks, a.nrep), 256, 0, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    for (int s = 0; s < nsys; ++s) {
        if (cufftSetStream(c2r[s], st) != CUFFT_SUCCESS) return cudaErrorUnknown;
        if (cufftExecC2R(c2r[s], reinterpret_cast<cufftComplex*>(a.pme_spec + spec_off[s]), a.pme_grid + grid_off[s]) !=
            CUFFT_SUCCESS)
            return cudaErrorUnknown;
    }
    k_pme_gather<<<bricks, kBrickThreads, a.pme_smem, st>>>(a);
    if (a.total_pert) k_pme_gather_displaced<<<(a.total_pert / 2 + 3) / 4, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sdm_pme_prepare(int smem_bytes) {
    cudaError_t e = cudaFuncSetAttribute(k_pme_spread, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_pme_gather, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
}
