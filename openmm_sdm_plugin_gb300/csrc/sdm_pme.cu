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

__device__ __forceinline__ int pme_rep_by_atom(const SdmRep* rep, int nrep, int gi) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (rep[mid].atom_win <= gi) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// round(v * 2^32) via two 32-bit conversions (|v| < 2^30)
__device__ __forceinline__ unsigned long long pme_fix64(float v) {
    const float a = rintf(v);
    const int hi = __float2int_rn(a);
    const int lo = __float2int_rn(__fmul_rn(__fsub_rn(v, a), 4294967296.0f));
    return (unsigned long long)(((long long)hi << 32) + (long long)lo);
}

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

// scaled fractional coordinate u = K frac(v / L) (v already wrapped into [0, L))
struct Stencil {
    int base[3];          // floor(u)
    float M[3][kOrder], dM[3][kOrder];
};

__device__ __forceinline__ void make_stencil(const SdmSys& S, const double p[3], Stencil& st) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double f = p[k] * S.invL[k];
        f -= floor(f);
        const float u = (float)(f * (double)S.pme_grid[k]);
        int fl = (int)floorf(u);
        float w = u - (float)fl;
        if (fl >= S.pme_grid[k]) { fl -= S.pme_grid[k]; }
        st.base[k] = fl;
        bspline5(w, st.M[k], st.dM[k]);
    }
}

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
                atomicAdd(row + i2, (unsigned long long)__double2ll_rn((double)(qab * st.M[2][c]) * kGridFix));
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

// state-0 charges of every particle of every replica
__global__ void k_pme_spread(SdmArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < a.total_atoms; gi += stride) {
        const int r = pme_rep_by_atom(a.rep, a.nrep, gi);
        const SdmRep& R = a.rep[r];
        const SdmSys& S = a.sys[R.sys];
        const int i = gi - R.atom_win;
        const float q = a.pme_charge[S.atom_base + i];
        if (q == 0.0f) continue;
        const double p[3] = {a.w[3 * (size_t)gi], a.w[3 * (size_t)gi + 1], a.w[3 * (size_t)gi + 2]};
        Stencil st;
        make_stencil(S, p, st);
        spread(a.pme_acc + R.pg_win, S, st, q);
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

// fixed point -> float grids (both grids of every replica); clears the accumulators
__global__ void k_pme_to_float(SdmArgs a) {
    const long long n = a.pme_total_grid;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long v = (long long)a.pme_acc[k];
        a.pme_acc[k] = 0ull;
        a.pme_grid[k] = (float)((double)v * (1.0 / kGridFix));
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
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += (long long)gridDim.x * blockDim.x) {
        const float t = theta[k];
        const float2 z = spec[k];
        const int m2 = (int)(k % K2h);
        const double wgt = (m2 == 0 || (2 * m2 == S.pme_grid[2])) ? 0.5 : 1.0;
        e += wgt * (double)t * ((double)z.x * z.x + (double)z.y * z.y);
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

// forces of both states and the reciprocal part of u
__global__ void k_pme_gather(SdmArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < a.total_atoms; gi += stride) {
        const int r = pme_rep_by_atom(a.rep, a.nrep, gi);
        const SdmRep& R = a.rep[r];
        const SdmSys& S = a.sys[R.sys];
        const int i = gi - R.atom_win;
        const float q = a.pme_charge[S.atom_base + i];
        if (q == 0.0f) continue;
        const float* phi1 = a.pme_grid + R.pg_win;
        const float* phiD = phi1 + R.pg_size;
        const double p[3] = {a.w[3 * (size_t)gi], a.w[3 * (size_t)gi + 1], a.w[3 * (size_t)gi + 2]};
        Stencil sx;
        make_stencil(S, p, sx);
        float v1, g1[3], vd, gd[3];
        interp(phi1, S, sx, v1, g1);
        interp(phiD, S, sx, vd, gd);
        const float sc[3] = {(float)(S.pme_grid[0] * S.invL[0]), (float)(S.pme_grid[1] * S.invL[1]),
                             (float)(S.pme_grid[2] * S.invL[2])};
        const size_t gsl = (size_t)R.slot_win + a.inv[gi];
        unsigned long long* F0[3] = {a.F0x, a.F0y, a.F0z};
        unsigned long long* dF[3] = {a.dFx, a.dFy, a.dFz};
        float f0[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            f0[k] = -q * sc[k] * g1[k];
            pme_red(F0[k] + gsl, f0[k], a.status);
        }
        const int gp = a.topo_grp[S.atom_base + i];
        if (gp == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) pme_red(dF[k] + gsl, -q * sc[k] * gd[k], a.status);
        }
    }
}

// displaced particles: forces at y in state 1 and the reciprocal part of u
__global__ void k_pme_gather_displaced(SdmArgs a) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;   // one per displaced particle
    if (item >= a.total_pert / 2) return;
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
    double du = 0.0;
    if (q != 0.0f) {
        const float* phi1 = a.pme_grid + R.pg_win;
        const float* phiD = phi1 + R.pg_size;
        Stencil sx, sy;
        make_stencil(S, a.pert_pos[pi].y, sx);        // state 0: x
        make_stencil(S, a.pert_pos[pi + 1].y, sy);    // state 1: y = x + d
        float v1x, g1x[3], vdx, gdx[3], v1y, g1y[3], vdy, gdy[3];
        interp(phi1, S, sx, v1x, g1x);
        interp(phiD, S, sx, vdx, gdx);
        interp(phi1, S, sy, v1y, g1y);
        interp(phiD, S, sy, vdy, gdy);
        du = (double)q * ((double)v1y - (double)v1x) + 0.5 * (double)q * ((double)vdy - (double)vdx);
        const float sc[3] = {(float)(S.pme_grid[0] * S.invL[0]), (float)(S.pme_grid[1] * S.invL[1]),
                             (float)(S.pme_grid[2] * S.invL[2])};
        const size_t gsl = (size_t)R.slot_win + a.inv[R.atom_win + p];
        unsigned long long* dF[3] = {a.dFx, a.dFy, a.dFz};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float f1 = -q * sc[k] * (g1y[k] + gdy[k]);
            const float f0 = -q * sc[k] * g1x[k];
            pme_red(dF[k] + gsl, f1 - f0, a.status);
        }
    }
    a.pme_du[item] = du;
}

}  // namespace

// Launch sequence of the reciprocal part (every replica of every system);
// plans[s] are the R2C / C2R plans of system s (batch: 2 grids per replica).
cudaError_t sdm_launch_pme(const SdmArgs& a, const cufftHandle* r2c, const cufftHandle* c2r, const long long* grid_off,
                           const long long* spec_off, int nsys, int conv_blocks, cudaStream_t st) {
    const int ns = 152 * 16;
    k_pme_spread<<<ns, 128, 0, st>>>(a);
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
    k_pme_gather<<<ns, 128, 0, st>>>(a);
    if (a.total_pert) k_pme_gather_displaced<<<(a.total_pert / 2 + 127) / 128, 128, 0, st>>>(a);
    return cudaGetLastError();
}
