// sdm_restraints.cu -- group-1 restraints of the reference's SDMUtils
// (python/SDMUtils.py) on the device (sm_103a).
//
// The reference adds them to LangevinIntegratorSDM's force group 1 as OpenMM
// custom forces (CustomCentroidBondForce SDMUtils.py:32-157,
// CustomCompoundBondForce SDMUtils.py:160-257); the integrator adds group-1
// energies and forces to the SDM result.  Here one block per replica
// evaluates them in FP64 on the caller's coordinates (no periodic images, as
// the custom forces default to): centroids by block reductions, the
// reference-particle terms in one thread, forces into the fixed-point F0
// accumulators (state independent: they reach F, F0 and F1 alike), the
// energy into rs_e (added to E_pot by the finalize kernel).
#include <cuda_runtime.h>

#include "../../include/sdm_capi.h"
#include "sdm_types.h"

namespace {

constexpr int kRsThreads = 128;

// round(v * 2^32) via two 32-bit conversions (|v| < 2^30)
__device__ __forceinline__ unsigned long long rs_fix64(float v) {
    const float a = rintf(v);
    const int hi = __float2int_rn(a);
    const int lo = __float2int_rn(__fmul_rn(__fsub_rn(v, a), 4294967296.0f));
    return (unsigned long long)(((long long)hi << 32) + (long long)lo);
}

__device__ __forceinline__ void rs_red(unsigned long long* p, double v, int* status) {
    const float f = (float)v;
    if (!(fabsf(f) < 1.0e9f)) {
        atomicOr(status, SDM_DEV_FORCE_OVERFLOW);
        return;
    }
    atomicAdd(p, rs_fix64(f));
}

__device__ double rs_block_sum(double v, double* red) {
    // fixed-shape tree: deterministic
    const int t = threadIdx.x;
    red[t] = v;
    __syncthreads();
    for (int s = kRsThreads / 2; s > 0; s >>= 1) {
        if (t < s) red[t] += red[t + s];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// ---- small FP64 vector helpers ----
struct V3 {
    double x, y, z;
};
__device__ __forceinline__ V3 v3(const double* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(V3 a) { return sqrt(dot(a, a)); }

// gradient of u/|u| contracted with g: (g - (g.n) n) / |u|
__device__ __forceinline__ V3 unit_back(V3 g, V3 n, double len) { return (1.0 / len) * (g - dot(g, n) * n); }

// v - P floor(v/P + 0.5) (SDMUtils.py:78-88)
__device__ __forceinline__ double rs_wrap(double v, double period) {
    return v - period * floor(v / period + 0.5);
}

// flat-bottom window (SDMUtils.py:69-71): energy and dE/dv; step(0) = 1
__device__ double rs_flat(double v, double lo, double hi, double period, double kf, double& dv) {
    const double db = rs_wrap(v - hi, period), da = rs_wrap(v - lo, period);
    const double dm = rs_wrap(v - 0.5 * (lo + hi), period);
    const double up = (dm >= 0.0) ? fmax(0.0, db) : 0.0;
    const double dn = (-dm >= 0.0) ? fmax(0.0, -da) : 0.0;
    dv = kf * (up - dn);
    return 0.5 * kf * (up * up + dn * dn);
}

// angle at p2 (atan2 of |u x v| and u.v) and its gradient
__device__ double rs_angle(V3 p1, V3 p2, V3 p3, V3 g[3]) {
    const V3 u = p1 - p2, v = p3 - p2;
    const V3 c = cross(u, v);
    const double s = norm(c), t = dot(u, v);
    const double den = s * s + t * t;
    const double inv_s = s > 0.0 ? 1.0 / s : 0.0;   // collinear: the sine term has no direction
    const V3 gu = (1.0 / den) * ((t * inv_s) * cross(v, c) - s * v);
    const V3 gv = (1.0 / den) * ((t * inv_s) * cross(c, u) - s * u);
    g[0] = gu;
    g[1] = -1.0 * (gu + gv);
    g[2] = gv;
    return atan2(s, t);
}

// IUPAC dihedral (trans = pi, cis = 0) and its gradient (Blondel and Karplus,
// J. Comput. Chem. 17, 1132 (1996), written for b1 = p2 - p1, b2 = p3 - p2,
// b3 = p4 - p3)
__device__ double rs_dihedral(V3 p1, V3 p2, V3 p3, V3 p4, V3 g[4]) {
    const V3 b1 = p2 - p1, b2 = p3 - p2, b3 = p4 - p3;
    const V3 m = cross(b1, b2), n = cross(b2, b3);
    const double lb2 = norm(b2);
    const double mm = dot(m, m), nn = dot(n, n);
    const V3 g1 = (mm > 0.0 ? -lb2 / mm : 0.0) * m;
    const V3 g4 = (nn > 0.0 ? lb2 / nn : 0.0) * n;
    const double f1 = dot(b1, b2) / (lb2 * lb2), f3 = dot(b3, b2) / (lb2 * lb2);
    g[0] = g1;
    g[1] = (-(1.0 + f1)) * g1 + f3 * g4;
    g[2] = f1 * g1 + (-(1.0 + f3)) * g4;
    g[3] = g4;
    return atan2(lb2 * dot(b1, n), dot(m, n));
}

// (k/2)(1 - cos) of the angle between u and v; adds dE/du, dE/dv
__device__ double rs_cos_term(V3 u, V3 v, double k, V3& gu, V3& gv) {
    const double lu = norm(u), lv = norm(v);
    const V3 nu = (1.0 / lu) * u, nv = (1.0 / lv) * v;
    const double c = dot(nu, nv);
    gu = (-0.5 * k) * unit_back(nv, nu, lu);
    gv = (-0.5 * k) * unit_back(nu, nv, lv);
    return 0.5 * k * (1.0 - c);
}

// psi term (SDMUtils.py:212-246): (k/2)(1 - cos) between the parts of
// x3 - x1 and x5 - x4 orthogonal to x2 - x1; gradient by reverse-mode chain
__device__ double rs_psi(V3 x1, V3 x2, V3 x3, V3 x4, V3 x5, double k, V3 g[5]) {
    const V3 d1 = x2 - x1;
    const double l1 = norm(d1);
    const V3 n1 = (1.0 / l1) * d1;
    const V3 d0 = x3 - x1, d3 = x5 - x4;
    const double pa = dot(d0, n1), pb = dot(d3, n1);
    const V3 v = d0 - pa * n1, w = d3 - pb * n1;
    const double lv = norm(v), lw = norm(w);
    const V3 vn = (1.0 / lv) * v, wn = (1.0 / lw) * w;
    const double c = dot(vn, wn);
    const double gc = -0.5 * k;
    const V3 gv = unit_back(gc * wn, vn, lv), gw = unit_back(gc * vn, wn, lw);
    V3 gd0 = gv, gd3 = gw;
    const double ga = -dot(gv, n1), gb = -dot(gw, n1);
    V3 gn1 = (-pa) * gv + (-pb) * gw;
    gd0 = gd0 + ga * n1;
    gn1 = gn1 + ga * d0;
    gd3 = gd3 + gb * n1;
    gn1 = gn1 + gb * d3;
    const V3 gd1 = unit_back(gn1, n1, l1);
    g[0] = -1.0 * (gd1 + gd0);
    g[1] = gd1;
    g[2] = gd0;
    g[3] = -1.0 * gd3;
    g[4] = gd3;
    return 0.5 * k * (1.0 - c);
}

__device__ __forceinline__ void gadd(double (*gp)[3], int slot, V3 g) {
    gp[slot][0] += g.x;
    gp[slot][1] += g.y;
    gp[slot][2] += g.z;
}

__global__ void __launch_bounds__(kRsThreads) k_restraints(SdmArgs a) {
    __shared__ double red[kRsThreads];
    __shared__ double cent[2][3];   // centroids
    __shared__ double gc[2][3];     // dE/dc_g / W_g
    __shared__ double gp[12][3];    // dE/dx of the reference particles (slots as rs_ref)
    const int r = blockIdx.x, t = threadIdx.x;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    if (!S.rs_on) {   // block-uniform
        if (t == 0) a.rs_e[r] = 0.0;
        return;
    }
    const double* x = a.x + 3 * (size_t)R.x_off;
    const double* P = a.rs_prm + S.rs_prm;
    const int* idx = a.rs_idx + S.rs_base;
    const double* w = a.rs_w + S.rs_base;
    if (S.rs_on & 1) {
#pragma unroll 1
        for (int g = 0; g < 2; ++g) {
            const int n = g ? S.rs_nrcpt : S.rs_nlig, off = g ? S.rs_nlig : 0;
            double s[3] = {0.0, 0.0, 0.0};
            for (int k = t; k < n; k += kRsThreads) {
                const int i = idx[off + k];
                const double wi = w[off + k];
                s[0] += wi * x[3 * (size_t)i];
                s[1] += wi * x[3 * (size_t)i + 1];
                s[2] += wi * x[3 * (size_t)i + 2];
            }
            const double invw = P[g ? SDM_RS_INVW_RCPT : SDM_RS_INVW_LIG];
#pragma unroll 1
            for (int c = 0; c < 3; ++c) {
                const double tot = rs_block_sum(s[c], red);
                if (t == 0) cent[g][c] = tot * invw;
            }
        }
    }
    if (t < 36) gp[t / 3][t % 3] = 0.0;
    if (t < 6) gc[t / 3][t % 3] = 0.0;
    __syncthreads();
    if (t == 0) {
        const double lam = a.rs_lam[r];
        double E = 0.0;
        if (S.rs_on & 1) {
            const V3 D = V3{cent[0][0], cent[0][1], cent[0][2]} - V3{P[SDM_RS_OFF], P[SDM_RS_OFF + 1], P[SDM_RS_OFF + 2]} -
                         V3{cent[1][0], cent[1][1], cent[1][2]};
            const double d = norm(D), tol = P[SDM_RS_TOLCM];
            if (d >= tol && d > 0.0) {
                E += lam * 0.5 * P[SDM_RS_KFCM] * (d - tol) * (d - tol);
                const double coef = lam * P[SDM_RS_KFCM] * (d - tol) / d;
                gc[0][0] = coef * D.x * P[SDM_RS_INVW_LIG];
                gc[0][1] = coef * D.y * P[SDM_RS_INVW_LIG];
                gc[0][2] = coef * D.z * P[SDM_RS_INVW_LIG];
                gc[1][0] = -coef * D.x * P[SDM_RS_INVW_RCPT];
                gc[1][1] = -coef * D.y * P[SDM_RS_INVW_RCPT];
                gc[1][2] = -coef * D.z * P[SDM_RS_INVW_RCPT];
            }
        }
        if (S.rs_on & 2) {
            V3 q[6];
            for (int k = 0; k < 6; ++k) q[k] = v3(x + 3 * (size_t)S.rs_ref[k]);   // r0 r1 r2 l0 l1 l2
            const double pi = 3.14159265358979323846;
            V3 g[4];
            double dv;
            // theta = angle(r0, l0, l1), period pi
            double v = rs_angle(q[0], q[3], q[4], g);
            E += lam * rs_flat(v, P[SDM_RS_ALO], P[SDM_RS_AHI], pi, P[SDM_RS_KFA], dv);
            gadd(gp, 0, (lam * dv) * g[0]);
            gadd(gp, 3, (lam * dv) * g[1]);
            gadd(gp, 4, (lam * dv) * g[2]);
            // phi1 = dihedral(r1, r0, l0, l1)
            v = rs_dihedral(q[1], q[0], q[3], q[4], g);
            E += lam * rs_flat(v, P[SDM_RS_D1LO], P[SDM_RS_D1HI], 2.0 * pi, P[SDM_RS_KFD1], dv);
            gadd(gp, 1, (lam * dv) * g[0]);
            gadd(gp, 0, (lam * dv) * g[1]);
            gadd(gp, 3, (lam * dv) * g[2]);
            gadd(gp, 4, (lam * dv) * g[3]);
            // phi2 = dihedral(r0, l0, l1, l2)
            v = rs_dihedral(q[0], q[3], q[4], q[5], g);
            E += lam * rs_flat(v, P[SDM_RS_D2LO], P[SDM_RS_D2HI], 2.0 * pi, P[SDM_RS_KFD2], dv);
            gadd(gp, 0, (lam * dv) * g[0]);
            gadd(gp, 3, (lam * dv) * g[1]);
            gadd(gp, 4, (lam * dv) * g[2]);
            gadd(gp, 5, (lam * dv) * g[3]);
        }
        if (S.rs_on & 4) {   // alignment (no control parameter, as in the reference)
            V3 q[6];
            for (int k = 0; k < 6; ++k) q[k] = v3(x + 3 * (size_t)S.rs_ref[6 + k]);   // a0 a1 a2 b0 b1 b2
            const V3 a0 = q[0], a1 = q[1], a2 = q[2], b0 = q[3], b1 = q[4], b2 = q[5];
            // (kd/2)|b0 - off - a0|^2
            const V3 dd = b0 - V3{P[SDM_RS_AOFF], P[SDM_RS_AOFF + 1], P[SDM_RS_AOFF + 2]} - a0;
            E += 0.5 * P[SDM_RS_KDISPL] * dot(dd, dd);
            gadd(gp, 9, P[SDM_RS_KDISPL] * dd);
            gadd(gp, 6, (-P[SDM_RS_KDISPL]) * dd);
            // (kt/2)(1 - cos) between b1 - b0 and a1 - a0
            V3 gu, gv;
            E += rs_cos_term(b1 - b0, a1 - a0, P[SDM_RS_KTHETA], gu, gv);
            gadd(gp, 10, gu);
            gadd(gp, 9, -1.0 * gu);
            gadd(gp, 7, gv);
            gadd(gp, 6, -1.0 * gv);
            // psi, both orders, k_psi/2 each (SDMUtils.py:248-254)
            V3 g5[5];
            E += rs_psi(b0, b1, b2, a0, a2, 0.5 * P[SDM_RS_KPSI], g5);
            gadd(gp, 9, g5[0]);
            gadd(gp, 10, g5[1]);
            gadd(gp, 11, g5[2]);
            gadd(gp, 6, g5[3]);
            gadd(gp, 8, g5[4]);
            E += rs_psi(a0, a1, a2, b0, b2, 0.5 * P[SDM_RS_KPSI], g5);
            gadd(gp, 6, g5[0]);
            gadd(gp, 7, g5[1]);
            gadd(gp, 8, g5[2]);
            gadd(gp, 9, g5[3]);
            gadd(gp, 11, g5[4]);
        }
        a.rs_e[r] = E;
    }
    __syncthreads();
    unsigned long long* F0[3] = {a.F0x, a.F0y, a.F0z};
    if (S.rs_on & 1) {
        for (int k = t; k < S.rs_nlig + S.rs_nrcpt; k += kRsThreads) {
            const int g = k < S.rs_nlig ? 0 : 1;
            const int i = idx[k];
            const size_t sl = (size_t)R.slot_win + a.inv[R.atom_win + i];
#pragma unroll
            for (int c = 0; c < 3; ++c) rs_red(F0[c] + sl, -gc[g][c] * w[k], a.status);
        }
    }
    const bool used = (t < 6 && (S.rs_on & 2)) || (t >= 6 && t < 12 && (S.rs_on & 4));
    if (used) {
        const size_t sl = (size_t)R.slot_win + a.inv[R.atom_win + S.rs_ref[t]];
#pragma unroll
        for (int c = 0; c < 3; ++c) rs_red(F0[c] + sl, -gp[t][c], a.status);
    }
}

}  // namespace

cudaError_t sdm_launch_restraints(const SdmArgs& a, cudaStream_t st) {
    if (!a.rs_any) return cudaSuccess;
    k_restraints<<<a.nrep, kRsThreads, 0, st>>>(a);
    return cudaGetLastError();
}
