// sdm_kernels.cu -- CUDA kernels (sm_103a) of the SDM two-state force.
//
// Pipeline of one evaluation (every launch covers all replicas of all systems):
//   k_cells     wrap coordinates, integer cells, cell histogram
//   k_scan      per-replica column prefix sums (particles, clusters) and the
//               global work-item prefix (last block)
//   k_bucket    scatter particles into their cell (cells of a column consecutive)
//   k_cellsort  rank of every particle inside its cell by (z, particle index);
//               cells are z-ordered within a column -> column slots
//   k_clusters  cluster-local FP32 coordinates, parameters, bounding boxes,
//               exclusion partners as slots
//   k_pair      persistent main pass: every pair at the original coordinates
//               (U0, F0), LJ + reaction field, FP32 math, fixed-point forces
//   k_pert_prep the displaced particles' positions in both states
//   k_perturb   perturbation pass: only pairs whose displacements differ, at
//               both states -> u (FP64) and dF = F1 - F0 (fixed point)
//   k_combine   deterministic reduction of u, soft core, bias, weight s
//               (needs no main-pass result: runs beside it)
//   k_finalize_mix  F = F0 + s dF in original particle order; one more block
//               per replica reduces U0 and writes the results
//               (k_langevin: the same layout with the stochastic-dynamics
//               update; k_mix: the state forces)
//
// Reference correspondence: the two nonbonded evaluations of
// openmmapi/src/LangevinIntegratorSDM.cpp:158-176 (OpenMM NonbondedForce at x
// and x+d), the displacement MakeState2 (platforms/opencl/src/kernels/
// langevin.cl:198-206), the combine of platforms/reference/src/
// ReferenceSDMKernels.cpp:247-318 and the mix kernel sdmForce
// (langevin.cl:72-87).  The save/restore copies of the reference
// (SaveState1/SaveState2/RestoreState1, langevin.cl:147-192) disappear: both
// states are evaluated from the same resident coordinates.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/sdm_capi.h"
#include "sdm_types.h"

#define SDM_WARPS 4
#define SDM_JL_CAP 256
#define SDM_RING 64
#define SDM_INVALID_COORD 1.0e6f

namespace {

// ------------------------------------------------------------------------- //
// small helpers                                                             //
// ------------------------------------------------------------------------- //
__device__ __forceinline__ double wrap1(double v, double L, double invL) {
    double t = floor(__dmul_rn(v, invL));
    double w = __dsub_rn(v, __dmul_rn(t, L));
    if (w >= L) w = __dsub_rn(w, L);
    if (w < 0.0) w = __dadd_rn(w, L);
    return w;
}

__device__ __forceinline__ int cell_of(double w, double invg, int M) {
    int c = __double2int_rd(__dmul_rn(w, invg));
    c = c < 0 ? 0 : c;
    return c > M - 1 ? M - 1 : c;
}

__device__ __forceinline__ int wrap_cell(int n, int M) {
    if (2 * n > M) n -= M;
    else if (2 * n <= -M) n += M;
    return n;
}


__device__ __forceinline__ float img32(float d, float L, float invL) {
    float t = rintf(__fmul_rn(d, invL));
    return __fmaf_rn(-L, t, d);
}

__device__ __forceinline__ float r2_chain(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

__device__ __forceinline__ float fast_rsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float fast_rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Ewald screening: erfc(x) = R(t) exp(-x^2), t = 1 / (1 + kErfcP x), R a
// degree-7 polynomial in t fitted to erfc(x) exp(x^2) for 0 <= x <= 4
// (least squares with Lawson reweighting, csrc/fit_erfc.py): relative error
// 2e-8 in exact arithmetic, 4e-7 evaluated in FP32 with the exponential.
// The exponential is the one the Ewald force needs anyway.  Valid for
// beta rc <= 4, i.e. Ewald tolerances >= 5.7e-8 (checked on the host).
constexpr float kErfcP = 0.46f;
__device__ __forceinline__ float2 erfc_scaled2(float2 x) {
    const float2 t = make_float2(fast_rcp(__fmaf_rn(kErfcP, x.x, 1.0f)), fast_rcp(__fmaf_rn(kErfcP, x.y, 1.0f)));
    float2 r = __ffma2_rn(make_float2(0.10056333988904953f, 0.10056333988904953f), t,
                          make_float2(-0.5065137147903442f, -0.5065137147903442f));
    r = __ffma2_rn(r, t, make_float2(0.8315963745117188f, 0.8315963745117188f));
    r = __ffma2_rn(r, t, make_float2(-0.3618384897708893f, -0.3618384897708893f));
    r = __ffma2_rn(r, t, make_float2(0.4733056426048279f, 0.4733056426048279f));
    r = __ffma2_rn(r, t, make_float2(0.19405683875083923f, 0.19405683875083923f));
    r = __ffma2_rn(r, t, make_float2(0.269482284784317f, 0.269482284784317f));
    return __ffma2_rn(r, t, make_float2(-0.0006523068295791745f, -0.0006523068295791745f));
}
__device__ __forceinline__ float erfc_scaled(float x) {
    const float t = fast_rcp(__fmaf_rn(kErfcP, x, 1.0f));
    float r = __fmaf_rn(0.10056333988904953f, t, -0.5065137147903442f);
    r = __fmaf_rn(r, t, 0.8315963745117188f);
    r = __fmaf_rn(r, t, -0.3618384897708893f);
    r = __fmaf_rn(r, t, 0.4733056426048279f);
    r = __fmaf_rn(r, t, 0.19405683875083923f);
    r = __fmaf_rn(r, t, 0.269482284784317f);
    return __fmaf_rn(r, t, -0.0006523068295791745f);
}


__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// replica lookup by window base (rep[] sorted by every window)
__device__ __forceinline__ int rep_by_atom(const SdmRep* rep, int nrep, int gi) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (rep[mid].atom_win <= gi) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int rep_by_col(const SdmRep* rep, int nrep, int gi) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (rep[mid].col_win <= gi) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int rep_by_slot(const SdmRep* rep, int nrep, int gi) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (rep[mid].slot_win <= gi) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int rep_by_pert(const SdmRep* rep, int nrep, int gi) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (rep[mid].pert_win <= gi) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int rep_by_ex(const SdmRep* rep, int nrep, int gi) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (rep[mid].ex_win <= gi) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int rep_by_item(const int* prefix, int nrep, int item) {
    int lo = 0, hi = nrep - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ------------------------------------------------------------------------- //
// K1: cells                                                                 //
// ------------------------------------------------------------------------- //
__global__ void k_cells(SdmArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < a.total_atoms; gi += stride) {
        const int r = rep_by_atom(a.rep, a.nrep, gi);
        const SdmRep& R = a.rep[r];
        const SdmSys& S = a.sys[R.sys];
        const int i = gi - R.atom_win;
        const double* xp = a.x + 3 * (R.x_off + i);
        int c[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            // 0 <= v < L (1 - 2^-40): floor(v / L) rounds to 0 and the wrap is
            // the identity; only other coordinates take the FP64 wrap
            double w = xp[k];
            const long long b = __double_as_longlong(w);
            if (!(b >= 0 && b < S.wrap_lim[k])) {
                // NaN / Inf (exponent all ones): reported; the particle lands in
                // a clamped cell and fails every distance test
                if (((b >> 52) & 0x7ff) == 0x7ff) atomicOr(a.status, SDM_DEV_COORD_NONFINITE);
                w = wrap1(w, S.box[k], S.invL[k]);
            }
            a.w[3 * (size_t)gi + k] = w;
            c[k] = cell_of(w, S.invg[k], S.M[k]);
        }
        const int col = c[0] * S.M[1] + c[1];
        a.cellinfo[gi] = make_int2(col, c[2]);
        atomicAdd(&a.cel_cnt[R.cel_win + col * S.M[2] + c[2]], 1);
    }
}

// ------------------------------------------------------------------------- //
// K2: column prefix sums; the last block builds the work-item prefix        //
// ------------------------------------------------------------------------- //
__device__ __forceinline__ int4 warp_incl_scan3(int4 v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, v.x, o);
        const int y = __shfl_up_sync(0xffffffffu, v.y, o);
        const int z = __shfl_up_sync(0xffffffffu, v.z, o);
        if (lane_id() >= o) { v.x += x; v.y += y; v.z += z; }
    }
    return v;
}

// Column prefixes of particles, clusters and list-building groups (a.jg <=
// SDM_JG z-consecutive clusters of one column); the group table (first cluster,
// clusters) of every group.  The last block builds the work-item prefix of
// the main pass and the group prefix of the list builder over replicas.
__global__ void __launch_bounds__(1024) k_scan(SdmArgs a, int* item_prefix, int* grp_prefix, int* done) {
    __shared__ int4 wsum[32];
    __shared__ int last;
    const int r = blockIdx.x;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int ncol = S.ncol, mz = S.M[2];
    const int* ccnt = a.cel_cnt + R.cel_win;
    int* coff = a.cel_off + R.cel_win;
    int* cnt = a.col_cnt + R.col_win;
    int* aoff = a.col_aoff + R.col_win;
    int* cl = a.col_cl + R.col_win;
    int2* grp = a.cl_grp + R.cl_win;
    const int per = (ncol + blockDim.x - 1) / blockDim.x;
    const int beg = min(ncol, (int)threadIdx.x * per);
    const int end = min(ncol, beg + per);
    int4 s = make_int4(0, 0, 0, 0);
    for (int c = beg; c < end; ++c) {
        int n = 0;
        for (int z = 0; z < mz; ++z) n += ccnt[c * mz + z];
        cnt[c] = n;
        const int nc = (n + 7) >> 3;
        s.x += n;
        s.y += nc;
        s.z += (nc + a.jg - 1) / a.jg;
    }
    int4 inc = warp_incl_scan3(s);
    const int wid = threadIdx.x >> 5;
    if (lane_id() == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int4 v = (lane_id() < (int)(blockDim.x >> 5)) ? wsum[lane_id()] : make_int4(0, 0, 0, 0);
        v = warp_incl_scan3(v);
        wsum[lane_id()] = v;
    }
    __syncthreads();
    int4 base = make_int4(inc.x - s.x, inc.y - s.y, inc.z - s.z, 0);
    if (wid > 0) { base.x += wsum[wid - 1].x; base.y += wsum[wid - 1].y; base.z += wsum[wid - 1].z; }
    for (int c = beg; c < end; ++c) {
        aoff[c] = base.x;
        cl[c] = base.y;
        int o = base.x;
        for (int z = 0; z < mz; ++z) { coff[c * mz + z] = o; o += ccnt[c * mz + z]; }
        const int nc = (cnt[c] + 7) >> 3;
        for (int k = 0; k < nc; k += a.jg) grp[base.z++] = make_int2(base.y + k, min(a.jg, nc - k));
        base.x += cnt[c];
        base.y += nc;
    }
    if (threadIdx.x == blockDim.x - 1) {
        aoff[ncol] = base.x;
        cl[ncol] = base.y;
        coff[ncol * mz] = base.x;
        a.ncl[r] = base.y;
        a.ngrp[r] = base.z;
    }
    // last block computes the prefixes over replicas (no waiting involved)
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(done, 1) == (int)gridDim.x - 1);
    __syncthreads();
    if (last) {
        __threadfence();
        // sequential chunks + block scan, same as above
        const int nrep = a.nrep;
        const int per2 = (nrep + blockDim.x - 1) / blockDim.x;
        const int b2 = min(nrep, (int)threadIdx.x * per2);
        const int e2 = min(nrep, b2 + per2);
        int4 t = make_int4(0, 0, 0, 0);
        for (int q = b2; q < e2; ++q) {
            t.x += ((volatile int*)a.ncl)[q] * a.split;
            t.y += ((volatile int*)a.ngrp)[q];
        }
        int4 inc2 = warp_incl_scan3(t);
        __syncthreads();
        if (lane_id() == 31) wsum[wid] = inc2;
        __syncthreads();
        if (wid == 0) {
            int4 v = (lane_id() < (int)(blockDim.x >> 5)) ? wsum[lane_id()] : make_int4(0, 0, 0, 0);
            v = warp_incl_scan3(v);
            wsum[lane_id()] = v;
        }
        __syncthreads();
        int b = inc2.x - t.x + (wid > 0 ? wsum[wid - 1].x : 0);
        int bg = inc2.y - t.y + (wid > 0 ? wsum[wid - 1].y : 0);
        for (int q = b2; q < e2; ++q) {
            item_prefix[q] = b;
            grp_prefix[q] = bg;
            b += ((volatile int*)a.ncl)[q] * a.split;
            bg += ((volatile int*)a.ngrp)[q];
        }
        if (threadIdx.x == blockDim.x - 1) { item_prefix[nrep] = b; grp_prefix[nrep] = bg; }
        if (threadIdx.x == 0) *done = 0;
    }
}

// ------------------------------------------------------------------------- //
// K3: bucket                                                                //
// ------------------------------------------------------------------------- //
__global__ void k_bucket(SdmArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < a.total_atoms; gi += stride) {
        const int r = rep_by_atom(a.rep, a.nrep, gi);
        const SdmRep& R = a.rep[r];
        const int2 ci = a.cellinfo[gi];
        const int cell = R.cel_win + ci.x * a.sys[R.sys].M[2] + ci.y;
        const int pos = atomicAdd(&a.cel_fill[cell], 1);
        a.bucket[R.atom_win + a.cel_off[cell] + pos] = gi - R.atom_win;
    }
}

// ------------------------------------------------------------------------- //
// K4: rank sort of every cell by (z, particle)                              //
// ------------------------------------------------------------------------- //
// The bucket holds each column's particles cell by cell (z cells ascending),
// and the z cell is monotone in z: ranking every particle inside its own cell
// gives the column's order by (z, particle).  Keys are the bit patterns of the
// wrapped z coordinates (non-negative doubles order like their bits once -0.0
// is canonicalised) with the particle index as tie-break: integer compares
// only (FP64 compares are slow on GB300).
__device__ __forceinline__ unsigned long long zkey(double z) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(z);
    return b == 0x8000000000000000ull ? 0ull : b;   // -0.0 -> +0.0 without the FP64 pipe
}

__global__ void k_cellsort(SdmArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < a.total_atoms; gi += stride) {
        const int r = rep_by_atom(a.rep, a.nrep, gi);
        const SdmRep& R = a.rep[r];
        const int mz = a.sys[R.sys].M[2];
        const int ai = a.bucket[gi];
        const int2 ci = a.cellinfo[R.atom_win + ai];
        const int cell = R.cel_win + ci.x * mz + ci.y;
        const int cb = a.cel_off[cell], ce = a.cel_off[cell + 1];
        const unsigned long long zi = zkey(a.w[3 * (size_t)(R.atom_win + ai) + 2]);
        int rank = 0;
        for (int q = cb; q < ce; ++q) {
            const int aj = a.bucket[R.atom_win + q];
            const unsigned long long zj = zkey(a.w[3 * (size_t)(R.atom_win + aj) + 2]);
            rank += (zj < zi) || (zj == zi && aj < ai);
        }
        const int col = R.col_win + ci.x;
        const int slot = 8 * a.col_cl[col] + (cb - a.col_aoff[col]) + rank;
        a.perm[R.slot_win + slot] = ai;
        a.inv[R.atom_win + ai] = slot;
        if ((slot & 7) == 0) {   // a cluster's reference cell is its first particle's cell
            const int m1 = a.sys[R.sys].M[1];
            const int cx = ci.x / m1;
            a.cl_ref[R.cl_win + (slot >> 3)] = make_int4(cx, ci.x - cx * m1, ci.y, ci.x);
        }
    }
    // padding slots at the end of every column
    for (int gc = blockIdx.x * blockDim.x + threadIdx.x; gc < a.total_cols; gc += stride) {
        const int r = rep_by_col(a.rep, a.nrep, gc);
        const SdmRep& R = a.rep[r];
        if (gc - R.col_win >= a.sys[R.sys].ncol) continue;
        const int send = 8 * a.col_cl[gc + 1];
        for (int s = 8 * a.col_cl[gc] + a.col_cnt[gc]; s < send; ++s) a.perm[R.slot_win + s] = -1;
    }
}

// ------------------------------------------------------------------------- //
// K5: cluster data                                                          //
// ------------------------------------------------------------------------- //
__global__ void k_clusters(SdmArgs a) {
    const int stride = gridDim.x * blockDim.x;   // multiple of 8 (block size multiple of 32)
    const int lane = lane_id();
    const unsigned gmask = 0xffu << (lane & 24);
    for (int gs = blockIdx.x * blockDim.x + threadIdx.x; gs < a.total_slots; gs += stride) {
        const int r = rep_by_slot(a.rep, a.nrep, gs);
        const SdmRep& R = a.rep[r];
        const SdmSys& S = a.sys[R.sys];
        const int s = gs - R.slot_win;
        const int C = s >> 3, t = s & 7;
        if (C >= a.ncl[r]) continue;   // uniform over the 8-lane group
        const int p = a.perm[gs];
        const int4 ref = a.cl_ref[R.cl_win + C];   // written by k_cellsort
        const int cx = ref.x, cy = ref.y, cz = ref.z;
        const double* org = a.cell_org + S.org_base;
        const double Rr[3] = {org[cx], org[S.M[0] + cy], org[S.M[0] + S.M[1] + cz]};
        float X[3];
        float4 q4;
        float2 p2;
        int g = 0;
        int4 ex = make_int4(-1, -1, -1, -1);
        if (p >= 0) {
            const double* wp = a.w + 3 * (size_t)(R.atom_win + p);
#pragma unroll
            for (int k = 0; k < 3; ++k) X[k] = __double2float_rn(__dsub_rn(wp[k], Rr[k]));
            const int ta = S.atom_base + p;
            q4 = make_float4(X[0], X[1], X[2], a.topo_q[ta]);
            p2 = make_float2(a.topo_hs[ta], a.topo_se[ta]);
            g = a.topo_grp[ta];
            const int4 pe = a.topo_ex4[ta];
            if (pe.x == -2) {
                ex = make_int4(-2, -2, -2, -2);
            } else {
                const int pv[4] = {pe.x, pe.y, pe.z, pe.w};
                int v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = (pv[u] >= 0) ? a.inv[R.atom_win + pv[u]] : -1;
                ex = make_int4(v[0], v[1], v[2], v[3]);
            }
        } else {
            X[0] = X[1] = X[2] = SDM_INVALID_COORD;
            q4 = make_float4(X[0], X[1], X[2], 0.0f);
            p2 = make_float2(0.0f, 0.0f);
        }
        // the slot's fixed-point force accumulators start the call at zero
        // (every later force goes in by integer atomics; slots past the
        // replica's clusters are read by nobody)
        a.F0x[gs] = 0ull; a.F0y[gs] = 0ull; a.F0z[gs] = 0ull;
        a.dFx[gs] = 0ull; a.dFy[gs] = 0ull; a.dFz[gs] = 0ull;
        a.clX[gs] = q4;
        a.clP[gs] = p2;
        a.grp[gs] = g;
        a.clM[gs] = (p >= 0) ? a.topo_mol[S.atom_base + p] : -1 - t;
        a.excl4[gs] = ex;
        // bounding box over valid slots
        float lo[3], hi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = (p >= 0) ? X[k] : 3.0e38f;
            hi[k] = (p >= 0) ? X[k] : -3.0e38f;
        }
#pragma unroll
        for (int o = 1; o < 8; o <<= 1)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(gmask, lo[k], o, 8));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(gmask, hi[k], o, 8));
            }
        // exclusion-linked clusters: distinct clusters (other than C) holding
        // partners of this cluster's particles, ascending; -2 when more than 8
        // or unknown.  Extracted as successive minima over the 8-lane group.
        const int e4[4] = {ex.x, ex.y, ex.z, ex.w};
        int pc[4];
        bool many = false;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            many |= (e4[k] == -2);
            const int cc = e4[k] >> 3;
            pc[k] = (e4[k] >= 0 && cc != C) ? cc : 0x7fffffff;
        }
        many = __any_sync(gmask, many);
        int link[8];
        int last = -1;
#pragma unroll
        for (int u = 0; u < 9; ++u) {
            int m = 0x7fffffff;
#pragma unroll
            for (int k = 0; k < 4; ++k) m = (pc[k] > last && pc[k] < m) ? pc[k] : m;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) m = min(m, __shfl_xor_sync(gmask, m, o, 8));
            if (u < 8) link[u] = (m == 0x7fffffff) ? -1 : m;
            else if (m != 0x7fffffff) many = true;
            last = m;
        }
        // absolute z of the first and last particle (rounded outwards, monotone
        // along a column), for the z-range searches of the list builder
        const double wz = (p >= 0) ? a.w[3 * (size_t)(R.atom_win + p) + 2] : 0.0;
        const unsigned vm = (__ballot_sync(gmask, p >= 0) >> (lane & 24)) & 0xffu;
        const int lastv = 31 - __clz(vm);
        const double wz0 = __shfl_sync(gmask, wz, 0, 8);
        const double wzl = __shfl_sync(gmask, wz, lastv, 8);
        if (t == 0) {
            const int cw = R.cl_win + C;
            a.cl_zb[cw] = make_float2(__double2float_rd(wz0) - 1.0e-4f, __double2float_ru(wzl) + 1.0e-4f);
            // w: the reference z cell, so candidate scans need no cl_ref load
            a.cl_bbc[cw] = make_float4(__fmul_rn(0.5f, __fadd_rn(lo[0], hi[0])),
                                       __fmul_rn(0.5f, __fadd_rn(lo[1], hi[1])),
                                       __fmul_rn(0.5f, __fadd_rn(lo[2], hi[2])), __int_as_float(cz));
            a.cl_bbh[cw] = make_float4(__fmul_rn(0.5f, __fsub_rn(hi[0], lo[0])),
                                       __fmul_rn(0.5f, __fsub_rn(hi[1], lo[1])),
                                       __fmul_rn(0.5f, __fsub_rn(hi[2], lo[2])), 0.0f);
            a.cl_link[2 * (size_t)cw] = many ? make_int4(-2, -2, -2, -2)
                                             : make_int4(link[0], link[1], link[2], link[3]);
            a.cl_link[2 * (size_t)cw + 1] = many ? make_int4(-2, -2, -2, -2)
                                                 : make_int4(link[4], link[5], link[6], link[7]);
        }
        // the replica's largest cluster z extent: one atomic per replica present
        // in the warp (same-address atomics serialise in L2: one per cluster
        // cost ~30 us per call on the 22-replica batch)
        {
            const unsigned act = __activemask();   // the 8-lane groups of valid clusters
            const unsigned same = __match_any_sync(act, r);
            const unsigned zmax = __reduce_max_sync(same, __float_as_uint(fmaxf(hi[2], 0.0f)));
            if (lane == __ffs(same) - 1) atomicMax(&a.extz[r], zmax);
        }
    }
}

// per-pair minimum image is needed unless the largest cluster z extent stays
// below the host threshold tz = 0.5*Lz - rc - 1e-3 (rounded down to float)
__device__ __forceinline__ bool replica_image_mode(const SdmArgs& a, const SdmSys& S, int r) {
    if (S.img_static) return true;
    return !(__uint_as_float(a.extz[r]) < S.tz);
}

enum { MODE_EVAL = 0, MODE_COUNT = 1, MODE_EMIT = 2 };

struct WarpSmem {               // perturbation pass scratch
    int4 jl[SDM_JL_CAP];        // (J, Sx, Sy, Sz)
    int4 rng[64];               // (Jbegin, prefix, Sx bits, Sy bits)
};

struct Ring {                   // one tile ring: 64 prepared j entries
    float4 a[SDM_RING];         // (xs, ys, zs, q)
    float4 b[SDM_RING];         // (hs, se, mask bits, slot bits)
};

// cluster-pair list entries per staged chunk (SDM_OPT_STAGE_CHUNK): 8, 12 (default) or 16
#define SDM_CH_DEFAULT 12

// Two-level cp.async pipeline: list entries two chunks ahead, the candidate
// particles (8 per entry) one chunk ahead of the chunk being filtered.
// i-cluster data of particles (2u, 2u+1) in three 16-byte words per u, read
// as shared-memory broadcasts: (q, q', sigma/2, sigma'/2),
// (2 sqrt(eps), 2 sqrt(eps'), -x, -x'), (-y, -y', -z, -z')
struct IPar3 {
    float4 a[4], b[4], c[4];
};

template <int CH>
struct EvalSmem {
    Ring lj;                    // j with epsilon != 0
    Ring co;                    // j with epsilon == 0 (Coulomb only)
    int4 je[3][CH];             // list entries of chunks c, c+1, c+2
    float4 sx[2][CH * 8];       // staged cluster-local coordinates + charge of candidates
    float2 sp[2][CH * 8];       // staged (sigma/2, 2 sqrt(eps)) of candidates
    int sm_[2][CH * 8];         // staged molecule ids of candidates
    IPar3 ip;                   // i-cluster parameters by particle pair, read as broadcasts
    int im[8];                  // i-cluster molecule ids
    float4 ib[2];               // i-cluster box centre and half extents (w: list cutoff squared)
};


__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Force accumulators of the 8 i particles in pairs (2u, 2u+1) for the packed
// FP32x2 pipe: sum_j fs (x_j - x_i), i.e. minus the force on i.
struct ICluster {
    float2 ax[4], ay[4], az[4];
};

// round(v * 2^32) as a 64-bit two's-complement integer from two 32-bit
// conversions (|v| < 2^30, checked by the caller); avoids the float->int64
// conversion, which runs on the narrow FP64 pipe.
__device__ __forceinline__ unsigned long long fix64(float v) {
    const float a = rintf(v);
    const int hi = __float2int_rn(a);
    const int lo = __float2int_rn(__fmul_rn(__fsub_rn(v, a), 4294967296.0f));
    return (unsigned long long)(((long long)hi << 32) + (long long)lo);
}

__device__ __forceinline__ void red_fix(unsigned long long* p, float v, int* status) {
    if (!(fabsf(v) < 1.0e9f)) atomicOr(status, SDM_DEV_FORCE_OVERFLOW);
    atomicAdd(p, fix64(v));
}

// ------------------------------------------------------------------------- //
// K6a: cluster-pair lists.  For i-cluster I: every cluster J >= I (slot     //
// order) of the half stencil whose shifted bounding box comes within        //
// rc + margin of I's box, as (J | needmask<<31, Sx, Sy, Sz).                //
// ------------------------------------------------------------------------- //
__device__ __forceinline__ int wrap_add(int c, int o, int M) {
    c += o;
    if (c < 0) c += M;
    else if (c >= M) c -= M;
    return c;
}

// first J in [lo, hi) of a column with zhi_J >= z (zhi non-decreasing)
__device__ __forceinline__ int lower_zhi(const float2* zb, int lo, int hi, float z) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (zb[mid].y < z) lo = mid + 1; else hi = mid;
    }
    return lo;
}
// first J in [lo, hi) with zlo_J > z (zlo non-decreasing)
__device__ __forceinline__ int upper_zlo(const float2* zb, int lo, int hi, float z) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (zb[mid].x <= z) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Per-warp scratch of the list builder: candidate ranges of one stencil round
// and the group's clusters (box centre with the reference z cell in w, half
// extents, exclusion-linked clusters).
struct JlSmem {
    int4 rng[64];               // (Jbegin | own column << 31, prefix, Sx bits, Sy bits)
    float4 bc[SDM_JG];
    float4 bh[SDM_JG];
    int4 lk[SDM_JG][2];
};

// The lists of the nI <= a.jg <= SDM_JG z-consecutive clusters I0.. of one column.
// The column searches run once over the union of the members' z windows and
// each candidate's box is loaded once; every member then applies its own
// box test (the rule of a list built for that cluster alone) and appends to
// its own list in candidate order.
template <bool IMG>
__device__ void build_jlist(const SdmArgs& a, int r, int g, JlSmem& js) {
    const int lane = lane_id();
    const SdmRep R = a.rep[r];
    const SdmSys S = a.sys[R.sys];
    const int2 gi = a.cl_grp[R.cl_win + g];
    const int I0 = gi.x, nI = gi.y;
    const int cw0 = R.cl_win + I0;
    const int4 ref = a.cl_ref[cw0];   // column (x, y, id): the same for every member
    if (lane < nI) {
        js.bc[lane] = a.cl_bbc[cw0 + lane];
        js.bh[lane] = a.cl_bbh[cw0 + lane];
    }
    if (lane < 2 * nI) js.lk[lane >> 1][lane & 1] = a.cl_link[2 * (size_t)cw0 + lane];
    __syncwarp();
    const float rclc = S.rcl + 2.0e-4f;
    const float rclc2 = rclc * rclc;
    const float* tabx = a.shift_tab + S.shift_base;
    const float* taby = tabx + 2 * S.M[0] + 1;
    const float* tabz = taby + 2 * S.M[1] + 1;
    const int* colcl = a.col_cl + R.col_win;
    const float2* zb = a.cl_zb + R.cl_win;
    // union over the members: z window (absolute, conservative) and xy box
    float ZA = 3.0e38f, ZB = -3.0e38f, ulx = 3.0e38f, uhx = -3.0e38f, uly = 3.0e38f, uhy = -3.0e38f;
    for (int b = 0; b < nI; ++b) {
        const float4 bc = js.bc[b], bh = js.bh[b];
        const float z0 = tabz[__float_as_int(bc.w) + S.M[2]] + bc.z;
        ZA = fminf(ZA, z0 - bh.z - rclc - 1.0e-4f);
        ZB = fmaxf(ZB, z0 + bh.z + rclc + 1.0e-4f);
        ulx = fminf(ulx, bc.x - bh.x); uhx = fmaxf(uhx, bc.x + bh.x);
        uly = fminf(uly, bc.y - bh.y); uhy = fmaxf(uhy, bc.y + bh.y);
    }
    const float Lz = S.Lf[2];
    const bool wholez = IMG || (ZB - ZA >= Lz);
    float za1 = fmaxf(ZA, 0.0f), zb1 = fminf(ZB, Lz), za2 = 1.0f, zb2 = 0.0f;  // empty 2nd piece
    if (ZA < 0.0f) { za2 = ZA + Lz; zb2 = Lz; }
    else if (ZB > Lz) { za2 = 0.0f; zb2 = ZB - Lz; }
    int mycnt = 0;   // lane b < nI: entries of member b so far
    for (int k0 = 0; k0 < S.hst_count; k0 += 32) {
        const int k = k0 + lane;
        int jb1 = 0, c1 = 0, jb2 = 0, c2 = 0;
        float Sx = 0.f, Sy = 0.f;
        bool own = false;
        if (k < S.hst_count) {
            const int2 off = a.stencil[S.hst_base + k];
            const int ccx = wrap_add(ref.x, off.x, S.M[0]);
            const int ccy = wrap_add(ref.y, off.y, S.M[1]);
            const int colid = ccx * S.M[1] + ccy;
            own = colid == ref.w;
            bool ok = S.half_geo ? true : (colid >= ref.w);
            Sx = tabx[wrap_cell(ccx - ref.x, S.M[0]) + S.M[0]];
            Sy = taby[wrap_cell(ccy - ref.y, S.M[1]) + S.M[1]];
            if (!IMG && ok) {
                // conservative xy gap between the members' union box and the column's slab
                const float lox = Sx - 1.0e-4f, hix = Sx + S.gf[0] + 1.0e-4f;
                const float loy = Sy - 1.0e-4f, hiy = Sy + S.gf[1] + 1.0e-4f;
                const float gx = fmaxf(0.0f, fmaxf(lox - uhx, ulx - hix));
                const float gy = fmaxf(0.0f, fmaxf(loy - uhy, uly - hiy));
                ok = gx * gx + gy * gy < rclc2;
            }
            if (ok) {
                int lo = colcl[colid];
                const int hi = colcl[colid + 1];
                if (own) lo = I0;  // own column: clusters J >= I0 (each member: J >= its own index)
                if (wholez) {
                    jb1 = lo;
                    c1 = hi - lo;
                } else {
                    jb1 = lower_zhi(zb, lo, hi, za1);
                    c1 = upper_zlo(zb, jb1, hi, zb1) - jb1;
                    if (za2 <= zb2) {
                        jb2 = lower_zhi(zb, lo, hi, za2);
                        c2 = upper_zlo(zb, jb2, hi, zb2) - jb2;
                        // the two pieces are disjoint in z; clusters are counted once
                        if (jb2 < jb1 + c1 && jb2 + c2 > jb1) {
                            const int u0 = min(jb1, jb2), u1 = max(jb1 + c1, jb2 + c2);
                            jb1 = u0; c1 = u1 - u0; c2 = 0;
                        }
                    }
                }
                c1 = max(c1, 0);
                c2 = max(c2, 0);
            }
        }
        // the columns' candidate ranges (up to two per lane) in lane order, then
        // the candidates flattened over all lanes: every lane takes one per round
        const bool h1 = c1 > 0, h2 = c2 > 0;
        const unsigned hb1 = __ballot_sync(0xffffffffu, h1), hb2 = __ballot_sync(0xffffffffu, h2);
        int incl = c1 + c2;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        {
            const unsigned lt = (1u << lane) - 1u;
            const int ri = __popc(hb1 & lt) + __popc(hb2 & lt);
            const int ob = own ? (int)0x80000000 : 0;
            if (h1) js.rng[ri] = make_int4(jb1 | ob, incl - c1 - c2, __float_as_int(Sx), __float_as_int(Sy));
            if (h2) js.rng[ri + (h1 ? 1 : 0)] = make_int4(jb2 | ob, incl - c2, __float_as_int(Sx), __float_as_int(Sy));
        }
        const int nr = __popc(hb1) + __popc(hb2);
        __syncwarp();
        for (int e0 = 0; e0 < total; e0 += 32) {
            const int e = e0 + lane;
            int J = 0, czj = 0;
            bool inr = false, ownc = false;
            float cSx = 0.f, cSy = 0.f;
            float4 cj = make_float4(0.f, 0.f, 0.f, 0.f), hjb = cj;
            if (e < total) {
                int lo = 0, hi = nr - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (js.rng[mid].y <= e) lo = mid; else hi = mid - 1;
                }
                const int4 rg = js.rng[lo];
                J = (rg.x & 0x7fffffff) + (e - rg.y);
                ownc = rg.x < 0;
                cSx = __int_as_float(rg.z);
                cSy = __int_as_float(rg.w);
                const int jw = R.cl_win + J;
                cj = a.cl_bbc[jw];
                hjb = a.cl_bbh[jw];
                czj = __float_as_int(cj.w);
                inr = true;
            }
#pragma unroll 1
            for (int b = 0; b < nI; ++b) {
                const int I = I0 + b;
                const float4 bc = js.bc[b], bh = js.bh[b];
                bool pass = false;
                int4 en = make_int4(0, 0, 0, 0);
                if (inr && (!ownc || J >= I)) {
                    const float sz = tabz[wrap_cell(czj - __float_as_int(bc.w), S.M[2]) + S.M[2]];
                    float dx = cj.x + cSx - bc.x, dy = cj.y + cSy - bc.y, dz = cj.z + sz - bc.z;
                    if (IMG) {
                        dx = img32(dx, S.Lf[0], S.invLf[0]);
                        dy = img32(dy, S.Lf[1], S.invLf[1]);
                        dz = img32(dz, S.Lf[2], S.invLf[2]);
                    }
                    const float gx = fmaxf(fabsf(dx) - bh.x - hjb.x, 0.0f);
                    const float gy = fmaxf(fabsf(dy) - bh.y - hjb.y, 0.0f);
                    const float gz = fmaxf(fabsf(dz) - bh.z - hjb.z, 0.0f);
                    pass = gx * gx + gy * gy + gz * gz < rclc2;
                    const int4 lkA = js.lk[b][0], lkB = js.lk[b][1];
                    // clusters sharing an exclusion with I: the relation is symmetric,
                    // so I's own (complete unless -2) partner list decides every J
                    const bool nm = (J == I) || lkA.x == -2 || lkA.x == J || lkA.y == J || lkA.z == J ||
                                    lkA.w == J || lkB.x == J || lkB.y == J || lkB.z == J || lkB.w == J;
                    en = make_int4(J | (nm ? (int)0x80000000 : 0), __float_as_int(cSx), __float_as_int(cSy),
                                   __float_as_int(sz));
                }
                const unsigned bal = __ballot_sync(0xffffffffu, pass);
                const int base = __shfl_sync(0xffffffffu, mycnt, b);
                if (pass) {
                    const int pos = base + __popc(bal & ((1u << lane) - 1u));
                    if (pos < a.jl_cap) a.jl[(size_t)(cw0 + b) * a.jl_cap + pos] = en;
                }
                if (lane == b) mycnt += __popc(bal);
            }
        }
        __syncwarp();   // rng is rewritten by the next stencil round
    }
    if (lane < nI) {
        a.jl_cnt[cw0 + lane] = mycnt;
        if (mycnt > a.jl_cap) atomicOr(a.status, SDM_DEV_LIST_OVERFLOW);
    }
    __syncwarp();   // js is rewritten by the warp's next group
}

// DYN: every warp takes groups from a per-call counter until none is left
// (warps that finish early take more; the launch ends with the last group,
// not the last of a fixed share).  Otherwise warp w builds groups w, w + W,
// ... (no counter round trip; the host picks this form when there are about
// as many groups as warps).  Both build the same lists.
__device__ __forceinline__ int next_group(const SdmArgs& a) {
    int g = 0;
    if (lane_id() == 0) g = atomicAdd(&a.work_counter[0], 1);
    return __shfl_sync(0xffffffffu, g, 0);
}

template <bool DYN>
__global__ void __launch_bounds__(256, 4) k_jlist(SdmArgs a, const int* grp_prefix) {
    __shared__ JlSmem js_all[8];
    JlSmem& js = js_all[threadIdx.x >> 5];
    const int total = grp_prefix[a.nrep];
    const int W = DYN ? 0 : gridDim.x * (blockDim.x >> 5);
    for (int item = DYN ? next_group(a) : blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); item < total;
         item = DYN ? next_group(a) : item + W) {
        const int r = rep_by_item(grp_prefix, a.nrep, item);
        const int g = item - grp_prefix[r];
        if (replica_image_mode(a, a.sys[a.rep[r].sys], r)) build_jlist<true>(a, r, g, js);
        else build_jlist<false>(a, r, g, js);
    }
}

// ------------------------------------------------------------------------- //
// K6b: main pass                                                            //
// ------------------------------------------------------------------------- //

// One tile of 32 j (one per lane) against the 8 i of the cluster (warp-
// uniform i, packed FP32x2 over i pairs).  MASKED: the lane's allowed-i bits
// m apply; otherwise every i is allowed.  Out-of-range pairs are removed by
// one select of r^2 to +inf per pair (rsqrt gives 0, and every force and
// Lennard-Jones term carries a factor 1/r^2) and one select of the charge
// product for the reaction-field or Ewald energy; the pair rule is the FP32
// r^2 of these roundings below the FP32 cutoff square.  LJ = false: the j
// have epsilon = 0 (Coulomb only).  Inactive lanes add no j force or energy.
template <int MODE, bool IMG, bool PME, bool MASKED, bool LJ = true>
__device__ __forceinline__ void pair_tile(const SdmArgs& a, const SdmSys& S, const SdmRep& R, const IPar3& ip,
                                           const float4& A, float hj_s, float ej_s, unsigned m, bool active,
                                           int slot, ICluster& ic, float& ef, long long& npair) {
    const float2 xs = make_float2(A.x, A.x), ys = make_float2(A.y, A.y), zs = make_float2(A.z, A.z);
    const float2 qj = make_float2(A.w, A.w), hj = make_float2(hj_s, hj_s), ej = make_float2(ej_s, ej_s);
    const float rc2 = S.rc2f;
    const float inf = __int_as_float(0x7f800000);
    const float2 krf = make_float2(S.krf, S.krf), ncrf = make_float2(-S.crf, -S.crf);
    const float2 krf2 = make_float2(-2.0f * S.krf, -2.0f * S.krf);
    const float2 one_n = make_float2(-1.0f, -1.0f), c12 = make_float2(12.0f, 12.0f),
                 c6n = make_float2(-6.0f, -6.0f);
    float2 fjx = make_float2(0.f, 0.f), fjy = fjx, fjz = fjx, e = fjx;
    int cnt = 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const float4 pa = ip.a[u], pb = ip.b[u], pc = ip.c[u];
        float2 dx = __fadd2_rn(xs, make_float2(pb.z, pb.w));
        float2 dy = __fadd2_rn(ys, make_float2(pc.x, pc.y));
        float2 dz = __fadd2_rn(zs, make_float2(pc.z, pc.w));
        if (IMG) {
            dx = make_float2(img32(dx.x, S.Lf[0], S.invLf[0]), img32(dx.y, S.Lf[0], S.invLf[0]));
            dy = make_float2(img32(dy.x, S.Lf[1], S.invLf[1]), img32(dy.y, S.Lf[1], S.invLf[1]));
            dz = make_float2(img32(dz.x, S.Lf[2], S.invLf[2]), img32(dz.y, S.Lf[2], S.invLf[2]));
        }
        const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        bool ok0 = r2.x < rc2, ok1 = r2.y < rc2;
        if (MASKED) {
            ok0 = ok0 && ((m >> (2 * u)) & 1u);
            ok1 = ok1 && ((m >> (2 * u + 1)) & 1u);
        }
        if (MODE == MODE_COUNT) {
            cnt += (ok0 ? 1 : 0) + (ok1 ? 1 : 0);
            continue;
        }
        const float2 ir = make_float2(fast_rsqrt(ok0 ? r2.x : inf), fast_rsqrt(ok1 ? r2.y : inf));
        const float2 ir2 = __fmul2_rn(ir, ir);
        const float2 qq = __fmul2_rn(make_float2(pa.x, pa.y), qj);
        const float2 qqe = make_float2(ok0 ? qq.x : 0.0f, ok1 ? qq.y : 0.0f);
        float2 fc;
        if (PME) {
            const float2 xb = __fmul2_rn(__fmul2_rn(r2, ir), make_float2(S.beta_f, S.beta_f));
            const float2 gx = make_float2(__expf(-xb.x * xb.x), __expf(-xb.y * xb.y));
            const float2 eci = __fmul2_rn(__fmul2_rn(erfc_scaled2(xb), gx), ir);
            fc = __fmul2_rn(qq, __ffma2_rn(make_float2(S.c2_f, S.c2_f), gx, eci));
            e = __ffma2_rn(qqe, eci, e);
        } else {
            fc = __fmul2_rn(qq, __ffma2_rn(krf2, r2, ir));
            e = __ffma2_rn(qqe, __ffma2_rn(krf, r2, __fadd2_rn(ir, ncrf)), e);
        }
        float2 fs;
        if (LJ) {
            const float2 sg = __fadd2_rn(make_float2(pa.z, pa.w), hj);
            const float2 s2 = __fmul2_rn(__fmul2_rn(sg, sg), ir2);
            const float2 s6 = __fmul2_rn(__fmul2_rn(s2, s2), s2);
            const float2 t6 = __fmul2_rn(__fmul2_rn(make_float2(pb.x, pb.y), ej), s6);
            e = __ffma2_rn(t6, __fadd2_rn(s6, one_n), e);
            fs = __fmul2_rn(__ffma2_rn(t6, __ffma2_rn(c12, s6, c6n), fc), ir2);
        } else {
            fs = __fmul2_rn(fc, ir2);   // j with epsilon = 0: Coulomb only
        }
        fjx = __ffma2_rn(fs, dx, fjx);
        fjy = __ffma2_rn(fs, dy, fjy);
        fjz = __ffma2_rn(fs, dz, fjz);
        ic.ax[u] = __ffma2_rn(fs, dx, ic.ax[u]);
        ic.ay[u] = __ffma2_rn(fs, dy, ic.ay[u]);
        ic.az[u] = __ffma2_rn(fs, dz, ic.az[u]);
    }
    if (MODE == MODE_COUNT) {
        npair += cnt;
    } else if (active) {
        const float gx = __fadd_rn(fjx.x, fjx.y), gy = __fadd_rn(fjy.x, fjy.y), gz = __fadd_rn(fjz.x, fjz.y);
        const size_t gsl = (size_t)R.slot_win + slot;
        if (!(fmaxf(fabsf(gx), fmaxf(fabsf(gy), fabsf(gz))) < 1.0e9f)) atomicOr(a.status, SDM_DEV_FORCE_OVERFLOW);
        atomicAdd(a.F0x + gsl, fix64(gx));
        atomicAdd(a.F0y + gsl, fix64(gy));
        atomicAdd(a.F0z + gsl, fix64(gz));
        ef += __fadd_rn(e.x, e.y);
    }
}

// One tile of a ring: every lane owns one j of the ring window [head,
// head+count) and sweeps the 8 i-particles of the cluster.  LJ = false is the
// ring of j with epsilon = 0: Lennard-Jones vanishes for every i, Coulomb only.
template <int MODE, bool IMG, bool LJ, bool PME>
__device__ __forceinline__ void eval_tile(const SdmArgs& a, const SdmSys& S, const SdmRep& R,
                                          const Ring& rg, const IPar3& ip, unsigned head, int count,
                                          ICluster& ic, float& ef, long long& npair) {
    const int lane = lane_id();
    const unsigned idx = (head + lane) & (SDM_RING - 1);
    const bool active = lane < count;
    // inactive lanes use zeros, never stale ring contents, and allow no i
    const float4 A = active ? rg.a[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 B = active ? rg.b[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned m = active ? __float_as_uint(B.z) : 0u;
    pair_tile<MODE, IMG, PME, true, LJ>(a, S, R, ip, A, B.x, B.y, m, active, __float_as_int(B.w), ic, ef, npair);
}

// The remainders of both rings at the end of an i-cluster in one tile when
// they fit: lanes < nl take the LJ ring's entries, the next nc the Coulomb
// ring's, all through the Lennard-Jones tile (epsilon = 0 makes its LJ terms
// add exactly zero, so those pairs' forces are the Coulomb tile's bits).
template <int MODE, bool IMG, bool PME, int CH>
__device__ __forceinline__ void eval_tile_both(const SdmArgs& a, const SdmSys& S, const SdmRep& R,
                                               const EvalSmem<CH>& sm, unsigned hl, int nl, unsigned hc, int nc,
                                               ICluster& ic, float& ef, long long& npair) {
    const int lane = lane_id();
    const bool fromlj = lane < nl;
    const Ring& rg = fromlj ? sm.lj : sm.co;
    const unsigned idx = (fromlj ? hl + lane : hc + (lane - nl)) & (SDM_RING - 1);
    const bool active = lane < nl + nc;
    const float4 A = active ? rg.a[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 B = active ? rg.b[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned m = active ? __float_as_uint(B.z) : 0u;
    pair_tile<MODE, IMG, PME, true, true>(a, S, R, sm.ip, A, B.x, B.y, m, active, __float_as_int(B.w), ic, ef, npair);
}

// Computes the allowed-i mask of candidate slot j (cluster J) against
// i-cluster I (valid-i bits vmask).
__device__ __forceinline__ unsigned j_mask(const SdmArgs& a, const SdmSys& S, const SdmRep& R,
                                           int I, int J, int sj, unsigned vmask, bool needmask) {
    unsigned m = vmask;
    if (!needmask) return m;
    const int t = sj & 7;
    if (J == I) m &= (1u << t) - 1u;
    const int4 ex = a.excl4[R.slot_win + sj];
    const int i0 = 8 * I;
    if (ex.x == -2) {
        const int p = a.perm[R.slot_win + sj];
        const int ta = S.atom_base + p;
        for (int k = a.excl_off[ta]; k < a.excl_off[ta + 1]; ++k) {
            const int s2 = a.inv[R.atom_win + a.excl_idx[k]];
            if (s2 >= i0 && s2 < i0 + 8) m &= ~(1u << (s2 - i0));
        }
    } else {
        const int e4[4] = {ex.x, ex.y, ex.z, ex.w};
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (e4[k] >= i0 && e4[k] < i0 + 8) m &= ~(1u << (e4[k] - i0));
    }
    return m;
}

// reduce-scatter of the 24 i-force partial sums of a warp; lanes 0,4,..,28
// add the i forces (allowed by vmask) into the fixed-point accumulators
__device__ __forceinline__ void reduce_i_forces(const SdmArgs& a, const ICluster& ic, unsigned vmask, int slot0) {
    const int lane = lane_id();
    float v[24];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        v[6 * u] = -ic.ax[u].x; v[6 * u + 1] = -ic.ay[u].x; v[6 * u + 2] = -ic.az[u].x;
        v[6 * u + 3] = -ic.ax[u].y; v[6 * u + 4] = -ic.ay[u].y; v[6 * u + 5] = -ic.az[u].y;
    }
    {
        const bool up = lane & 16;
#pragma unroll
        for (int k = 0; k < 12; ++k) {
            const float send = up ? v[k] : v[k + 12];
            const float keep = up ? v[k + 12] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
        }
    }
    {
        const bool up = lane & 8;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float send = up ? v[k] : v[k + 6];
            const float keep = up ? v[k + 6] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
    }
    {
        const bool up = lane & 4;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float send = up ? v[k] : v[k + 3];
            const float keep = up ? v[k + 3] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v[k] += __shfl_xor_sync(0xffffffffu, v[k], 2);
        v[k] += __shfl_xor_sync(0xffffffffu, v[k], 1);
    }
    if ((lane & 3) == 0) {
        const int ti = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
        if ((vmask >> ti) & 1u) {
            const size_t gsl = (size_t)slot0 + ti;
            red_fix(a.F0x + gsl, v[0], a.status);
            red_fix(a.F0y + gsl, v[1], a.status);
            red_fix(a.F0z + gsl, v[2], a.status);
        }
    }
}

template <int MODE, bool IMG, bool PME, int SDM_CH>
__device__ void process_cluster(const SdmArgs& a, int r, int I, int part, EvalSmem<SDM_CH>& sm) {
    const int lane = lane_id();
    const SdmRep R = a.rep[r];
    const SdmSys S = a.sys[R.sys];
    const int cw = R.cl_win + I;
    const int slot0 = R.slot_win + 8 * I;
    // i-cluster particles, replicated in every lane
    ICluster ic;
    {
        float4 xi4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 pi2 = make_float2(0.f, 0.f);
        if (lane < 8) { xi4 = a.clX[slot0 + lane]; pi2 = a.clP[slot0 + lane]; }
        __syncwarp();
        if (lane < 8) {
            const int u = lane >> 1, h = lane & 1;
            reinterpret_cast<float*>(&sm.ip.a[u])[h] = xi4.w;
            reinterpret_cast<float*>(&sm.ip.a[u])[2 + h] = pi2.x;
            reinterpret_cast<float*>(&sm.ip.b[u])[h] = pi2.y;
            reinterpret_cast<float*>(&sm.ip.b[u])[2 + h] = -xi4.x;
            reinterpret_cast<float*>(&sm.ip.c[u])[h] = -xi4.y;
            reinterpret_cast<float*>(&sm.ip.c[u])[2 + h] = -xi4.z;
            sm.im[lane] = a.clM[slot0 + lane];
        }
        if (lane == 0) {
            float4 c = a.cl_bbc[cw], h = a.cl_bbh[cw];
            h.w = S.rcl2f;
            sm.ib[0] = c;
            sm.ib[1] = h;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            ic.ax[u] = make_float2(0.f, 0.f); ic.ay[u] = ic.ax[u]; ic.az[u] = ic.ax[u];
        }
        __syncwarp();
    }
    const unsigned vmask = __ballot_sync(0xffffffffu, lane < 8 && a.perm[slot0 + (lane & 7)] >= 0) & 0xffu;
    const int njl = min(a.jl_cnt[cw], a.jl_cap);
    const int ebeg = (njl * part) / a.split, eend = (njl * (part + 1)) / a.split;
    const int4* jl = a.jl + (size_t)cw * a.jl_cap;

    unsigned hl = 0, tl = 0, hc = 0, tc = 0;  // ring counters (uniform)
    float ef = 0.0f;
    long long npair = 0;
    int emit_n = 0;
    const int t = lane & 7, q = lane >> 3;

    const int nent = eend - ebeg;
    const int nchunk = (nent + SDM_CH - 1) / SDM_CH;
    // lanes 0..15 copy one list entry each
    auto issue_entries = [&](int c) {
        if (c < nchunk && lane < SDM_CH) {
            const int e = ebeg + c * SDM_CH + lane;
            if (e < eend) cp_async16(&sm.je[c % 3][lane], jl + e);
        }
    };
    // 128 candidate particles of chunk c: lane copies particles lane, lane+32, lane+64, lane+96
    auto issue_atoms = [&](int c) {
        if (c >= nchunk) return;
        const int nch = min(SDM_CH, eend - (ebeg + c * SDM_CH));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int idx = lane + 32 * k;
            const int e = idx >> 3;
            if (e < nch) {
                const int sj = 8 * (sm.je[c % 3][e].x & 0x7fffffff) + (idx & 7);
                cp_async16(&sm.sx[c & 1][idx], a.clX + R.slot_win + sj);
                cp_async8(&sm.sp[c & 1][idx], a.clP + R.slot_win + sj);
                if (S.excl_clique) cp_async4(&sm.sm_[c & 1][idx], a.clM + R.slot_win + sj);
            }
        }
    };
    issue_entries(0);
    cp_async_commit();
    issue_entries(1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    issue_atoms(0);
    cp_async_commit();
    for (int c = 0; c < nchunk; ++c) {
        issue_entries(c + 2);
        cp_async_commit();
        cp_async_wait<1>();   // entries of c+1 and particles of c have landed (this lane)
        __syncwarp();         // ... and for every lane
        issue_atoms(c + 1);
        cp_async_commit();
        const int nch = min(SDM_CH, eend - (ebeg + c * SDM_CH));
        for (int g = 0; g < SDM_CH / 4; ++g) {
            const int e = 4 * g + q;   // entry of this lane's 8-lane group
            if (4 * g >= nch) break;   // uniform
            // lanes past the chunk's last entry read that entry (initialised
            // staging) and are dropped by `valid`: straight-line code for all lanes
            const bool valid = e < nch;
            const int ee = valid ? e : nch - 1;
            const int4 en = sm.je[c % 3][ee];
            const float4 X4 = sm.sx[c & 1][8 * ee + t];
            const float2 P = sm.sp[c & 1][8 * ee + t];
            const int J = en.x & 0x7fffffff;
            const bool nm = en.x < 0;
            const int sj = 8 * J + t;
            const float xs = __fadd_rn(X4.x, __int_as_float(en.y));
            const float ys = __fadd_rn(X4.y, __int_as_float(en.z));
            const float zs = __fadd_rn(X4.z, __int_as_float(en.w));
            bool pass;
            {
                const float4 bc = sm.ib[0], bh = sm.ib[1];   // re-read: keeps registers free
                float tx = __fsub_rn(xs, bc.x), ty = __fsub_rn(ys, bc.y), tz = __fsub_rn(zs, bc.z);
                if (IMG) {
                    tx = img32(tx, S.Lf[0], S.invLf[0]);
                    ty = img32(ty, S.Lf[1], S.invLf[1]);
                    tz = img32(tz, S.Lf[2], S.invLf[2]);
                }
                const float ex = fmaxf(__fsub_rn(fabsf(tx), bh.x), 0.0f);
                const float ey = fmaxf(__fsub_rn(fabsf(ty), bh.y), 0.0f);
                const float ez = fmaxf(__fsub_rn(fabsf(tz), bh.z), 0.0f);
                // padding slots carry 1e6 coordinates: they fail the box test
                // unless image mode wraps them back, hence the explicit test there
                pass = valid && r2_chain(ex, ey, ez) < bh.w;
                if (IMG) pass = pass && (X4.x < 1.0e5f);
            }
            unsigned m = vmask;
            if (S.excl_clique) {
                // excluded <=> same molecule: compare with the 8 i ids (uniform branch)
                if (__any_sync(0xffffffffu, pass && nm)) {
                    const int mj = sm.sm_[c & 1][8 * ee + t];
                    unsigned mm = vmask & ((J == I) ? ((1u << t) - 1u) : 0xffu);
#pragma unroll
                    for (int u = 0; u < 8; ++u) mm = (sm.im[u] == mj) ? (mm & ~(1u << u)) : mm;
                    m = nm ? mm : vmask;
                }
                pass = pass && m != 0u;
            } else if (pass) {
                m = j_mask(a, S, R, I, J, sj, vmask, nm);
                pass = m != 0u;
            }
            if (MODE == MODE_EMIT) {
                const unsigned bal = __ballot_sync(0xffffffffu, pass);
                const int pos = __popc(bal & ((1u << lane) - 1u));
                if (pass && emit_n + pos < a.ex_cap) {
                    const size_t o = (size_t)I * a.ex_cap + emit_n + pos;
                    a.ex_slot[o] = sj;
                    a.ex_mask[o] = (unsigned char)m;
                }
                emit_n += __popc(bal);
                continue;
            }
            const bool lj = pass && P.y != 0.0f;
            const bool co = pass && P.y == 0.0f;
            const unsigned bl = __ballot_sync(0xffffffffu, lj);
            const unsigned bco = __ballot_sync(0xffffffffu, co);
            const unsigned lt = (1u << lane) - 1u;
            if (lj) {
                const unsigned idx = (tl + __popc(bl & lt)) & (SDM_RING - 1);
                sm.lj.a[idx] = make_float4(xs, ys, zs, X4.w);
                sm.lj.b[idx] = make_float4(P.x, P.y, __uint_as_float(m), __int_as_float(sj));
            }
            if (co) {
                const unsigned idx = (tc + __popc(bco & lt)) & (SDM_RING - 1);
                sm.co.a[idx] = make_float4(xs, ys, zs, X4.w);
                sm.co.b[idx] = make_float4(P.x, P.y, __uint_as_float(m), __int_as_float(sj));
            }
            tl += __popc(bl);
            tc += __popc(bco);
            __syncwarp();
            if (tl - hl >= 32u) {
                eval_tile<MODE, IMG, true, PME>(a, S, R, sm.lj, sm.ip, hl, 32, ic, ef, npair);
                hl += 32u;
            }
            if (tc - hc >= 32u) {
                eval_tile<MODE, IMG, false, PME>(a, S, R, sm.co, sm.ip, hc, 32, ic, ef, npair);
                hc += 32u;
            }
            __syncwarp();
        }
    }
    cp_async_wait<0>();
    __syncwarp();
    if (MODE == MODE_EMIT) {
        if (lane == 0 && part == 0) {
            a.ex_cnt[I] = emit_n;
            if (emit_n > a.ex_cap) atomicOr(a.status, 1 << 16);
        }
        return;
    }
    const int nl = (int)(tl - hl), nc = (int)(tc - hc);
    if (nl > 0 && nc > 0 && nl + nc <= 32) {
        eval_tile_both<MODE, IMG, PME>(a, S, R, sm, hl, nl, hc, nc, ic, ef, npair);
    } else {
        if (nl > 0) eval_tile<MODE, IMG, true, PME>(a, S, R, sm.lj, sm.ip, hl, nl, ic, ef, npair);
        if (nc > 0) eval_tile<MODE, IMG, false, PME>(a, S, R, sm.co, sm.ip, hc, nc, ic, ef, npair);
    }
    if (MODE == MODE_COUNT) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) npair += __shfl_xor_sync(0xffffffffu, npair, o);
        if (lane == 0) atomicAdd((unsigned long long*)&a.counts[2 * r], (unsigned long long)npair);
        return;
    }
    reduce_i_forces(a, ic, vmask, slot0);
    double ed = (double)ef;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ed += __shfl_xor_sync(0xffffffffu, ed, o);
    if (lane == 0) a.e_part[(size_t)cw * a.split + part] = ed;
}

// NW warps per CTA, each with its own EvalSmem in dynamic shared memory;
// MINB CTAs per SM fit the register file: registers per thread are capped at
// 65536 / (MINB * NW * 32), rounded down to the allocation unit of 8
template <int MODE, int MINB, int NW, bool PME = false, int CH = SDM_CH_DEFAULT>
__global__ void __launch_bounds__(NW * 32) __maxnreg__((65536 / (MINB * NW * 32)) & ~7)
k_pair(SdmArgs a, const int* item_prefix) {
    extern __shared__ __align__(16) unsigned char pair_smem[];
    EvalSmem<CH>& sm = reinterpret_cast<EvalSmem<CH>*>(pair_smem)[threadIdx.x >> 5];
    const int total = item_prefix[a.nrep];
    // dynamic schedule: each warp takes the next item from a counter (zeroed
    // at the start of every evaluation), so CTAs that become resident late
    // (other branches of the graph still running) just take fewer items
    for (;;) {
        int item = 0;
        if (lane_id() == 0) item = atomicAdd(&a.work_counter[2], 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        const int r = rep_by_item(item_prefix, a.nrep, item);
        const int local = item - item_prefix[r];
        const int I = local / a.split, part = local - I * a.split;
        if (MODE == MODE_EMIT && r != a.ex_rep) continue;
        if (replica_image_mode(a, a.sys[a.rep[r].sys], r)) process_cluster<MODE, true, PME, CH>(a, r, I, part, sm);
        else process_cluster<MODE, false, PME, CH>(a, r, I, part, sm);
    }
}

// ------------------------------------------------------------------------- //
// K7: perturbation pass                                                     //
// ------------------------------------------------------------------------- //
__device__ __forceinline__ void pair_terms(const SdmSys& S, float r2, float qq, float sg, float eps4,
                                           float& e, float& fs) {
    const float ir = fast_rsqrt(r2);
    const float ir2 = ir * ir;
    const float s2 = sg * sg * ir2;
    const float s6 = s2 * s2 * s2;
    const float t6 = eps4 * s6;
    if (S.pme) {   // Ewald direct space
        const float xb = r2 * ir * S.beta_f;
        const float gx = __expf(-xb * xb);
        const float ec = erfc_scaled(xb) * gx * ir;
        e = fmaf(t6, s6 - 1.0f, qq * ec);
        fs = fmaf(t6, fmaf(12.0f, s6, -6.0f), qq * fmaf(S.c2_f, gx, ec)) * ir2;
        return;
    }
    e = fmaf(t6, s6 - 1.0f, qq * fmaf(S.krf, r2, ir - S.crf));
    fs = fmaf(t6, fmaf(12.0f, s6, -6.0f), qq * fmaf(-2.0f * S.krf, r2, ir)) * ir2;
}

// Position of every perturbation item's displaced particle in its state:
// y = wrap(w + st d), its cell and cell-local FP32 coordinates (one thread per item)
__global__ void k_pert_prep(SdmArgs a) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= a.total_pert) return;
    const int r = rep_by_pert(a.rep, a.nrep, item);
    const SdmRep R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int local = item - R.pert_win;
    const int pidx = local >> 1, st = local & 1;
    const int p = a.D_idx[S.D_base + pidx];
    const int tp = S.atom_base + p;
    const double* wp = a.w + 3 * (size_t)(R.atom_win + p);
    SdmPertPos pp;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double v = st ? __dadd_rn(wp[k], a.topo_d[3 * (size_t)tp + k]) : wp[k];
        pp.y[k] = wrap1(v, S.box[k], S.invL[k]);
        pp.cy[k] = cell_of(pp.y[k], S.invg[k], S.M[k]);
        pp.o[k] = __double2float_rn(__dsub_rn(pp.y[k], __dmul_rn((double)pp.cy[k], S.g[k])));
    }
    a.pert_pos[item] = pp;
}

template <int MODE, bool IMG>
__device__ void process_perturb(const SdmArgs& a, int r, int local, int part, WarpSmem& sm) {
    const int lane = lane_id();
    const SdmRep R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int pidx = local >> 1, st = local & 1;
    const float sgn = st ? 1.0f : -1.0f;
    const int p = a.D_idx[S.D_base + pidx];
    const int tp = S.atom_base + p;
    const int gp = a.topo_grp[tp];
    // position of the displaced particle in this state (computed once per item by k_pert_prep)
    const SdmPertPos pp = a.pert_pos[R.pert_win + local];
    const double y[3] = {pp.y[0], pp.y[1], pp.y[2]};
    const int cy[3] = {pp.cy[0], pp.cy[1], pp.cy[2]};
    const float o[3] = {pp.o[0], pp.o[1], pp.o[2]};
    const float qp = a.topo_q[tp], hp = a.topo_hs[tp], sp_ = a.topo_se[tp];
    const int cxb = a.cx_off[S.cx_base + pidx], cxe = a.cx_off[S.cx_base + pidx + 1];
    const float rclc = S.rcl + 2.0e-4f;
    const float rclc2 = rclc * rclc;
    const float* tabx = a.shift_tab + S.shift_base;
    const float* taby = tabx + 2 * S.M[0] + 1;
    const float* tabz = taby + 2 * S.M[1] + 1;
    const int nst = S.fst_count;
    const int* colcl = a.col_cl + R.col_win;
    // energy as an unevaluated float-float sum es + ec (TwoSum on the FP32
    // pipe): FP64-level accuracy without per-pair work on the narrow FP64 pipe
    float es = 0.f, ec = 0.f;
    auto acc = [&](float v) {
        const float t = __fadd_rn(es, v);
        const float bp = __fsub_rn(t, es);
        ec = __fadd_rn(ec, __fadd_rn(__fsub_rn(es, __fsub_rn(t, bp)), __fsub_rn(v, bp)));
        es = t;
    };
    float fpx = 0.f, fpy = 0.f, fpz = 0.f;
    long long npair = 0;
    int jl_n = 0;

    auto eval_j = [&](float dx, float dy, float dz, float r2, float qj, float hj, float ej, int sj) {
        float e, fs;
        pair_terms(S, r2, qp * qj, hp + hj, sp_ * ej, e, fs);
        acc(sgn * e);
        const float f = sgn * fs;
        if (sj >= 0) {
            const size_t gsl = (size_t)R.slot_win + sj;
            red_fix(a.dFx + gsl, f * dx, a.status);
            red_fix(a.dFy + gsl, f * dy, a.status);
            red_fix(a.dFz + gsl, f * dz, a.status);
        }
        fpx = fmaf(-f, dx, fpx);
        fpy = fmaf(-f, dy, fpy);
        fpz = fmaf(-f, dz, fpz);
    };

    auto phase_b = [&]() {
        for (int g0 = 0; g0 < jl_n; g0 += 4) {
            const int e = g0 + (lane >> 3);
            if (e < jl_n) {
                const int4 en = sm.jl[e];
                const int sj = 8 * en.x + (lane & 7);
                const size_t gsl = (size_t)R.slot_win + sj;
                const float4 X4 = a.clX[gsl];
                float dx = __fsub_rn(__fadd_rn(X4.x, __int_as_float(en.y)), o[0]);
                float dy = __fsub_rn(__fadd_rn(X4.y, __int_as_float(en.z)), o[1]);
                float dz = __fsub_rn(__fadd_rn(X4.z, __int_as_float(en.w)), o[2]);
                if (IMG) {
                    dx = img32(dx, S.Lf[0], S.invLf[0]);
                    dy = img32(dy, S.Lf[1], S.invLf[1]);
                    dz = img32(dz, S.Lf[2], S.invLf[2]);
                }
                const float r2 = r2_chain(dx, dy, dz);
                bool ok = (r2 < S.rc2f) && X4.x < 1.0e5f && a.grp[gsl] == 0;
                if (ok && cxe > cxb) {
                    const int pj = a.perm[gsl];
                    for (int k = cxb; k < cxe; ++k) ok = ok && (a.cx_idx[k] != pj);
                }
                if (ok) {
                    if (MODE == MODE_COUNT) npair += st;
                    else {
                        const float2 P = a.clP[gsl];
                        eval_j(dx, dy, dz, r2, X4.w, P.x, P.y, sj);
                    }
                }
            }
        }
        jl_n = 0;
    };

    // z window of the point (absolute, conservative) and its pieces inside [0, Lz):
    // particles of a column outside it are farther than the cutoff in z
    const float zq = __double2float_rn(y[2]);
    const float ZA = zq - rclc - 1.0e-4f, ZB = zq + rclc + 1.0e-4f;
    const float Lz = S.Lf[2];
    const bool wholez = IMG || (ZB - ZA >= Lz);
    float za1 = fmaxf(ZA, 0.0f), zb1 = fminf(ZB, Lz), za2 = 1.0f, zb2 = 0.0f;  // empty 2nd piece
    if (ZA < 0.0f) { za2 = ZA + Lz; zb2 = Lz; }
    else if (ZB > Lz) { za2 = 0.0f; zb2 = ZB - Lz; }
    // this part's share of the full stencil
    const int kb = (nst * part) / SDM_PERT_PARTS, ke = (nst * (part + 1)) / SDM_PERT_PARTS;
    for (int k0 = kb; k0 < ke; k0 += 32) {
        const int k = k0 + lane;
        int cntJ = 0, Jb = 0, cnt2 = 0, Jb2 = 0;
        float Sx = 0.f, Sy = 0.f;
        if (k < ke) {
            const int2 off = a.stencil[S.fst_base + k];
            const int ccx = wrap_add(cy[0], off.x, S.M[0]);
            const int ccy = wrap_add(cy[1], off.y, S.M[1]);
            const int colid = ccx * S.M[1] + ccy;
            Sx = tabx[wrap_cell(ccx - cy[0], S.M[0]) + S.M[0]];
            Sy = taby[wrap_cell(ccy - cy[1], S.M[1]) + S.M[1]];
            bool ok = true;
            if (!IMG) {
                const float lox = Sx - 1.0e-4f, hix = Sx + S.gf[0] + 1.0e-4f;
                const float loy = Sy - 1.0e-4f, hiy = Sy + S.gf[1] + 1.0e-4f;
                const float gx = fmaxf(0.0f, fmaxf(lox - o[0], o[0] - hix));
                const float gy = fmaxf(0.0f, fmaxf(loy - o[1], o[1] - hiy));
                ok = gx * gx + gy * gy < rclc2;
            }
            if (ok) {
                const int lo = colcl[colid], hi = colcl[colid + 1];
                if (wholez) {
                    Jb = lo;
                    cntJ = hi - lo;
                } else {
                    // the clusters holding the column's particles of the z cells
                    // that overlap the window (particles outside those cells are
                    // farther than the cutoff in z): cell offsets instead of
                    // binary searches over the cluster z bounds
                    const int* coff = a.cel_off + R.cel_win + colid * S.M[2];
                    const int a0 = a.col_aoff[R.col_win + colid];
                    const float ig = (float)S.invg[2];
                    auto crange = [&](float z0, float z1, int& jb, int& n) {
                        const int c0 = min(max(__float2int_rd((z0 - 1.0e-3f) * ig), 0), S.M[2] - 1);
                        const int c1 = min(max(__float2int_rd((z1 + 1.0e-3f) * ig), 0), S.M[2] - 1);
                        const int p0 = coff[c0] - a0, p1 = coff[c1 + 1] - a0;
                        jb = lo + (p0 >> 3);
                        n = p1 > p0 ? ((p1 + 7) >> 3) - (p0 >> 3) : 0;
                    };
                    crange(za1, zb1, Jb, cntJ);
                    if (za2 <= zb2) {
                        crange(za2, zb2, Jb2, cnt2);
                        // the two pieces are disjoint in z; clusters are counted once
                        if (cnt2 > 0 && cntJ > 0 && Jb2 < Jb + cntJ && Jb2 + cnt2 > Jb) {
                            const int u0 = min(Jb, Jb2), u1 = max(Jb + cntJ, Jb2 + cnt2);
                            Jb = u0; cntJ = u1 - u0; cnt2 = 0;
                        }
                    }
                }
                cntJ = max(cntJ, 0);
                cnt2 = max(cnt2, 0);
            }
        }
        // up to two cluster ranges per column, in lane order
        const bool h1 = cntJ > 0, h2 = cnt2 > 0;
        const unsigned hb1 = __ballot_sync(0xffffffffu, h1), hb2 = __ballot_sync(0xffffffffu, h2);
        int incl = cntJ + cnt2;
#pragma unroll
        for (int oo = 1; oo < 32; oo <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, oo);
            if (lane >= oo) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        {
            const unsigned lt = (1u << lane) - 1u;
            const int ri = __popc(hb1 & lt) + __popc(hb2 & lt);
            if (h1) sm.rng[ri] = make_int4(Jb, incl - cntJ - cnt2, __float_as_int(Sx), __float_as_int(Sy));
            if (h2) sm.rng[ri + (h1 ? 1 : 0)] = make_int4(Jb2, incl - cnt2, __float_as_int(Sx), __float_as_int(Sy));
        }
        const int nr = __popc(hb1) + __popc(hb2);
        __syncwarp();
        for (int e0 = 0; e0 < total; e0 += 32) {
            const int e = e0 + lane;
            bool pass = false;
            int4 en = make_int4(0, 0, 0, 0);
            if (e < total) {
                int lo = 0, hi = nr - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (sm.rng[mid].y <= e) lo = mid; else hi = mid - 1;
                }
                const int4 rg = sm.rng[lo];
                const int J = rg.x + (e - rg.y);
                const int jw = R.cl_win + J;
                const float4 cj = a.cl_bbc[jw];
                const float4 hjb = a.cl_bbh[jw];
                const float sz = tabz[wrap_cell(__float_as_int(cj.w) - cy[2], S.M[2]) + S.M[2]];
                const float sx = __int_as_float(rg.z), sy = __int_as_float(rg.w);
                float dx = cj.x + sx - o[0], dy = cj.y + sy - o[1], dz = cj.z + sz - o[2];
                if (IMG) {
                    dx = img32(dx, S.Lf[0], S.invLf[0]);
                    dy = img32(dy, S.Lf[1], S.invLf[1]);
                    dz = img32(dz, S.Lf[2], S.invLf[2]);
                }
                const float gx = fmaxf(fabsf(dx) - hjb.x, 0.0f);
                const float gy = fmaxf(fabsf(dy) - hjb.y, 0.0f);
                const float gz = fmaxf(fabsf(dz) - hjb.z, 0.0f);
                pass = gx * gx + gy * gy + gz * gz < rclc2;
                en = make_int4(J, __float_as_int(sx), __float_as_int(sy), __float_as_int(sz));
            }
            const unsigned bal = __ballot_sync(0xffffffffu, pass);
            if (pass) sm.jl[jl_n + __popc(bal & ((1u << lane) - 1u))] = en;
            jl_n += __popc(bal);
            __syncwarp();
            if (jl_n > SDM_JL_CAP - 32) phase_b();
            __syncwarp();
        }
    }
    phase_b();
    // displaced-displaced pairs with different displacement vectors (this part's share)
    const int qb = (S.nD * part) / SDM_PERT_PARTS, qe = (S.nD * (part + 1)) / SDM_PERT_PARTS;
    for (int q0 = qb; q0 < qe; q0 += 32) {
        const int qi = q0 + lane;
        if (qi < qe) {
            const int qa = a.D_idx[S.D_base + qi];
            const int tq = S.atom_base + qa;
            const int gq = a.topo_grp[tq];
            if (gq != gp && gq != 0 && qa > p) {
                const SdmPertPos& pq = a.pert_pos[R.pert_win + 2 * qi + st];
                float d[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double yq = pq.y[k];
                    double v = __dsub_rn(yq, y[k]);
                    const double tt = rint(__dmul_rn(v, S.invL[k]));
                    v = __dsub_rn(v, __dmul_rn(tt, S.box[k]));
                    d[k] = __double2float_rn(v);
                }
                const float r2 = r2_chain(d[0], d[1], d[2]);
                bool ok = r2 < S.rc2f;
                for (int k = cxb; k < cxe && ok; ++k) ok = (a.cx_idx[k] != qa);
                if (ok) {
                    if (MODE == MODE_COUNT) npair += st;
                    else eval_j(d[0], d[1], d[2], r2, a.topo_q[tq], a.topo_hs[tq], a.topo_se[tq],
                                a.inv[R.atom_win + qa]);
                }
            }
        }
    }
    if (MODE == MODE_COUNT) {
#pragma unroll
        for (int oo = 16; oo > 0; oo >>= 1) npair += __shfl_xor_sync(0xffffffffu, npair, oo);
        if (lane == 0 && npair) atomicAdd((unsigned long long*)&a.counts[2 * r + 1], (unsigned long long)npair);
        return;
    }
#pragma unroll
    for (int oo = 16; oo > 0; oo >>= 1) {
        fpx += __shfl_xor_sync(0xffffffffu, fpx, oo);
        fpy += __shfl_xor_sync(0xffffffffu, fpy, oo);
        fpz += __shfl_xor_sync(0xffffffffu, fpz, oo);
        const float os = __shfl_xor_sync(0xffffffffu, es, oo), oc = __shfl_xor_sync(0xffffffffu, ec, oo);
        acc(os);
        ec = __fadd_rn(ec, oc);
    }
    if (lane == 0) {
        const size_t gsl = (size_t)R.slot_win + a.inv[R.atom_win + p];
        red_fix(a.dFx + gsl, fpx, a.status);
        red_fix(a.dFy + gsl, fpy, a.status);
        red_fix(a.dFz + gsl, fpz, a.status);
        a.p_part[(size_t)(R.pert_win + local) * SDM_PERT_PARTS + part] = (double)es + (double)ec;
    }
}

template <int MODE>
__global__ void __launch_bounds__(SDM_WARPS * 32) k_perturb(SdmArgs a) {
    __shared__ WarpSmem smem[SDM_WARPS];
    WarpSmem& sm = smem[threadIdx.x >> 5];
    const int lane = lane_id();
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(&a.work_counter[1], 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= a.total_pert * SDM_PERT_PARTS) break;
        const int pi = item / SDM_PERT_PARTS, part = item - pi * SDM_PERT_PARTS;
        const int r = rep_by_pert(a.rep, a.nrep, pi);
        const int local = pi - a.rep[r].pert_win;
        const SdmSys& S = a.sys[a.rep[r].sys];
        if (replica_image_mode(a, S, r)) process_perturb<MODE, true>(a, r, local, part, sm);
        else process_perturb<MODE, false>(a, r, local, part, sm);
    }
}

// ------------------------------------------------------------------------- //
// Adjoint: parameter derivatives of U0 and U1 for the displaced particles   //
// ------------------------------------------------------------------------- //
struct AdjSmem {
    int4 jl[SDM_JL_CAP];
    int4 rng[64];
    int ex[128];                // exclusion partners of the particle (system-local)
};

__device__ __forceinline__ bool adj_excluded(const AdjSmem& sm, const SdmArgs& a, int eb, int ne, int j) {
    bool e = false;
    if (ne <= 128) {
        for (int k = 0; k < ne; ++k) e |= (sm.ex[k] == j);
    } else {
        for (int k = 0; k < ne; ++k) e |= (a.excl_idx[eb + k] == j);
    }
    return e;
}

// One adjoint item (replica, displaced particle, state) per warp: every
// partner of the particle in that state
template <bool IMG>
__device__ void process_adjoint(const SdmArgs& a, int r, int local, AdjSmem& sm) {
    const int lane = lane_id();
    const SdmRep R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int pidx = local >> 1, st = local & 1;
    const int p = a.D_idx[S.D_base + pidx];
    const int tp = S.atom_base + p;
    // the particle's position in this state, as the evaluation's k_pert_prep
    // computed it (the adjoint differentiates that evaluation)
    const SdmPertPos pp = a.pert_pos[R.pert_win + local];
    const double y[3] = {pp.y[0], pp.y[1], pp.y[2]};
    const int cy[3] = {pp.cy[0], pp.cy[1], pp.cy[2]};
    const float o[3] = {pp.o[0], pp.o[1], pp.o[2]};
    const float hp = a.topo_hs[tp], sp_ = a.topo_se[tp];
    const int eb = a.excl_off[tp], ne = a.excl_off[tp + 1] - eb;
    __syncwarp();
    for (int k = lane; k < ne && k < 128; k += 32) sm.ex[k] = a.excl_idx[eb + k];
    __syncwarp();
    const float rclc = S.rcl + 2.0e-4f;
    const float rclc2 = rclc * rclc;
    const float* tabx = a.shift_tab + S.shift_base;
    const float* taby = tabx + 2 * S.M[0] + 1;
    const float* tabz = taby + 2 * S.M[1] + 1;
    const int nst = S.fst_count;
    const int* colcl = a.col_cl + R.col_win;
    // z window of the point (absolute, conservative) and its pieces inside
    // [0, Lz): the clusters of a column outside it are beyond the cutoff
    const float2* zb = a.cl_zb + R.cl_win;
    const float zq = __double2float_rn(y[2]);
    const float ZA = zq - rclc - 1.0e-4f, ZB = zq + rclc + 1.0e-4f;
    const float Lz = S.Lf[2];
    const bool wholez = IMG || (ZB - ZA >= Lz);
    float za1 = fmaxf(ZA, 0.0f), zb1 = fminf(ZB, Lz), za2 = 1.0f, zb2 = 0.0f;  // empty 2nd piece
    if (ZA < 0.0f) { za2 = ZA + Lz; zb2 = Lz; }
    else if (ZB > Lz) { za2 = 0.0f; zb2 = ZB - Lz; }
    const float sqrtK = 11.787089759563214f;
    double gq = 0.0, gs = 0.0, ge = 0.0;
    int jl_n = 0;

    auto acc = [&](float r2, float qj, float hj, float ej) {
        const float ir = fast_rsqrt(r2), ir2 = ir * ir;
        const float phi = sqrtK * qj * fmaf(S.krf, r2, ir - S.crf);
        const float sg = hp + hj;
        const float s2 = sg * sg * ir2, s6 = s2 * s2 * s2, t6 = sp_ * ej * s6;
        const float elj = t6 * (s6 - 1.0f);
        const float dsg = sg > 0.0f ? 0.5f * t6 * fmaf(12.0f, s6, -6.0f) / sg : 0.0f;
        gq += (double)phi;
        gs += (double)dsg;
        ge += (double)elj;
    };

    auto phase_b = [&]() {
        for (int g0 = 0; g0 < jl_n; g0 += 4) {
            const int e = g0 + (lane >> 3);
            if (e < jl_n) {
                const int4 en = sm.jl[e];
                const int sj = 8 * en.x + (lane & 7);
                const size_t gsl = (size_t)R.slot_win + sj;
                const float4 X4 = a.clX[gsl];
                float dx = __fsub_rn(__fadd_rn(X4.x, __int_as_float(en.y)), o[0]);
                float dy = __fsub_rn(__fadd_rn(X4.y, __int_as_float(en.z)), o[1]);
                float dz = __fsub_rn(__fadd_rn(X4.z, __int_as_float(en.w)), o[2]);
                if (IMG) {
                    dx = img32(dx, S.Lf[0], S.invLf[0]);
                    dy = img32(dy, S.Lf[1], S.invLf[1]);
                    dz = img32(dz, S.Lf[2], S.invLf[2]);
                }
                const float r2 = r2_chain(dx, dy, dz);
                bool ok = (r2 < S.rc2f) && X4.x < 1.0e5f && a.grp[gsl] == 0;
                if (ok && ne > 0) ok = !adj_excluded(sm, a, eb, ne, a.perm[gsl]);
                if (ok) {
                    const float2 P = a.clP[gsl];
                    acc(r2, X4.w, P.x, P.y);
                }
            }
        }
        jl_n = 0;
    };

    for (int k0 = 0; k0 < nst; k0 += 32) {
        const int k = k0 + lane;
        int cntJ = 0, Jb = 0, cnt2 = 0, Jb2 = 0;
        float Sx = 0.f, Sy = 0.f;
        if (k < nst) {
            const int2 off = a.stencil[S.fst_base + k];
            const int ccx = wrap_add(cy[0], off.x, S.M[0]);
            const int ccy = wrap_add(cy[1], off.y, S.M[1]);
            const int colid = ccx * S.M[1] + ccy;
            Sx = tabx[wrap_cell(ccx - cy[0], S.M[0]) + S.M[0]];
            Sy = taby[wrap_cell(ccy - cy[1], S.M[1]) + S.M[1]];
            bool ok = true;
            if (!IMG) {
                const float lox = Sx - 1.0e-4f, hix = Sx + S.gf[0] + 1.0e-4f;
                const float loy = Sy - 1.0e-4f, hiy = Sy + S.gf[1] + 1.0e-4f;
                const float gx = fmaxf(0.0f, fmaxf(lox - o[0], o[0] - hix));
                const float gy = fmaxf(0.0f, fmaxf(loy - o[1], o[1] - hiy));
                ok = gx * gx + gy * gy < rclc2;
            }
            if (ok) {
                const int lo = colcl[colid], hi = colcl[colid + 1];
                if (wholez) {
                    Jb = lo;
                    cntJ = hi - lo;
                } else {
                    Jb = lower_zhi(zb, lo, hi, za1);
                    cntJ = upper_zlo(zb, Jb, hi, zb1) - Jb;
                    if (za2 <= zb2) {
                        Jb2 = lower_zhi(zb, lo, hi, za2);
                        cnt2 = upper_zlo(zb, Jb2, hi, zb2) - Jb2;
                        // the two pieces are disjoint in z; clusters are counted once
                        if (cnt2 > 0 && cntJ > 0 && Jb2 < Jb + cntJ && Jb2 + cnt2 > Jb) {
                            const int u0 = min(Jb, Jb2), u1 = max(Jb + cntJ, Jb2 + cnt2);
                            Jb = u0; cntJ = u1 - u0; cnt2 = 0;
                        }
                    }
                }
                cntJ = max(cntJ, 0);
                cnt2 = max(cnt2, 0);
            }
        }
        // up to two cluster ranges per column, in lane order
        const bool h1 = cntJ > 0, h2 = cnt2 > 0;
        const unsigned hb1 = __ballot_sync(0xffffffffu, h1), hb2 = __ballot_sync(0xffffffffu, h2);
        int incl = cntJ + cnt2;
#pragma unroll
        for (int oo = 1; oo < 32; oo <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, oo);
            if (lane >= oo) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        {
            const unsigned lt = (1u << lane) - 1u;
            const int ri = __popc(hb1 & lt) + __popc(hb2 & lt);
            if (h1) sm.rng[ri] = make_int4(Jb, incl - cntJ - cnt2, __float_as_int(Sx), __float_as_int(Sy));
            if (h2) sm.rng[ri + (h1 ? 1 : 0)] = make_int4(Jb2, incl - cnt2, __float_as_int(Sx), __float_as_int(Sy));
        }
        const int nr = __popc(hb1) + __popc(hb2);
        __syncwarp();
        for (int e0 = 0; e0 < total; e0 += 32) {
            const int e = e0 + lane;
            bool pass = false;
            int4 en = make_int4(0, 0, 0, 0);
            if (e < total) {
                int lo = 0, hi = nr - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (sm.rng[mid].y <= e) lo = mid; else hi = mid - 1;
                }
                const int4 rg = sm.rng[lo];
                const int J = rg.x + (e - rg.y);
                const int jw = R.cl_win + J;
                const float4 cj = a.cl_bbc[jw];
                const float4 hjb = a.cl_bbh[jw];
                const float sz = tabz[wrap_cell(__float_as_int(cj.w) - cy[2], S.M[2]) + S.M[2]];
                const float sx = __int_as_float(rg.z), sy = __int_as_float(rg.w);
                float dx = cj.x + sx - o[0], dy = cj.y + sy - o[1], dz = cj.z + sz - o[2];
                if (IMG) {
                    dx = img32(dx, S.Lf[0], S.invLf[0]);
                    dy = img32(dy, S.Lf[1], S.invLf[1]);
                    dz = img32(dz, S.Lf[2], S.invLf[2]);
                }
                const float gx = fmaxf(fabsf(dx) - hjb.x, 0.0f);
                const float gy = fmaxf(fabsf(dy) - hjb.y, 0.0f);
                const float gz = fmaxf(fabsf(dz) - hjb.z, 0.0f);
                pass = gx * gx + gy * gy + gz * gz < rclc2;
                en = make_int4(J, __float_as_int(sx), __float_as_int(sy), __float_as_int(sz));
            }
            const unsigned bal = __ballot_sync(0xffffffffu, pass);
            if (pass) sm.jl[jl_n + __popc(bal & ((1u << lane) - 1u))] = en;
            jl_n += __popc(bal);
            __syncwarp();
            if (jl_n > SDM_JL_CAP - 32) phase_b();
            __syncwarp();
        }
    }
    phase_b();
    // every other displaced particle, at its own state-s position
    for (int q0 = 0; q0 < S.nD; q0 += 32) {
        const int qi = q0 + lane;
        if (qi < S.nD) {
            const int qa = a.D_idx[S.D_base + qi];
            if (qa != p) {
                const int tq = S.atom_base + qa;
                const SdmPertPos& pq = a.pert_pos[R.pert_win + 2 * qi + st];
                float d[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double yq = pq.y[k];
                    double v = __dsub_rn(yq, y[k]);
                    const double tt = rint(__dmul_rn(v, S.invL[k]));
                    v = __dsub_rn(v, __dmul_rn(tt, S.box[k]));
                    d[k] = __double2float_rn(v);
                }
                const float r2 = r2_chain(d[0], d[1], d[2]);
                if (r2 < S.rc2f && !adj_excluded(sm, a, eb, ne, qa))
                    acc(r2, a.topo_q[tq], a.topo_hs[tq], a.topo_se[tq]);
            }
        }
    }
#pragma unroll
    for (int oo = 16; oo > 0; oo >>= 1) {
        gq += __shfl_xor_sync(0xffffffffu, gq, oo);
        gs += __shfl_xor_sync(0xffffffffu, gs, oo);
        ge += __shfl_xor_sync(0xffffffffu, ge, oo);
    }
    if (lane == 0) {
        double* out = a.adj + 3 * (size_t)(R.pert_win + local);
        out[0] = gq;
        out[1] = gs;
        out[2] = ge;
    }
}

__global__ void __launch_bounds__(SDM_WARPS * 32) k_adjoint(SdmArgs a) {
    __shared__ AdjSmem smem[SDM_WARPS];
    AdjSmem& sm = smem[threadIdx.x >> 5];
    const int W = gridDim.x * SDM_WARPS;
    for (int item = blockIdx.x * SDM_WARPS + (threadIdx.x >> 5); item < a.total_pert; item += W) {
        const int r = rep_by_pert(a.rep, a.nrep, item);
        const int local = item - a.rep[r].pert_win;
        const SdmSys& S = a.sys[a.rep[r].sys];
        if (replica_image_mode(a, S, r)) process_adjoint<true>(a, r, local, sm);
        else process_adjoint<false>(a, r, local, sm);
    }
}

// ------------------------------------------------------------------------- //
// Backward of U_r = U0 + W (the differentiable potential), one launch        //
// ------------------------------------------------------------------------- //
// Given g_r = dL/dU_r: dL/dx = -g_r F (mixed force); dL/dd_i = -sum_r g_r s_r
// F1_ri over the replicas of i's system; the displaced particles' parameter
// gradients sum_r g_r ((1 - s_r) G_r0 + s_r G_r1) over the adjoint sums G;
// and g_r times the partial derivatives of W at fixed u' with respect to
// lambda1, lambda2, alpha, u0, w0 (integrated logistic; w0 also quadratic).
// Sums run over replicas in index order (fixed order, FP64).
__device__ __forceinline__ int sys_by_atom(const SdmArgs& a, int i) {
    int lo = 0, hi = a.nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.sys[mid].atom_base <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int sys_by_d(const SdmArgs& a, int k) {
    int lo = 0, hi = a.nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.sys[mid].D_base <= k) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_backward(SdmArgs a, BwdArgs b) {
    const long long total = b.n_x + b.n_d + b.n_p + b.n_b;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += stride) {
        long long q = t;
        if (q < b.n_x) {
            const int r = rep_by_atom(a.rep, a.nrep, (int)(q / 3));
            b.gx[q] = -b.g[r] * b.F[q];
            continue;
        }
        q -= b.n_x;
        if (q < b.n_d) {
            const int ia = (int)(q / 3), c = (int)(q - 3LL * ia);
            const SdmSys& S = a.sys[sys_by_atom(a, ia)];
            const int i = ia - S.atom_base;
            double acc = 0.0;
            for (int r = S.rep0; r < S.rep0 + S.nrep; ++r)
                acc = __fma_rn(b.g[r] * b.res[(size_t)r * SDM_NRESULTS + SDM_R_S],
                               b.F1[3 * (size_t)(a.rep[r].x_off + i) + c], acc);
            b.gd[q] = -acc;
            continue;
        }
        q -= b.n_d;
        if (q < b.n_p) {
            const int kd = (int)(q / 3), c = (int)(q - 3LL * kd);
            const SdmSys& S = a.sys[sys_by_d(a, kd)];
            const int k = kd - S.D_base;
            double acc = 0.0;
            for (int r = S.rep0; r < S.rep0 + S.nrep; ++r) {
                const double sw = b.res[(size_t)r * SDM_NRESULTS + SDM_R_S];
                const size_t e = ((size_t)(a.rep[r].pert_win / 2 + k) * 2) * 3 + c;
                acc = __fma_rn(b.g[r], __fma_rn(sw, b.G[e + 3], (1.0 - sw) * b.G[e]), acc);
            }
            // the third sum is 2 eps dU/deps: divided by 2 eps when eps is given
            if (c == 2 && b.eps) acc = b.eps[kd] > 0.0 ? acc / (2.0 * b.eps[kd]) : 0.0;
            b.gp[q] = acc;
            continue;
        }
        q -= b.n_p;
        {
            const int k = (int)(q / a.nrep), r = (int)(q - (long long)k * a.nrep);
            const double* p = a.params + (size_t)r * SDM_NPARAMS;
            const int method = (int)p[SDM_P_BIAS_METHOD];
            // lambda1, lambda2, alpha, u0 of the forward (rows of b.prm) or the handle's
            const double l1 = b.prm ? b.prm[r] : p[SDM_P_LAMBDA1];
            const double l2 = b.prm ? b.prm[a.nrep + r] : p[SDM_P_LAMBDA2];
            const double al = b.prm ? b.prm[2 * a.nrep + r] : p[SDM_P_ALPHA];
            const double u0 = b.prm ? b.prm[3 * a.nrep + r] : p[SDM_P_U0];
            const double be = b.res[(size_t)r * SDM_NRESULTS + SDM_R_BINDE];
            const bool ilog = method == SDM_ILOGISTIC, pos = ilog && al > 0.0;
            double d = 0.0;
            if (k == 4) {
                d = (ilog || method == SDM_QUADRATIC) ? 1.0 : 0.0;
            } else if (pos) {
                const double e = exp(-al * (be - u0)), ee = 1.0 + e, L = log(ee);
                const double dl = l2 - l1;
                d = k == 0 ? -L / al
                    : k == 1 ? L / al + be
                    : k == 2 ? dl * (-L / (al * al) - (be - u0) * e / (al * ee))
                             : dl * e / ee;
            } else if (k == 1 && ilog) {
                d = be;
            }
            b.gb[q] = b.g[r] * d;
        }
    }
}

// ------------------------------------------------------------------------- //
// K8: energies, soft core, bias (FP64)                                      //
// ------------------------------------------------------------------------- //
// ------------------------------------------------------------------------- //
// Exceptions (OpenMM NonbondedForce exceptions, e.g. 1-4 pairs)             //
// ------------------------------------------------------------------------- //
// E = K qq / r + 4 eps ((sigma/r)^12 - (sigma/r)^6) on the caller's
// coordinates (no cutoff, no reaction field, no periodic image), FP64; both
// states when the two displacements differ.  One thread per (replica,
// exception); forces enter the fixed-point F0 / dF of the two slots.
__device__ __forceinline__ void ex_terms(const double4_16a p, double dx, double dy, double dz, double& e, double& fs) {
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double ir2 = 1.0 / r2, ir = sqrt(ir2);
    const double s2 = p.y * p.y * ir2, s6 = s2 * s2 * s2, s12 = s6 * s6;
    const double ec = p.x * ir;
    e = ec + p.z * (s12 - s6);
    fs = (ec + p.z * (12.0 * s12 - 6.0 * s6)) * ir2;
}

__device__ __forceinline__ void red_fixd(unsigned long long* p, double v, int* status) {
    if (!(fabs(v) < 1.0e9)) {
        atomicOr(status, SDM_DEV_FORCE_OVERFLOW);
        return;
    }
    atomicAdd(p, (unsigned long long)__double2ll_rn(v * SDM_FIX_SCALE));
}

__global__ void k_except(SdmArgs a) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= a.total_ex) return;
    const int r = rep_by_ex(a.rep, a.nrep, item);
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int e = item - R.ex_win;
    const int2 pr = a.ex_pair[S.ex_base + e];
    const double4_16a prm = a.ex_prm[S.ex_base + e];
    const double* xi = a.x + 3 * (R.x_off + pr.x);
    const double* xj = a.x + 3 * (R.x_off + pr.y);
    const double* di = a.topo_d + 3 * (size_t)(S.atom_base + pr.x);
    const double* dj = a.topo_d + 3 * (size_t)(S.atom_base + pr.y);
    const size_t si = (size_t)R.slot_win + a.inv[R.atom_win + pr.x];
    const size_t sj = (size_t)R.slot_win + a.inv[R.atom_win + pr.y];
    const double d0[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
    double e0, f0;
    ex_terms(prm, d0[0], d0[1], d0[2], e0, f0);
    red_fixd(a.F0x + si, -f0 * d0[0], a.status);
    red_fixd(a.F0y + si, -f0 * d0[1], a.status);
    red_fixd(a.F0z + si, -f0 * d0[2], a.status);
    red_fixd(a.F0x + sj, f0 * d0[0], a.status);
    red_fixd(a.F0y + sj, f0 * d0[1], a.status);
    red_fixd(a.F0z + sj, f0 * d0[2], a.status);
    double du = 0.0;
    if (di[0] != dj[0] || di[1] != dj[1] || di[2] != dj[2]) {
        const double d1[3] = {(xj[0] + dj[0]) - (xi[0] + di[0]), (xj[1] + dj[1]) - (xi[1] + di[1]),
                              (xj[2] + dj[2]) - (xi[2] + di[2])};
        double e1, f1;
        ex_terms(prm, d1[0], d1[1], d1[2], e1, f1);
        du = e1 - e0;
        unsigned long long* dF[3] = {a.dFx, a.dFy, a.dFz};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double g = f1 * d1[k] - f0 * d0[k];   // dF on j; -g on i
            red_fixd(dF[k] + sj, g, a.status);
            red_fixd(dF[k] + si, -g, a.status);
        }
    }
    a.ex_e0[item] = e0;
    a.ex_du[item] = du;
}

// ------------------------------------------------------------------------- //
// PME: excluded pairs leave the reciprocal sum (-K qq erf(beta r)/r)          //
// ------------------------------------------------------------------------- //
// minimum-image separation from the wrapped coordinates: one FP64
// difference per component (|v| < L) rounded to FP32, plus dd (the FP32
// difference of the two displacements, 0 in state 1), wrapped in FP32 (the
// pair term itself is FP32; FP64 runs at 1/64 of the FP32 rate here)
__device__ __forceinline__ void xc_delta(const SdmSys& S, const double* wi, const double* wj, const float dd[3],
                                         float d[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float v = __double2float_rn(__dsub_rn(wj[k], wi[k]));
        d[k] = img32(__fadd_rn(v, dd[k]), S.Lf[k], S.invLf[k]);
    }
}

__device__ __forceinline__ void xc_terms(const SdmSys& S, float qq, const float d[3], float& e, float& fs) {
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float ir = rsqrtf(r2);
    const float xb = r2 * ir * S.beta_f;
    const float ef = erff(xb);
    e = -qq * ef * ir;
    fs = qq * (S.c2_f * __expf(-xb * xb) - ef * ir) * ir * ir;   // force on j = fs * d
}

__device__ double block_sum(double v, double* red);

// one block: 256 excluded pairs of replica blockIdx.y; the block's energy at
// x and its change at x + d go out as two partial sums (fixed-shape tree)
__device__ __forceinline__ void excl_corr_pair(const SdmArgs& a, const SdmRep& R, const SdmSys& S, int e,
                                               double& e0sum, double& dusum) {
    const int2 pr = a.xc_pair[S.xc_base + e];
    const float qq = a.xc_qq[S.xc_base + e];
    const double* wi = a.w + 3 * (size_t)(R.atom_win + pr.x);
    const double* wj = a.w + 3 * (size_t)(R.atom_win + pr.y);
    const size_t si = (size_t)R.slot_win + a.inv[R.atom_win + pr.x];
    const size_t sj = (size_t)R.slot_win + a.inv[R.atom_win + pr.y];
    float d0[3], e0, f0;
    const float zero[3] = {0.0f, 0.0f, 0.0f};
    xc_delta(S, wi, wj, zero, d0);
    xc_terms(S, qq, d0, e0, f0);
    unsigned long long* F0[3] = {a.F0x, a.F0y, a.F0z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        red_fix(F0[k] + sj, f0 * d0[k], a.status);
        red_fix(F0[k] + si, -f0 * d0[k], a.status);
    }
    double du = 0.0;
    // distinct displacement groups <=> distinct displacement vectors
    if (a.topo_grp[S.atom_base + pr.x] != a.topo_grp[S.atom_base + pr.y]) {
        const double* di = a.topo_d + 3 * (size_t)(S.atom_base + pr.x);
        const double* dj = a.topo_d + 3 * (size_t)(S.atom_base + pr.y);
        const float dd[3] = {__double2float_rn(__dsub_rn(dj[0], di[0])), __double2float_rn(__dsub_rn(dj[1], di[1])),
                             __double2float_rn(__dsub_rn(dj[2], di[2]))};
        float d1[3], e1, f1;
        xc_delta(S, wi, wj, dd, d1);
        xc_terms(S, qq, d1, e1, f1);
        du = (double)e1 - (double)e0;
        unsigned long long* dF[3] = {a.dFx, a.dFy, a.dFz};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float g = f1 * d1[k] - f0 * d0[k];
            red_fix(dF[k] + sj, g, a.status);
            red_fix(dF[k] + si, -g, a.status);
        }
    }
    e0sum = (double)e0;
    dusum = du;
}

__global__ void __launch_bounds__(256) k_excl_corr(SdmArgs a) {
    __shared__ double red[256];
    const int r = blockIdx.y;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double e0 = 0.0, du = 0.0;
    if (e < S.xc_count) excl_corr_pair(a, R, S, e, e0, du);
    e0 = block_sum(e0, red);
    du = block_sum(du, red);
    if (threadIdx.x == 0) {
        a.xc_e0[(size_t)r * gridDim.x + blockIdx.x] = e0;
        a.xc_du[(size_t)r * gridDim.x + blockIdx.x] = du;
    }
}

__device__ double block_sum(double v, double* red) {
    // deterministic: fixed-shape tree over a fixed partition
    const int t = threadIdx.x;
    red[t] = v;
    __syncthreads();
    for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
        if (t < s) red[t] += red[t + s];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// soft core of openmmapi/src/LangevinIntegratorSDM.cpp:125-149
__device__ double softcore(double u, int method, double umax, double a, double ub, double* fp) {
    if (u <= ub || method == SDM_NO_SOFTCORE) { *fp = 1.0; return u; }
    if (method == SDM_TANH_SOFTCORE) {
        const double t = tanh((u - ub) / umax);
        *fp = 1.0 - t * t;
        return umax * t + ub;
    }
    const double gu = (u - ub) / (a * (umax - ub));
    const double zeta = 1.0 + 2.0 * gu * (gu + 1.0);
    const double za = pow(zeta, a);
    *fp = 4.0 * (2.0 * gu + 1.0) / zeta * za / ((1.0 + za) * (1.0 + za));
    return (umax - ub) * (za - 1.0) / (za + 1.0) + ub;
}

// Combine record of a replica, written by k_combine, read by the finalize
enum { CMB_U, CMB_BE, CMB_FP, CMB_W, CMB_DW, CMB_DWDL, CMB_L1, CMB_L2, CMB_U0, CMB_W0 };
static_assert(CMB_W0 + 1 == SDM_CMB_FIELDS, "combine record size");

// The perturbation energy u of replica r (a fixed-order block reduction of
// the perturbation pass's, exceptions', excluded-pair corrections' and
// reciprocal space's parts) and the combine of
// platforms/reference/src/ReferenceSDMKernels.cpp:202-302: soft core, bias
// W, its derivative, dW/dlambda, and the mixing weight s of
// ReferenceSDMKernels.cpp:309-318.  None of it depends on the main pass.
// One block per replica.
__global__ void __launch_bounds__(256) k_combine(SdmArgs a) {
    __shared__ double red[256];
    const int r = blockIdx.x;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    double eu = 0.0;
    for (int k = threadIdx.x; k < 2 * S.nD * SDM_PERT_PARTS; k += blockDim.x)
        eu += a.p_part[(size_t)R.pert_win * SDM_PERT_PARTS + k];
    for (int k = threadIdx.x; k < S.ex_count; k += blockDim.x) eu += a.ex_du[R.ex_win + k];
    if (a.total_xc)
        for (int k = threadIdx.x; k < a.xc_blocks; k += blockDim.x) eu += a.xc_du[(size_t)r * a.xc_blocks + k];
    if (S.pme)
        for (int k = threadIdx.x; k < S.nD; k += blockDim.x) eu += a.pme_du[R.pert_win / 2 + k];
    const double u = block_sum(eu, red);
    if (threadIdx.x != 0) return;
    const double* p = a.params + (size_t)r * SDM_NPARAMS;
    const int method = (int)p[SDM_P_BIAS_METHOD];
    const int noneq = (int)p[SDM_P_NONEQ];
    const double lambdac = p[SDM_P_LAMBDA];
    double gamma = 0.0, wb = lambdac, w0 = 0.0, l1 = lambdac, l2 = lambdac, alpha = 1.0, u0 = 0.0;
    if (noneq == 1) {
        l1 = p[SDM_P_M_LAMBDA1] * lambdac + p[SDM_P_B_LAMBDA1];
        l2 = p[SDM_P_M_LAMBDA2] * lambdac + p[SDM_P_B_LAMBDA2];
        u0 = p[SDM_P_M_U0] * lambdac + p[SDM_P_B_U0];
        w0 = p[SDM_P_M_W0] * lambdac + p[SDM_P_B_W0];
    }
    if (method == SDM_QUADRATIC) {
        gamma = p[SDM_P_GAMMA];
        wb = p[SDM_P_WB];
        if (noneq != 1) w0 = p[SDM_P_W0];
    } else if (method == SDM_ILOGISTIC) {
        if (noneq != 1) { l1 = p[SDM_P_LAMBDA1]; l2 = p[SDM_P_LAMBDA2]; u0 = p[SDM_P_U0]; w0 = p[SDM_P_W0]; }
        alpha = p[SDM_P_ALPHA];
    }
    double fp;
    const double be = softcore(u, (int)p[SDM_P_SOFTCORE_METHOD], p[SDM_P_UMAX], p[SDM_P_ACORE],
                               p[SDM_P_UBCORE], &fp);
    // dW/dlambda sees the reference's function-scope lambda1, lambda2, alpha, u0
    // (ReferenceSDMKernels.cpp:214-217, 289-297): the scheduled values of its
    // non-equilibrium block are block-local (:236-239) and only the
    // integrated-logistic branch reloads them (:255-260).  For linear and
    // quadratic bias that is lambda1 = lambda2 (only their difference, 0,
    // enters), alpha = 1, u0 = 0 (the OpenCL platform does the same,
    // OpenCLSDMKernels.cpp:156-185,256-265).
    const bool ilog = method == SDM_ILOGISTIC;
    const double dl1 = ilog ? l1 : lambdac, dl2 = ilog ? l2 : lambdac, du0 = ilog ? u0 : 0.0;
    // e^(-alpha (u' - u0)) and log(1 + e^...), shared by the integrated-logistic
    // bias and dW/dlambda (one thread: the FP64 transcendentals are serial)
    double ex = 0.0, ee = 1.0, lee = 0.0;
    if (ilog || noneq == 1) {
        ex = exp(-alpha * (be - du0));
        ee = 1.0 + ex;
        lee = log(ee);
    }
    double ebias, bfp;
    if (method == SDM_QUADRATIC) {
        ebias = 0.5 * gamma * be * be + wb * be + w0;
        bfp = gamma * be + wb;
    } else if (method == SDM_ILOGISTIC) {
        ebias = 0.0;
        if (alpha > 0) ebias = ((l2 - l1) / alpha) * lee;
        ebias += l2 * be + w0;
        bfp = (l2 - l1) / ee + l1;
    } else {
        ebias = lambdac * be;
        bfp = lambdac;
    }
    double dwdl = 0.0;
    if (noneq == 1) {
        dwdl = (-lee / alpha) * p[SDM_P_M_LAMBDA1] + (be + lee / alpha) * p[SDM_P_M_LAMBDA2] +
               ((dl2 - dl1) * ex / ee) * p[SDM_P_M_U0] + p[SDM_P_M_W0];
    }
    double* c = a.cmb + (size_t)r * SDM_CMB_FIELDS;
    c[CMB_U] = u;
    c[CMB_BE] = be;
    c[CMB_FP] = fp;
    c[CMB_W] = ebias;
    c[CMB_DW] = bfp;
    c[CMB_DWDL] = dwdl;
    c[CMB_L1] = l1;
    c[CMB_L2] = l2;
    c[CMB_U0] = u0;
    c[CMB_W0] = w0;
    a.s_rep[r] = bfp * fp;
}

// U0 of replica r (fixed-order block reduction of the main pass's,
// exceptions', excluded-pair corrections' and reciprocal space's parts) and
// the replica's results, with the combine record of k_combine.  Thread 0
// writes.
__device__ void finalize_results(const SdmArgs& a, int r, double* red) {
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int ncl = a.ncl[r];
    double e0 = 0.0;
    const double* ep = a.e_part + (size_t)R.cl_win * a.split;
    for (int k = threadIdx.x; k < ncl * a.split; k += blockDim.x) e0 += ep[k];
    for (int k = threadIdx.x; k < S.ex_count; k += blockDim.x) e0 += a.ex_e0[R.ex_win + k];
    if (a.total_xc)
        for (int k = threadIdx.x; k < a.xc_blocks; k += blockDim.x) e0 += a.xc_e0[(size_t)r * a.xc_blocks + k];
    if (S.pme)
        for (int k = threadIdx.x; k < a.pme_conv_blocks; k += blockDim.x) e0 += a.pme_epart[(size_t)r * a.pme_conv_blocks + k];
    const double U0 = block_sum(e0, red) + S.e_const;
    if (threadIdx.x != 0) return;
    const double* c = a.cmb + (size_t)r * SDM_CMB_FIELDS;
    const double u = c[CMB_U];
    int st = *(volatile int*)a.status;
    if (!isfinite(U0) || !isfinite(u)) { st |= SDM_DEV_ENERGY_NONFINITE; atomicOr(a.status, SDM_DEV_ENERGY_NONFINITE); }
    double* o = a.results + (size_t)r * SDM_NRESULTS;
    o[SDM_R_U0] = U0;
    o[SDM_R_U1] = U0 + u;
    o[SDM_R_U] = u;
    o[SDM_R_BINDE] = c[CMB_BE];
    o[SDM_R_FP] = c[CMB_FP];
    o[SDM_R_W] = c[CMB_W];
    o[SDM_R_DW] = c[CMB_DW];
    o[SDM_R_S] = c[CMB_DW] * c[CMB_FP];
    o[SDM_R_EPOT] = U0 + c[CMB_W] + (a.rs_any ? a.rs_e[r] : 0.0);   // + group-1 restraints
    o[SDM_R_DWDLAMBDA] = c[CMB_DWDL];
    o[SDM_R_LAMBDA1] = c[CMB_L1];
    o[SDM_R_LAMBDA2] = c[CMB_L2];
    o[SDM_R_U0PARAM] = c[CMB_U0];
    o[SDM_R_W0PARAM] = c[CMB_W0];
    o[SDM_R_STATUS] = (double)st;
    o[SDM_R_RESERVED] = (double)ncl;
}


// ------------------------------------------------------------------------- //
// K9: mix                                                                   //
// ------------------------------------------------------------------------- //
// fixed point 2^32 -> double: one conversion, the scale applied to the
// exponent field (exact: every nonzero value is >= 1 before scaling)
__device__ __forceinline__ double fix_to_double(unsigned long long v) {
    // the conversion (double)(long long)v / 2^32 in integer arithmetic (the
    // integer-to-FP64 conversion runs on GB300's narrow FP64 pipe): the
    // magnitude normalised by its leading zeros, 52 mantissa bits rounded to
    // nearest, ties to even, as the conversion rounds; the exponent field
    // carries the 2^-32 scale (every nonzero value stays normal)
    if (v == 0ull) return 0.0;
    const unsigned long long sign = v & 0x8000000000000000ull;
    unsigned long long m = sign ? (0ull - v) : v;        // |v| (2^63 for the most negative value)
    const int lz = __clzll((long long)m);
    m <<= lz;                                             // leading one at bit 63
    const unsigned long long mant = (m >> 11) & 0x000FFFFFFFFFFFFFull;
    const unsigned long long rest = m & 0x7FFull;         // the 11 bits below the mantissa
    unsigned long long bits = ((unsigned long long)(63 - lz + 1023 - 32) << 52) | mant;
    if (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) bits += 1ull;   // a carry moves into the exponent
    return __longlong_as_double((long long)(sign | bits));
}

__global__ void k_mix(SdmArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < a.total_atoms; gi += stride) {
        const int r = rep_by_atom(a.rep, a.nrep, gi);
        const SdmRep& R = a.rep[r];
        const int i = gi - R.atom_win;
        const size_t gsl = (size_t)R.slot_win + a.inv[gi];
        const double s = a.forces ? a.s_rep[r] : 0.0;
        const double f0[3] = {fix_to_double(a.F0x[gsl]), fix_to_double(a.F0y[gsl]), fix_to_double(a.F0z[gsl])};
        const double df[3] = {fix_to_double(a.dFx[gsl]), fix_to_double(a.dFy[gsl]), fix_to_double(a.dFz[gsl])};
        const size_t o = 3 * (size_t)(R.x_off + i);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (a.forces) a.forces[o + k] = __fma_rn(s, df[k], f0[k]);
            if (a.F0out) a.F0out[o + k] = f0[k];
            if (a.F1out) a.F1out[o + k] = f0[k] + df[k];
        }
    }
}

// Finalize and mix in one launch (the evaluation without a Langevin step):
// blockIdx.y = replica; blockIdx.x < gridDim.x - 1 mixes a slice of
// kMixSlice particles with the weight s of k_combine, the last block reduces
// U0 and writes the replica's results beside them.
constexpr int kMixSlice = 2048;
__global__ void __launch_bounds__(256) k_finalize_mix(SdmArgs a) {
    __shared__ double red[256];
    const int r = blockIdx.y;
    const SdmRep& R = a.rep[r];
    if (blockIdx.x == gridDim.x - 1) {   // uniform per block
        finalize_results(a, r, red);
        return;
    }
    const int i0 = blockIdx.x * kMixSlice;
    if (i0 >= R.n) return;
    const double sw = a.forces ? a.s_rep[r] : 0.0;
    const int i1 = min(R.n, i0 + kMixSlice);
    // kMixBatch particles per thread and round: every gather of the round is
    // issued before the first conversion (the slot gathers are L2 latency)
    constexpr int kMixBatch = 4;
    for (int ib = i0 + threadIdx.x; ib < i1; ib += kMixBatch * blockDim.x) {
        unsigned long long v[kMixBatch][6];
#pragma unroll
        for (int q = 0; q < kMixBatch; ++q) {
            const int i = ib + q * (int)blockDim.x;
            const size_t gsl = (size_t)R.slot_win + a.inv[R.atom_win + (i < i1 ? i : ib)];
            v[q][0] = a.F0x[gsl]; v[q][1] = a.F0y[gsl]; v[q][2] = a.F0z[gsl];
            v[q][3] = a.dFx[gsl]; v[q][4] = a.dFy[gsl]; v[q][5] = a.dFz[gsl];
        }
#pragma unroll
        for (int q = 0; q < kMixBatch; ++q) {
            const int i = ib + q * (int)blockDim.x;
            if (i >= i1) break;
            const size_t o = 3 * (size_t)(R.x_off + i);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double f0 = fix_to_double(v[q][k]), df = fix_to_double(v[q][3 + k]);
                if (a.forces) a.forces[o + k] = __fma_rn(sw, df, f0);
                if (a.F0out) a.F0out[o + k] = f0;
                if (a.F1out) a.F1out[o + k] = f0 + df;
            }
        }
    }
}

// ------------------------------------------------------------------------- //
// K10: Langevin update with the mixed force                                  //
// ------------------------------------------------------------------------- //
// The stochastic-dynamics step of
// platforms/reference/src/ReferenceStochasticDynamicsSDM.cpp:131-266 (the SD
// leap-frog of GROMACS 3.1.4 do_update_sd) on the hybrid force of
// platforms/reference/src/ReferenceSDMKernels.cpp:309-318, per particle:
//   v  <- vscale v + fscale m^-1 F + noise m^-1/2 N(0,1)
//   x' =  x + dt v,   v <- (x' - x) / dt,   x <- x'
// with F = F0 + s dF (+ external forces).  Same operation order as the
// reference, no contraction, FP64.  Particles with m^-1 = 0 do not move.
// The normal deviates come from a counter-based generator: SplitMix64's
// output mixing (Steele, Lea and Flood, OOPSLA 2014) of (seed, step, particle
// component pair) gives two 32-bit uniforms per hash, Box-Muller turns them
// into two normals (FP32).
__device__ __forceinline__ unsigned long long sm64_mix(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float2 lv_normals(unsigned long long seed, unsigned long long step,
                                             unsigned long long counter) {
    const unsigned long long h =
        sm64_mix(seed ^ sm64_mix(step * 0x9E3779B97F4A7C15ull ^ counter * 0xD1B54A32D192ED03ull));
    const float u1 = (float)((unsigned)(h >> 40) + 1u) * 5.9604644775390625e-08f;   // (0, 1]
    const float u2 = (float)((unsigned)(h >> 8) & 0xffffffu) * 5.9604644775390625e-08f;
    const float r = sqrtf(-2.0f * logf(u1));
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    return make_float2(r * cs, r * sn);
}

// The stochastic-dynamics update in the finalize's launch, laid out as
// k_finalize_mix: blockIdx.y = replica; blockIdx.x < gridDim.x - 1 updates a
// slice of kMixSlice particles with the weight s of k_combine, the last block
// writes the replica's results.
__global__ void __launch_bounds__(256) k_langevin(SdmArgs a) {
    __shared__ double red[256];
    const int r = blockIdx.y;
    const SdmRep& R = a.rep[r];
    if (blockIdx.x == gridDim.x - 1) {   // uniform per block
        finalize_results(a, r, red);
        return;
    }
    const int i0 = blockIdx.x * kMixSlice;
    if (i0 >= R.n) return;
    const double s = a.s_rep[r];
    const double* prm = a.lv_prm;
    const double dt = prm[SDM_LV_DT], vscale = prm[SDM_LV_VSCALE], fscale = prm[SDM_LV_FSCALE];
    const double noise = prm[SDM_LV_NOISE], invdt = prm[SDM_LV_INVDT];
    const unsigned long long seed = (unsigned long long)__double_as_longlong(prm[SDM_LV_SEED]);
    const unsigned long long step = (unsigned long long)__double_as_longlong(prm[SDM_LV_STEP]);
    const int i1 = min(R.n, i0 + kMixSlice);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int gi = R.atom_win + i;
        const size_t pi = (size_t)R.x_off + i;   // particle in the concatenated order
        const double im = a.lv_invm[pi];
        // rigid-water particles leave x' in lv_xp; k_settle constrains and sets x and v
        const bool cons = a.st_any && a.st_flag[a.sys[R.sys].atom_base + i];
        if (im == 0.0) {
            if (cons)
                for (int k = 0; k < 3; ++k) a.lv_xp[3 * pi + k] = a.lv_x[3 * pi + k];
            continue;
        }
        const size_t gsl = (size_t)R.slot_win + a.inv[gi];
        const double f0[3] = {fix_to_double(a.F0x[gsl]), fix_to_double(a.F0y[gsl]), fix_to_double(a.F0z[gsl])};
        const double df[3] = {fix_to_double(a.dFx[gsl]), fix_to_double(a.dFy[gsl]), fix_to_double(a.dFz[gsl])};
        const float2 n01 = lv_normals(seed, step, 2 * pi), n2x = lv_normals(seed, step, 2 * pi + 1);
        const double nrm[3] = {(double)n01.x, (double)n01.y, (double)n2x.x};
        const double sq = sqrt(im);
        const double fsi = __dmul_rn(fscale, im), nsq = __dmul_rn(noise, sq);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double f = __fma_rn(s, df[k], f0[k]);
            if (a.lv_fext) f = __dadd_rn(f, a.lv_fext[3 * pi + k]);
            const double x = a.lv_x[3 * pi + k];
            const double v = __dadd_rn(__dadd_rn(__dmul_rn(vscale, a.lv_v[3 * pi + k]), __dmul_rn(fsi, f)),
                                       __dmul_rn(nsq, nrm[k]));
            const double xp = __dadd_rn(x, __dmul_rn(dt, v));
            if (cons) {
                a.lv_xp[3 * pi + k] = xp;
            } else {
                a.lv_v[3 * pi + k] = __dmul_rn(invdt, __dsub_rn(xp, x));
                a.lv_x[3 * pi + k] = xp;
            }
        }
    }
}

// ---- rigid waters: SETTLE (Miyamoto and Kollman, J. Comput. Chem. 13, 952 (1992)) ----
// Per water, old positions A0 B0 C0 (O H H, constrained) and unconstrained
// new A1 B1 C1.  Frame: origin the new centre of mass D, z normal to the old
// molecule plane, y along the new O's in-plane direction.  The constrained
// positions keep the new z coordinates (corrections along old bonds lie in
// the old plane); the canonical water is tilted by phi (from z of O) and psi
// (from z of H - H), then turned by theta about z so that the corrections
// exert no torque about the old positions (they are central forces along the
// old bonds): alpha sin(theta) + beta cos(theta) = gamma.
struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double d3dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 d3cross(D3 a, D3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ D3 d3unit(D3 a) {
    const double s = rsqrt(d3dot(a, a));
    return {a.x * s, a.y * s, a.z * s};
}
__device__ __forceinline__ D3 d3frame(D3 o, D3 e1, D3 e2, D3 e0, double x, double y, double z) {
    return {o.x + x * e1.x + y * e2.x + z * e0.x, o.y + x * e1.y + y * e2.y + z * e0.y,
            o.z + x * e1.z + y * e2.z + z * e0.z};
}

// one thread per water of replica blockIdx.y
__global__ void __launch_bounds__(128) k_settle(SdmArgs a) {
    const int r = blockIdx.y;
    const SdmRep& R = a.rep[r];
    const SdmSys& S = a.sys[R.sys];
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= S.st_count) return;
    const int* t = a.st_idx + 3 * (size_t)(S.st_base + w);
    const size_t p[3] = {(size_t)R.x_off + t[0], (size_t)R.x_off + t[1], (size_t)R.x_off + t[2]};
    const double invdt = a.lv_prm[SDM_LV_INVDT];
    const double im0 = a.lv_invm[p[0]], im1 = a.lv_invm[p[1]], im2 = a.lv_invm[p[2]];
    // positions, hydrogens in the minimum image of their oxygen
    double x0[3][3], x1[3][3], back[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            x0[j][k] = a.lv_x[3 * p[j] + k];
            x1[j][k] = a.lv_xp[3 * p[j] + k];
            back[j][k] = 0.0;
        }
#pragma unroll
    for (int j = 1; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            x0[j][k] -= S.box[k] * rint((x0[j][k] - x0[0][k]) * S.invL[k]);
            const double s1 = S.box[k] * rint((x1[j][k] - x1[0][k]) * S.invL[k]);
            x1[j][k] -= s1;
            back[j][k] = s1;   // restores the new position's own image
        }
    double P[3][3];
    if (im0 == 0.0 || im1 == 0.0 || im2 == 0.0) {   // a fixed particle: no constraint
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) P[j][k] = x1[j][k];
    } else {
        const double mo = 1.0 / im0, mh = 2.0 / (im1 + im2);
        const double rc = 0.5 * S.st_dhh;
        const double hgt = sqrt(fmax(S.st_doh * S.st_doh - rc * rc, 0.0));
        const double ra = 2.0 * mh * hgt / (mo + 2.0 * mh), rb = hgt - ra;
        const double invm = 1.0 / (mo + 2.0 * mh);
        const D3 A0{x0[0][0], x0[0][1], x0[0][2]}, B0{x0[1][0], x0[1][1], x0[1][2]}, C0{x0[2][0], x0[2][1], x0[2][2]};
        const D3 A1{x1[0][0], x1[0][1], x1[0][2]}, B1{x1[1][0], x1[1][1], x1[1][2]}, C1{x1[2][0], x1[2][1], x1[2][2]};
        const D3 Dc{(mo * A1.x + mh * (B1.x + C1.x)) * invm, (mo * A1.y + mh * (B1.y + C1.y)) * invm,
                    (mo * A1.z + mh * (B1.z + C1.z)) * invm};
        const D3 b0 = d3sub(B0, A0), c0 = d3sub(C0, A0);
        const D3 a1 = d3sub(A1, Dc), b1 = d3sub(B1, Dc), c1 = d3sub(C1, Dc);
        const D3 e0 = d3unit(d3cross(b0, c0));
        const D3 e1 = d3unit(d3cross(a1, e0));
        const D3 e2 = d3cross(e0, e1);
        const double xb0 = d3dot(e1, b0), yb0 = d3dot(e2, b0), xc0 = d3dot(e1, c0), yc0 = d3dot(e2, c0);
        const double za1 = d3dot(e0, a1);
        const double xb1 = d3dot(e1, b1), yb1 = d3dot(e2, b1), zb1 = d3dot(e0, b1);
        const double xc1 = d3dot(e1, c1), yc1 = d3dot(e2, c1), zc1 = d3dot(e0, c1);
        const double sphi = za1 / ra, cphi = sqrt(fmax(1.0 - sphi * sphi, 0.0));
        const double spsi = (zb1 - zc1) / (2.0 * rc * cphi), cpsi = sqrt(fmax(1.0 - spsi * spsi, 0.0));
        const double ya2 = ra * cphi;
        const double xb2 = -rc * cpsi, yb2 = -rb * cphi - rc * spsi * sphi;
        const double xc2 = rc * cpsi, yc2 = -rb * cphi + rc * spsi * sphi;
        const double al = xb0 * xb2 + yb0 * yb2 + xc0 * xc2 + yc0 * yc2;
        const double be = xb0 * yb2 - yb0 * xb2 + xc0 * yc2 - yc0 * xc2;
        const double ga = xb0 * yb1 - yb0 * xb1 + xc0 * yc1 - yc0 * xc1;
        const double ab = al * al + be * be;
        const double sth = (al * ga - be * sqrt(fmax(ab - ga * ga, 0.0))) / ab;
        const double cth = sqrt(fmax(1.0 - sth * sth, 0.0));
        const D3 Pa = d3frame(Dc, e1, e2, e0, -ya2 * sth, ya2 * cth, za1);
        const D3 Pb = d3frame(Dc, e1, e2, e0, xb2 * cth - yb2 * sth, xb2 * sth + yb2 * cth, zb1);
        const D3 Pc = d3frame(Dc, e1, e2, e0, xc2 * cth - yc2 * sth, xc2 * sth + yc2 * cth, zc1);
        P[0][0] = Pa.x; P[0][1] = Pa.y; P[0][2] = Pa.z;
        P[1][0] = Pb.x; P[1][1] = Pb.y; P[1][2] = Pb.z;
        P[2][0] = Pc.x; P[2][1] = Pc.y; P[2][2] = Pc.z;
    }
    const double imj[3] = {im0, im1, im2};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (imj[j] == 0.0) continue;   // fixed: x and v untouched
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            a.lv_v[3 * p[j] + k] = (P[j][k] - x0[j][k]) * invdt;
            a.lv_x[3 * p[j] + k] = P[j][k] + back[j][k];
        }
    }
}

// advances the step counter of the Langevin parameter block (last node of a step)
__global__ void k_lv_tick(double* prm) {
    const unsigned long long st = (unsigned long long)__double_as_longlong(prm[SDM_LV_STEP]);
    prm[SDM_LV_STEP] = __longlong_as_double((long long)(st + 1));
}

}  // namespace

// ------------------------------------------------------------------------- //
// launchers (called by sdm_capi.cpp)                                        //
// ------------------------------------------------------------------------- //
static int g_num_sms = 0;

static int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

static int grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    long long cap = (long long)num_sms() * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

extern "C++" {

cudaError_t sdm_launch_prep(const SdmArgs& a, int* item_prefix, int* grp_prefix, int* done, cudaStream_t st,
                            cudaEvent_t* ev, int nev, unsigned ev_flags) {
    int e = 0;
    auto mark = [&]() { if (ev && e < nev) cudaEventRecordWithFlags(ev[e++], st, ev_flags); };
    mark();
    k_cells<<<grid_for(a.total_atoms, 256), 256, 0, st>>>(a);
    mark();
    k_scan<<<a.nrep, 1024, 0, st>>>(a, item_prefix, grp_prefix, done);
    mark();
    k_bucket<<<grid_for(a.total_atoms, 256), 256, 0, st>>>(a);
    mark();
    k_cellsort<<<grid_for(a.total_atoms > a.total_cols ? a.total_atoms : a.total_cols, 256), 256, 0, st>>>(a);
    mark();
    k_clusters<<<grid_for(a.total_slots, 256), 256, 0, st>>>(a);
    mark();
    return cudaGetLastError();
}

cudaError_t sdm_launch_jlist(const SdmArgs& a, const int* grp_prefix, cudaStream_t st) {
    // one wave (the launch bounds give 4 CTAs per SM); the counter pays off
    // once the groups (at least particles / (8 jg)) outnumber the warps
    const int grid = num_sms() * 4;
    if ((long long)a.total_atoms > 8LL * a.jg * grid * 8) k_jlist<true><<<grid, 256, 0, st>>>(a, grp_prefix);
    else k_jlist<false><<<grid, 256, 0, st>>>(a, grp_prefix);
    return cudaGetLastError();
}

// Pair-kernel shapes: (warps per CTA, CTAs per SM the registers are bounded for).
// Registers are held per SM sub-partition and a CTA's warps are spread over
// the 4 sub-partitions, so only CTAs of 4 warps balance: 3 or 4 warps per
// sub-partition give 168 or 128 registers per thread (5 would give 96, where
// the kernel spills).
#define SDM_PAIR_SHAPES(X) X(4, 3) X(4, 4)

template <int MODE, int MINB, int NW, bool PME = false, int CH = SDM_CH_DEFAULT>
static cudaError_t pair_attr() {
    return cudaFuncSetAttribute(k_pair<MODE, MINB, NW, PME, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(NW * sizeof(EvalSmem<CH>)));
}

// Raises the dynamic shared memory limit of every pair-kernel shape on the
// current device (called once per handle, outside any stream capture).
cudaError_t sdm_pair_prepare() {
    cudaError_t e = cudaSuccess;
#define SDM_ATTR(NW, MB)                                                                   \
    if (e == cudaSuccess) e = pair_attr<MODE_EVAL, MB, NW, false, 8>();                    \
    if (e == cudaSuccess) e = pair_attr<MODE_EVAL, MB, NW, false, 12>();                   \
    if (e == cudaSuccess) e = pair_attr<MODE_EVAL, MB, NW, false, 16>();                   \
    if (e == cudaSuccess) e = pair_attr<MODE_EVAL, MB, NW, true, 8>();                     \
    if (e == cudaSuccess) e = pair_attr<MODE_EVAL, MB, NW, true, 12>();                    \
    if (e == cudaSuccess) e = pair_attr<MODE_EVAL, MB, NW, true, 16>();
    SDM_PAIR_SHAPES(SDM_ATTR)
#undef SDM_ATTR
    if (e == cudaSuccess) e = pair_attr<MODE_COUNT, 3, 4>();
    if (e == cudaSuccess) e = pair_attr<MODE_EMIT, 3, 4>();
    return e;
}

// Register bound (MINB) of the pair kernel launched with ctas_per_sm CTAs:
// the tightest built bound that still admits that many CTAs, 0 if none.
static int pair_minb(int ctas_per_sm) {
    int best = 0;
#define SDM_PICK(NW, MB) \
    if (ctas_per_sm <= MB && (best == 0 || MB < best)) best = MB;
    SDM_PAIR_SHAPES(SDM_PICK)
#undef SDM_PICK
    return best;
}

// CTAs of pair-kernel shape (NW, MB) the occupancy calculator places on one SM
template <int MODE, int MINB, int NW, int CH>
static int pair_resident() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pair<MODE, MINB, NW, false, CH>, NW * 32,
                                                      NW * sizeof(EvalSmem<CH>)) != cudaSuccess)
        return 0;
    return n;
}

// CTAs per SM that are resident when ctas_per_sm are requested with a staging
// chunk of `chunk` list entries (current device); 0 when no pair kernel is
// built for the request
int sdm_pair_resident(int ctas_per_sm, int chunk) {
    const int mb = pair_minb(ctas_per_sm);
#define SDM_RES(NW, MB)                                                                         \
    if (mb == MB) {                                                                             \
        const int n = chunk == 8 ? pair_resident<MODE_EVAL, MB, NW, 8>()                        \
                      : chunk == 16 ? pair_resident<MODE_EVAL, MB, NW, 16>()                    \
                                    : pair_resident<MODE_EVAL, MB, NW, 12>();                   \
        return std::min(ctas_per_sm, n);                                                        \
    }
    SDM_PAIR_SHAPES(SDM_RES)
#undef SDM_RES
    return 0;
}

// resident = CTAs per SM that fit (sdm_pair_resident): the persistent static
// schedule covers every item with any grid, so the grid never exceeds one wave
template <int MB, int NW, int CH>
static void launch_pair_eval(const SdmArgs& a, const int* item_prefix, int grid, bool pme, cudaStream_t st) {
    const size_t smem = NW * sizeof(EvalSmem<CH>);
    if (pme) k_pair<MODE_EVAL, MB, NW, true, CH><<<grid, NW * 32, smem, st>>>(a, item_prefix);
    else k_pair<MODE_EVAL, MB, NW, false, CH><<<grid, NW * 32, smem, st>>>(a, item_prefix);
}

cudaError_t sdm_launch_pair(const SdmArgs& a, const int* item_prefix, int mode, int ctas_per_sm,
                            int resident, bool pme, int chunk, cudaStream_t st) {
    const int grid = num_sms() * std::max(1, std::min(ctas_per_sm, resident));
    if (mode == MODE_EVAL) {
        const int mb = pair_minb(ctas_per_sm);
#define SDM_GO(NW, MB)                                                                    \
        if (mb == MB) {                                                                \
            if (chunk == 8) launch_pair_eval<MB, NW, 8>(a, item_prefix, grid, pme, st);  \
            else if (chunk == 16) launch_pair_eval<MB, NW, 16>(a, item_prefix, grid, pme, st); \
            else launch_pair_eval<MB, NW, 12>(a, item_prefix, grid, pme, st);            \
            return cudaGetLastError();                                                 \
        }
        SDM_PAIR_SHAPES(SDM_GO)
#undef SDM_GO
        return cudaErrorInvalidValue;
    } else if (mode == MODE_COUNT) {
        k_pair<MODE_COUNT, 3, 4><<<num_sms() * 3, 4 * 32, 4 * sizeof(EvalSmem<SDM_CH_DEFAULT>), st>>>(a, item_prefix);
    } else {
        k_pair<MODE_EMIT, 3, 4><<<num_sms() * 3, 4 * 32, 4 * sizeof(EvalSmem<SDM_CH_DEFAULT>), st>>>(a, item_prefix);
    }
    return cudaGetLastError();
}

cudaError_t sdm_launch_backward(const SdmArgs& a, const BwdArgs& b, cudaStream_t st) {
    const long long total = b.n_x + b.n_d + b.n_p + b.n_b;
    if (total == 0) return cudaSuccess;
    k_backward<<<grid_for(total, 256), 256, 0, st>>>(a, b);
    return cudaGetLastError();
}

cudaError_t sdm_launch_perturb(const SdmArgs& a, int mode, cudaStream_t st) {
    if (a.total_pert == 0) return cudaSuccess;
    k_pert_prep<<<(a.total_pert + 127) / 128, 128, 0, st>>>(a);
    int grid = (a.total_pert * SDM_PERT_PARTS + SDM_WARPS - 1) / SDM_WARPS;
    const int cap = num_sms() * 8;
    if (grid > cap) grid = cap;
    if (mode == MODE_COUNT) k_perturb<MODE_COUNT><<<grid, SDM_WARPS * 32, 0, st>>>(a);
    else k_perturb<MODE_EVAL><<<grid, SDM_WARPS * 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sdm_launch_exceptions(const SdmArgs& a, cudaStream_t st) {
    if (a.total_ex) k_except<<<(a.total_ex + 127) / 128, 128, 0, st>>>(a);
    if (a.total_xc) k_excl_corr<<<dim3(a.xc_blocks, a.nrep), 256, 0, st>>>(a);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------- //
// Host-engine interop: reordered positions in, fixed-point forces out       //
// ------------------------------------------------------------------------- //
// x[3 index[k] + c] = posq[k].c (+ corr[k].c): the position array of an
// engine that keeps particles in its own order (float4 or double4, with the
// FP32 correction term of mixed precision)
template <typename V>
__global__ void k_gather_posq(const V* posq, const V* corr, const int* index, int n, double* x) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const V p = posq[k];
        double v[3] = {(double)p.x, (double)p.y, (double)p.z};
        if (corr) {
            const V c = corr[k];
            v[0] = __dadd_rn(v[0], (double)c.x);
            v[1] = __dadd_rn(v[1], (double)c.y);
            v[2] = __dadd_rn(v[2], (double)c.z);
        }
        const size_t o = 3 * (size_t)index[k];
        x[o] = v[0];
        x[o + 1] = v[1];
        x[o + 2] = v[2];
    }
}

// buf[c * padded + k] += round(f[3 index[k] + c] * 2^32): forces added into a
// component-major 2^32 fixed-point buffer in the engine's order
__global__ void k_scatter_fixed(const double* f, const int* index, int n, int padded, long long* buf) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const size_t o = 3 * (size_t)index[k];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            buf[(size_t)c * padded + k] += __double2ll_rn(__dmul_rn(f[o + c], SDM_FIX_SCALE));
    }
}

cudaError_t sdm_launch_gather_positions(const void* posq, const void* corr, int double_precision,
                                        const int* index, int n, double* x, cudaStream_t st) {
    const int grid = grid_for(n, 256);
    if (double_precision)
        k_gather_posq<double4_16a><<<grid, 256, 0, st>>>((const double4_16a*)posq, (const double4_16a*)corr, index, n, x);
    else
        k_gather_posq<float4><<<grid, 256, 0, st>>>((const float4*)posq, (const float4*)corr, index, n, x);
    return cudaGetLastError();
}

cudaError_t sdm_launch_scatter_forces(const double* f, const int* index, int n, int padded, long long* buf,
                                      cudaStream_t st) {
    k_scatter_fixed<<<grid_for(n, 256), 256, 0, st>>>(f, index, n, padded, buf);
    return cudaGetLastError();
}

cudaError_t sdm_launch_adjoint(const SdmArgs& a, cudaStream_t st) {
    if (a.total_pert == 0) return cudaSuccess;
    int grid = (a.total_pert + SDM_WARPS - 1) / SDM_WARPS;
    const int cap = num_sms() * 8;
    if (grid > cap) grid = cap;
    k_adjoint<<<grid, SDM_WARPS * 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sdm_launch_mix(const SdmArgs& a, cudaStream_t st) {
    k_mix<<<grid_for(a.total_atoms, 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sdm_launch_finalize(const SdmArgs& a, cudaStream_t st) {
    if (a.lv_x) {   // Langevin step: the mixed force feeds the update directly
        k_langevin<<<dim3((a.max_rep_atoms + kMixSlice - 1) / kMixSlice + 1, a.nrep), 256, 0, st>>>(a);
        if (a.st_any) k_settle<<<dim3((a.st_max + 127) / 128, a.nrep), 128, 0, st>>>(a);
        k_lv_tick<<<1, 1, 0, st>>>(a.lv_prm);
    } else {
        k_finalize_mix<<<dim3((a.max_rep_atoms + kMixSlice - 1) / kMixSlice + 1, a.nrep), 256, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t sdm_launch_combine(const SdmArgs& a, cudaStream_t st) {
    k_combine<<<a.nrep, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // extern "C++"

// ========================================================================= //
// Allocation-free evaluation of one small system (sdm_evaluate_noalloc)     //
// ========================================================================= //
//
// Some callers cannot allocate device memory when they need a force: code
// that records the call into a CUDA graph (cudaMalloc is not allowed while a
// stream is being captured), hosts whose memory manager owns every device
// byte (a simulation engine's context or a framework's caching allocator,
// where an allocation behind their back breaks their accounting or fails
// under a fixed budget), and latency-bound drivers that cannot afford the
// implicit device synchronisation of cudaMalloc/cudaFree.  For them this
// entry point evaluates one system of at most SDM_NOALLOC_MAX_PARTICLES
// particles with every piece of scratch in one file-scope device array.
//
// The pair work is the all-pairs variant of the main and perturbation
// passes: every pair i<j is evaluated at the original coordinates and, when
// the displacements of i and j differ, at the displaced coordinates too, with
// the same FP32 pair terms, 2^32 fixed-point force accumulation and FP64
// energies as the handle path.  Cost grows as N^2, which is why the size is
// capped.

namespace {

constexpr int kNaMax = SDM_NOALLOC_MAX_PARTICLES;
constexpr int kNaBlocks = 304;            // 2 x 152 SMs
constexpr int kNaThreads = 256;
constexpr int kNaWarps = kNaBlocks * (kNaThreads / 32);
constexpr int kNaExclSmem = 128;          // per-warp cached exclusion partners

// byte layout of the scratch array
constexpr size_t kNaF0 = 0;                                       // u64[3*max]
constexpr size_t kNaDF = kNaF0 + 3ull * kNaMax * 8;              // u64[3*max]
constexpr size_t kNaQ = kNaDF + 3ull * kNaMax * 8;               // float[max] q*sqrt(K)
constexpr size_t kNaHS = kNaQ + 4ull * kNaMax;                   // float[max] sigma/2
constexpr size_t kNaSE = kNaHS + 4ull * kNaMax;                  // float[max] 2 sqrt(eps)
constexpr size_t kNaDB = kNaSE + 4ull * kNaMax;                  // u64[3*max] displacement bits
constexpr size_t kNaEP = kNaDB + 3ull * kNaMax * 8;              // double[warps] U0 partials
constexpr size_t kNaUP = kNaEP + 8ull * kNaWarps;                // double[warps] u partials
constexpr size_t kNaST = kNaUP + 8ull * kNaWarps;                // int status
constexpr size_t kNaBytes = (kNaST + 256 + 255) & ~size_t(255);

static_assert(kNaBytes == SDM_NOALLOC_SCRATCH_BYTES, "scratch size must match the header");

// The scratch.  Every GPU that loads the library holds it until exit.  In
// host code this name is only a host-side stand-in: kernels receive the
// device address taken with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_sdm_noalloc_scratch[kNaBytes];

struct NaArgs {
    int n;
    const double* x;
    const double* q;
    const double* sig;
    const double* eps;
    const int* eoff;
    const int* eidx;
    const double* d;
    double box[3], invL[3];
    float rc2f, krf, crf;
    double p[SDM_NPARAMS];
    double* results;
    double* forces;
    unsigned char* scratch;  // device address of g_sdm_noalloc_scratch
};

__device__ __forceinline__ unsigned long long* na_u64(const NaArgs& a, size_t off) {
    return reinterpret_cast<unsigned long long*>(a.scratch + off);
}
__device__ __forceinline__ float* na_f32(const NaArgs& a, size_t off) {
    return reinterpret_cast<float*>(a.scratch + off);
}
__device__ __forceinline__ double* na_f64(const NaArgs& a, size_t off) {
    return reinterpret_cast<double*>(a.scratch + off);
}

// clears what must start at zero and converts the per-particle parameters
__global__ void k_na_prep(NaArgs a) {
    const int stride = gridDim.x * blockDim.x;
    const double sk = 11.787089759563214;  // sqrt(138.935456)
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * a.n; k += stride) {
        na_u64(a, kNaF0)[k] = 0ull;
        na_u64(a, kNaDF)[k] = 0ull;
        const double dv = a.d ? a.d[k] : 0.0;
        na_u64(a, kNaDB)[k] = (unsigned long long)__double_as_longlong(__dadd_rn(dv, 0.0));
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        na_f32(a, kNaQ)[i] = (float)(a.q[i] * sk);
        na_f32(a, kNaHS)[i] = (float)(0.5 * a.sig[i]);
        na_f32(a, kNaSE)[i] = (float)(2.0 * sqrt(a.eps[i]));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *reinterpret_cast<int*>(a.scratch + kNaST) = 0;
}

__device__ __forceinline__ float na_delta(const NaArgs& a, double xi, double xj, int k) {
    double v = __dsub_rn(xj, xi);
    v = __dsub_rn(v, __dmul_rn(rint(__dmul_rn(v, a.invL[k])), a.box[k]));
    return __double2float_rn(v);
}

__device__ __forceinline__ void na_red(const NaArgs& a, unsigned long long* p, float v) {
    if (!(fabsf(v) < 1.0e9f)) atomicOr(reinterpret_cast<int*>(a.scratch + kNaST), SDM_DEV_FORCE_OVERFLOW);
    atomicAdd(p, fix64(v));
}

__global__ void __launch_bounds__(kNaThreads) k_na_pairs(NaArgs a) {
    __shared__ int ex[kNaThreads / 32][kNaExclSmem];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int w = blockIdx.x * (blockDim.x >> 5) + wib;
    const float* qf = na_f32(a, kNaQ);
    const float* hs = na_f32(a, kNaHS);
    const float* se = na_f32(a, kNaSE);
    const unsigned long long* db = na_u64(a, kNaDB);
    unsigned long long* F0 = na_u64(a, kNaF0);
    unsigned long long* dF = na_u64(a, kNaDF);
    double e0 = 0.0, eu = 0.0;
    for (int i = w; i < a.n; i += kNaWarps) {
        const int eb = a.eoff[i], ee = a.eoff[i + 1];
        const int ne = ee - eb;
        __syncwarp();
        for (int k = lane; k < ne && k < kNaExclSmem; k += 32) ex[wib][k] = a.eidx[eb + k];
        __syncwarp();
        const double xi0 = a.x[3 * i], xi1 = a.x[3 * i + 1], xi2 = a.x[3 * i + 2];
        const unsigned long long di0 = db[3 * i], di1 = db[3 * i + 1], di2 = db[3 * i + 2];
        const double dd0 = __longlong_as_double((long long)di0), dd1 = __longlong_as_double((long long)di1),
                     dd2 = __longlong_as_double((long long)di2);
        const float qi = qf[i], hi = hs[i], ei = se[i];
        float f0x = 0.f, f0y = 0.f, f0z = 0.f, dfx = 0.f, dfy = 0.f, dfz = 0.f;
        for (int j = i + 1 + lane; j < a.n; j += 32) {
            bool excl = false;
            if (ne <= kNaExclSmem) {
                for (int k = 0; k < ne; ++k) excl |= (ex[wib][k] == j);
            } else {
                for (int k = eb; k < ee; ++k) excl |= (a.eidx[k] == j);
            }
            if (excl) continue;
            const double xj0 = a.x[3 * j], xj1 = a.x[3 * j + 1], xj2 = a.x[3 * j + 2];
            const float qq = qi * qf[j], sg = hi + hs[j], e4 = ei * se[j];
            // state 1 of the reference: original coordinates
            const float ax = na_delta(a, xi0, xj0, 0), ay = na_delta(a, xi1, xj1, 1), az = na_delta(a, xi2, xj2, 2);
            const float r2a = r2_chain(ax, ay, az);
            float ea = 0.f, fa = 0.f;
            const bool oka = r2a < a.rc2f;
            if (oka) {
                const float ir = fast_rsqrt(r2a), ir2 = ir * ir;
                const float s2 = sg * sg * ir2, s6 = s2 * s2 * s2, t6 = e4 * s6;
                ea = fmaf(t6, s6 - 1.0f, qq * fmaf(a.krf, r2a, ir - a.crf));
                fa = fmaf(t6, fmaf(12.0f, s6, -6.0f), qq * fmaf(-2.0f * a.krf, r2a, ir)) * ir2;
                e0 += (double)ea;
                f0x = fmaf(-fa, ax, f0x); f0y = fmaf(-fa, ay, f0y); f0z = fmaf(-fa, az, f0z);
                na_red(a, F0 + 3 * j, fa * ax);
                na_red(a, F0 + 3 * j + 1, fa * ay);
                na_red(a, F0 + 3 * j + 2, fa * az);
            }
            const unsigned long long dj0 = db[3 * j], dj1 = db[3 * j + 1], dj2 = db[3 * j + 2];
            if (dj0 == di0 && dj1 == di1 && dj2 == di2) continue;   // unchanged pair
            // state 2 of the reference: displaced coordinates
            const double yj0 = __dadd_rn(xj0, __longlong_as_double((long long)dj0));
            const double yj1 = __dadd_rn(xj1, __longlong_as_double((long long)dj1));
            const double yj2 = __dadd_rn(xj2, __longlong_as_double((long long)dj2));
            const float bx = na_delta(a, __dadd_rn(xi0, dd0), yj0, 0);
            const float by = na_delta(a, __dadd_rn(xi1, dd1), yj1, 1);
            const float bz = na_delta(a, __dadd_rn(xi2, dd2), yj2, 2);
            const float r2b = r2_chain(bx, by, bz);
            float eb2 = 0.f, fb = 0.f;
            if (r2b < a.rc2f) {
                const float ir = fast_rsqrt(r2b), ir2 = ir * ir;
                const float s2 = sg * sg * ir2, s6 = s2 * s2 * s2, t6 = e4 * s6;
                eb2 = fmaf(t6, s6 - 1.0f, qq * fmaf(a.krf, r2b, ir - a.crf));
                fb = fmaf(t6, fmaf(12.0f, s6, -6.0f), qq * fmaf(-2.0f * a.krf, r2b, ir)) * ir2;
            }
            eu += (double)eb2 - (double)ea;
            const float gx = fb * bx - fa * ax, gy = fb * by - fa * ay, gz = fb * bz - fa * az;
            dfx -= gx; dfy -= gy; dfz -= gz;
            na_red(a, dF + 3 * j, gx);
            na_red(a, dF + 3 * j + 1, gy);
            na_red(a, dF + 3 * j + 2, gz);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            f0x += __shfl_xor_sync(0xffffffffu, f0x, o);
            f0y += __shfl_xor_sync(0xffffffffu, f0y, o);
            f0z += __shfl_xor_sync(0xffffffffu, f0z, o);
            dfx += __shfl_xor_sync(0xffffffffu, dfx, o);
            dfy += __shfl_xor_sync(0xffffffffu, dfy, o);
            dfz += __shfl_xor_sync(0xffffffffu, dfz, o);
        }
        if (lane == 0) {
            na_red(a, F0 + 3 * i, f0x); na_red(a, F0 + 3 * i + 1, f0y); na_red(a, F0 + 3 * i + 2, f0z);
            na_red(a, dF + 3 * i, dfx); na_red(a, dF + 3 * i + 1, dfy); na_red(a, dF + 3 * i + 2, dfz);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e0 += __shfl_xor_sync(0xffffffffu, e0, o);
        eu += __shfl_xor_sync(0xffffffffu, eu, o);
    }
    if (lane == 0) {
        na_f64(a, kNaEP)[w] = e0;
        na_f64(a, kNaUP)[w] = eu;
    }
}

// soft core, bias and weight of one lambda state, the same formulas as the
// handle path's finalize kernel
__device__ void na_combine(const double* p, double U0, double u, int st, double* o) {
    const int method = (int)p[SDM_P_BIAS_METHOD];
    const int noneq = (int)p[SDM_P_NONEQ];
    const double lambdac = p[SDM_P_LAMBDA];
    double gamma = 0.0, wb = lambdac, w0 = 0.0, l1 = lambdac, l2 = lambdac, alpha = 1.0, u0 = 0.0;
    if (noneq == 1) {
        l1 = p[SDM_P_M_LAMBDA1] * lambdac + p[SDM_P_B_LAMBDA1];
        l2 = p[SDM_P_M_LAMBDA2] * lambdac + p[SDM_P_B_LAMBDA2];
        u0 = p[SDM_P_M_U0] * lambdac + p[SDM_P_B_U0];
        w0 = p[SDM_P_M_W0] * lambdac + p[SDM_P_B_W0];
    }
    if (method == SDM_QUADRATIC) {
        gamma = p[SDM_P_GAMMA];
        wb = p[SDM_P_WB];
        if (noneq != 1) w0 = p[SDM_P_W0];
    } else if (method == SDM_ILOGISTIC) {
        if (noneq != 1) { l1 = p[SDM_P_LAMBDA1]; l2 = p[SDM_P_LAMBDA2]; u0 = p[SDM_P_U0]; w0 = p[SDM_P_W0]; }
        alpha = p[SDM_P_ALPHA];
    }
    double fp;
    const double be = softcore(u, (int)p[SDM_P_SOFTCORE_METHOD], p[SDM_P_UMAX], p[SDM_P_ACORE],
                               p[SDM_P_UBCORE], &fp);
    double ebias, bfp;
    if (method == SDM_QUADRATIC) {
        ebias = 0.5 * gamma * be * be + wb * be + w0;
        bfp = gamma * be + wb;
    } else if (method == SDM_ILOGISTIC) {
        const double ee = 1.0 + exp(-alpha * (be - u0));
        ebias = 0.0;
        if (alpha > 0) ebias = ((l2 - l1) / alpha) * log(ee);
        ebias += l2 * be + w0;
        bfp = (l2 - l1) / ee + l1;
    } else {
        ebias = lambdac * be;
        bfp = lambdac;
    }
    double dwdl = 0.0;
    if (noneq == 1) {
        // linear and quadratic bias: lambda1 = lambda2, alpha = 1, u0 = 0, as in k_combine
        const bool ilog = method == SDM_ILOGISTIC;
        const double dl1 = ilog ? l1 : lambdac, dl2 = ilog ? l2 : lambdac, du0 = ilog ? u0 : 0.0;
        const double ee = 1.0 + exp(-alpha * (be - du0));
        dwdl = (-log(ee) / alpha) * p[SDM_P_M_LAMBDA1] + (be + log(ee) / alpha) * p[SDM_P_M_LAMBDA2] +
               ((dl2 - dl1) * exp(-alpha * (be - du0)) / ee) * p[SDM_P_M_U0] + p[SDM_P_M_W0];
    }
    if (!isfinite(U0) || !isfinite(u)) st |= SDM_DEV_ENERGY_NONFINITE;
    o[SDM_R_U0] = U0;
    o[SDM_R_U1] = U0 + u;
    o[SDM_R_U] = u;
    o[SDM_R_BINDE] = be;
    o[SDM_R_FP] = fp;
    o[SDM_R_W] = ebias;
    o[SDM_R_DW] = bfp;
    o[SDM_R_S] = bfp * fp;
    o[SDM_R_EPOT] = U0 + ebias;
    o[SDM_R_DWDLAMBDA] = dwdl;
    o[SDM_R_LAMBDA1] = l1;
    o[SDM_R_LAMBDA2] = l2;
    o[SDM_R_U0PARAM] = u0;
    o[SDM_R_W0PARAM] = w0;
    o[SDM_R_STATUS] = (double)st;
    o[SDM_R_RESERVED] = 0.0;
}

__global__ void __launch_bounds__(256) k_na_finalize(NaArgs a) {
    __shared__ double red[256];
    double e0 = 0.0, eu = 0.0;
    for (int k = threadIdx.x; k < kNaWarps; k += blockDim.x) {
        e0 += na_f64(a, kNaEP)[k];
        eu += na_f64(a, kNaUP)[k];
    }
    const double U0 = block_sum(e0, red);
    const double u = block_sum(eu, red);
    if (threadIdx.x == 0)
        na_combine(a.p, U0, u, *reinterpret_cast<volatile int*>(a.scratch + kNaST), a.results);
}

__global__ void k_na_mix(NaArgs a) {
    const double sc = 1.0 / SDM_FIX_SCALE;
    const double s = a.results[SDM_R_S];
    const unsigned long long* F0 = na_u64(a, kNaF0);
    const unsigned long long* dF = na_u64(a, kNaDF);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * a.n; k += gridDim.x * blockDim.x)
        a.forces[k] = (double)(long long)F0[k] * sc + s * ((double)(long long)dF[k] * sc);
}

}  // namespace

void sdm_set_thread_error(const char* msg);

// device address of the scratch array, taken once per device with that device current
static unsigned char* g_na_addr[64];
static bool g_na_ready[64];
static std::mutex g_na_mutex;

extern "C" sdm_status sdm_evaluate_noalloc(int num_particles, const double* x, const double* charge,
                                           const double* sigma, const double* epsilon,
                                           const int* excl_offsets, const int* excl_indices,
                                           const double* displacement, const double* box,
                                           double cutoff, double eps_rf, const double* params,
                                           double* results, double* forces, void* stream) {
    if (num_particles < 1 || num_particles > SDM_NOALLOC_MAX_PARTICLES) {
        sdm_set_thread_error("sdm_evaluate_noalloc: num_particles must be in 1..SDM_NOALLOC_MAX_PARTICLES (8192)");
        return SDM_ERR_INVALID_ARGUMENT;
    }
    if (!x || !charge || !sigma || !epsilon || !excl_offsets || !excl_indices || !box || !params || !results) {
        sdm_set_thread_error("sdm_evaluate_noalloc: a required pointer is NULL");
        return SDM_ERR_INVALID_ARGUMENT;
    }
    for (int k = 0; k < 3; ++k)
        if (!(box[k] > 0.0) || !(cutoff > 0.0) || !(cutoff < 0.5 * box[k])) {
            sdm_set_thread_error("sdm_evaluate_noalloc: need 0 < cutoff < box/2 in every axis");
            return SDM_ERR_INVALID_ARGUMENT;
        }
    if (!(eps_rf > 0.0)) {
        sdm_set_thread_error("sdm_evaluate_noalloc: reaction_field_dielectric must be > 0");
        return SDM_ERR_INVALID_ARGUMENT;
    }
    const double bm = params[SDM_P_BIAS_METHOD], sm = params[SDM_P_SOFTCORE_METHOD];
    if (!(bm == 0.0 || bm == 1.0 || bm == 2.0) || !(sm == 0.0 || sm == 1.0 || sm == 2.0)) {
        sdm_set_thread_error("sdm_evaluate_noalloc: Unknown bias or soft core method");
        return SDM_ERR_UNKNOWN_METHOD;
    }
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess || dev < 0 || dev >= 64) {
        sdm_set_thread_error("sdm_evaluate_noalloc: no current CUDA device");
        return SDM_ERR_NO_DEVICE;
    }
    {
        std::lock_guard<std::mutex> lk(g_na_mutex);
        if (!g_na_ready[dev]) {
            void* p = nullptr;
            ce = cudaGetSymbolAddress(&p, g_sdm_noalloc_scratch);
            if (ce != cudaSuccess || !p) {
                sdm_set_thread_error("sdm_evaluate_noalloc: cudaGetSymbolAddress failed");
                return SDM_ERR_CUDA;
            }
            g_na_addr[dev] = static_cast<unsigned char*>(p);
            g_na_ready[dev] = true;
        }
    }
    NaArgs a;
    a.n = num_particles;
    a.x = x;
    a.q = charge;
    a.sig = sigma;
    a.eps = epsilon;
    a.eoff = excl_offsets;
    a.eidx = excl_indices;
    a.d = displacement;
    for (int k = 0; k < 3; ++k) { a.box[k] = box[k]; a.invL[k] = 1.0 / box[k]; }
    a.rc2f = (float)(cutoff * cutoff);
    a.krf = (float)((eps_rf - 1.0) / ((2.0 * eps_rf + 1.0) * cutoff * cutoff * cutoff));
    a.crf = (float)(3.0 * eps_rf / ((2.0 * eps_rf + 1.0) * cutoff));
    for (int k = 0; k < SDM_NPARAMS; ++k) a.p[k] = params[k];
    a.results = results;
    a.forces = forces;
    a.scratch = g_na_addr[dev];
    cudaStream_t st = (cudaStream_t)stream;
    k_na_prep<<<64, 256, 0, st>>>(a);
    k_na_pairs<<<kNaBlocks, kNaThreads, 0, st>>>(a);
    k_na_finalize<<<1, 256, 0, st>>>(a);
    if (forces) k_na_mix<<<32, 256, 0, st>>>(a);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) {
        sdm_set_thread_error(cudaGetErrorString(ce));
        return SDM_ERR_CUDA;
    }
    return SDM_OK;
}
