"""ctypes bindings of the FP64 CPU oracle (``oracle/sdm_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``, where it is the checker or the timed
CPU baseline -- never the product path.  See ``sdm_oracle.c`` for the
reference files each routine restates.

PARITY UNPINNED: the reference has no tests, golden vectors or fixtures for
this path and cannot be built here (it needs OpenMM), so the restatements are
cross-checked against independent implementations, closed forms and
invariances rather than against the reference's outputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "sdm_oracle.c")
_LIB = os.path.join(_HERE, "libsdm_oracle.so")
_lock = threading.Lock()
_lib = None

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_l = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

K_COULOMB = 138.935456   # kJ nm / (mol e^2) (OpenMM's ONE_4PI_EPS0, as in sdm_oracle.c)


def build(force: bool = False) -> str:
    """Compiles the oracle with gcc (OpenMP, no FP contraction)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp",
               "-o", _LIB + ".tmp", _SRC, "-lm"]
        subprocess.check_call(cmd)
        os.replace(_LIB + ".tmp", _LIB)
    return _LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB)
            sysargs = [C.c_int, _d, _d, _d, _i, _i, _d, C.c_double, C.c_double]
            L.orc_nonbonded.argtypes = sysargs + [_d, C.c_void_p, C.c_void_p, C.c_int]
            L.orc_nonbonded.restype = C.c_double
            L.orc_sdm_states.argtypes = sysargs + [_d, _d, _d, C.c_void_p, C.c_void_p, _l, C.c_int]
            L.orc_softcore.argtypes = [C.c_double, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.POINTER(C.c_double)]
            L.orc_softcore.restype = C.c_double
            L.orc_combine.argtypes = [_d, C.c_double, C.c_double, _d]
            L.orc_eval_state.argtypes = sysargs + [_d, _d, _d, _d, C.c_void_p, C.c_int]
            L.orc_build_clusters.argtypes = [C.c_int, _d, _d, _i, C.c_int, _i,
                                             C.POINTER(C.c_int), _i, _f, _i]
            L.orc_build_clusters.restype = C.c_int
            L.orc_image_mode.argtypes = [_d, _i, C.c_double, C.c_int, _i, _f]
            L.orc_sdm_f32rule.argtypes = sysargs + [_i, _d, _d, _d, C.c_void_p, C.c_void_p, _l]
            L.orc_sdm_f32rule.restype = C.c_int
            L.orc_emit_lists.argtypes = [C.c_int, _i, _i, _d, C.c_double, _i, _d, C.c_int,
                                         C.POINTER(C.c_int), _i, _i, _i, _u8]
            L.orc_emit_lists.restype = C.c_longlong
            _lib = L
    return _lib


# --------------------------------------------------------------------------- #
def excl_csr(n: int, pairs: np.ndarray):
    """Symmetric CSR (offsets, sorted partners) of an (E,2) exclusion list."""
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    a = np.concatenate([pairs[:, 0], pairs[:, 1]])
    b = np.concatenate([pairs[:, 1], pairs[:, 0]])
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    keep = np.ones(len(a), bool)
    if len(a):
        keep[1:] = (a[1:] != a[:-1]) | (b[1:] != b[:-1])
    a, b = a[keep], b[keep]
    off = np.zeros(n + 1, np.int32)
    np.add.at(off, a + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    return off, np.ascontiguousarray(b.astype(np.int32))


class OracleSystem:
    """Topology bundle for the oracle calls (one SDMSystem, any replica)."""

    def __init__(self, sysm):
        self.sys = sysm
        self.n = sysm.n
        self.q = np.ascontiguousarray(sysm.charge, np.float64)
        self.sig = np.ascontiguousarray(sysm.sigma, np.float64)
        self.eps = np.ascontiguousarray(sysm.epsilon, np.float64)
        self.off, self.idx = excl_csr(self.n, sysm.exclusions)
        if len(self.idx) == 0:
            self.idx = np.zeros(1, np.int32)
        self.box = np.ascontiguousarray(sysm.box, np.float64)
        self.rc = float(sysm.cutoff)
        self.eps_rf = float(sysm.eps_rf)
        self.d = np.ascontiguousarray(sysm.displacement, np.float64).reshape(-1)
        xp = getattr(sysm, "exceptions", None)
        self.exc = None if xp is None or not len(xp) else np.asarray(xp, np.int64).reshape(-1, 2)
        self.exc_prm = None if self.exc is None else np.asarray(sysm.exception_params, np.float64).reshape(-1, 3)

    def _args(self):
        return (self.n, self.q, self.sig, self.eps, self.off, self.idx, self.box, self.rc,
                self.eps_rf)

    def nonbonded(self, y, forces=True, nthreads=1):
        y = np.ascontiguousarray(y, np.float64).reshape(-1)
        f = np.zeros(3 * self.n) if forces else None
        npairs = C.c_longlong(0)
        e = lib().orc_nonbonded(*self._args(), y,
                                f.ctypes.data if forces else None, C.addressof(npairs), nthreads)
        return e, (f.reshape(-1, 3) if forces else None), npairs.value

    def exceptions(self, x):
        """Exception pairs (OpenMM NonbondedForce exceptions; the 1-4 pairs of
        example/desmonddmsfile75.py:813-848): E = K qq/r + 4 eps((s/r)^12 - (s/r)^6)
        on the given coordinates, no cutoff, no reaction field, no periodic image.
        Returns (E0, du, F0, dF): du and dF only over pairs whose displacements
        differ (the others are identical in both states)."""
        n = self.n
        F0 = np.zeros((n, 3))
        dF = np.zeros((n, 3))
        if self.exc is None:
            return 0.0, 0.0, F0, dF
        x = np.asarray(x, np.float64).reshape(-1, 3)
        d = self.d.reshape(-1, 3)
        i, j = self.exc[:, 0], self.exc[:, 1]
        kqq = K_COULOMB * self.exc_prm[:, 0]
        sg, e4 = self.exc_prm[:, 1], 4.0 * self.exc_prm[:, 2]

        def terms(dv, sel):
            r2 = (dv ** 2).sum(1)
            ir2 = 1.0 / r2
            ir = np.sqrt(ir2)
            s6 = (sg[sel] * sg[sel] * ir2) ** 3
            e = kqq[sel] * ir + e4[sel] * (s6 * s6 - s6)
            fs = (kqq[sel] * ir + e4[sel] * (12.0 * s6 * s6 - 6.0 * s6)) * ir2
            return e, fs[:, None] * dv    # force on j (minus: on i)
        d0 = x[j] - x[i]
        e0, f0 = terms(d0, slice(None))
        np.add.at(F0, j, f0)
        np.add.at(F0, i, -f0)
        ch = np.any(d[i] != d[j], axis=1)
        du = 0.0
        if ch.any():
            d1 = (x[j] + d[j]) - (x[i] + d[i])
            e1, f1 = terms(d1[ch], ch)
            du = float((e1 - e0[ch]).sum())
            g = f1 - f0[ch]
            np.add.at(dF, j[ch], g)
            np.add.at(dF, i[ch], -g)
        return float(e0.sum()), du, F0, dF

    def states(self, x, forces=True, nthreads=1):
        """FP64 rule: returns dict U0, U1, u_direct, F0, F1, counts."""
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        out = np.zeros(3)
        F0 = np.zeros(3 * self.n) if forces else None
        F1 = np.zeros(3 * self.n) if forces else None
        cnt = np.zeros(4, np.int64)
        lib().orc_sdm_states(*self._args(), x, self.d, out,
                             F0.ctypes.data if forces else None,
                             F1.ctypes.data if forces else None, cnt, nthreads)
        r = dict(U0=out[0], U1=out[1], u_direct=out[2], P0=int(cnt[0]), P1=int(cnt[1]),
                 P1delta=int(cnt[2]), Pc0=int(cnt[3]))
        if forces:
            r["F0"], r["F1"] = F0.reshape(-1, 3), F1.reshape(-1, 3)
        if self.exc is not None:
            e0, du, fx0, dfx = self.exceptions(x)
            r["U0"] += e0
            r["U1"] += e0 + du
            r["u_direct"] += du
            if forces:
                r["F0"] = r["F0"] + fx0
                r["F1"] = r["F1"] + fx0 + dfx
        return r

    def f32rule(self, x, M):
        """FP32 pair-inclusion rule of the CUDA path, FP64 arithmetic."""
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        out = np.zeros(3)
        F0 = np.zeros(3 * self.n)
        dF = np.zeros(3 * self.n)
        cnt = np.zeros(3, np.int64)
        img = lib().orc_sdm_f32rule(*self._args(), np.ascontiguousarray(M, np.int32), x, self.d,
                                    out, F0.ctypes.data, dF.ctypes.data, cnt)
        if img < 0:
            raise RuntimeError("oracle clustering capacity exceeded")
        r = dict(U0=out[0], u=out[1], U1=out[2], F0=F0.reshape(-1, 3), dF=dF.reshape(-1, 3),
                 P0=int(cnt[0]), P1delta=int(cnt[1]), Pc0=int(cnt[2]), image_mode=img)
        if self.exc is not None:
            e0, du, fx0, dfx = self.exceptions(x)
            r["U0"] += e0
            r["u"] += du
            r["U1"] = r["U0"] + r["u"]
            r["F0"] = r["F0"] + fx0
            r["dF"] = r["dF"] + dfx
        return r

    def clusters(self, x, M):
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        M = np.ascontiguousarray(M, np.int32)
        ncol = int(M[0] * M[1])
        cap = self.n + 8 * ncol + 8
        perm = np.zeros(cap, np.int32)
        ref = np.zeros(3 * cap, np.int32)
        X = np.zeros(4 * cap, np.float32)
        colcl = np.zeros(ncol + 1, np.int32)
        ncl = C.c_int(0)
        ns = lib().orc_build_clusters(self.n, x, self.box, M, cap, perm, C.byref(ncl), ref, X, colcl)
        if ns < 0:
            raise RuntimeError("capacity")
        k = ncl.value
        img = lib().orc_image_mode(self.box, M, self.rc, k, perm, X)
        return dict(perm=perm[:ns], ref=ref[:3 * k].reshape(-1, 3), X=X[:4 * ns].reshape(-1, 4),
                    colcl=colcl, ncl=k, image_mode=img)

    def lists(self, x, M, cap_per_cluster=2048):
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        M = np.ascontiguousarray(M, np.int32)
        ncol = int(M[0] * M[1])
        capcl = (self.n + 8 * ncol + 8) // 8 + 1
        perm = np.zeros(8 * capcl + 8, np.int32)
        cnt = np.zeros(capcl, np.int32)
        es = np.zeros(capcl * cap_per_cluster, np.int32)
        em = np.zeros(capcl * cap_per_cluster, np.uint8)
        ncl = C.c_int(0)
        tot = lib().orc_emit_lists(self.n, self.off, self.idx, self.box, self.rc, M, x,
                                   cap_per_cluster, C.byref(ncl), perm, cnt, es, em)
        if tot < 0:
            raise RuntimeError("list capacity exceeded")
        k = ncl.value
        return dict(ncl=k, cnt=cnt[:k], slot=es.reshape(capcl, -1)[:k], mask=em.reshape(capcl, -1)[:k],
                    total=int(tot))


def softcore(u, method, umax, acore, ub):
    fp = C.c_double(0.0)
    v = lib().orc_softcore(float(u), int(method), float(umax), float(acore), float(ub), C.byref(fp))
    return v, fp.value


def combine(params: np.ndarray, U0: float, U1: float) -> np.ndarray:
    out = np.zeros(12)
    lib().orc_combine(np.ascontiguousarray(params, np.float64), float(U0), float(U1), out)
    return out


COMBINE_FIELDS = ("u", "u_soft", "fp", "W", "dW", "s", "E_pot", "dWdlambda", "lambda1",
                  "lambda2", "u0", "w0")


def eval_state(osys: OracleSystem, x, params, nthreads=1, forces=True):
    """One full FP64 lambda-state evaluation (two nonbonded passes + combine)."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    res = np.zeros(14)
    F = np.zeros(3 * osys.n) if forces else None
    lib().orc_eval_state(*osys._args(), x, osys.d, np.ascontiguousarray(params, np.float64), res,
                         F.ctypes.data if forces else None, nthreads)
    return res, (F.reshape(-1, 3) if forces else None)


# --------------------------------------------------------------------------- #
# Langevin update (platforms/reference/src/ReferenceStochasticDynamicsSDM.cpp)
# --------------------------------------------------------------------------- #
MOLAR_GAS_CONSTANT = 0.008314462618   # kJ/(mol K), k_B N_A (CODATA 2018)


def langevin_coefficients(step_size, friction, temperature):
    """(vscale, fscale, noise scale) of ReferenceStochasticDynamicsSDM.cpp:145-148
    with tau = 1/friction (ReferenceSDMKernels.cpp:327)."""
    tau = 1.0 / friction
    vscale = np.exp(-step_size / tau)
    fscale = (1.0 - vscale) * tau
    kT = MOLAR_GAS_CONSTANT * temperature
    noise = np.sqrt(2.0 * kT / tau) * np.sqrt(0.5 * (1.0 - vscale * vscale) * tau)
    return vscale, fscale, noise


def shake_waters(x_old, xp, inv_mass, waters, d_oh, d_hh, box, tol=1e-13, maxit=200):
    """Rigid 3-site waters (O, H, H) by SHAKE iterated to convergence: the
    unconstrained positions xp move along the old bond vectors, mass
    weighted, until |O-H| = d_oh and |H-H| = d_hh (the constraint step the
    reference's integrator applies between the position update and the
    velocity recomputation, ReferenceStochasticDynamicsSDM.cpp:131-266).
    All waters at once; tol bounds |r^2 - d^2| / d^2 (FP64 coordinates of a
    few nm round r^2 - d^2 to ~1e-14 of d^2).  Hydrogens are taken in the
    minimum image of their oxygen and written back in their own image.
    Waters with a fixed particle are left as they are.  Returns (N, 3)."""
    x_old = np.asarray(x_old, np.float64).reshape(-1, 3)
    out = np.array(xp, np.float64).reshape(-1, 3)
    im = np.asarray(inv_mass, np.float64).reshape(-1)
    box = np.asarray(box, np.float64)
    W = np.asarray(waters, np.int64).reshape(-1, 3)
    W = W[np.all(im[W] != 0.0, axis=1)]
    if not len(W):
        return out
    x0 = x_old[W].copy()          # (nw, 3 atoms, 3)
    x1 = out[W].copy()
    shift = np.zeros_like(x1)
    for j in (1, 2):
        x0[:, j] = x0[:, 0] + _min_image(x0[:, j] - x0[:, 0], box)
        u = x1[:, 0] + _min_image(x1[:, j] - x1[:, 0], box)
        shift[:, j] = x1[:, j] - u
        x1[:, j] = u
    m = im[W]                     # (nw, 3) inverse masses
    cons = ((0, 1, d_oh), (0, 2, d_oh), (1, 2, d_hh))
    for _ in range(maxit):
        worst = 0.0
        for i, j, d in cons:
            r, r0 = x1[:, i] - x1[:, j], x0[:, i] - x0[:, j]
            diff = np.einsum("wk,wk->w", r, r) - d * d
            worst = max(worst, float(np.abs(diff).max()) / (d * d))
            g = diff / (2.0 * np.einsum("wk,wk->w", r0, r) * (m[:, i] + m[:, j]))
            x1[:, i] -= (g * m[:, i])[:, None] * r0
            x1[:, j] += (g * m[:, j])[:, None] * r0
        if worst < tol:
            break
    else:
        raise RuntimeError(f"SHAKE did not converge ({worst:.2e} after {maxit} iterations)")
    out[W] = x1 + shift
    return out


def langevin_update(x, v, inv_mass, F, step_size, friction, temperature, normals=None, waters=None,
                    d_oh=None, d_hh=None, box=None):
    """One stochastic-dynamics step (updatePart1, updatePart2 and the velocity
    recomputation of ReferenceStochasticDynamicsSDM.cpp:131-266), FP64 in the
    reference's operation order.  x, v, F: (N, 3); inv_mass: (N,); normals:
    (N, 3) standard normal deviates (None: zeros).  With `waters` ((W, 3)
    O, H, H indices), d_oh, d_hh and box the waters are held rigid
    (shake_waters) before the velocities are recomputed."""
    vscale, fscale, noise = langevin_coefficients(step_size, friction, temperature)
    x = np.asarray(x, np.float64).reshape(-1, 3)
    v = np.asarray(v, np.float64).reshape(-1, 3)
    F = np.asarray(F, np.float64).reshape(-1, 3)
    im = np.asarray(inv_mass, np.float64).reshape(-1, 1)
    n = np.zeros_like(x) if normals is None else np.asarray(normals, np.float64).reshape(-1, 3)
    move = (im[:, 0] != 0.0)
    v1 = vscale * v + (fscale * im) * F + (noise * np.sqrt(im)) * n
    xp = x + step_size * v1
    if waters is not None and len(waters):
        xp = np.where(move[:, None], xp, x)
        xp = shake_waters(x, xp, im[:, 0], waters, d_oh, d_hh, box)
        # a water's unwrapped velocity: (x' - x) of the images the constraint used
        v2 = (1.0 / step_size) * (xp - x)
        for w in np.asarray(waters, np.int64).reshape(-1, 3):
            for j in (1, 2):
                v2[w[j]] = (1.0 / step_size) * _min_image(xp[w[j]] - x[w[j]], np.asarray(box, np.float64))
    else:
        v2 = (1.0 / step_size) * (xp - x)
    xo = np.where(move[:, None], xp, x)
    vo = np.where(move[:, None], v2, v)
    return xo, vo


# --------------------------------------------------------------------------- #
# Ewald electrostatics (the reference's explicit-solvent setup uses PME,
# example/test_explicit.py:64 through OpenMM NonbondedForce; restated from the
# published Ewald decomposition, not from OpenMM source)
# --------------------------------------------------------------------------- #
def ewald_beta(cutoff, tolerance):
    """Splitting parameter beta = sqrt(-ln(2 tol)) / rc (1/nm): erfc(beta rc) ~ tol."""
    return np.sqrt(-np.log(2.0 * tolerance)) / cutoff


def _min_image(dv, box):
    return dv - box * np.round(dv / box)


def ewald(x, q, box, beta, cutoff, exclusions=(), kmax=None, forces=True):
    """Ewald sum, FP64, orthorhombic box.  Returns dict with the direct part
    (pairs within the cutoff, minimum image, excluded pairs skipped), the
    excluded-pair correction -K qq erf(beta r)/r, the reciprocal sum over
    k = 2 pi n / L with |n_k| <= kmax, the self term -K beta/sqrt(pi) sum q^2,
    the neutralising-background term -K pi Q^2 / (2 V beta^2), their total
    and the forces (N, 3).  Direct space is all-pairs: for small systems."""
    from math import erf, erfc
    x = np.asarray(x, np.float64).reshape(-1, 3)
    q = np.asarray(q, np.float64)
    box = np.asarray(box, np.float64)
    n = len(q)
    V = float(np.prod(box))
    F = np.zeros((n, 3))
    excl = {(min(a, b), max(a, b)) for a, b in np.asarray(exclusions, np.int64).reshape(-1, 2)}
    # direct space
    iu, ju = np.triu_indices(n, 1)
    dv = _min_image(x[ju] - x[iu], box)
    r = np.sqrt((dv ** 2).sum(1))
    keep = r < cutoff
    if excl:
        ex_mask = np.array([(a, b) in excl for a, b in zip(iu, ju)])
        keep &= ~ex_mask
    ec = np.array([erfc(beta * v) for v in r[keep]])
    qq = K_COULOMB * q[iu[keep]] * q[ju[keep]]
    rk = r[keep]
    e_dir = float((qq * ec / rk).sum())
    fs = qq * (ec / rk + 2.0 * beta / np.sqrt(np.pi) * np.exp(-(beta * rk) ** 2)) / rk ** 2
    if forces:
        fv = fs[:, None] * dv[keep]
        np.add.at(F, ju[keep], fv)
        np.add.at(F, iu[keep], -fv)
    # excluded pairs: remove their reciprocal-space interaction
    e_ex = 0.0
    if excl:
        pa = np.array(sorted(excl), np.int64)
        dvx = _min_image(x[pa[:, 1]] - x[pa[:, 0]], box)
        rx = np.sqrt((dvx ** 2).sum(1))
        qqx = K_COULOMB * q[pa[:, 0]] * q[pa[:, 1]]
        ef = np.array([erf(beta * v) for v in rx])
        e_ex = float(-(qqx * ef / rx).sum())
        fsx = -qqx * (ef / rx - 2.0 * beta / np.sqrt(np.pi) * np.exp(-(beta * rx) ** 2)) / rx ** 2
        if forces:
            fv = fsx[:, None] * dvx
            np.add.at(F, pa[:, 1], fv)
            np.add.at(F, pa[:, 0], -fv)
    # reciprocal space
    if kmax is None:
        kmax = [int(np.ceil(1.8 * beta * L)) for L in box]   # exp(-pi^2 n^2/(beta L)^2) < ~1e-14
    ns = np.stack(np.meshgrid(*[np.arange(-k, k + 1) for k in kmax], indexing="ij"), -1).reshape(-1, 3)
    ns = ns[np.any(ns != 0, axis=1)]
    kv = 2.0 * np.pi * ns / box
    k2 = (kv ** 2).sum(1)
    g = np.exp(-k2 / (4.0 * beta * beta)) / k2
    e_rec = 0.0
    for s in range(0, len(kv), 4096):
        ph = x @ kv[s:s + 4096].T                   # (N, chunk)
        c, sn = np.cos(ph), np.sin(ph)
        Sc, Ss = q @ c, q @ sn
        gs = g[s:s + 4096]
        e_rec += float((gs * (Sc ** 2 + Ss ** 2)).sum())
        if forces:
            # F_i = (4 pi K / V) q_i sum_k g k (sin(k x_i) Sc - cos(k x_i) Ss)
            w = gs * 1.0
            F += (4.0 * np.pi * K_COULOMB / V) * q[:, None] * (
                (sn * (w * Sc)[None, :] - c * (w * Ss)[None, :]) @ kv[s:s + 4096])
    e_rec *= 2.0 * np.pi * K_COULOMB / V
    e_self = float(-K_COULOMB * beta / np.sqrt(np.pi) * (q ** 2).sum())
    Q = float(q.sum())
    e_bg = float(-K_COULOMB * np.pi * Q * Q / (2.0 * V * beta * beta))
    total = e_dir + e_ex + e_rec + e_self + e_bg
    return dict(direct=e_dir, excluded=e_ex, reciprocal=e_rec, self=e_self, background=e_bg,
                total=total, F=F)


def pme_grid_size(beta, box, tolerance):
    """Grid points per axis: the smallest n >= 2 beta L / (3 tol^(1/5)) whose
    prime factors are 2, 3, 5 and 7 (the published OpenMM rule)."""
    out = []
    for L in np.asarray(box, np.float64):
        n = int(np.ceil(2.0 * beta * L / (3.0 * tolerance ** 0.2)))
        n = max(n, 6)
        while True:
            m = n
            for p in (2, 3, 5, 7):
                while m % p == 0:
                    m //= p
            if m == 1:
                break
            n += 1
        out.append(n)
    return np.array(out, np.int64)


def _bspline(w, order):
    """Cardinal B-spline weights M_order(w + j) and derivatives M'_order(w + j),
    j = 0..order-1, for fractional offsets w in [0, 1) (vectorised over w).
    Element j belongs to grid point floor(u) - j."""
    w = np.asarray(w, np.float64)
    M = np.zeros(w.shape + (order,))
    M[..., 0] = w            # M_2(w)
    M[..., 1] = 1.0 - w      # M_2(w + 1)
    dM = None
    for k in range(3, order + 1):
        if k == order:       # M'_k(x) = M_{k-1}(x) - M_{k-1}(x - 1)
            dM = np.zeros_like(M)
            for j in range(k):
                dM[..., j] = (M[..., j] if j < k - 1 else 0.0) - (M[..., j - 1] if j > 0 else 0.0)
        new = np.zeros_like(M)
        for j in range(k):   # M_k(x) = (x M_{k-1}(x) + (k - x) M_{k-1}(x - 1)) / (k - 1), x = w + j
            xj = w + j
            cur = M[..., j] if j < k - 1 else 0.0
            prev = M[..., j - 1] if j > 0 else 0.0
            new[..., j] = (xj * cur + (k - xj) * prev) / (k - 1)
        M = new
    return M, dM


def spme(x, q, box, beta, grid, order=5, forces=True):
    """Smooth particle-mesh Ewald reciprocal energy and forces (Essmann et
    al., J. Chem. Phys. 103, 8577 (1995)), FP64, orthorhombic box.  Particle i
    spreads onto grid points floor(u_i) - j, j = 0..order-1 (periodic), u_i =
    K x_i / L.  Returns (E, F, phi) with phi the real-space potential grid
    (theta_rec convolved with Q)."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    q = np.asarray(q, np.float64)
    box = np.asarray(box, np.float64)
    K = np.asarray(grid, np.int64)
    n = len(q)
    u = (x / box) % 1.0 * K
    fl = np.floor(u).astype(np.int64)
    w = u - fl
    Ms, dMs, idx = [], [], []
    for d in range(3):
        M, dM = _bspline(w[:, d], order)
        Ms.append(M); dMs.append(dM)
        idx.append((fl[:, d][:, None] - np.arange(order)[None, :]) % K[d])
    Q = np.zeros(tuple(K))
    for a in range(order):
        for b in range(order):
            wab = q * Ms[0][:, a] * Ms[1][:, b]
            for c in range(order):
                np.add.at(Q, (idx[0][:, a], idx[1][:, b], idx[2][:, c]), wab * Ms[2][:, c])
    # B-spline moduli |b(m)|^2 and the Ewald kernel
    Mint, _ = _bspline(np.zeros(1), order)      # M_order(j), j = 0..order-1
    bmod = []
    for d in range(3):
        m = np.arange(K[d])
        j = np.arange(order - 1)
        s2 = np.abs((Mint[0, j + 1][None, :] * np.exp(2j * np.pi * m[:, None] * j[None, :] / K[d])).sum(1)) ** 2
        # for odd orders the sum vanishes at the Nyquist index: use the mean of the neighbours
        z = s2 < 1e-7
        if z.any():
            s2[z] = 0.5 * (s2[(np.nonzero(z)[0] - 1) % K[d]] + s2[(np.nonzero(z)[0] + 1) % K[d]])
        bmod.append(1.0 / s2)
    mm = [np.where(np.arange(k) <= k // 2, np.arange(k), np.arange(k) - k) / L for k, L in zip(K, box)]
    m2 = mm[0][:, None, None] ** 2 + mm[1][None, :, None] ** 2 + mm[2][None, None, :] ** 2
    V = float(np.prod(box))
    with np.errstate(divide="ignore", invalid="ignore"):
        C = np.exp(-np.pi ** 2 * m2 / beta ** 2) / (np.pi * V * m2)
    C[0, 0, 0] = 0.0
    BC = C * bmod[0][:, None, None] * bmod[1][None, :, None] * bmod[2][None, None, :]
    FQ = np.fft.fftn(Q)
    E = 0.5 * K_COULOMB * float((BC * np.abs(FQ) ** 2).sum())
    phi = np.real(np.fft.ifftn(BC * FQ)) * np.prod(K)
    F = None
    if forces:
        F = np.zeros((n, 3))
        for a in range(order):
            for b in range(order):
                for c in range(order):
                    p = phi[idx[0][:, a], idx[1][:, b], idx[2][:, c]]
                    F[:, 0] -= dMs[0][:, a] * Ms[1][:, b] * Ms[2][:, c] * p
                    F[:, 1] -= Ms[0][:, a] * dMs[1][:, b] * Ms[2][:, c] * p
                    F[:, 2] -= Ms[0][:, a] * Ms[1][:, b] * dMs[2][:, c] * p
        F *= K_COULOMB * q[:, None] * (K / box)[None, :]
    return E, F, phi


# --------------------------------------------------------------------------
# Group-1 restraints of the reference's SDMUtils (python/SDMUtils.py): the
# custom-force energy expressions restated in numpy (FP64, no periodic
# images); forces by central differences of that energy, so the check does
# not share the kernel's analytic gradients.
# --------------------------------------------------------------------------
def _rs_wrap(v, period):
    """v - P floor(v/P + 0.5) (SDMUtils.py:78-88)."""
    return v - period * np.floor(v / period + 0.5)


def _rs_flat(v, lo, hi, period, kf):
    """(kf/2) (step(dm) max(0, db)^2 + step(-dm) max(0, -da)^2), step(0) = 1."""
    db, da = _rs_wrap(v - hi, period), _rs_wrap(v - lo, period)
    dm = _rs_wrap(v - 0.5 * (lo + hi), period)
    return 0.5 * kf * ((dm >= 0) * max(0.0, db) ** 2 + (-dm >= 0) * max(0.0, -da) ** 2)


def _rs_angle(p1, p2, p3):
    u, v = p1 - p2, p3 - p2
    return np.arctan2(np.linalg.norm(np.cross(u, v)), u @ v)


def _rs_dihedral(p1, p2, p3, p4):
    """IUPAC dihedral: trans = pi, cis = 0."""
    b1, b2, b3 = p2 - p1, p3 - p2, p4 - p3
    n = np.cross(b2, b3)
    return np.arctan2(np.linalg.norm(b2) * (b1 @ n), np.cross(b1, b2) @ n)


def _rs_cos(u, v):
    return (u @ v) / (np.linalg.norm(u) * np.linalg.norm(v))


def _rs_perp(d, n1):
    return d - (d @ n1) * n1


def restraint_energy(x, rs, control=1.0):
    """Energy (kJ/mol) of the restraints `rs` (fields of
    openmm_sdm_plugin_gb300.systems.Restraints) at coordinates x (N, 3)."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    E = 0.0
    lig, rcpt = list(rs.lig_particles), list(rs.rcpt_particles)
    if lig and rcpt:
        wl = np.ones(len(lig)) if rs.lig_weights is None else np.asarray(rs.lig_weights, np.float64)
        wr = np.ones(len(rcpt)) if rs.rcpt_weights is None else np.asarray(rs.rcpt_weights, np.float64)
        c1 = (wl[:, None] * x[lig]).sum(0) / wl.sum()
        c2 = (wr[:, None] * x[rcpt]).sum(0) / wr.sum()
        d = np.linalg.norm(c1 - np.asarray(rs.offset, np.float64) - c2)
        E += control * 0.5 * rs.kfcm * (d >= rs.tolcm) * (d - rs.tolcm) ** 2
        if rs.use_angles:
            r0, r1, _ = (x[i] for i in rs.rcpt_ref)
            l0, l1, l2 = (x[i] for i in rs.lig_ref)
            terms = ((_rs_angle(r0, l0, l1), rs.kf_angle, rs.angle_center, rs.angle_tol, np.pi),
                     (_rs_dihedral(r1, r0, l0, l1), rs.kf_dihedral1, rs.dihedral1_center, rs.dihedral1_tol,
                      2 * np.pi),
                     (_rs_dihedral(r0, l0, l1, l2), rs.kf_dihedral2, rs.dihedral2_center, rs.dihedral2_tol,
                      2 * np.pi))
            for v, kf, c, tol, per in terms:
                E += control * _rs_flat(v, c - tol, c + tol, per, kf)
    if rs.use_alignment:
        a0, a1, a2 = (x[i] for i in rs.liga_ref)
        b0, b1, b2 = (x[i] for i in rs.ligb_ref)
        E += 0.5 * rs.kf_displ * np.sum((b0 - np.asarray(rs.align_offset, np.float64) - a0) ** 2)
        E += 0.5 * rs.k_theta * (1.0 - _rs_cos(b1 - b0, a1 - a0))
        nb = (b1 - b0) / np.linalg.norm(b1 - b0)
        na = (a1 - a0) / np.linalg.norm(a1 - a0)
        E += 0.25 * rs.k_psi * (1.0 - _rs_cos(_rs_perp(b2 - b0, nb), _rs_perp(a2 - a0, nb)))
        E += 0.25 * rs.k_psi * (1.0 - _rs_cos(_rs_perp(a2 - a0, na), _rs_perp(b2 - b0, na)))
    return float(E)


def restraint_forces(x, rs, control=1.0, h=1e-6):
    """-dE/dx (N, 3) by central differences over the restraint's particles."""
    x = np.array(x, np.float64).reshape(-1, 3)
    idx = set(rs.lig_particles) | set(rs.rcpt_particles)
    if rs.use_angles:
        idx |= set(rs.rcpt_ref) | set(rs.lig_ref)
    if rs.use_alignment:
        idx |= set(rs.liga_ref) | set(rs.ligb_ref)
    F = np.zeros_like(x)
    for i in sorted(idx):
        for k in range(3):
            v = x[i, k]
            x[i, k] = v + h
            ep = restraint_energy(x, rs, control)
            x[i, k] = v - h
            em = restraint_energy(x, rs, control)
            x[i, k] = v
            F[i, k] = -(ep - em) / (2 * h)
    return F
