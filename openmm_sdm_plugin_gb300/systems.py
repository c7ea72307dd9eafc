"""Seeded synthetic SDM systems (host-side, numpy).

Each generator returns an :class:`SDMSystem`: an orthorhombic periodic box,
per-particle charge / LJ sigma / LJ epsilon, the symmetric exclusion list
(all intramolecular pairs), the per-particle displacement map and the SDM
schedule parameters of every replica.

The systems stand in for the reference's example inputs
(``example/test.py:172-191`` sets up the integrator with an ILogistic bias and a
Rational soft core; ``example/desmonddmsfile75.py:776-808`` builds the
NonbondedForce).  No public benchmark is involved: these are seeded synthetic
inputs with the shapes, sizes and value distributions of the workloads:

* ``config0``   930 sites, 3.0 nm box, one 30-atom ligand displaced by (1,0,0) nm
* ``config1``   7,500 rigid 3-site waters + two 40-atom ligands (A: +d, B: -d),
                6.2 nm box, d=(1.5,0,0) nm  -> 22,580 particles
* ``config2``   22 replicas of ``config1`` (independent jitter/orientations) with a
                22-state lambda schedule
* ``config3``   uneven multi-system batch (host-guest, 2k-60k particles)
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

# Bias and soft-core method ids, identical to the reference's integer constants
# (openmmapi/include/LangevinIntegratorSDM.h:120-122 and :143-145).
LINEAR, QUADRATIC, ILOGISTIC = 0, 1, 2
NO_SOFTCORE, TANH_SOFTCORE, RATIONAL_SOFTCORE = 0, 1, 2

WATER_Q_O, WATER_Q_H = -0.834, 0.417
WATER_SIG_O, WATER_EPS_O = 0.315, 0.636
WATER_OH, WATER_HOH_DEG = 0.09572, 104.52


@dataclasses.dataclass
class SDMParams:
    """SDM schedule of one replica (one lambda state).

    Field meanings follow the reference integrator's setters
    (openmmapi/include/LangevinIntegratorSDM.h:75-370).
    """
    bias_method: int = ILOGISTIC
    softcore_method: int = RATIONAL_SOFTCORE
    lambdac: float = 1.0       # setLambda (Linear bias slope)
    lambda1: float = 1.0
    lambda2: float = 1.0
    alpha: float = 1.0         # 1/(kJ/mol)
    u0: float = 0.0            # kJ/mol
    w0: float = 0.0            # kJ/mol (setW0coeff)
    gamma: float = 0.0         # Quadratic bias
    wb: float = 1.0            # Quadratic bias linear coefficient (setWBcoeff)
    umax: float = 200.0
    acore: float = 0.25
    ubcore: float = 0.0
    # non-equilibrium schedule: p(lambda) = slope*lambda + intercept
    noneq: int = 0
    m_lambda1: float = 0.0
    m_lambda2: float = 0.0
    m_u0: float = 0.0
    m_w0: float = 0.0
    b_lambda1: float = 0.0
    b_lambda2: float = 0.0
    b_u0: float = 0.0
    b_w0: float = 0.0

    def as_array(self) -> np.ndarray:
        """Packs the fields in the order of ``sdm_params`` (include/sdm_capi.h)."""
        return np.array([
            self.bias_method, self.softcore_method, self.lambdac, self.lambda1,
            self.lambda2, self.alpha, self.u0, self.w0, self.gamma, self.wb,
            self.umax, self.acore, self.ubcore, self.noneq, self.m_lambda1,
            self.m_lambda2, self.m_u0, self.m_w0, self.b_lambda1,
            self.b_lambda2, self.b_u0, self.b_w0], dtype=np.float64)


@dataclasses.dataclass
class Restraints:
    """Group-1 restraints of the reference's SDMUtils (python/SDMUtils.py),
    in nm, rad and kJ/mol (see sdm_restraints in include/sdm_capi.h).

    Centroid restraint (SDMUtils.addRestraintForce): flat-bottom harmonic on
    the distance between the weighted centroids of `lig_particles` and
    `rcpt_particles` (minus `offset`); with `use_angles`, flat-bottom windows
    on angle(r0, l0, l1), dihedral(r1, r0, l0, l1), dihedral(r0, l0, l1, l2).
    All scaled by the replica's control parameter.  Alignment restraint
    (SDMUtils.addAlignmentForce) between ligands A and B."""
    lig_particles: Sequence[int] = ()
    rcpt_particles: Sequence[int] = ()
    lig_weights: Optional[Sequence[float]] = None    # None: 1 (the reference weights by mass)
    rcpt_weights: Optional[Sequence[float]] = None
    kfcm: float = 0.0                # kJ/mol/nm^2
    tolcm: float = 0.0               # nm
    offset: Sequence[float] = (0.0, 0.0, 0.0)
    use_angles: bool = False
    rcpt_ref: Sequence[int] = (0, 0, 0)
    lig_ref: Sequence[int] = (0, 0, 0)
    kf_angle: float = 0.0            # kJ/mol/rad^2
    angle_center: float = 0.0        # rad
    angle_tol: float = 0.0
    kf_dihedral1: float = 0.0
    dihedral1_center: float = 0.0
    dihedral1_tol: float = 0.0
    kf_dihedral2: float = 0.0
    dihedral2_center: float = 0.0
    dihedral2_tol: float = 0.0
    use_alignment: bool = False
    liga_ref: Sequence[int] = (0, 0, 0)
    ligb_ref: Sequence[int] = (0, 0, 0)
    kf_displ: float = 0.0            # kJ/mol/nm^2
    k_theta: float = 0.0             # kJ/mol
    k_psi: float = 0.0               # kJ/mol
    align_offset: Sequence[float] = (0.0, 0.0, 0.0)


@dataclasses.dataclass
class SDMSystem:
    name: str
    box: np.ndarray            # (3,) nm
    charge: np.ndarray         # (N,) e
    sigma: np.ndarray          # (N,) nm
    epsilon: np.ndarray        # (N,) kJ/mol
    exclusions: np.ndarray     # (E,2) int32, i<j, each unordered pair once
    displacement: np.ndarray   # (N,3) nm
    positions: np.ndarray      # (R,N,3) nm, one coordinate set per replica
    params: List[SDMParams]    # R entries
    cutoff: float = 1.0
    eps_rf: float = 78.5
    ligand_atoms: Optional[np.ndarray] = None   # indices of displaced particles
    exceptions: Optional[np.ndarray] = None     # (X,2) int32 pairs with own parameters (also excluded)
    exception_params: Optional[np.ndarray] = None  # (X,3) charge product e^2, sigma nm, epsilon kJ/mol
    masses: Optional[np.ndarray] = None         # (N,) g/mol (dynamics only)
    nonbonded_method: str = "rf"                # "rf" (reaction field) or "pme"
    ewald_tolerance: float = 5e-4               # PME
    pme_grid: Optional[Sequence[int]] = None    # PME grid (None: from the tolerance)
    restraints: Optional[Restraints] = None     # group-1 restraints (SDMUtils)

    @property
    def n(self) -> int:
        return int(self.charge.shape[0])

    @property
    def replicas(self) -> int:
        return int(self.positions.shape[0])

    def replica(self, r: int) -> "SDMSystem":
        return dataclasses.replace(self, positions=self.positions[r:r + 1].copy(),
                                   params=[self.params[r]])


# --------------------------------------------------------------------------- #
# building blocks
# --------------------------------------------------------------------------- #
def _rigid_cluster(rng, n, rmax, dmin):
    """n points inside a sphere of radius rmax with pairwise spacing >= dmin."""
    pts = []
    tries = 0
    while len(pts) < n:
        tries += 1
        if tries > 200000:
            raise RuntimeError("cannot place rigid cluster")
        p = rng.uniform(-rmax, rmax, 3)
        if p @ p > rmax * rmax:
            continue
        if pts and np.min(np.linalg.norm(np.asarray(pts) - p, axis=1)) < dmin:
            continue
        pts.append(p)
    pts = np.asarray(pts)
    return pts - pts.mean(axis=0)


def _random_rotations(rng, k):
    q = rng.normal(size=(k, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
        2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
        2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        axis=-1).reshape(k, 3, 3)


def rigid_waters(s: "SDMSystem"):
    """(waters (W, 3) O H H indices, d_oh, d_hh) of a synthetic system: its
    leading particles are 3-site waters of the model geometry (O-H 0.09572 nm,
    H-O-H 104.52 degrees); W counts the leading (O, H, H) triples, where the
    hydrogens carry no Lennard-Jones term."""
    sig = np.asarray(s.epsilon)
    w = 0
    while 3 * w + 2 < s.n and sig[3 * w] != 0.0 and sig[3 * w + 1] == 0.0 and sig[3 * w + 2] == 0.0:
        w += 1
    waters = np.arange(3 * w, dtype=np.int32).reshape(-1, 3)
    d_hh = 2.0 * WATER_OH * math.sin(math.radians(WATER_HOH_DEG) / 2)
    return waters, WATER_OH, d_hh


def _water_frame():
    th = math.radians(WATER_HOH_DEG) / 2
    b = WATER_OH
    return np.array([[0.0, 0.0, 0.0],
                     [b * math.sin(th), b * math.cos(th), 0.0],
                     [-b * math.sin(th), b * math.cos(th), 0.0]])


def _lattice(shape, box):
    nx, ny, nz = shape
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                             indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    return (g + 0.5) * (np.asarray(box) / np.asarray(shape))


def _intra_pairs(first, count):
    idx = np.arange(first, first + count)
    a, b = np.triu_indices(count, 1)
    return np.stack([idx[a], idx[b]], axis=1)


def _ligand_params(rng, n):
    sig = rng.uniform(0.25, 0.35, n)
    eps = rng.uniform(0.2, 0.8, n)
    q = np.full(n, 0.4)
    q[rng.permutation(n)[: n // 2]] = -0.4
    return q, sig, eps


def _pick_lattice_sites(sites, box, centers, nkeep):
    """Keeps the nkeep lattice sites farthest (min-image) from all centers."""
    d = np.full(len(sites), np.inf)
    for c in centers:
        v = sites - c
        v -= box * np.round(v / box)
        d = np.minimum(d, np.linalg.norm(v, axis=1))
    order = np.argsort(-d, kind="stable")
    return np.sort(order[:nkeep])


# --------------------------------------------------------------------------- #
# config 0: 930 sites, plain SDM, Reference-runnable
# --------------------------------------------------------------------------- #
def config0(seed: int = 0, variant: str = "a") -> SDMSystem:
    rng = np.random.default_rng(seed)
    box = np.array([3.0, 3.0, 3.0])
    lig_c = box / 2
    d = np.array([1.0, 0.0, 0.0])
    sites = _lattice((10, 10, 10), box) + rng.uniform(-0.05, 0.05, (1000, 3))
    if variant == "b":
        keep = np.ones(1000, bool)
        for c in (lig_c, lig_c + d):
            v = sites - c
            v -= box * np.round(v / box)
            r = np.linalg.norm(v, axis=1)
            r[~keep] = np.inf
            keep[np.argsort(r, kind="stable")[:50]] = False
        solvent = sites[keep]
    else:
        solvent = sites[_pick_lattice_sites(sites, box, [lig_c], 900)]
    lig = _rigid_cluster(rng, 30, 0.35, 0.15) + lig_c
    pos = np.concatenate([solvent, lig]) % box
    n = len(pos)
    sig = rng.uniform(0.25, 0.35, n)
    eps = rng.uniform(0.2, 0.8, n)
    q = np.empty(n)
    qs = np.full(900, 0.4)
    qs[rng.permutation(900)[:450]] = -0.4
    ql = np.full(30, 0.4)
    ql[rng.permutation(30)[:15]] = -0.4
    q[:900], q[900:] = qs, ql
    excl = _intra_pairs(900, 30)
    disp = np.zeros((n, 3))
    disp[900:] = d
    prm = SDMParams(bias_method=ILOGISTIC, softcore_method=RATIONAL_SOFTCORE,
                    lambdac=0.5, lambda1=0.5, lambda2=0.5, alpha=0.0, u0=0.0,
                    w0=0.0, umax=200.0, acore=1.0 / 16.0, ubcore=100.0)
    return SDMSystem(f"config0{variant}", box, q, sig, eps, excl.astype(np.int32),
                     disp, pos[None].copy(), [prm], cutoff=0.9, eps_rf=78.5,
                     ligand_atoms=np.arange(900, 930))


# --------------------------------------------------------------------------- #
# config 1: 7,500 waters + two 40-atom ligands, 22,580 particles
# --------------------------------------------------------------------------- #
_CFG1_BOX = np.array([6.2, 6.2, 6.2])
_CFG1_SHAPE = (20, 20, 19)
_CFG1_D = np.array([1.5, 0.0, 0.0])
_CFG1_CA = np.array([2.35, 3.1, 3.1])


def _cfg1_ligands(seed):
    rng = np.random.default_rng(seed)
    la = _rigid_cluster(rng, 40, 0.45, 0.15)
    lb = _rigid_cluster(rng, 40, 0.45, 0.15)
    qa, sa, ea = _ligand_params(rng, 40)
    qb, sb, eb = _ligand_params(rng, 40)
    return (la, qa, sa, ea), (lb, qb, sb, eb)


def _cfg1_coords(seed, ligands):
    rng = np.random.default_rng(seed)
    box = _CFG1_BOX
    ca, cb = _CFG1_CA, _CFG1_CA + _CFG1_D
    sites = _lattice(_CFG1_SHAPE, box)
    keep = _pick_lattice_sites(sites, box, [ca, cb], 7500)
    centres = sites[keep] + rng.uniform(-0.05, 0.05, (7500, 3))
    rot = _random_rotations(rng, 7500)
    water = (centres[:, None, :] + np.einsum("kij,aj->kai", rot, _water_frame())).reshape(-1, 3)
    (la, *_), (lb, *_) = ligands
    pos = np.concatenate([water, la + ca, lb + cb]) % box
    return pos


def _cfg1_topology(ligands):
    (la, qa, sa, ea), (lb, qb, sb, eb) = ligands
    nw = 7500
    n = 3 * nw + 80
    q = np.empty(n)
    sig = np.zeros(n)
    eps = np.zeros(n)
    q[0:3 * nw:3] = WATER_Q_O
    q[1:3 * nw:3] = WATER_Q_H
    q[2:3 * nw:3] = WATER_Q_H
    sig[0:3 * nw:3] = WATER_SIG_O
    eps[0:3 * nw:3] = WATER_EPS_O
    q[3 * nw:3 * nw + 40], sig[3 * nw:3 * nw + 40], eps[3 * nw:3 * nw + 40] = qa, sa, ea
    q[3 * nw + 40:], sig[3 * nw + 40:], eps[3 * nw + 40:] = qb, sb, eb
    w = np.arange(nw) * 3
    excl = [np.stack([w, w + 1], 1), np.stack([w, w + 2], 1), np.stack([w + 1, w + 2], 1),
            _intra_pairs(3 * nw, 40), _intra_pairs(3 * nw + 40, 40)]
    excl = np.concatenate(excl).astype(np.int32)
    disp = np.zeros((n, 3))
    disp[3 * nw:3 * nw + 40] = _CFG1_D
    disp[3 * nw + 40:] = -_CFG1_D
    return q, sig, eps, excl, disp


def config1(seed: int = 1, variant: str = "a") -> SDMSystem:
    ligands = _cfg1_ligands(seed)
    q, sig, eps, excl, disp = _cfg1_topology(ligands)
    pos = _cfg1_coords(seed, ligands)
    if variant == "b":
        prm = SDMParams(lambdac=0.3, lambda1=0.2, lambda2=0.3, alpha=0.1, u0=110.0,
                        w0=0.0, umax=200.0, acore=1.0 / 16.0, ubcore=100.0)
    else:
        prm = SDMParams(lambdac=0.3, lambda1=0.3, lambda2=0.3, alpha=0.1, u0=110.0,
                        w0=0.0, umax=200.0, acore=1.0 / 16.0, ubcore=100.0)
    return SDMSystem(f"config1{variant}", _CFG1_BOX.copy(), q, sig, eps, excl, disp,
                     pos[None].copy(), [prm], cutoff=1.0, eps_rf=78.5,
                     ligand_atoms=np.arange(22500, 22580))


def lambda_schedule(nstates: int) -> List[SDMParams]:
    """Two-leg stand-in schedule: lambda_k=k/(n-1), lambda2=lambda_k,
    lambda1=lambda_k-0.1*sin(pi*lambda_k), alpha=0.1, u0=110, w0=0."""
    out = []
    for k in range(nstates):
        lam = k / (nstates - 1) if nstates > 1 else 1.0
        out.append(SDMParams(lambdac=lam, lambda1=lam - 0.1 * math.sin(math.pi * lam),
                             lambda2=lam, alpha=0.1, u0=110.0, w0=0.0, umax=200.0,
                             acore=1.0 / 16.0, ubcore=100.0))
    return out


def config2(nrep: int = 22, seed: int = 1) -> SDMSystem:
    """nrep replicas of config1 (seeds 100..100+nrep-1 for the solvent)."""
    ligands = _cfg1_ligands(seed)
    q, sig, eps, excl, disp = _cfg1_topology(ligands)
    pos = np.stack([_cfg1_coords(100 + r, ligands) for r in range(nrep)])
    return SDMSystem(f"config2x{nrep}", _CFG1_BOX.copy(), q, sig, eps, excl, disp, pos,
                     lambda_schedule(nrep) if nrep > 1 else [config1().params[0]],
                     cutoff=1.0, eps_rf=78.5, ligand_atoms=np.arange(22500, 22580))


# --------------------------------------------------------------------------- #
# config 3: uneven host-guest systems
# --------------------------------------------------------------------------- #
def host_guest(n_target: int, seed: int, nstates: int = 16, rc: float = 1.0,
               density: float = 33.0) -> SDMSystem:
    """Water-like solvent at `density` molecules/nm^3 around a guest of 20-60
    atoms displaced by one vector with |d| in [1.2, 2.0] nm.

    The box edge is max((nwat/density)^(1/3), 2*(rc+|d|)); when the second
    term wins the solvent is spread at a lower density so that the particle
    count stays at `n_target`.
    """
    rng = np.random.default_rng(seed)
    ng = int(rng.integers(20, 61))
    nw = max(1, (n_target - ng) // 3)
    dlen = rng.uniform(1.2, 2.0)
    dv = rng.normal(size=3)
    dv *= dlen / np.linalg.norm(dv)
    edge = max((nw / density) ** (1.0 / 3.0), 2.0 * (rc + dlen) + 0.05)
    box = np.array([edge, edge, edge])
    k = int(math.ceil(nw ** (1.0 / 3.0)))
    while k ** 3 < nw + 2 * ng:
        k += 1
    sites = _lattice((k, k, k), box)
    cg = box / 2 - dv / 2
    keep = _pick_lattice_sites(sites, box, [cg, cg + dv], nw)
    spacing = edge / k
    jit = min(0.05, 0.15 * spacing)
    centres = sites[keep] + rng.uniform(-jit, jit, (nw, 3))
    rot = _random_rotations(rng, nw)
    water = (centres[:, None, :] + np.einsum("kij,aj->kai", rot, _water_frame())).reshape(-1, 3)
    guest = _rigid_cluster(rng, ng, max(0.35, 0.11 * ng ** (1 / 3) + 0.1), 0.15) + cg
    pos = np.concatenate([water, guest]) % box
    n = 3 * nw + ng
    q = np.empty(n)
    sig = np.zeros(n)
    eps = np.zeros(n)
    q[0:3 * nw:3] = WATER_Q_O
    q[1:3 * nw:3] = WATER_Q_H
    q[2:3 * nw:3] = WATER_Q_H
    sig[0:3 * nw:3] = WATER_SIG_O
    eps[0:3 * nw:3] = WATER_EPS_O
    qg, sg, eg = _ligand_params(rng, ng)
    if ng % 2:
        qg[-1] = 0.0
    q[3 * nw:], sig[3 * nw:], eps[3 * nw:] = qg, sg, eg
    w = np.arange(nw) * 3
    excl = np.concatenate([np.stack([w, w + 1], 1), np.stack([w, w + 2], 1),
                           np.stack([w + 1, w + 2], 1), _intra_pairs(3 * nw, ng)]).astype(np.int32)
    disp = np.zeros((n, 3))
    disp[3 * nw:] = dv
    sched = lambda_schedule(nstates)
    # every lambda state gets its own coordinate set (independent jitter)
    reps = [pos]
    for s in range(1, nstates):
        r2 = np.random.default_rng([seed, s])
        c2 = sites[keep] + r2.uniform(-jit, jit, (nw, 3))
        rot2 = _random_rotations(r2, nw)
        w2 = (c2[:, None, :] + np.einsum("kij,aj->kai", rot2, _water_frame())).reshape(-1, 3)
        reps.append(np.concatenate([w2, guest]) % box)
    return SDMSystem(f"hostguest{n}", box, q, sig, eps, excl, disp, np.stack(reps), sched,
                     cutoff=rc, eps_rf=78.5, ligand_atoms=np.arange(3 * nw, n))


def config3(nsys: int = 64, nstates: int = 16, seed: int = 3, nmin: int = 2000,
            nmax: int = 60000) -> List[SDMSystem]:
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nsys)).astype(int)
    return [host_guest(int(s), seed * 1000 + i, nstates) for i, s in enumerate(sizes)]
