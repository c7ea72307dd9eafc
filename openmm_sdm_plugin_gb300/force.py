"""Host-side mirror of the reference's SDM parameter API over the C ABI.

``SDMForce`` carries exactly the SDM parameter surface of the reference's
``LangevinIntegratorSDM`` (openmmapi/include/LangevinIntegratorSDM.h:53-522,
exposed to Python by python/SDMplugin.i:71-146): the same setter/getter
names, argument meanings, defaults (openmmapi/src/LangevinIntegratorSDM.cpp:48-85)
and error behaviour (an unknown soft-core method raises, as
LangevinIntegratorSDM.cpp:147 throws).  On top of that it holds what the
reference takes from OpenMM's NonbondedForce in force group 2: per-particle
charge/sigma/epsilon, exclusions and exceptions (the 1-4 pairs), the
electrostatics (CutoffPeriodic reaction field or PME with its Ewald
tolerance), cutoff, reaction-field dielectric and the periodic box.

``evaluate`` does what one reference step does to the nonbonded group
(LangevinIntegratorSDM.cpp:158-176 plus ReferenceSDMKernels.cpp:202-318 without
the Langevin update) on the GPU and returns the hybrid energy and forces;
``getBindE``/``getPotEnergy`` then return the values the reference's getters
would.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

from . import capi
from .systems import Restraints, SDMParams, SDMSystem


class SDMForce:
    # method ids (LangevinIntegratorSDM.h:120-122, :143-145)
    LinearMethod = 0
    QuadraticMethod = 1
    ILogisticMethod = 2
    NoSoftCoreMethod = 0
    TanhMethod = 1
    RationalMethod = 2
    # nonbonded method ids of OpenMM's NonbondedForce that the path supports
    CutoffPeriodic = 2
    PME = 4

    def __init__(self, nParticles: int = 0):
        self._q: List[float] = []
        self._sig: List[float] = []
        self._eps: List[float] = []
        self._excl: List[tuple] = []
        self._exc: List[tuple] = []      # (i, j, charge product, sigma, epsilon)
        self._method = SDMForce.CutoffPeriodic
        self._ewald_tol = 5e-4
        self._pme_grid = None            # explicit PME grid (None: from the tolerance)
        self._displ = np.zeros((nParticles, 3))
        for _ in range(nParticles):
            self.addParticle(0.0, 0.0, 0.0)
        self._box = np.array([0.0, 0.0, 0.0])
        self._cutoff = 1.0
        self._eps_rf = 78.3
        self._p = SDMParams(bias_method=0, softcore_method=0, lambdac=1.0, lambda1=1.0,
                            lambda2=1.0, alpha=1.0, u0=0.0, w0=0.0, gamma=0.0, wb=1.0,
                            umax=200.0, acore=0.25, ubcore=0.0)
        self._ntmax = 0.0
        self._work = 0.0
        self._bind_e = 0.0
        self._pot_e = 0.0
        self._last = None
        self._handle: Optional[capi.Handle] = None
        self._topology_dirty = True
        self._displ_dirty = False
        self._params_dirty = True
        self._restraints: Optional[Restraints] = None   # group-1 restraints (SDMUtils mirror)
        self._restraints_dirty = False
        self._restraint_control = 1.0
        self._control_dirty = False

    # -- NonbondedForce-like topology ---------------------------------------
    def addParticle(self, charge: float, sigma: float, epsilon: float) -> int:
        self._q.append(float(charge))
        self._sig.append(float(sigma))
        self._eps.append(float(epsilon))
        if self._displ.shape[0] < len(self._q):
            self._displ = np.vstack([self._displ, np.zeros((1, 3))])
        self._topology_dirty = True
        return len(self._q) - 1

    def setParticleParameters(self, index: int, charge: float, sigma: float, epsilon: float):
        self._q[index], self._sig[index], self._eps[index] = float(charge), float(sigma), float(epsilon)
        self._topology_dirty = True

    def getParticleParameters(self, index: int):
        return self._q[index], self._sig[index], self._eps[index]

    def getNumParticles(self) -> int:
        return len(self._q)

    def addExclusion(self, i: int, j: int) -> int:
        self._excl.append((int(i), int(j)))
        self._topology_dirty = True
        return len(self._excl) - 1

    def getNumExclusions(self) -> int:
        return len(self._excl)

    def addException(self, particle1: int, particle2: int, chargeProd: float, sigma: float, epsilon: float,
                     replace: bool = False) -> int:
        """OpenMM NonbondedForce.addException: the pair is excluded from the
        nonbonded sum; with a charge product or a well depth it interacts
        with these parameters instead (the 1-4 pairs of
        example/desmonddmsfile75.py:813-848)."""
        i, j = int(particle1), int(particle2)
        key = (min(i, j), max(i, j))
        for k, e in enumerate(self._exc):
            if (min(e[0], e[1]), max(e[0], e[1])) == key:
                if not replace:
                    raise ValueError(f"there is already an exception for particles {i} and {j}")
                self._exc[k] = (i, j, float(chargeProd), float(sigma), float(epsilon))
                self._topology_dirty = True
                return k
        self._exc.append((i, j, float(chargeProd), float(sigma), float(epsilon)))
        self._topology_dirty = True
        return len(self._exc) - 1

    def getNumExceptions(self) -> int:
        return len(self._exc)

    def getExceptionParameters(self, index: int):
        return self._exc[index]

    def setNonbondedMethod(self, method: int):
        if int(method) not in (SDMForce.CutoffPeriodic, SDMForce.PME):
            raise ValueError("the nonbonded method must be CutoffPeriodic (reaction field) or PME")
        self._method = int(method)
        self._topology_dirty = True

    def getNonbondedMethod(self) -> int:
        return self._method

    def setEwaldErrorTolerance(self, tol: float):
        self._ewald_tol = float(tol)
        self._topology_dirty = True

    def getEwaldErrorTolerance(self) -> float:
        return self._ewald_tol

    # the model of the path has neither (the reference's loader turns the
    # dispersion correction off, example/desmonddmsfile75.py:427-428)
    def setUseDispersionCorrection(self, use: bool):
        if use:
            raise ValueError("the dispersion correction is not supported")

    def getUseDispersionCorrection(self) -> bool:
        return False

    def setUseSwitchingFunction(self, use: bool):
        if use:
            raise ValueError("switching functions are not supported")

    def getUseSwitchingFunction(self) -> bool:
        return False

    def setCutoffDistance(self, rc: float):
        self._cutoff = float(rc)
        self._topology_dirty = True

    def getCutoffDistance(self) -> float:
        return self._cutoff

    def setReactionFieldDielectric(self, e: float):
        self._eps_rf = float(e)
        self._topology_dirty = True

    def getReactionFieldDielectric(self) -> float:
        return self._eps_rf

    def setPeriodicBoxVectors(self, a, b, c):
        a, b, c = (np.asarray(v, np.float64) for v in (a, b, c))
        if np.count_nonzero(a[1:]) or b[0] or b[2] or c[0] or c[1]:
            raise ValueError("only orthorhombic boxes are supported")
        self._box = np.array([a[0], b[1], c[2]])
        self._topology_dirty = True

    def getPeriodicBoxVectors(self):
        return (np.array([self._box[0], 0, 0]), np.array([0, self._box[1], 0]),
                np.array([0, 0, self._box[2]]))

    # -- SDM parameters (names of LangevinIntegratorSDM) --------------------
    def _set(self, field, v):
        setattr(self._p, field, float(v))
        self._params_dirty = True

    def setLambda(self, v): self._set("lambdac", v)
    def getLambda(self): return self._p.lambdac
    def setBiasMethod(self, m): self._p.bias_method = int(m); self._params_dirty = True
    def getBiasMethod(self): return int(self._p.bias_method)
    def setSoftCoreMethod(self, m): self._p.softcore_method = int(m); self._params_dirty = True
    def getSoftCoreMethod(self): return int(self._p.softcore_method)
    def setGamma(self, v): self._set("gamma", v)
    def getGamma(self): return self._p.gamma
    def setWBcoeff(self, v): self._set("wb", v)
    def getWBcoeff(self): return self._p.wb
    def setW0coeff(self, v): self._set("w0", v)
    def getW0coeff(self): return self._p.w0
    def setLambda1(self, v): self._set("lambda1", v)
    def getLambda1(self): return self._p.lambda1
    def setLambda2(self, v): self._set("lambda2", v)
    def getLambda2(self): return self._p.lambda2
    def setAlpha(self, v): self._set("alpha", v)
    def getAlpha(self): return self._p.alpha
    def setU0(self, v): self._set("u0", v)
    def getU0(self): return self._p.u0
    def setUmax(self, v): self._set("umax", v)
    def getUmax(self): return self._p.umax
    def setAcore(self, v): self._set("acore", v)
    def getAcore(self): return self._p.acore
    def setUbcore(self, v): self._set("ubcore", v)
    def getUbcore(self): return self._p.ubcore
    def setNoneqtmax(self, v): self._ntmax = float(v)
    def getNoneqtmax(self): return self._ntmax
    def setNonEquilibrium(self, v): self._p.noneq = int(v); self._params_dirty = True
    def getNonEquilibrium(self): return int(self._p.noneq)
    def setNoneqWorkvalue(self, v): self._work = float(v)
    def getNoneqWorkvalue(self): return self._work
    def setlambda1Slope(self, v): self._set("m_lambda1", v)
    def getlambda1Slope(self): return self._p.m_lambda1
    def setlambda2Slope(self, v): self._set("m_lambda2", v)
    def getlambda2Slope(self): return self._p.m_lambda2
    def setu0Slope(self, v): self._set("m_u0", v)
    def getu0Slope(self): return self._p.m_u0
    def setw0Slope(self, v): self._set("m_w0", v)
    def getw0Slope(self): return self._p.m_w0
    def setlambda1intercept(self, v): self._set("b_lambda1", v)
    def getlambda1intercept(self): return self._p.b_lambda1
    def setlambda2intercept(self, v): self._set("b_lambda2", v)
    def getlambda2intercept(self): return self._p.b_lambda2
    def setu0intercept(self, v): self._set("b_u0", v)
    def getu0intercept(self): return self._p.b_u0
    def setw0intercept(self, v): self._set("b_w0", v)
    def getw0intercept(self): return self._p.b_w0

    def setDisplacement(self, atom: int, dx: float, dy: float, dz: float):
        self._displ[atom] = (dx, dy, dz)
        self._displ_dirty = True

    def getDisplacement(self, atom: int):
        return tuple(float(v) for v in self._displ[atom])

    def getBindE(self) -> float:
        return self._bind_e

    def setBindE(self, v: float):
        self._bind_e = float(v)

    def getPotEnergy(self) -> float:
        return self._pot_e

    def setPotEnergy(self, v: float):
        self._pot_e = float(v)

    def getPerturbationEnergy(self):
        """(u, U0, U1, W, W') of the last evaluation."""
        r = self._last
        if r is None:
            raise RuntimeError("no evaluation yet")
        return (r[capi.R_U], r[capi.R_U0], r[capi.R_U1], r[capi.R_W], r[capi.R_DW])

    # -- group-1 restraints (set through SDMUtils) --------------------------
    def _set_restraints(self, rs: Optional[Restraints]):
        self._restraints = rs
        self._restraints_dirty = True

    def setParameter(self, name: str, value: float):
        """Context.setParameter for SDMRestraintControlParameter (SDMUtils.py:99)."""
        if name != SDMUtils.RestraintControlParameterName:
            raise KeyError(name)
        self._restraint_control = float(value)
        self._control_dirty = True

    def getParameter(self, name: str) -> float:
        if name != SDMUtils.RestraintControlParameterName:
            raise KeyError(name)
        return self._restraint_control

    def getRestraintEnergy(self) -> float:
        """Group-1 restraint energy of the last evaluation (part of getPotEnergy)."""
        return float(self._handle.restraint_energies()[0]) if self._handle is not None else 0.0

    # -- evaluation -------------------------------------------------------
    def _system(self) -> SDMSystem:
        n = len(self._q)
        # exclusions: addExclusion pairs and every exception pair, each once
        seen, pairs = set(), []
        for i, j in list(self._excl) + [(e[0], e[1]) for e in self._exc]:
            key = (min(i, j), max(i, j))
            if key not in seen:
                seen.add(key)
                pairs.append((i, j))
        ex = np.array(pairs, np.int32).reshape(-1, 2)
        live = [e for e in self._exc if e[2] != 0.0 or e[4] != 0.0]
        xp = np.array([e[:2] for e in live], np.int32).reshape(-1, 2) if live else None
        xprm = np.array([e[2:] for e in live], np.float64).reshape(-1, 3) if live else None
        return SDMSystem("SDMForce", self._box.copy(), np.array(self._q), np.array(self._sig),
                         np.array(self._eps), ex, self._displ[:n].copy(), np.zeros((1, n, 3)),
                         [self._p], cutoff=self._cutoff, eps_rf=self._eps_rf, exceptions=xp,
                         exception_params=xprm,
                         nonbonded_method="pme" if self._method == SDMForce.PME else "rf",
                         ewald_tolerance=self._ewald_tol, pme_grid=self._pme_grid)

    def _sync(self, device: int = 0):
        if self._topology_dirty or self._handle is None:
            if self._handle is not None:
                self._handle.close()
            self._handle = capi.Handle([self._system()], device=device)
            self._topology_dirty = False
            self._displ_dirty = False
            self._params_dirty = True
            self._restraints_dirty = self._restraints is not None
            self._control_dirty = self._restraint_control != 1.0
        if self._displ_dirty:
            self._handle.set_displacement(0, self._displ[:len(self._q)])
            self._displ_dirty = False
        if self._params_dirty:
            if self._p.softcore_method not in (0, 1, 2):
                raise capi.SdmError(capi.SDM_ERR_UNKNOWN_METHOD, "Unknown soft core method")
            self._handle.set_params(0, self._p.as_array())
            self._params_dirty = False
        if self._restraints_dirty:
            self._handle.set_restraints(0, self._restraints)
            self._restraints_dirty = False
        if self._control_dirty:
            self._handle.set_restraint_control(0, self._restraint_control)
            self._control_dirty = False

    def evaluate(self, positions, device: int = 0):
        """Returns (E_pot, forces[N,3]) of the nonbonded group, FP64."""
        self._sync(device)
        res, f = self._handle.evaluate(np.asarray(positions, np.float64).reshape(-1, 3))
        r = res[0]
        self._last = r
        self._bind_e = float(r[capi.R_BINDE])
        self._pot_e = float(r[capi.R_EPOT])
        return self._pot_e, f

    def close(self):
        if self._handle is not None:
            self._handle.close()
            self._handle = None


class LangevinIntegratorSDM(SDMForce):
    """Host mirror of the reference integrator (``LangevinIntegratorSDM.h``,
    ``openmmapi/src/LangevinIntegratorSDM.cpp``): the SDM parameters of
    :class:`SDMForce` plus temperature (K), friction (1/ps), step size (ps) and
    random seed.  ``step(n)`` advances positions and velocities on the GPU:
    per step the two-state evaluation and the stochastic-dynamics update
    (``sdm_langevin_step``, one CUDA graph per step, no host synchronisation).
    Masses come from ``setParticleMass`` (0 holds a particle fixed, as a zero
    mass does in the reference).  Constraints: rigid 3-site waters
    (``setRigidWaters``, SETTLE on the device); other constraints are not
    applied."""

    def __init__(self, temperature: float, frictionCoeff: float, stepSize: float, nParticles: int = 0):
        self._mass = []
        super().__init__(nParticles)
        self._temperature = float(temperature)
        self._friction = float(frictionCoeff)
        self._step_size = float(stepSize)
        self._seed = 0
        self._lv_dirty = True
        self._step_count = 0
        self._time = 0.0             # ps, the context time of the reference integrator
        self._x = self._v = self._im = self._res = None
        self._waters = None          # rigid waters: ((W, 3) O H H, d_oh, d_hh)
        self._waters_dirty = False

    def addParticle(self, charge: float, sigma: float, epsilon: float, mass: float = 1.0) -> int:
        k = super().addParticle(charge, sigma, epsilon)
        self._mass.append(float(mass))
        return k

    def setParticleMass(self, index: int, mass: float):
        self._mass[index] = float(mass)
        self._im = None

    def getParticleMass(self, index: int) -> float:
        return self._mass[index]

    def setTemperature(self, t): self._temperature = float(t); self._lv_dirty = True
    def getTemperature(self): return self._temperature
    def setFriction(self, f): self._friction = float(f); self._lv_dirty = True
    def getFriction(self): return self._friction
    def setStepSize(self, dt): self._step_size = float(dt); self._lv_dirty = True
    def getStepSize(self): return self._step_size
    def setRandomNumberSeed(self, seed): self._seed = int(seed); self._lv_dirty = True
    def getRandomNumberSeed(self): return self._seed
    def setTime(self, t): self._time = float(t)
    def getTime(self): return self._time

    def setRigidWaters(self, waters, d_oh: float, d_hh: float):
        """Holds the (O, H, H) waters rigid in step() (the reference context's
        constraints on them; SETTLE on the device).  waters: (W, 3) indices or
        None to remove."""
        self._waters = None if waters is None else (np.asarray(waters, np.int32).reshape(-1, 3), float(d_oh),
                                                     float(d_hh))
        self._waters_dirty = True

    def _sync(self, device: int = 0):
        rebuilt = self._topology_dirty or self._handle is None
        super()._sync(device)
        if rebuilt:   # a new handle holds neither the waters nor the Langevin parameters
            self._waters_dirty = self._waters is not None
            self._lv_dirty = True
        if self._waters_dirty:
            if self._waters is None:
                self._handle.set_rigid_waters(0, None)
            else:
                self._handle.set_rigid_waters(0, *self._waters)
            self._waters_dirty = False

    def setState(self, positions, velocities=None, device: int = 0):
        """Uploads positions (and velocities, default zero), FP64 (N, 3)."""
        import torch
        x = np.ascontiguousarray(np.asarray(positions, np.float64).reshape(-1, 3))
        v = np.zeros_like(x) if velocities is None else np.asarray(velocities, np.float64).reshape(-1, 3)
        n = len(self._q)
        if x.shape[0] != n or v.shape != x.shape:
            raise ValueError(f"positions and velocities must be ({n}, 3)")
        dev = torch.device("cuda", device)
        self._x = torch.from_numpy(x.copy()).to(dev)
        self._v = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
        self._res = torch.zeros((1, capi.NRESULTS), dtype=torch.float64, device=dev)
        self._im = None

    def getState(self):
        """(positions, velocities) as host FP64 arrays."""
        import torch
        torch.cuda.synchronize(self._x.device)
        return self._x.cpu().numpy(), self._v.cpu().numpy()

    def step(self, steps: int = 1):
        """Advances `steps` steps.  With setNonEquilibrium(1) each step is one
        call, as in the reference kernel (ReferenceSDMKernels.cpp:229-245,
        289-302): lambda = t / Ntmax at the start of the step, lambda1,
        lambda2, u0 and w0 of the schedule written back, and the work value
        raised by (dt / Ntmax) dW/dlambda."""
        if self._x is None:
            raise RuntimeError("setState first")
        if int(self._p.noneq) != 1:
            self._advance(int(steps))
            return
        if not self._ntmax > 0.0:
            raise ValueError("non-equilibrium steps need setNoneqtmax(t) with t > 0")
        for _ in range(int(steps)):
            self._p.lambdac = self._time / self._ntmax
            self._params_dirty = True
            r = self._advance(1)
            self._p.lambda1, self._p.lambda2 = float(r[capi.R_L1]), float(r[capi.R_L2])
            self._p.u0, self._p.w0 = float(r[capi.R_U0P]), float(r[capi.R_W0P])
            self._work += self._step_size / self._ntmax * float(r[capi.R_DWDL])

    def _advance(self, steps: int):
        """`steps` fused steps on the device; returns the results of the last."""
        import torch
        # the kernels take raw pointers: the resident buffers must match the
        # particle count (a particle added after setState would not)
        n = len(self._q)
        if self._x.shape[0] != n or self._v.shape[0] != n:
            raise ValueError(f"the state holds {self._x.shape[0]} particles, the system {n}: call setState")
        self._sync(self._x.device.index or 0)
        if self._im is None:
            m = np.asarray(self._mass[:len(self._q)], np.float64)
            im = np.where(m > 0, 1.0 / np.where(m > 0, m, 1.0), 0.0)
            self._im = torch.from_numpy(im).to(self._x.device)
        if self._lv_dirty:
            self._handle.set_langevin(self._step_size, self._friction, self._temperature, self._seed,
                                      self._step_count)
            self._lv_dirty = False
        self._handle.langevin_step(self._x.data_ptr(), self._v.data_ptr(), self._im.data_ptr(),
                                   self._res.data_ptr(), int(steps),
                                   stream=torch.cuda.current_stream(self._x.device).cuda_stream)
        self._step_count += int(steps)
        self._time += int(steps) * self._step_size
        r = self._res[0].cpu().numpy()
        self._last = r
        self._bind_e = float(r[capi.R_BINDE])
        self._pot_e = float(r[capi.R_EPOT])
        return r


class SDMUtils:
    """Host mirror of the reference's SDMUtils (python/SDMUtils.py) for a
    mirror force (SDMForce or LangevinIntegratorSDM): the same method names,
    argument names and meanings, with plain numbers in OpenMM's internal
    units (nm, rad, kJ/mol) where the reference takes unit quantities.  The
    restraints are evaluated on the device in the same call as the SDM force
    (group 1 of the reference).  The centroids are mass weighted (the
    reference's CustomCentroidBondForce default) when the force has masses
    (LangevinIntegratorSDM), equally weighted otherwise.  One centroid
    restraint and one alignment restraint per force."""
    RestraintControlParameterName = "SDMRestraintControlParameter"
    LinearMethod, QuadraticMethod, ILogisticMethod = 0, 1, 2
    NoSoftCoreMethod, TanhSoftCoreMethod, RationalSoftCoreMethod = 0, 1, 2

    def __init__(self, force: SDMForce):
        self.force = force
        self._cm = None      # fields of the centroid restraint
        self._align = None   # fields of the alignment restraint

    def getControlParameterName(self) -> str:
        return self.RestraintControlParameterName

    def _weights(self, particles):
        m = getattr(self.force, "_mass", None)
        return None if m is None else [m[i] for i in particles]

    def _push(self):
        fields = {}
        if self._cm:
            fields.update(self._cm)
        if self._align:
            fields.update(self._align)
        self.force._set_restraints(Restraints(**fields) if fields else None)

    def addRestraintForce(self, lig_cm_particles=None, rcpt_cm_particles=None, kfcm=0.0, tolcm=0.0,
                          lig_ref_particles=None, rcpt_ref_particles=None, angle_center=0.0, kfangle=0.0,
                          angletol=math.radians(10.0), dihedral1center=0.0, kfdihedral1=0.0,
                          dihedral1tol=math.radians(10.0), dihedral2center=0.0, kfdihedral2=0.0,
                          dihedral2tol=math.radians(10.0), offset=(0.0, 0.0, 0.0)):
        """SDMUtils.addRestraintForce (python/SDMUtils.py:32-157)."""
        if not (lig_cm_particles and rcpt_cm_particles):
            return
        if self._cm is not None:
            raise NotImplementedError("one centroid restraint per force")
        do_angles = False
        if lig_ref_particles and rcpt_ref_particles:
            if not (len(lig_ref_particles) == 3 and len(rcpt_ref_particles) == 3):
                raise ValueError("Invalid lists of reference atoms")
            do_angles = True
        lig, rcpt = [int(i) for i in lig_cm_particles], [int(i) for i in rcpt_cm_particles]
        self._cm = dict(lig_particles=lig, rcpt_particles=rcpt, lig_weights=self._weights(lig),
                        rcpt_weights=self._weights(rcpt), kfcm=float(kfcm), tolcm=float(tolcm),
                        offset=tuple(float(v) for v in offset), use_angles=do_angles)
        if do_angles:
            self._cm.update(rcpt_ref=tuple(int(i) for i in rcpt_ref_particles),
                            lig_ref=tuple(int(i) for i in lig_ref_particles),
                            kf_angle=float(kfangle), angle_center=float(angle_center), angle_tol=float(angletol),
                            kf_dihedral1=float(kfdihedral1), dihedral1_center=float(dihedral1center),
                            dihedral1_tol=float(dihedral1tol), kf_dihedral2=float(kfdihedral2),
                            dihedral2_center=float(dihedral2center), dihedral2_tol=float(dihedral2tol))
        self._push()

    def addAlignmentForce(self, liga_ref_particles=None, ligb_ref_particles=None, kfdispl=0.0, ktheta=0.0,
                          kpsi=0.0, offset=(0.0, 0.0, 0.0)):
        """SDMUtils.addAlignmentForce (python/SDMUtils.py:160-257)."""
        if not (liga_ref_particles and ligb_ref_particles):
            raise ValueError("Invalid lists of reference atoms")
        if not (len(liga_ref_particles) == 3 and len(ligb_ref_particles) == 3):
            raise ValueError("Invalid lists of reference atoms")
        if self._align is not None:
            raise NotImplementedError("one alignment restraint per force")
        self._align = dict(use_alignment=True, liga_ref=tuple(int(i) for i in liga_ref_particles),
                           ligb_ref=tuple(int(i) for i in ligb_ref_particles), kf_displ=float(kfdispl),
                           k_theta=float(ktheta), k_psi=float(kpsi),
                           align_offset=tuple(float(v) for v in offset))
        self._push()


def _fill_from_system(f: SDMForce, s: SDMSystem, replica: int, masses=None) -> SDMForce:
    for k, (q, sg, ep) in enumerate(zip(s.charge, s.sigma, s.epsilon)):
        if masses is None:
            f.addParticle(q, sg, ep)
        else:
            f.addParticle(q, sg, ep, mass=float(masses[k]))
    for i, j in np.asarray(s.exclusions).reshape(-1, 2):
        f.addExclusion(int(i), int(j))
    if s.exceptions is not None:
        for (i, j), (qq, sg, ep) in zip(np.asarray(s.exceptions).reshape(-1, 2),
                                        np.asarray(s.exception_params).reshape(-1, 3)):
            f.addException(int(i), int(j), float(qq), float(sg), float(ep))
    f.setNonbondedMethod(SDMForce.PME if s.nonbonded_method == "pme" else SDMForce.CutoffPeriodic)
    f.setEwaldErrorTolerance(s.ewald_tolerance)
    f._pme_grid = None if s.pme_grid is None else tuple(int(v) for v in s.pme_grid)
    f.setCutoffDistance(s.cutoff)
    f.setReactionFieldDielectric(s.eps_rf)
    f.setPeriodicBoxVectors((s.box[0], 0, 0), (0, s.box[1], 0), (0, 0, s.box[2]))
    for i in np.nonzero(np.any(s.displacement != 0, axis=1))[0]:
        f.setDisplacement(int(i), *s.displacement[i])
    f._p = dataclasses.replace(s.params[replica])
    f._params_dirty = True
    return f


def force_from_system(s: SDMSystem, replica: int = 0) -> SDMForce:
    """Builds an SDMForce from a system (synthetic or read by dms.read_dms):
    particles, exclusions, exceptions, electrostatics, box, displacement and
    the SDM parameters of `replica`."""
    return _fill_from_system(SDMForce(), s, replica)


def integrator_from_system(s: SDMSystem, temperature: float, frictionCoeff: float, stepSize: float,
                           replica: int = 0) -> "LangevinIntegratorSDM":
    """A LangevinIntegratorSDM mirror for a system, as the reference's example
    builds LangevinIntegratorSDM(temperature, friction, step size, N) and sets
    its SDM parameters and displacements (example/test.py:172-188).  Masses
    come from s.masses (required)."""
    if s.masses is None:
        raise ValueError("the system has no masses (SDMSystem.masses)")
    return _fill_from_system(LangevinIntegratorSDM(temperature, frictionCoeff, stepSize), s, replica,
                             masses=np.asarray(s.masses, np.float64))
