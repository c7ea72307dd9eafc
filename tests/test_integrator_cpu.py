"""Host logic of the integrator mirror's non-equilibrium protocol
(LangevinIntegratorSDM.step with setNonEquilibrium(1)), with the device step
replaced by the oracle's combine on fixed state energies: per step
lambda = t / Ntmax at the start of the step, the schedule's lambda1, lambda2,
u0, w0 written back, and the work raised by (dt / Ntmax) dW/dlambda
(ReferenceSDMKernels.cpp:229-245, 289-302)."""
import math

import numpy as np
import pytest

import oracle
from openmm_sdm_plugin_gb300 import capi, systems as S
from openmm_sdm_plugin_gb300.force import LangevinIntegratorSDM

P_LAMBDA = 2          # SDM_P_LAMBDA
U0, U1 = -1000.0, -960.0
SCHEDULE = dict(m1=0.5, b1=0.1, m2=0.8, b2=0.1, mu0=10.0, bu0=30.0, mw0=2.0, bw0=-1.0)


def _integrator(dt=0.002, ntmax=0.01):
    integ = LangevinIntegratorSDM(300.0, 1.0, dt)
    integ.setBiasMethod(S.ILOGISTIC)
    integ.setSoftCoreMethod(S.NO_SOFTCORE)
    integ.setAlpha(0.1)
    integ.setNonEquilibrium(1)
    integ.setNoneqtmax(ntmax)
    c = SCHEDULE
    integ.setlambda1Slope(c["m1"]); integ.setlambda1intercept(c["b1"])
    integ.setlambda2Slope(c["m2"]); integ.setlambda2intercept(c["b2"])
    integ.setu0Slope(c["mu0"]); integ.setu0intercept(c["bu0"])
    integ.setw0Slope(c["mw0"]); integ.setw0intercept(c["bw0"])
    return integ


def _fake_device(integ, seen):
    """Stand-in for one fused device step: records the lambda it was given
    and returns the oracle's combine of (U0, U1) in the results layout."""
    def advance(steps):
        assert steps == 1
        p = integ._p.as_array().copy()
        seen.append(p[P_LAMBDA])
        c = dict(zip(oracle.COMBINE_FIELDS, oracle.combine(p, U0, U1)))
        r = np.zeros(capi.NRESULTS)
        r[capi.R_DWDL], r[capi.R_L1], r[capi.R_L2] = c["dWdlambda"], c["lambda1"], c["lambda2"]
        r[capi.R_U0P], r[capi.R_W0P] = c["u0"], c["w0"]
        integ._time += integ._step_size
        return r
    return advance


def _dw_dlambda(lam, alpha=0.1):
    # the reference's analytic derivative, restated (ReferenceSDMKernels.cpp:289-302)
    c = SCHEDULE
    l1, l2, u0 = c["m1"] * lam + c["b1"], c["m2"] * lam + c["b2"], c["mu0"] * lam + c["bu0"]
    u = U1 - U0
    e = math.exp(-alpha * (u - u0))
    ee = 1.0 + e
    return (-math.log(ee) / alpha * c["m1"] + (u + math.log(ee) / alpha) * c["m2"]
            + (l2 - l1) * e / ee * c["mu0"] + c["mw0"])


def test_non_equilibrium_schedule_and_work(oracle_lib):
    dt, T = 0.002, 0.01
    integ = _integrator(dt, T)
    seen = []
    integ._advance = _fake_device(integ, seen)
    integ._x = object()       # positions resident (the device step is replaced)
    integ.step(5)
    t, lams, work = 0.0, [], 0.0
    for _ in range(5):
        lam = t / T
        lams.append(lam)
        work += dt / T * _dw_dlambda(lam)
        t += dt
    assert seen == lams
    assert integ.getNoneqWorkvalue() == pytest.approx(work, rel=1e-12)
    assert integ.getTime() == t
    c = SCHEDULE
    assert integ.getLambda() == lams[-1]
    assert integ.getLambda1() == pytest.approx(c["m1"] * lams[-1] + c["b1"], rel=1e-15)
    assert integ.getLambda2() == pytest.approx(c["m2"] * lams[-1] + c["b2"], rel=1e-15)
    assert integ.getU0() == pytest.approx(c["mu0"] * lams[-1] + c["bu0"], rel=1e-15)
    assert integ.getW0coeff() == pytest.approx(c["mw0"] * lams[-1] + c["bw0"], rel=1e-15)
    # work continues from the stored value, as setNoneqWorkvalue allows
    integ.setNoneqWorkvalue(1.5)
    integ.step(1)
    assert integ.getNoneqWorkvalue() == pytest.approx(1.5 + dt / T * _dw_dlambda(t / T), rel=1e-12)


def test_non_equilibrium_needs_ntmax():
    integ = _integrator(ntmax=0.0)
    integ._x = object()
    integ._advance = lambda steps: pytest.fail("stepped without Ntmax")
    with pytest.raises(ValueError, match="setNoneqtmax"):
        integ.step(1)


def test_equilibrium_steps_go_in_one_call():
    integ = _integrator()
    integ.setNonEquilibrium(0)
    calls = []
    integ._x = object()
    integ._advance = lambda steps: calls.append(steps)
    integ.step(7)
    assert calls == [7] and integ.getNoneqWorkvalue() == 0.0


class _FakeHandle:
    """Records the configuration calls a mirror makes on its handle."""
    made = []

    def __init__(self, systems, device=0):
        self.calls = []
        _FakeHandle.made.append(self)

    def __getattr__(self, name):
        def call(*args, **kw):
            self.calls.append(name)
        return call


def test_a_rebuilt_handle_gets_the_langevin_parameters_and_waters_again(monkeypatch):
    """A topology change after stepping makes a new handle; the integrator
    mirror sends it the rigid waters at once and the Langevin parameters
    before its next step."""
    from openmm_sdm_plugin_gb300 import force as F
    monkeypatch.setattr(F.capi, "Handle", _FakeHandle)
    _FakeHandle.made = []
    integ = F.LangevinIntegratorSDM(300.0, 1.0, 0.002)
    for _ in range(6):
        integ.addParticle(0.0, 0.3, 0.5, mass=16.0)
    integ.setPeriodicBoxVectors((3, 0, 0), (0, 3, 0), (0, 0, 3))
    integ.setRigidWaters([[0, 1, 2], [3, 4, 5]], 0.09572, 0.15139)
    integ._sync()
    integ._lv_dirty = False          # as after the first step's set_langevin
    integ._sync()                    # nothing changed: same handle, nothing re-sent
    assert len(_FakeHandle.made) == 1 and not integ._lv_dirty
    integ.setCutoffDistance(1.2)     # topology change: a new handle
    integ._sync()
    assert len(_FakeHandle.made) == 2
    assert "set_rigid_waters" in _FakeHandle.made[1].calls and "set_params" in _FakeHandle.made[1].calls
    assert integ._lv_dirty


def test_state_must_match_the_particle_count():
    """The fused step takes raw device pointers, so the mirror refuses a state
    whose size differs from the system's before any device call."""
    integ = LangevinIntegratorSDM(300.0, 1.0, 0.002)
    for _ in range(4):
        integ.addParticle(0.0, 0.3, 0.5, mass=16.0)
    with pytest.raises(ValueError, match=r"\(4, 3\)"):
        integ.setState(np.zeros((3, 3)))
    with pytest.raises(ValueError, match=r"\(4, 3\)"):
        integ.setState(np.zeros((4, 3)), np.zeros((5, 3)))
    integ._x = integ._v = np.zeros((4, 3))   # a state of 4 particles ...
    integ.addParticle(0.0, 0.3, 0.5)         # ... then a fifth particle
    with pytest.raises(ValueError, match="setState"):
        integ.step(1)
