"""GPU tests of the fused Langevin step (sdm_langevin_step) against the
restated stochastic-dynamics update of the oracle
(ReferenceStochasticDynamicsSDM.cpp:131-266 on the hybrid force of
ReferenceSDMKernels.cpp:309-318)."""
import numpy as np
import pytest

import oracle
from openmm_sdm_plugin_gb300 import capi, systems as S

pytestmark = pytest.mark.gpu

DT, FRICTION = 0.002, 5.0


def _setup(nrep=2, seed=11):
    import torch
    s = S.config2(nrep=nrep)
    h = capi.Handle([s])
    for r, p in enumerate(s.params):
        h.set_params(r, p.as_array())
    rng = np.random.default_rng(seed)
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    n = x.shape[0]
    v = rng.normal(scale=0.5, size=(n, 3))
    im = 1.0 / rng.uniform(1.0, 16.0, n)
    im[rng.choice(n, 50, replace=False)] = 0.0    # fixed particles
    fext = rng.normal(scale=10.0, size=(n, 3))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return s, h, x, v, im, fext, dev


def test_langevin_step_matches_restated_update_at_zero_temperature():
    import torch
    s, h, x, v, im, fext, dev = _setup()
    res_h, F = h.evaluate(x)                      # the SDM force at x
    h.set_langevin(DT, FRICTION, 0.0, seed=5)
    xd, vd, imd, fd = dev(x), dev(v), dev(im), dev(fext)
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    h.langevin_step(xd.data_ptr(), vd.data_ptr(), imd.data_ptr(), rd.data_ptr(), 1, fd.data_ptr())
    torch.cuda.synchronize()
    xo, vo = oracle.langevin_update(x, v, im, F + fext, DT, FRICTION, 0.0)
    assert np.array_equal(xd.cpu().numpy(), xo)
    assert np.array_equal(vd.cpu().numpy(), vo)
    assert np.array_equal(rd.cpu().numpy()[:, :14], res_h[:, :14])   # energies at the start point
    assert h.check_status() == 0


def test_langevin_noise_is_standard_normal_and_fresh_each_step():
    import torch
    s, h, x, v, im, fext, dev = _setup(nrep=1)
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    imd = dev(im)

    def one(T, step):
        h.set_langevin(DT, FRICTION, T, seed=123, step=step)
        xd, vd = dev(x), dev(v)
        h.langevin_step(xd.data_ptr(), vd.data_ptr(), imd.data_ptr(), rd.data_ptr(), 1)
        torch.cuda.synchronize()
        return vd.cpu().numpy()

    v0 = one(0.0, 0)
    _, _, ns = oracle.langevin_coefficients(DT, FRICTION, 300.0)
    mv = im != 0
    scale = ns * np.sqrt(im[mv])[:, None]
    n_a = ((one(300.0, 0) - v0)[mv] / scale).reshape(-1)
    n_b = ((one(300.0, 1) - v0)[mv] / scale).reshape(-1)
    n_a2 = ((one(300.0, 0) - v0)[mv] / scale).reshape(-1)
    m = n_a.size
    assert abs(n_a.mean()) < 5.0 / np.sqrt(m)
    assert abs(n_a.var() - 1.0) < 6.0 * np.sqrt(2.0 / m)
    assert abs(np.mean(n_a ** 3)) < 6.0 * np.sqrt(15.0 / m)           # symmetric
    assert abs(np.mean(n_a ** 4) - 3.0) < 6.0 * np.sqrt(96.0 / m)      # Gaussian tails
    assert abs(np.corrcoef(n_a, n_b)[0, 1]) < 5.0 / np.sqrt(m)         # other step: fresh deviates
    assert np.allclose(n_a, n_a2, atol=1e-6)                           # same (seed, step): same deviates


def test_langevin_steps_chain_and_fixed_particles():
    import torch
    s, h, x, v, im, fext, dev = _setup()
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    imd, fd = dev(im), dev(fext)
    h.set_langevin(DT, FRICTION, 300.0, seed=9, step=40)
    xa, va = dev(x), dev(v)
    h.langevin_step(xa.data_ptr(), va.data_ptr(), imd.data_ptr(), rd.data_ptr(), 3, fd.data_ptr())
    h.set_langevin(DT, FRICTION, 300.0, seed=9, step=40)
    xb, vb = dev(x), dev(v)
    for _ in range(3):   # graph replays, the device step counter advances
        h.langevin_step(xb.data_ptr(), vb.data_ptr(), imd.data_ptr(), rd.data_ptr(), 1, fd.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(xa.cpu().numpy(), xb.cpu().numpy())
    assert np.array_equal(va.cpu().numpy(), vb.cpu().numpy())
    fixed = im == 0
    assert np.array_equal(xa.cpu().numpy()[fixed], x[fixed])
    assert np.array_equal(va.cpu().numpy()[fixed], v[fixed])
    moved = np.abs(xa.cpu().numpy() - x).max(axis=1)
    assert (moved[~fixed] > 0).all() and np.isfinite(moved).all()
    # the energies are those of the last step's start point
    assert np.isfinite(rd.cpu().numpy()[:, :14]).all()
    assert h.check_status() == 0


def test_langevin_parameter_checks():
    s, h, *_ = _setup(nrep=1)
    for bad in ((0.0, 1.0, 300.0), (0.002, 0.0, 300.0), (0.002, 1.0, -1.0)):
        with pytest.raises(capi.SdmError):
            h.set_langevin(*bad)


def test_integrator_mirror_chains_steps_like_the_restated_update():
    """LangevinIntegratorSDM (host mirror of the reference integrator): three
    T = 0 steps equal three restated updates, each on the force the library
    evaluates at the current positions."""
    from openmm_sdm_plugin_gb300.force import LangevinIntegratorSDM, force_from_system
    s = S.config0(variant="b")
    ref = force_from_system(s)
    integ = LangevinIntegratorSDM(0.0, 2.0, 0.001)
    for q, sg, ep in zip(s.charge, s.sigma, s.epsilon):
        integ.addParticle(q, sg, ep, mass=14.0)
    for i, j in s.exclusions:
        integ.addExclusion(int(i), int(j))
    integ.setCutoffDistance(s.cutoff)
    integ.setReactionFieldDielectric(s.eps_rf)
    integ.setPeriodicBoxVectors((s.box[0], 0, 0), (0, s.box[1], 0), (0, 0, s.box[2]))
    for i in np.nonzero(np.any(s.displacement != 0, axis=1))[0]:
        integ.setDisplacement(int(i), *s.displacement[i])
    integ._p = ref._p
    integ.setParticleMass(0, 0.0)     # held fixed
    rng = np.random.default_rng(3)
    x = s.positions[0].copy()
    v = rng.normal(scale=0.2, size=x.shape)
    integ.setState(x, v)
    integ.step(3)
    xg, vg = integ.getState()
    im = np.full(s.n, 1.0 / 14.0)
    im[0] = 0.0
    for _ in range(3):
        _, F = ref.evaluate(x)
        x, v = oracle.langevin_update(x, v, im, F, 0.001, 2.0, 0.0)
    assert np.array_equal(xg, x)
    assert np.array_equal(vg, v)
    assert np.isfinite(integ.getPerturbationEnergy()).all()
    assert np.isfinite(integ.getBindE()) and np.isfinite(integ.getPotEnergy())
    integ.close()
    ref.close()


def _rigid_setup(nrep=2):
    s, h, x, v, im, fext, dev = _setup(nrep=nrep)
    w, d_oh, d_hh = S.rigid_waters(s)
    # model masses (O 15.999, H 1.008) on the waters, a few ligand particles fixed
    m = np.full(x.shape[0], 12.011)
    for r in range(nrep):
        base = r * s.n
        m[base + w[:, 0]] = 15.999
        m[base + w[:, 1]] = m[base + w[:, 2]] = 1.008
    im = 1.0 / m
    for r in range(nrep):
        im[r * s.n + s.n - 5:r * s.n + s.n] = 0.0
    h.set_rigid_waters(0, w, d_oh, d_hh)
    return s, h, x, v, im, fext, dev, (w, d_oh, d_hh)


def _all_waters(s, w, nrep):
    return np.concatenate([w + r * s.n for r in range(nrep)])


def test_rigid_waters_step_matches_shake_oracle():
    """T = 0 step with SETTLE on every water of two replicas against the
    oracle's SHAKE iterated to convergence (the same constraint problem);
    waters that straddle the box boundary included."""
    import torch
    s, h, x, v, im, fext, dev, (w, d_oh, d_hh) = _rigid_setup()
    ws = _all_waters(s, w, 2)
    # translate and wrap particle by particle (the physics is unchanged):
    # waters cut by the box faces now straddle them
    x = x + np.array([0.5, 0.37, 0.21]) * s.box
    x = x - s.box * np.floor(x / s.box)
    straddle = np.abs(x[ws[:, 1:]] - x[ws[:, :1]]).max(axis=(1, 2)) > 0.5 * s.box.min()
    assert straddle.sum() > 10
    _, F = h.evaluate(x)
    h.set_langevin(DT, FRICTION, 0.0, seed=5)
    xd, vd, imd, fd = dev(x), dev(v), dev(im), dev(fext)
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    h.langevin_step(xd.data_ptr(), vd.data_ptr(), imd.data_ptr(), rd.data_ptr(), 1, fd.data_ptr())
    torch.cuda.synchronize()
    xo, vo = oracle.langevin_update(x, v, im, F + fext, DT, FRICTION, 0.0, waters=ws, d_oh=d_oh, d_hh=d_hh,
                                    box=s.box)
    xg, vg = xd.cpu().numpy(), vd.cpu().numpy()
    assert np.abs(xg - xo).max() < 1e-11
    assert np.abs(vg - vo).max() < 1e-7
    others = np.setdiff1d(np.arange(x.shape[0]), ws.reshape(-1))
    assert np.array_equal(xg[others], xo[others]) and np.array_equal(vg[others], vo[others])
    assert h.check_status() == 0


def test_rigid_waters_stay_rigid_over_steps():
    import torch
    s, h, x, v, im, fext, dev, (w, d_oh, d_hh) = _rigid_setup()
    h.set_langevin(DT, FRICTION, 300.0, seed=3)
    xd, vd, imd = dev(x), dev(v * 0.0), dev(im)
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    h.langevin_step(xd.data_ptr(), vd.data_ptr(), imd.data_ptr(), rd.data_ptr(), 20)
    torch.cuda.synchronize()
    xg = xd.cpu().numpy()
    ws = _all_waters(s, w, 2)

    def dist(i, j):
        d = xg[ws[:, i]] - xg[ws[:, j]]
        d -= s.box * np.round(d / s.box)
        return np.linalg.norm(d, axis=1)
    assert np.abs(dist(0, 1) - d_oh).max() < 1e-10
    assert np.abs(dist(0, 2) - d_oh).max() < 1e-10
    assert np.abs(dist(1, 2) - d_hh).max() < 1e-10
    assert np.isfinite(rd.cpu().numpy()[:, :14]).all() and h.check_status() == 0


def test_rigid_water_input_checks():
    s, h, *_ = _setup(nrep=1)
    w, d_oh, d_hh = S.rigid_waters(s)
    for bad in ((np.array([[0, 1, s.n]]), d_oh, d_hh), (np.array([[0, 1, 2], [2, 3, 4]]), d_oh, d_hh),
                (w, d_oh, 2.5 * d_oh), (w, -d_oh, d_hh)):
        with pytest.raises(capi.SdmError):
            h.set_rigid_waters(0, *bad)
    h.set_rigid_waters(0, w, d_oh, d_hh)
    h.set_rigid_waters(0, None)   # removes them


def test_integrator_mirror_rigid_waters():
    """LangevinIntegratorSDM.setRigidWaters: a T = 0 step of the mirror equals
    the oracle's update with SHAKE on the same waters, and the waters stay
    rigid over noisy steps."""
    from openmm_sdm_plugin_gb300.force import LangevinIntegratorSDM, force_from_system
    s = S.config2(nrep=1)
    w, d_oh, d_hh = S.rigid_waters(s)
    m = np.full(s.n, 12.011)
    m[w[:, 0]] = 15.999
    m[w[:, 1]] = m[w[:, 2]] = 1.008
    ref = force_from_system(s)
    integ = LangevinIntegratorSDM(0.0, FRICTION, DT)
    for k, (q, sg, ep) in enumerate(zip(s.charge, s.sigma, s.epsilon)):
        integ.addParticle(q, sg, ep, mass=m[k])
    for i, j in s.exclusions:
        integ.addExclusion(int(i), int(j))
    integ.setCutoffDistance(s.cutoff)
    integ.setReactionFieldDielectric(s.eps_rf)
    integ.setPeriodicBoxVectors((s.box[0], 0, 0), (0, s.box[1], 0), (0, 0, s.box[2]))
    for i in np.nonzero(np.any(s.displacement != 0, axis=1))[0]:
        integ.setDisplacement(int(i), *s.displacement[i])
    integ._p = ref._p
    integ.setRigidWaters(w, d_oh, d_hh)
    x = s.positions[0].copy()
    v = np.random.default_rng(4).normal(scale=0.3, size=x.shape)
    integ.setState(x, v)
    integ.step(1)
    xg, vg = integ.getState()
    _, F = ref.evaluate(x)
    xo, vo = oracle.langevin_update(x, v, 1.0 / m, F, DT, FRICTION, 0.0, waters=w, d_oh=d_oh, d_hh=d_hh,
                                    box=s.box)
    assert np.abs(xg - xo).max() < 1e-11
    assert np.abs(vg - vo).max() < 1e-7
    integ.setTemperature(300.0)
    integ.step(10)
    xg, _ = integ.getState()
    for a, b, d0 in ((0, 1, d_oh), (0, 2, d_oh), (1, 2, d_hh)):
        d = xg[w[:, a]] - xg[w[:, b]]
        d -= s.box * np.round(d / s.box)
        assert np.abs(np.linalg.norm(d, axis=1) - d0).max() < 1e-10
    assert np.isfinite(integ.getBindE()) and np.isfinite(integ.getPotEnergy())
    integ.close()
    ref.close()


def test_langevin_steps_equal_in_every_branch_mode():
    """Three steps at 300 K with the graph's second branch joined after the
    main pass (default), before it, and with one stream: the same positions,
    velocities and results bit for bit (same seed and step counter)."""
    import torch
    s, h, x, v, im, fext, dev = _setup()
    imd, fd = dev(im), dev(fext)
    out = {}
    for ov in (2, 1, 0):
        h.set_option(capi.OPT_OVERLAP, ov)
        h.set_langevin(DT, FRICTION, 300.0, seed=3, step=7)
        xa, va = dev(x), dev(v)
        rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
        h.langevin_step(xa.data_ptr(), va.data_ptr(), imd.data_ptr(), rd.data_ptr(), 3, fd.data_ptr())
        torch.cuda.synchronize()
        out[ov] = (xa.cpu().numpy(), va.cpu().numpy(), rd.cpu().numpy())
    for ov in (1, 0):
        for a, b in zip(out[ov], out[2]):
            assert np.array_equal(a, b), ov
    assert h.check_status() == 0
