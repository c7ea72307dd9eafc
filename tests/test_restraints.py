"""Group-1 restraints of the reference's SDMUtils (python/SDMUtils.py:32-257)
through the C ABI (sdm_set_restraints) against the oracle's restatement of
the custom-force expressions (oracle.restraint_energy, forces by central
differences): centroid distance, angle and dihedral windows, alignment;
the control parameter; removal; input checks; the fused Langevin step."""
import dataclasses

import numpy as np
import pytest

import oracle
from openmm_sdm_plugin_gb300 import capi, systems as S

pytestmark = pytest.mark.gpu


def _system(nrep=2, seed=4):
    s = S.config0(variant="b")
    rng = np.random.default_rng(seed)
    x0 = s.positions[0]
    pos = np.stack([x0 + (rng.normal(scale=0.01, size=x0.shape) if r else 0.0) for r in range(nrep)])
    return dataclasses.replace(s, positions=pos, params=[s.params[0]] * nrep)


def _restraints(s, x):
    """Every term active at x: centroid tolerance below the distance,
    windows centred 0.5 rad away from the current angle and dihedrals."""
    rng = np.random.default_rng(9)
    lig = np.arange(900, 930)
    c = x[lig].mean(0)
    near = np.argsort(np.linalg.norm(x[:900] - c, axis=1))[:60]
    rcpt = near[20:]
    rcpt_ref, lig_ref = tuple(int(i) for i in near[:3]), (900, 905, 911)
    r0, r1, _ = (x[i] for i in rcpt_ref)
    l0, l1, l2 = (x[i] for i in lig_ref)
    th = oracle._rs_angle(r0, l0, l1)
    p1 = oracle._rs_dihedral(r1, r0, l0, l1)
    p2 = oracle._rs_dihedral(r0, l0, l1, l2)
    wl, wr = rng.uniform(1.0, 16.0, lig.size), rng.uniform(1.0, 16.0, rcpt.size)
    d = np.linalg.norm((wl[:, None] * x[lig]).sum(0) / wl.sum() - np.array([0.1, 0.0, 0.0])
                       - (wr[:, None] * x[rcpt]).sum(0) / wr.sum())
    return S.Restraints(lig_particles=lig, rcpt_particles=rcpt, lig_weights=wl, rcpt_weights=wr,
                        kfcm=800.0, tolcm=0.5 * d, offset=(0.1, 0.0, 0.0),
                        use_angles=True, rcpt_ref=rcpt_ref, lig_ref=lig_ref,
                        kf_angle=120.0, angle_center=th + 0.5, angle_tol=0.1,
                        kf_dihedral1=90.0, dihedral1_center=p1 - 0.5, dihedral1_tol=0.15,
                        kf_dihedral2=60.0, dihedral2_center=p2 + 0.5, dihedral2_tol=0.2,
                        use_alignment=True, liga_ref=(900, 903, 907), ligb_ref=(915, 919, 924),
                        kf_displ=300.0, k_theta=40.0, k_psi=25.0, align_offset=(0.2, -0.1, 0.05))


def _handle(s):
    h = capi.Handle([s])
    for r, p in enumerate(s.params):
        h.set_params(r, p.as_array())
    return h


def _f_tol(ref):
    # restraint forces reach the accumulators as FP32 values (then 2^-32 fixed point)
    return 2e-6 * np.abs(ref).max() + 1e-6


def test_restraint_energies_and_forces_against_oracle():
    s = _system()
    rs = _restraints(s, s.positions[0])
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    h0 = _handle(s)
    res0, F0 = h0.evaluate(x)
    A0, B0 = h0.state_forces()
    h = _handle(dataclasses.replace(s, restraints=rs))
    res, F = h.evaluate(x)
    A, B = h.state_forces()
    e = h.restraint_energies()
    n = s.n
    for r in range(s.replicas):
        xr = s.positions[r]
        eo = oracle.restraint_energy(xr, rs)
        assert eo > 1.0   # every term contributes at these coordinates
        assert abs(e[r] - eo) < 1e-9 * abs(eo)
        assert abs((res[r, capi.R_EPOT] - res0[r, capi.R_EPOT]) - eo) < 1e-9 * abs(eo) + 1e-9
        # the SDM energies themselves are untouched
        assert res[r, capi.R_U0] == res0[r, capi.R_U0] and res[r, capi.R_U] == res0[r, capi.R_U]
        fo = oracle.restraint_forces(xr, rs)
        sl = slice(r * n, (r + 1) * n)
        tol = _f_tol(fo)
        assert np.abs((F[sl] - F0[sl]) - fo).max() < tol
        assert np.abs((A[sl] - A0[sl]) - fo).max() < tol     # state 0
        assert np.abs((B[sl] - B0[sl]) - fo).max() < tol     # state 1: the same group-1 force
    assert res[0, capi.R_STATUS] == 0


def test_control_parameter_scales_the_centroid_terms_only():
    s = _system()
    rs = _restraints(s, s.positions[0])
    h = _handle(dataclasses.replace(s, restraints=rs))
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    h.set_restraint_control(1, 0.25)
    h.evaluate(x)
    e = h.restraint_energies()
    align = dataclasses.replace(rs, lig_particles=(), rcpt_particles=(), use_angles=False)
    for r, lam in ((0, 1.0), (1, 0.25)):
        xr = s.positions[r]
        full = oracle.restraint_energy(xr, rs, control=lam)
        assert abs(e[r] - full) < 1e-9 * abs(full)
        # only the alignment part survives lambda_r = 0
        ea = oracle.restraint_energy(xr, align)
        assert abs(full - ea - lam * (oracle.restraint_energy(xr, rs) - ea)) < 1e-9 * abs(full)


def test_removing_restraints_and_graph_replay():
    import torch
    s = _system(nrep=1)
    rs = _restraints(s, s.positions[0])
    h = _handle(dataclasses.replace(s, restraints=rs))
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    xd = torch.from_numpy(x).cuda()
    rd = torch.zeros((1, capi.NRESULTS), dtype=torch.float64, device="cuda")
    fd = torch.zeros_like(xd)
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(2):   # capture, then replay
        h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), st)
    torch.cuda.synchronize()
    with_r = rd.cpu().numpy().copy()
    h.set_restraints(0, None)   # drops the cached graphs: the next call captures anew
    h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), st)
    torch.cuda.synchronize()
    h0 = _handle(s)
    res0, F0 = h0.evaluate(x)
    assert np.array_equal(rd.cpu().numpy()[:, :14], res0[:, :14])
    assert np.array_equal(fd.cpu().numpy(), F0)
    assert abs(with_r[0, capi.R_EPOT] - res0[0, capi.R_EPOT] - oracle.restraint_energy(x, rs)) < 1e-6
    assert np.all(h.restraint_energies() == 0.0)


def test_restraint_input_checks():
    s = _system(nrep=1)
    h = _handle(s)
    x0 = s.positions[0]
    good = _restraints(s, x0)
    for bad in (dataclasses.replace(good, lig_particles=(0, s.n)),
                dataclasses.replace(good, lig_weights=np.full(30, -1.0)),
                dataclasses.replace(good, tolcm=-0.1),
                dataclasses.replace(good, liga_ref=(0, 1, s.n)),
                dataclasses.replace(good, lig_particles=(), rcpt_particles=()),   # angles without groups
                dataclasses.replace(good, kfcm=float("nan"))):
        with pytest.raises(capi.SdmError):
            h.set_restraints(0, bad)
    with pytest.raises(capi.SdmError):
        h.set_restraint_control(5, 1.0)
    h.set_restraints(0, good)
    res, _ = h.evaluate(x0)
    assert res[0, capi.R_STATUS] == 0


def test_langevin_step_includes_the_restraint_forces():
    import torch
    s = dataclasses.replace(_system(nrep=1), restraints=None)
    rs = _restraints(s, s.positions[0])
    s = dataclasses.replace(s, restraints=rs)
    h = _handle(s)
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    _, F = h.evaluate(x)     # SDM force + restraint forces at x
    rng = np.random.default_rng(2)
    v = rng.normal(scale=0.3, size=x.shape)
    im = np.full(s.n, 1.0 / 12.0)
    h.set_langevin(0.001, 2.0, 0.0, seed=1)
    xd, vd, imd = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (x, v, im))
    rd = torch.zeros((1, capi.NRESULTS), dtype=torch.float64, device="cuda")
    h.langevin_step(xd.data_ptr(), vd.data_ptr(), imd.data_ptr(), rd.data_ptr(), 1)
    torch.cuda.synchronize()
    xo, vo = oracle.langevin_update(x, v, im, F, 0.001, 2.0, 0.0)
    assert np.array_equal(xd.cpu().numpy(), xo)
    assert np.array_equal(vd.cpu().numpy(), vo)


def test_sdmutils_mirror_through_sdmforce():
    """SDMUtils.addRestraintForce / addAlignmentForce on the SDMForce mirror:
    the restraint energy inside getPotEnergy, the control parameter through
    setParameter (SDMRestraintControlParameter)."""
    from openmm_sdm_plugin_gb300.force import SDMUtils, force_from_system
    s = _system(nrep=1)
    x = s.positions[0]
    rs = _restraints(s, x)
    plain = force_from_system(s)
    e_plain, _ = plain.evaluate(x)
    f = force_from_system(s)
    u = SDMUtils(f)
    u.addRestraintForce(lig_cm_particles=list(rs.lig_particles), rcpt_cm_particles=list(rs.rcpt_particles),
                        kfcm=rs.kfcm, tolcm=rs.tolcm, lig_ref_particles=list(rs.lig_ref),
                        rcpt_ref_particles=list(rs.rcpt_ref), angle_center=rs.angle_center, kfangle=rs.kf_angle,
                        angletol=rs.angle_tol, dihedral1center=rs.dihedral1_center,
                        kfdihedral1=rs.kf_dihedral1, dihedral1tol=rs.dihedral1_tol,
                        dihedral2center=rs.dihedral2_center, kfdihedral2=rs.kf_dihedral2,
                        dihedral2tol=rs.dihedral2_tol, offset=rs.offset)
    u.addAlignmentForce(liga_ref_particles=list(rs.liga_ref), ligb_ref_particles=list(rs.ligb_ref),
                        kfdispl=rs.kf_displ, ktheta=rs.k_theta, kpsi=rs.k_psi, offset=rs.align_offset)
    ref = dataclasses.replace(rs, lig_weights=None, rcpt_weights=None)   # SDMForce has no masses
    e, _ = f.evaluate(x)
    assert abs((e - e_plain) - oracle.restraint_energy(x, ref)) < 1e-8 * abs(e)
    assert abs(f.getRestraintEnergy() - oracle.restraint_energy(x, ref)) < 1e-9 * abs(e - e_plain)
    f.setParameter(u.getControlParameterName(), 0.5)
    e_half, _ = f.evaluate(x)
    assert abs(f.getRestraintEnergy() - oracle.restraint_energy(x, ref, control=0.5)) < 1e-9 * abs(e)
    f.close()
    plain.close()


@pytest.mark.parametrize("method", ["rf", "pme"])
def test_restraints_on_the_second_system_of_a_handle(method):
    """Restraints on system 1 only of a two-system handle (own offsets into
    the restraint data), reaction field and PME: system 0's replica has no
    restraint energy, system 1's replicas match the oracle."""
    a = dataclasses.replace(S.config0(variant="b"), nonbonded_method=method)
    b = dataclasses.replace(S.host_guest(1500, seed=7, nstates=2), nonbonded_method=method)
    xb = b.positions[0]
    lig = np.asarray(b.ligand_atoms)
    others = np.setdiff1d(np.arange(b.n), lig)
    near = others[np.argsort(np.linalg.norm(xb[others] - xb[lig].mean(0), axis=1))[:50]]
    rs = S.Restraints(lig_particles=lig, rcpt_particles=near, kfcm=600.0, tolcm=0.0,
                      use_alignment=True, liga_ref=tuple(int(i) for i in lig[:3]),
                      ligb_ref=tuple(int(i) for i in near[:3]), kf_displ=50.0, k_theta=10.0, k_psi=5.0)
    h = capi.Handle([a, dataclasses.replace(b, restraints=rs)])
    reps = [(a, 0), (b, 0), (b, 1)]
    for r, (s, k) in enumerate(reps):
        h.set_params(r, s.params[k].as_array())
    x = np.concatenate([a.positions[0], b.positions[0], b.positions[1]])
    res, F = h.evaluate(x)
    e = h.restraint_energies()
    assert e[0] == 0.0
    for r in (1, 2):
        eo = oracle.restraint_energy(b.positions[r - 1], rs)
        assert eo > 0.0 and abs(e[r] - eo) < 1e-9 * eo
    assert (res[:, capi.R_STATUS] == 0).all()
