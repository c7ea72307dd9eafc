"""CPU checks of the restraint pieces: the SDMUtils mirror builds the
restraint description the reference's SDMUtils arguments mean
(python/SDMUtils.py:32-257), the oracle's terms against closed forms."""
import math

import numpy as np
import pytest

import oracle
from openmm_sdm_plugin_gb300 import systems as S
from openmm_sdm_plugin_gb300.force import LangevinIntegratorSDM, SDMForce, SDMUtils


def test_mirror_builds_the_restraint_description():
    f = LangevinIntegratorSDM(300.0, 1.0, 0.002)
    for i in range(12):
        f.addParticle(0.0, 0.3, 0.1, mass=1.0 + i)
    u = SDMUtils(f)
    assert u.getControlParameterName() == "SDMRestraintControlParameter"
    u.addRestraintForce(lig_cm_particles=[0, 1, 2], rcpt_cm_particles=[6, 7], kfcm=50.0, tolcm=0.2,
                        lig_ref_particles=[0, 1, 2], rcpt_ref_particles=[6, 7, 8], angle_center=1.0, kfangle=3.0)
    rs = f._restraints
    assert rs.lig_weights == [1.0, 2.0, 3.0] and rs.rcpt_weights == [7.0, 8.0]   # masses
    assert rs.use_angles and rs.angle_tol == pytest.approx(math.radians(10.0))
    assert not rs.use_alignment
    u.addAlignmentForce(liga_ref_particles=[0, 1, 2], ligb_ref_particles=[3, 4, 5], kfdispl=7.0,
                        offset=(0.1, 0.0, 0.0))
    rs = f._restraints
    assert rs.use_alignment and rs.kf_displ == 7.0 and rs.kfcm == 50.0   # both restraints kept
    with pytest.raises(NotImplementedError):
        u.addRestraintForce(lig_cm_particles=[0], rcpt_cm_particles=[6])
    with pytest.raises(ValueError):
        SDMUtils(SDMForce(4)).addRestraintForce(lig_cm_particles=[0], rcpt_cm_particles=[1],
                                                lig_ref_particles=[0, 1], rcpt_ref_particles=[1, 2, 3])
    g = SDMForce(4)
    SDMUtils(g).addRestraintForce(lig_cm_particles=[], rcpt_cm_particles=[1])   # the reference returns
    assert g._restraints is None
    with pytest.raises(KeyError):
        g.setParameter("lambda", 1.0)


def test_oracle_restraint_terms_closed_forms():
    x = np.zeros((12, 3))
    x[0] = [1.0, 0.0, 0.0]
    x[1] = [0.0, 0.0, 0.0]
    rs = S.Restraints(lig_particles=[0], rcpt_particles=[1], kfcm=10.0, tolcm=0.25)
    assert oracle.restraint_energy(x, rs) == pytest.approx(0.5 * 10.0 * 0.75 ** 2)
    assert oracle.restraint_energy(x, rs, control=0.5) == pytest.approx(0.25 * 10.0 * 0.75 ** 2)
    F = oracle.restraint_forces(x, rs)
    assert F[0] == pytest.approx([-10.0 * 0.75, 0, 0], abs=1e-6) and F[1] == pytest.approx([7.5, 0, 0], abs=1e-6)
    # flat bottom: inside the tolerance nothing
    x[0] = [0.2, 0.0, 0.0]
    assert oracle.restraint_energy(x, rs) == 0.0
    # flat-bottom angle window: angle 90 degrees, window [100, 120] degrees
    assert oracle._rs_flat(math.radians(90), math.radians(100), math.radians(120), math.pi, 2.0) == \
        pytest.approx(0.5 * 2.0 * math.radians(10) ** 2)
    assert oracle._rs_flat(math.radians(110), math.radians(100), math.radians(120), math.pi, 2.0) == 0.0
    # the alignment displacement term
    x = np.zeros((6, 3))
    x[3] = [0.3, 0.0, 0.0]
    x[1] = x[0] + [0, 0, 1]
    x[4] = x[3] + [0, 0, 1]
    x[2] = x[0] + [1, 0, 0]
    x[5] = x[3] + [1, 0, 0]
    al = S.Restraints(use_alignment=True, liga_ref=(0, 1, 2), ligb_ref=(3, 4, 5), kf_displ=4.0,
                      k_theta=3.0, k_psi=2.0, align_offset=(0.1, 0.0, 0.0))
    assert oracle.restraint_energy(x, al) == pytest.approx(0.5 * 4.0 * 0.2 ** 2)   # aligned: no theta/psi


def test_integrator_mirror_records_rigid_waters():
    f = LangevinIntegratorSDM(300.0, 1.0, 0.002, nParticles=6)
    f.setRigidWaters([[0, 1, 2], [3, 4, 5]], 0.09572, 0.1514)
    w, d_oh, d_hh = f._waters
    assert w.tolist() == [[0, 1, 2], [3, 4, 5]] and d_oh == 0.09572 and d_hh == 0.1514
    assert f._waters_dirty
    f.setRigidWaters(None, 0.0, 0.0)
    assert f._waters is None and f._waters_dirty
