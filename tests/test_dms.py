"""DMS ingest and NonbondedForce exceptions (1-4 pairs).

CPU: the reader on a small DMS file written here, the committed TEMOA
fixture (tests/golden/temoa_g1_g4.npz, made by tests/golden/make_dms_fixture.py
from the reference's example/temoa-g1-g4.dms), the oracle's exception terms.
GPU: exceptions through the C ABI against the oracle, and the real TEMOA
system (20,446 particles, 606 exceptions, guests displaced by +-2.2 nm per
axis as in the reference's example/test_explicit.py) against the oracle.
"""
import dataclasses
import os
import sqlite3

import numpy as np
import pytest

import oracle
from helpers import FORCE_RMS_REL_TOL, U_ABS_TOL, energy_tol, rms_rel
from openmm_sdm_plugin_gb300 import capi, dms, systems as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "temoa_g1_g4.npz")


def temoa_system(params=None):
    p = params or S.SDMParams(bias_method=S.ILOGISTIC, softcore_method=S.RATIONAL_SOFTCORE, lambdac=0.5,
                              lambda1=0.5, lambda2=0.5, alpha=0.0, u0=0.0, w0=0.0, umax=200.0,
                              acore=1.0 / 16.0, ubcore=100.0)
    # G1 (resid 2) +22 A and G4 (resid 3) -22 A per axis
    return dms.load_compact(GOLDEN, displacement={2: (2.2, 2.2, 2.2), 3: (-2.2, -2.2, -2.2)}, params=[p])


def _write_dms(path):
    con = sqlite3.connect(path)
    c = con.cursor()
    c.execute("CREATE TABLE particle (id INTEGER PRIMARY KEY, x FLOAT, y FLOAT, z FLOAT, charge FLOAT, "
              "mass FLOAT, resid INTEGER, resname TEXT, nbtype INTEGER)")
    c.execute("CREATE TABLE nonbonded_param (id INTEGER PRIMARY KEY, sigma FLOAT, epsilon FLOAT, type TEXT)")
    c.execute("CREATE TABLE exclusion (p0 INTEGER, p1 INTEGER)")
    c.execute("CREATE TABLE pair_12_6_es_param (id INTEGER PRIMARY KEY, aij FLOAT, bij FLOAT, qij FLOAT)")
    c.execute("CREATE TABLE pair_12_6_es_term (p0 INTEGER, p1 INTEGER, param INTEGER)")
    c.execute("CREATE TABLE global_cell (id INTEGER PRIMARY KEY, x FLOAT, y FLOAT, z FLOAT)")
    c.execute("CREATE TABLE nonbonded_info (vdw_funct TEXT, vdw_rule TEXT, es_funct TEXT)")
    c.executemany("INSERT INTO nonbonded_param VALUES (?,?,?,?)", [(0, 3.0, 0.2, "C"), (1, 0.0, 0.0, "H")])
    c.executemany("INSERT INTO particle VALUES (?,?,?,?,?,?,?,?,?)",
                  [(0, 1.0, 2.0, 3.0, -0.5, 12.0, 1, "LIG", 0), (1, 2.0, 2.0, 3.0, 0.25, 1.0, 1, "LIG", 1),
                   (2, 3.0, 2.5, 3.0, 0.25, 1.0, 1, "LIG", 1), (3, 10.0, 10.0, 10.0, 0.0, 12.0, 2, "WAT", 0)])
    c.executemany("INSERT INTO exclusion VALUES (?,?)", [(0, 1), (0, 2), (1, 2)])
    c.execute("INSERT INTO pair_12_6_es_param VALUES (0, 4.0e5, 6.0e2, 0.1)")
    c.execute("INSERT INTO pair_12_6_es_term VALUES (0, 2, 0)")
    c.executemany("INSERT INTO global_cell VALUES (?,?,?,?)", [(1, 30.0, 0, 0), (2, 0, 31.0, 0), (3, 0, 0, 32.0)])
    c.execute("INSERT INTO nonbonded_info VALUES ('vdw_12_6', 'arithmetic/geometric', '')")
    con.commit()
    con.close()


def test_read_dms_units(tmp_path):
    p = str(tmp_path / "tiny.dms")
    _write_dms(p)
    s = dms.read_dms(p, cutoff=0.9, displacement={1: (0.5, 0.0, 0.0)})
    assert s.n == 4
    assert np.allclose(s.box, [3.0, 3.1, 3.2])
    assert np.allclose(s.positions[0, 0], [0.1, 0.2, 0.3])
    assert np.allclose(s.sigma, [0.3, 0.0, 0.0, 0.3]) and np.allclose(s.epsilon, [0.2 * 4.184, 0, 0, 0.2 * 4.184])
    assert np.allclose(s.charge, [-0.5, 0.25, 0.25, 0.0]) and np.allclose(s.masses, [12, 1, 1, 12])
    assert sorted(map(tuple, s.exclusions.tolist())) == [(0, 1), (0, 2), (1, 2)]
    a, b = 4.0e5 * 4.184 * 1e-12, 6.0e2 * 4.184 * 1e-6
    assert s.exceptions.tolist() == [[0, 2]]
    assert np.allclose(s.exception_params[0], [0.1, (a / b) ** (1 / 6), b * b / (4 * a)], rtol=1e-12)
    assert np.array_equal(s.ligand_atoms, [0, 1, 2]) and np.allclose(s.displacement[:3, 0], 0.5)


def test_read_dms_rejects_unsupported(tmp_path):
    p = str(tmp_path / "bad.dms")
    _write_dms(p)
    con = sqlite3.connect(p)
    con.execute("DELETE FROM exclusion WHERE p0 = 0 AND p1 = 2")
    con.commit()
    con.close()
    with pytest.raises(NotImplementedError):
        dms.read_dms(p)


def test_temoa_fixture_is_consistent():
    s = temoa_system()
    assert s.n == 20446 and len(s.exceptions) == 606 and len(s.exclusions) == 21503
    assert len(s.ligand_atoms) == 38
    assert abs(s.charge.sum() + 0.001) < 1e-5
    key = lambda p: np.minimum(p[:, 0], p[:, 1]) * s.n + np.maximum(p[:, 0], p[:, 1])
    assert np.isin(key(s.exceptions.astype(np.int64)), key(s.exclusions.astype(np.int64))).all()
    assert (s.box > 2 * s.cutoff).all()


def test_oracle_exception_terms():
    """Two particles with one exception: closed-form energy and force, both
    states (different displacements), no periodic image."""
    s = S.config0(variant="b")
    n = s.n
    i, j = 900, 0            # ligand particle and a solvent particle: different displacements
    ex = np.array([[i, j]], np.int32)
    prm = np.array([[0.3, 0.31, 0.5]])
    s2 = dataclasses.replace(s, exclusions=np.concatenate([s.exclusions, ex]), exceptions=ex,
                             exception_params=prm)
    o = oracle.OracleSystem(s2)
    x = s.positions[0]
    e0, du, F0, dF = o.exceptions(x)

    def ef(d):
        r = np.linalg.norm(d)
        sr6 = (0.31 / r) ** 6
        e = oracle.K_COULOMB * 0.3 / r + 4 * 0.5 * (sr6 * sr6 - sr6)
        fs = (oracle.K_COULOMB * 0.3 / r + 4 * 0.5 * (12 * sr6 * sr6 - 6 * sr6)) / r ** 2
        return e, fs * d
    d0 = x[j] - x[i]
    d1 = (x[j] + s.displacement[j]) - (x[i] + s.displacement[i])
    ea, fa = ef(d0)
    eb, fb = ef(d1)
    assert e0 == pytest.approx(ea, rel=1e-12) and du == pytest.approx(eb - ea, rel=1e-10, abs=1e-12)
    assert np.allclose(F0[j], fa, rtol=1e-12) and np.allclose(F0[i], -fa, rtol=1e-12)
    assert np.allclose(dF[j], fb - fa, rtol=1e-10, atol=1e-12)
    assert np.count_nonzero(np.abs(F0).sum(1)) == 2


def _synthetic_exceptions(s, rng):
    """Exceptions inside the ligand (same displacement) and between ligand and
    solvent (different displacements), all of them excluded too."""
    lig = s.ligand_atoms
    a = rng.choice(lig, 12, replace=False)
    b = rng.choice(np.setdiff1d(np.arange(s.n), lig), 12, replace=False)
    pairs = np.concatenate([np.stack([a[:6], a[6:]], 1), np.stack([a, b], 1)]).astype(np.int32)
    prm = np.stack([rng.uniform(-0.2, 0.2, len(pairs)), rng.uniform(0.25, 0.35, len(pairs)),
                    rng.uniform(0.1, 0.5, len(pairs))], 1)
    excl = np.concatenate([s.exclusions, pairs]).astype(np.int32)
    return dataclasses.replace(s, exclusions=excl, exceptions=pairs, exception_params=prm)


def _check(s, h, x, res, F, F0, F1):
    o = oracle.OracleSystem(s)
    a = o.f32rule(x, h.grid(0))
    b = o.states(x)
    n0 = max(a["P0"], 1)
    assert abs(res[capi.R_U0] - a["U0"]) < energy_tol(a["U0"], n0), (res[capi.R_U0], a["U0"])
    assert abs(res[capi.R_U0] - b["U0"]) < energy_tol(b["U0"], n0) + 0.05
    assert rms_rel(F0, a["F0"]) < 1e-5
    assert rms_rel(F0, b["F0"]) < FORCE_RMS_REL_TOL
    assert rms_rel(F1, a["F0"] + a["dF"]) < 1e-5
    assert rms_rel(F1, b["F1"]) < FORCE_RMS_REL_TOL
    assert abs(res[capi.R_U] - a["u"]) < U_ABS_TOL, (res[capi.R_U], a["u"])
    assert abs(res[capi.R_U] - b["u_direct"]) < U_ABS_TOL, (res[capi.R_U], b["u_direct"])
    sw = res[capi.R_S]
    assert rms_rel(F, sw * b["F1"] + (1 - sw) * b["F0"]) < FORCE_RMS_REL_TOL


@pytest.mark.gpu
def test_exceptions_parity_both_states():
    s = _synthetic_exceptions(S.config0(variant="b"), np.random.default_rng(2))
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    _check(s, h, x, res[0], F, F0, F1)
    assert res[0, capi.R_STATUS] == 0


@pytest.mark.gpu
def test_temoa_dms_system_parity():
    s = temoa_system()
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    _check(s, h, x, res[0], F, F0, F1)
    c = h.count_pairs(x)
    a = oracle.OracleSystem(s).f32rule(x, h.grid(0))
    assert int(c[0, 0]) == a["P0"] and int(c[0, 1]) == a["P1delta"]
    assert res[0, capi.R_STATUS] == 0


@pytest.mark.gpu
def test_exceptions_on_the_second_branch_same_bits():
    """With a second graph branch the 1-4 exceptions and the combine run
    there, beside the main pass (their forces are integer atomics into the
    same accumulators); one stream runs them after it.  Every branch mode,
    captured and eager, gives the same results and forces bit for bit."""
    s = temoa_system()
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    x = s.positions[0]
    out = {}
    for overlap in (2, 1, 0):
        for graph in (1, 0):
            h.set_option(capi.OPT_OVERLAP, overlap)
            h.set_option(capi.OPT_GRAPH, graph)
            r, F = h.evaluate(x)
            out[overlap, graph] = (r, F) + h.state_forces()
    ref = out[2, 1]
    assert ref[0][0, capi.R_STATUS] == 0
    for k, v in out.items():
        for a, b in zip(v, ref):
            assert np.array_equal(a, b), k


def test_mirror_from_a_dms_system_carries_its_nonbonded_force():
    """force_from_system / integrator_from_system on the TEMOA system: the
    mirror's system descriptor holds the same exclusions (each once, in the
    same order), the 1-4 exceptions with their parameters, the electrostatics
    and the masses (OpenMM NonbondedForce.addException semantics: every
    exception excluded, the interacting ones with their own terms)."""
    from openmm_sdm_plugin_gb300 import force_from_system, integrator_from_system
    s = temoa_system()
    f = force_from_system(s)
    d = f._system()
    assert np.array_equal(d.exclusions, s.exclusions)
    assert np.array_equal(d.exceptions, s.exceptions)
    assert np.array_equal(d.exception_params, s.exception_params)
    assert d.nonbonded_method == "rf" and d.cutoff == s.cutoff and d.eps_rf == s.eps_rf
    assert np.array_equal(d.displacement, s.displacement)
    assert np.array_equal(d.params[0].as_array(), s.params[0].as_array())
    integ = integrator_from_system(s, 300.0, 1.0, 0.002)
    assert np.array_equal(integ._system().exceptions, s.exceptions)
    assert [integ.getParticleMass(i) for i in range(s.n)] == list(s.masses)
    with pytest.raises(ValueError, match="masses"):
        integrator_from_system(dataclasses.replace(s, masses=None), 300.0, 1.0, 0.002)
    pme = force_from_system(dataclasses.replace(s, nonbonded_method="pme", ewald_tolerance=2e-4))._system()
    assert pme.nonbonded_method == "pme" and pme.ewald_tolerance == 2e-4


def test_mirror_exception_rules():
    from openmm_sdm_plugin_gb300 import SDMForce
    f = SDMForce()
    for _ in range(4):
        f.addParticle(0.1, 0.3, 0.5)
    f.setPeriodicBoxVectors((3, 0, 0), (0, 3, 0), (0, 0, 3))
    f.addExclusion(0, 1)
    f.addException(1, 0, 0.0, 1.0, 0.0)          # excluded, no own term (already excluded: once)
    f.addException(2, 3, -0.05, 0.3, 0.2)        # a 1-4 pair
    with pytest.raises(ValueError, match="already an exception"):
        f.addException(3, 2, 0.0, 1.0, 0.0)
    assert f.addException(3, 2, -0.07, 0.31, 0.25, replace=True) == 1
    assert f.getNumExceptions() == 2 and f.getExceptionParameters(1) == (3, 2, -0.07, 0.31, 0.25)
    d = f._system()
    assert d.exclusions.tolist() == [[0, 1], [3, 2]]    # the pair as the replacing call gave it
    assert d.exceptions.tolist() == [[3, 2]] and d.exception_params.tolist() == [[-0.07, 0.31, 0.25]]
    with pytest.raises(ValueError, match="CutoffPeriodic"):
        f.setNonbondedMethod(3)                   # Ewald
    f.setNonbondedMethod(SDMForce.PME)
    assert f._system().nonbonded_method == "pme"
    f.setUseDispersionCorrection(False)
    f.setUseSwitchingFunction(False)
    for setter in (f.setUseDispersionCorrection, f.setUseSwitchingFunction):
        with pytest.raises(ValueError, match="not supported"):
            setter(True)


@pytest.mark.gpu
def test_mirror_evaluates_a_dms_system_like_the_c_abi():
    """The mirror built from the TEMOA system (1-4 exceptions included)
    evaluates exactly as the C ABI on the same system."""
    from openmm_sdm_plugin_gb300 import force_from_system
    s = temoa_system()
    f = force_from_system(s)
    e, F = f.evaluate(s.positions[0])
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    res, Fh = h.evaluate(s.positions[0])
    assert e == res[0, capi.R_EPOT] and f.getBindE() == res[0, capi.R_BINDE]
    assert np.array_equal(F, Fh)
    f.close()
    h.close()
