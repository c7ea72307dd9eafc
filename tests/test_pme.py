"""PME mode (nonbonded_method = SDM_NB_PME) against the oracle: Lennard-Jones
from the FP64 C oracle (charges zeroed), Ewald direct space, excluded-pair,
self and background terms from oracle.ewald, reciprocal space from the
restated smooth PME (oracle.spme) on the same grid and spline order; both SDM
states.  The restated SPME itself is pinned against the exact Ewald sum and
the rock-salt Madelung constant in tests/test_oracle.py."""
import dataclasses

import numpy as np
import pytest

import oracle
from helpers import FORCE_RMS_REL_TOL, U_ABS_TOL, rms_rel
from openmm_sdm_plugin_gb300 import capi, systems as S

pytestmark = pytest.mark.gpu

TOL = 5e-4


def _pme(s):
    return dataclasses.replace(s, nonbonded_method="pme", ewald_tolerance=TOL)


def _oracle_states(s, x):
    beta = oracle.ewald_beta(s.cutoff, TOL)
    K = list(s.pme_grid) if s.pme_grid is not None else oracle.pme_grid_size(beta, s.box, TOL)
    lj = oracle.OracleSystem(dataclasses.replace(s, charge=np.zeros(s.n))).states(x)

    def coul(y):
        d = oracle.ewald(y, s.charge, s.box, beta, s.cutoff, s.exclusions, kmax=[0, 0, 0])
        er, fr, _ = oracle.spme(y, s.charge, s.box, beta, K)
        return d["total"] + er, d["F"] + fr
    c0, f0 = coul(x)
    c1, f1 = coul(x + s.displacement)
    return dict(U0=lj["U0"] + c0, U1=lj["U1"] + c1, F0=lj["F0"] + f0, F1=lj["F1"] + f1)


def _check(res, F, F0, F1, o):
    # the direct-space pair set is the FP32 rule's; pairs at the cutoff
    # carry erfc(beta rc) ~ tol of their Coulomb term: U0 within 0.02 kJ/mol
    assert abs(res[capi.R_U0] - o["U0"]) < 0.02 + 1e-6 * abs(o["U0"]), (res[capi.R_U0], o["U0"])
    assert abs(res[capi.R_U] - (o["U1"] - o["U0"])) < U_ABS_TOL, (res[capi.R_U], o["U1"] - o["U0"])
    assert rms_rel(F0, o["F0"]) < FORCE_RMS_REL_TOL
    assert rms_rel(F1, o["F1"]) < FORCE_RMS_REL_TOL
    sw = res[capi.R_S]
    assert rms_rel(F, sw * o["F1"] + (1 - sw) * o["F0"]) < FORCE_RMS_REL_TOL
    assert res[capi.R_STATUS] == 0


def test_pme_two_states_against_oracle():
    s = _pme(S.config0(variant="b"))
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    _check(res[0], F, F0, F1, _oracle_states(s, x))


def test_pme_batched_replicas_and_graph_replay():
    """Three lambda states with their own coordinates in one call (batched
    cuFFT plans), eager and graph replays equal bit for bit."""
    import torch
    s = _pme(S.host_guest(1500, seed=5, nstates=3))
    h = capi.Handle([s])
    for r, p in enumerate(s.params):
        h.set_params(r, p.as_array())
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    n = s.n
    for r in range(3):
        sl = slice(r * n, (r + 1) * n)
        _check(res[r], F[sl], F0[sl], F1[sl], _oracle_states(s, s.positions[r]))
    xd = torch.from_numpy(x).cuda()
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    fd = torch.zeros_like(xd)
    for _ in range(3):
        h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(rd.cpu().numpy()[:, :14], res[:, :14])
    assert np.array_equal(fd.cpu().numpy(), F)


def test_pme_fine_grid_global_memory_path():
    """A 160^3 grid on the 930-site box (one-cell bricks, sub-grids up to the
    27,648-point shared-memory cap): one brick's stencils span more points
    than the cap, so that brick spreads and interpolates through global
    memory while the others use their sub-grids; both in one evaluation."""
    s = dataclasses.replace(_pme(S.config0(variant="b")), pme_grid=(160, 160, 160))
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    _check(res[0], F, F0, F1, _oracle_states(s, x))


def test_pme_uneven_systems_in_one_handle():
    """Two different PME systems (own grids, own batched cuFFT plans) and
    their replicas in one call."""
    a = _pme(S.config0(variant="b"))
    b = _pme(S.host_guest(1500, seed=7, nstates=2))
    h = capi.Handle([a, b])
    reps = [(a, 0), (b, 0), (b, 1)]
    for r, (s, k) in enumerate(reps):
        h.set_params(r, s.params[k].as_array())
    x = np.concatenate([a.positions[0], b.positions[0], b.positions[1]])
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    off = 0
    for r, (s, k) in enumerate(reps):
        sl = slice(off, off + s.n)
        _check(res[r], F[sl], F0[sl], F1[sl], _oracle_states(s, s.positions[k]))
        off += s.n


def test_pme_net_charge_and_no_displacement():
    """A charged system (neutralising-background term) with no displaced
    particle: u = 0 and F1 = F0 exactly, U0 against the oracle."""
    s0 = S.config0(variant="b")
    q = s0.charge.copy()
    q[np.nonzero(q)[0][:5]] += 0.2          # net charge +1
    s = _pme(dataclasses.replace(s0, charge=q, displacement=np.zeros_like(s0.displacement)))
    assert abs(s.charge.sum() - 1.0) < 1e-9
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    assert res[0, capi.R_U] == 0.0
    assert np.array_equal(F0, F1)
    _check(res[0], F, F0, F1, _oracle_states(s, x))


def test_pme_rejects_mixed_methods_and_adjoint():
    s = S.config0(variant="b")
    with pytest.raises(capi.SdmError):
        capi.Handle([s, _pme(s)])
    h = capi.Handle([_pme(s)])
    h.set_params(0, s.params[0].as_array())
    h.evaluate(s.positions[0])
    with pytest.raises(capi.SdmError):
        h.adjoint(30)


def test_pme_reciprocal_space_on_the_second_branch():
    """SDM_OPT_OVERLAP 2 runs the reciprocal space on the graph's second
    branch beside the list build and the main pass: the same bits as one
    stream and as the branch joined before the main pass."""
    s = _pme(S.host_guest(1500, seed=5, nstates=3))
    h = capi.Handle([s])
    for r, p in enumerate(s.params):
        h.set_params(r, p.as_array())
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    out = {}
    for ov in (0, 1, 2):
        h.set_option(capi.OPT_OVERLAP, ov)
        r, F = h.evaluate(x)
        out[ov] = (r, F) + h.state_forces()
    ref = out[0]
    assert np.all(ref[0][:, capi.R_STATUS] == 0)
    for k, v in out.items():
        for a, b in zip(v, ref):
            assert np.array_equal(a, b), k
