"""Size-independent properties at the full benchmark size: 22 replicas x
22,580 particles in one batched call (the workload of bench.py).

- Each replica of the batch equals the same replica evaluated alone (the
  replicas share no data).
- The state forces obey Newton's third law (pair forces only).
- 22 lambda states on one coordinate set give the same U0, U1, u, F0 and F1,
  and the mixed forces differ only by (s_r - s_q) dF.
- Two calls give the same bits.
- Every replica of the batch against both oracle rules (the parity test of
  the benchmark input itself; oracle calls on a thread pool).

Tolerances are far below any real error. The terms are the same, and the
fixed-point force sums do not depend on order, so agreement is expected to
the last bit; the margin only covers summation orders.  Named to run after
the other parity files."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from helpers import check_replica, oracle_replica
from openmm_sdm_plugin_gb300 import capi, systems as S

pytestmark = pytest.mark.gpu

NREP = 22
U_TOL = 1e-6        # kJ/mol, on energies of ~1e5 kJ/mol
F_TOL = 1e-3        # kJ/mol/nm, on forces of ~1e3 kJ/mol/nm


def _handle(sysms):
    h = capi.Handle(sysms)
    r = 0
    for s in sysms:
        for p in s.params:
            h.set_params(r, p.as_array())
            r += 1
    return h


@pytest.fixture(scope="module")
def full():
    s = S.config2(nrep=NREP)
    h = _handle([s])
    res, F = h.evaluate(s.positions.reshape(-1, 3))
    F0, F1 = h.state_forces()
    yield s, h, res, F, F0, F1
    h.close()


def test_batch_equals_each_replica_alone(full):
    s, h, res, F, F0, F1 = full
    n = s.n
    assert np.all(res[:, capi.R_STATUS] == 0)
    for r in range(NREP):
        hr = _handle([s.replica(r)])
        rr, Fr = hr.evaluate(s.positions[r])
        F0r, F1r = hr.state_forces()
        hr.close()
        sl = slice(r * n, (r + 1) * n)
        for k in (capi.R_U0, capi.R_U1, capi.R_U, capi.R_EPOT):
            assert abs(res[r, k] - rr[0, k]) < U_TOL, (r, k, res[r, k], rr[0, k])
        assert np.abs(F[sl] - Fr).max() < F_TOL, r
        assert np.abs(F0[sl] - F0r).max() < F_TOL, r
        assert np.abs(F1[sl] - F1r).max() < F_TOL, r


def test_state_forces_obey_newtons_third_law(full):
    s, h, res, F, F0, F1 = full
    n = s.n
    for r in range(NREP):
        sl = slice(r * n, (r + 1) * n)
        for G in (F0[sl], F1[sl], F[sl]):
            assert np.abs(G.sum(axis=0)).max() < 1e-6 * np.abs(G).sum(), r


def test_lambda_states_on_one_coordinate_set(full):
    s, h, res, F, F0, F1 = full
    x = np.concatenate([s.positions[0]] * NREP)
    res2, Fm = h.evaluate(x)
    G0, G1 = h.state_forces()
    n = s.n
    for k in (capi.R_U0, capi.R_U1, capi.R_U):
        assert np.abs(res2[:, k] - res2[0, k]).max() < U_TOL, k
    dF = G1[:n] - G0[:n]
    sw = res2[:, capi.R_S]
    assert np.unique(np.round(sw, 12)).size > 1   # the 22 states mix differently
    for r in range(NREP):
        sl = slice(r * n, (r + 1) * n)
        assert np.abs(G0[sl] - G0[:n]).max() < F_TOL and np.abs(G1[sl] - G1[:n]).max() < F_TOL, r
        assert np.abs(Fm[sl] - (G0[:n] + sw[r] * dF)).max() < F_TOL, r


def test_two_calls_give_the_same_bits(full):
    s, h, res, F, F0, F1 = full
    res2, F2 = h.evaluate(s.positions.reshape(-1, 3))
    assert np.array_equal(res2[:, :capi.R_STATUS], res[:, :capi.R_STATUS])
    assert np.array_equal(F2, F)


def test_every_replica_against_the_oracle(full):
    """All 22 replicas of the benchmark batch against the FP64 and FP32-rule
    oracles, with the tolerances of every other parity test (u 5e-3 kJ/mol,
    forces 1e-4 rms relative against the FP64 rule)."""
    s, h, res, F, F0, F1 = full
    n = s.n
    M = h.grid(0)
    # the oracle's C calls release the GIL, so threads run them in parallel
    with ThreadPoolExecutor(max_workers=min(NREP, os.cpu_count() or 1)) as ex:
        outs = list(ex.map(lambda r: oracle_replica(s.replica(r), s.positions[r], M), range(NREP)))
    for r in range(NREP):
        sl = slice(r * n, (r + 1) * n)
        check_replica(s.replica(r), s.positions[r], res[r], F[sl], F0[sl], F1[sl], M, ab=outs[r])
