"""The uneven multi-system batch: 64 host-guest systems of 2,010 to 54,820
particles (log-uniform sizes, seed 3), 16 lambda states each, all 1,024
replicas in one handle and one evaluation call.

- Every replica's status is clean and its energies finite.
- A sample of replicas against both oracle rules, with the tolerances of
  every other parity test: the smallest and the largest system, and four
  others, each at a different lambda state (the replica index inside its
  system varies).
- Per system, lambda states that share a coordinate set would give the same
  U0 and u; here every state has its own coordinates, so the check is that
  the batch equals each sampled system evaluated in a handle of its own.

Named to run after the other parity files."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from helpers import check_replica, oracle_replica
from openmm_sdm_plugin_gb300 import capi, systems as S

pytestmark = pytest.mark.gpu

U_TOL = 1e-6        # kJ/mol: batch vs the same system alone (same terms, same order)
F_TOL = 1e-3        # kJ/mol/nm


def _handle(sysms):
    h = capi.Handle(sysms)
    r = 0
    for s in sysms:
        for p in s.params:
            h.set_params(r, p.as_array())
            r += 1
    return h


@pytest.fixture(scope="module")
def batch():
    sysms = S.config3()
    h = _handle(sysms)
    x = np.concatenate([s.positions.reshape(-1, 3) for s in sysms])
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    yield sysms, h, res, F, F0, F1
    h.close()


def _offsets(sysms):
    """(first replica, first particle row) of every system in the batch."""
    rep, row = [], []
    r = o = 0
    for s in sysms:
        rep.append(r)
        row.append(o)
        r += s.replicas
        o += s.replicas * s.n
    return rep, row


def _sample(sysms):
    sizes = np.array([s.n for s in sysms])
    order = np.argsort(sizes)
    picks = [int(order[0]), int(order[-1]), int(order[len(order) // 4]), int(order[len(order) // 2]),
             int(order[3 * len(order) // 4]), int(order[-2])]
    # a different lambda state of each sampled system
    return [(k, (3 * i + 1) % sysms[k].replicas) for i, k in enumerate(picks)]


def test_batch_status_and_shape(batch):
    sysms, h, res, F, F0, F1 = batch
    assert res.shape[0] == sum(s.replicas for s in sysms) == 64 * 16
    assert F.shape[0] == sum(s.replicas * s.n for s in sysms)
    assert np.all(res[:, capi.R_STATUS] == 0)
    assert np.isfinite(res[:, :capi.R_STATUS]).all()
    assert np.isfinite(F).all()


def test_sampled_replicas_against_the_oracle(batch):
    sysms, h, res, F, F0, F1 = batch
    rep0, row0 = _offsets(sysms)
    picks = _sample(sysms)
    assert min(s.n for s in sysms) in [sysms[k].n for k, _ in picks]
    assert max(s.n for s in sysms) in [sysms[k].n for k, _ in picks]

    def run(kq):
        k, q = kq
        s = sysms[k]
        return oracle_replica(s.replica(q), s.positions[q], h.grid(k))

    with ThreadPoolExecutor(max_workers=min(len(picks), os.cpu_count() or 1)) as ex:
        outs = list(ex.map(run, picks))
    for (k, q), ab in zip(picks, outs):
        s = sysms[k]
        r = rep0[k] + q
        sl = slice(row0[k] + q * s.n, row0[k] + (q + 1) * s.n)
        check_replica(s.replica(q), s.positions[q], res[r], F[sl], F0[sl], F1[sl], h.grid(k), ab=ab)


def test_sampled_systems_equal_their_own_handles(batch):
    sysms, h, res, F, F0, F1 = batch
    rep0, row0 = _offsets(sysms)
    for k, _ in _sample(sysms)[:3]:
        s = sysms[k]
        hs = _handle([s])
        rs, Fs = hs.evaluate(s.positions.reshape(-1, 3))
        hs.close()
        sl = slice(row0[k], row0[k] + s.replicas * s.n)
        for key in (capi.R_U0, capi.R_U1, capi.R_U, capi.R_EPOT):
            assert np.abs(res[rep0[k]:rep0[k] + s.replicas, key] - rs[:, key]).max() < U_TOL, (k, key)
        assert np.abs(F[sl] - Fs).max() < F_TOL, k
