"""CPU checks of the oracle's rigid-water constraint (oracle.shake_waters), the
checker of the device SETTLE step: the constrained positions meet the
distances, the corrections are internal (mass-weighted sum zero per water)
and lie along the old bond vectors (in the old water plane), hydrogens keep
their own periodic image, waters with a fixed particle are left alone, and
a problem that does not converge raises."""
import numpy as np
import pytest

import oracle
from openmm_sdm_plugin_gb300 import systems as S


def _waters(nw=400, seed=7, kick=0.004):
    s = S.config2(nrep=1)
    w, d_oh, d_hh = S.rigid_waters(s)
    w = w[:nw]
    x = s.positions[0].copy()
    rng = np.random.default_rng(seed)
    xp = x + rng.normal(scale=kick, size=x.shape)
    m = np.full(s.n, 12.011)
    m[w[:, 0]] = 15.999
    m[w[:, 1]] = m[w[:, 2]] = 1.008
    return s, w, d_oh, d_hh, x, xp, 1.0 / m


def _bond(x, w, i, j, box):
    d = x[w[:, i]] - x[w[:, j]]
    return d - box * np.round(d / box)


def test_distances_are_met():
    s, w, d_oh, d_hh, x, xp, im = _waters()
    y = oracle.shake_waters(x, xp, im, w, d_oh, d_hh, s.box)
    for i, j, d in ((0, 1, d_oh), (0, 2, d_oh), (1, 2, d_hh)):
        assert np.abs(np.linalg.norm(_bond(y, w, i, j, s.box), axis=1) - d).max() < 1e-12
    # the unconstrained positions were off by ~1e-2 relative
    assert np.abs(np.linalg.norm(_bond(xp, w, 0, 1, s.box), axis=1) - d_oh).max() > 1e-3


def test_corrections_are_internal_and_along_old_bonds():
    s, w, d_oh, d_hh, x, xp, im = _waters()
    y = oracle.shake_waters(x, xp, im, w, d_oh, d_hh, s.box)
    c = (y - xp)[w]                                    # (nw, 3 atoms, 3)
    m = (1.0 / im)[w][:, :, None]
    # constraint forces are internal: the mass-weighted correction sums to
    # zero, up to the rounding of coordinates of a few nm (ulp ~1e-15) times
    # masses up to 16
    assert np.abs((m * c).sum(axis=1)).max() < 16 * 64 * np.spacing(s.box.max())
    # and lie along the old bond vectors: no component normal to the old plane
    n0 = np.cross(_bond(x, w, 1, 0, s.box), _bond(x, w, 2, 0, s.box))
    n0 /= np.linalg.norm(n0, axis=1, keepdims=True)
    assert np.abs(np.einsum("wak,wk->wa", c, n0)).max() < 1e-13
    assert np.abs(c).max() > 1e-4                      # the corrections are not trivially zero


def test_hydrogens_keep_their_own_image():
    s, w, d_oh, d_hh, x, xp, im = _waters()
    # wrap particle by particle after a shift: some waters straddle the box faces
    t = np.array([0.5, 0.37, 0.21]) * s.box
    x2 = x + t
    x2 -= s.box * np.floor(x2 / s.box)
    xp2 = xp + (x2 - x)
    straddle = np.abs(x2[w[:, 1:]] - x2[w[:, :1]]).max(axis=(1, 2)) > 0.5 * s.box.min()
    assert straddle.sum() > 5
    y = oracle.shake_waters(x, xp, im, w, d_oh, d_hh, s.box)
    y2 = oracle.shake_waters(x2, xp2, im, w, d_oh, d_hh, s.box)
    # the same constrained molecules, each particle in the image it came in
    k = np.round((x2 - x) / s.box - t / s.box)
    assert np.abs((y2 - y) - (t + k * s.box)).max() < 1e-12
    assert np.abs(y2[w] - xp2[w]).max() < 0.1


def test_waters_with_a_fixed_particle_are_left_alone():
    s, w, d_oh, d_hh, x, xp, im = _waters(nw=10)
    im = im.copy()
    im[w[3, 1]] = 0.0
    y = oracle.shake_waters(x, xp, im, w, d_oh, d_hh, s.box)
    assert np.array_equal(y[w[3]], xp[w[3]])
    assert not np.array_equal(y[w[4]], xp[w[4]])
    others = np.setdiff1d(np.arange(s.n), w.reshape(-1))
    assert np.array_equal(y[others], xp[others])


def test_non_convergence_raises():
    s, w, d_oh, d_hh, x, xp, im = _waters(nw=10, kick=0.02)
    with pytest.raises(RuntimeError, match="did not converge"):
        oracle.shake_waters(x, xp, im, w, d_oh, d_hh, s.box, maxit=1)
