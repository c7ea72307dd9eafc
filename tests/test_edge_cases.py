"""Edge cases of the two-state evaluation through the C ABI: a box whose
cell grid is one cell per axis (per-pair minimum image in every kernel,
clusters with padding slots), tiny particle counts, and a displacement
shared by every particle (u = 0 and F1 = F0 exactly)."""
import numpy as np
import pytest

from openmm_sdm_plugin_gb300 import capi, systems as S
from helpers import check_replica

pytestmark = pytest.mark.gpu


def _tiny(n, L, seed=3, shared_displacement=False, rc=1.0):
    rng = np.random.default_rng(seed)
    g = int(np.ceil(n ** (1.0 / 3.0)))
    grid = np.stack(np.meshgrid(*[np.arange(g)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    x = (grid + 0.5) * (L / g) + rng.uniform(-0.04, 0.04, (n, 3))
    q = rng.uniform(-0.5, 0.5, n)
    q -= q.mean()
    sig = rng.uniform(0.25, 0.32, n)
    eps = rng.uniform(0.1, 0.6, n)
    ex = np.array([[0, 1], [2, 3]], np.int32) if n >= 4 else np.zeros((0, 2), np.int32)
    d = np.zeros((n, 3))
    if shared_displacement:
        d[:] = [0.7, -0.3, 0.2]
    else:
        d[:min(3, n)] = [0.45, 0.1, 0.0]
    p = S.SDMParams(bias_method=S.ILOGISTIC, softcore_method=S.RATIONAL_SOFTCORE, lambda1=0.3, lambda2=0.6,
                    alpha=0.05, u0=10.0, w0=1.0, umax=50.0, acore=0.25, ubcore=10.0)
    return S.SDMSystem(name=f"tiny{n}", box=np.array([L, L, L]), charge=q, sigma=sig, epsilon=eps,
                       exclusions=ex, displacement=d, positions=x[None].copy(), params=[p], cutoff=rc,
                       eps_rf=78.5, ligand_atoms=np.nonzero(np.any(d != 0, axis=1))[0])


@pytest.mark.parametrize("n,L", [(2, 2.2), (9, 2.3), (20, 2.5), (64, 2.6)])
def test_tiny_systems_one_cell_per_axis(n, L):
    s = _tiny(n, L)
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    M = h.grid(0)
    assert n > 9 or max(M) <= 2   # the small boxes collapse the cell grid
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    check_replica(s, x, res[0], F, F0, F1, M)
    assert res[0, capi.R_STATUS] == 0


def test_shared_displacement_gives_zero_u_and_equal_state_forces():
    s = _tiny(64, 2.6, shared_displacement=True)
    h = capi.Handle([s])
    h.set_params(0, s.params[0].as_array())
    res, F = h.evaluate(s.positions[0])
    F0, F1 = h.state_forces()
    assert res[0, capi.R_U] == 0.0 and res[0, capi.R_U1] == res[0, capi.R_U0]
    assert np.array_equal(F0, F1)
    assert np.array_equal(F, F0)


def test_unknown_method_ids_are_rejected():
    """Bias and soft-core ids other than 0, 1, 2 (including NaN, fractions and
    values beyond int range) are SDM_ERR_UNKNOWN_METHOD, as the reference
    throws "Unknown soft core method" (LangevinIntegratorSDM.cpp:147); the
    replica keeps its last valid parameters."""
    s = _tiny(20, 2.5)
    h = capi.Handle([s])
    good = s.params[0].as_array()
    h.set_params(0, good)
    for k in (0, 1):   # SDM_P_BIAS_METHOD, SDM_P_SOFTCORE_METHOD
        for v in (3.0, -1.0, 1.5, np.nan, np.inf, 1e300):
            p = good.copy()
            p[k] = v
            with pytest.raises(capi.SdmError) as e:
                h.set_params(0, p)
            assert e.value.status == capi.SDM_ERR_UNKNOWN_METHOD
    res, _ = h.evaluate(s.positions[0])
    assert res[0, capi.R_STATUS] == 0 and np.isfinite(res[0, :capi.R_STATUS]).all()
