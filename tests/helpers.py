"""Shared comparison helpers for the parity tests (the oracle is the checker)."""
import numpy as np

# tolerances (floating point; stated once, used by every parity test)
U_ABS_TOL = 5.0e-3          # kJ/mol: perturbation energy u vs the FP64 oracle
FORCE_RMS_REL_TOL = 1.0e-4  # ||F - F_ref||_2 / ||F_ref||_2
ENERGY_REL_TOL = 1.0e-6     # U0, U1 relative to the sum of |pair energy| scale


def rms_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def energy_tol(U, npairs):
    """Tolerance for a sum of npairs FP32 pair energies: relative 1e-6 of
    |U| plus a random-walk term of 1e-5 kJ/mol per sqrt(pair)."""
    return ENERGY_REL_TOL * abs(U) + 1.0e-5 * np.sqrt(max(npairs, 1))


def oracle_replica(s, x, M):
    """Both oracle rules for one replica: (FP32-rule dict, FP64-rule dict)."""
    import oracle
    o = oracle.OracleSystem(s)
    return o.f32rule(x, M), o.states(x)


def check_replica(s, x, res, F, F0, F1, M, strict_u=True, ab=None):
    """One replica of a device evaluation against both oracle rules: U0, u,
    F0, F1 and the mixed force, and the combine on the device's own energies
    against the restated reference combine.  `ab` takes oracle results
    computed beforehand (oracle_replica), e.g. on a thread pool."""
    import pytest

    import oracle
    from openmm_sdm_plugin_gb300 import capi
    a, b = ab if ab is not None else oracle_replica(s, x, M)
    n0 = max(a["P0"], 1)
    assert abs(res[capi.R_U0] - a["U0"]) < energy_tol(a["U0"], n0), (res[capi.R_U0], a["U0"])
    assert abs(res[capi.R_U0] - b["U0"]) < energy_tol(b["U0"], n0) + 0.05
    assert rms_rel(F0, a["F0"]) < 1e-5
    assert rms_rel(F0, b["F0"]) < FORCE_RMS_REL_TOL
    assert rms_rel(F1, a["F0"] + a["dF"]) < 1e-5
    assert rms_rel(F1, b["F1"]) < FORCE_RMS_REL_TOL
    u_ref = b["u_direct"]
    tol = U_ABS_TOL if strict_u else max(U_ABS_TOL, 1e-6 * abs(u_ref))
    assert abs(res[capi.R_U] - a["u"]) < tol, (res[capi.R_U], a["u"])
    assert abs(res[capi.R_U] - u_ref) < tol, (res[capi.R_U], u_ref)
    assert res[capi.R_U1] == pytest.approx(res[capi.R_U0] + res[capi.R_U], rel=1e-15)
    # combine on the device's own energies matches the restated reference combine
    p = s.params[0].as_array()
    comb = oracle.combine(p, res[capi.R_U0], res[capi.R_U1])
    assert res[capi.R_BINDE] == pytest.approx(comb[1], rel=1e-9, abs=1e-9)
    assert res[capi.R_W] == pytest.approx(comb[3], rel=1e-9, abs=1e-9)
    assert res[capi.R_DW] == pytest.approx(comb[4], rel=1e-9, abs=1e-12)
    assert res[capi.R_S] == pytest.approx(comb[5], rel=1e-9, abs=1e-12)
    assert res[capi.R_EPOT] == pytest.approx(comb[6], rel=1e-12)
    # mixed force
    sw = res[capi.R_S]
    Fref = sw * b["F1"] + (1 - sw) * b["F0"]
    assert rms_rel(F, Fref) < FORCE_RMS_REL_TOL
    return a, b
