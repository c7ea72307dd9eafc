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
