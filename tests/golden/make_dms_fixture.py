"""Writes tests/golden/temoa_g1_g4.npz from the reference's example input
example/temoa-g1-g4.dms (TEMOA host, guests G1 and G4, 6,734 waters, ions;
20,446 particles) through the package's own DMS reader, so that the GPU
parity test runs on a real system where the reference tree is absent.

    python tests/golden/make_dms_fixture.py <reference>/example/temoa-g1-g4.dms

Positions, charges and masses are stored as float32 (the fixture defines the
test input); LJ parameters by type; exclusions and 1-4 exceptions as read.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
from openmm_sdm_plugin_gb300 import dms  # noqa: E402


def main(path):
    s = dms.read_dms(path)
    types, nbtype = np.unique(np.stack([s.sigma, s.epsilon], 1), axis=0, return_inverse=True)
    import sqlite3
    con = sqlite3.connect(f"file:{path}?mode=ro", uri=True)
    resid = np.array([r[0] for r in con.execute("SELECT resid FROM particle ORDER BY id")], np.int16)
    con.close()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "temoa_g1_g4.npz")
    np.savez_compressed(out, box=s.box, positions=s.positions[0].astype(np.float32),
                        charge=s.charge.astype(np.float32), mass=s.masses.astype(np.float32),
                        lj_types=types, nbtype=nbtype.astype(np.uint8), resid=resid,
                        exclusions=s.exclusions.astype(np.int32), exceptions=s.exceptions.astype(np.int32),
                        exception_params=s.exception_params)
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main(sys.argv[1])
