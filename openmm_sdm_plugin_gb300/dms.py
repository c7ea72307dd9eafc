"""Desmond DMS (SQLite) input for the SDM force.

Reads what the SDM nonbonded evaluation needs from a DMS file, with the
tables and unit conversions of the reference's example reader
(example/desmonddmsfile75.py):

  particle         x, y, z (Angstrom), charge (e), mass (g/mol), nbtype, resid, resname
  nonbonded_param  sigma (Angstrom), epsilon (kcal/mol), via particle.nbtype
                   (desmonddmsfile75.py:792-802)
  exclusion        p0, p1: excluded pairs (desmonddmsfile75.py:804-810)
  pair_12_6_es_*   1-4 exceptions: aij (kcal A^12), bij (kcal A^6), qij (e^2) ->
                   sigma = (a/b)^(1/6), epsilon = b^2/(4a); a or b = 0 gives
                   epsilon 0, sigma 1 (desmonddmsfile75.py:813-848); every one
                   must also be excluded
  global_cell      periodic cell vectors (Angstrom); must be orthorhombic
  nonbonded_info   vdw_rule: Lorentz-Berthelot ("arithmetic/geometric") only

Bonded terms, constraints, restraints and virtual sites are not read (they
are the caller's group-1 forces).  The reference builds PME or reaction
field from the same tables; this path is reaction field with a cutoff.
"""
from __future__ import annotations

import sqlite3
from typing import Dict, Optional, Sequence

import numpy as np

from .systems import SDMParams, SDMSystem

ANGSTROM = 0.1        # nm
KCAL = 4.184          # kJ


def _tables(con):
    return {r[0] for r in con.execute("SELECT name FROM sqlite_master WHERE type='table'")}


def read_dms(path: str, cutoff: float = 1.0, eps_rf: float = 78.5,
             displacement: Optional[Dict[int, Sequence[float]]] = None,
             params: Optional[SDMParams] = None) -> SDMSystem:
    """SDMSystem (one replica) from a DMS file.

    displacement: residue id -> displacement vector (nm) of that residue's
    particles (the reference's setDisplacement per ligand atom,
    example/test_explicit.py); params: SDM parameters of the replica.
    """
    con = sqlite3.connect(f"file:{path}?mode=ro", uri=True)
    try:
        tabs = _tables(con)
        for t in ("particle", "nonbonded_param", "global_cell"):
            if t not in tabs:
                raise ValueError(f"DMS file {path} has no {t} table")
        if "nonbonded_info" in tabs:
            row = con.execute("SELECT vdw_rule FROM nonbonded_info").fetchone()
            rule = (row[0] or "").lower() if row else ""
            if rule and rule != "arithmetic/geometric":
                raise NotImplementedError(f"vdw_rule {rule!r}: only Lorentz-Berthelot is supported")
        rows = con.execute(
            """SELECT particle.id, x, y, z, charge, mass, resid, sigma, epsilon
               FROM particle INNER JOIN nonbonded_param ON particle.nbtype = nonbonded_param.id
               ORDER BY particle.id""").fetchall()
        ids = np.array([r[0] for r in rows], np.int64)
        if not np.array_equal(ids, np.arange(len(ids)) + ids[0]):
            raise ValueError("particle ids are not contiguous")
        base = int(ids[0])
        a = np.array([r[1:] for r in rows], np.float64)
        pos = a[:, 0:3] * ANGSTROM
        charge, mass, resid = a[:, 3], a[:, 4], a[:, 5].astype(np.int64)
        sigma, epsilon = a[:, 6] * ANGSTROM, a[:, 7] * KCAL
        cell = np.array(con.execute("SELECT x, y, z FROM global_cell ORDER BY id").fetchall(), np.float64)
        if cell.shape != (3, 3) or np.count_nonzero(cell - np.diag(np.diag(cell))):
            raise NotImplementedError("only orthorhombic cells are supported")
        box = np.diag(cell) * ANGSTROM
        excl = np.array(con.execute("SELECT p0, p1 FROM exclusion").fetchall(), np.int64).reshape(-1, 2) - base
        excl = np.sort(excl, axis=1)
        exc = np.zeros((0, 2), np.int64)
        exc_prm = np.zeros((0, 3))
        if "pair_12_6_es_term" in tabs:
            pr = con.execute(
                """SELECT p0, p1, aij, bij, qij FROM pair_12_6_es_term INNER JOIN pair_12_6_es_param
                   ON pair_12_6_es_term.param = pair_12_6_es_param.id""").fetchall()
            if pr:
                pa = np.array(pr, np.float64)
                exc = pa[:, 0:2].astype(np.int64) - base
                aij = pa[:, 2] * KCAL * ANGSTROM ** 12
                bij = pa[:, 3] * KCAL * ANGSTROM ** 6
                zero = (aij == 0.0) | (bij == 0.0)
                safe_a = np.where(zero, 1.0, aij)
                safe_b = np.where(zero, 1.0, bij)
                eps14 = np.where(zero, 0.0, safe_b ** 2 / (4.0 * safe_a))
                sig14 = np.where(zero, 1.0, (safe_a / safe_b) ** (1.0 / 6.0))
                exc_prm = np.stack([pa[:, 4], sig14, eps14], axis=1)
    finally:
        con.close()
    n = pos.shape[0]
    # every exception must also be an exclusion (desmonddmsfile75.py:841-848)
    if len(exc):
        key = lambda p: np.minimum(p[:, 0], p[:, 1]) * n + np.maximum(p[:, 0], p[:, 1])
        if not np.isin(key(exc), key(excl)).all():
            raise NotImplementedError("all pair_12_6_es_terms must have a corresponding exclusion")
    disp = np.zeros((n, 3))
    lig = []
    for rid, vec in (displacement or {}).items():
        sel = resid == int(rid)
        if not sel.any():
            raise ValueError(f"no particles with resid {rid}")
        disp[sel] = np.asarray(vec, np.float64)
        lig.append(np.nonzero(sel)[0])
    return SDMSystem(name=path.rsplit("/", 1)[-1], box=box, charge=charge, sigma=sigma, epsilon=epsilon,
                     exclusions=excl.astype(np.int32), displacement=disp, positions=pos[None].copy(),
                     params=[params if params is not None else SDMParams()], cutoff=cutoff, eps_rf=eps_rf,
                     ligand_atoms=np.concatenate(lig) if lig else None,
                     exceptions=exc.astype(np.int32), exception_params=exc_prm, masses=mass)


def load_compact(path: str, displacement: Optional[Dict[int, Sequence[float]]] = None,
                 params: Optional[Sequence[SDMParams]] = None, cutoff: float = 1.0,
                 eps_rf: float = 78.5) -> SDMSystem:
    """SDMSystem from the compact npz form of a DMS-derived system (fields box,
    positions, charge, mass, lj_types + nbtype, resid, exclusions,
    exceptions, exception_params; written by tests/golden/make_dms_fixture.py).
    One replica per entry of `params` (default one), all at the stored
    coordinates; `displacement` maps residue ids to vectors (nm)."""
    z = np.load(path)
    t = z["lj_types"][z["nbtype"]]
    resid = z["resid"].astype(np.int64)
    n = t.shape[0]
    disp = np.zeros((n, 3))
    for rid, vec in (displacement or {}).items():
        disp[resid == int(rid)] = np.asarray(vec, np.float64)
    ps = list(params) if params is not None else [SDMParams()]
    pos = np.repeat(z["positions"].astype(np.float64)[None], len(ps), axis=0)
    return SDMSystem(name=path.rsplit("/", 1)[-1], box=z["box"].astype(np.float64),
                     charge=z["charge"].astype(np.float64), sigma=t[:, 0].copy(), epsilon=t[:, 1].copy(),
                     exclusions=z["exclusions"], displacement=disp, positions=pos, params=ps, cutoff=cutoff,
                     eps_rf=eps_rf, ligand_atoms=np.nonzero(np.any(disp != 0, axis=1))[0],
                     exceptions=z["exceptions"], exception_params=z["exception_params"],
                     masses=z["mass"].astype(np.float64))
