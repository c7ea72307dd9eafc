"""The allocation-free entry point against the handle entry point.

sdm_evaluate_noalloc serves callers that cannot allocate device memory when
they need a force (graph-capturing code, hosts whose allocator owns all
device memory, latency-bound loops).  It keeps its scratch in one device
array shared by every call, so this test calls it twice in a row and checks
both results against sdm_evaluate on the same inputs, with the tolerances of
the other parity tests.  Further cases compare it with the FP64 oracle and
cover its other branches: no displacement map (u = 0), no force output, a
particle whose exclusion list is too long for the per-warp shared-memory copy
(the global-memory scan), a force overflow reported in the status word, and a
system at the size limit.  This file is collected last on purpose.
"""
import dataclasses

import numpy as np
import pytest

from helpers import FORCE_RMS_REL_TOL, U_ABS_TOL, energy_tol, rms_rel
from openmm_sdm_plugin_gb300 import capi, systems as S


def _csr(n, pairs):
    pairs = np.asarray(pairs, np.int64).reshape(-1, 2)
    a = np.concatenate([pairs[:, 0], pairs[:, 1]])
    b = np.concatenate([pairs[:, 1], pairs[:, 0]])
    o = np.lexsort((b, a))
    a, b = a[o], b[o]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, a + 1, 1)
    return np.cumsum(off).astype(np.int32), b.astype(np.int32)


def test_noalloc_rejects_oversize_without_launching(built_lib):
    with pytest.raises(capi.SdmError) as e:
        capi.evaluate_noalloc(capi.NOALLOC_MAX_PARTICLES + 1, 1, 1, 1, 1, 1, 1, 0, [3, 3, 3],
                              0.9, 78.5, np.zeros(22), 1)
    assert e.value.status == capi.SDM_ERR_INVALID_ARGUMENT
    assert "8192" in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["b"])
def test_noalloc_matches_handle_path_twice(variant):
    import torch
    s = S.config0(variant=variant)
    n = s.n
    x = np.ascontiguousarray(s.positions[0])
    p = s.params[0].as_array()
    # existing entry point
    h = capi.Handle([s])
    h.set_params(0, p)
    ref_res, ref_F = h.evaluate(x)
    ref = ref_res[0]
    h.close()
    # allocation-free entry point: all buffers belong to the caller
    dev = torch.device("cuda", 0)
    t = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    off, idx = _csr(n, s.exclusions)
    xd, qd, sd, ed = t(x), t(s.charge), t(s.sigma), t(s.epsilon)
    dd = t(s.displacement)
    od, id_ = t(off, torch.int32), t(idx, torch.int32)
    st = torch.cuda.Stream(device=dev)
    for call in range(2):
        rd = torch.full((capi.NRESULTS,), float("nan"), dtype=torch.float64, device=dev)
        fd = torch.full((n, 3), float("nan"), dtype=torch.float64, device=dev)
        capi.evaluate_noalloc(n, xd.data_ptr(), qd.data_ptr(), sd.data_ptr(), ed.data_ptr(),
                              od.data_ptr(), id_.data_ptr(), dd.data_ptr(), s.box, s.cutoff, s.eps_rf,
                              p, rd.data_ptr(), fd.data_ptr(), st.cuda_stream)
        st.synchronize()
        r = rd.cpu().numpy()
        F = fd.cpu().numpy()
        assert r[capi.R_STATUS] == 0, call
        assert abs(r[capi.R_U0] - ref[capi.R_U0]) < energy_tol(ref[capi.R_U0], 50000), call
        assert abs(r[capi.R_U] - ref[capi.R_U]) < U_ABS_TOL, call
        for k in (capi.R_BINDE, capi.R_W, capi.R_EPOT):
            assert abs(r[k] - ref[k]) < U_ABS_TOL + 1e-6 * abs(ref[k]), (call, k)
        assert abs(r[capi.R_S] - ref[capi.R_S]) < 1e-6, call
        assert rms_rel(F, ref_F) < FORCE_RMS_REL_TOL, call


def _noalloc(s, x, p, displacement=True, forces=True):
    """One sdm_evaluate_noalloc call on device copies of the system's arrays:
    (results, mixed forces or None)."""
    import torch
    n = s.n
    dev = torch.device("cuda", 0)
    t = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    off, idx = _csr(n, s.exclusions)
    if idx.size == 0:
        idx = np.zeros(1, np.int32)
    xd, qd, sd, ed = t(x), t(s.charge), t(s.sigma), t(s.epsilon)
    dd = t(s.displacement) if displacement else None
    od, id_ = t(off, torch.int32), t(idx, torch.int32)
    rd = torch.full((capi.NRESULTS,), float("nan"), dtype=torch.float64, device=dev)
    fd = torch.full((n, 3), float("nan"), dtype=torch.float64, device=dev) if forces else None
    st = torch.cuda.Stream(device=dev)
    capi.evaluate_noalloc(n, xd.data_ptr(), qd.data_ptr(), sd.data_ptr(), ed.data_ptr(),
                          od.data_ptr(), id_.data_ptr(), dd.data_ptr() if dd is not None else 0,
                          s.box, s.cutoff, s.eps_rf, p, rd.data_ptr(),
                          fd.data_ptr() if fd is not None else 0, st.cuda_stream)
    st.synchronize()
    return rd.cpu().numpy(), (fd.cpu().numpy() if fd is not None else None)


def _check_oracle(s, x, r, F):
    import oracle
    b = oracle.OracleSystem(s).states(x)
    assert r[capi.R_STATUS] == 0
    assert abs(r[capi.R_U0] - b["U0"]) < energy_tol(b["U0"], b["P0"]) + 0.05, (r[capi.R_U0], b["U0"])
    assert abs(r[capi.R_U] - b["u_direct"]) < U_ABS_TOL, (r[capi.R_U], b["u_direct"])
    sw = r[capi.R_S]
    assert rms_rel(F, sw * b["F1"] + (1 - sw) * b["F0"]) < FORCE_RMS_REL_TOL
    return b


@pytest.mark.gpu
def test_noalloc_against_the_oracle():
    s = S.config0(variant="b")
    x = s.positions[0]
    r, F = _noalloc(s, x, s.params[0].as_array())
    _check_oracle(s, x, r, F)


@pytest.mark.gpu
def test_noalloc_without_displacement_or_forces():
    import oracle
    s = S.config0(variant="b")
    x = s.positions[0]
    p = s.params[0].as_array()
    r_full, _ = _noalloc(s, x, p)
    # no displacement map: state 2 equals state 1, u = 0 and F = F0
    r, F = _noalloc(s, x, p, displacement=False)
    assert r[capi.R_STATUS] == 0
    assert r[capi.R_U] == 0.0
    assert r[capi.R_U0] == r_full[capi.R_U0]
    b = oracle.OracleSystem(s).states(x)
    assert rms_rel(F, b["F0"]) < FORCE_RMS_REL_TOL
    # no force output: the same results, bit for bit
    r2, F2 = _noalloc(s, x, p, forces=False)
    assert F2 is None
    assert np.array_equal(r2, r_full)


@pytest.mark.gpu
def test_noalloc_long_exclusion_list_matches_handle_and_oracle():
    # particle 0 excludes its 150 nearest neighbours: more than the per-warp
    # shared-memory copy holds, so its partners are scanned in global memory
    s = S.config0(variant="b")
    x = s.positions[0]
    dv = x - x[0]
    dv -= s.box * np.round(dv / s.box)
    near = np.argsort(np.einsum("ij,ij->i", dv, dv))[1:151]
    extra = np.stack([np.zeros(150, np.int64), near], 1)
    ex = np.unique(np.sort(np.concatenate([s.exclusions, extra]), axis=1), axis=0).astype(np.int32)
    s2 = dataclasses.replace(s, exclusions=ex)
    p = s2.params[0].as_array()
    r, F = _noalloc(s2, x, p)
    _check_oracle(s2, x, r, F)
    h = capi.Handle([s2])
    h.set_params(0, p)
    ref_res, ref_F = h.evaluate(x)
    h.close()
    assert abs(r[capi.R_U0] - ref_res[0, capi.R_U0]) < energy_tol(ref_res[0, capi.R_U0], 50000)
    assert abs(r[capi.R_U] - ref_res[0, capi.R_U]) < U_ABS_TOL
    assert rms_rel(F, ref_F) < FORCE_RMS_REL_TOL


@pytest.mark.gpu
def test_noalloc_force_overflow_in_status():
    # the clash variant: displaced ligand atoms land on solvent sites, state-2
    # pair forces beyond the fixed-point range
    s = S.config0(variant="a")
    r, F = _noalloc(s, s.positions[0], s.params[0].as_array())
    assert int(r[capi.R_STATUS]) & capi.DEV_FORCE_OVERFLOW
    # the next call on a clean system starts from a cleared status word
    sb = S.config0(variant="b")
    rb, _ = _noalloc(sb, sb.positions[0], sb.params[0].as_array())
    assert rb[capi.R_STATUS] == 0


@pytest.mark.gpu
def test_noalloc_at_the_size_limit():
    n_max = capi.NOALLOC_MAX_PARTICLES
    hg = S.host_guest(n_max - 30, 41, nstates=1)
    pad = n_max - hg.n
    rng = np.random.default_rng(42)
    pos = np.concatenate([hg.positions[0], rng.uniform(0, hg.box, (pad, 3))])
    z = np.zeros(pad)
    s = dataclasses.replace(
        hg, charge=np.concatenate([hg.charge, z]), sigma=np.concatenate([hg.sigma, z]),
        epsilon=np.concatenate([hg.epsilon, z]),
        displacement=np.concatenate([hg.displacement, np.zeros((pad, 3))]), positions=pos[None],
        ligand_atoms=hg.ligand_atoms)
    assert s.n == n_max
    r, F = _noalloc(s, s.positions[0], s.params[0].as_array())
    _check_oracle(s, s.positions[0], r, F)
