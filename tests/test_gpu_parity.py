"""GPU parity tests: the CUDA path through the C ABI against the FP64 oracle.

Two oracle rules are used (see oracle/sdm_oracle.c):
  * fp32 rule  -- the exact pair sets of the CUDA kernels, FP64 arithmetic:
                  index maps, lists and pair counts must agree bit for bit,
                  energies/forces to FP32-rounding level;
  * fp64 rule  -- the physics oracle (a pair interacts iff its FP64 distance
                  is below the cutoff): u within 5e-3 kJ/mol, forces within
                  1e-4 rms relative.
"""
import dataclasses

import numpy as np
import pytest

import oracle
from helpers import FORCE_RMS_REL_TOL, U_ABS_TOL, check_replica, energy_tol, rms_rel
from openmm_sdm_plugin_gb300 import capi, systems as S

pytestmark = pytest.mark.gpu


def _handle(sysms):
    h = capi.Handle(sysms)
    r = 0
    for s in sysms:
        for p in s.params:
            h.set_params(r, p.as_array())
            r += 1
    return h


def test_config0_parity():
    s = S.config0(variant="b")
    h = _handle([s])
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    check_replica(s, x, res[0], F, F0, F1, h.grid(0))
    assert res[0, capi.R_STATUS] == 0


def test_nonfinite_coordinates_are_reported():
    """A NaN or Inf coordinate sets SDM_DEV_COORD_NONFINITE: the host call
    fails with SDM_ERR_OVERFLOW, the device status carries the bit, and the
    next call on finite coordinates is clean."""
    s = S.config0(variant="b")
    h = _handle([s])
    for bad in (np.nan, np.inf, -np.inf):
        x = s.positions[0].copy()
        x[17, 1] = bad
        with pytest.raises(capi.SdmError) as e:
            h.evaluate(x)
        assert e.value.status == capi.SDM_ERR_OVERFLOW
        h.set_option(capi.OPT_VERIFY, 0)
        res, _ = h.evaluate(x)
        h.set_option(capi.OPT_VERIFY, 1)
        assert int(res[0, capi.R_STATUS]) & capi.DEV_COORD_NONFINITE
        assert h.check_status() & capi.DEV_COORD_NONFINITE
    res, F = h.evaluate(s.positions[0])
    assert res[0, capi.R_STATUS] == 0 and np.isfinite(F).all()


def test_config0a_clash_overflow_is_reported():
    """Config 0a displaces the ligand into solvent: state-2 forces reach
    ~5.6e9 kJ/mol/nm, beyond the 2^31 range of the 2^32-scaled fixed point.
    The host call must fail with SDM_ERR_OVERFLOW; energies, u and F0 stay
    valid and are still checked."""
    s = S.config0(variant="a")
    h = _handle([s])
    x = s.positions[0]
    with pytest.raises(capi.SdmError) as e:
        h.evaluate(x)
    assert e.value.status == capi.SDM_ERR_OVERFLOW
    h.set_option(capi.OPT_VERIFY, 0)
    res, F = h.evaluate(x)
    assert int(res[0, capi.R_STATUS]) & 1
    assert h.check_status() & 1
    F0, _ = h.state_forces()
    o = oracle.OracleSystem(s)
    b = o.states(x)
    a = o.f32rule(x, h.grid(0))
    assert abs(res[0, capi.R_U0] - b["U0"]) < energy_tol(b["U0"], b["P0"]) + 0.05
    # u is dominated by clash pairs at r ~ 0.05 nm, where the r^-12 term
    # amplifies FP32 coordinate rounding (~1e-6 relative in r) twelve-fold:
    # the achievable relative accuracy is ~1e-5, so the bound is 1e-4
    assert abs(res[0, capi.R_U] - a["u"]) < 1e-4 * abs(a["u"])
    assert abs(res[0, capi.R_U] - b["u_direct"]) < 1e-4 * abs(b["u_direct"])
    assert rms_rel(F0, b["F0"]) < FORCE_RMS_REL_TOL


def test_config1_parity():
    s = S.config1()
    h = _handle([s])
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    a, b = check_replica(s, x, res[0], F, F0, F1, h.grid(0))
    print("config1 U0", res[0, capi.R_U0], "u", res[0, capi.R_U], "oracle u", b["u_direct"])


def test_config1b_logistic_term():
    s = S.config1(variant="b")
    h = _handle([s])
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    check_replica(s, x, res[0], F, F0, F1, h.grid(0))


def test_pair_counts_exact():
    for s in (S.config0(), S.config0(variant="b"), S.config1()):
        h = _handle([s])
        c = h.count_pairs(s.positions[0])
        a = oracle.OracleSystem(s).f32rule(s.positions[0], h.grid(0))
        assert int(c[0, 0]) == a["P0"]
        assert int(c[0, 1]) == a["P1delta"]


def _assert_lists_match_oracle(g, s, x, M):
    o = oracle.OracleSystem(s)
    c = o.clusters(x, M)
    assert g["ncl"] == c["ncl"]
    assert np.array_equal(g["perm"], c["perm"])
    ol = o.lists(x, M)
    assert np.array_equal(g["cnt"], ol["cnt"])
    for I in range(g["ncl"]):
        k = g["cnt"][I]
        gs, gm = g["slot"][I, :k], g["mask"][I, :k]
        order = np.argsort(gs, kind="stable")
        assert np.array_equal(gs[order], ol["slot"][I, :k])
        assert np.array_equal(gm[order], ol["mask"][I, :k])


@pytest.mark.parametrize("which", ["config0", "config1"])
def test_clusters_and_lists_bit_exact(which):
    s = S.config0() if which == "config0" else S.config1()
    h = _handle([s])
    x = s.positions[0]
    _assert_lists_match_oracle(h.export_lists(0, x), s, x, h.grid(0))


def test_batched_lists_bit_exact():
    """The 22-replica batch has more list-building groups than the builder's
    resident warps, so after their first group the warps take groups from a
    counter; the first and the last replica's clusters and lists still equal
    the oracle's bit for bit."""
    s = S.config2(22)
    h = _handle([s])
    h.evaluate(s.positions.reshape(-1, 3))   # every replica's coordinates resident
    for r in (0, 21):
        x = s.positions[r]
        _assert_lists_match_oracle(h.export_lists(r, x), s.replica(r), x, h.grid(0))


def test_list_groups_give_the_same_lists():
    """Lists built for groups of 1, 2 and 4 z-consecutive clusters (and the
    automatic choice) hold the same entries per i-cluster; the evaluations
    agree to FP32 summation order (tile composition may differ)."""
    s = S.config1()
    h = _handle([s])
    x = s.positions[0]
    assert h.get_option(capi.OPT_LIST_GROUP) == 0
    ref = None
    for g in (0, 1, 2, 4):
        h.set_option(capi.OPT_LIST_GROUP, g)
        L = h.export_lists(0, x)
        res, F = h.evaluate(x)
        ent = [sorted(zip(L["slot"][I, :L["cnt"][I]].tolist(), L["mask"][I, :L["cnt"][I]].tolist()))
               for I in range(L["ncl"])]
        if ref is None:
            ref = (ent, res, F)
            continue
        assert ent == ref[0], g
        for k in (capi.R_U0, capi.R_U1, capi.R_U):
            assert abs(res[0, k] - ref[1][0, k]) <= 1e-6 * max(1.0, abs(ref[1][0, k])), (g, k)
        assert np.abs(F - ref[2]).max() < 1e-3, g
    with pytest.raises(capi.SdmError):
        h.set_option(capi.OPT_LIST_GROUP, 3)


def test_batched_replicas_match_single():
    s = S.config2(nrep=4)
    h = _handle([s])
    x = s.positions.reshape(-1, 3)
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    n = s.n
    M = h.grid(0)
    for r in range(4):
        sr = s.replica(r)
        sl = slice(r * n, (r + 1) * n)
        check_replica(sr, s.positions[r], res[r], F[sl], F0[sl], F1[sl], M)


def test_uneven_multisystem_batch():
    sysms = [S.host_guest(2500, 11, nstates=2), S.host_guest(7000, 12, nstates=3),
             S.host_guest(4000, 13, nstates=1)]
    h = _handle(sysms)
    x = np.concatenate([s.positions.reshape(-1, 3) for s in sysms])
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    off = 0
    r = 0
    for k, s in enumerate(sysms):
        M = h.grid(k)
        for q in range(s.replicas):
            sr = s.replica(q)
            sl = slice(off, off + s.n)
            check_replica(sr, s.positions[q], res[r], F[sl], F0[sl], F1[sl], M)
            off += s.n
            r += 1


def test_deterministic_bitwise():
    s = S.config1()
    h = _handle([s])
    x = s.positions[0]
    r1, F1 = h.evaluate(x)
    r2, F2 = h.evaluate(x)
    assert np.array_equal(r1, r2)
    assert np.array_equal(F1, F2)


def test_overlapped_perturbation_pass_same_bits():
    """The perturbation pass on a second stream branch joined after (default)
    or before the main pass, against one stream, captured and eager: the same
    results and forces bit for bit, state forces included."""
    s = S.config2(nrep=3)
    h = _handle([s])
    x = s.positions.reshape(-1, 3)
    assert h.get_option(capi.OPT_OVERLAP) == 2
    out = {}
    for overlap in (2, 1, 0):
        for graph in (1, 0):
            h.set_option(capi.OPT_OVERLAP, overlap)
            h.set_option(capi.OPT_GRAPH, graph)
            r, F = h.evaluate(x)
            out[overlap, graph] = (r, F) + h.state_forces()
    ref = out[2, 1]
    assert np.all(ref[0][:, capi.R_STATUS] == 0)
    for k, v in out.items():
        for a, b in zip(v, ref):
            assert np.array_equal(a, b), k


@pytest.mark.parametrize("bias", [0, 1, 2])
@pytest.mark.parametrize("soft", [0, 1, 2])
def test_bias_and_softcore_methods(bias, soft):
    s = S.config0(variant="b")
    s.params = [S.SDMParams(bias_method=bias, softcore_method=soft, lambdac=0.4, lambda1=0.25,
                            lambda2=0.6, alpha=0.05, u0=50.0, w0=1.5, gamma=0.002, wb=0.3,
                            umax=200.0, acore=1 / 16, ubcore=20.0)]
    h = _handle([s])
    res, F = h.evaluate(s.positions[0])
    comb = oracle.combine(s.params[0].as_array(), res[0, capi.R_U0], res[0, capi.R_U1])
    for k, idx in ((1, capi.R_BINDE), (2, capi.R_FP), (3, capi.R_W), (4, capi.R_DW), (5, capi.R_S)):
        assert res[0, idx] == pytest.approx(comb[k], rel=1e-9, abs=1e-12)


@pytest.mark.parametrize("bias", [0, 1, 2])
def test_nonequilibrium_dwdlambda(bias):
    # linear and quadratic bias: the reference's dW/dlambda sees alpha = 1 and
    # u0 = 0 (ReferenceSDMKernels.cpp:214-217,236-239,289-297); the oracle's CPU
    # tests pin that scoping, this compares the device with the oracle
    s = S.config0(variant="b")
    s.params = [S.SDMParams(bias_method=bias, softcore_method=2, alpha=0.1, noneq=1, lambdac=0.3,
                            m_lambda1=0.8, m_lambda2=1.0, m_u0=20.0, m_w0=2.0, b_lambda1=0.05,
                            b_u0=100.0, gamma=0.01, wb=0.4, umax=200, acore=1 / 16, ubcore=100)]
    h = _handle([s])
    res, _ = h.evaluate(s.positions[0])
    comb = oracle.combine(s.params[0].as_array(), res[0, capi.R_U0], res[0, capi.R_U1])
    assert res[0, capi.R_DWDL] == pytest.approx(comb[7], rel=1e-9)
    assert res[0, capi.R_W] == pytest.approx(comb[3], rel=1e-9, abs=1e-12)
    assert res[0, capi.R_L1] == pytest.approx(0.8 * 0.3 + 0.05)
    assert res[0, capi.R_U0P] == pytest.approx(20 * 0.3 + 100)


def test_device_api_and_graph_replay():
    import torch
    s = S.config2(nrep=2)
    h = _handle([s])
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    rh, Fh = h.evaluate(x)
    xd = torch.from_numpy(x).cuda()
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    fd = torch.zeros_like(xd)
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(3):  # first call captures, the next ones replay the graph
        h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), st)
    torch.cuda.synchronize()
    assert np.array_equal(rd.cpu().numpy()[:, :14], rh[:, :14])
    assert np.array_equal(fd.cpu().numpy(), Fh)


def test_page_locked_host_buffers_in_place():
    """sdm_evaluate on page-locked host buffers (coordinates read in place by
    the kernels) equals the staged-copy path bit for bit, with page-locked or
    pageable outputs."""
    import torch
    s = S.config2(nrep=2)
    h = _handle([s])
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    assert h.get_option(capi.OPT_ZERO_COPY) == 0   # default: staged copies
    r_st, F_st = h.evaluate(x)
    h.set_option(capi.OPT_ZERO_COPY, 1)
    xp = torch.from_numpy(x.copy()).pin_memory()
    rp = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64).pin_memory()
    fp = torch.zeros_like(xp).pin_memory()
    for _ in range(3):   # capture, then replays of the graph with host-memory pointers
        rp.zero_()
        fp.zero_()
        h.evaluate_host_ptrs(xp.data_ptr(), rp.data_ptr(), fp.data_ptr())
        assert np.array_equal(rp.numpy()[:, :14], r_st[:, :14])
        assert np.array_equal(fp.numpy(), F_st)
    rn = np.zeros((h.nrep, capi.NRESULTS))
    h.evaluate_host_ptrs(xp.data_ptr(), rn.ctypes.data, fp.data_ptr())   # pageable results
    assert np.array_equal(rn[:, :14], r_st[:, :14])
    assert h.get_option(capi.OPT_ZERO_COPY) == 1


def test_translation_invariance_and_zero_displacement():
    s = S.config0(variant="b")
    h = _handle([s])
    x = s.positions[0]
    r1, _ = h.evaluate(x)
    r2, _ = h.evaluate(x + np.array([3.0 * 7 + 0.25, -3.0 * 2, 0.5]))
    assert abs(r1[0, capi.R_U] - r2[0, capi.R_U]) < U_ABS_TOL
    h.set_displacement(0, np.zeros((s.n, 3)))
    r3, F3 = h.evaluate(x)
    assert r3[0, capi.R_U] == 0.0
    F0, F1 = h.state_forces()
    assert np.array_equal(F0, F1)


def test_sdmforce_api_end_to_end():
    from openmm_sdm_plugin_gb300 import force_from_system
    s = S.config0(variant="b")
    f = force_from_system(s)
    E, F = f.evaluate(s.positions[0])
    o = oracle.OracleSystem(s)
    res, Fr = oracle.eval_state(o, s.positions[0], s.params[0].as_array())
    assert f.getBindE() == pytest.approx(res[1], abs=U_ABS_TOL)
    assert E == pytest.approx(res[6], abs=0.05)
    assert rms_rel(F, Fr) < FORCE_RMS_REL_TOL
    f.setSoftCoreMethod(9)
    with pytest.raises(capi.SdmError):
        f.evaluate(s.positions[0])


def _nonclique(s):
    """config1 with extra exclusions that make the exclusion graph non-clique:
    each water oxygen excluded with the next water's oxygen (one chain through
    the solvent), and each ligand particle with one solvent oxygen."""
    nw = (s.n - 80) // 3
    o = np.arange(nw - 1) * 3
    lig = np.arange(s.n - 80, s.n)
    extra = [np.stack([o, o + 3], 1), np.stack([(np.arange(80) * 97 % nw) * 3, lig], 1)]
    excl = np.concatenate([s.exclusions] + extra).astype(np.int32)
    return dataclasses.replace(s, name=s.name + "-nonclique", exclusions=excl)


def test_nonclique_exclusions_parity():
    s = _nonclique(S.config1())
    h = _handle([s])
    x = s.positions[0]
    res, F = h.evaluate(x)
    F0, F1 = h.state_forces()
    check_replica(s, x, res[0], F, F0, F1, h.grid(0))
    c = h.count_pairs(x)
    a = oracle.OracleSystem(s).f32rule(x, h.grid(0))
    assert int(c[0, 0]) == a["P0"]
    assert int(c[0, 1]) == a["P1delta"]
    g = h.export_lists(0, x)
    ol = oracle.OracleSystem(s).lists(x, h.grid(0))
    assert np.array_equal(g["cnt"], ol["cnt"])
    for I in range(g["ncl"]):
        k = g["cnt"][I]
        order = np.argsort(g["slot"][I, :k], kind="stable")
        assert np.array_equal(g["slot"][I, :k][order], ol["slot"][I, :k])
        assert np.array_equal(g["mask"][I, :k][order], ol["mask"][I, :k])


def test_pair_schedule_options():
    """Every accepted CTAs-per-SM request gives the same results; requests
    without a built register bound are refused; the launch never exceeds
    the resident CTAs."""
    s = S.config0(variant="b")
    h = _handle([s])
    x = s.positions[0]
    ref, Fref = h.evaluate(x)
    for c in (1, 2, 3, 4):
        h.set_option(capi.OPT_CTAS_PER_SM, c)
        res_c = h.get_option(capi.OPT_PAIR_RESIDENT)
        assert 1 <= res_c <= c
        for sp in (1, 2, 4):
            h.set_option(capi.OPT_SPLIT, sp)
            res, F = h.evaluate(x)
            if sp == 1:   # same work items, other warps: bit-identical
                assert np.array_equal(res[:, :capi.R_STATUS], ref[:, :capi.R_STATUS])
                assert np.array_equal(F, Fref)
            else:         # FP32 partial sums over other groups of list entries
                assert np.allclose(res[:, :capi.R_STATUS], ref[:, :capi.R_STATUS], rtol=1e-6, atol=1e-6)
                assert rms_rel(F, Fref) < 1e-6
    for bad in (0, 5):
        with pytest.raises(capi.SdmError):
            h.set_option(capi.OPT_CTAS_PER_SM, bad)


def test_default_stream_calls_are_ordered_with_torch():
    """On torch's default stream (cuda_stream 0, CUDA's legacy stream) the
    device calls are ordered with the caller's work: coordinates written by a
    torch copy just before the call are the ones evaluated, and results read
    by torch just after are the call's (the call bridges to the handle's
    stream with two event edges; no explicit synchronisation here)."""
    import torch
    s = S.config2(nrep=3)
    h = _handle([s])
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    ref_res, ref_F = h.evaluate(x)
    xh = torch.from_numpy(x).pin_memory()
    xd = torch.zeros_like(xh, device="cuda")
    rd = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    fd = torch.zeros_like(xd)
    assert torch.cuda.current_stream().cuda_stream == 0
    for k in range(6):
        xd.zero_()
        rd.zero_()
        xd.copy_(xh, non_blocking=True)           # default stream
        h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), 0)
        got = rd.cpu().numpy()                     # default stream, then host
        assert np.array_equal(got[:, :capi.R_STATUS], ref_res[:, :capi.R_STATUS]), k
        assert np.array_equal(fd.cpu().numpy(), ref_F), k
