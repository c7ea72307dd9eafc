"""Differentiation (backward of the SDM potential).

CPU: the dense FP64 torch reference against the oracle; the partial
derivatives of W against finite differences of the restated combine.
GPU: the autograd Function (adjoint kernel) against FP64 central finite
differences of the oracle (h = 1e-5, the 930-site system) and against the
dense FP64 torch reference (a 2k-particle host-guest system).
"""
import dataclasses

import numpy as np
import pytest
import torch

import oracle
from dense_sdm import candidate_pairs, potential
from openmm_sdm_plugin_gb300 import systems as S
from openmm_sdm_plugin_gb300 import capi
from openmm_sdm_plugin_gb300.autograd import bias_partials

GRAD_REL_TOL = 2e-4   # gradient vs FP64 reference: FP32 pair terms, FP64 sums


def _params(alpha=0.1):
    return S.SDMParams(bias_method=2, softcore_method=2, lambdac=0.4, lambda1=0.2, lambda2=0.5,
                       alpha=alpha, u0=110.0, w0=1.5, umax=200.0, acore=1 / 16, ubcore=100.0)


def _system():
    s = S.config0(variant="b")
    s.params = [_params()]
    return s


def _u_lambda_oracle(s, p, q=None, sig=None, eps=None, d=None, x=None):
    s2 = dataclasses.replace(s, charge=s.charge if q is None else q, sigma=s.sigma if sig is None else sig,
                             epsilon=s.epsilon if eps is None else eps,
                             displacement=s.displacement if d is None else d)
    o = oracle.OracleSystem(s2)
    res, _ = oracle.eval_state(o, s.positions[0] if x is None else x, p.as_array(), forces=False)
    return res[6]


def test_dense_reference_matches_oracle():
    s = _system()
    p = s.params[0]
    x = torch.tensor(s.positions[0])
    t = lambda a: torch.tensor(np.asarray(a, np.float64))
    U, u = potential(s, x, t(s.charge), t(s.sigma), t(s.epsilon), t(s.displacement), t(p.lambda1),
                     t(p.lambda2), t(p.alpha), t(p.u0), t(p.w0), p)
    o = oracle.OracleSystem(s)
    res, _ = oracle.eval_state(o, s.positions[0], p.as_array(), forces=False)
    assert float(u) == pytest.approx(res[0], rel=1e-10, abs=1e-8)
    assert float(U) == pytest.approx(res[6], rel=1e-10, abs=1e-8)


@pytest.mark.parametrize("be", [-30.0, 50.0, 110.0, 180.0])
def test_bias_partials_fd(be):
    p = _params()
    h = 1e-6
    d = bias_partials(p, be)
    for key in ("lambda1", "lambda2", "alpha", "u0", "w0"):
        pp = dataclasses.replace(p, **{key: getattr(p, key) + h})
        pm = dataclasses.replace(p, **{key: getattr(p, key) - h})
        # W at fixed u' = be: combine with soft core off and u = be
        Wp = oracle.combine(dataclasses.replace(pp, softcore_method=0).as_array(), 0.0, be)[3]
        Wm = oracle.combine(dataclasses.replace(pm, softcore_method=0).as_array(), 0.0, be)[3]
        assert d[key] == pytest.approx((Wp - Wm) / (2 * h), rel=1e-6, abs=1e-8), key


@pytest.mark.parametrize("method", [0, 1, 2])
def test_bias_partials_batched_matches_scalar(method):
    """The batched partials used on the device equal the scalar ones, per
    replica, for every bias method (alpha = 0 included)."""
    from openmm_sdm_plugin_gb300.autograd import bias_partials_device
    rng = np.random.default_rng(method)
    R = 7
    be = rng.uniform(-50, 250, R)
    l1, l2 = rng.uniform(0, 1, R), rng.uniform(0, 1, R)
    al = np.where(np.arange(R) % 3 == 0, 0.0, rng.uniform(0.01, 0.3, R))
    u0 = rng.uniform(50, 150, R)
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    out = bias_partials_device(torch.full((R,), method), t(be), t(l1), t(l2), t(al), t(u0))
    for r in range(R):
        p = S.SDMParams(bias_method=method, lambda1=l1[r], lambda2=l2[r], alpha=al[r], u0=u0[r])
        ref = bias_partials(p, be[r])
        for k, key in enumerate(("lambda1", "lambda2", "alpha", "u0", "w0")):
            assert float(out[k][r]) == pytest.approx(ref[key], rel=1e-13, abs=1e-13), (r, key)


def _gpu_grads(s):
    from openmm_sdm_plugin_gb300.autograd import SDMEngine, sdm_potential
    eng = SDMEngine(s)
    D = eng.D
    f64 = dict(dtype=torch.float64)
    x = torch.tensor(s.positions, **f64, requires_grad=True)
    qD = torch.tensor(s.charge[D], **f64, requires_grad=True)
    sD = torch.tensor(s.sigma[D], **f64, requires_grad=True)
    eD = torch.tensor(s.epsilon[D], **f64, requires_grad=True)
    d = torch.tensor(s.displacement, **f64, requires_grad=True)
    ps = s.params
    vec = lambda k: torch.tensor([getattr(p, k) for p in ps], **f64, requires_grad=True)
    l1, l2, al, u0, w0 = vec("lambda1"), vec("lambda2"), vec("alpha"), vec("u0"), vec("w0")
    U = sdm_potential(eng, x, qD, sD, eD, d, l1, l2, al, u0, w0)
    U.sum().backward()
    eng.close()
    return D, U.detach(), dict(x=x.grad, q=qD.grad, sigma=sD.grad, eps=eD.grad, d=d.grad, lambda1=l1.grad,
                               lambda2=l2.grad, alpha=al.grad, u0=u0.grad, w0=w0.grad)


@pytest.mark.gpu
def test_gradients_vs_oracle_central_differences():
    s = _system()
    p = s.params[0]
    D, U, g = _gpu_grads(s)
    U_ref = _u_lambda_oracle(s, p)
    assert float(U[0]) == pytest.approx(U_ref, abs=0.05)
    h = 1e-5
    rng = np.random.default_rng(0)
    ks = rng.choice(len(D), 4, replace=False)
    for name, arr, grad in (("q", s.charge, g["q"]), ("sigma", s.sigma, g["sigma"]),
                            ("eps", s.epsilon, g["eps"])):
        for k in ks:
            a_p = arr.copy(); a_p[D[k]] += h
            a_m = arr.copy(); a_m[D[k]] -= h
            Up = _u_lambda_oracle(s, p, **{("q" if name == "q" else "sig" if name == "sigma" else "eps"): a_p})
            Um = _u_lambda_oracle(s, p, **{("q" if name == "q" else "sig" if name == "sigma" else "eps"): a_m})
            fd = (Up - Um) / (2 * h)
            assert float(grad[k]) == pytest.approx(fd, rel=GRAD_REL_TOL, abs=1e-3), (name, k)
    # the ligand's displacement vector: d = v * (1,0,0) for every ligand site
    for c in range(3):
        dp = s.displacement.copy(); dp[D, c] += h
        dm = s.displacement.copy(); dm[D, c] -= h
        fd = (_u_lambda_oracle(s, p, d=dp) - _u_lambda_oracle(s, p, d=dm)) / (2 * h)
        assert float(g["d"][D, c].sum()) == pytest.approx(fd, rel=GRAD_REL_TOL, abs=1e-3), c
    for key in ("lambda1", "lambda2", "alpha", "u0", "w0"):
        fd = (_u_lambda_oracle(s, dataclasses.replace(p, **{key: getattr(p, key) + h})) -
              _u_lambda_oracle(s, dataclasses.replace(p, **{key: getattr(p, key) - h}))) / (2 * h)
        assert float(g[key][0]) == pytest.approx(fd, rel=GRAD_REL_TOL, abs=1e-4), key
    # positions: one solvent site and one ligand site
    for i in (5, int(D[3])):
        xp = s.positions[0].copy(); xp[i, 1] += h
        xm = s.positions[0].copy(); xm[i, 1] -= h
        fd = (_u_lambda_oracle(s, p, x=xp) - _u_lambda_oracle(s, p, x=xm)) / (2 * h)
        assert float(g["x"][0, i, 1]) == pytest.approx(fd, rel=GRAD_REL_TOL, abs=1e-3), i


@pytest.mark.gpu
def test_gradients_vs_dense_torch_2k():
    s = S.host_guest(2000, 4, nstates=2)
    s.params = [_params(), dataclasses.replace(_params(), lambda1=0.6, lambda2=0.7, u0=90.0)]
    D, U, g = _gpu_grads(s)
    t = lambda a, rg=False: torch.tensor(np.asarray(a, np.float64), requires_grad=rg)
    for r in range(2):
        p = s.params[r]
        x = t(s.positions[r], True)
        q, sg, ep, d = t(s.charge, True), t(s.sigma, True), t(s.epsilon, True), t(s.displacement, True)
        sc = [t(getattr(p, k), True) for k in ("lambda1", "lambda2", "alpha", "u0", "w0")]
        pairs = candidate_pairs(s, s.positions[r], s.displacement)
        Ur, _ = potential(s, x, q, sg, ep, d, *sc, p, pairs=pairs)
        Ur.backward()
        assert float(U[r]) == pytest.approx(float(Ur.detach()), abs=0.05)
        gr = {"q": q.grad[D], "sigma": sg.grad[D], "eps": ep.grad[D]}
        for k, key in enumerate(("lambda1", "lambda2", "alpha", "u0", "w0")):
            assert float(g[key][r]) == pytest.approx(float(sc[k].grad), rel=GRAD_REL_TOL, abs=1e-4), key
        assert torch.allclose(g["x"][r], x.grad, rtol=1e-4, atol=1e-3 * float(x.grad.abs().max()))
        if r == 0:
            acc = {k: v.clone() for k, v in gr.items()}
            accd = d.grad.clone()
        else:
            for k in acc:
                acc[k] += gr[k]
            accd += d.grad
    # parameters are shared by both replicas: gradients add up
    for key in ("q", "sigma", "eps"):
        ref = acc[key]
        scale = float(ref.abs().max())
        assert torch.allclose(g[key], ref, rtol=GRAD_REL_TOL, atol=1e-4 * scale), key
    scale = float(accd.abs().max())
    assert torch.allclose(g["d"], accd, rtol=GRAD_REL_TOL, atol=1e-4 * scale)


@pytest.mark.gpu
def test_ti_dudlambda_chain_rule():
    """dU/dlambda of the stand-in two-leg schedule (lambda2 = l, lambda1 =
    l - 0.1 sin(pi l)) by autograd through the schedule vs finite differences."""
    from openmm_sdm_plugin_gb300.autograd import SDMEngine, sdm_potential
    s = _system()
    eng = SDMEngine(s)
    D = eng.D
    f64 = dict(dtype=torch.float64)

    def U_of(lam_value, grad=False):
        lam = torch.tensor([lam_value], **f64, requires_grad=grad)
        l2 = lam
        l1 = lam - 0.1 * torch.sin(np.pi * lam)
        a = torch.tensor([0.1], **f64)
        u0 = torch.tensor([110.0], **f64)
        w0 = torch.tensor([0.0], **f64)
        U = sdm_potential(eng, torch.tensor(s.positions, **f64), torch.tensor(s.charge[D], **f64),
                          torch.tensor(s.sigma[D], **f64), torch.tensor(s.epsilon[D], **f64),
                          torch.tensor(s.displacement, **f64), l1, l2, a, u0, w0)
        return U, lam

    U, lam = U_of(0.37, grad=True)
    U.sum().backward()
    h = 1e-5
    fd = (float(U_of(0.37 + h)[0]) - float(U_of(0.37 - h)[0])) / (2 * h)
    eng.close()
    assert float(lam.grad) == pytest.approx(fd, rel=1e-6, abs=1e-6)


@pytest.mark.gpu
def test_num_perturbed_follows_the_displacement_rule_and_device_adjoint_matches():
    """The adjoint output holds 6 doubles per (replica, displaced particle);
    the library's count is the one callers size their buffers from.  A
    particle is displaced iff its displacement vector is nonzero (-0.0 counts
    as zero).  The device variant writes the same sums as the host one."""
    from openmm_sdm_plugin_gb300 import capi
    s = S.config2(nrep=2)
    h = capi.Handle([s])
    for r in range(2):
        h.set_params(r, s.params[r].as_array())
    nd = int(np.count_nonzero(np.any(s.displacement != 0, axis=1)))
    assert h.num_perturbed() == 2 * nd
    d = s.displacement.copy()
    lig = np.nonzero(np.any(d != 0, axis=1))[0]
    d[lig[0]] = [-0.0, -0.0, -0.0]
    d[0] = [0.0, 0.0, 1e-300]
    h.set_displacement(0, d)
    assert h.num_perturbed() == 2 * nd
    d[lig[1]] = 0.0
    h.set_displacement(0, d)
    assert h.num_perturbed() == 2 * (nd - 1)
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    h.evaluate(x)
    G = h.adjoint()
    out = torch.full((6 * h.num_perturbed(),), float("nan"), dtype=torch.float64, device="cuda")
    st = torch.cuda.Stream()
    h.adjoint_device(out.data_ptr(), st.cuda_stream)
    st.synchronize()
    assert np.array_equal(out.cpu().numpy(), G.reshape(-1))
    with pytest.raises(ValueError):
        h.adjoint(n_displaced=nd)
    h.close()


@pytest.mark.gpu
def test_library_backward_matches_torch_formulas():
    """sdm_backward_device (one kernel) against the same gradients written as
    torch operations on the forward's outputs: three lambda states (every
    bias method), random upstream gradients, all outputs at 1e-12; outputs
    that are not wanted are skipped."""
    from openmm_sdm_plugin_gb300.autograd import SDMEngine, bias_partials_device
    s = S.host_guest(1500, seed=5, nstates=3)
    for r, m in enumerate((0, 1, 2)):
        s.params[r] = dataclasses.replace(s.params[r], bias_method=m, alpha=0.05 * (r + 1), u0=20.0 * r)
    eng = SDMEngine(s)
    dev = eng.dev
    f64 = dict(dtype=torch.float64, device=dev)
    D = eng.D
    x = torch.tensor(s.positions, **f64)
    vec = lambda k: torch.tensor([getattr(p, k) for p in s.params], **f64)
    lam = [vec(k) for k in ("lambda1", "lambda2", "alpha", "u0", "w0")]
    qD, sD, eD = (torch.tensor(a[D], **f64) for a in (s.charge, s.sigma, s.epsilon))
    d = torch.tensor(s.displacement, **f64)
    U, sw, F, F1, G, res = eng.run(x, qD, sD, eD, d, *lam)
    res, F, F1, G = res.clone(), F.clone(), F1.clone(), G.clone()
    prm = torch.stack(lam[:4])
    g = torch.randn(eng.R, **f64)
    gx, gp, gd, gb = eng.backward(g, res, F, F1, G, eD, prm, (True, True, True, True))
    torch.cuda.synchronize()
    s_ = res[:, capi.R_S]
    w = torch.stack([(1.0 - s_), s_], dim=1)
    gD = torch.einsum("r,rs,rksc->kc", g, w, G)
    ref_e = torch.where(eD > 0, gD[:, 2] / (2.0 * eD), torch.zeros_like(eD))
    part = bias_partials_device(eng.methods, res[:, capi.R_BINDE], *lam[:4])
    close = lambda a, b: torch.allclose(a, b, rtol=1e-12, atol=1e-12 * float(b.abs().max() + 1e-300))
    assert close(gx, -g[:, None, None] * F)
    assert close(gd, -torch.einsum("r,r,rnc->nc", g, s_, F1))
    assert close(gp[:, 0], gD[:, 0]) and close(gp[:, 1], gD[:, 1]) and close(gp[:, 2], ref_e)
    for k in range(5):
        assert close(gb[k], g * part[k]), k
    # nothing requested but the bias rows
    gx2, gp2, gd2, gb2 = eng.backward(g, res, F, F1, G, eD, prm, (False, False, False, True))
    assert gx2 is None and gp2 is None and gd2 is None and torch.equal(gb2, gb)
    eng.close()


@pytest.mark.gpu
def test_backward_device_two_systems_against_numpy():
    """sdm_backward_device on a handle of two systems (3 and 2 lambda states,
    different sizes and ligands): every output against the same sums in
    numpy from the evaluation's results, forces, state forces and adjoint
    sums; per-system displacement and parameter gradients over that system's
    replicas only."""
    from openmm_sdm_plugin_gb300.autograd import bias_partials
    sysms = [S.host_guest(1500, seed=5, nstates=3), S.host_guest(2200, seed=7, nstates=2)]
    h = capi.Handle(sysms)
    r = 0
    for s_ in sysms:
        for p in s_.params:
            h.set_params(r, p.as_array())
            r += 1
    R = h.nrep
    f64 = dict(dtype=torch.float64, device="cuda")
    x = torch.from_numpy(np.concatenate([s_.positions.reshape(-1, 3) for s_ in sysms])).to(**f64)
    res = torch.zeros((R, capi.NRESULTS), **f64)
    F = torch.zeros_like(x)
    F1 = torch.zeros_like(x)
    npert = h.num_perturbed()
    G = torch.zeros(6 * npert, **f64)
    st = torch.cuda.Stream()
    s0 = st.cuda_stream
    h.evaluate_device(x.data_ptr(), res.data_ptr(), F.data_ptr(), s0)
    h.state_forces_device(0, F1.data_ptr(), s0)
    h.adjoint_device(G.data_ptr(), s0)
    Ds = [np.nonzero(np.any(np.asarray(s_.displacement).reshape(-1, 3) != 0, axis=1))[0] for s_ in sysms]
    eps = torch.from_numpy(np.concatenate([s_.epsilon[D] for s_, D in zip(sysms, Ds)])).to(**f64)
    g = torch.randn(R, **f64)
    natoms = sum(s_.n for s_ in sysms)
    gx = torch.empty_like(x)
    gd = torch.empty((natoms, 3), **f64)
    gp = torch.empty((eps.numel(), 3), **f64)
    gb = torch.empty((5, R), **f64)
    h.backward_device(g.data_ptr(), res.data_ptr(), F.data_ptr(), F1.data_ptr(), G.data_ptr(), eps.data_ptr(), 0,
                      gx.data_ptr(), gd.data_ptr(), gp.data_ptr(), gb.data_ptr(), s0)
    torch.cuda.synchronize()
    res_, F_, F1_, G_, g_ = (t.cpu().numpy() for t in (res, F, F1, G, g))
    gx_, gd_, gp_, gb_ = (t.cpu().numpy() for t in (gx, gd, gp, gb))
    sw = res_[:, capi.R_S]
    close = lambda a, b: np.allclose(a, b, rtol=1e-12, atol=1e-12 * (np.abs(b).max() + 1e-300))
    # rows of every replica, replicas numbered system by system
    row, r, rep_rows, rep_sys = 0, 0, [], []
    for k, s_ in enumerate(sysms):
        for q in range(s_.replicas):
            rep_rows.append(slice(row, row + s_.n))
            rep_sys.append(k)
            row += s_.n
    for q in range(R):
        assert close(gx_[rep_rows[q]], -g_[q] * F_[rep_rows[q]])
    Gq = G_.reshape(-1, 2, 3)
    d0, a0, p0 = 0, 0, 0
    for k, (s_, D) in enumerate(zip(sysms, Ds)):
        reps = [q for q in range(R) if rep_sys[q] == k]
        ref_d = -sum(g_[q] * sw[q] * F1_[rep_rows[q]] for q in reps)
        assert close(gd_[a0:a0 + s_.n], ref_d), k
        ref_p = np.zeros((len(D), 3))
        for q in reps:
            off = sum(len(Ds[rep_sys[qq]]) for qq in range(q))
            ref_p += g_[q] * ((1 - sw[q]) * Gq[off:off + len(D), 0] + sw[q] * Gq[off:off + len(D), 1])
        ref_p[:, 2] = np.where(s_.epsilon[D] > 0, ref_p[:, 2] / (2 * s_.epsilon[D]), 0.0)
        assert close(gp_[p0:p0 + len(D)], ref_p), k
        a0 += s_.n
        p0 += len(D)
    q = 0
    for s_ in sysms:
        for p in s_.params:
            ref = bias_partials(p, res_[q, capi.R_BINDE])
            for kk, key in enumerate(("lambda1", "lambda2", "alpha", "u0", "w0")):
                assert gb_[kk, q] == pytest.approx(g_[q] * ref[key], rel=1e-12, abs=1e-12), (q, key)
            q += 1
    h.close()
