"""CPU tests of the FP64 oracle: analytic known answers, dense cross-checks,
self-consistency and the restated combine (soft core, bias, mix)."""
import math

import numpy as np
import pytest

import oracle
from openmm_sdm_plugin_gb300 import systems as S

K = 138.935456


def two_particles(r, q=(0.5, -0.5), sig=(0.3, 0.34), eps=(0.5, 0.8), rc=1.0, erf=78.5, box=5.0):
    s = S.SDMSystem("pair", np.array([box] * 3), np.array(q), np.array(sig), np.array(eps),
                    np.zeros((0, 2), np.int32), np.zeros((2, 3)),
                    np.array([[[1.0, 1.0, 1.0], [1.0 + r, 1.0, 1.0]]]), [S.SDMParams()],
                    cutoff=rc, eps_rf=erf)
    return s


def analytic_pair(r, q, sig, eps, rc, erf):
    sg = 0.5 * (sig[0] + sig[1])
    ep = math.sqrt(eps[0] * eps[1])
    krf = (erf - 1) / ((2 * erf + 1) * rc ** 3)
    crf = 3 * erf / ((2 * erf + 1) * rc)
    e_lj = 4 * ep * ((sg / r) ** 12 - (sg / r) ** 6)
    e_rf = K * q[0] * q[1] * (1 / r + krf * r * r - crf)
    de_lj = 4 * ep * (-12 * sg ** 12 / r ** 13 + 6 * sg ** 6 / r ** 7)
    de_rf = K * q[0] * q[1] * (-1 / r ** 2 + 2 * krf * r)
    return e_lj + e_rf, de_lj + de_rf


@pytest.mark.parametrize("r", [0.25, 0.3, 0.5, 0.9, 0.999])
def test_pair_known_answer(r):
    s = two_particles(r)
    o = oracle.OracleSystem(s)
    e, f, n = o.nonbonded(s.positions[0])
    ea, dea = analytic_pair(r, s.charge, s.sigma, s.epsilon, 1.0, 78.5)
    assert n == 1
    assert e == pytest.approx(ea, rel=1e-12, abs=1e-12)
    # force on particle 1 (at larger x) is -dE/dr along +x
    assert f[1, 0] == pytest.approx(-dea, rel=1e-10)
    assert f[0, 0] == pytest.approx(dea, rel=1e-10)


def test_rf_energy_vanishes_at_cutoff():
    s = two_particles(0.999999999, sig=(0.0, 0.0), eps=(0.0, 0.0))
    o = oracle.OracleSystem(s)
    e, _, _ = o.nonbonded(s.positions[0])
    assert abs(e) < 1e-6


def test_beyond_cutoff_and_minimum_image():
    s = two_particles(1.0001)
    assert oracle.OracleSystem(s).nonbonded(s.positions[0])[2] == 0
    # across the periodic boundary: particles at 0.1 and box-0.2 are 0.3 apart
    s = two_particles(0.3)
    s.positions[0] = [[0.1, 1, 1], [4.8, 1, 1]]
    e, f, n = oracle.OracleSystem(s).nonbonded(s.positions[0])
    ea, dea = analytic_pair(0.3, s.charge, s.sigma, s.epsilon, 1.0, 78.5)
    assert n == 1 and e == pytest.approx(ea, rel=1e-12)


def dense_reference(s, y):
    """O(N^2) numpy FP64 energy/forces (minimum image, exclusions)."""
    n = s.n
    d = y[None, :, :] - y[:, None, :]
    d -= s.box * np.round(d / s.box)
    r2 = (d * d).sum(-1)
    iu = np.triu_indices(n, 1)
    mask = np.zeros((n, n), bool)
    mask[iu] = True
    ex = np.asarray(s.exclusions).reshape(-1, 2)
    mask[ex[:, 0], ex[:, 1]] = False
    mask[ex[:, 1], ex[:, 0]] = False
    mask &= r2 < s.cutoff ** 2
    i, j = np.nonzero(mask)
    r = np.sqrt(r2[i, j])
    sg = 0.5 * (s.sigma[i] + s.sigma[j])
    ep = np.sqrt(s.epsilon[i] * s.epsilon[j])
    qq = K * s.charge[i] * s.charge[j]
    rc, e_ = s.cutoff, s.eps_rf
    krf = (e_ - 1) / ((2 * e_ + 1) * rc ** 3)
    crf = 3 * e_ / ((2 * e_ + 1) * rc)
    sr6 = (sg / r) ** 6
    E = (4 * ep * (sr6 * sr6 - sr6) + qq * (1 / r + krf * r * r - crf)).sum()
    fs = (4 * ep * (12 * sr6 * sr6 - 6 * sr6) + qq * (1 / r - 2 * krf * r * r)) / (r * r)
    F = np.zeros((n, 3))
    np.add.at(F, j, fs[:, None] * d[i, j])
    np.add.at(F, i, -fs[:, None] * d[i, j])
    return E, F, len(i)


@pytest.mark.parametrize("variant", ["a", "b"])
def test_config0_dense_crosscheck(variant):
    s = S.config0(variant=variant)
    o = oracle.OracleSystem(s)
    x = s.positions[0]
    r = o.states(x)
    E0, F0, n0 = dense_reference(s, x)
    E1, F1, n1 = dense_reference(s, x + s.displacement)
    assert r["P0"] == n0 and r["P1"] == n1
    assert r["U0"] == pytest.approx(E0, rel=1e-11)
    assert r["U1"] == pytest.approx(E1, rel=1e-11)
    assert np.abs(r["F0"] - F0).max() < 1e-8 * max(1, np.abs(F0).max())
    assert np.abs(r["F1"] - F1).max() < 1e-8 * max(1, np.abs(F1).max())
    # u accumulated directly over changed pairs equals U1-U0
    assert r["u_direct"] == pytest.approx(r["U1"] - r["U0"], rel=1e-9, abs=1e-8)


def test_invariances_config0():
    s = S.config0(variant="b")
    o = oracle.OracleSystem(s)
    x = s.positions[0]
    r = o.states(x)
    # Newton's third law
    assert np.abs(r["F0"].sum(0)).max() < 1e-7
    # translation invariance (periodic)
    r2 = o.states(x + np.array([0.37, -1.2, 2.9]))
    assert r2["U0"] == pytest.approx(r["U0"], rel=1e-10)
    assert r2["u_direct"] == pytest.approx(r["u_direct"], rel=1e-8, abs=1e-8)
    # zero displacement -> u == 0 and equal states
    s0 = S.config0(variant="b")
    s0.displacement[:] = 0
    r0 = oracle.OracleSystem(s0).states(x)
    assert r0["u_direct"] == 0.0 and r0["U1"] == r0["U0"]


def test_f32_rule_matches_fp64_rule_config1():
    s = S.config1()
    o = oracle.OracleSystem(s)
    x = s.positions[0]
    M = np.array([14, 14, 14], np.int32)
    a = o.f32rule(x, M)
    b = o.states(x)
    assert abs(a["P0"] - b["P0"]) <= 5
    assert abs(a["P1delta"] - b["P1delta"]) <= 2
    assert a["U0"] == pytest.approx(b["U0"], abs=0.05)
    assert abs(a["u"] - b["u_direct"]) < 1e-2
    assert a["image_mode"] == 0


# ----------------------------------------------------------------- combine
def ref_softcore(u, method, umax, a, ub):
    """Independent restatement (python) of LangevinIntegratorSDM::SoftCoreF."""
    if u <= ub or method == 0:
        return u, 1.0
    if method == 1:
        t = math.tanh((u - ub) / umax)
        return umax * t + ub, 1 - t * t
    gu = (u - ub) / (a * (umax - ub))
    z = 1 + 2 * gu * (gu + 1)
    za = z ** a
    return (umax - ub) * (za - 1) / (za + 1) + ub, 4 * (2 * gu + 1) / z * za / (1 + za) ** 2


@pytest.mark.parametrize("method", [0, 1, 2])
@pytest.mark.parametrize("u", [-50.0, 0.0, 99.0, 100.0, 101.0, 150.0, 1e3, 1e6, 6e7])
def test_softcore_matches_python(method, u):
    v, fp = oracle.softcore(u, method, 200.0, 1 / 16, 100.0)
    rv, rfp = ref_softcore(u, method, 200.0, 1 / 16, 100.0)
    assert v == pytest.approx(rv, rel=1e-14, abs=1e-12)
    assert fp == pytest.approx(rfp, rel=1e-12, abs=1e-300)


@pytest.mark.parametrize("method", [1, 2])
def test_softcore_derivative_fd(method):
    for u in [100.5, 120.0, 180.0, 300.0, 2000.0]:
        h = 1e-5
        vp, _ = oracle.softcore(u + h, method, 200.0, 1 / 16, 100.0)
        vm, _ = oracle.softcore(u - h, method, 200.0, 1 / 16, 100.0)
        _, fp = oracle.softcore(u, method, 200.0, 1 / 16, 100.0)
        assert fp == pytest.approx((vp - vm) / (2 * h), rel=1e-6, abs=1e-8)
    # continuity at ubcore and the cap umax for the rational form
    v, _ = oracle.softcore(100.0 + 1e-12, method, 200.0, 1 / 16, 100.0)
    assert v == pytest.approx(100.0, abs=1e-9)
    v, _ = oracle.softcore(1e12, 2, 200.0, 1 / 16, 100.0)
    assert v < 200.0


def test_unknown_softcore_is_nan():
    v, fp = oracle.softcore(150.0, 7, 200.0, 1 / 16, 100.0)
    assert math.isnan(v) and math.isnan(fp)


def _combine_py(p, U0, U1):
    """Independent python restatement of ReferenceSDMKernels.cpp:202-302."""
    be, fp = ref_softcore(U1 - U0, int(p.softcore_method), p.umax, p.acore, p.ubcore)
    lam = p.lambdac
    if p.bias_method == 1:
        W = 0.5 * p.gamma * be * be + p.wb * be + p.w0
        dW = p.gamma * be + p.wb
    elif p.bias_method == 2:
        ee = 1 + math.exp(-p.alpha * (be - p.u0))
        W = ((p.lambda2 - p.lambda1) / p.alpha) * math.log(ee) if p.alpha > 0 else 0.0
        W += p.lambda2 * be + p.w0
        dW = (p.lambda2 - p.lambda1) / ee + p.lambda1
    else:
        W = lam * be
        dW = lam
    return be, fp, W, dW, dW * fp, U0 + W


@pytest.mark.parametrize("bias", [0, 1, 2])
@pytest.mark.parametrize("soft", [0, 1, 2])
@pytest.mark.parametrize("alpha", [0.0, 0.1])
def test_combine_matches_python(bias, soft, alpha):
    p = S.SDMParams(bias_method=bias, softcore_method=soft, lambdac=0.37, lambda1=0.2,
                    lambda2=0.45, alpha=alpha, u0=110, w0=3.0, gamma=0.01, wb=0.6, umax=200,
                    acore=1 / 16, ubcore=100)
    for U0, U1 in [(-1000.0, -900.0), (5.0, 200.0), (0.0, 1e5)]:
        out = oracle.combine(p.as_array(), U0, U1)
        ref = _combine_py(p, U0, U1)
        for k, v in zip((1, 2, 3, 4, 5, 6), ref):
            assert out[k] == pytest.approx(v, rel=1e-12, abs=1e-12)


def test_alpha_zero_logistic_weight():
    # with alpha=0 the ILogistic branch skips the log term and W'=(l1+l2)/2
    p = S.SDMParams(bias_method=2, softcore_method=0, lambda1=0.2, lambda2=0.6, alpha=0.0, u0=0)
    out = oracle.combine(p.as_array(), 0.0, 50.0)
    assert out[4] == pytest.approx(0.4)
    assert out[3] == pytest.approx(0.6 * 50.0)


def test_noneq_dwdlambda_fd():
    p = S.SDMParams(bias_method=2, softcore_method=2, alpha=0.1, noneq=1, lambdac=0.3,
                    m_lambda1=0.8, m_lambda2=1.0, m_u0=20.0, m_w0=2.0, b_lambda1=0.05,
                    b_lambda2=0.0, b_u0=100.0, b_w0=-1.0, umax=200, acore=1 / 16, ubcore=100)
    U0, U1 = -500.0, -380.0
    out = oracle.combine(p.as_array(), U0, U1)
    h = 1e-6
    pp = S.SDMParams(**{**p.__dict__, "lambdac": 0.3 + h})
    pm = S.SDMParams(**{**p.__dict__, "lambdac": 0.3 - h})
    Wp = oracle.combine(pp.as_array(), U0, U1)[3]
    Wm = oracle.combine(pm.as_array(), U0, U1)[3]
    assert out[7] == pytest.approx((Wp - Wm) / (2 * h), rel=1e-6)
    # the parameters follow p = m*lambda + b
    assert out[8] == pytest.approx(0.8 * 0.3 + 0.05)
    assert out[10] == pytest.approx(20 * 0.3 + 100)


def _noneq_dwdl_reference_scoping(p, U0, U1, lambda_before):
    """ReferenceSDMKernels.cpp:202-302 for NonEquilibrium = 1, written with the
    reference's variable scopes: the function-scope lambda1/lambda2/alpha/u0
    (:214-217) start from the lambda before the step, 1 and 0; the scheduled
    values of the non-equilibrium block (:236-239) are block-local and go only
    to the integrator's setters; the integrated-logistic branch (:255-260)
    reloads them from the integrator.  dW/dlambda (:289-297) reads the
    function-scope names."""
    lambda1 = lambda2 = lambda_before
    alpha, u0 = 1.0, 0.0
    lambdac = p.lambdac                      # t / Ntmax, assigned to the outer name (:233)
    set_l1 = p.m_lambda1 * lambdac + p.b_lambda1
    set_l2 = p.m_lambda2 * lambdac + p.b_lambda2
    set_u0 = p.m_u0 * lambdac + p.b_u0
    if p.bias_method == 2:
        lambda1, lambda2, alpha, u0 = set_l1, set_l2, p.alpha, set_u0
    be, _ = ref_softcore(U1 - U0, int(p.softcore_method), p.umax, p.acore, p.ubcore)
    ee = 1.0 + math.exp(-alpha * (be - u0))
    dwdl1 = -math.log(ee) / alpha
    dwdl2 = be + math.log(ee) / alpha
    dwdu0 = (lambda2 - lambda1) * math.exp(-alpha * (be - u0)) / ee
    return dwdl1 * p.m_lambda1 + dwdl2 * p.m_lambda2 + dwdu0 * p.m_u0 + 1.0 * p.m_w0


@pytest.mark.parametrize("bias", [0, 1, 2])
@pytest.mark.parametrize("soft", [0, 2])
def test_noneq_dwdlambda_reference_scoping(bias, soft):
    p = S.SDMParams(bias_method=bias, softcore_method=soft, alpha=0.1, noneq=1, lambdac=0.3,
                    m_lambda1=0.8, m_lambda2=1.0, m_u0=20.0, m_w0=2.0, b_lambda1=0.05,
                    b_lambda2=0.0, b_u0=100.0, b_w0=-1.0, gamma=0.01, wb=0.4, umax=200,
                    acore=1 / 16, ubcore=100)
    for U0, U1 in [(-500.0, -380.0), (10.0, 5.0), (0.0, 30.0)]:
        out = oracle.combine(p.as_array(), U0, U1)
        # the lambda before the step only enters as lambda2 - lambda1 = 0
        for lam_before in (0.0, 0.29, 0.7):
            ref = _noneq_dwdl_reference_scoping(p, U0, U1, lam_before)
            assert out[7] == pytest.approx(ref, rel=1e-13, abs=1e-13)
        # the integrator receives the scheduled parameters for every method
        assert out[8] == pytest.approx(0.8 * 0.3 + 0.05)
        assert out[10] == pytest.approx(20 * 0.3 + 100)
    if bias != 2:
        # differs from the derivative of W along the schedule: alpha = 1 and u0 = 0
        be, _ = ref_softcore(120.0, soft, 200.0, 1 / 16, 100.0)
        l1e = math.log(1.0 + math.exp(-be))
        assert oracle.combine(p.as_array(), -500.0, -380.0)[7] == pytest.approx(
            -l1e * 0.8 + (be + l1e) * 1.0 + 2.0, rel=1e-13)


def test_mixed_force_eval_state():
    s = S.config0(variant="b")
    o = oracle.OracleSystem(s)
    res, F = oracle.eval_state(o, s.positions[0], s.params[0].as_array())
    st = o.states(s.positions[0])
    sw = res[5]
    assert np.allclose(F, sw * st["F1"] + (1 - sw) * st["F0"], rtol=1e-12, atol=1e-9)
    assert res[12] == pytest.approx(st["U0"]) and res[13] == pytest.approx(st["U1"])


def test_cluster_build_properties():
    s = S.config1()
    o = oracle.OracleSystem(s)
    M = np.array([14, 14, 14], np.int32)
    c = o.clusters(s.positions[0], M)
    perm = c["perm"]
    valid = perm[perm >= 0]
    assert np.array_equal(np.sort(valid), np.arange(s.n))
    # every cluster's first slot is valid; padding only at cluster ends
    p8 = perm.reshape(-1, 8)
    assert (p8[:, 0] >= 0).all()
    for row in p8:
        v = row >= 0
        assert not (np.diff(v.astype(int)) > 0).any()


def test_langevin_coefficients_and_update():
    """Restated stochastic-dynamics step: closed forms at T = 0 and its limits."""
    dt, fr = 0.004, 1.0
    vs, fs, ns = oracle.langevin_coefficients(dt, fr, 0.0)
    assert vs == pytest.approx(np.exp(-dt * fr), rel=1e-15)
    assert fs == pytest.approx((1 - np.exp(-dt * fr)) / fr, rel=1e-15)
    assert ns == 0.0
    # noise^2 = kT (1 - vscale^2): the velocity variance of one step from rest
    _, _, n300 = oracle.langevin_coefficients(dt, fr, 300.0)
    assert n300 ** 2 == pytest.approx(oracle.MOLAR_GAS_CONSTANT * 300.0 * (1 - np.exp(-2 * dt * fr)), rel=1e-12)
    rng = np.random.default_rng(7)
    x = rng.uniform(0, 3, (5, 3)); v = rng.normal(size=(5, 3)); F = rng.normal(size=(5, 3))
    im = np.array([1 / 12.0, 1 / 16.0, 0.0, 1.0, 0.5])
    xo, vo = oracle.langevin_update(x, v, im, F, dt, fr, 0.0)
    v1 = vs * v + fs * im[:, None] * F
    assert np.allclose(vo[im != 0], v1[im != 0], rtol=1e-12)
    assert np.allclose(xo[im != 0], (x + dt * v1)[im != 0], rtol=1e-15)
    assert np.array_equal(xo[2], x[2]) and np.array_equal(vo[2], v[2])   # m^-1 = 0: fixed


def test_ewald_madelung_constant_of_rock_salt():
    """Golden value: the Madelung constant of NaCl, M = 1.747565 (per ion pair
    E = -M K q^2 / r0), from a 2x2x2 conventional-cell lattice (64 ions)."""
    a = 0.56                                  # nm, conventional cell; r0 = a/2
    pts, qs = [], []
    for i in range(4):
        for j in range(4):
            for k in range(4):
                pts.append((i * a / 2, j * a / 2, k * a / 2))
                qs.append(1.0 if (i + j + k) % 2 == 0 else -1.0)
    x = np.array(pts) + 0.013
    q = np.array(qs)
    box = np.array([2 * a] * 3)
    for beta in (10.0, 12.0):                 # erfc(beta rc) < 1e-13 at rc = 0.55 nm
        e = oracle.ewald(x, q, box, beta, cutoff=0.55, forces=True)
        M = -e["total"] * (a / 2) / (oracle.K_COULOMB * len(q) / 2)
        assert M == pytest.approx(1.747565, abs=2e-6)
        assert np.abs(e["F"]).max() < 1e-6 * oracle.K_COULOMB    # lattice sites: no net force


def test_ewald_forces_are_minus_gradient():
    rng = np.random.default_rng(4)
    n = 24
    box = np.array([1.9, 2.0, 2.1])
    x = rng.uniform(0, 1, (n, 3)) * box
    q = rng.choice([-0.5, 0.5], n)
    q[0] += 0.1                                # net charge: background term
    excl = np.array([[0, 1], [2, 3], [4, 7]])
    beta, rc = 3.0, 0.9
    e = oracle.ewald(x, q, box, beta, rc, excl)
    h = 1e-6
    for i, k in ((0, 0), (3, 1), (7, 2), (11, 0)):
        xp, xm = x.copy(), x.copy()
        xp[i, k] += h
        xm[i, k] -= h
        # small moves: no pair crosses the cutoff
        g = (oracle.ewald(xp, q, box, beta, rc, excl, forces=False)["total"]
             - oracle.ewald(xm, q, box, beta, rc, excl, forces=False)["total"]) / (2 * h)
        assert e["F"][i, k] == pytest.approx(-g, rel=1e-5, abs=1e-4)
    # independent of beta when converged (the split is exact)
    e2 = oracle.ewald(x, q, box, 3.6, rc, excl)
    assert e2["total"] == pytest.approx(e["total"], rel=2e-4, abs=2e-3)


def test_spme_matches_ewald_reciprocal():
    """The restated smooth PME converges to the exact reciprocal Ewald sum."""
    rng = np.random.default_rng(8)
    n = 60
    box = np.array([2.0, 2.2, 2.4])
    x = rng.uniform(0, 1, (n, 3)) * box
    q = rng.uniform(-0.6, 0.6, n)
    q -= q.mean()
    beta = 3.2
    ew = oracle.ewald(x, q, box, beta, 0.9)
    # exact reciprocal forces: total minus direct minus nothing else (no exclusions)
    ew_d = oracle.ewald(x, q, box, beta, 0.9, kmax=[0, 0, 0])
    Frec = ew["F"] - ew_d["F"]
    for K, tol in ((24, 2e-4), (48, 1e-6)):
        E, F, _ = oracle.spme(x, q, box, beta, [K, K, K], order=5)
        assert E == pytest.approx(ew["reciprocal"], rel=tol)
        assert np.sqrt(((F - Frec) ** 2).sum() / (Frec ** 2).sum()) < 50 * tol
    assert list(oracle.pme_grid_size(3.2, [6.2, 6.2, 6.2], 5e-4)) == [63, 63, 63]   # ceil(60.5) -> 3^2 7
