"""CPU-side checks of the C ABI: the library builds, loads and exports every
symbol the header declares; creation without a GPU fails cleanly."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "sdm_capi.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sdm_[a-z_]+)\s*\(", txt)))


def test_header_declares_expected(built_lib):
    from openmm_sdm_plugin_gb300 import capi
    syms = declared_symbols()
    assert set(capi.EXPORTED) == set(syms)


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_create_rejects_bad_arguments_without_touching_gpu(built_lib):
    from openmm_sdm_plugin_gb300 import capi
    L = capi.load_library()
    h = C.c_void_p()
    assert L.sdm_create(None, 0, 0, C.byref(h)) == capi.SDM_ERR_INVALID_ARGUMENT
    assert b"system" in L.sdm_last_error(None)
    assert L.sdm_destroy(None) == capi.SDM_OK


def test_no_gpu_reports_no_device(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from openmm_sdm_plugin_gb300 import capi, systems
    with pytest.raises(capi.SdmError) as e:
        capi.Handle([systems.config0()])
    assert e.value.status in (capi.SDM_ERR_NO_DEVICE, capi.SDM_ERR_CUDA)


def test_params_layout_matches_header():
    from openmm_sdm_plugin_gb300 import systems
    txt = open(os.path.join(ROOT, "include", "sdm_capi.h")).read()
    names = re.findall(r"SDM_P_([A-Z0-9_]+) = (\d+)", txt)
    assert len(names) == 22
    p = systems.SDMParams(bias_method=2, softcore_method=1, lambdac=0.1, lambda1=0.2, lambda2=0.3,
                          alpha=0.4, u0=0.5, w0=0.6, gamma=0.7, wb=0.8, umax=0.9, acore=1.0,
                          ubcore=1.1, noneq=1, m_lambda1=1.2, m_lambda2=1.3, m_u0=1.4, m_w0=1.5,
                          b_lambda1=1.6, b_lambda2=1.7, b_u0=1.8, b_w0=1.9)
    a = p.as_array()
    expect = dict(BIAS_METHOD=2, SOFTCORE_METHOD=1, LAMBDA=0.1, LAMBDA1=0.2, LAMBDA2=0.3,
                  ALPHA=0.4, U0=0.5, W0=0.6, GAMMA=0.7, WB=0.8, UMAX=0.9, ACORE=1.0, UBCORE=1.1,
                  NONEQ=1, M_LAMBDA1=1.2, M_LAMBDA2=1.3, M_U0=1.4, M_W0=1.5, B_LAMBDA1=1.6,
                  B_LAMBDA2=1.7, B_U0=1.8, B_W0=1.9)
    for nm, idx in names:
        assert a[int(idx)] == pytest.approx(expect[nm]), nm


def test_force_api_mirrors_reference_setters():
    """Every SDM setter/getter of the reference SWIG interface exists on SDMForce."""
    from openmm_sdm_plugin_gb300 import SDMForce
    names = ["setLambda", "getLambda", "getBindE", "setBindE", "getPotEnergy", "setPotEnergy",
             "getUmax", "setUmax", "getAcore", "setAcore", "getUbcore", "setUbcore",
             "setBiasMethod", "getBiasMethod", "setSoftCoreMethod", "getSoftCoreMethod",
             "setGamma", "getGamma", "setWBcoeff", "getWBcoeff", "setW0coeff", "getW0coeff",
             "setLambda1", "getLambda1", "setLambda2", "getLambda2", "setAlpha", "getAlpha",
             "setU0", "getU0", "setNoneqtmax", "getNoneqtmax", "getNonEquilibrium",
             "setNoneqWorkvalue", "getNoneqWorkvalue", "setlambda1Slope", "getlambda1Slope",
             "setlambda2Slope", "getlambda2Slope", "setu0Slope", "getu0Slope", "setw0Slope",
             "getw0Slope", "setlambda1intercept", "getlambda1intercept", "setlambda2intercept",
             "getlambda2intercept", "setu0intercept", "getu0intercept", "setw0intercept",
             "getw0intercept", "setDisplacement", "getDisplacement"]
    f = SDMForce(3)
    for n in names:
        assert callable(getattr(f, n)), n
    # reference defaults (LangevinIntegratorSDM.cpp:48-85)
    assert f.getUmax() == 200.0 and f.getAcore() == 0.25 and f.getUbcore() == 0.0
    assert f.getBiasMethod() == 0 and f.getSoftCoreMethod() == 0
    assert f.getLambda1() == 1.0 and f.getAlpha() == 1.0 and f.getWBcoeff() == 1.0
    f.setDisplacement(1, 1.0, 2.0, 3.0)
    assert f.getDisplacement(1) == (1.0, 2.0, 3.0)
    assert f.getDisplacement(0) == (0.0, 0.0, 0.0)


def _bad(s, **kw):
    import dataclasses
    return dataclasses.replace(s, **kw)


def _with(a, i, v):
    a = np.array(a, dtype=float)
    a[i] = v
    return a


def test_descriptor_errors_are_reported_before_any_device_query(built_lib):
    """Every system descriptor is validated on the host before the library
    looks for a device, so these errors read the same with or without a GPU."""
    from openmm_sdm_plugin_gb300 import capi, systems
    s = systems.config0(variant="b")
    ex = np.asarray(s.exclusions).copy()
    ex[0, 1] = s.n
    cases = [
        (_bad(s, sigma=_with(s.sigma, 0, np.inf)), "sigma/epsilon must be finite"),
        (_bad(s, epsilon=_with(s.epsilon, 3, -1.0)), "sigma/epsilon must be finite"),
        (_bad(s, charge=_with(s.charge, 5, np.nan)), "charges finite"),
        (_bad(s, cutoff=0.6 * float(s.box.min())), "below half the box edge"),
        (_bad(s, box=np.array([s.box[0], 0.0, s.box[2]])), "box edges must be finite"),
        (_bad(s, eps_rf=0.0), "reaction_field_dielectric"),
        (_bad(s, exclusions=ex), "exclusion index out of range"),
        (_bad(s, nonbonded_method="pme", ewald_tolerance=0.7), "ewald_tolerance"),
        (_bad(s, displacement=_with(s.displacement, (7, 1), np.nan)), "non-finite displacement"),
        (_bad(s, displacement=_with(s.displacement, (2, 0), -np.inf)), "non-finite displacement"),
    ]
    for bad, msg in cases:
        with pytest.raises(capi.SdmError) as e:
            capi.Handle([s, bad])
        assert e.value.status == capi.SDM_ERR_INVALID_ARGUMENT, (msg, e.value)
        assert "system 1" in str(e.value) and msg in str(e.value), str(e.value)


def test_tune_key_names_the_workload(built_lib):
    """The autotuner's cache key: mean particles per replica, density,
    cutoff, replicas, systems, electrostatics, SM count; the coordinates do
    not enter it.  Computed on the host (no device)."""
    import dataclasses
    from openmm_sdm_plugin_gb300 import capi, systems
    s = systems.config2(nrep=3)
    k = capi.tune_key([s], 152)
    rho = s.n / float(np.prod(s.box))
    assert k == (f"sdm-tune-v1 n={s.n} rho={rho:.1f} rc={s.cutoff:.3f} replicas=3 systems=1 "
                 f"method=rf sms=152"), k
    moved = dataclasses.replace(s, positions=s.positions + 0.01)
    assert capi.tune_key([moved], 152) == k
    assert capi.tune_key([s], 148) != k
    assert capi.tune_key([systems.config2(nrep=2)], 152) != k
    assert capi.tune_key([dataclasses.replace(s, nonbonded_method="pme")], 152) != k
    assert capi.tune_key([dataclasses.replace(s, cutoff=1.1)], 152) != k
    two = capi.tune_key([s, systems.config0(variant="b")], 152)
    assert "systems=2" in two and "replicas=4" in two
