"""The OpenMM force plugin (openmm_sdm_plugin_gb300/shim, SDMPluginGB300::
SDMForce) compiled against the OpenMM API subset of tests/openmm_api and
linked with libsdm_gb300.so.

CPU: what the plugin reads from a NonbondedForce (exclusions from every
exception, interacting exceptions with their parameters, method, cutoff,
reaction-field dielectric, Ewald tolerance; the reference integrator's
parameter defaults), the models it refuses, a clean OpenMMException when no
GPU is present, and the kernel factory that registerKernelFactories puts on
the CUDA platform.  GPU: energy, forces and results through a Context equal
the C ABI's evaluation of the same system bit for bit, before and after
updateParametersInContext, on the host path and through the CalcSDMForce
kernel on a stand-in of OpenMM's CUDA platform (tests/openmm_api/CudaSubset.cpp)."""
import dataclasses
import os
import subprocess

import numpy as np
import pytest

from openmm_sdm_plugin_gb300 import capi, systems as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
API = os.path.join(ROOT, "tests", "openmm_api")
SHIM = os.path.join(ROOT, "openmm_sdm_plugin_gb300", "shim")
METHODS = {"rf": 2, "pme": 4}   # OpenMM NonbondedForce::CutoffPeriodic, ::PME
P_LAMBDA1 = 3                   # SDM_P_LAMBDA1


@pytest.fixture(scope="module")
def driver(built_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("shim") / "shim_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
           "-I", API, "-I", os.path.join(ROOT, "include"), "-I", SHIM,
           os.path.join(SHIM, "SDMForceGB300.cpp"), os.path.join(API, "ApiSubset.cpp"),
           os.path.join(API, "shim_driver.cpp"), "-o", exe, built_lib,
           "-Wl,-rpath," + os.path.dirname(built_lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def openmm_exceptions(s):
    """The exception list of the NonbondedForce the reference builds for s:
    every excluded pair once, with its own parameters where it interacts
    (zero charge product and well depth otherwise)."""
    own = {}
    if s.exceptions is not None:
        for (i, j), prm in zip(np.asarray(s.exceptions).reshape(-1, 2), np.asarray(s.exception_params).reshape(-1, 3)):
            own[(min(i, j), max(i, j))] = prm
    ex = []
    for i, j in np.asarray(s.exclusions).reshape(-1, 2):
        qq, sg, ep = own.get((min(i, j), max(i, j)), (0.0, 1.0, 0.0))
        ex.append((i, j, qq, sg, ep))
    return np.array(ex, np.float64).reshape(-1, 5)


def write_input(path, s, p, x, method=None, dispersion=False):
    ex = openmm_exceptions(s)
    m = METHODS[s.nonbonded_method] if method is None else method
    with open(path, "wb") as f:
        np.array([s.n, ex.shape[0], m, int(dispersion)], np.int32).tofile(f)
        np.array([*s.box, s.cutoff, s.eps_rf, s.ewald_tolerance], np.float64).tofile(f)
        for a in (p.as_array(), s.charge, s.sigma, s.epsilon, s.displacement, x, ex):
            np.ascontiguousarray(a, np.float64).reshape(-1).tofile(f)


def run(driver, mode, tmp_path, s, p, x, **kw):
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, s, p, x, **kw)
    r = subprocess.run([driver, mode, inp, out], capture_output=True, text=True, timeout=300)
    return r, out


def _dms_system():
    from openmm_sdm_plugin_gb300 import dms
    p = S.SDMParams(bias_method=S.ILOGISTIC, softcore_method=S.RATIONAL_SOFTCORE, lambda1=0.3, lambda2=0.6,
                    alpha=0.05, u0=10.0, w0=1.0, umax=50.0, acore=0.25, ubcore=10.0)
    return dms.load_compact(os.path.join(ROOT, "tests", "golden", "temoa_g1_g4.npz"),
                            displacement={2: (2.2, 2.2, 2.2), 3: (-2.2, -2.2, -2.2)}, params=[p])


def test_describe_copies_the_nonbonded_force(driver, tmp_path):
    s = _dms_system()
    p = s.params[0]
    r, out = run(driver, "describe", tmp_path, s, p, s.positions[0])
    assert r.returncode == 0, r.stderr
    b = open(out, "rb").read()
    ne, nx, method, group = np.frombuffer(b[:16], np.int32)
    o = 16
    excl = np.frombuffer(b[o:o + 8 * ne], np.int32).reshape(-1, 2); o += 8 * ne
    pairs = np.frombuffer(b[o:o + 8 * nx], np.int32).reshape(-1, 2); o += 8 * nx
    rest = np.frombuffer(b[o:], np.float64)
    prm, rest = rest[:3 * nx].reshape(-1, 3), rest[3 * nx:]
    displ, rest = rest[:3 * s.n].reshape(-1, 3), rest[3 * s.n:]
    cutoff, eps_rf, tol, boxsum = rest[:4]
    params = rest[4:]
    assert group == 2 and method == capi.NB_REACTION_FIELD
    assert np.array_equal(excl, s.exclusions)
    ex = openmm_exceptions(s)
    live = (ex[:, 2] != 0) | (ex[:, 4] != 0)
    assert nx == live.sum() == len(s.exceptions)
    assert np.array_equal(pairs, ex[live, :2].astype(np.int32))
    assert np.array_equal(prm, ex[live, 2:])
    assert np.array_equal(displ, s.displacement)
    assert (cutoff, eps_rf, tol, boxsum) == (s.cutoff, s.eps_rf, s.ewald_tolerance, s.box.sum())
    assert np.array_equal(params, p.as_array())


def test_defaults_are_the_reference_integrators(driver, tmp_path):
    """Parameters left unset keep LangevinIntegratorSDM's constructor defaults
    (LangevinIntegratorSDM.cpp:56-75): the driver sets every one, so a system
    written with the defaults must read back unchanged."""
    s = S.config0(variant="b")
    p = S.SDMParams(bias_method=S.LINEAR, softcore_method=S.NO_SOFTCORE, lambdac=1.0, lambda1=1.0, lambda2=1.0,
                    alpha=1.0, u0=0.0, w0=0.0, gamma=0.0, wb=1.0, umax=200.0, acore=0.25, ubcore=0.0)
    r, out = run(driver, "describe", tmp_path, s, p, s.positions[0])
    assert r.returncode == 0, r.stderr
    params = np.frombuffer(open(out, "rb").read(), np.float64)[-capi.NPARAMS:]
    assert np.array_equal(params, p.as_array())


@pytest.mark.parametrize("kw,msg", [(dict(method=0), "CutoffPeriodic"), (dict(method=3), "CutoffPeriodic"),
                                    (dict(dispersion=True), "DispersionCorrection")])
def test_refuses_other_models(driver, tmp_path, kw, msg):
    s = S.config0(variant="b")
    r, _ = run(driver, "describe", tmp_path, s, s.params[0], s.positions[0], **kw)
    assert r.returncode == 3 and msg in r.stderr, r.stderr


def test_no_gpu_raises_openmm_exception(driver, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    s = S.config0(variant="b")
    r, _ = run(driver, "evaluate", tmp_path, s, s.params[0], s.positions[0])
    assert r.returncode == 3 and "sdm_create failed" in r.stderr, r.stderr


def _reference_order(s):
    """s with its exceptions in the plugin's order (exclusion order), so that
    the C ABI sums the exception terms in the same order."""
    ex = openmm_exceptions(s)
    live = (ex[:, 2] != 0) | (ex[:, 4] != 0)
    if not live.any():
        return s
    return dataclasses.replace(s, exceptions=ex[live, :2].astype(np.int32), exception_params=ex[live, 2:].copy())


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["config0", "temoa", "config0_pme"])
def test_context_evaluation_equals_the_c_abi(driver, tmp_path, which):
    if which == "temoa":
        s = _dms_system()
    else:
        s = S.config0(variant="b").replica(0)
        if which == "config0_pme":
            s = dataclasses.replace(s, nonbonded_method="pme", ewald_tolerance=5e-4)
    p = s.params[0]
    x = s.positions[0]
    r, out = run(driver, "evaluate", tmp_path, s, p, x)
    assert r.returncode == 0, r.stderr
    got = np.frombuffer(open(out, "rb").read(), np.float64).reshape(2, -1)
    ref = _reference_order(s)
    h = capi.Handle([ref])
    for k, lam1_shift in enumerate((0.0, 0.1)):
        a = p.as_array().copy()
        a[P_LAMBDA1] += lam1_shift
        h.set_params(0, a)
        res, F = h.evaluate(x)
        e, rr, ff = got[k, 0], got[k, 1:1 + capi.NRESULTS], got[k, 1 + capi.NRESULTS:].reshape(-1, 3)
        assert e == res[0, capi.R_EPOT]
        assert np.array_equal(rr, res[0])
        assert np.array_equal(ff, F.reshape(-1, 3))
    assert got[1, 1 + capi.R_L1] != got[0, 1 + capi.R_L1]
    h.close()


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "include", "cuda.h")):
            return c
    pytest.skip("CUDA toolkit headers not found")


@pytest.fixture(scope="module")
def cuda_driver(built_lib, tmp_path_factory):
    """The driver with the CUDA-platform stand-in (tests/openmm_api/CudaSubset.cpp)
    and the plugin's platform kernel (shim/SDMCudaKernels.cpp)."""
    cuda = _cuda_home()
    exe = str(tmp_path_factory.mktemp("shim_cuda") / "shim_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
           "-DSDM_TEST_CUDA_PLATFORM", "-I", API, "-I", os.path.join(ROOT, "include"), "-I", SHIM,
           "-I", os.path.join(cuda, "include"),
           os.path.join(SHIM, "SDMForceGB300.cpp"), os.path.join(SHIM, "SDMCudaKernels.cpp"),
           os.path.join(API, "ApiSubset.cpp"), os.path.join(API, "CudaSubset.cpp"),
           os.path.join(API, "shim_driver.cpp"), "-o", exe, built_lib,
           "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(built_lib) + ":" + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_kernel_factory_registers_on_the_cuda_platform(cuda_driver, tmp_path):
    """registerKernelFactories (the plugin entry OpenMM calls on loading)
    registers CalcSDMForce with the CUDA platform only; the kernel is created
    by name through the platform, an unknown name is refused.  No GPU needed:
    the kernel touches the device only when it first executes."""
    out = str(tmp_path / "factory.txt")
    r = subprocess.run([cuda_driver, "factory", "-", out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = open(out).read().splitlines()
    assert "platform Reference supports 0" in lines
    assert "platform CUDA supports 1" in lines
    assert "kernel CalcSDMForce" in lines
    assert any(ln.startswith("unknown refused:") for ln in lines)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "double"])
@pytest.mark.parametrize("which", ["config0", "temoa"])
def test_cuda_platform_kernel_equals_the_c_abi(cuda_driver, tmp_path, precision, which):
    """SDMForce on the CUDA platform runs the CalcSDMForce kernel: positions
    gathered from the platform's shuffled posq (with the mixed-precision
    correction), forces added into its 2^32 fixed-point buffer.  The energy,
    the results and the forces equal the C ABI's on the same coordinates, bit
    for bit (forces at the buffer's 2^-32 resolution); also for forces without
    the energy (results read afterwards) and after updateParametersInContext."""
    s = _dms_system() if which == "temoa" else S.config0(variant="b").replica(0)
    p = s.params[0]
    x = np.ascontiguousarray(s.positions[0], np.float64)
    r, out = run(cuda_driver, "cuda-" + precision, tmp_path, s, p, x)
    assert r.returncode == 0, r.stderr
    raw = np.frombuffer(open(out, "rb").read(), np.float64)
    n3 = 3 * s.n
    f_async, res_async = raw[:n3].reshape(-1, 3), raw[n3:n3 + capi.NRESULTS]
    got = raw[n3 + capi.NRESULTS:].reshape(2, -1)
    if precision == "mixed":
        # the positions the kernel sees: float(x) + float(x - float(x))
        hi = x.astype(np.float32).astype(np.float64)
        x = hi + (x - hi).astype(np.float32).astype(np.float64)
    fix = lambda F: np.rint(np.asarray(F) * 2.0 ** 32) / 2.0 ** 32
    ref = _reference_order(s)
    h = capi.Handle([ref])
    for k, lam1_shift in enumerate((0.0, 0.1)):
        a = p.as_array().copy()
        a[P_LAMBDA1] += lam1_shift
        h.set_params(0, a)
        res, F = h.evaluate(x)
        e, rr, ff = got[k, 0], got[k, 1:1 + capi.NRESULTS], got[k, 1 + capi.NRESULTS:].reshape(-1, 3)
        assert e == res[0, capi.R_EPOT]
        assert np.array_equal(rr[:capi.R_STATUS], res[0, :capi.R_STATUS])
        assert np.array_equal(ff, fix(F.reshape(-1, 3)))
        if k == 0:
            assert np.array_equal(f_async, ff)
            assert np.array_equal(res_async[:capi.R_STATUS], res[0, :capi.R_STATUS])
    h.close()


@pytest.fixture(scope="module")
def fake_driver(tmp_path_factory):
    """The same driver linked against the C-ABI stand-in of
    tests/openmm_api/fake_sdm.cpp (results follow from the parameters)."""
    exe = str(tmp_path_factory.mktemp("shim_fake") / "shim_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
           "-I", API, "-I", os.path.join(ROOT, "include"), "-I", SHIM,
           os.path.join(SHIM, "SDMForceGB300.cpp"), os.path.join(API, "ApiSubset.cpp"),
           os.path.join(API, "shim_driver.cpp"), os.path.join(API, "fake_sdm.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_non_equilibrium_protocol_on_context_time(fake_driver, tmp_path):
    """lambda = t / Ntmax at every evaluation (parameters pushed once per
    new time), and the work the reference integrator accumulates,
    sum_k (dt / Ntmax) dW/dlambda(t_k), read after each step; a second
    evaluation at the same time adds nothing; setNoneqWorkvalue restarts
    the sum (ReferenceSDMKernels.cpp:229-245, 289-302)."""
    s = S.config0(variant="b")
    T, dt, nsteps = 0.02, 0.002, 7
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, s, s.params[0], s.positions[0])
    with open(inp, "ab") as f:
        np.array([T, dt], np.float64).tofile(f)
        np.array([nsteps], np.int32).tofile(f)
    r = subprocess.run([fake_driver, "noneq", inp, out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    v = np.frombuffer(open(out, "rb").read(), np.float64)
    per_step, (w1, w2, w3) = v[:-3].reshape(-1, 2), v[-3:]
    assert per_step.shape[0] == nsteps + 1
    t, work, lams = 0.0, 0.0, []
    for _ in range(nsteps):
        lams.append(t / T)
        work += dt / T * (3.0 + 2.0 * (t / T))   # the stand-in's dW/dlambda
        t += dt
    assert np.array_equal(per_step[:nsteps, 0], 100.0 * np.array(lams))
    assert np.all(np.diff(per_step[:, 1]) == 1.0)      # one parameter push per new time
    assert w1 == pytest.approx(work, rel=1e-14)
    assert w2 == 1.5
    assert w3 == pytest.approx(1.5 + dt / T * (3.0 + 2.0 * (t / T)), rel=1e-14)


def test_box_change_rebuilds_the_handle(fake_driver, tmp_path):
    """A context whose box changes (a barostat) gets a new handle, made with
    the new box and the context's parameters; a triclinic box is refused."""
    s = S.config0(variant="b")
    r, out = run(fake_driver, "rebox", tmp_path, s, s.params[0], s.positions[0])
    assert r.returncode == 3 and "rectangular" in r.stderr, r.stderr
    raw = np.frombuffer(open(out, "rb").read(), np.float64)
    v, pe = raw[:9].reshape(3, 3), raw[9:]
    pushes, box_x, creates = v[:, 0], v[:, 1], v[:, 2]
    # getPerturbationEnergy: (u, U0, U1, W, W') from the results' own slots
    assert list(pe) == [7.0, s.box[0] + 0.1, creates[2], 11.0, 13.0]
    # the same box keeps the handle; the new box makes a new one, created
    # with that box and given the parameters once
    assert list(box_x) == [s.box[0], s.box[0], s.box[0] + 0.1]
    assert creates[1] == creates[0] and creates[2] == creates[0] + 1
    assert list(pushes) == [1.0, 1.0, 1.0]


def test_failed_parameter_update_changes_nothing(fake_driver, tmp_path):
    """updateParametersInContext is all or nothing: a non-finite displacement
    is refused before anything is pushed, a displacement the library refuses
    brings the handle back to the parameters it had, and a handle re-created
    later (box change) gets the last good parameters."""
    s = S.config0(variant="b")
    p = dataclasses.replace(s.params[0], bias_method=0, lambdac=0.3)
    r, out = run(fake_driver, "atomic", tmp_path, s, p, s.positions[0])
    assert r.returncode == 0, r.stderr
    e0, e1, e2, e3, creates, threw = np.frombuffer(open(out, "rb").read(), np.float64)
    assert threw == 3.0
    # the fake's energy is 100 lambda: every evaluation still sees lambda = 0.3
    assert e0 == pytest.approx(30.0) and e1 == e0 and e2 == e0 and e3 == e0
    assert creates == 2.0


def test_makefile_builds_the_plugin_library(driver, tmp_path):
    """The maintainer's recipe (openmm_sdm_plugin_gb300/shim/Makefile) against
    an OPENMM_DIR made of the API subset (headers, and a libOpenMM.so of its
    bodies): it builds libSDMPluginGB300.so, and a program linked with that
    library reads a NonbondedForce as the statically built driver does."""
    root = tmp_path / "openmm"
    (root / "lib").mkdir(parents=True)
    os.symlink(API, root / "include")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I", API,
                        os.path.join(API, "ApiSubset.cpp"), "-o", str(root / "lib" / "libOpenMM.so")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    plugin = str(tmp_path / "libSDMPluginGB300.so")
    r = subprocess.run(["make", "-s", "-C", SHIM, f"OPENMM_DIR={root}", f"OUT={plugin}"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    exe = str(tmp_path / "linked_driver")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", API, "-I", os.path.join(ROOT, "include"), "-I", SHIM,
                        os.path.join(API, "shim_driver.cpp"), "-o", exe, plugin, str(root / "lib" / "libOpenMM.so"),
                        "-Wl,-rpath," + str(tmp_path) + ":" + str(root / "lib")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    s = _dms_system()
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    ra, out_a = run(exe, "describe", tmp_path / "a", s, s.params[0], s.positions[0])
    rb, out_b = run(driver, "describe", tmp_path / "b", s, s.params[0], s.positions[0])
    assert ra.returncode == 0 and rb.returncode == 0, ra.stderr + rb.stderr
    assert open(out_a, "rb").read() == open(out_b, "rb").read()
    # the CUDA platform library, against a libOpenMMCUDA.so of the CUDA stand-in:
    # it exports the plugin entry points OpenMM calls
    cuda = _cuda_home()
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I", API, "-I", os.path.join(cuda, "include"),
                        os.path.join(API, "CudaSubset.cpp"), "-o", str(root / "lib" / "libOpenMMCUDA.so"),
                        str(root / "lib" / "libOpenMM.so"), "-L", os.path.join(cuda, "lib64"), "-lcudart"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    plugin_cuda = str(tmp_path / "libSDMPluginGB300CUDA.so")
    r = subprocess.run(["make", "-s", "-C", SHIM, "cuda", f"OPENMM_DIR={root}", f"OUT={plugin}",
                        f"OUT_CUDA={plugin_cuda}", f"CUDA_HOME={cuda}"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    syms = subprocess.run(["nm", "-D", "--defined-only", plugin_cuda], capture_output=True, text=True).stdout
    for name in ("registerKernelFactories", "registerPlatforms"):
        assert f" T {name}" in syms, name
