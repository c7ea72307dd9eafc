"""The allocation-free entry point against the handle entry point.

sdm_evaluate_noalloc serves callers that cannot allocate device memory when
they need a force (graph-capturing code, hosts whose allocator owns all
device memory, latency-bound loops).  It keeps its scratch in one device
array shared by every call, so this test calls it twice in a row and checks
both results against sdm_evaluate on the same inputs, with the tolerances of
the other parity tests.  This file is collected last on purpose.
"""
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
