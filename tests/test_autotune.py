"""The autotuner (sdm_autotune_cached): every staging chunk and schedule of
the main pass timed on the production path, then the list-building group and
the graph's second branch on the fastest of them; the choice cached under the
workload key and read back by a second handle (an older cache line without
the last two fields reads with their defaults); the chosen setting gives the
same results as the default one within the parity tolerances."""
import os

import numpy as np
import pytest

from helpers import FORCE_RMS_REL_TOL, U_ABS_TOL, energy_tol, rms_rel
from openmm_sdm_plugin_gb300 import capi, systems as S

pytestmark = pytest.mark.gpu


def _handle(s):
    h = capi.Handle([s])
    for r in range(s.replicas):
        h.set_params(r, s.params[r].as_array())
    return h


def test_autotune_chooses_caches_and_keeps_results(tmp_path):
    import torch
    s = S.config2(nrep=4)
    x = np.ascontiguousarray(s.positions.reshape(-1, 3))
    h = _handle(s)
    ref_res, ref_F = h.evaluate(x)
    xd = torch.from_numpy(x).cuda()
    cache = str(tmp_path / "tune.txt")
    r1 = h.autotune(xd.data_ptr(), cache)
    assert not r1["from_cache"] and r1["ms"] > 0
    assert r1["stage_chunk"] in (8, 12, 16) and r1["ctas_per_sm"] in (3, 4) and r1["split"] in (1, 2)
    assert h.get_option(capi.OPT_STAGE_CHUNK) == r1["stage_chunk"]
    assert h.get_option(capi.OPT_CTAS_PER_SM) == r1["ctas_per_sm"]
    assert h.get_option(capi.OPT_SPLIT) == r1["split"]
    assert r1["list_group"] in (1, 2, 4) and r1["overlap"] in (0, 1, 2)
    assert h.get_option(capi.OPT_LIST_GROUP) == r1["list_group"]
    assert h.get_option(capi.OPT_OVERLAP) == r1["overlap"]
    res, F = h.evaluate(x)
    for r in range(4):
        assert abs(res[r, capi.R_U] - ref_res[r, capi.R_U]) < U_ABS_TOL
        assert abs(res[r, capi.R_U0] - ref_res[r, capi.R_U0]) < energy_tol(ref_res[r, capi.R_U0], 4.5e6)
    assert rms_rel(F, ref_F) < FORCE_RMS_REL_TOL
    h.close()
    lines = open(cache).read().splitlines()
    key = capi.tune_key([s], torch.cuda.get_device_properties(0).multi_processor_count)
    assert len(lines) == 1 and lines[0].startswith(key + "|")
    # a second handle of the same workload takes the choice from the cache
    h2 = _handle(S.config2(nrep=4))
    r2 = h2.autotune(xd.data_ptr(), cache)
    assert r2["from_cache"]
    fields = ("stage_chunk", "ctas_per_sm", "split", "list_group", "overlap")
    assert all(r2[k] == r1[k] for k in fields)
    assert h2.get_option(capi.OPT_STAGE_CHUNK) == r1["stage_chunk"]
    assert h2.get_option(capi.OPT_LIST_GROUP) == r1["list_group"]
    h2.close()
    assert os.path.exists(cache)
    # a line written before the last two fields existed: list group 4, branch 2
    with open(cache, "w") as f:
        f.write(f"{key}|{r1['stage_chunk']} {r1['ctas_per_sm']} {r1['split']} 0.5\n")
    h3 = _handle(S.config2(nrep=4))
    h3.set_option(capi.OPT_LIST_GROUP, 1)
    h3.set_option(capi.OPT_OVERLAP, 0)
    r3 = h3.autotune(xd.data_ptr(), cache)
    assert r3["from_cache"] and r3["list_group"] == 4 and r3["overlap"] == 2
    assert h3.get_option(capi.OPT_LIST_GROUP) == 4 and h3.get_option(capi.OPT_OVERLAP) == 2
    h3.close()
