"""Host logic of the N>1 benchmark path on CPU ranks (gloo, world size 2).

Each rank evaluates its own independent batch of replicas (replicas only, no
data-path collective); the job time is the slowest rank's and the job rate
counts the units of every rank.  Here each rank times a small FP64 oracle
evaluation of its own replica so the ranks really differ in time.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import time

    import torch.distributed as dist

    import bench
    import oracle
    from openmm_sdm_plugin_gb300 import systems as S
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s = S.config0(seed=rank, variant="b")       # rank-specific replica
    o = oracle.OracleSystem(s)
    t0 = time.perf_counter()
    res, _ = oracle.eval_state(o, s.positions[0], s.params[0].as_array())
    dt = time.perf_counter() - t0 + 0.05 * rank  # rank 1 is the slow one
    tmax = bench.max_over_ranks(dt, dist)
    out[rank] = (dt, tmax, bench.whole_job_rate(3, world, tmax), float(res[0]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_replicas_only():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    d0, d1 = out[0], out[1]
    # every rank sees the slowest rank's time
    assert d0[1] == d1[1] == pytest.approx(max(d0[0], d1[0]))
    # whole-job rate: units of all ranks over the job time
    assert d0[2] == pytest.approx(3 * world / d0[1])
    # the ranks evaluated different replicas (independent work)
    assert d0[3] != d1[3]


def test_cpu_baselines_object(oracle_lib):
    """The bench line's cpu_baseline object: one host core, the oracle port,
    a value per config, samples named."""
    import bench
    from openmm_sdm_plugin_gb300 import systems as S
    c = bench.cpu_baselines(S.config2(2), budget_s=0.01, budget_small_s=0.01)
    assert c["kind"] == "port" and c["cores"] == 1 and c["unit"] == bench.UNIT
    assert c["value"] > 0 and c["value"] == c["per_config"]["config1_22580"]["value"]
    assert c["per_config"]["config0_930"]["value"] > c["value"]
    assert "930 sites" in c["per_config"]["config0_930"]["sample"]
