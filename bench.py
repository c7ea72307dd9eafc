#!/usr/bin/env python3
"""Benchmark of the SDM two-state force on GB300.

Metric: lambda-state force evaluations per second.  One lambda-state
evaluation = U0, U1, u (FP64), u', W, W' and the mixed force F for all
particles of one replica, from the current coordinates (cells, clusters and
neighbour candidates are rebuilt every call; nothing is reused).

Workload (headline): 22 replicas of the 22,580-particle relative-binding
system (7,500 rigid 3-site waters + two 40-atom ligands displaced by +/-d,
6.2 nm box, 1.0 nm reaction-field cutoff), each replica with its own seeded
coordinates and lambda state, evaluated in one batched call replayed as a
CUDA graph.  The plain form (one replica per call) is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs its own 22-replica batch on its own GPU (weak
scaling, no data-path collective); times are max-reduced over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SDM lambda-state force evals/s at 23k atoms x 22 lambda, batched vs plain, 1 GB300"
UNIT = "lambda-state evals/s"
FLOP_PER_PAIR = 52  # FP32 flops per pair per state (FMA = 2, rsqrt = 1)
# kernels of one batched evaluation: k_cells k_scan k_bucket k_cellsort k_clusters
# k_jlist k_pair k_pert_prep k_perturb k_combine k_finalize_mix
KERNELS_PER_STEP = 11
# Algorithmic bytes of the O(N) kernels, each datum read or written once
# (per particle, per cluster slot, per cell): k_cells reads x (24 B) and
# writes the wrapped copy (24 B), the cell pair (8 B) and a histogram count
# (4 B);
# k_bucket reads the cell pair and offset and writes the count and the
# bucket entry (20 B); k_cellsort reads the bucket entry, cell pair, cell
# bounds, z, column offsets and writes perm, inv and the cluster's reference
# cell (46 B); k_clusters reads perm, position, five per-particle
# parameters, the exclusion partners and their slots (80 B) and writes the
# cluster-ordered coordinates, parameters, group, molecule and exclusion
# slots (48 B), zeroes the slot's six fixed-point force words (48 B) and, per
# cluster of 8 slots, reads its reference cell and origin (40 B) and writes
# z bounds, box and links (72 B); the finalize
# reads inv and the six force words and writes the three mixed components
# (76 B); k_scan reads the cell counts and writes the cell offsets (8 B per
# cell, the column tables 12 B per column).
ON_BYTES = {"k_cells": (60, 0, 0, 0), "k_bucket": (20, 0, 0, 0), "k_cellsort": (46, 0, 0, 0),
            "k_clusters": (0, 190, 0, 0), "k_combine+k_finalize_mix": (76, 0, 0, 0), "k_scan": (0, 0, 8, 12)}
NREP = 22
WORKLOAD = ("config2: 22 replicas x 22,580 particles (7,500 waters + 2x40 ligand), 6.2 nm box, "
            "rc 1.0 nm reaction field, one batched call per step")
# dram__bytes_read.sum + dram__bytes_write.sum of one k_pair launch on this
# workload: a stored figure, the 4-replica ncu capture summarised in
# profiles/k_pair_config2x4.md scaled by 22/4 (cold cache between replay passes)
K_PAIR_DRAM_BYTES_PER_LAUNCH = (22.318080e6 + 0.0) * 22 / 4
K_PAIR_TRAFFIC_SOURCE = ("stored: ncu capture of 4 replicas of the same workload x 22/4 "
                         "(profiles/k_pair_config2x4.md)")


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"sm_max_mhz": 2070.0, "hbm_gbs": 6800.0}, "fallback"


class ClockSampler:
    """nvidia-smi sampler during the timed region (clocks + throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(seconds: float, dist, device=None) -> float:
    """Slowest rank's time (the job's time); identity on a single process."""
    if dist is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, world: int, seconds_max: float) -> float:
    """Units processed by all ranks over the slowest rank's time (weak scaling)."""
    return units_per_rank * world / seconds_max


def cpu_baseline_port(sysm, nthreads: int, budget_s: float = 10.0):
    """FP64 oracle (the CPU restatement of the reference path) on a bounded
    sample: whole lambda states of the workload, one after another."""
    import oracle
    o = oracle.OracleSystem(sysm)
    x = sysm.positions
    p = [q.as_array() for q in sysm.params]
    t0 = time.perf_counter()
    n = 0
    while True:
        oracle.eval_state(o, x[n % len(x)], p[n % len(p)], nthreads=nthreads)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def cpu_baselines(sysm, budget_s: float = 10.0, budget_small_s: float = 2.0):
    """The cpu_baseline object: the FP64 oracle on one host core, on whole
    lambda states of one 22,580-particle replica of the workload (`value`),
    with the 930-site system timed beside it (`per_config`)."""
    from openmm_sdm_plugin_gb300 import systems as S
    v1, n1, dt1 = cpu_baseline_port(sysm.replica(0), nthreads=1, budget_s=budget_s)
    s0 = S.config0(variant="b")
    v0, n0, dt0 = cpu_baseline_port(s0, nthreads=1, budget_s=budget_small_s)
    return {"value": v1, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n1} FP64 lambda-state evaluations of one 22,580-particle replica in {dt1:.1f} s",
            "per_config": {
                "config1_22580": {"value": v1, "unit": UNIT, "sample": f"{n1} states in {dt1:.1f} s"},
                "config0_930": {"value": v0, "unit": UNIT, "sample": f"{n0} states of {s0.n} sites in {dt0:.1f} s"}}}


def run_reference(args):
    """--impl reference: the reference path's CPU implementation on the host cores.

    The reference's own Reference platform cannot be built here (it links
    OpenMM, which is absent), so the FP64 oracle port stands in, using every
    host thread."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from openmm_sdm_plugin_gb300 import systems as S
    import oracle
    oracle.build()
    sysm = S.config2(NREP)
    nth = os.cpu_count() or 1
    o = oracle.OracleSystem(sysm)
    params = [q.as_array() for q in sysm.params]
    # each step: a bounded sample of the 22-state batch (states k, k+1, ...
    # round robin), sized from the warm-up so that all steps take ~60 s
    k = 0
    t0 = time.perf_counter()
    for _ in range(max(1, args.warmup)):
        oracle.eval_state(o, sysm.positions[k % NREP], params[k % NREP], nthreads=nth)
        k += 1
    t_state = (time.perf_counter() - t0) / max(1, args.warmup)
    per_step = max(1, min(NREP, int(60.0 / max(args.steps * t_state, 1e-9))))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for _ in range(per_step):
            oracle.eval_state(o, sysm.positions[k % NREP], params[k % NREP], nthreads=nth)
            k += 1
        times.append(time.perf_counter() - t0)
    total = sum(times)
    v = per_step * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD,
                   "sample": f"{per_step} lambda states per step (round robin over the 22)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": f"{per_step} full FP64 lambda-state evaluations per step"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference Reference platform unbuildable here (needs OpenMM); FP64 oracle port"}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default schedule instead of the autotuner's choice")
    ap.add_argument("--tune-cache", default=None,
                    help="autotuner cache file (default: sdm_tune_cache.txt in the system temp directory)")
    ap.add_argument("--ctas", type=int, default=0, help="pair-kernel CTAs per SM (0 = library default)")
    ap.add_argument("--split", type=int, default=0, help="work items per i-cluster (0 = default)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import __graft_entry__ as ge
    from openmm_sdm_plugin_gb300 import capi, systems as S

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if rank == 0:
        ge.build()
    if dist is not None:
        dist.barrier()
    warm = max(3, args.warmup)

    # ---------------- workload ----------------
    sysm = S.config2(NREP)
    n = sysm.n
    h = capi.Handle([sysm], device=local)
    for r in range(NREP):
        h.set_params(r, sysm.params[r].as_array())
    xh = np.ascontiguousarray(sysm.positions.reshape(-1, 3))
    counts = h.count_pairs(xh)           # product diagnostic: P0, P1delta per replica
    P0 = int(counts[:, 0].sum())
    P1 = int(counts[:, 1].sum())
    flop_per_launch = FLOP_PER_PAIR * (P0 + P1)

    dev = torch.device("cuda", local)
    # a dedicated stream: flushes, events and graph replays all go on it (the
    # legacy default stream has handle 0, which the C ABI reads as "own stream")
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    assert sptr != 0
    xd = torch.from_numpy(xh).to(dev)
    rd = torch.zeros((NREP, capi.NRESULTS), dtype=torch.float64, device=dev)
    fd = torch.zeros_like(xd)
    for hh in (h,):
        if args.ctas:
            hh.set_option(capi.OPT_CTAS_PER_SM, args.ctas)
        if args.split:
            hh.set_option(capi.OPT_SPLIT, args.split)
    tuned = None
    if not args.no_autotune and not (args.ctas or args.split):
        import tempfile
        cache = args.tune_cache or os.path.join(tempfile.gettempdir(), "sdm_tune_cache.txt")
        # the lists are sized by a first evaluation, then every schedule is timed
        h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), sptr)
        torch.cuda.synchronize()
        h.check_status()
        tuned = h.autotune(xd.data_ptr(), cache)
    l2 = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    def flush():
        with torch.cuda.stream(stream):
            l2.zero_()

    # plain form: one replica per call
    s1 = sysm.replica(0)
    h1 = capi.Handle([s1], device=local)
    h1.set_params(0, s1.params[0].as_array())
    if args.ctas:
        h1.set_option(capi.OPT_CTAS_PER_SM, args.ctas)
    if args.split:
        h1.set_option(capi.OPT_SPLIT, args.split)
    x1 = xd[:n].contiguous()
    r1 = torch.zeros((1, capi.NRESULTS), dtype=torch.float64, device=dev)
    f1 = torch.zeros_like(x1)
    tuned1 = None
    if tuned is not None:
        h1.evaluate_device(x1.data_ptr(), r1.data_ptr(), f1.data_ptr(), sptr)
        torch.cuda.synchronize()
        h1.check_status()
        tuned1 = h1.autotune(x1.data_ptr(), cache)

    def timed(fn, steps, warmup, per_kernel=None, pre=None):
        for _ in range(warmup):
            if pre is not None:
                pre()
            fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        pk = []
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        for k in range(steps):
            flush()
            if pre is not None:   # untimed: runs before the start event
                pre()
            ev[k][0].record(stream)
            fn()
            ev[k][1].record(stream)
            if per_kernel is not None:
                ev[k][1].synchronize()
                pk.append(per_kernel())
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        ms = [a.elapsed_time(b) for a, b in ev]
        return ms, pk

    # ---- batched (headline): the uninstrumented graph ----
    h.set_option(capi.OPT_PROFILE, 0)
    sampler = ClockSampler(local)
    sampler.start()
    t_wall0 = time.perf_counter()
    ms_b, _ = timed(lambda: h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), sptr),
                    args.steps, warm)
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    tot_b = max_over_ranks(sum(ms_b) / 1e3, dist, dev)
    value = whole_job_rate(NREP * args.steps, world, tot_b)
    ncl_tot = int(rd[:, capi.R_NCL].sum().item())   # clusters of all replicas (headline call)
    # per-kernel times: a second timed region of the same call with CUDA events
    # recorded between the kernels inside the graph (the event nodes add to the
    # call, so the headline region above runs without them)
    h.set_option(capi.OPT_PROFILE, 2)
    n_prof = min(args.steps, 100)
    ms_prof, pk = timed(lambda: h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), sptr),
                        n_prof, warm, per_kernel=h.kernel_times)
    h.set_option(capi.OPT_PROFILE, 0)
    jlist_ms = [d["k_jlist"] for d in pk]
    pair_ms = [d["k_pair"] for d in pk]
    pert_ms = [d["k_pert_prep+k_perturb"] for d in pk]
    pair_avg = sum(pair_ms) / len(pair_ms)
    breakdown = {k: sum(d[k] for d in pk) / len(pk) for k in pk[0]}

    # ---- plain: one replica per call ----
    h1.set_option(capi.OPT_PROFILE, 0)
    ms_p, _ = timed(lambda: h1.evaluate_device(x1.data_ptr(), r1.data_ptr(), f1.data_ptr(), sptr),
                    args.steps, warm)
    plain = args.steps / (sum(ms_p) / 1e3)

    # ---- fused Langevin dynamics on the same batch (evaluation + update per step) ----
    h.set_option(capi.OPT_PROFILE, 0)
    # Masses of the synthetic model (O 15.999, H 1.008, ligand 12.011); the
    # model's waters are rigid only under constraints, which this step does
    # not apply, so every timed step starts again from the benchmark
    # configuration (restored outside the timed region, like the L2 flush)
    # while the generator's step counter keeps advancing.
    g = torch.Generator().manual_seed(5)
    x0l = xd.clone()
    v0l = torch.randn(xd.shape, generator=g, dtype=torch.float64).mul_(0.3).to(dev)
    sig = torch.from_numpy(np.tile(sysm.sigma, NREP)).to(dev)
    nw3 = 3 * ((sysm.n - 80) // 3)
    mass = torch.full((xd.shape[0],), 12.011, dtype=torch.float64, device=dev)
    idx = torch.arange(xd.shape[0], device=dev) % sysm.n
    mass[(idx < nw3) & (sig != 0)] = 15.999
    mass[(idx < nw3) & (sig == 0)] = 1.008
    iml = 1.0 / mass
    xl, vl = x0l.clone(), v0l.clone()

    def reset():
        with torch.cuda.stream(stream):
            xl.copy_(x0l)
            vl.copy_(v0l)

    h.set_langevin(0.002, 1.0, 300.0, seed=17)
    ms_l, _ = timed(lambda: h.langevin_step(xl.data_ptr(), vl.data_ptr(), iml.data_ptr(), rd.data_ptr(), 1,
                                            0, sptr), args.steps, warm, pre=reset)
    tot_l = max_over_ranks(sum(ms_l) / 1e3, dist, dev)
    langevin = {"value": whole_job_rate(NREP * args.steps, world, tot_l), "unit": "lambda-state MD steps/s",
                "ms_per_step": sum(ms_l) / len(ms_l), "device_status": h.check_status(),
                "workload": "sdm_langevin_step on the 22-replica batch: two-state evaluation, mix and "
                            "stochastic-dynamics update in one CUDA graph per step (dt 2 fs, 1/ps, 300 K), "
                            "every step from the benchmark configuration"}

    # ---- parameter-gradient sums (the adjoint pass) after every evaluation ----
    # sdm_adjoint synchronises and returns host sums, so this field is timed
    # by the host clock around evaluation + adjoint
    nd_tot = NREP * int(np.count_nonzero(np.any(sysm.displacement != 0, axis=1)))
    nadj = min(args.steps, 100)

    def adj_call():
        h.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), sptr)
        h.adjoint(nd_tot)
    for _ in range(warm):
        adj_call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(nadj):
        adj_call()
    torch.cuda.synchronize()
    t_adj = max_over_ranks(time.perf_counter() - t0, dist, dev)
    adjoint = {"value": whole_job_rate(NREP * nadj, world, t_adj),
               "unit": "lambda-state evals with parameter-gradient sums/s",
               "ms_per_call": 1e3 * t_adj / nadj, "steps": nadj, "clock": "host (the call synchronises)",
               "workload": "the benchmark batch: evaluation, then sdm_adjoint (the sums behind dU0/dp, "
                           "dU1/dp of the displaced particles' charge, sigma, epsilon) every call"}

    # ---- the same batch with PME electrostatics (smooth PME, order 5, tol 5e-4) ----
    import dataclasses
    sys_pme = dataclasses.replace(sysm, nonbonded_method="pme", ewald_tolerance=5e-4)
    hp = capi.Handle([sys_pme], device=local)
    for r in range(NREP):
        hp.set_params(r, sys_pme.params[r].as_array())
    tunedp = None
    if tuned is not None:
        hp.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), sptr)
        torch.cuda.synchronize()
        hp.check_status()
        tunedp = hp.autotune(xd.data_ptr(), cache)
    npme = min(args.steps, 100)
    ms_pm, _ = timed(lambda: hp.evaluate_device(xd.data_ptr(), rd.data_ptr(), fd.data_ptr(), sptr), npme, warm)
    tot_pm = max_over_ranks(sum(ms_pm) / 1e3, dist, dev)
    pme = {"value": whole_job_rate(NREP * npme, world, tot_pm), "unit": UNIT, "ms_per_call": sum(ms_pm) / npme,
           "steps": npme, "device_status": hp.check_status(), "tuning": tunedp,
           "workload": "the benchmark batch (22 x 22,580 particles) with PME instead of reaction field: "
                       "Ewald direct space in the pair kernels, excluded-pair corrections, reciprocal space "
                       "of both states (state-0 grid and the displaced-charge difference, cuFFT) per replica"}
    hp.close()

    # ---- a real system: the TEMOA DMS fixture (20,446 particles, 606 1-4
    # exceptions), the same 22-state schedule, one batched call per step ----
    temoa = None
    tpath = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "temoa_g1_g4.npz")
    if os.path.exists(tpath):
        from openmm_sdm_plugin_gb300 import dms
        st_t = dms.load_compact(tpath, displacement={2: (2.2, 2.2, 2.2), 3: (-2.2, -2.2, -2.2)},
                                params=sysm.params)
        ht = capi.Handle([st_t], device=local)
        for r in range(NREP):
            ht.set_params(r, st_t.params[r].as_array())
        xt = torch.from_numpy(np.ascontiguousarray(st_t.positions.reshape(-1, 3))).to(dev)
        rt = torch.zeros((NREP, capi.NRESULTS), dtype=torch.float64, device=dev)
        ft = torch.zeros_like(xt)
        nt = min(args.steps, 100)
        ms_t, _ = timed(lambda: ht.evaluate_device(xt.data_ptr(), rt.data_ptr(), ft.data_ptr(), sptr), nt, warm)
        tot_t = max_over_ranks(sum(ms_t) / 1e3, dist, dev)
        temoa = {"value": whole_job_rate(NREP * nt, world, tot_t), "unit": UNIT, "ms_per_call": sum(ms_t) / nt,
                 "steps": nt, "device_status": ht.check_status(),
                 "workload": "temoa-g1-g4 (tests/golden fixture of the reference's example DMS): 22 lambda "
                             "states x 20,446 particles, the stored coordinates, guests displaced +-2.2 nm/axis"}
        ht.close()

    # ---- the uneven multi-system batch: 64 host-guest systems x 16 lambda
    # states (1,024 replicas, 2,010-54,820 particles each) in one call ----
    ms3, c3 = [], None
    s3 = S.config3()
    h3 = capi.Handle(s3, device=local)
    r = 0
    for sy in s3:
        for p in sy.params:
            h3.set_params(r, p.as_array())
            r += 1
    x3h = np.ascontiguousarray(np.concatenate([sy.positions.reshape(-1, 3) for sy in s3]))
    cnt3 = h3.count_pairs(x3h)
    x3 = torch.from_numpy(x3h).to(dev)
    r3 = torch.zeros((h3.nrep, capi.NRESULTS), dtype=torch.float64, device=dev)
    f3 = torch.zeros_like(x3)
    tuned3 = None
    if tuned is not None:
        h3.evaluate_device(x3.data_ptr(), r3.data_ptr(), f3.data_ptr(), sptr)
        torch.cuda.synchronize()
        h3.check_status()
        tuned3 = h3.autotune(x3.data_ptr(), cache)
    h3.set_option(capi.OPT_PROFILE, 0)
    n3 = min(args.steps, 20)
    ms3, _ = timed(lambda: h3.evaluate_device(x3.data_ptr(), r3.data_ptr(), f3.data_ptr(), sptr), n3, warm)
    tot3 = max_over_ranks(sum(ms3) / 1e3, dist, dev)
    h3.set_option(capi.OPT_PROFILE, 2)
    _, pk3 = timed(lambda: h3.evaluate_device(x3.data_ptr(), r3.data_ptr(), f3.data_ptr(), sptr), n3, warm,
                   per_kernel=h3.kernel_times)
    pair3 = sum(d["k_pair"] for d in pk3) / len(pk3)
    flop3 = FLOP_PER_PAIR * int(cnt3.sum())
    config3 = {"value": whole_job_rate(h3.nrep * n3, world, tot3), "unit": UNIT, "ms_per_call": sum(ms3) / n3,
               "steps": n3, "device_status": h3.check_status(), "replicas": h3.nrep,
               "particles": int(sum(sy.n * sy.replicas for sy in s3)),
               "pair_kernel_ms": pair3, "pair_frac": None, "tuning": tuned3,
               "flop_per_launch": flop3,
               "workload": "config3: 64 host-guest systems (2,010-54,820 particles, log-uniform, seed 3) x 16 "
                           "lambda states, every replica its own coordinates, one batched call per step"}
    h3.close()
    del x3, r3, f3

    # ---- backward: the 22-state batch through the autograd Function, forward
    # (evaluation, state-1 forces, adjoint sums) and backward (gradients for
    # positions, ligand charge/sigma/epsilon, displacement map, lambda1,
    # lambda2, alpha, u0, w0), all device-resident on one stream ----
    from openmm_sdm_plugin_gb300.autograd import SDMEngine, sdm_potential
    eng = SDMEngine(sysm, device=local)
    Dl = eng.D
    f64 = dict(dtype=torch.float64, device=dev)
    xg = xd.view(NREP, n, 3).clone().requires_grad_(True)
    qD = torch.tensor(sysm.charge[Dl], **f64).requires_grad_(True)
    sD = torch.tensor(sysm.sigma[Dl], **f64).requires_grad_(True)
    eD = torch.tensor(sysm.epsilon[Dl], **f64).requires_grad_(True)
    dg = torch.tensor(sysm.displacement, **f64).requires_grad_(True)
    vec = lambda k: torch.tensor([getattr(p, k) for p in sysm.params], **f64).requires_grad_(True)
    lams = [vec(k) for k in ("lambda1", "lambda2", "alpha", "u0", "w0")]
    leaves = [xg, qD, sD, eD, dg] + lams

    def bwd_step():
        for t in leaves:
            t.grad = None
        with torch.cuda.stream(stream):
            U = sdm_potential(eng, xg, qD, sD, eD, dg, *lams)
            U.sum().backward()

    nb = min(args.steps, 100)
    ms_bw, _ = timed(bwd_step, nb, warm)
    tot_bw = max_over_ranks(sum(ms_bw) / 1e3, dist, dev)
    backward = {"value": whole_job_rate(NREP * nb, world, tot_bw),
                "unit": "lambda-state evals with full gradients/s", "ms_per_step": sum(ms_bw) / nb, "steps": nb,
                "device_status": eng.h.check_status(),
                "workload": "config4: forward + backward of the 22-state config2 batch through the "
                            "torch.autograd.Function (dU/dx, dU/dq, dU/dsigma, dU/depsilon of the 80 ligand "
                            "particles, dU/dd, dU/dlambda1, dU/dlambda2, dU/dalpha, dU/du0, dU/dw0), device timed"}
    eng.close()

    # ---- e2e through the host C ABI: pinned host inputs/outputs ----
    h.set_option(capi.OPT_PROFILE, 0)
    xpin = torch.from_numpy(xh.copy()).pin_memory()
    rpin = torch.zeros((NREP, capi.NRESULTS), dtype=torch.float64).pin_memory()
    fpin = torch.zeros_like(xpin).pin_memory()
    import ctypes as C
    L = capi.load_library()

    def e2e_step():
        st = L.sdm_evaluate(h.h, C.c_void_p(xpin.data_ptr()), C.c_void_p(rpin.data_ptr()),
                            C.c_void_p(fpin.data_ptr()))
        if st != 0:
            raise capi.SdmError(st, L.sdm_last_error(h.h).decode())

    def e2e_run():
        for _ in range(warm):
            e2e_step()
        ms = []
        for _ in range(args.steps):
            flush()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2e_step()   # host coordinates in, evaluation, host results and forces out, synchronise
            ms.append(1e3 * (time.perf_counter() - t0))
        return ms

    # page-locked host buffers, copied in and out by the copy engines (the
    # library default) ...
    e2e_ms = e2e_run()
    tot_e = max_over_ranks(sum(e2e_ms) / 1e3, dist, dev)
    e2e = whole_job_rate(NREP * args.steps, world, tot_e)
    # ... and, for comparison, the coordinates read in place by k_cells over
    # the host link (SDM_OPT_ZERO_COPY)
    h.set_option(capi.OPT_ZERO_COPY, 1)
    e2e_ms_zc = e2e_run()
    h.set_option(capi.OPT_ZERO_COPY, 0)
    tot_ez = max_over_ranks(sum(e2e_ms_zc) / 1e3, dist, dev)
    e2e_zc = whole_job_rate(NREP * args.steps, world, tot_ez)
    # check the batch result once against nothing but itself: status clean
    status = h.check_status()

    # ---- roofline of the pair kernel (FP32 pipe) ----
    peaks, src = _peaks()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fmax = float(peaks.get("sm_max_mhz", 2070.0))
    peak_tf = nsm * 128 * 2 * fmax * 1e6 / 1e12
    achieved_tf = flop_per_launch / (pair_avg * 1e-3) / 1e12
    config3["pair_frac"] = flop3 / (config3["pair_kernel_ms"] * 1e-3) / 1e12 / peak_tf
    f_run = clocks.get("sm_mhz")
    jl_avg = sum(jlist_ms) / len(jlist_ms)
    pt_avg = sum(pert_ms) / len(pert_ms)

    roof = {"bound": "fp32", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
            "frac": achieved_tf / peak_tf, "traffic": K_PAIR_DRAM_BYTES_PER_LAUNCH,
            "traffic_source": K_PAIR_TRAFFIC_SOURCE,
            "kernel": "k_pair (main pass, all 22 replicas)",
            "peak_source": f"{nsm} SMs x 128 FP32 lanes x 2 x {fmax:.0f} MHz ({src} sm_max_mhz)",
            "frac_at_run_clock": (achieved_tf / (nsm * 256 * f_run * 1e6 / 1e12)) if f_run else None,
            "pair_kernel_ms": pair_avg, "perturb_kernel_ms": pt_avg, "jlist_kernel_ms": jl_avg,
            "frac_pair_path": (flop_per_launch / ((pair_avg + jl_avg + pt_avg) * 1e-3) / 1e12) / peak_tf,
            "frac_whole_call": (flop_per_launch / (sum(ms_b) / len(ms_b) * 1e-3) / 1e12) / peak_tf,
            "flop_per_launch": flop_per_launch, "P0": P0, "P1delta": P1}

    # O(N) kernels against the measured HBM bandwidth: algorithmic bytes per
    # launch (ON_BYTES x particles, slots, cells, columns) over the in-graph
    # event times of the profiled region
    Mg = h.grid(0)
    units = (NREP * n, 8 * ncl_tot, NREP * int(Mg[0] * Mg[1] * Mg[2]), NREP * int(Mg[0] * Mg[1]))
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    on_kernels = {}
    for k, per in ON_BYTES.items():
        if k not in breakdown:
            continue
        b = float(sum(pu * u for pu, u in zip(per, units)))
        gbs = b / (breakdown[k] * 1e-3) / 1e9
        on_kernels[k] = {"ms": breakdown[k], "bytes": b, "gbs": gbs, "frac_hbm": gbs / hbm}
    on_kernels["peak_gbs"] = hbm

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baselines(sysm)

    h2d = xh.nbytes
    d2h = xh.nbytes + NREP * capi.NRESULTS * 8
    plain_obj = {"value": plain, "unit": UNIT, "ms_per_call": sum(ms_p) / len(ms_p), "tuning": tuned1,
                 "workload": "config1: one 22,580-particle replica per call (CUDA graph)"}
    # secondary fields first, the headline keys last (a reader of the line's
    # tail sees value, e2e, roofline, plain and batched_over_plain)
    line = {
        "kernel_ms": breakdown,
        "on_kernels": on_kernels,
        "kernel_timing": {"steps": n_prof, "ms_per_step_instrumented": sum(ms_prof) / len(ms_prof),
                          "how": "CUDA events between the kernels inside the replayed graph, over a second "
                                 "timed region of the headline call; the headline region runs the graph "
                                 "without them"},
        "langevin": langevin,
        "dms_temoa": temoa,
        "pme": pme,
        "adjoint": adjoint,
        "config3": config3,
        "backward": backward,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "device_status": status,
        "wall_s_timed_region": t_wall,
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warm, "ms_per_step": sum(ms_b) / len(ms_b), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 pairs, int64 fixed-point forces, f64 energies",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD,
                   "replicas_per_gpu": NREP, "particles": n, "l2": "flushed (256 MB write) before every timed step",
                   "parallelism": f"replicas only, {world} independent rank(s)",
                   "schedule": {"split": h.get_option(capi.OPT_SPLIT), "ctas_per_sm": h.get_option(capi.OPT_CTAS_PER_SM),
                                "ctas_resident": h.get_option(capi.OPT_PAIR_RESIDENT),
                                "stage_chunk": h.get_option(capi.OPT_STAGE_CHUNK),
                                "list_group": h.get_option(capi.OPT_LIST_GROUP) or 4,
                                "overlap": h.get_option(capi.OPT_OVERLAP),
                                "autotuned": tuned is not None,
                                "tuning": tuned}},
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": sum(e2e_ms) / len(e2e_ms),
                "path": "sdm_evaluate (host C ABI) on page-locked host buffers, cudaMemcpyAsync in and out",
                "coords_in_place": {"value": e2e_zc, "ms_per_step": sum(e2e_ms_zc) / len(e2e_ms_zc),
                                    "path": "same call, SDM_OPT_ZERO_COPY=1: k_cells reads the host coordinates"}},
        "roofline": roof,
        "plain": plain_obj,
        "batched_over_plain": value / world / plain,
    }
    if rank == 0:
        print(json.dumps(line))
    h.close()
    h1.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
