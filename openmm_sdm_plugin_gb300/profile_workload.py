"""Runs a fixed synthetic SDM workload a few times (for profilers).

  python -m openmm_sdm_plugin_gb300.profile_workload [--replicas 22] [--calls 3] [--eager] [--pme]
      [--chunk 8|12|16] [--ctas 3|4]

The workload is the batched relative-binding system used by the benchmark:
`--replicas` copies of the 22,580-particle system with independent seeded
coordinates.  Each call is one evaluation of all replicas (device buffers).
`--pme` evaluates the same systems with PME electrostatics (tolerance 5e-4).
"""
from __future__ import annotations

import argparse
import dataclasses

import numpy as np

from . import build as _build
from . import capi, systems


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--replicas", type=int, default=22)
    ap.add_argument("--calls", type=int, default=3)
    ap.add_argument("--eager", action="store_true", help="no CUDA graph")
    ap.add_argument("--config", default="config2", choices=["config2", "config0"])
    ap.add_argument("--pme", action="store_true", help="PME electrostatics instead of reaction field")
    ap.add_argument("--chunk", type=int, default=None, help="list entries per staged chunk (SDM_OPT_STAGE_CHUNK)")
    ap.add_argument("--ctas", type=int, default=None, help="pair-kernel CTAs per SM")
    a = ap.parse_args()
    _build.build()
    import torch
    s = systems.config2(a.replicas) if a.config == "config2" else systems.config0(variant="b")
    if a.pme:
        s = dataclasses.replace(s, nonbonded_method="pme", ewald_tolerance=5e-4)
    h = capi.Handle([s])
    for r in range(h.nrep):
        h.set_params(r, s.params[r].as_array())
    if a.eager:
        h.set_option(capi.OPT_GRAPH, 0)
    if a.chunk is not None:
        h.set_option(capi.OPT_STAGE_CHUNK, a.chunk)
    if a.ctas is not None:
        h.set_option(capi.OPT_CTAS_PER_SM, a.ctas)
    x = torch.from_numpy(np.ascontiguousarray(s.positions.reshape(-1, 3))).cuda()
    res = torch.zeros((h.nrep, capi.NRESULTS), dtype=torch.float64, device="cuda")
    f = torch.zeros_like(x)
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(a.calls):
        h.evaluate_device(x.data_ptr(), res.data_ptr(), f.data_ptr(), st)
    torch.cuda.synchronize()
    status = h.check_status()
    r = res.cpu().numpy()
    print(f"replicas={h.nrep} U0[0]={r[0, capi.R_U0]:.4f} u[0]={r[0, capi.R_U]:.6f} status={status}")
    h.close()
    return 0 if status == 0 else 1


if __name__ == "__main__":
    raise SystemExit(main())
