"""Run a named workload for a few steps, for profiling one kernel in isolation.

    python profile_case.py pipe --steps 10 --form f32
    python profile_case.py cube --n 128 --steps 10
    python profile_case.py pipe --graph-steps 20   # then 20 graph-replayed steps

Workloads: ``pipe`` (64x64x256 cylinder at 25% haematocrit, 279 RBC),
``cube`` (periodic fluid box of edge n with a Kolmogorov force, no cells),
``kolmogorov`` (the 128^3 suspension of RBC, PLT and WBC).  The case runs
the batched launch with the given tuning (``--tune`` as eight integers) and
prints the per-stage CUDA-event times of the last steps (each stage on its
own) and the per-kernel times inside the batched step; ``--graph-steps``
then runs that many whole steps the way ``iterate`` does (CUDA graph replay
in the batched launch, fused kernels), for a profiler to capture.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from hemocell_gb300 import _lib as L  # noqa: E402
from hemocell_gb300 import cases  # noqa: E402


def build_case(name: str, n: int):
    if name == "pipe":
        return cases.pipe_ht25(seed=1)
    if name == "cube":
        return cases.Case(f"cube_{n}", (n, n, n), (1, 1, 1), body_mode=L.HC_BODY_KOLMOGOROV, body=(1e-6, 0.0, 0.0))
    if name == "kolmogorov":
        return cases.kolmogorov_mix(n=n, seed=1)
    raise SystemExit(f"unknown workload {name}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["pipe", "cube", "kolmogorov"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--form", choices=["f32", "f64"], default="f32")
    ap.add_argument("--tune", type=int, nargs=8, default=None)
    ap.add_argument("--graph-steps", type=int, default=0)
    a = ap.parse_args(argv)
    case = build_case(a.workload, a.n)
    form = L.HC_FORM_MIXED_F32 if a.form == "f32" else L.HC_FORM_PLAIN_F64
    hc = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    if a.tune:
        hc.set_tuning(a.tune)
    hc.iterate(a.warmup)
    hc.sync()
    stages = hc.profile_stages(a.steps)
    kernels = hc.profile_kernels(max(a.steps, 2))
    if a.graph_steps:
        hc.iterate(a.graph_steps)
        hc.sync()
    print(json.dumps({"workload": case.name, "nodes": case.N, "vertices": case.nvertices, "tuning": hc.tuning(),
                      "stages_us": {k: round(v * 1e3, 2) for k, v in stages.items()},
                      "kernels_us": {k: round(v * 1e3, 2) for k, v in kernels.items()},
                      "status": hc.device_status()}))
    hc.close()


if __name__ == "__main__":
    main()
