"""Benchmark of the GB300 HemoCell IB-LBM step (MLUPS including IBM and cell forces).

Workload: the 25%-hematocrit pipe, 64x64x256 D3Q19 lattice, a 30-lu-radius
cylinder of bounce-back walls along z, Poiseuille body force, 279 RBCs
(642 vertices each) from a seeded packing.  A step is one HemoCell::iterate():
spread, collide+stream, interpolate+advance, membrane forces.

Arms:
  default            the GB300 library: headline = FP32 mixed form, batched
                     launch, whole step replayed as a CUDA graph; the FP64
                     plain per-stage form is timed beside it.
  --impl reference   the reference's CPU path of this step: the reference
                     itself cannot be built here (Palabos/MPI/HDF5 are not in
                     its tree), so its FP64 CPU restatement (oracle/) runs on
                     all host cores.

One JSON line on stdout.  Timing: CUDA events on the handle's stream around
exactly K steps after W warm-up steps; the per-step working set (~190 MB in
FP32, ~370 MB in FP64) exceeds the 129 MB L2, so no flush is inserted.
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

# algorithmic bytes per fluid node and per vertex of one step
BYTES_NODE = {"f32": 2 * 19 * 4 + 2 * 3 * 4, "f64": 2 * 19 * 8 + 2 * 3 * 8}
BYTES_VERTEX = {"f32": 2 * 3 * 8 + 2 * 2 * 3 * 4, "f64": 2 * 3 * 3 * 8}
# DRAM bytes per fluid node of the collide-stream kernel, measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum on the 64x64x256 pipe)
K1_TRAFFIC_PER_NODE = {"f32": None, "f64": None}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[4 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def build_case(steps: int):
    from hemocell_gb300 import cases
    case = cases.pipe_ht25(seed=1)
    case.steps = steps
    return case


def time_form(case, form, launch, steps, warmup, tune_cache):
    from hemocell_gb300 import _lib as L
    hc = case.build(form=form, launch=launch)
    if tune_cache is not None:
        hc.autotune(tune_cache)
    hc.iterate(warmup)
    hc.sync()
    with ClockSampler() as cs:
        ms = hc.time_steps(steps)
    prof = hc.profile_stages(5)
    st = hc.stats()
    status = hc.device_status()
    tuning = hc.tuning()
    hc.close()
    return ms, prof, cs.summary(), st, status, tuning


def e2e_form(case, form, launch, steps, warmup):
    """Same metric through the public API with host buffers: every step the
    host sets the body force (setExternalVector) from host memory, iterates,
    and reads the vertex positions back into a pinned host buffer."""
    import torch
    from hemocell_gb300 import _lib as L
    hc = case.build(form=form, launch=launch)
    V = hc.stats().vertices
    pos = torch.empty((V, 3), dtype=torch.float64, pin_memory=True).numpy()
    body = np.array(case.body, np.float64)
    for _ in range(warmup):
        hc.setExternalVector(case.body_mode, body)
        hc.iterate(1)
        hc.read_positions(pos)
    t0 = time.perf_counter()
    for _ in range(steps):
        hc.setExternalVector(case.body_mode, body)
        hc.iterate(1)
        hc.read_positions(pos)
    dt = time.perf_counter() - t0
    hc.close()
    h2d = 3 * case.dims[2] * (4 if form == L.HC_FORM_MIXED_F32 else 8)
    d2h = V * 3 * 8
    return dt, h2d, d2h


def cpu_baseline(case, budget_s: float = 12.0, threads: int = 0):
    """FP64 CPU restatement (oracle/) on a bounded sample of the same workload."""
    from oracle import oracle as orc
    threads = threads or (os.cpu_count() or 1)
    o = orc.apply_case(case, threads=threads)
    t0 = time.perf_counter()
    o.step(1)
    one = time.perf_counter() - t0
    n = max(1, min(50, int(budget_s / max(one, 1e-3))))
    t0 = time.perf_counter()
    o.step(n)
    dt = time.perf_counter() - t0
    return case.N * n / dt / 1e6, n, threads


def run_reference(args):
    """--impl reference: the CPU restatement of the reference path, all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    case = build_case(args.steps)
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    o = orc.apply_case(case, threads=threads)
    t0 = time.perf_counter()
    o.step(args.warmup)
    per_step = (time.perf_counter() - t0) / max(args.warmup, 1)
    # bounded sample: at most ~60 s of CPU work whatever K is
    n = max(1, min(args.steps, int(60.0 / max(per_step, 1e-4))))
    t0 = time.perf_counter()
    o.step(n)
    dt = time.perf_counter() - t0
    mlups = case.N * n / dt / 1e6
    line = {
        "impl": "reference", "metric": "MLUPS incl. IBM+cell forces", "value": mlups, "unit": "MLUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / n * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "pipe_ht25 64x64x256, 279 RBC (642 vertices), 25% Ht", "nodes": case.N,
                   "vertices": case.nvertices, "form": "FP64 CPU restatement (oracle port)"},
        "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": f"{n} full steps of the workload (of {args.steps} requested) after "
                                   f"{args.warmup} warm-up"},
        "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 plain form")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    import __graft_entry__ as g
    g.build()
    from hemocell_gb300 import _lib as L
    case = build_case(args.steps)
    fluid = int((case.flags_array() == 0).sum())
    tune_cache = None if args.no_autotune else os.path.join(ROOT, "hemocell_gb300", "_build", "tuning.txt")

    if world > 1:
        torch.distributed.barrier()
    ms, prof, clocks, st, status, tuning = time_form(case, L.HC_FORM_MIXED_F32, L.HC_LAUNCH_BATCHED, args.steps,
                                                     args.warmup, tune_cache)
    ms_max = ms
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_max = float(t.item())
    value = world * case.N * args.steps / (ms_max * 1e3)
    peak, peak_kind = measured_peaks()
    k1_ms = prof["collide_stream"]
    k1_bytes = fluid * BYTES_NODE["f32"]
    achieved = k1_bytes / (k1_ms * 1e-3) / 1e9
    traffic = None if K1_TRAFFIC_PER_NODE["f32"] is None else K1_TRAFFIC_PER_NODE["f32"] * fluid
    step_bytes = fluid * BYTES_NODE["f32"] + st.vertices * BYTES_VERTEX["f32"]
    step_gbs = step_bytes / (ms / args.steps * 1e-3) / 1e9

    extra = {}
    if not args.no_plain:
        ms64, prof64, _, _, status64, tuning64 = time_form(case, L.HC_FORM_PLAIN_F64, L.HC_LAUNCH_PER_STAGE,
                                                          args.steps, args.warmup, tune_cache)
        mlups64 = case.N * args.steps / (ms64 * 1e3)
        extra["fp64_plain"] = {"value": mlups64, "unit": "MLUPS", "ms_per_step": ms64 / args.steps,
                               "stages_ms": prof64, "tuning": tuning64, "status": status64}
        extra["fp32_batched_over_fp64_plain"] = value / world / mlups64

    e2e_dt, h2d, d2h = e2e_form(case, L.HC_FORM_MIXED_F32, L.HC_LAUNCH_BATCHED, max(20, args.steps // 4),
                                args.warmup)
    e2e_steps = max(20, args.steps // 4)
    e2e_val = world * case.N * e2e_steps / e2e_dt / 1e6

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu_val, n_cpu, cores = cpu_baseline(case)
        cpu = {"value": cpu_val, "unit": "MLUPS", "cores": cores, "kind": "port",
               "sample": f"{n_cpu} full steps of the same workload (FP64 CPU restatement, OpenMP)"}

    if rank == 0:
        line = {
            "metric": "MLUPS incl. IBM+cell forces", "value": value, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "pipe_ht25 64x64x256 D3Q19, R=30 cylinder, 279 RBC (642 vertices), 25% Ht",
                       "form": "mixed FP32 populations f_i-w_i / FP64 positions+volume, batched + CUDA graph",
                       "nodes": case.N, "fluid_nodes": fluid, "vertices": st.vertices, "cells": st.cells,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "working set per step > 129 MB L2, no flush"},
            "fluid_mlups": world * fluid * args.steps / (ms_max * 1e3),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": "k_collide_stream<float>",
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": k1_bytes,
                         "launch_ms": k1_ms},
            "step_roofline": {"bytes_per_step": step_bytes, "achieved_gbs": step_gbs, "frac": step_gbs / peak},
            "stages_ms": prof,
            "clocks": clocks,
            "e2e": {"value": e2e_val, "unit": "MLUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": 4 * args.steps,
            "cpu_baseline": cpu,
            "tuning": tuning,
            "device_status": status,
        }
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
