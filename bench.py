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
exactly K steps after W warm-up steps, that K-step region repeated until the
repeats span at least half a second (the line reports the median, with the
clock samples of the whole window); the per-step working set (~190 MB in
FP32, ~370 MB in FP64) exceeds the 129 MB L2, so no flush is inserted.
"""
from __future__ import annotations

import os

# the serving leg runs up to 64 solves on their own streams: give the device
# enough hardware queues that they do not serialise (read at context creation)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import argparse
import json
import math
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
# node velocity: 19 populations pulled, the force and the mask read, the
# velocity written (float4 in FP32, three doubles in FP64)
BYTES_NODE_VELOCITY = {"f32": 19 * 4 + 16 + 4 + 16, "f64": 19 * 8 + 24 + 4 + 24}
PIPE_WORKLOAD = ("pipe_ht25 64x64x256 D3Q19, R=30 cylinder, 279 RBC (642 vertices, 81 um^3 each), 25% Ht "
                 "of the lumen by mesh volume")
# The reference's `Volume` key (90 um^3, examples/oneCellShear/RBC.xml) is read
# by no code; its own haematocrit printouts count 77 um^3 per RBC
# (cases/performance_testing/performance_testing.cpp:122).  The Evans-Fung
# shape of R = 3.91 um encloses 81.76 um^3 and its 1280-face mesh 81.05 um^3,
# which sets the pipe's 279 cells (about 250 at 90 um^3).
RBC_VOLUME_NOTE = "RBC 81.05 um^3 (Evans-Fung mesh, R=3.91 um); 279 cells, ~250 at the unused Volume key's 90 um^3"
PROFILE_TRAFFIC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                               "step_kernels_pipe_ht25_64x64x256.md")


def profiled_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` (dram__bytes_read.sum +
    dram__bytes_write.sum inside graph-replayed pipe steps) from the committed
    ncu summary, whose lines "TRAFFIC <kernel> <bytes> <commit>" state the
    source commit; None when the summary has no such line."""
    try:
        with open(PROFILE_TRAFFIC) as fh:
            for line in fh:
                parts = line.split()
                if len(parts) >= 3 and parts[0] == "TRAFFIC" and parts[1] == kernel:
                    return float(parts[2]), (parts[3] if len(parts) > 3 else None)
    except OSError:
        pass
    return None, None


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def smi_id(local: int) -> str:
    """nvidia-smi's id of CUDA device `local` of this process: its entry of
    CUDA_VISIBLE_DEVICES (an index or a UUID) when that is set."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").strip()
    if vis:
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if local < len(ids):
            return ids[local]
    return str(local)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self, index=None):
        self.index = smi_id(int(os.environ.get("LOCAL_RANK", "0"))) if index is None else index
        self.samples = []
        self.proc = None

    def wait_first(self, timeout: float = 3.0):
        """Block until the first sample has arrived (nvidia-smi takes a moment
        to start), so that the samples cover the timed window."""
        t0 = time.perf_counter()
        while self.proc and not self.samples and time.perf_counter() - t0 < timeout:
            time.sleep(0.01)
        return self

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
                "reasons": reasons, "samples": len(self.samples), "timed_repeats": getattr(self, "repeats", None)}


def build_case(steps: int):
    from hemocell_gb300 import cases
    case = cases.pipe_ht25(seed=1)
    case.steps = steps
    return case


MIN_SPAN_S = 0.5


def repeat_timed(fn, min_span_s: float = MIN_SPAN_S, min_repeats: int = 3, max_repeats: int = 100000):
    """Run fn() (which times one K-step region and returns its ms) until the
    repeats span min_span_s of wall time; returns the list of timings."""
    out = []
    t0 = time.perf_counter()
    while len(out) < max_repeats:
        out.append(fn())
        if len(out) >= min_repeats and time.perf_counter() - t0 >= min_span_s:
            break
    return out


def time_form(case, form, launch, steps, warmup, tune_cache):
    """Median device time (ms) of `steps` steps over repeats spanning half a
    second, with the clock samples of that window."""
    from hemocell_gb300 import _lib as L
    hc = case.build(form=form, launch=launch)
    if tune_cache is not None:
        hc.autotune(tune_cache)
    hc.iterate(warmup)
    hc.sync()
    with ClockSampler() as cs:
        cs.wait_first()
        reps = repeat_timed(lambda: hc.time_steps(steps))
    ms = statistics.median(reps)
    cs.repeats = len(reps)
    # each kernel's device time inside the step as the graph runs it (events
    # on the handle's stream, launches queued ahead of the GPU)
    prof = hc.profile_kernels(200)
    st = hc.stats()
    status = hc.device_status()
    tuning = hc.tuning()
    hc.close()
    return ms, prof, cs.summary(), st, status, tuning


def e2e_form(case, form, launch, steps, warmup, tune_cache=None):
    """Same metric through the public API with host buffers: every step the
    host sets the body force (setExternalVector, which copies the per-plane
    profile to the device from pinned memory), iterates, and starts copying
    the positions into one of two pinned host buffers; the copy of step k
    runs on its own stream during step k+1, and the host waits for it before
    that buffer is used again (the last one is waited for inside the timed
    region too)."""
    import torch
    from hemocell_gb300 import _lib as L
    hc = case.build(form=form, launch=launch)
    if tune_cache is not None:
        hc.autotune(tune_cache)         # the launch shapes the device-timed leg runs with
    V = hc.stats().vertices
    pos = [torch.empty((V, 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
    body = np.array(case.body, np.float64)

    def run(n):
        for k in range(n):
            hc.setExternalVector(case.body_mode, body)
            hc.iterate(1)
            hc.read_positions_async(pos[k & 1], k & 1)
            if k >= 1:
                hc.wait_positions((k - 1) & 1)
        hc.wait_positions((n - 1) & 1)

    run(warmup)

    def one():
        t0 = time.perf_counter()
        run(steps)
        return time.perf_counter() - t0

    dt = statistics.median(repeat_timed(one))
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


def max_over_ranks(x: float) -> float:
    """Largest x over the ranks of the process group (x itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_mlups(world: int, nodes: int, steps: int, ms_max: float) -> float:
    """Whole-job MLUPS of `world` independent replicas timed by the slowest."""
    return world * nodes * steps / (ms_max * 1e3)


def rel_l2(a, b) -> float:
    d = np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    n = np.linalg.norm(np.asarray(b, np.float64))
    return float(d / n) if n > 0 else float(d)


def mixed_error_leg(case, steps: int = 2000, every: int = 100):
    """The mixed FP32 form against the FP64 plain form (which matches the FP64
    oracle within 1e-10) on the same workload: velocity and density relative
    L2 over the fluid, and per-cell volume difference, every `every` steps."""
    from hemocell_gb300 import _lib as L
    a = case.build(form=L.HC_FORM_MIXED_F32, launch=L.HC_LAUNCH_BATCHED)
    b = case.build(form=L.HC_FORM_PLAIN_F64, launch=L.HC_LAUNCH_BATCHED)
    fluid = case.flags_array() == 0
    _, v0 = b.read_cells()
    rec = {"steps": [], "u_rel_l2": [], "rho_rel_l2": [], "volume_rel_max": [], "volume_drift_f32": [],
           "volume_drift_f64": []}
    for k in range(every, steps + 1, every):
        a.iterate(every)
        b.iterate(every)
        ra, ua = a.read_fluid()
        rb, ub = b.read_fluid()
        _, va = a.read_cells()
        _, vb = b.read_cells()
        rec["steps"].append(k)
        rec["u_rel_l2"].append(rel_l2(ua[:, fluid], ub[:, fluid]))
        rec["rho_rel_l2"].append(rel_l2(ra[fluid], rb[fluid]))
        rec["volume_rel_max"].append(float(np.max(np.abs(va - vb) / v0)))
        rec["volume_drift_f32"].append(float(np.max(np.abs(va - v0) / v0)))
        rec["volume_drift_f64"].append(float(np.max(np.abs(vb - v0) / v0)))
    a.close()
    b.close()
    return rec


def kolmogorov_leg(steps: int, warmup: int, tune_cache):
    """128^3 periodic cube, Kolmogorov forcing, 30% RBC volume fraction with
    platelets (1 per 10 RBC) and 2 WBC: MLUPS of both forms, batched."""
    from hemocell_gb300 import _lib as L
    from hemocell_gb300 import cases
    t0 = time.perf_counter()
    case = cases.kolmogorov_mix(n=128, seed=1)
    pack_s = time.perf_counter() - t0
    out = {"workload": "kolmogorov_128: 128^3 periodic, F_x = A sin(2 pi z/128), 30% RBC (642 vertices), "
                       "PLT (162 vertices) 1 per 10 RBC, 2 WBC (2562 vertices)",
           "cells": len(case.cells), "vertices": case.nvertices, "packing_s": pack_s}
    peak, _ = measured_peaks()
    for name, form in (("fp32_batched", L.HC_FORM_MIXED_F32), ("fp64_batched", L.HC_FORM_PLAIN_F64)):
        ms, prof, clocks, st, status, tuning = time_form(case, form, L.HC_LAUNCH_BATCHED, steps, warmup,
                                                         tune_cache)
        out[name] = {"value": case.N * steps / (ms * 1e3), "unit": "MLUPS", "ms_per_step": ms / steps,
                     "kernels_ms": prof, "tuning": tuning, "status": status, "clocks": clocks}
        # the collide-stream on a lattice without walls (every node fluid)
        k1_bytes = case.N * BYTES_NODE["f32" if form == L.HC_FORM_MIXED_F32 else "f64"]
        gbs = k1_bytes / (prof["collide_stream"] * 1e-3) / 1e9
        out[name]["collide_stream_roofline"] = {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                                                "algorithmic_bytes_per_launch": k1_bytes}
    out["fp32_over_fp64"] = out["fp32_batched"]["value"] / out["fp64_batched"]["value"]
    out["_case"] = case
    return out


def timescale_leg(steps: int, warmup: int):
    """The pipe with the RBC mechanics every 20 steps and the velocity update
    every step (stepMaterialEvery = 20 of the reference's performance-testing
    configurations): FP32 batched, whole 20-step cycles replayed as one graph."""
    from hemocell_gb300 import _lib as L
    from hemocell_gb300 import cases
    case = cases.pipe_ht25(seed=1)
    hc = case.build(form=L.HC_FORM_MIXED_F32, launch=L.HC_LAUNCH_BATCHED)
    hc.setMaterialTimeScaleSeparation([20], velocity_every=1)
    hc.iterate(max(warmup, 40))
    hc.sync()
    n = max(40, steps // 20 * 20)
    ms = hc.time_steps(n)
    status = hc.device_status()
    hc.close()
    return {"workload": "pipe_ht25 64x64x256, 279 RBC, RBC mechanics every 20 steps", "steps": n,
            "value": case.N * n / (ms * 1e3), "unit": "MLUPS", "ms_per_step": ms / n, "status": status}


def small_box_kernels():
    """Per-kernel device times of one small solve (32^3 box, one RBC) in the
    three forms: why batching raises FP64 throughput less than FP32's."""
    from hemocell_gb300 import _lib as L
    from hemocell_gb300 import serving as S
    r = S.Request(id=0, arrival=0.0, n=32, n_rbc=1, shear_rate=200.0, stiffness=1.0, steps=500, seed=7)
    s = S.Solve(r)
    out = {"box": "32^3 sheared box, one RBC (642 vertices)", "nodes": 32 ** 3}
    for name, form in (("f32_batched", L.HC_FORM_MIXED_F32), ("f64_batched", L.HC_FORM_PLAIN_F64)):
        hc = s.build(form, L.HC_LAUNCH_BATCHED)
        hc.iterate(10)
        out[name + "_kernels_ms"] = hc.profile_kernels(100)
        hc.close()
    hc = s.build(L.HC_FORM_PLAIN_F64, L.HC_LAUNCH_PER_STAGE)
    hc.iterate(10)
    out["f64_per_stage_ms_per_step"] = hc.time_steps(100) / 100
    hc.close()
    return out


def serving_leg(args, fp64_pipe_mlups=None):
    """Continuous batching of the streams of independent sheared-box solves
    (box edge 32-96, 1-8 RBC, 500-5000 steps, Poisson arrivals at 200/s),
    seeds 1, 2 and 3: per seed, the same requests served one at a time in the
    plain FP64 form, and batched in FP32 and in FP64; then the seed-1 stream
    saturated (FP32) and at half the measured capacity."""
    import torch
    from hemocell_gb300 import _lib as L
    from hemocell_gb300 import serving as S
    free, _ = torch.cuda.mem_get_info()
    budget = int(min(0.5 * free, 64 << 30))

    def trim(d):
        return {k: v for k, v in d.items() if k != "results"}

    per_seed = {}
    for seed in ((1, 2, 3) if args.serve_solo > 0 else ()):
        stream = S.request_stream(seed=seed, rate=200.0, count=10000)
        reqs = stream[:args.serve_solo]
        solves = {r.id: S.Solve(r) for r in reqs}        # geometry and packing, outside the clock
        kw = dict(budget_bytes=budget, max_slots=64, chunk_steps=50, solves=solves)
        solo = S.solo(reqs, L.HC_FORM_PLAIN_F64, L.HC_LAUNCH_PER_STAGE, solves=solves)
        b32 = S.serve(reqs, L.HC_FORM_MIXED_F32, **kw)
        b64 = S.serve(reqs, L.HC_FORM_PLAIN_F64, **kw)
        per_seed[str(seed)] = {"requests": len(reqs), "solo_plain_f64": trim(solo), "batched_f32": trim(b32),
                               "batched_f64": trim(b64),
                               "speedup_f32_vs_solo": b32["solves_per_s"] / solo["solves_per_s"],
                               "speedup_f64_vs_solo": b64["solves_per_s"] / solo["solves_per_s"]}
    # the saturated FP32 stream of each seed asked for (the first n requests of
    # the seed's 10,000), then the first seed's stream at half its capacity
    seeds = [int(x) for x in str(args.serve_seeds).split(",") if x.strip()]
    sat_by_seed, sub32, rate_sub = {}, None, None
    for k, seed in enumerate(seeds):
        stream = S.request_stream(seed=seed, rate=200.0, count=10000)
        head = stream[:args.serve_requests]
        solves = {r.id: S.Solve(r) for r in head}
        kw = dict(budget_bytes=budget, max_slots=64, chunk_steps=50, solves=solves)
        sat_by_seed[str(seed)] = trim(S.serve(head, L.HC_FORM_MIXED_F32, **kw))
        if k == 0:
            rate_sub = 0.5 * sat_by_seed[str(seed)]["solves_per_s"]
            sub = S.with_arrivals(head[: max(8, args.serve_requests // 3)], rate_sub, seed=2)
            sub32 = S.serve(sub, L.HC_FORM_MIXED_F32, **kw)
        del solves, kw
    small = small_box_kernels()
    geo = lambda k: (math.exp(sum(math.log(per_seed[s][k]) for s in per_seed) / len(per_seed))
                     if per_seed else None)
    out = {
        "workload": "independent sheared boxes, edge U{32,48,64,96}, 1-8 RBC (642 vertices), shear 50-500/s, "
                    "kLink/kBend x log-U(0.5,5), 500-5000 steps; Poisson arrivals at 200/s",
        "budget_bytes": budget, "max_slots": 64, "chunk_steps": 50,
        "per_seed": per_seed,
        "speedup_f32_vs_solo_geomean": geo("speedup_f32_vs_solo"),
        "speedup_f64_vs_solo_geomean": geo("speedup_f64_vs_solo"),
        "saturated_f32_200_per_s": dict(sat_by_seed[str(seeds[0])], seed=seeds[0]),
        "subsaturated_f32": dict(trim(sub32), offered_rate_target=rate_sub, seed=seeds[0]),
        "small_box": small,
    }
    if len(seeds) > 1:
        out["saturated_f32_by_seed"] = sat_by_seed
    if fp64_pipe_mlups:
        # the FP64 arithmetic bound: the pipe's FP64 form keeps the FP64 pipe
        # busy, so no mix of solves steps FP64 lattices much faster than that
        solo_mlups = [per_seed[s]["solo_plain_f64"]["mlups"] for s in per_seed]
        out["fp64_note"] = {"fp64_pipe_mlups": fp64_pipe_mlups, "solo_plain_f64_mlups": solo_mlups,
                            "ceiling_over_solo": [fp64_pipe_mlups / m for m in solo_mlups]}
    return out


def step_kernel_names(tuning) -> dict:
    """The FP32 kernels that the tuned batched step launches, by `hc_profile_kernels`' keys."""
    kind = tuning[7] & 0xFF
    cs = "k_collide_stream<float>" if kind == 0 else ("k_collide_stream_fluid<float>" if kind == 1
                                                       else "k_collide_stream_bulk<float>")
    nv = {0x000: "k_node_velocity<float>", 0x100: "k_node_velocity_fluid<float>",
          0x200: "k_node_velocity_packed<float>", 0x300: "k_node_velocity_dense<float>"}[tuning[7] & 0x300]
    mech = {1: "k_mechanics_scatter<float>", 2: "k_mechanics_staged<float>"}.get(tuning[6], "k_mechanics<float>")
    return {"collide_stream": cs, "node_velocity": nv, "mechanics": mech}


def pipe_config(case, nvertices: int) -> dict:
    """The `config` of both arms: the workload only (the arithmetic of each
    arm is in its top-level `form`)."""
    return {"workload": PIPE_WORKLOAD, "nodes": case.N, "fluid_nodes": int((case.flags_array() == 0).sum()),
            "vertices": nvertices, "cells": len(case.cells), "rbc_volume": RBC_VOLUME_NOTE,
            "l2": "working set per step > 129 MB L2, no flush"}


def run_reference(args):
    """--impl reference: the CPU restatement of the reference path, all host
    threads.  The workload (meshes, placement, packing) is built by the
    oracle's own geometry, so this arm loads no part of the GPU library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as orc
    from hemocell_gb300 import cases
    case = cases.pipe_ht25(seed=1, geo=orc.geometry)
    case.steps = args.steps
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
        "config": pipe_config(case, case.nvertices),
        "form": "FP64 CPU restatement of the step (oracle port), OpenMP over all host threads",
        "native_libraries": sorted({os.path.basename(l.split()[-1]) for l in open("/proc/self/maps")
                                    if l.rstrip().endswith(".so") and ROOT in l}),
        "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": f"{n} full steps of the workload (of {args.steps} requested) after "
                                   f"{args.warmup} warm-up"},
        "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 plain form")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-stream leg")
    ap.add_argument("--no-kolmogorov", action="store_true", help="skip the 128^3 suspension leg")
    ap.add_argument("--no-mixed-error", action="store_true", help="skip the FP32-vs-FP64 error report")
    ap.add_argument("--serve-requests", type=int, default=96, help="requests of the saturated FP32 stream")
    ap.add_argument("--serve-seeds", default="1", help="seeds of the saturated FP32 stream, comma-separated")
    ap.add_argument("--serve-solo", type=int, default=12, help="requests run one at a time (and batched) "
                                                                 "for the speed-up")
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
    from hemocell_gb300 import hemocell as _hc
    _hc.set_default_device(local)   # every handle and batch of this rank on its own GPU

    import __graft_entry__ as g
    if world > 1:
        # one rank compiles; the others find the objects up to date
        if rank == 0:
            g.build()
        torch.distributed.barrier()
    g.build()
    from hemocell_gb300 import _lib as L
    case = build_case(args.steps)
    fluid = int((case.flags_array() == 0).sum())
    tune_cache = None if args.no_autotune else os.path.join(ROOT, "hemocell_gb300", "_build", "tuning.txt")

    if world > 1:
        torch.distributed.barrier()
    ms, prof, clocks, st, status, tuning = time_form(case, L.HC_FORM_MIXED_F32, L.HC_LAUNCH_BATCHED, args.steps,
                                                     args.warmup, tune_cache)
    ms_max = max_over_ranks(ms)
    value = replicas_mlups(world, case.N, args.steps, ms_max)
    peak, peak_kind = measured_peaks()
    step_bytes = fluid * BYTES_NODE["f32"] + st.vertices * BYTES_VERTEX["f32"]
    step_gbs = step_bytes / (ms / args.steps * 1e-3) / 1e9
    # each kernel of the step against HBM: algorithmic bytes of one launch over
    # its live time inside the step
    kernel_bytes = {"collide_stream": fluid * BYTES_NODE["f32"],
                    "node_velocity": fluid * BYTES_NODE_VELOCITY["f32"],
                    "mechanics": st.vertices * BYTES_VERTEX["f32"]}
    kernel_names = step_kernel_names(tuning)
    kernels = {}
    for k, b in kernel_bytes.items():
        gbs = b / (prof[k] * 1e-3) / 1e9
        tr, tr_commit = profiled_traffic(kernel_names[k])
        kernels[k] = {"kernel": kernel_names[k], "launch_ms": prof[k], "share": prof[k] / prof["step"],
                      "algorithmic_bytes_per_launch": b, "achieved_gbs": gbs, "frac": gbs / peak,
                      "traffic": tr, "traffic_commit": tr_commit}
    dominant = max(kernel_bytes, key=lambda k: prof[k])
    dom = kernels[dominant]

    extra = {}
    if not args.no_plain:
        ms64, prof64, clocks64, _, status64, tuning64 = time_form(case, L.HC_FORM_PLAIN_F64, L.HC_LAUNCH_PER_STAGE,
                                                                  args.steps, args.warmup, tune_cache)
        mlups64 = case.N * args.steps / (ms64 * 1e3)
        extra["fp64_plain"] = {"value": mlups64, "unit": "MLUPS", "ms_per_step": ms64 / args.steps,
                               "launch": "per stage", "kernels_ms": prof64, "tuning": tuning64,
                               "status": status64, "clocks": clocks64}
        extra["fp32_batched_over_fp64_plain"] = value / world / mlups64
        # the precision-matched form: FP64 batched (graph), on the device and
        # through the public API with host copies
        msb, profb, clocksb, _, statusb, tuningb = time_form(case, L.HC_FORM_PLAIN_F64, L.HC_LAUNCH_BATCHED,
                                                             args.steps, args.warmup, tune_cache)
        e64_dt, e64_h2d, e64_d2h = e2e_form(case, L.HC_FORM_PLAIN_F64, L.HC_LAUNCH_BATCHED, args.steps,
                                            args.warmup, tune_cache)
        extra["fp64_batched"] = {
            "value": case.N * args.steps / (msb * 1e3), "unit": "MLUPS", "ms_per_step": msb / args.steps,
            "kernels_ms": profb, "tuning": tuningb, "status": statusb, "clocks": clocksb,
            "e2e": {"value": case.N * args.steps / e64_dt / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": e64_h2d,
                    "d2h_bytes_per_step": e64_d2h}}

    e2e_dt, h2d, d2h = e2e_form(case, L.HC_FORM_MIXED_F32, L.HC_LAUNCH_BATCHED, args.steps, args.warmup,
                                tune_cache)
    e2e_val = world * case.N * args.steps / e2e_dt / 1e6

    if not args.no_mixed_error:
        extra["mixed_vs_fp64"] = mixed_error_leg(case)
    extra["materials_every_20"] = timescale_leg(min(args.steps, 2000), args.warmup)
    if not args.no_kolmogorov:
        extra["kolmogorov"] = kolmogorov_leg(min(args.steps, 1000), args.warmup, tune_cache)
    if not args.no_serving:
        extra["serving"] = serving_leg(args, extra.get("fp64_batched", {}).get("value"))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu_val, n_cpu, cores = cpu_baseline(case)
        cpu = {"value": cpu_val, "unit": "MLUPS", "cores": cores, "kind": "port",
               "sample": f"{n_cpu} full steps of the same workload (FP64 CPU restatement, OpenMP)",
               "label": "CPU restatement of HemoCell (not the HemoCell binary)", "cpu": cpu_model()}
        # the other configurations, bounded slices
        from hemocell_gb300 import cases
        shear = cases.shear_single_rbc(n=50, shear_rate=100.0, seed=1)
        v0, n0, _ = cpu_baseline(shear, budget_s=4.0)
        cpu["shear_rbc_50"] = {"value": v0, "unit": "MLUPS", "sample": f"{n0} steps of the 50^3 sheared RBC"}
        if "kolmogorov" in extra and "_case" in extra["kolmogorov"]:
            v3, n3, _ = cpu_baseline(extra["kolmogorov"]["_case"], budget_s=8.0)
            cpu["kolmogorov_128"] = {"value": v3, "unit": "MLUPS", "sample": f"{n3} steps of the 128^3 suspension"}
    if "kolmogorov" in extra:
        extra["kolmogorov"].pop("_case", None)
    if cpu is not None and "fp64_batched" in extra:
        # like for like: the same FP64 arithmetic on the GPU and on the host cores
        fb = extra["fp64_batched"]
        fb["over_cpu"] = fb["value"] / cpu["value"]
        fb["e2e_over_cpu"] = fb["e2e"]["value"] / cpu["value"]

    if rank == 0:
        line = {
            "metric": "MLUPS incl. IBM+cell forces", "value": value, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": pipe_config(case, st.vertices),
            "form": "mixed FP32 populations f_i-w_i / FP64 positions+volume, batched + CUDA graph",
            "parallelism": "replicas" if world > 1 else "single",
            "fluid_mlups": world * fluid * args.steps / (ms_max * 1e3),
            # the dominant kernel of the step (the largest live time)
            "roofline": {"bound": "hbm", "achieved": dom["achieved_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": dom["frac"], "traffic": dom["traffic"], "kernel": dom["kernel"],
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": dom["algorithmic_bytes_per_launch"],
                         "launch_ms": dom["launch_ms"], "share_of_step": dom["share"]},
            "kernels_roofline": kernels,
            "step_roofline": {"bytes_per_step": step_bytes, "achieved_gbs": step_gbs, "frac": step_gbs / peak,
                              # N (all nodes) x 176 B + V x 72 B per step
                              "frac_all_nodes": (case.N * BYTES_NODE["f32"] + st.vertices * 72) /
                                                (ms / args.steps * 1e-3) / 1e9 / peak},
            "kernels_ms": prof,
            "clocks": clocks,
            "e2e": {"value": e2e_val, "unit": "MLUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            # per step: collide-stream, node velocity, force assembly (with the
            # next spread, and interpolation + advance unless bit 11 of tune[7]
            # keeps them a kernel of their own)
            "gpu_launches": (4 if tuning[7] & 0x800 else 3) * args.steps,
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
