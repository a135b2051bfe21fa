"""Serving loop: a stream of independent single-cell shear solves run with
continuous batching on one device (hc_batch_*), against the same stream run
one solve at a time.

A request is a sheared box of edge n in {32, 48, 64, 96} lattice nodes with
1-8 RBCs (642 vertices), a wall shear rate in 50-500 1/s, kLink and kBend
scaled by one log-uniform factor in 0.5-5 and 500-5000 steps; requests arrive
as a Poisson process.  The server admits arrived requests first come first
served while their estimated device bytes fit the batch's budget and a slot
is free, so requests that arrive while others are on the GPU join as memory
frees up; every resident solve is stepped concurrently on its own stream.
Latency is completion minus arrival.  There is no counterpart in the
reference, which runs one simulation per MPI job.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, replace
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _lib as L
from . import cases
from .hemocell import Batch, HemoCell, Material, estimate_device_bytes, pack_cells, place_cells

BOX_EDGES = (32, 48, 64, 96)


@dataclass(frozen=True)
class Request:
    id: int
    arrival: float      # seconds after the start of the stream
    n: int              # box edge (lattice nodes)
    n_rbc: int
    shear_rate: float   # 1/s
    stiffness: float    # factor on kLink and kBend
    steps: int
    seed: int


def request_stream(seed: int, rate: float, count: int) -> List[Request]:
    """Seeded Poisson arrivals at `rate` per second with the request mix above."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(count):
        out.append(Request(id=i, arrival=float(arrivals[i]), n=int(rng.choice(BOX_EDGES)),
                           n_rbc=int(rng.integers(1, 9)), shear_rate=float(rng.uniform(50.0, 500.0)),
                           stiffness=float(math.exp(rng.uniform(math.log(0.5), math.log(5.0)))),
                           steps=int(rng.integers(500, 5001)), seed=int(rng.integers(1, 2 ** 31))))
    return out


def with_arrivals(reqs: Sequence[Request], rate: float, seed: int) -> List[Request]:
    """The same requests re-timed as a Poisson process of another rate."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    t = np.cumsum(gaps) - gaps[0]
    return [replace(r, arrival=float(t[i])) for i, r in enumerate(reqs)]


_RBC = {}


def _rbc():
    if "t" not in _RBC:
        _RBC["t"] = cases.rbc_type(600)
    return _RBC["t"]


class Solve:
    """Set-up of one request: geometry, walls, material and packed cells."""

    def __init__(self, req: Request):
        t = _rbc()
        n = req.n
        self.req = req
        self.dims = (n, n, n)
        self.flags, self.walls = cases.shear_walls(self.dims, req.shear_rate)
        m = t.material
        self.material = Material(kLink=m.kLink * req.stiffness, kBend=m.kBend * req.stiffness, kVolume=m.kVolume,
                                 kArea=m.kArea, eta_m=m.eta_m, radius=m.radius)
        centres, angles, _ = pack_cells(self.dims, (1, 1, 0), self.flags, [t.mesh], [req.n_rbc], margin=0.5,
                                        seed=req.seed)
        self.xyz = place_cells(t.mesh, centres, angles)
        self.n_cells = int(centres.shape[0])
        self.nvertices = int(self.xyz.shape[0])

    def bytes(self, form: int) -> int:
        return estimate_device_bytes(self.dims, form, self.nvertices, self.n_cells)

    def build(self, form: int, launch: int) -> HemoCell:
        t = _rbc()
        hc = HemoCell(*self.dims, periodic=(1, 1, 0), dx=cases.DX, dt=cases.DT, rho_p=cases.RHO_P,
                      kBT_p=cases.KBT, tau=1.0, form=form, launch=launch)
        hc.set_flags(self.flags)
        for cls, u in self.walls.items():
            hc.set_wall_velocity(cls, u)
        hc.latticeEquilibrium(1.0)
        hc.addCellType(t.name, t.model, self.material, t.mesh)
        if self.n_cells:
            hc.add_cells_xyz(0, self.xyz)
        return hc


def read_result(hc: HemoCell, fluid: bool = False) -> Dict[str, np.ndarray]:
    out = {"x": hc.read_positions()}
    if fluid:
        _, u = hc.read_fluid()
        out["u"] = u
    return out


def fifo_latencies(arrivals: Sequence[float], service: Sequence[float]):
    """Latencies of a single FIFO server with the given service times, and the
    time its last job ends."""
    end = arrivals[0] if len(arrivals) else 0.0
    lat = []
    for a, d in zip(arrivals, service):
        end = max(end, a) + d
        lat.append(end - a)
    return lat, end


def _percentiles(lat: Sequence[float]) -> dict:
    a = np.asarray(lat, np.float64)
    if a.size == 0:
        return {"p50_s": None, "p99_s": None, "mean_s": None}
    return {"p50_s": float(np.percentile(a, 50)), "p99_s": float(np.percentile(a, 99)), "mean_s": float(a.mean())}


def serve(reqs: Sequence[Request], form: int, budget_bytes: int, max_slots: int = 64, chunk_steps: int = 50,
          launch: int = L.HC_LAUNCH_BATCHED, keep_results: bool = False, fluid: bool = False,
          solves: Optional[Dict[int, Solve]] = None) -> dict:
    """Run the stream in real time with continuous batching; every request
    runs to completion.  Returns throughput, latencies and, if asked, each
    request's final state."""
    solves = {} if solves is None else solves
    for r in reqs:                       # host set-up of geometry and packing, before the clock
        if r.id not in solves:
            solves[r.id] = Solve(r)
    batch = Batch(budget_bytes, max_slots=max_slots, chunk_steps=chunk_steps)
    pending = deque(sorted(reqs, key=lambda r: r.arrival))
    by_id = {r.id: r for r in reqs}
    lat, done_at, admitted_at, results = {}, {}, {}, {}
    node_steps = 0
    peak_resident = 0
    t0 = time.perf_counter()
    try:
        in_flight = 0
        while pending or in_flight:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                r = pending[0]
                s = solves[r.id]
                if not batch.fits(s.bytes(form)):
                    break
                hc = s.build(form, launch)
                if not batch.admit(hc, r.steps, r.id):
                    hc.close()
                    break
                pending.popleft()
                admitted_at[r.id] = time.perf_counter() - t0
                in_flight += 1
            peak_resident = max(peak_resident, in_flight)
            wait = 2.0
            if pending and in_flight == 0:
                wait = max(0.0, (pending[0].arrival - (time.perf_counter() - t0)) * 1e3)
            if in_flight:
                batch.pump(min(wait, 2.0))
            elif wait > 0:
                time.sleep(min(wait, 2.0) / 1e3)
            while True:
                got = batch.pop()
                if got is None:
                    break
                tag, hc, status = got
                if status != L.HC_OK:
                    raise RuntimeError(f"request {tag} failed: {hc._lib.hc_last_error(hc._h).decode()}")
                res = read_result(hc, fluid) if keep_results else {"x": hc.read_positions()}
                t_done = time.perf_counter() - t0
                batch.release(hc)
                in_flight -= 1
                r = by_id[tag]
                done_at[tag] = t_done
                lat[tag] = t_done - r.arrival
                node_steps += r.n ** 3 * r.steps
                if keep_results:
                    results[tag] = res
        stats = batch.stats()
    finally:
        batch.close()
    first = min(r.arrival for r in reqs)
    makespan = max(done_at.values()) - first
    out = {"requests": len(reqs), "completed": len(done_at), "solves_per_s": len(done_at) / makespan,
           "makespan_s": makespan, "mlups": node_steps / makespan / 1e6, "peak_resident": peak_resident,
           "offered_rate": (len(reqs) - 1) / max(1e-9, max(r.arrival for r in reqs) - first),
           "refused_admissions": stats["refused"], **_percentiles(list(lat.values()))}
    if keep_results:
        out["results"] = results
    return out


def solo(reqs: Sequence[Request], form: int = L.HC_FORM_PLAIN_F64, launch: int = L.HC_LAUNCH_PER_STAGE,
         keep_results: bool = False, fluid: bool = False, solves: Optional[Dict[int, Solve]] = None) -> dict:
    """The same stream served one solve at a time (FIFO, one server).  Each
    solve is set up, stepped and read back alone; its service time is
    measured, and the queue is replayed on those times (a single server's
    completions do not depend on idle waiting, so none is slept)."""
    solves = {} if solves is None else solves
    order = sorted(reqs, key=lambda r: r.arrival)
    service, results = {}, {}
    node_steps = 0
    for r in order:
        s = solves.get(r.id) or Solve(r)
        t = time.perf_counter()
        hc = s.build(form, launch)
        hc.iterate(r.steps)
        res = read_result(hc, fluid) if keep_results else {"x": hc.read_positions()}
        hc.close()
        service[r.id] = time.perf_counter() - t
        node_steps += r.n ** 3 * r.steps
        if keep_results:
            results[r.id] = res
    lat, end = fifo_latencies([r.arrival for r in order], [service[r.id] for r in order])
    makespan = end - order[0].arrival
    out = {"requests": len(order), "completed": len(order), "solves_per_s": len(order) / makespan,
           "makespan_s": makespan, "mlups": node_steps / makespan / 1e6,
           "busy_s": float(sum(service.values())), **_percentiles(lat)}
    if keep_results:
        out["results"] = results
    return out
