"""Generates the golden fixtures in this folder from the FP64 CPU oracle.

The reference (HemoCell on Palabos, MPI and HDF5) cannot be built here and
ships no golden vectors or known-answer tests, so these dumps of the oracle
are the pins: the oracle is checked against them on every CPU run
(tests/test_golden.py), and the GPU plain form against them on the GPU
(tests/test_gpu_golden.py).  Regenerate only when the restated algorithm
changes on purpose:

    python tests/golden/make_golden.py            # stage dumps, 50^3 shear (1000 steps), 64^3 suspension (300)
    python tests/golden/make_golden.py --pipe     # also the 64x64x256 pipe, 2000 steps (minutes)

Every input comes from the seeded builders in hemocell_gb300.cases, run
with the oracle's own geometry (meshes, placement, packing: oracle/geometry.cpp),
so no part of a fixture comes from the product library; only outputs are
stored.  Large floating-point arrays are rounded to 40 mantissa bits (a
relative change of at most 2^-41, about 5e-13) and stored byte-shuffled (the
eight bytes of each double in eight planes) before compression, which keeps
the full-field dumps of the larger runs to a few MB.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hemocell_gb300 import cases  # noqa: E402
from oracle import oracle as orc  # noqa: E402

STAGE_FILE = os.path.join(HERE, "stages_mixed_box.npz")
SHEAR_FILE = os.path.join(HERE, "shear_rbc_50_1000.npz")
PIPE_FILE = os.path.join(HERE, "pipe_ht25_2000.npz")
SUSPENSION_FILE = os.path.join(HERE, "kolmogorov_64_300.npz")
GEO = orc.geometry


KEEP_BITS = 40   # mantissa bits kept in the large arrays: 2^-41 relative, far below the tolerances


def save(path: str, d: dict) -> None:
    """np.savez_compressed, with the float64 arrays of more than 64 values
    rounded to KEEP_BITS mantissa bits and byte-shuffled."""
    out = {}
    drop = 52 - KEEP_BITS
    for k, v in d.items():
        v = np.asarray(v)
        if v.dtype == np.float64 and v.size > 64:
            bits = np.ascontiguousarray(v).reshape(-1).view(np.uint64)
            bits = (bits + np.uint64(1 << (drop - 1))) & ~np.uint64((1 << drop) - 1)
            out["shuffled__" + k] = np.ascontiguousarray(bits.view(np.uint8).reshape(-1, 8).T)
            out["shape__" + k] = np.array(v.shape, np.int64)
        else:
            out[k] = v
    np.savez_compressed(path, **out)


def load(path: str) -> dict:
    raw = np.load(path)
    d = {}
    for k in raw.files:
        if k.startswith("shuffled__"):
            name = k[len("shuffled__"):]
            d[name] = np.ascontiguousarray(raw[k].T).view(np.float64).reshape(tuple(raw["shape__" + name]))
        elif not k.startswith("shape__"):
            d[k] = raw[k]
    return d


def sample_nodes(N: int, fluid: np.ndarray) -> np.ndarray:
    """About 2000 nodes spread over the lattice (odd stride), fluid only: the
    density and velocity of a wall node are not part of the solution."""
    idx = np.arange(0, N, (N // 2000) | 1)
    return idx[fluid[idx]]


def stage_dumps(threads: int = 0) -> dict:
    """Mixed box (one RBC, PLT and WBC, moving walls, uniform body force):
    three full steps, then each stage of a fourth step on its own."""
    case = cases.mixed_box(geo=GEO)
    o = orc.apply_case(case, threads=threads)
    o.step(3)
    out = {}
    o.stage("spread")
    F = o.read_force_field(0)
    nz = np.flatnonzero(np.any(F != 0.0, axis=0)).astype(np.int32)
    out["spread_nodes"] = nz
    out["spread_F"] = F[:, nz]
    o.stage("collide_stream")
    rho, u = o.read_fluid()
    idx = sample_nodes(case.N, case.flags_array() == 0)
    out["collide_rho"] = rho[idx]
    out["collide_u"] = u[:, idx]
    o.stage("interpolate")
    out["interp_v"] = o.read_vertices()[1]
    o.stage("advance")
    out["advance_x"] = o.read_vertices()[0]
    o.stage("mechanics", 1)
    out["mechanics_f"] = o.read_vertices()[2]
    return out


def shear_run(threads: int = 0) -> dict:
    """50^3 Couette box, one RBC (642 vertices), shear 100/s, 1000 steps."""
    case = cases.shear_single_rbc(n=50, shear_rate=100.0, seed=1, geo=GEO)
    o = orc.apply_case(case, threads=threads)
    o.step(1000)
    return run_summary(case, o)


def pipe_run(threads: int = 0) -> dict:
    """64x64x256 pipe at 25% haematocrit (279 RBC), 2000 steps: the summary
    plus every vertex position and velocity."""
    case = cases.pipe_ht25(seed=1, geo=GEO)
    o = orc.apply_case(case, threads=threads)
    o.step(2000)
    return run_summary(case, o)


def suspension_case(geo=GEO):
    """The 128^3 suspension's configuration at 64^3: periodic, Kolmogorov
    forcing, RBC at 30% volume, PLT 1 per 10 RBC and one 2562-vertex WBC."""
    return cases.kolmogorov_mix(n=64, rbc_fraction=0.30, n_wbc=1, plt_per_rbc=0.1, seed=2, geo=geo)


def suspension_run(threads: int = 0) -> dict:
    case = suspension_case()
    o = orc.apply_case(case, threads=threads)
    o.step(300)
    return run_summary(case, o)


def run_summary(case, o, positions: bool = True) -> dict:
    """Compact state: per-cell centroids and volumes, plane- and column-averaged
    velocity, sampled fluid, tile lists; full positions for small cases."""
    nx, ny, nz = case.dims
    x, v, _ = o.read_vertices()
    alive, vol = o.read_cells()
    rho, u = o.read_fluid()
    fluid = case.flags_array() == 0
    uf = np.where(fluid[None, :], u, 0.0).reshape(3, nz, ny, nx)
    cnt = fluid.reshape(nz, ny, nx)
    nvs = [xyz.shape[0] for _, xyz in case.cells]
    offs = np.concatenate([[0], np.cumsum(nvs)])
    centroids = np.array([x[offs[c]:offs[c + 1]].mean(axis=0) for c in range(len(nvs))])
    idx = sample_nodes(case.N, fluid)
    out = dict(alive=alive, volume=vol, centroids=centroids,
               u_plane=uf.sum(axis=(2, 3)) / np.maximum(cnt.sum(axis=(1, 2)), 1),
               u_column=uf.sum(axis=1) / np.maximum(cnt.sum(axis=0), 1),
               rho_sample=rho[idx], u_sample=u[:, idx],
               mass=np.array([rho[fluid].sum()]))
    b = o.bins((8, 8, 8), None, case.dims)
    out["vertex_tile"] = b["vertex_tile"]
    out["tile_offsets"] = b["tile_offsets"]
    out["tile_cell_offsets"] = b["tile_cell_offsets"]
    out["tile_cells"] = b["tile_cells"]
    if positions:
        out["x"] = x
        out["v"] = v
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pipe", action="store_true")
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args()
    meta = {}
    meta_path = os.path.join(HERE, "generated_with.json")
    if os.path.exists(meta_path):
        with open(meta_path) as fh:
            meta = json.load(fh).get("runs", {})
    for name, fn, path in [("stages", stage_dumps, STAGE_FILE), ("shear", shear_run, SHEAR_FILE),
                           ("suspension", suspension_run, SUSPENSION_FILE)] + (
            [("pipe", pipe_run, PIPE_FILE)] if a.pipe else []):
        t = time.time()
        d = fn(a.threads)
        save(path, d)
        meta[name] = {"file": os.path.basename(path), "seconds": round(time.time() - t, 1)}
        print(name, meta[name], {k: getattr(v, "shape", None) for k, v in d.items()})
    with open(meta_path, "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "oracle": "oracle/oracle.cpp (FP64, "
                   "-ffp-contract=off)", "numpy": np.__version__, "runs": meta}, fh, indent=1)


if __name__ == "__main__":
    main()
