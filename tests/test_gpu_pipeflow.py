"""The reference's pipe-flow validation (Validation.Pipeflow,
tests/validation/pipeflow/test_pipeflow.cpp:14-106 of HemoCell) on the GPU,
from the reference's own inputs (config_pipeflow.xml, RBC.pos, PLT.pos,
RBC.xml, PLT.xml and examples/pipeflow/tube.stl, parsed into
tests/golden/pipeflow_validation.npz by make_pipeflow_fixture.py):

  - the tube is voxelised from the STL (getFlagMatrixFromSTL with refDir and
    refDirN of the configuration and its fixed one-node margin,
    helper/voxelizeDomain.cpp:81), periodic along x;
  - lbm_pipe_parameters (mechanics/constantConversion.cpp:61-73): radius from
    the fluid area of the x = 0 slice, u_lbm_max = Re nu / (2 R), driving force
    8 nu (u_max / 2) / R^2 along x;
  - RBC_FROM_SPHERE and ELLIPSOID_FROM_SPHERE cells from the .pos files,
    admitted as loadParticles admits them, materials every 2 steps and the
    particle velocity every 2 steps;
  - 100 fluid-only warm-up steps, then 1000 iterations.

Checked at every iteration, as the reference does: 42 cells (of the 253 in
the .pos files) are in the pipe; from iteration 100 the apparent relative
viscosity 0.5 u_max / mean|u| over the fluid lies in (1.03, 3.0) and the mean
vertex force (membrane + repulsion) is below 4 pN.

The count of 42 depends on conventions that Palabos sets and the reference
tree does not hold (DEFscaledMesh's scaling and offset of the STL, inflate()
of the voxelised surface).  This build's choices -- the tube's y extent spans
refDirN lattice units, one node of margin, no inflation, and loadParticles
admitting a cell only when every vertex lies inside the lattice's box and off
wall nodes -- admit exactly 42 (36 RBC, 6 PLT)."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pipeflow_validation.npz")


def write_ascii_stl(path, tris):
    with open(path, "w") as fh:
        fh.write("solid tube\n")
        for t in tris:
            fh.write(" facet normal 0 0 0\n  outer loop\n")
            for v in t:
                fh.write("   vertex " + " ".join(repr(float(c)) for c in v) + "\n")
            fh.write("  endloop\n endfacet\n")
        fh.write("endsolid tube\n")


def material(fx, cell):
    from hemocell_gb300 import Material
    return Material(kLink=float(fx[f"{cell}_kLink"]), kBend=float(fx[f"{cell}_kBend"]),
                    kVolume=float(fx[f"{cell}_kVolume"]), kArea=float(fx[f"{cell}_kArea"]),
                    eta_m=float(fx[f"{cell}_eta_m"]), radius=float(fx[f"{cell}_radius"]))


def test_pipeflow_validation(built, tmp_path):
    from hemocell_gb300 import HemoCell, _lib as L
    from hemocell_gb300 import cases
    from hemocell_gb300.hemocell import voxelize_stl
    fx = np.load(FIX)
    cfg = {k[4:]: float(fx[k]) for k in fx.files if k.startswith("cfg_")}
    stl = str(tmp_path / "tube.stl")
    write_ascii_stl(stl, fx["stl_triangles"])
    flags, dims = voxelize_stl(stl, ref_dir=int(cfg["refDir"]), ref_length=cfg["refDirN"], margin=1,
                               open_ends=True)
    nx, ny, nz = dims
    fl = flags.reshape(nz, ny, nx)
    # lbm_pipe_parameters: the radius from the fluid area of the x = 0 slice
    R = math.sqrt(float((fl[:, :, 0] == 0).sum()) / math.pi)
    dx, dt = cfg["dx"], cfg["dt"]
    nu = cfg["nuP"] * dt / dx ** 2
    u_max = cfg["Re"] * nu / (R * 2)
    force = 8 * nu * (u_max * 0.5) / R / R
    assert 24.0 < R < 26.0

    hc = HemoCell(nx, ny, nz, periodic=(1, 0, 0), dx=dx, dt=dt, nu_p=cfg["nuP"], rho_p=cfg["rhoP"],
                  kBT_p=cfg["kBT"], tau=0.0, form=L.HC_FORM_PLAIN_F64, launch=L.HC_LAUNCH_BATCHED)
    try:
        assert abs(hc.units()["tau"] - (3 * nu + 0.5)) < 1e-12
        hc.set_flags(flags)
        hc.latticeEquilibrium(1.0)
        hc.setExternalVector(L.HC_BODY_UNIFORM, (force, 0.0, 0.0))
        geo = cases.PRODUCT
        rbc = geo.rbc_mesh(int(fx["RBC_minNumTriangles"]), float(fx["RBC_radius"]) / dx)
        plt = geo.ellipsoid_mesh(int(fx["PLT_minNumTriangles"]), float(fx["PLT_radius"]) / dx,
                                 float(fx["PLT_aspectRatio"]))
        plt.inner = geo.antipodal_pairs(plt.xyz)
        t_rbc = hc.addCellType("RBC", L.HC_MODEL_RBC_HIGH_ORDER, material(fx, "RBC"), rbc)
        t_plt = hc.addCellType("PLT", L.HC_MODEL_PLT_SIMPLE, material(fx, "PLT"), plt)

        # 100 collide-streams of the fluid alone; the reference has its cells
        # loaded but not coupled meanwhile, and hemocell.iter stays at 0
        hc.iterate(100)
        every = int(cfg["stepMaterialEvery"])
        loaded_rbc = hc.loadParticles(t_rbc, fx["RBC_pos"][:, :3], fx["RBC_pos"][:, 3:])
        loaded_plt = hc.loadParticles(t_plt, fx["PLT_pos"][:, :3], fx["PLT_pos"][:, 3:])
        hc.setMaterialTimeScaleSeparation([every, every], velocity_every=int(cfg["stepParticleEvery"]))
        n_cells = int(loaded_rbc.sum() + loaded_plt.sum())
        print(f"admitted {loaded_rbc.sum()} of {len(loaded_rbc)} RBC and {loaded_plt.sum()} of "
              f"{len(loaded_plt)} PLT")
        assert (int(loaded_rbc.sum()), int(loaded_plt.sum())) == (36, 6) and n_cells == 42

        df = cfg["rhoP"] * dx ** 4 / dt ** 2
        fluid = flags == 0
        nv = [rbc.nv] * int(loaded_rbc.sum()) + [plt.nv] * int(loaded_plt.sum())
        visc, fmean = [], []
        for it in range(1, 1001):
            hc.iterate(1)
            hc.setExternalVector(L.HC_BODY_UNIFORM, (force, 0.0, 0.0))
            alive = hc.read_cells()[0]
            assert int(alive.sum()) == n_cells, it
            if it < 100:
                continue
            _, u = hc.read_fluid()
            avg = float(np.linalg.norm(u[:, fluid], axis=0).mean())
            v = 0.5 * u_max / avg
            _, _, f = hc.read_vertices()
            keep = np.repeat(alive.astype(bool), nv)
            fm = float(np.linalg.norm(f[keep], axis=1).mean()) * df * 1e12
            visc.append(v)
            fmean.append(fm)
            assert 1.03 < v < 3.0, (it, v)
            assert fm < 4.0, (it, fm)
        print(f"relative apparent viscosity {visc[0]:.3f} (iteration 100) .. {visc[-1]:.3f} (1000); "
              f"mean vertex force at most {max(fmean):.3f} pN")
        assert hc.device_status() & 1 == 0
    finally:
        hc.close()

