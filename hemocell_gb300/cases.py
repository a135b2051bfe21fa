"""Seeded synthetic workloads of the IB-LBM step.

Each builder returns a :class:`Case`: lattice, walls, body force, cell types
(meshes + SI materials) and placed cells.  The same Case is applied to a
:class:`~hemocell_gb300.hemocell.HemoCell` handle (``Case.build``) and, in the
tests, to the FP64 CPU oracle, so both start from identical inputs.

Workloads (no public data set is involved; everything comes from seeds):
  shear_single_rbc  50^3 Couette, moving bounce-back walls, one RBC
  pipe_ht25         64x64x256 cylinder R=30 lu, body force, RBCs at 25% Ht
  kolmogorov_mix    128^3 periodic, Kolmogorov forcing, RBC+PLT+WBC suspension
  small_*           reduced versions for parity tests
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from types import SimpleNamespace
from typing import List, Optional, Tuple

import numpy as np

from . import _lib as L
from .hemocell import HemoCell, Material, Mesh, antipodal_pairs, ellipsoid_mesh, icosphere, pack_cells, \
    place_cells, pos_to_lattice, rbc_mesh

# The geometry functions a workload is built with.  PRODUCT is this library's
# (host code of libhcgpu.so); a checker may pass any object with the same
# functions, e.g. an independent restatement, to build the same workload
# without this library.
PRODUCT = SimpleNamespace(icosphere=icosphere, rbc_mesh=rbc_mesh, ellipsoid_mesh=ellipsoid_mesh,
                          antipodal_pairs=antipodal_pairs, place_cells=place_cells, pack_cells=pack_cells,
                          pos_to_lattice=pos_to_lattice)

DX = 0.5e-6
DT = 1e-7
RHO_P = 1025.0
KBT = 4.100531391e-21

# MaterialModel values of the reference's material files
RBC_MATERIAL = Material(kLink=15.0, kBend=80.0, kVolume=20.0, kArea=5.0, eta_m=0.0, radius=3.91e-6)  # examples/oneCellShear/RBC.xml
PLT_MATERIAL = Material(kLink=25.0, kBend=250.0, kVolume=100.0, kArea=8.0, eta_m=0.0, radius=1.0e-6)  # tests/validation/pipeflow/PLT.xml constants
WBC_MATERIAL = Material(kLink=60.0, kBend=200.0, kVolume=20.0, kArea=20.0, eta_m=1.0e-9, kInnerRigid=6.40625e-12,
                        kCytoskeleton=6.40625e-15, coreRadius=2.5e-6, radius=4.0e-6)  # examples/cell_shapes/WBC_HO.xml


@dataclass
class CellTypeSpec:
    name: str
    model: int
    material: Material
    mesh: Mesh


@dataclass
class Case:
    name: str
    dims: Tuple[int, int, int]
    periodic: Tuple[int, int, int]
    tau: float = 1.0
    flags: Optional[np.ndarray] = None
    walls: dict = field(default_factory=dict)       # class -> (ux, uy, uz)
    body_mode: int = L.HC_BODY_NONE
    body: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    types: List[CellTypeSpec] = field(default_factory=list)
    cells: List[Tuple[int, np.ndarray]] = field(default_factory=list)  # (type, (nv,3) positions)
    steps: int = 100

    @property
    def N(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    @property
    def nvertices(self) -> int:
        return sum(c[1].shape[0] for c in self.cells)

    def flags_array(self) -> np.ndarray:
        return np.zeros(self.N, np.uint8) if self.flags is None else self.flags

    def build(self, form: int = L.HC_FORM_PLAIN_F64, launch: int = L.HC_LAUNCH_PER_STAGE, device=None,
              tile=(8, 8, 8)) -> HemoCell:
        hc = HemoCell(*self.dims, periodic=self.periodic, dx=DX, dt=DT, rho_p=RHO_P, kBT_p=KBT, tau=self.tau,
                      form=form, launch=launch, device=device, tile=tile)
        if self.flags is not None:
            hc.set_flags(self.flags)
        for cls, u in self.walls.items():
            hc.set_wall_velocity(cls, u)
        hc.latticeEquilibrium(1.0)
        hc.setExternalVector(self.body_mode, self.body)
        for t in self.types:
            hc.addCellType(t.name, t.model, t.material, t.mesh)
        # group consecutive cells of one type into one call
        i = 0
        while i < len(self.cells):
            t = self.cells[i][0]
            j = i
            while j < len(self.cells) and self.cells[j][0] == t:
                j += 1
            hc.add_cells_xyz(t, np.concatenate([c[1] for c in self.cells[i:j]]))
            i = j
        return hc


def splitmix64(seed: int):
    s = seed & 0xFFFFFFFFFFFFFFFF
    while True:
        s = (s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        yield (z ^ (z >> 31)) >> 11


def seeded_angles(seed: int, n: int) -> np.ndarray:
    g = splitmix64(seed)
    return np.array([[(next(g) / 2 ** 53) * 2 * math.pi - math.pi for _ in range(3)] for _ in range(n)])


def rbc_type(min_triangles: int = 600, geo=PRODUCT) -> CellTypeSpec:
    mesh = geo.rbc_mesh(min_triangles, RBC_MATERIAL.radius / DX)
    return CellTypeSpec("RBC", L.HC_MODEL_RBC_HIGH_ORDER, RBC_MATERIAL, mesh)


def plt_type(min_triangles: int = 320, radius_m: float = 1.0e-6, aspect: float = 0.25, geo=PRODUCT) -> CellTypeSpec:
    mesh = geo.ellipsoid_mesh(min_triangles, radius_m / DX, aspect)
    mesh.inner = geo.antipodal_pairs(mesh.xyz)
    mat = Material(**{**PLT_MATERIAL.__dict__, "radius": radius_m})
    return CellTypeSpec("PLT", L.HC_MODEL_PLT_SIMPLE, mat, mesh)


def wbc_type(min_triangles: int = 5120, geo=PRODUCT) -> CellTypeSpec:
    mesh = geo.icosphere(min_triangles, WBC_MATERIAL.radius / DX)
    mesh.inner = geo.antipodal_pairs(mesh.xyz)
    return CellTypeSpec("WBC", L.HC_MODEL_WBC_HIGH_ORDER, WBC_MATERIAL, mesh)


def shear_walls(n: Tuple[int, int, int], shear_rate: float) -> Tuple[np.ndarray, dict]:
    """Couette box: wall nodes at z=0 (class 1, +x) and z=nz-1 (class 2, -x);
    vHalf = (nz-1) * shearrate_lbm / 2 as helper/hemocellInit.hh:75-77."""
    nx, ny, nz = n
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[0] = 1
    flags[nz - 1] = 2
    v_half = (nz - 1) * shear_rate * DT * 0.5
    return flags.reshape(-1), {1: (v_half, 0.0, 0.0), 2: (-v_half, 0.0, 0.0)}


def shear_single_rbc(n: int = 50, shear_rate: float = 100.0, seed: int = 1, min_triangles: int = 600,
                     steps: int = 1000, geo=PRODUCT) -> Case:
    """Single RBC in Couette shear (examples/oneCellShear analogue)."""
    dims = (n, n, n)
    flags, walls = shear_walls(dims, shear_rate)
    t = rbc_type(min_triangles, geo)
    centre = np.array([[(n - 1) / 2.0] * 3])
    xyz = geo.place_cells(t.mesh, centre, seeded_angles(seed, 1))
    return Case(f"shear_rbc_{n}", dims, (1, 1, 0), flags=flags, walls=walls, types=[t], cells=[(0, xyz)],
                steps=steps)


def cylinder_flags(nx: int, ny: int, nz: int, radius: float) -> np.ndarray:
    """Bounce-back nodes outside a cylinder along z centred in the cross-section."""
    cx, cy = (nx - 1) / 2.0, (ny - 1) / 2.0
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    solid2d = ((X - cx) ** 2 + (Y - cy) ** 2) > radius ** 2
    return np.broadcast_to(solid2d.astype(np.uint8), (nz, ny, nx)).reshape(-1).copy()


def pipe_ht25(nx: int = 64, ny: int = 64, nz: int = 256, radius: float = 30.0, ht: float = 0.25,
              u_max_phys: float = 1e-3, seed: int = 1, min_triangles: int = 600, steps: int = 2000,
              n_cells: Optional[int] = None, geo=PRODUCT) -> Case:
    """Pipe flow at a given hematocrit (examples/pipeflow analogue): body force
    F_z = 4 nu u_max / R^2 (Poiseuille), RBCs packed >= 1 lu from the wall."""
    flags = cylinder_flags(nx, ny, nz, radius)
    t = rbc_type(min_triangles, geo)
    vol = _mesh_volume(t.mesh)
    lumen = float((flags == 0).sum())
    if n_cells is None:
        n_cells = int(round(ht * lumen / vol))
    centres, angles, types = geo.pack_cells((nx, ny, nz), (1, 1, 1), flags, [t.mesh], [n_cells], margin=1.0,
                                            seed=seed)
    xyz = geo.place_cells(t.mesh, centres, angles)
    nv = t.mesh.nv
    cells = [(0, xyz[k * nv:(k + 1) * nv]) for k in range(centres.shape[0])]
    nu = (1.0 - 0.5) / 3.0
    u_max = u_max_phys * DT / DX
    fz = 4.0 * nu * u_max / radius ** 2
    return Case(f"pipe_{nx}x{ny}x{nz}", (nx, ny, nz), (1, 1, 1), flags=flags, body_mode=L.HC_BODY_UNIFORM,
                body=(0.0, 0.0, fz), types=[t], cells=cells, steps=steps)


def kolmogorov_mix(n: int = 128, rbc_fraction: float = 0.30, n_wbc: int = 2, plt_per_rbc: float = 0.1,
                   u_peak: float = 5e-3, seed: int = 1, steps: int = 1000, rbc_triangles: int = 600,
                   plt_triangles: int = 320, wbc_triangles: int = 5120, geo=PRODUCT) -> Case:
    """Heterogeneous suspension in a periodic cube with Kolmogorov forcing
    F_x = A sin(2 pi z / n), A = u_peak nu k^2 (cases/kolmogorovFlow analogue)."""
    dims = (n, n, n)
    types = [rbc_type(rbc_triangles, geo), plt_type(plt_triangles, geo=geo), wbc_type(wbc_triangles, geo)]
    n_rbc = int(round(rbc_fraction * n ** 3 / _mesh_volume(types[0].mesh)))
    n_plt = int(round(plt_per_rbc * n_rbc))
    counts = [n_rbc, n_plt, n_wbc]
    centres, angles, tids = geo.pack_cells(dims, (1, 1, 1), None, [t.mesh for t in types], counts, margin=0.0,
                                           seed=seed)
    cells = []
    for t in range(3):
        sel = np.where(tids == t)[0]
        if len(sel) == 0:
            continue
        xyz = geo.place_cells(types[t].mesh, centres[sel], angles[sel])
        nv = types[t].mesh.nv
        cells += [(t, xyz[k * nv:(k + 1) * nv]) for k in range(len(sel))]
    nu = (1.0 - 0.5) / 3.0
    A = u_peak * nu * (2 * math.pi / n) ** 2
    return Case(f"kolmogorov_{n}", dims, (1, 1, 1), body_mode=L.HC_BODY_KOLMOGOROV, body=(A, 0.0, 0.0),
                types=types, cells=cells, steps=steps)


def mixed_box(seed: int = 5, n: Tuple[int, int, int] = (20, 18, 16), wall: bool = True, geo=PRODUCT) -> Case:
    """Small box with one cell of each type (RBC 162, PLT 42, WBC 162 vertices)
    and, optionally, moving walls: the stage-by-stage parity case."""
    nx, ny, nz = n
    if wall:
        flags, walls = shear_walls(n, 5000.0)
        periodic = (1, 1, 0)
    else:
        flags, walls, periodic = None, {}, (1, 1, 1)
    types = [rbc_type(320, geo), plt_type(80, radius_m=1.0e-6, aspect=0.4, geo=geo), wbc_type(320, geo)]
    rng = np.random.default_rng(seed)
    cells = []
    centres = [((nx - 1) / 2, (ny - 1) / 2 - 3.5, (nz - 1) / 2), ((nx - 1) / 2 + 4, (ny - 1) / 2 + 5, (nz - 1) / 2),
               ((nx - 1) / 2 - 4.5, (ny - 1) / 2 + 4.0, (nz - 1) / 2 + 1)]
    for t, c in enumerate(centres):
        ang = rng.uniform(-np.pi, np.pi, size=(1, 3))
        xyz = geo.place_cells(types[t].mesh, np.array([c]), ang)
        cells.append((t, xyz))
    return Case("mixed_box", n, periodic, flags=flags, walls=walls, types=types, cells=cells,
                body_mode=1, body=(2e-6, -1e-6, 5e-7))


def repulsion_box(geo=PRODUCT) -> Case:
    """Two RBCs (162 vertices) stacked close together in a 24x24x16 Couette box,
    the lower one about a lattice unit from the bottom wall: the repulsion
    parity case (inter-cell pairs and wall pushes both occur)."""
    n = (24, 24, 16)
    flags, walls = shear_walls(n, 2000.0)
    t = rbc_type(320, geo)
    # -pi/2 about x turns the template's disc axis (y) onto z: the discs stack
    q = -math.pi / 2
    cells = [(0, geo.place_cells(t.mesh, np.array([[11.5, 11.5, 3.6]]), np.array([[q, 0.0, 0.0]]))),
             (0, geo.place_cells(t.mesh, np.array([[12.0, 11.0, 8.2]]), np.array([[q + 0.1, -0.05, 0.2]])))]
    return Case("repulsion_box", n, (1, 1, 0), flags=flags, walls=walls, types=[t], cells=cells)


def stretch_cell(min_triangles: int = 600, geo=PRODUCT) -> Case:
    """Single RBC in a closed 52x26x26 box (tests/validation/stretch_cell):
    nuP 1.1e-6, dt 1e-7 -> tau 1.82; box faces are static walls; the cell is
    placed by the test's stretch_RBC.pos line "12.0 6 6 90 0 0" (centre in
    micrometres, angles in degrees), which turns the template's disc axis (y)
    onto z: the disc lies in the x-y plane (axial = x, transverse = y as the
    test measures them)."""
    nz = 26
    dims = (2 * nz, nz, nz)
    flags = np.zeros((dims[2], dims[1], dims[0]), np.uint8)
    flags[0, :, :] = flags[-1, :, :] = 1
    flags[:, 0, :] = flags[:, -1, :] = 1
    flags[:, :, 0] = flags[:, :, -1] = 1
    t = rbc_type(min_triangles, geo)
    centre, angles = geo.pos_to_lattice([[12.0, 6.0, 6.0]], [[90.0, 0.0, 0.0]], DX)
    xyz = geo.place_cells(t.mesh, centre, angles)
    tau = 3.0 * 1.1e-6 * DT / DX ** 2 + 0.5
    return Case("stretch_cell", dims, (0, 0, 0), tau=tau, flags=flags.reshape(-1), walls={1: (0.0, 0.0, 0.0)},
                types=[t], cells=[(0, xyz)], steps=10000)


def stretch_forces(xyz: np.ndarray, force_pN: float, n_forced: int = 7):
    """HemoCellStretch (helper/hemoCellStretch.cpp:30-78): the n lowest-x
    vertices get -F/n along x, the n highest-x +F/n; returns (ids, forces)."""
    df = RHO_P * DX ** 4 / DT ** 2
    f = force_pN * 1e-12 / df / n_forced
    order = np.argsort(xyz[:, 0], kind="stable")
    ids = np.concatenate([order[:n_forced], order[::-1][:n_forced]]).astype(np.int32)
    forces = np.zeros((2 * n_forced, 3))
    forces[:n_forced, 0] = -f
    forces[n_forced:, 0] = f
    return ids, forces


def _mesh_volume(m: Mesh) -> float:
    v0, v1, v2 = (m.xyz[m.tris[:, k]] for k in range(3))
    return float(np.einsum("ij,ij->i", v0, np.cross(v1, v2)).sum() / 6.0)


def mesh_volume(m: Mesh) -> float:
    return _mesh_volume(m)
