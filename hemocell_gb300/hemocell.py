"""Python mirror of HemoCell's case-program API over the C ABI.

Names follow the reference façade (hemocell.h:68-253): ``HemoCell``,
``addCellType``, ``loadParticles``-style placement, ``iterate``,
``setMaterialTimeScaleSeparation``, ``setParticleVelocityUpdateTimeScaleSeparation``
and the driver's ``setExternalVector``.  Errors raise ``HemoCellError`` with
the library's message (the reference prints through hlog and exits).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _lib as L


class HemoCellError(RuntimeError):
    pass


def _dp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(L.D)


def _ip(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(L.I)


@dataclass
class Material:
    """MaterialModel block of <celltype>.xml in SI units."""
    kLink: float = 15.0
    kBend: float = 80.0
    kVolume: float = 20.0
    kArea: float = 5.0
    eta_m: float = 0.0
    kInnerRigid: float = 0.0
    kCytoskeleton: float = 0.0
    coreRadius: float = 0.0
    radius: float = 3.91e-6

    def as_c(self) -> L.hc_material:
        return L.hc_material(self.kLink, self.kBend, self.kVolume, self.kArea, self.eta_m, self.kInnerRigid,
                             self.kCytoskeleton, self.coreRadius, self.radius)

    def as_array(self) -> np.ndarray:
        return np.array([self.kLink, self.kBend, self.kVolume, self.kArea, self.eta_m, self.kInnerRigid,
                         self.kCytoskeleton, self.coreRadius, self.radius], dtype=np.float64)


@dataclass
class Mesh:
    xyz: np.ndarray        # (nv, 3) float64, lattice units
    tris: np.ndarray       # (nf, 3) int32, outward oriented
    inner: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))

    @property
    def nv(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def nf(self) -> int:
        return int(self.tris.shape[0])


def _mesh_call(fn, *args, est_nf: int) -> Mesh:
    est_nv = est_nf // 2 + 2
    xyz = np.zeros((est_nv, 3), np.float64)
    tris = np.zeros((est_nf, 3), np.int32)
    nv = C.c_int()
    nf = C.c_int()
    rc = fn(*args, _dp(xyz), est_nv, _ip(tris), est_nf, C.byref(nv), C.byref(nf))
    if rc != L.HC_OK:
        raise HemoCellError("mesh generation failed")
    return Mesh(xyz[: nv.value].copy(), tris[: nf.value].copy())


def _faces_for(min_triangles: int) -> int:
    nf = 20
    while nf < min_triangles:
        nf *= 4
    return nf


def icosphere(min_triangles: int, radius: float) -> Mesh:
    """WBC_SPHERE: constructSphereIcosahedron (helper/meshGeneratingFunctions.hh:31-151)."""
    return _mesh_call(L.lib().hc_mesh_icosphere, min_triangles, radius, est_nf=_faces_for(min_triangles))


def rbc_mesh(min_triangles: int, radius: float) -> Mesh:
    """RBC_FROM_SPHERE: Evans-Fung biconcave map (helper/meshGeneratingFunctions.hh:153-168)."""
    return _mesh_call(L.lib().hc_mesh_rbc, min_triangles, radius, est_nf=_faces_for(min_triangles))


def ellipsoid_mesh(min_triangles: int, radius: float, aspect: float) -> Mesh:
    """ELLIPSOID_FROM_SPHERE (helper/meshGeneratingFunctions.hh:170-183)."""
    return _mesh_call(L.lib().hc_mesh_ellipsoid, min_triangles, radius, aspect, est_nf=_faces_for(min_triangles))


def antipodal_pairs(xyz: np.ndarray) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, np.float64)
    out = np.zeros((xyz.shape[0], 2), np.int32)
    n = L.lib().hc_mesh_antipodal_pairs(_dp(xyz), xyz.shape[0], _ip(out), xyz.shape[0])
    if n < 0:
        raise HemoCellError("antipodal pair search failed")
    return out[:n].copy()


def place_cells(mesh: Mesh, centres: np.ndarray, angles: np.ndarray) -> np.ndarray:
    """Vertex positions of cells placed as loadParticles does (io/readPositionsBloodCells.cpp:290-361)."""
    centres = np.ascontiguousarray(centres, np.float64).reshape(-1, 3)
    angles = np.ascontiguousarray(angles, np.float64).reshape(-1, 3)
    n = centres.shape[0]
    out = np.zeros((n * mesh.nv, 3), np.float64)
    xyz = np.ascontiguousarray(mesh.xyz, np.float64)
    rc = L.lib().hc_place_cells(_dp(xyz), mesh.nv, n, _dp(centres), _dp(angles), _dp(out))
    if rc != L.HC_OK:
        raise HemoCellError("placement failed")
    return out


def pos_to_lattice(pos_um, angles_deg, dx: float):
    """Lines of a .pos file (centre in micrometres, three angles in degrees) as
    loadParticles reads them (io/readPositionsBloodCells.cpp:218-224, 327-351):
    centres in lattice units, angles in radians and negated (the reference's
    right- to left-handed conversion)."""
    pos = np.asarray(pos_um, np.float64).reshape(-1, 3)
    ang = np.asarray(angles_deg, np.float64).reshape(-1, 3)
    return pos * (1e-6 / dx) + 0.0, (ang * (math.pi / 180.0)) * -1.0


def pack_cells(dims, periodic, solid: Optional[np.ndarray], meshes: Sequence[Mesh], counts: Sequence[int],
               margin: float, seed: int, max_attempts: int = 20000):
    """Seeded non-overlapping random packing; returns (centres, angles, types)."""
    nt = len(meshes)
    total = int(sum(counts))
    xyzs = [np.ascontiguousarray(m.xyz, np.float64) for m in meshes]
    triss = [np.ascontiguousarray(m.tris, np.int32) for m in meshes]
    xp = (L.D * nt)(*[_dp(a) for a in xyzs])
    tp = (L.I * nt)(*[_ip(a) for a in triss])
    nvs = np.array([m.nv for m in meshes], np.int32)
    nfs = np.array([m.nf for m in meshes], np.int32)
    cnt = np.array(counts, np.int32)
    per = np.array(periodic, np.int32)
    centres = np.zeros((max(total, 1), 3), np.float64)
    angles = np.zeros((max(total, 1), 3), np.float64)
    types = np.zeros(max(total, 1), np.int32)
    sp = None if solid is None else np.ascontiguousarray(solid, np.uint8).ctypes.data_as(L.U8)
    n = L.lib().hc_pack_cells(dims[0], dims[1], dims[2], _ip(per), sp, nt, xp, _ip(nvs), tp, _ip(nfs), _ip(cnt),
                              float(margin), C.c_ulonglong(seed), max_attempts, _dp(centres), _dp(angles), _ip(types))
    if n < 0:
        raise HemoCellError("packing failed")
    return centres[:n].copy(), angles[:n].copy(), types[:n].copy()


_default_device = 0


def set_default_device(device: int) -> None:
    """The CUDA device of handles and batches created without an explicit one
    (one process per GPU: its local rank)."""
    global _default_device
    _default_device = int(device)


def default_device() -> int:
    return _default_device


class HemoCell:
    """One GB300-resident HemoCell instance (a D3Q19 lattice with its cells)."""

    def __init__(self, nx: int, ny: int, nz: int, periodic=(1, 1, 1), dx: float = 0.5e-6, dt: float = 1e-7,
                 nu_p: float = 0.0, rho_p: float = 1025.0, kBT_p: float = 4.100531391e-21, tau: float = 1.0,
                 form: int = L.HC_FORM_PLAIN_F64, launch: int = L.HC_LAUNCH_PER_STAGE, device: Optional[int] = None,
                 tile=(8, 8, 8)):
        p = L.hc_params()
        p.nx, p.ny, p.nz = nx, ny, nz
        for a in range(3):
            p.periodic[a] = int(periodic[a])
            p.tile[a] = int(tile[a])
        p.dx, p.dt, p.nu_p, p.rho_p, p.kBT_p, p.tau = dx, dt, nu_p, rho_p, kBT_p, tau
        p.form, p.launch, p.device = form, launch, _default_device if device is None else device
        self._lib = L.lib()
        h = self._lib.hc_create(C.byref(p))
        if not h:
            raise HemoCellError(self._lib.hc_last_error(None).decode())
        self._h = C.c_void_p(h)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dx = dx
        self.N = nx * ny * nz
        self.form = form
        self.types: list[Mesh] = []
        self.cell_types: list[int] = []
        self._pending: dict[int, np.ndarray] = {}

    # --- lifecycle
    def close(self):
        if getattr(self, "_batch", None) is not None:
            return  # a Batch owns the handle until it is released
        if getattr(self, "_h", None):
            self._lib.hc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise HemoCellError(self._lib.hc_last_error(self._h).decode() or f"error {rc}")
        return rc

    # --- units
    def units(self) -> dict:
        out = np.zeros(6)
        self._check(self._lib.hc_derived_units(self._h, _dp(out)))
        return dict(zip(("tau", "nu_lbm", "dm", "df", "kBT_lbm", "f_limit"), out.tolist()))

    # --- lattice set-up
    def set_flags(self, flags: np.ndarray):
        f = np.ascontiguousarray(flags, np.uint8).reshape(-1)
        assert f.size == self.N
        self._check(self._lib.hc_set_flags(self._h, f.ctypes.data_as(L.U8)))

    def set_wall_velocity(self, cls: int, u):
        u = np.ascontiguousarray(u, np.float64)
        self._check(self._lib.hc_set_wall_velocity(self._h, cls, _dp(u)))

    def setExternalVector(self, mode: int, p=(0.0, 0.0, 0.0)):
        p = np.ascontiguousarray(p, np.float64)
        self._check(self._lib.hc_set_body_force(self._h, mode, _dp(p)))

    set_body_force = setExternalVector

    def latticeEquilibrium(self, rho: float = 1.0, u=(0.0, 0.0, 0.0)):
        u = np.ascontiguousarray(u, np.float64)
        self._check(self._lib.hc_init_equilibrium(self._h, rho, _dp(u)))

    # --- cells
    def addCellType(self, name: str, model: int, material: Material, mesh: Mesh) -> int:
        xyz = np.ascontiguousarray(mesh.xyz, np.float64)
        tris = np.ascontiguousarray(mesh.tris, np.int32)
        inner = np.ascontiguousarray(mesh.inner, np.int32).reshape(-1, 2)
        m = material.as_c()
        t = self._check(self._lib.hc_add_cell_type(self._h, name.encode(), model, C.byref(m), _dp(xyz), mesh.nv,
                                                   _ip(tris), mesh.nf, _ip(inner) if len(inner) else None,
                                                   len(inner)))
        self.types.append(mesh)
        return t

    def add_cells(self, type_id: int, centres: np.ndarray, angles: np.ndarray) -> int:
        centres = np.ascontiguousarray(centres, np.float64).reshape(-1, 3)
        angles = np.ascontiguousarray(angles, np.float64).reshape(-1, 3)
        first = self._check(self._lib.hc_add_cells(self._h, type_id, centres.shape[0], _dp(centres), _dp(angles)))
        self.cell_types += [type_id] * centres.shape[0]
        return first

    def loadParticles(self, type_id: int, pos_um, angles_deg) -> np.ndarray:
        """HemoCell::loadParticles for one cell type from the rows of its
        .pos file (centres in micrometres, angles in degrees): the cells the
        reference admits (no vertex on a wall node or outside the lattice) are
        added; returns the per-row mask of the cells added."""
        centres, angles = pos_to_lattice(pos_um, angles_deg, self.dx)
        centres = np.ascontiguousarray(centres, np.float64)
        angles = np.ascontiguousarray(angles, np.float64)
        mask = np.zeros(centres.shape[0], np.int32)
        self._check(self._lib.hc_load_cells(self._h, type_id, centres.shape[0], _dp(centres), _dp(angles),
                                            _ip(mask)))
        self.cell_types += [type_id] * int(mask.sum())
        return mask.astype(bool)

    def add_cells_xyz(self, type_id: int, xyz: np.ndarray) -> int:
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        n = xyz.shape[0] // self.types[type_id].nv
        first = self._check(self._lib.hc_add_cells_xyz(self._h, type_id, n, _dp(xyz)))
        self.cell_types += [type_id] * n
        return first

    def setMaterialTimeScaleSeparation(self, every: Sequence[int], velocity_every: int = 1):
        e = np.ascontiguousarray(every, np.int32)
        self._check(self._lib.hc_set_timescales(self._h, _ip(e), len(e), velocity_every))

    def set_vertex_forces(self, ids, forces):
        """Constant external vertex forces added before every spread (HemoCellStretch)."""
        ids = np.ascontiguousarray(ids, np.int32).reshape(-1)
        forces = np.ascontiguousarray(forces, np.float64).reshape(-1, 3)
        self._check(self._lib.hc_set_vertex_forces(self._h, len(ids), _ip(ids) if len(ids) else None,
                                                   _dp(forces) if len(ids) else None))

    # --- stepping
    def setRepulsion(self, repulsionConstant: float, repulsionCutoff: float, timescale: int = 1):
        """HemoCell::setRepulsion: cutoff in micrometres (converted with dx)."""
        self._check(self._lib.hc_set_repulsion(self._h, repulsionConstant, repulsionCutoff * 1e-6 / self.dx,
                                               int(timescale)))

    def enableBoundaryParticles(self, constant: float, cutoff: float, timestep: int = 1):
        """HemoCell::enableBoundaryParticles: cutoff in micrometres."""
        self._check(self._lib.hc_set_boundary_repulsion(self._h, constant, cutoff * 1e-6 / self.dx, int(timestep)))

    def read_repulsion(self) -> np.ndarray:
        out = np.zeros((self.stats().vertices, 3))
        self._check(self._lib.hc_read_repulsion(self._h, _dp(out)))
        return out

    def iterate(self, nsteps: int = 1):
        self._check(self._lib.hc_step(self._h, nsteps))

    def stage(self, s: int):
        self._check(self._lib.hc_stage(self._h, s))

    def sync(self):
        self._check(self._lib.hc_sync(self._h))

    def time_steps(self, nsteps: int) -> float:
        """Device time (ms) of nsteps, CUDA events on the handle's stream."""
        ms = C.c_double()
        self._check(self._lib.hc_time_steps(self._h, nsteps, C.byref(ms)))
        return ms.value

    def profile_stages(self, nsteps: int) -> dict:
        out = np.zeros(5)
        self._check(self._lib.hc_profile_stages(self._h, nsteps, _dp(out)))
        return dict(zip(("spread", "collide_stream", "interp_advance", "mechanics", "step"), out.tolist()))

    def profile_kernels(self, nsteps: int) -> dict:
        """Device time (ms per step) of each kernel inside the batched step as
        iterate runs it: collide-stream, node velocity (or interpolation +
        advance when unfused), force assembly, whole step."""
        out = np.zeros(4)
        self._check(self._lib.hc_profile_kernels(self._h, nsteps, _dp(out)))
        return dict(zip(("collide_stream", "node_velocity", "mechanics", "step"), out.tolist()))

    def read_positions(self, out: Optional[np.ndarray] = None):
        """Positions only, into a caller-owned (V,3) float64 buffer (pinned for
        speed), or a new array when none is given."""
        if out is None:
            out = np.zeros((self.stats().vertices, 3))
        self._check(self._lib.hc_read_vertices(self._h, _dp(out), None, None))
        return out

    def read_positions_async(self, out: np.ndarray, slot: int = 0) -> None:
        """Start copying the positions (after the steps queued so far) into a
        caller-owned C-contiguous (V,3) float64 buffer in pinned host memory,
        without waiting; the copy runs on its own stream while later steps
        compute.  ``out`` must stay alive and untouched until
        ``wait_positions(slot)``; two slots allow double buffering."""
        nv = self._lib.hc_vertex_count(self._h)   # stats() would wait for the stream
        if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.shape != (nv, 3):
            raise HemoCellError("read_positions_async needs a C-contiguous (V,3) float64 buffer")
        if not hasattr(self, "_pending"):
            self._pending = {}
        self._pending[slot] = out
        self._check(self._lib.hc_read_positions_async(self._h, _dp(out), slot))

    def wait_positions(self, slot: int = 0) -> np.ndarray:
        """Wait for the copy started by read_positions_async(slot); returns its buffer."""
        self._check(self._lib.hc_wait_positions(self._h, slot))
        return getattr(self, "_pending", {}).pop(slot, None)

    # --- readback
    def read_fluid(self):
        rho = np.zeros(self.N)
        u = np.zeros(3 * self.N)
        self._check(self._lib.hc_read_fluid(self._h, _dp(rho), _dp(u)))
        return rho, u.reshape(3, self.N)

    def read_populations(self) -> np.ndarray:
        f = np.zeros(19 * self.N)
        self._check(self._lib.hc_read_populations(self._h, _dp(f)))
        return f.reshape(19, self.N)

    def write_populations(self, f: np.ndarray):
        f = np.ascontiguousarray(f, np.float64).reshape(-1)
        self._check(self._lib.hc_write_populations(self._h, _dp(f)))

    def read_force_field(self, which: int = 0) -> np.ndarray:
        F = np.zeros(3 * self.N)
        self._check(self._lib.hc_read_force_field(self._h, _dp(F), which))
        return F.reshape(3, self.N)

    def write_force_field(self, F: np.ndarray):
        F = np.ascontiguousarray(F, np.float64).reshape(-1)
        self._check(self._lib.hc_write_force_field(self._h, _dp(F)))

    def stats(self) -> L.hc_stats:
        s = L.hc_stats()
        self._check(self._lib.hc_get_stats(self._h, C.byref(s)))
        return s

    def read_vertices(self):
        V = self.stats().vertices
        x = np.zeros((V, 3))
        v = np.zeros((V, 3))
        f = np.zeros((V, 3))
        self._check(self._lib.hc_read_vertices(self._h, _dp(x), _dp(v), _dp(f)))
        return x, v, f

    def write_vertices(self, x=None, v=None, f=None):
        conv = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (x, v, f)]
        self._check(self._lib.hc_write_vertices(self._h, *[_dp(a) for a in conv]))

    def read_cells(self):
        n = self.stats().cells
        alive = np.zeros(n, np.int32)
        vol = np.zeros(n)
        self._check(self._lib.hc_read_cells(self._h, _ip(alive), _dp(vol)))
        return alive, vol

    def cell_info(self) -> np.ndarray:
        """(cells, 16): centroid, mean velocity, area, volume, stretch, bbox, type."""
        out = np.zeros((self.stats().cells, 16))
        self._check(self._lib.hc_cell_info(self._h, _dp(out)))
        return out

    def writeCellInfo_CSV(self, directory: str, si_units: bool = False):
        self._check(self._lib.hc_write_cell_info_csv(self._h, directory.encode(), 1 if si_units else 0))

    def writeOutput(self, directory: str, si_units: bool = False):
        """Fluid and particle fields as XDMF over raw arrays in <directory>/hdf5/."""
        self._check(self._lib.hc_write_output(self._h, directory.encode(), 1 if si_units else 0))

    def saveCheckPoint(self, directory: str):
        self._check(self._lib.hc_save_checkpoint(self._h, directory.encode()))

    def loadCheckPoint(self, directory: str):
        self._check(self._lib.hc_load_checkpoint(self._h, directory.encode()))

    def read_bins(self):
        st = self.stats()
        V = st.vertices
        # tiles are fixed by the parameters; size buffers generously
        ntiles_max = self.N
        vn = np.zeros(max(V, 1), np.int32)
        vt = np.zeros(max(V, 1), np.int32)
        to = np.zeros(ntiles_max + 1, np.int32)
        tv = np.zeros(max(V, 1), np.int32)
        tco = np.zeros(ntiles_max + 1, np.int32)
        tc = np.zeros(max(V, 1), np.int32)
        nt = self._check(self._lib.hc_read_bins(self._h, _ip(vn), _ip(vt), _ip(to), _ip(tv), _ip(tco), _ip(tc),
                                                max(V, 1)))
        return dict(vertex_node=vn[:V], vertex_tile=vt[:V], tile_offsets=to[: nt + 1],
                    tile_vertices=tv[: to[nt]], tile_cell_offsets=tco[: nt + 1], tile_cells=tc[: tco[nt]])

    def read_neighbours(self):
        """Per tile, the sorted distinct cells of the tile and its 26
        neighbouring tiles (the cells within the kernel halo), as CSR:
        (offsets[ntiles + 1], cells)."""
        b = self.read_bins()
        nt = len(b["tile_cell_offsets"]) - 1
        cap = max(27 * len(b["tile_cells"]), 1)
        off = np.zeros(nt + 1, np.int32)
        cells = np.zeros(cap, np.int32)
        r = self._check(self._lib.hc_read_neighbours(self._h, _ip(off), _ip(cells), cap))
        assert r == nt
        return off, cells[: off[nt]].copy()

    def device_status(self) -> int:
        s = C.c_uint()
        self._check(self._lib.hc_device_status(self._h, C.byref(s)))
        return s.value

    def autotune(self, cache: str = ""):
        self._check(self._lib.hc_autotune(self._h, cache.encode()))

    def tuning(self) -> list:
        t = np.zeros(8, np.int32)
        self._check(self._lib.hc_get_tuning(self._h, _ip(t)))
        return t.tolist()

    def set_tuning(self, t):
        t = np.ascontiguousarray(t, np.int32)
        self._check(self._lib.hc_set_tuning(self._h, _ip(t)))


def voxelize_stl(path: str, ref_dir: int = 0, ref_length: float = 100.0, margin: int = 1,
                 open_ends: bool = True):
    """getFlagMatrixFromSTL: (flags, dims) of a closed STL surface; flags per
    node (x fastest) 0 fluid inside, 1 wall outside."""
    lib = L.lib()
    dims = np.zeros(3, np.int32)
    if lib.hc_stl_voxelize(path.encode(), ref_dir, float(ref_length), margin, int(open_ends), _ip(dims), None, 0):
        raise HemoCellError(lib.hc_last_error(None).decode())
    n = int(np.prod(dims.astype(np.int64)))
    flags = np.zeros(n, np.uint8)
    if lib.hc_stl_voxelize(path.encode(), ref_dir, float(ref_length), margin, int(open_ends), _ip(dims),
                           flags.ctypes.data_as(L.U8), n):
        raise HemoCellError(lib.hc_last_error(None).decode())
    return flags, tuple(int(d) for d in dims)


def estimate_device_bytes(dims, form: int, nvertices: int, ncells: int, tile=(8, 8, 8)) -> int:
    """Upper bound of the device bytes of a handle (hc_estimate_device_bytes)."""
    p = L.hc_params()
    p.nx, p.ny, p.nz = dims
    for a in range(3):
        p.tile[a] = int(tile[a])
    p.form = form
    b = L.lib().hc_estimate_device_bytes(C.byref(p), int(nvertices), int(ncells))
    if b < 0:
        raise HemoCellError("invalid parameters for the estimate")
    return int(b)


class Batch:
    """Continuous batching of independent solves on one device (hc_batch_*).

    ``admit`` hands a set-up :class:`HemoCell` to the batch, which then owns
    its handle; ``pump`` keeps every resident solve's stream fed and reports
    how many finished; ``pop`` returns a finished solve (readable through its
    ``read_*`` methods) and ``release`` frees it and its share of the budget.
    """

    def __init__(self, budget_bytes: int, max_slots: int = 64, chunk_steps: int = 50, device: Optional[int] = None):
        self._lib = L.lib()
        dev = _default_device if device is None else device
        b = self._lib.hc_batch_create(dev, int(budget_bytes), int(max_slots), int(chunk_steps))
        if not b:
            raise HemoCellError(self._lib.hc_last_error(None).decode())
        self._b = C.c_void_p(b)
        self._owned: dict[int, HemoCell] = {}

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise HemoCellError(self._lib.hc_batch_last_error(self._b).decode() or f"error {rc}")
        return rc

    def fits(self, nbytes: int) -> bool:
        return self._check(self._lib.hc_batch_fits(self._b, int(nbytes))) == 1

    def admit(self, hc: HemoCell, nsteps: int, tag: int) -> bool:
        """True if admitted (the batch now owns hc's handle); False if it does
        not fit the budget or the slots now (hc stays the caller's)."""
        rc = self._lib.hc_batch_admit(self._b, hc._h, int(nsteps), int(tag))
        if rc == L.HC_ERR_MEMORY:
            return False
        self._check(rc)
        hc._batch = self
        self._owned[hc._h.value] = hc
        return True

    def pump(self, wait_ms: float = 1.0) -> int:
        return self._check(self._lib.hc_batch_pump(self._b, float(wait_ms)))

    def pop(self):
        """(tag, HemoCell, status) of one finished solve, or None."""
        tag = C.c_longlong()
        h = C.c_void_p()
        st = C.c_int()
        if self._check(self._lib.hc_batch_pop(self._b, C.byref(tag), C.byref(h), C.byref(st))) == 0:
            return None
        return tag.value, self._owned[h.value], st.value

    def release(self, hc: HemoCell, destroy: bool = True):
        key = hc._h.value
        self._check(self._lib.hc_batch_release(self._b, hc._h, 1 if destroy else 0))
        self._owned.pop(key, None)
        hc._batch = None
        if destroy:
            hc._h = None

    def stats(self) -> dict:
        st = L.hc_batch_stats()
        self._check(self._lib.hc_batch_get_stats(self._b, C.byref(st)))
        return {n: getattr(st, n) for n, _ in L.hc_batch_stats._fields_}

    def close(self):
        if getattr(self, "_b", None):
            self._lib.hc_batch_destroy(self._b)
            for hc in self._owned.values():
                hc._batch = None
                hc._h = None
            self._owned.clear()
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
