"""ctypes binding of the FP64 CPU oracle (test infrastructure only).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; the product never does.  ``apply_case``
feeds a :class:`hemocell_gb300.cases.Case` to the oracle, converting the SI
materials with the oracle's own restatement of the unit conversions.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
U8 = C.POINTER(C.c_uint8)
P = C.c_void_p

_SIG = {
    "orc_create": (P, [C.c_int] * 6 + [C.c_double, C.c_double]),
    "orc_destroy": (None, [P]),
    "orc_set_threads": (None, [C.c_int]),
    "orc_set_flags": (None, [P, U8]),
    "orc_set_wall_velocity": (None, [P, C.c_int, D]),
    "orc_set_body_force": (None, [P, C.c_int, D]),
    "orc_init_equilibrium": (None, [P, C.c_double, D]),
    "orc_add_cell_type": (C.c_int, [P, C.c_int, C.c_int, D, C.c_int, I, C.c_int, I, D]),
    "orc_add_cell": (C.c_int, [P, C.c_int, D]),
    "orc_set_timescales": (None, [P, I, C.c_int]),
    "orc_set_vertex_forces": (None, [P, C.c_int, I, D]),
    "orc_step": (None, [P, C.c_int]),
    "orc_set_repulsion": (None, [P, C.c_double, C.c_double, C.c_int]),
    "orc_set_boundary_repulsion": (None, [P, C.c_double, C.c_double, C.c_int]),
    "orc_stage_repulsion": (None, [P]),
    "orc_read_repulsion": (None, [P, D]),
    "orc_stage_spread": (None, [P]),
    "orc_stage_collide_stream": (None, [P]),
    "orc_stage_interpolate": (None, [P]),
    "orc_stage_advance": (None, [P]),
    "orc_stage_mechanics": (None, [P, C.c_int]),
    "orc_num_nodes": (C.c_long, [P]),
    "orc_num_vertices": (C.c_int, [P]),
    "orc_num_cells": (C.c_int, [P]),
    "orc_iter": (C.c_int, [P]),
    "orc_read_fluid": (None, [P, D, D]),
    "orc_read_populations": (None, [P, D]),
    "orc_write_populations": (None, [P, D]),
    "orc_read_force_field": (None, [P, D, C.c_int]),
    "orc_write_force_field": (None, [P, D]),
    "orc_read_vertices": (None, [P, D, D, D]),
    "orc_write_vertices": (None, [P, D, D, D]),
    "orc_read_cells": (None, [P, I, D]),
    "orc_bins": (C.c_int, [P, C.c_int, C.c_int, C.c_int, D, I, I, I, I, I, I, C.c_int]),
    "orc_neighbours": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, I, I, I, I, C.c_int]),
    "orc_type_sizes": (C.c_int, [P, C.c_int, I]),
    "orc_type_constants": (None, [P, C.c_int, I, D, D, I, I, D, D, I, D]),
    "orc_units": (None, [C.c_double] * 6 + [D]),
    "orc_material_scale": (None, [C.c_int, C.c_int, D, C.c_double, C.c_double, D, D]),
    "orc_mesh_icosphere": (C.c_int, [C.c_int, C.c_double, D, C.c_int, I, C.c_int, I, I]),
    "orc_mesh_rbc": (C.c_int, [C.c_int, C.c_double, D, C.c_int, I, C.c_int, I, I]),
    "orc_mesh_ellipsoid": (C.c_int, [C.c_int, C.c_double, C.c_double, D, C.c_int, I, C.c_int, I, I]),
    "orc_mesh_antipodal_pairs": (C.c_int, [D, C.c_int, I, C.c_int]),
    "orc_place_cells": (None, [D, C.c_int, C.c_int, D, D, D]),
    "orc_pos_to_lattice": (None, [C.c_int, D, D, C.c_double, D, D]),
    "orc_pack_cells": (C.c_int, [C.c_int, C.c_int, C.c_int, I, U8, C.c_int, C.POINTER(D), I, C.POINTER(I), I, I,
                                 C.c_double, C.c_ulonglong, C.c_int, D, D, I]),
}

_lib = None


def build() -> str:
    """Compile liboracle.so with its Makefile (g++, OpenMP)."""
    r = subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        for n, (r, a) in _SIG.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(D)


def _i(a):
    return None if a is None else a.ctypes.data_as(I)


def units(dx, dt, nu_p, rho_p, kBT_p, tau_override) -> np.ndarray:
    out = np.zeros(6)
    lib().orc_units(dx, dt, nu_p, rho_p, kBT_p, tau_override, _d(out))
    return out


def material_scale(model: int, nfaces: int, u: np.ndarray, dx: float, dt: float, mat: np.ndarray) -> np.ndarray:
    k = np.zeros(9)
    lib().orc_material_scale(model, nfaces, _d(np.ascontiguousarray(u, np.float64)), dx, dt,
                             _d(np.ascontiguousarray(mat, np.float64)), _d(k))
    return k


class Oracle:
    def __init__(self, nx, ny, nz, periodic=(1, 1, 1), tau=1.0, f_limit=1e300, threads: int = 0):
        self.L = lib()
        if threads:
            self.L.orc_set_threads(threads)
        self.s = C.c_void_p(self.L.orc_create(nx, ny, nz, *[int(p) for p in periodic], tau, f_limit))
        self.N = nx * ny * nz
        self.type_nv = []

    def __del__(self):
        if getattr(self, "s", None):
            self.L.orc_destroy(self.s)
            self.s = None

    def set_flags(self, flags):
        f = np.ascontiguousarray(flags, np.uint8)
        self.L.orc_set_flags(self.s, f.ctypes.data_as(U8))

    def set_wall_velocity(self, cls, u):
        self.L.orc_set_wall_velocity(self.s, cls, _d(np.ascontiguousarray(u, np.float64)))

    def set_body_force(self, mode, p):
        self.L.orc_set_body_force(self.s, mode, _d(np.ascontiguousarray(p, np.float64)))

    def init_equilibrium(self, rho=1.0, u=(0, 0, 0)):
        self.L.orc_init_equilibrium(self.s, rho, _d(np.ascontiguousarray(u, np.float64)))

    def add_cell_type(self, model, xyz, tris, inner, k):
        xyz = np.ascontiguousarray(xyz, np.float64)
        tris = np.ascontiguousarray(tris, np.int32)
        inner = np.ascontiguousarray(inner, np.int32).reshape(-1, 2)
        k = np.ascontiguousarray(k, np.float64)
        self.type_nv.append(xyz.shape[0])
        return self.L.orc_add_cell_type(self.s, model, xyz.shape[0], _d(xyz), tris.shape[0], _i(tris),
                                        inner.shape[0], _i(inner) if len(inner) else None, _d(k))

    def add_cell(self, t, xyz):
        return self.L.orc_add_cell(self.s, t, _d(np.ascontiguousarray(xyz, np.float64)))

    def set_timescales(self, every, velocity_every=1):
        e = np.ascontiguousarray(every, np.int32)
        self.L.orc_set_timescales(self.s, _i(e), velocity_every)

    def set_vertex_forces(self, ids, forces):
        ids = np.ascontiguousarray(ids, np.int32).reshape(-1)
        forces = np.ascontiguousarray(forces, np.float64).reshape(-1, 3)
        self.L.orc_set_vertex_forces(self.s, len(ids), _i(ids), _d(forces))

    def set_repulsion(self, k, cutoff_lu, every=1):
        self.L.orc_set_repulsion(self.s, float(k), float(cutoff_lu), int(every))

    def set_boundary_repulsion(self, k, cutoff_lu, every=1):
        self.L.orc_set_boundary_repulsion(self.s, float(k), float(cutoff_lu), int(every))

    def read_repulsion(self):
        f = np.zeros((self.nvertices(), 3))
        self.L.orc_read_repulsion(self.s, _d(f))
        return f

    def step(self, n=1):
        self.L.orc_step(self.s, n)

    def stage(self, name, forced=1):
        if name == "repulsion":
            self.L.orc_stage_repulsion(self.s)
        elif name == "mechanics":
            self.L.orc_stage_mechanics(self.s, forced)
        else:
            getattr(self.L, "orc_stage_" + name)(self.s)

    def read_fluid(self):
        rho = np.zeros(self.N)
        u = np.zeros(3 * self.N)
        self.L.orc_read_fluid(self.s, _d(rho), _d(u))
        return rho, u.reshape(3, self.N)

    def read_populations(self):
        f = np.zeros(19 * self.N)
        self.L.orc_read_populations(self.s, _d(f))
        return f.reshape(19, self.N)

    def write_populations(self, f):
        self.L.orc_write_populations(self.s, _d(np.ascontiguousarray(f, np.float64).reshape(-1)))

    def read_force_field(self, which=0):
        F = np.zeros(3 * self.N)
        self.L.orc_read_force_field(self.s, _d(F), which)
        return F.reshape(3, self.N)

    def write_force_field(self, F):
        self.L.orc_write_force_field(self.s, _d(np.ascontiguousarray(F, np.float64).reshape(-1)))

    def nvertices(self):
        return self.L.orc_num_vertices(self.s)

    def read_vertices(self):
        V = self.nvertices()
        x, v, f = np.zeros((V, 3)), np.zeros((V, 3)), np.zeros((V, 3))
        self.L.orc_read_vertices(self.s, _d(x), _d(v), _d(f))
        return x, v, f

    def write_vertices(self, x=None, v=None, f=None):
        conv = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (x, v, f)]
        self.L.orc_write_vertices(self.s, *[_d(a) for a in conv])

    def read_cells(self):
        n = self.L.orc_num_cells(self.s)
        alive = np.zeros(n, np.int32)
        vol = np.zeros(n)
        self.L.orc_read_cells(self.s, _i(alive), _d(vol))
        return alive, vol

    def bins(self, tile=(8, 8, 8), x=None, dims=None):
        V = self.nvertices()
        nx, ny, nz = dims
        nt = -(-nx // tile[0]) * -(-ny // tile[1]) * -(-nz // tile[2])
        vn, vt = np.zeros(max(V, 1), np.int32), np.zeros(max(V, 1), np.int32)
        to, tco = np.zeros(nt + 1, np.int32), np.zeros(nt + 1, np.int32)
        tv, tc = np.zeros(max(V, 1), np.int32), np.zeros(max(V, 1), np.int32)
        xx = None if x is None else np.ascontiguousarray(x, np.float64)
        r = self.L.orc_bins(self.s, *tile, _d(xx), _i(vn), _i(vt), _i(to), _i(tv), _i(tco), _i(tc), max(V, 1))
        assert r == nt
        return dict(vertex_node=vn[:V], vertex_tile=vt[:V], tile_offsets=to, tile_vertices=tv[: to[nt]],
                    tile_cell_offsets=tco, tile_cells=tc[: tco[nt]])

    def neighbours(self, tile=(8, 8, 8), x=None, dims=None, periodic=(1, 1, 1)):
        """Per tile, the sorted distinct cells of the tile and its 26 neighbours (CSR)."""
        b = self.bins(tile, x, dims)
        nt3 = [-(-dims[a] // tile[a]) for a in range(3)]
        nt = nt3[0] * nt3[1] * nt3[2]
        cap = max(27 * len(b["tile_cells"]), 1)
        off, cells = np.zeros(nt + 1, np.int32), np.zeros(cap, np.int32)
        tco = np.ascontiguousarray(b["tile_cell_offsets"], np.int32)
        tc = np.ascontiguousarray(np.append(b["tile_cells"], 0), np.int32)
        r = self.L.orc_neighbours(*nt3, *[int(p) for p in periodic], _i(tco), _i(tc), _i(off), _i(cells), cap)
        assert r == nt
        return off, cells[: off[nt]].copy()

    def type_constants(self, t):
        sz = np.zeros(4, np.int32)
        self.L.orc_type_sizes(self.s, t, _i(sz))
        nv, nf, ne, ni = sz.tolist()
        out = dict(edges=np.zeros((ne, 2), np.int32), edge_l0=np.zeros(ne), edge_angle0=np.zeros(ne),
                   ring=np.zeros((nv, 6), np.int32), ring_n=np.zeros(nv, np.int32), patch_d0=np.zeros(nv),
                   tri_a0=np.zeros(nf), bend_outer=np.zeros((ne, 2), np.int32), scalars=np.zeros(4))
        self.L.orc_type_constants(self.s, t, _i(out["edges"]), _d(out["edge_l0"]), _d(out["edge_angle0"]),
                                  _i(out["ring"]), _i(out["ring_n"]), _d(out["patch_d0"]), _d(out["tri_a0"]),
                                  _i(out["bend_outer"]), _d(out["scalars"]))
        return out


def apply_case(case, threads: int = 0, dx=0.5e-6, dt=1e-7, rho_p=1025.0, kBT=4.100531391e-21) -> Oracle:
    """Build an oracle instance from a hemocell_gb300.cases.Case."""
    u = units(dx, dt, 0.0, rho_p, kBT, case.tau)
    o = Oracle(*case.dims, periodic=case.periodic, tau=u[0], f_limit=u[5], threads=threads)
    o.set_flags(case.flags_array())
    for cls, w in case.walls.items():
        o.set_wall_velocity(cls, w)
    o.init_equilibrium(1.0)
    o.set_body_force(case.body_mode, case.body)
    for t in case.types:
        k = material_scale(t.model, t.mesh.nf, u, dx, dt, t.material.as_array())
        o.add_cell_type(t.model, t.mesh.xyz, t.mesh.tris, t.mesh.inner, k)
    for t, xyz in case.cells:
        o.add_cell(t, xyz)
    return o


# ---------------------------------------------------------------------------
# Cell geometry (oracle/geometry.cpp): the oracle's own mesh generators,
# placement and packer.  ``geometry`` offers the functions a workload builder
# needs (the same names and argument meaning as the product's), so a
# hemocell_gb300.cases workload can be built without the product library.

class Mesh:
    """A closed triangle mesh: xyz (nv, 3) lattice units, tris (nf, 3)
    outward oriented, inner (ni, 2) inner-link vertex pairs."""

    def __init__(self, xyz, tris, inner=None):
        self.xyz = xyz
        self.tris = tris
        self.inner = np.zeros((0, 2), np.int32) if inner is None else inner

    @property
    def nv(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def nf(self) -> int:
        return int(self.tris.shape[0])


def _mesh(fn, *args, min_triangles):
    nf_cap = 20
    while nf_cap < min_triangles:
        nf_cap *= 4
    nv_cap = nf_cap // 2 + 2
    xyz = np.zeros((nv_cap, 3))
    tris = np.zeros((nf_cap, 3), np.int32)
    nv, nf = C.c_int(), C.c_int()
    rc = fn(*args, _d(xyz), nv_cap, _i(tris), nf_cap, C.byref(nv), C.byref(nf))
    if rc != 0:
        raise RuntimeError("oracle mesh buffers too small")
    return Mesh(xyz[: nv.value].copy(), tris[: nf.value].copy())


class _Geometry:
    """Workload geometry from the oracle alone (helper/meshGeneratingFunctions.hh,
    io/readPositionsBloodCells.cpp, and the project's seeded packer)."""

    @staticmethod
    def icosphere(min_triangles: int, radius: float) -> Mesh:
        return _mesh(lib().orc_mesh_icosphere, min_triangles, radius, min_triangles=min_triangles)

    @staticmethod
    def rbc_mesh(min_triangles: int, radius: float) -> Mesh:
        return _mesh(lib().orc_mesh_rbc, min_triangles, radius, min_triangles=min_triangles)

    @staticmethod
    def ellipsoid_mesh(min_triangles: int, radius: float, aspect: float) -> Mesh:
        return _mesh(lib().orc_mesh_ellipsoid, min_triangles, radius, aspect, min_triangles=min_triangles)

    @staticmethod
    def antipodal_pairs(xyz) -> np.ndarray:
        xyz = np.ascontiguousarray(xyz, np.float64)
        out = np.zeros((max(xyz.shape[0], 1), 2), np.int32)
        n = lib().orc_mesh_antipodal_pairs(_d(xyz), xyz.shape[0], _i(out), out.shape[0])
        if n < 0:
            raise RuntimeError("antipodal pair buffer too small")
        return out[:n].copy()

    @staticmethod
    def place_cells(mesh, centres, angles) -> np.ndarray:
        centres = np.ascontiguousarray(centres, np.float64).reshape(-1, 3)
        angles = np.ascontiguousarray(angles, np.float64).reshape(-1, 3)
        n = centres.shape[0]
        out = np.zeros((n * mesh.nv, 3))
        lib().orc_place_cells(_d(np.ascontiguousarray(mesh.xyz, np.float64)), mesh.nv, n, _d(centres), _d(angles),
                              _d(out))
        return out

    @staticmethod
    def pos_to_lattice(pos_um, angles_deg, dx):
        pos = np.ascontiguousarray(pos_um, np.float64).reshape(-1, 3)
        ang = np.ascontiguousarray(angles_deg, np.float64).reshape(-1, 3)
        c, a = np.zeros_like(pos), np.zeros_like(ang)
        lib().orc_pos_to_lattice(pos.shape[0], _d(pos), _d(ang), float(dx), _d(c), _d(a))
        return c, a

    @staticmethod
    def pack_cells(dims, periodic, solid, meshes, counts, margin, seed, max_attempts=20000):
        nt = len(meshes)
        total = int(sum(counts))
        xyzs = [np.ascontiguousarray(m.xyz, np.float64) for m in meshes]
        triss = [np.ascontiguousarray(m.tris, np.int32) for m in meshes]
        xp = (D * nt)(*[_d(a) for a in xyzs])
        tp = (I * nt)(*[_i(a) for a in triss])
        nvs = np.array([m.nv for m in meshes], np.int32)
        nfs = np.array([m.nf for m in meshes], np.int32)
        cnt = np.array(counts, np.int32)
        per = np.array(periodic, np.int32)
        centres = np.zeros((max(total, 1), 3))
        angles = np.zeros((max(total, 1), 3))
        types = np.zeros(max(total, 1), np.int32)
        sp = None if solid is None else np.ascontiguousarray(solid, np.uint8).ctypes.data_as(U8)
        n = lib().orc_pack_cells(dims[0], dims[1], dims[2], _i(per), sp, nt, xp, _i(nvs), tp, _i(nfs), _i(cnt),
                                 float(margin), C.c_ulonglong(seed), max_attempts, _d(centres), _d(angles), _i(types))
        return centres[:n].copy(), angles[:n].copy(), types[:n].copy()


geometry = _Geometry()
