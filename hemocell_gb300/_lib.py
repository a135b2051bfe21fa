"""ctypes binding of ``libhcgpu.so`` (the C ABI declared in include/hemocell_gb300.h).

The library is built in-tree by :func:`hemocell_gb300.build.build`.  Loading
fails loudly when it is missing: there is no CPU fallback for the step.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# HEMOCELL_GB300_CHECKED=1 loads the bounds-checked build (hemocell_gb300.build
# build(checked=True)) in place of the product library
LIB_PATH = os.path.join(HERE, "libhcgpu_checked.so" if os.environ.get("HEMOCELL_GB300_CHECKED") == "1"
                        else "libhcgpu.so")

HC_OK = 0
HC_ERR_INVALID = -1
HC_ERR_CUDA = -2
HC_ERR_MEMORY = -3
HC_ERR_STATE = -4
HC_ERR_NUMERIC = -5

HC_FORM_PLAIN_F64 = 0
HC_FORM_MIXED_F32 = 1
HC_LAUNCH_PER_STAGE = 0
HC_LAUNCH_BATCHED = 1
HC_MODEL_RBC_HIGH_ORDER = 0
HC_MODEL_PLT_SIMPLE = 1
HC_MODEL_WBC_HIGH_ORDER = 2
HC_BODY_NONE = 0
HC_BODY_UNIFORM = 1
HC_BODY_KOLMOGOROV = 2
HC_STAGE_SPREAD = 0
HC_STAGE_COLLIDE_STREAM = 1
HC_STAGE_INTERPOLATE = 2
HC_STAGE_ADVANCE = 3
HC_STAGE_MECHANICS = 4
HC_STAGE_MECHANICS_FORCED = 5
HC_STAGE_BIN = 6
HC_STAGE_REPULSION = 7


class hc_params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("periodic", C.c_int * 3),
                ("dx", C.c_double), ("dt", C.c_double), ("nu_p", C.c_double), ("rho_p", C.c_double),
                ("kBT_p", C.c_double), ("tau", C.c_double), ("form", C.c_int), ("launch", C.c_int),
                ("device", C.c_int), ("tile", C.c_int * 3)]


class hc_material(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("kLink", "kBend", "kVolume", "kArea", "eta_m", "kInnerRigid",
                                          "kCytoskeleton", "coreRadius", "radius")]


class hc_stats(C.Structure):
    _fields_ = [("nodes", C.c_longlong), ("vertices", C.c_int), ("cells", C.c_int), ("cells_alive", C.c_int),
                ("types", C.c_int), ("iter", C.c_int), ("tau", C.c_double), ("omega", C.c_double),
                ("device_bytes", C.c_longlong)]


class hc_batch_stats(C.Structure):
    _fields_ = [("active", C.c_int), ("finished", C.c_int), ("popped", C.c_int), ("max_slots", C.c_int),
                ("budget_bytes", C.c_longlong), ("bytes_in_use", C.c_longlong), ("admitted", C.c_longlong),
                ("completed", C.c_longlong), ("refused", C.c_longlong), ("steps_enqueued", C.c_longlong)]


P = C.c_void_p
D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
U8 = C.POINTER(C.c_uint8)

# name: (restype, argtypes)
SIGNATURES = {
    "hc_create": (P, [C.POINTER(hc_params)]),
    "hc_destroy": (C.c_int, [P]),
    "hc_last_error": (C.c_char_p, [P]),
    "hc_derived_units": (C.c_int, [P, D]),
    "hc_set_flags": (C.c_int, [P, U8]),
    "hc_set_wall_velocity": (C.c_int, [P, C.c_int, D]),
    "hc_set_body_force": (C.c_int, [P, C.c_int, D]),
    "hc_init_equilibrium": (C.c_int, [P, C.c_double, D]),
    "hc_add_cell_type": (C.c_int, [P, C.c_char_p, C.c_int, C.POINTER(hc_material), D, C.c_int, I, C.c_int, I,
                                   C.c_int]),
    "hc_add_cells": (C.c_int, [P, C.c_int, C.c_int, D, D]),
    "hc_add_cells_xyz": (C.c_int, [P, C.c_int, C.c_int, D]),
    "hc_load_cells": (C.c_int, [P, C.c_int, C.c_int, D, D, I]),
    "hc_set_timescales": (C.c_int, [P, I, C.c_int, C.c_int]),
    "hc_set_vertex_forces": (C.c_int, [P, C.c_int, I, D]),
    "hc_set_repulsion": (C.c_int, [P, C.c_double, C.c_double, C.c_int]),
    "hc_set_boundary_repulsion": (C.c_int, [P, C.c_double, C.c_double, C.c_int]),
    "hc_read_repulsion": (C.c_int, [P, D]),
    "hc_step": (C.c_int, [P, C.c_int]),
    "hc_stage": (C.c_int, [P, C.c_int]),
    "hc_sync": (C.c_int, [P]),
    "hc_time_steps": (C.c_int, [P, C.c_int, D]),
    "hc_profile_stages": (C.c_int, [P, C.c_int, D]),
    "hc_profile_kernels": (C.c_int, [P, C.c_int, D]),
    "hc_read_positions_async": (C.c_int, [P, D, C.c_int]),
    "hc_wait_positions": (C.c_int, [P, C.c_int]),
    "hc_vertex_count": (C.c_int, [P]),
    "hc_read_neighbours": (C.c_int, [P, I, I, C.c_int]),
    "hc_read_fluid": (C.c_int, [P, D, D]),
    "hc_read_populations": (C.c_int, [P, D]),
    "hc_write_populations": (C.c_int, [P, D]),
    "hc_read_force_field": (C.c_int, [P, D, C.c_int]),
    "hc_write_force_field": (C.c_int, [P, D]),
    "hc_read_vertices": (C.c_int, [P, D, D, D]),
    "hc_write_vertices": (C.c_int, [P, D, D, D]),
    "hc_read_cells": (C.c_int, [P, I, D]),
    "hc_read_bins": (C.c_int, [P, I, I, I, I, I, I, C.c_int]),
    "hc_bin_tiles_noalloc": (C.c_int, [P, P, C.c_int, C.c_int, P, P, P, P, C.c_int, P]),
    "hc_cell_info": (C.c_int, [P, D]),
    "hc_write_cell_info_csv": (C.c_int, [P, C.c_char_p, C.c_int]),
    "hc_write_output": (C.c_int, [P, C.c_char_p, C.c_int]),
    "hc_save_checkpoint": (C.c_int, [P, C.c_char_p]),
    "hc_load_checkpoint": (C.c_int, [P, C.c_char_p]),
    "hc_get_stats": (C.c_int, [P, C.POINTER(hc_stats)]),
    "hc_device_status": (C.c_int, [P, C.POINTER(C.c_uint)]),
    "hc_autotune": (C.c_int, [P, C.c_char_p]),
    "hc_get_tuning": (C.c_int, [P, I]),
    "hc_set_tuning": (C.c_int, [P, I]),
    "hc_stl_voxelize": (C.c_int, [C.c_char_p, C.c_int, C.c_double, C.c_int, C.c_int, I, U8, C.c_longlong]),
    "hc_mesh_icosphere": (C.c_int, [C.c_int, C.c_double, D, C.c_int, I, C.c_int, I, I]),
    "hc_mesh_rbc": (C.c_int, [C.c_int, C.c_double, D, C.c_int, I, C.c_int, I, I]),
    "hc_mesh_ellipsoid": (C.c_int, [C.c_int, C.c_double, C.c_double, D, C.c_int, I, C.c_int, I, I]),
    "hc_mesh_antipodal_pairs": (C.c_int, [D, C.c_int, I, C.c_int]),
    "hc_place_cells": (C.c_int, [D, C.c_int, C.c_int, D, D, D]),
    "hc_pack_cells": (C.c_int, [C.c_int, C.c_int, C.c_int, I, U8, C.c_int, C.POINTER(D), I, C.POINTER(I), I, I,
                                C.c_double, C.c_ulonglong, C.c_int, D, D, I]),
    "hc_estimate_device_bytes": (C.c_longlong, [C.POINTER(hc_params), C.c_int, C.c_int]),
    "hc_batch_create": (P, [C.c_int, C.c_longlong, C.c_int, C.c_int]),
    "hc_batch_destroy": (C.c_int, [P]),
    "hc_batch_last_error": (C.c_char_p, [P]),
    "hc_batch_fits": (C.c_int, [P, C.c_longlong]),
    "hc_batch_admit": (C.c_int, [P, P, C.c_int, C.c_longlong]),
    "hc_batch_pump": (C.c_int, [P, C.c_double]),
    "hc_batch_pop": (C.c_int, [P, C.POINTER(C.c_longlong), C.POINTER(P), I]),
    "hc_batch_release": (C.c_int, [P, P, C.c_int]),
    "hc_batch_get_stats": (C.c_int, [P, C.POINTER(hc_batch_stats)]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libhcgpu.so once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the GB300 step has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib
