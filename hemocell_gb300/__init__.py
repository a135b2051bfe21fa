"""GB300-native HemoCell IB-LBM time step.

The step (HemoCell::iterate) runs as hand-written sm_103a CUDA kernels in
``libhcgpu.so`` behind the C ABI of ``include/hemocell_gb300.h``; this
package holds the ctypes binding, a Python mirror of the HemoCell case API
and the seeded workload builders.
"""
from . import _lib
from .hemocell import HemoCell, HemoCellError, Material, Mesh, antipodal_pairs, ellipsoid_mesh, icosphere, \
    pack_cells, place_cells, rbc_mesh

__all__ = ["HemoCell", "HemoCellError", "Material", "Mesh", "antipodal_pairs", "ellipsoid_mesh", "icosphere",
           "pack_cells", "place_cells", "rbc_mesh", "_lib"]
