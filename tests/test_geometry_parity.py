"""The product's cell geometry against the oracle's own restatement, bit for
bit (CPU only): the mesh generators of helper/meshGeneratingFunctions.hh:31-271
(icosphere, the Evans-Fung RBC with the constructor's fixed rotation, the
ellipsoid), the antipodal inner links, loadParticles' placement
(io/readPositionsBloodCells.cpp:39-124, 290-361), the .pos unit conversion,
and the seeded packer, up to the full benchmark pipe.  The product side runs
the host code of libhcgpu.so; no GPU is needed."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def geo(built):
    from hemocell_gb300 import cases
    from oracle import oracle as orc
    return cases.PRODUCT, orc.geometry


def _same_mesh(a, b):
    return a.nv == b.nv and np.array_equal(a.xyz, b.xyz) and np.array_equal(a.tris, b.tris)


@pytest.mark.parametrize("fn,args", [("icosphere", (80, 1.0)), ("icosphere", (1280, 3.0)), ("icosphere", (5120, 8.0)),
                                     ("rbc_mesh", (320, 7.82)), ("rbc_mesh", (600, 7.82)),
                                     ("ellipsoid_mesh", (80, 2.0, 0.4)), ("ellipsoid_mesh", (320, 2.0, 0.25))])
def test_meshes_bit_exact(geo, fn, args):
    prod, orc = geo
    a, b = getattr(prod, fn)(*args), getattr(orc, fn)(*args)
    assert _same_mesh(a, b)
    assert np.array_equal(prod.antipodal_pairs(a.xyz), orc.antipodal_pairs(b.xyz))


def test_placement_and_pos_conversion_bit_exact(geo):
    prod, orc = geo
    m = prod.rbc_mesh(600, 7.82)
    rng = np.random.default_rng(7)
    pos = rng.uniform(0, 40, (20, 3))
    deg = rng.uniform(-180, 180, (20, 3))
    ca, aa = prod.pos_to_lattice(pos, deg, 0.5e-6)
    cb, ab = orc.pos_to_lattice(pos, deg, 0.5e-6)
    assert np.array_equal(ca, cb) and np.array_equal(aa, ab)
    assert np.array_equal(prod.place_cells(m, ca, aa), orc.place_cells(m, cb, ab))


@pytest.mark.parametrize("builder,kw", [
    ("mixed_box", {}),
    ("repulsion_box", {}),
    ("stretch_cell", {"min_triangles": 320}),
    ("shear_single_rbc", {"n": 50, "seed": 1}),
    ("kolmogorov_mix", {"n": 40, "rbc_fraction": 0.25, "n_wbc": 1, "plt_per_rbc": 0.2, "wbc_triangles": 1280,
                        "seed": 3}),
    ("pipe_ht25", {"seed": 1}),          # the benchmark workload: 279 RBC, about 10 s per side
])
def test_workloads_bit_exact(geo, builder, kw):
    """Every seeded workload, including its packing, is the same whichever
    side builds it."""
    from hemocell_gb300 import cases
    prod, orc = geo
    a = getattr(cases, builder)(geo=prod, **kw)
    b = getattr(cases, builder)(geo=orc, **kw)
    assert len(a.cells) == len(b.cells) > 0
    for (ta, xa), (tb, xb) in zip(a.cells, b.cells):
        assert ta == tb and np.array_equal(xa, xb)
    for sa, sb in zip(a.types, b.types):
        assert _same_mesh(sa.mesh, sb.mesh) and np.array_equal(sa.mesh.inner, sb.mesh.inner)
