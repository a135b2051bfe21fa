"""STL ingestion (getFlagMatrixFromSTL, helper/voxelizeDomain.cpp): a closed
tube written here as binary and as ASCII STL voxelises to the analytic
cylinder, with both ends opened by copying the neighbouring slices.  No GPU."""
import numpy as np
import pytest


def tube_triangles(radius, length, segments=96):
    """Closed cylinder along x: side quads as two triangles each, two caps."""
    th = np.linspace(0.0, 2 * np.pi, segments, endpoint=False)
    ring = np.stack([np.cos(th), np.sin(th)], axis=1) * radius
    tris = []
    for k in range(segments):
        a, b = ring[k], ring[(k + 1) % segments]
        p0, p1 = [0.0, *a], [0.0, *b]
        q0, q1 = [length, *a], [length, *b]
        tris += [(p0, q0, q1), (p0, q1, p1)]
        tris += [([0.0, 0.0, 0.0], p1, p0), ([length, 0.0, 0.0], q0, q1)]
    return np.array(tris, np.float64)


def write_binary(path, tris):
    with open(path, "wb") as fh:
        fh.write(b"\0" * 80)
        fh.write(np.uint32(len(tris)).tobytes())
        for t in tris:
            fh.write(np.zeros(3, np.float32).tobytes() + t.astype(np.float32).tobytes() + b"\0\0")


def write_ascii(path, tris):
    with open(path, "w") as fh:
        fh.write("solid tube\n")
        for t in tris:
            fh.write(" facet normal 0 0 0\n  outer loop\n")
            for v in t:
                fh.write(f"   vertex {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}\n")
            fh.write("  endloop\n endfacet\n")
        fh.write("endsolid tube\n")


@pytest.mark.parametrize("fmt", ["binary", "ascii"])
def test_tube_voxelises_to_the_cylinder(built, tmp_path, fmt):
    from hemocell_gb300.hemocell import voxelize_stl
    R, Lx = 7.3, 40.0
    path = str(tmp_path / f"tube_{fmt}.stl")
    (write_binary if fmt == "binary" else write_ascii)(path, tube_triangles(R, Lx))
    # 40 units long -> 80 lattice units: scale 2, radius 14.6 lattice units
    flags, dims = voxelize_stl(path, ref_dir=0, ref_length=80.0, margin=1, open_ends=True)
    nx, ny, nz = dims
    assert (nx, ny, nz) == (83, 33, 33)
    f = flags.reshape(nz, ny, nx)
    zz, yy = np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij")
    r = np.hypot(yy - (1 + 14.6), zz - (1 + 14.6))
    for X in (0, 1, 2, 40, nx - 2, nx - 1):
        sl = f[:, :, X]
        assert np.all(sl[r < 14.6 - 0.2] == 0), X      # inside: fluid
        assert np.all(sl[r > 14.6 + 0.2] == 1), X      # outside: wall
    # the open ends repeat the interior slices next to them
    assert np.array_equal(f[:, :, 0], f[:, :, 2]) and np.array_equal(f[:, :, nx - 1], f[:, :, nx - 3])


def test_closed_tube_keeps_its_caps(built, tmp_path):
    from hemocell_gb300.hemocell import voxelize_stl
    path = str(tmp_path / "tube.stl")
    write_binary(path, tube_triangles(5.0, 20.0))
    flags, dims = voxelize_stl(path, ref_dir=0, ref_length=20.0, margin=2, open_ends=False)
    f = flags.reshape(dims[2], dims[1], dims[0])
    assert np.all(f[:, :, 0] == 1) and np.all(f[:, :, 1] == 1)     # before the cap: outside
    assert np.any(f[:, :, 10] == 0)


def test_bad_stl_reports_the_reason(built, tmp_path):
    from hemocell_gb300.hemocell import HemoCellError, voxelize_stl
    p = tmp_path / "junk.stl"
    p.write_text("not an stl")
    with pytest.raises(HemoCellError, match="neither"):
        voxelize_stl(str(p))
