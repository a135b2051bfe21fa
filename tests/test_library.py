"""Host-side checks of the C ABI library (no GPU): it loads, exports every
symbol declared in include/hemocell_gb300.h, and its host helpers (meshes,
placement, packing, argument validation) behave."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "hemocell_gb300.h")).read()
    return sorted(set(re.findall(r"\b(hc_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(built):
    from hemocell_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_mesh_counts_and_closure(built):
    from hemocell_gb300 import cases, icosphere, rbc_mesh, ellipsoid_mesh
    for m, nv, nf in [(rbc_mesh(600, 7.82), 642, 1280), (ellipsoid_mesh(320, 2.0, 0.25), 162, 320),
                      (icosphere(5120, 8.0), 2562, 5120), (icosphere(80, 1.0), 42, 80)]:
        assert (m.nv, m.nf) == (nv, nf)
        assert m.nv - 3 * m.nf // 2 + m.nf == 2  # Euler characteristic of a sphere
        directed = set()
        for t in m.tris.tolist():
            for k in range(3):
                e = (t[k], t[(k + 1) % 3])
                assert e not in directed
                directed.add(e)
        assert all((b, a) in directed for a, b in directed)
        assert cases.mesh_volume(m) > 0  # outward orientation


def test_rbc_shape(built):
    """The biconcave template after the shape constructor's fixed rotation
    (pi/2, pi/2, 0): its axis lies along y, the disc spans x and z."""
    from hemocell_gb300 import cases, rbc_mesh
    m = rbc_mesh(600, 7.82)
    r = np.hypot(m.xyz[:, 0], m.xyz[:, 2])
    assert abs(r.max() - 7.82) < 1e-9
    assert 2.2 < m.xyz[:, 1].max() < 2.4   # Evans-Fung maximum half thickness ~0.29 R
    # the continuous Evans-Fung shape of R = 3.91 um encloses 81.76 um^3; the
    # 1280-face mesh a little less
    vol_um3 = cases.mesh_volume(m) * 0.5 ** 3
    assert 80.5 < vol_um3 < 81.76


def test_antipodal_pairs(built):
    from hemocell_gb300 import antipodal_pairs, icosphere
    m = icosphere(1280, 3.0)
    p = antipodal_pairs(m.xyz)
    assert len(p) == m.nv // 2
    assert np.allclose(m.xyz[p[:, 0]], -m.xyz[p[:, 1]])


def test_placement_matches_reference_rotation(built):
    from hemocell_gb300 import place_cells, rbc_mesh
    m = rbc_mesh(80, 4.0)
    ang = np.array([[0.3, -1.1, 2.0]])
    cen = np.array([[10.0, 11.0, 12.0]])
    got = place_cells(m, cen, ang)
    a, b, g = ang[0]
    # io/readPositionsBloodCells.cpp:39-118 column-first factors, product Rz*Ry*Rx
    Ax = np.array([[1, 0, 0], [0, np.cos(a), np.sin(a)], [0, -np.sin(a), np.cos(a)]])
    By = np.array([[np.cos(b), 0, -np.sin(b)], [0, 1, 0], [np.sin(b), 0, np.cos(b)]])
    Cz = np.array([[np.cos(g), np.sin(g), 0], [-np.sin(g), np.cos(g), 0], [0, 0, 1]])
    M = Cz @ By @ Ax
    c0 = (m.xyz.min(axis=0) + m.xyz.max(axis=0)) / 2
    expect = (m.xyz - c0) @ M.T + cen
    assert np.allclose(got, expect, atol=1e-12)


def test_stretch_cell_disc_lies_in_the_xy_plane(built):
    """stretch_RBC.pos places the cell with angles (90, 0, 0): the template's
    y axis turns onto z, so the disc spans x and y as the validation measures
    its axial (x) and transverse (y) diameters."""
    from hemocell_gb300 import cases
    xyz = cases.stretch_cell(320).cells[0][1]
    ext = np.ptp(xyz, axis=0) * 0.5          # micrometres
    assert abs(ext[0] - 7.82) < 1e-6 and abs(ext[1] - 7.82) < 1e-6
    assert ext[2] < 2.7


def test_packing_seeded_and_disjoint(built):
    from hemocell_gb300 import cases, pack_cells, rbc_mesh
    m = rbc_mesh(320, 7.82)
    flags = cases.cylinder_flags(40, 40, 48, 18.0)
    c1, a1, t1 = pack_cells((40, 40, 48), (1, 1, 1), flags, [m], [12], margin=1.0, seed=4)
    c2, a2, t2 = pack_cells((40, 40, 48), (1, 1, 1), flags, [m], [12], margin=1.0, seed=4)
    assert len(c1) == 12 and np.array_equal(c1, c2) and np.array_equal(a1, a2)
    # nearest nodes of different cells never coincide and never touch a wall
    from hemocell_gb300 import place_cells
    xyz = place_cells(m, c1, a1)
    nodes = np.floor(xyz + 0.5).astype(int) % np.array([40, 40, 48])
    idx = nodes[:, 0] + 40 * (nodes[:, 1] + 40 * nodes[:, 2])
    owner = np.repeat(np.arange(12), m.nv)
    seen = {}
    for i, o in zip(idx.tolist(), owner.tolist()):
        assert seen.setdefault(i, o) == o
    assert flags[idx].max() == 0


def test_create_rejects_bad_parameters(built):
    from hemocell_gb300 import HemoCell, HemoCellError
    with pytest.raises(HemoCellError, match="positive"):
        HemoCell(0, 4, 4)
    with pytest.raises(HemoCellError, match="tau"):
        HemoCell(4, 4, 4, tau=0.4)
    with pytest.raises(HemoCellError, match="form"):
        HemoCell(4, 4, 4, form=7)
