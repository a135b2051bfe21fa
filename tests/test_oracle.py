"""The FP64 CPU oracle against what pins it: unit constants derived by hand
from the reference's formulas, analytic LBM solutions, conservation laws of
the membrane models, and the committed golden vectors.  No GPU needed."""
import itertools

import numpy as np
import pytest

from conftest import rel_l2


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def test_units_match_reference_formulas(orc):
    # tau=1, dx=0.5um, dt=1e-7s, rhoP=1025, kBT=4.100531391e-21 (examples/oneCellShear/config.xml)
    u = orc.units(0.5e-6, 1e-7, 0.0, 1025.0, 4.100531391e-21, 1.0)
    tau, nu, dm, df, kbt, flim = u
    assert tau == 1.0 and abs(nu - 1 / 6) < 1e-16
    assert abs(dm - 1025 * 0.5e-6 ** 3) < 1e-30
    assert abs(df / 6.40625e-9 - 1) < 1e-12
    assert abs(kbt / (4.100531391e-21 / (6.40625e-9 * 0.5e-6)) - 1) < 1e-12
    assert abs(flim / (50e-12 / 6.40625e-9) - 1) < 1e-12
    # RBC material (examples/oneCellShear/RBC.xml): kLink 15, kBend 80, kVolume 20, kArea 5
    k = orc.material_scale(0, 1280, u, 0.5e-6, 1e-7, np.array([15, 80, 20, 5, 0, 0, 0, 0, 3.91e-6], float))
    assert abs(k[0] / (15 * kbt / (7.5e-9 / 0.5e-6)) - 1) < 1e-12
    assert abs(k[1] / (80 * kbt / (5e-7 / 0.5e-6)) - 1) < 1e-12
    assert abs(k[2] / (20 * kbt / (5e-7 / 0.5e-6)) - 1) < 1e-12
    assert abs(k[3] / (5 * kbt / (5e-7 / 0.5e-6)) - 1) < 1e-12
    # dt given, tau derived: tau = 3 nu dt/dx^2 + 1/2
    u2 = orc.units(0.5e-6, 0.5e-7, 1.1e-6, 1025.0, 4.100531391e-21, 0.0)
    assert abs(u2[0] - (3 * 1.1e-6 * 0.5e-7 / 0.25e-12 + 0.5)) < 1e-12


def _fluid_case(n, periodic, flags=None, walls=None, body=(0, 0, 0), mode=1):
    from hemocell_gb300 import cases
    return cases.Case("fluid", n, periodic, flags=flags, walls=walls or {}, body_mode=mode, body=body)


def test_couette_linear_profile(orc):
    """Moving bounce-back walls give the linear Couette profile; halfway
    bounce-back puts the walls at z=0.5 and z=nz-1.5."""
    from hemocell_gb300 import cases
    n = (4, 4, 18)
    flags, walls = cases.shear_walls(n, 1e5)
    o = orc.apply_case(_fluid_case(n, (1, 1, 0), flags, walls, mode=0))
    o.step(4000)
    _, u = o.read_fluid()
    ux = u[0].reshape(n[2], n[1], n[0])[:, 0, 0]
    uw = walls[1][0]
    z = np.arange(1, n[2] - 1)
    zb, zt = 0.5, n[2] - 1.5
    expect = uw + (-uw - uw) * (z - zb) / (zt - zb)
    assert np.max(np.abs(ux[1:-1] - expect)) < 1e-3 * abs(uw)


def test_poiseuille_parabolic_profile(orc):
    """Body-force-driven channel: u(z) = F/(2 nu) (z-zb)(zt-z) for BGK with
    halfway bounce-back at tau=1 (exact up to round-off for this scheme)."""
    n = (3, 3, 22)
    flags = np.zeros((n[2], n[1], n[0]), np.uint8)
    flags[0] = 1
    flags[-1] = 1
    F = 1e-6
    o = orc.apply_case(_fluid_case(n, (1, 1, 0), flags.reshape(-1), {1: (0, 0, 0)}, body=(F, 0, 0)))
    o.step(6000)
    _, u = o.read_fluid()
    ux = u[0].reshape(n[2], n[1], n[0])[:, 1, 1]
    nu = 1 / 6
    z = np.arange(1, n[2] - 1)
    zb, zt = 0.5, n[2] - 1.5
    expect = F / (2 * nu) * (z - zb) * (zt - z)
    assert rel_l2(ux[1:-1], expect) < 2e-3


def test_mass_conserved_periodic(orc):
    n = (8, 6, 5)
    rng = np.random.default_rng(0)
    o = orc.Oracle(*n, periodic=(1, 1, 1))
    w = np.array([1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6)
    f = w[:, None] * (1 + 0.01 * rng.standard_normal((19, np.prod(n))))
    o.write_populations(f)
    m0 = f.sum()
    o.step(50)
    assert abs(o.read_populations().sum() - m0) < 1e-11 * m0


def _single_cell(orc, spec, xyz):
    from hemocell_gb300 import cases
    n = (48, 48, 48)
    case = cases.Case("one", n, (1, 1, 1), types=[spec], cells=[(0, xyz)])
    return orc.apply_case(case)


@pytest.mark.parametrize("which", ["rbc", "plt", "wbc"])
def test_rest_shape_is_force_free_and_forces_balance(orc, which):
    from hemocell_gb300 import cases
    spec = {"rbc": lambda: cases.rbc_type(600), "plt": lambda: cases.plt_type(320),
            "wbc": lambda: cases.wbc_type(1280)}[which]()
    xyz = spec.mesh.xyz + 24.0
    o = _single_cell(orc, spec, xyz)
    o.stage("mechanics")
    _, _, f_rest = o.read_vertices()
    rng = np.random.default_rng(1)
    x = xyz + 0.05 * rng.standard_normal(xyz.shape)
    o.write_vertices(x, np.zeros_like(x), np.zeros_like(x))
    o.stage("mechanics")
    _, _, f = o.read_vertices()
    assert np.abs(f).max() > 1e-8
    assert np.abs(f_rest).max() < 1e-9 * np.abs(f).max()
    # internal forces sum to zero (link, area, volume, bending, inner links)
    assert np.abs(f.sum(axis=0)).max() < 1e-12 * np.abs(f).max() * len(f)


@pytest.mark.parametrize("which", ["rbc", "plt"])
def test_bending_and_volume_are_restoring(orc, which):
    """Pushing one vertex outward along its normal yields an inward force on it."""
    from hemocell_gb300 import cases
    spec = cases.rbc_type(600) if which == "rbc" else cases.plt_type(320)
    xyz = spec.mesh.xyz + 24.0
    o = _single_cell(orc, spec, xyz)
    c = xyz.mean(axis=0)
    i = int(np.argmax(np.linalg.norm(xyz - c, axis=1)))
    nrm = (xyz[i] - c) / np.linalg.norm(xyz[i] - c)
    x = xyz.copy()
    x[i] += 0.05 * nrm
    o.write_vertices(x, np.zeros_like(x), np.zeros_like(x))
    o.stage("mechanics")
    _, _, f = o.read_vertices()
    assert np.dot(f[i], nrm) < 0


def test_ring_and_edges_consistent(orc):
    from hemocell_gb300 import cases
    spec = cases.rbc_type(600)
    o = _single_cell(orc, spec, spec.mesh.xyz + 24.0)
    k = o.type_constants(0)
    assert k["edges"].shape == (1920, 2)
    assert np.all(k["edges"][:, 0] < k["edges"][:, 1])
    assert sorted(set(k["ring_n"].tolist())) == [5, 6]
    assert (k["ring_n"] == 5).sum() == 12
    # each ring entry is an edge neighbour
    es = set(map(tuple, k["edges"].tolist()))
    for v in range(0, 642, 37):
        for j in range(k["ring_n"][v]):
            a, b = sorted((v, int(k["ring"][v, j])))
            assert (a, b) in es
    vol_eq, area_mean, edge_mean, _ = k["scalars"]
    assert abs(vol_eq - cases.mesh_volume(spec.mesh)) < 1e-9 * vol_eq
    assert abs(area_mean - k["tri_a0"].mean()) < 1e-12
    assert abs(edge_mean - k["edge_l0"].mean()) < 1e-12


def test_repulsion_conserves_momentum_and_pushes_from_walls(built):
    """Inter-cell repulsion is pairwise equal and opposite (its sum vanishes);
    the wall term pushes the lower cell up, away from the bottom wall."""
    from hemocell_gb300 import cases
    from oracle import oracle as orc
    case = cases.repulsion_box()
    o = orc.apply_case(case)
    o.set_repulsion(1e-4, 2.0, 1)
    o.stage("repulsion")
    f = o.read_repulsion()
    assert np.count_nonzero(np.any(f != 0, axis=1)) > 50
    assert np.abs(f.sum(axis=0)).max() < 1e-12 * np.abs(f).sum()
    nv = case.cells[0][1].shape[0]
    assert f[:nv, 2].sum() < 0 < f[nv:, 2].sum()    # the stacked cells push apart
    w = orc.apply_case(case)
    w.set_boundary_repulsion(5e-5, 2.0, 1)
    w.stage("repulsion")
    fw = w.read_repulsion()
    assert fw[:nv, 2].sum() > 0 and np.all(fw[nv:] == 0)


def test_neighbour_lists_match_brute_force(orc):
    """The oracle's neighbour lists against a direct union over the 27 tiles
    around each tile (Python), periodic in x and y, walls in z."""
    from hemocell_gb300 import cases
    case = cases.mixed_box(wall=True)
    o = orc.apply_case(case, threads=1)
    o.step(2)
    tile = (4, 4, 4)
    b = o.bins(tile, None, case.dims)
    nt3 = [-(-case.dims[a] // tile[a]) for a in range(3)]
    tco, tc = b["tile_cell_offsets"], b["tile_cells"]
    off, cells = o.neighbours(tile, None, case.dims, case.periodic)
    expect_off, expect = [0], []
    for t in range(nt3[0] * nt3[1] * nt3[2]):
        c0 = (t % nt3[0], (t // nt3[0]) % nt3[1], t // (nt3[0] * nt3[1]))
        got = set()
        for d in itertools.product((-1, 0, 1), repeat=3):
            c = [c0[a] + d[a] for a in range(3)]
            if any(not case.periodic[a] and not 0 <= c[a] < nt3[a] for a in range(3)):
                continue
            c = [c[a] % nt3[a] for a in range(3)]
            u = c[0] + nt3[0] * (c[1] + nt3[1] * c[2])
            got.update(tc[tco[u]:tco[u + 1]].tolist())
        expect += sorted(got)
        expect_off.append(len(expect))
    assert np.array_equal(off, expect_off)
    assert np.array_equal(cells, expect)
    assert len(expect) > 0
