"""GPU parity of every stage of the IB-LBM step against the FP64 CPU oracle.

All calls go through the C ABI (libhcgpu.so via ctypes).  Tolerances:
  plain FP64 form: relative L2 <= 1e-12 for one stage, <= 1e-10 for runs of
  hundreds of steps (FP atomics and FMA contraction reorder roundings);
  integer outputs (bins, tile lists, cell ownership): bit-exact.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

STAGE_TOL = 1e-12
RUN_TOL = 1e-10


def _cases():
    from hemocell_gb300 import cases
    return cases


def _orc():
    from oracle import oracle
    return oracle


def mixed_box(seed=5, n=(20, 18, 16), wall=True):
    return _cases().mixed_box(seed=seed, n=n, wall=wall)


def randomize(case, hc, o, seed=11, amp=2e-3, famp=1e-4, xamp=0.05, vamp=1e-3):
    """Identical random populations, force field and vertex perturbations on both."""
    rng = np.random.default_rng(seed)
    w = np.array([1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6)
    f = w[:, None] * (1.0 + amp * rng.standard_normal((19, case.N)))
    F = famp * rng.standard_normal((3, case.N))
    hc.write_populations(f)
    o.write_populations(f)
    hc.write_force_field(F)
    o.write_force_field(F)
    x, _, _ = o.read_vertices()
    x = x + xamp * rng.standard_normal(x.shape)
    v = vamp * rng.standard_normal(x.shape)
    fv = 1e-4 * rng.standard_normal(x.shape)
    hc.write_vertices(x, v, fv)
    o.write_vertices(x, v, fv)
    return f, F, x, v, fv


def test_collide_stream_one_stage(built):
    case = mixed_box()
    hc = case.build()
    o = _orc().apply_case(case)
    randomize(case, hc, o)
    hc.stage(1)
    o.stage("collide_stream")
    fg, fo = hc.read_populations(), o.read_populations()
    fluid = case.flags_array() == 0
    assert rel_l2(fg[:, fluid], fo[:, fluid]) < STAGE_TOL
    assert rel_l2(hc.read_force_field(0)[:, fluid], o.read_force_field(0)[:, fluid]) < STAGE_TOL
    assert rel_l2(hc.read_force_field(1), o.read_force_field(1)) < STAGE_TOL
    hc.close()


def _k1_codes():
    # 1: one thread per fluid node; 0x100: node velocity per fluid node;
    # 0x200: node velocity over warp-packed tagged nodes; 0x300: node velocity
    # at every fluid node (0x1300: with the interior pull of bit 12); bulk
    # collide-stream: stages | CTAs per SM << 4
    return [1, 0x101, 0x200, 0x201, 0x300, 0x301, 0x1300, 3 | (1 << 4), 4 | (2 << 4), 2 | (3 << 4)]


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("code", _k1_codes())
@pytest.mark.parametrize("wall", [True, False])
def test_collide_stream_bulk_matches_direct(built, form, code, wall):
    """The bulk-copy collide-stream gives the same bits as the direct pull,
    with moving walls (bounce-back, y/z edges) and fully periodic."""
    case = mixed_box(wall=wall)
    a = case.build(form=form)
    b = case.build(form=form)
    randomize(case, a, _orc().apply_case(case))   # one oracle each: randomize perturbs the
    randomize(case, b, _orc().apply_case(case))   # oracle's own positions in place
    t = b.tuning()
    t[7] = code
    if code & 0xff == 1:
        t[0], t[1] = 256, 1
    b.set_tuning(t)
    a.stage(1)
    b.stage(1)
    assert np.array_equal(a.read_populations(), b.read_populations())
    assert np.array_equal(a.read_force_field(0), b.read_force_field(0))
    a.stage(2)                                  # node velocity + interpolation
    b.stage(2)
    assert np.array_equal(a.read_vertices()[1], b.read_vertices()[1])
    assert b.device_status() == 0
    a.close()
    b.close()


@pytest.mark.parametrize("form", [0, 1])
def test_bulk_collide_stream_full_steps(built, form):
    """Whole steps with the bulk collide-stream, batched and graph-replayed,
    against the direct collide-stream: FP64 within the run tolerance, FP32
    within 1e-5 (the spread's float atomics may add in another order)."""
    from hemocell_gb300 import _lib as L
    case = mixed_box(wall=True)
    a = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    b = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    t = b.tuning()
    t[7] = 4 | (1 << 4)
    b.set_tuning(t)
    a.iterate(60)
    b.iterate(60)
    tol = RUN_TOL if form == 0 else 1e-5
    assert rel_l2(b.read_vertices()[0], a.read_vertices()[0]) < tol
    assert rel_l2(b.read_fluid()[1], a.read_fluid()[1]) < tol
    # the same cells reach the walls in both; no pipeline wait ran out
    assert b.device_status() == a.device_status() and (b.device_status() & 4) == 0
    a.close()
    b.close()


@pytest.mark.parametrize("form", [0, 1])
def test_bulk_collide_stream_rejects_unsuitable_lattice(built, form):
    """nx = 50: FP32 rows of 200 bytes are not 16-byte multiples; FP64 rows
    are (400 bytes), but the 32-bit mask rows (200 bytes) are not, so the
    bulk copies of either form would start off a 16-byte boundary."""
    from hemocell_gb300.hemocell import HemoCellError
    C = _cases()
    case = C.shear_single_rbc(n=50, shear_rate=100.0, seed=1)
    hc = case.build(form=form)
    t = hc.tuning()
    t[7] = 4 | (1 << 4)
    with pytest.raises(HemoCellError):
        hc.set_tuning(t)
    hc.close()


@pytest.mark.parametrize("form", [0, 1])
def test_repulsion_stage(built, form):
    """applyRepulsionForce + applyBoundaryRepulsionForce against the oracle:
    FP64 within the stage tolerance, FP32 within 1e-5."""
    from hemocell_gb300 import _lib as L
    case = _cases().repulsion_box()
    hc = case.build(form=form)
    o = _orc().apply_case(case)
    hc._check(hc._lib.hc_set_repulsion(hc._h, 1e-4, 2.0, 1))
    hc._check(hc._lib.hc_set_boundary_repulsion(hc._h, 5e-5, 2.0, 1))
    o.set_repulsion(1e-4, 2.0, 1)
    o.set_boundary_repulsion(5e-5, 2.0, 1)
    hc.stage(L.HC_STAGE_REPULSION)
    o.stage("repulsion")
    fg, fo = hc.read_repulsion(), o.read_repulsion()
    assert np.count_nonzero(np.any(fo != 0, axis=1)) > 50
    assert rel_l2(fg, fo) < (STAGE_TOL if form == 0 else 1e-5)
    assert hc.device_status() == 0
    hc.close()


@pytest.mark.parametrize("launch", [0, 1])
def test_repulsion_full_steps(built, launch):
    """Whole FP64 steps with both repulsion terms (per stage, and batched with
    the fused spread) against the oracle after 60 steps."""
    case = _cases().repulsion_box()
    hc = case.build(launch=launch)
    o = _orc().apply_case(case)
    hc.setRepulsion(1e-4, 1.0)                 # micrometres: 2 lattice units
    hc.enableBoundaryParticles(5e-5, 1.0)
    o.set_repulsion(1e-4, 2.0, 1)
    o.set_boundary_repulsion(5e-5, 2.0, 1)
    hc.iterate(60)
    o.step(60)
    xg, vg, _ = hc.read_vertices()
    xo, vo, _ = o.read_vertices()
    assert rel_l2(xg, xo) < RUN_TOL
    assert rel_l2(vg, vo) < RUN_TOL
    fluid = case.flags_array() == 0
    assert rel_l2(hc.read_fluid()[1][:, fluid], o.read_fluid()[1][:, fluid]) < RUN_TOL
    hc.close()


def test_fluid_only_shear_100_steps(built):
    C = _cases()
    n = (16, 12, 20)
    flags, walls = C.shear_walls(n, 20000.0)
    case = C.Case("couette", n, (1, 1, 0), flags=flags, walls=walls, body_mode=1, body=(1e-6, 0, 0))
    hc = case.build()
    o = _orc().apply_case(case)
    hc.iterate(100)
    o.step(100)
    rg, ug = hc.read_fluid()
    ro, uo = o.read_fluid()
    fluid = flags == 0
    assert rel_l2(ug[:, fluid], uo[:, fluid]) < RUN_TOL
    assert rel_l2(rg[fluid], ro[fluid]) < RUN_TOL
    hc.close()


def test_spread_stage(built):
    case = mixed_box()
    hc = case.build()
    o = _orc().apply_case(case)
    randomize(case, hc, o)
    hc.stage(0)
    o.stage("spread")
    assert rel_l2(hc.read_force_field(0), o.read_force_field(0)) < STAGE_TOL
    _, _, fg = hc.read_vertices()
    _, _, fo = o.read_vertices()
    assert rel_l2(fg, fo) < STAGE_TOL
    hc.close()


def test_spread_force_limit_clamp(built):
    case = mixed_box()
    hc = case.build()
    o = _orc().apply_case(case)
    randomize(case, hc, o)
    x, _, _ = o.read_vertices()
    big = np.zeros_like(x)
    big[::7] = 0.05  # above f_limit (7.8e-3 lattice units)
    hc.write_vertices(None, None, big)
    o.write_vertices(None, None, big)
    hc.stage(0)
    o.stage("spread")
    _, _, fg = hc.read_vertices()
    _, _, fo = o.read_vertices()
    assert np.max(np.linalg.norm(fg, axis=1)) <= hc.units()["f_limit"] * (1 + 1e-12)
    assert rel_l2(fg, fo) < STAGE_TOL
    assert rel_l2(hc.read_force_field(0), o.read_force_field(0)) < STAGE_TOL
    hc.close()


def test_interpolate_stage(built):
    case = mixed_box()
    hc = case.build()
    o = _orc().apply_case(case)
    randomize(case, hc, o)
    hc.stage(2)
    o.stage("interpolate")
    _, vg, _ = hc.read_vertices()
    _, vo, _ = o.read_vertices()
    assert rel_l2(vg, vo) < STAGE_TOL
    hc.close()


def test_advance_and_bins_bit_exact(built):
    case = mixed_box()
    hc = case.build()
    o = _orc().apply_case(case)
    randomize(case, hc, o, vamp=0.3)
    hc.stage(3)
    o.stage("advance")
    xg, _, _ = hc.read_vertices()
    xo, _, _ = o.read_vertices()
    assert np.array_equal(xg, xo)  # x + v in FP64, one rounding on both sides
    ag, _ = hc.read_cells()
    ao, _ = o.read_cells()
    assert np.array_equal(ag, ao)
    bg = hc.read_bins()
    bo = o.bins((8, 8, 8), None, case.dims)
    for k in bo:
        assert np.array_equal(bg[k], bo[k]), k
    hc.close()


def _edge_coordinates(case, x, rng):
    """Vertex coordinates on the cases the mixed form's integer split of an
    FP64 coordinate must get right: integers, half-integers (floor(P + 0.5)
    ties), one ulp either side of each, and on periodic axes values below 1,
    exactly 0 and negative (the FP64 fallback)."""
    x = x.copy()
    idx = rng.permutation(len(x))
    edge = idx[: len(x) // 2]
    for k, i in enumerate(edge):
        a = k % 3
        base = float(np.floor(x[i, a]))
        kind = (k // 3) % 8
        if kind == 0:
            val = base + 0.5
        elif kind == 1:
            val = np.nextafter(base + 0.5, -np.inf)
        elif kind == 2:
            val = np.nextafter(base + 0.5, np.inf)
        elif kind == 3:
            val = base
        elif kind == 4:
            val = np.nextafter(base, np.inf)
        elif kind == 5:
            val = np.nextafter(base + 1.0, -np.inf)
        elif case.periodic[a]:
            val = (-0.3, 0.0, 0.5, 0.999999999999)[k % 4] if kind == 6 else -1.0 + (k % 5) * 0.25
        else:
            val = base + 0.25
        x[i, a] = val
    return x, edge


@pytest.mark.parametrize("wall", [False, True])
def test_stencil_edge_coordinates_fp32(built, wall):
    """The mixed form takes the stencil's base node and fractions, and each
    vertex's nearest node, from the bits of the FP64 position (FP64
    instructions below 1, for negative and non-finite coordinates).  On edge
    coordinates the spread and the interpolation match the FP64 oracle at the
    form's FP32 rounding, and the advance's positions, bins and cell states
    are bit-exact (velocities exactly representable in FP32, zero on the
    edge vertices, so x + v is the same double on both sides)."""
    from hemocell_gb300 import _lib as L
    case = mixed_box(wall=wall)
    hc = case.build(form=L.HC_FORM_MIXED_F32)
    o = _orc().apply_case(case)
    rng = np.random.default_rng(21)
    _, _, x, v, fv = randomize(case, hc, o)
    x, edge = _edge_coordinates(case, x, rng)
    v = v.astype(np.float32).astype(np.float64)
    v[edge] = 0.0
    fv = fv.astype(np.float32).astype(np.float64)
    hc.write_vertices(x, v, fv)
    o.write_vertices(x, v, fv)
    hc.stage(0)
    o.stage("spread")
    assert rel_l2(hc.read_force_field(0), o.read_force_field(0)) < 1e-5
    hc.stage(2)
    o.stage("interpolate")
    assert rel_l2(hc.read_vertices()[1], o.read_vertices()[1]) < 1e-5
    # the advance from exactly representable velocities
    hc.write_vertices(x, v, None)
    o.write_vertices(x, v, None)
    hc.stage(3)
    o.stage("advance")
    assert np.array_equal(hc.read_vertices()[0], o.read_vertices()[0])
    assert np.array_equal(hc.read_cells()[0], o.read_cells()[0])
    bg = hc.read_bins()
    bo = o.bins((8, 8, 8), None, case.dims)
    for k in bo:
        assert np.array_equal(bg[k], bo[k]), k
    assert hc.device_status() & 5 == 0
    hc.close()


@pytest.mark.parametrize("which", ["walls", "periodic", "suspension"])
def test_neighbour_lists_bit_exact(built, which):
    """hc_read_neighbours (per tile, the cells of the tile and its 26
    neighbours) against the oracle, on the same positions: bit-exact, with
    non-periodic walls in z, fully periodic, and on a 36^3 suspension whose
    4 x 4 x 4 tile grid wraps onto itself at the edges of 9-tile axes."""
    C = _cases()
    if which == "walls":
        case, tile = mixed_box(wall=True), (8, 8, 8)
    elif which == "periodic":
        case, tile = mixed_box(wall=False), (4, 4, 4)
    else:
        case = C.kolmogorov_mix(n=36, rbc_fraction=0.15, n_wbc=1, plt_per_rbc=0.5, wbc_triangles=320, seed=5)
        tile = (4, 4, 4)
    from hemocell_gb300 import _lib as L
    hc = case.build(tile=tile)
    o = _orc().apply_case(case)
    hc.iterate(5)
    o.step(5)
    xg, _, _ = hc.read_vertices()
    off, cells = hc.read_neighbours()
    off_o, cells_o = o.neighbours(tile, xg, case.dims, case.periodic)
    assert np.array_equal(off, off_o)
    assert np.array_equal(cells, cells_o)
    assert len(cells) > 0 and np.all(np.diff(off) >= 0)
    hc.close()


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("types", [[0], [1], [2], [0, 1, 2]])
def test_mechanics_stage(built, types, variant):
    """The three force-assembly variants (0 vertex gather, 1 face/edge
    scatter, 2 staged face/edge terms gathered per vertex) against the
    oracle's face/edge/vertex loops."""
    case = mixed_box()
    case.cells = [c for c in case.cells if c[0] in types]
    hc = case.build()
    t = hc.tuning()
    t[6] = variant
    hc.set_tuning(t)
    o = _orc().apply_case(case)
    randomize(case, hc, o, xamp=0.08)
    hc.stage(5)
    o.stage("mechanics", forced=1)
    _, _, fg = hc.read_vertices()
    _, _, fo = o.read_vertices()
    assert np.abs(fo).max() > 0
    assert rel_l2(fg, fo) < STAGE_TOL
    if variant != 1:  # no atomics: the same inputs give the same bits
        hc.stage(5)
        _, _, fg2 = hc.read_vertices()
        assert np.array_equal(fg, fg2)
    hc.close()


@pytest.mark.parametrize("variant", [0, 2])
def test_mechanics_stage_fp32(built, variant):
    """FP32 force assembly against the FP64 oracle (all three cell types)."""
    from hemocell_gb300 import _lib as L
    case = mixed_box()
    hc = case.build(form=L.HC_FORM_MIXED_F32)
    t = hc.tuning()
    t[6] = variant
    hc.set_tuning(t)
    o = _orc().apply_case(case)
    randomize(case, hc, o, xamp=0.08)
    hc.stage(5)
    o.stage("mechanics", forced=1)
    assert rel_l2(hc.read_vertices()[2], o.read_vertices()[2]) < 2e-5
    hc.close()


def test_staged_mechanics_falls_back_for_large_cells(built):
    """A 2562-vertex WBC does not fit the staged variant's shared memory in
    FP32: that cell takes the vertex-centric path (compiled into the other
    kernel, so only FP32 rounding may differ)."""
    from hemocell_gb300 import _lib as L
    C = _cases()
    t = C.wbc_type(5120)
    n = (40, 40, 40)
    xyz = C.place_cells(t.mesh, np.array([[19.5, 19.5, 19.5]]), np.array([[0.3, 0.2, 0.1]]))
    case = C.Case("wbc", n, (1, 1, 1), types=[t], cells=[(0, xyz)])
    out = []
    for variant in (0, 2):
        hc = case.build(form=L.HC_FORM_MIXED_F32)
        tt = hc.tuning()
        tt[6] = variant
        hc.set_tuning(tt)
        rng = np.random.default_rng(4)
        x, _, _ = hc.read_vertices()
        hc.write_vertices(x + 0.05 * rng.standard_normal(x.shape), None, None)
        hc.stage(5)
        out.append(hc.read_vertices()[2])
        hc.close()
    assert np.abs(out[0]).max() > 0 and rel_l2(out[1], out[0]) < 1e-6


def mixed_periodic(seed=9):
    """Periodic 40x36x32 box with one RBC, two PLTs and one WBC, not
    overlapping, in a Kolmogorov shear flow (F_x ~ sin(2 pi z / nz)) so the
    membranes deform: the batched/graph path end to end.  (In a uniform flow
    the cells only translate and their forces are FP64 round-off of the
    absolute-coordinate volume sum; comparing that noise is meaningless.)"""
    C = _cases()
    n = (40, 36, 32)
    types = [C.rbc_type(600), C.plt_type(320), C.wbc_type(1280)]
    rng = np.random.default_rng(seed)
    place = [(0, (11.0, 10.0, 16.0)), (1, (30.0, 8.0, 6.0)), (1, (30.0, 28.0, 26.0)), (2, (28.0, 22.0, 15.0))]
    cells = []
    for t, c in place:
        ang = rng.uniform(-np.pi, np.pi, size=(1, 3))
        cells.append((t, C.place_cells(types[t].mesh, np.array([c]), ang)))
    return C.Case("mixed_periodic", n, (1, 1, 1), types=types, cells=cells, body_mode=2, body=(2e-5, 0.0, 0.0))


def _per_type_errors(case, a, b):
    out, k = {}, 0
    for t, xyz in case.cells:
        n = xyz.shape[0]
        out.setdefault(t, []).append(rel_l2(a[k:k + n], b[k:k + n]))
        k += n
    return {t: max(v) for t, v in out.items()}


def test_full_step_mixed_types_batched_graph(built):
    from hemocell_gb300 import _lib as L
    case = mixed_periodic()
    o = _orc().apply_case(case)
    hp = case.build(launch=L.HC_LAUNCH_PER_STAGE)
    hb = case.build(launch=L.HC_LAUNCH_BATCHED)
    errs = []
    for chunk in (10, 40, 50):
        hp.iterate(chunk)
        hb.iterate(chunk)  # graph replay (2 steps per launch)
        o.step(chunk)
        xo, vo, _ = o.read_vertices()
        for name, hc in (("per_stage", hp), ("batched", hb)):
            xg, vg, _ = hc.read_vertices()
            errs.append((o_iter(o), name, rel_l2(xg, xo), rel_l2(vg, vo), _per_type_errors(case, vg, vo)))
    msg = "\n".join(map(str, errs))
    print(msg)
    for it, name, ex, ev, _ in errs:
        assert ex < RUN_TOL, msg
        assert ev < RUN_TOL, msg
    _, uo = o.read_fluid()
    for hc in (hp, hb):
        _, ug = hc.read_fluid()
        assert rel_l2(ug, uo) < RUN_TOL
        hc.close()


def o_iter(o):
    return o.L.orc_iter(o.s)


def test_batched_state_changes_between_steps(built):
    """The batched form spreads the next step's forces inside the membrane
    kernel; host-side changes between steps (vertex rewrite, body force,
    timescales) must fall back to the standalone spread and stay exact."""
    from hemocell_gb300 import _lib as L
    case = mixed_periodic()
    o = _orc().apply_case(case)
    hb = case.build(launch=L.HC_LAUNCH_BATCHED)
    hb.iterate(20)
    o.step(20)
    x, v, f = o.read_vertices()
    hb.write_vertices(x, v, f)
    o.write_vertices(x, v, f)
    hb.setExternalVector(case.body_mode, case.body)
    o.set_body_force(case.body_mode, case.body)
    hb.iterate(21)
    o.step(21)
    hb.setMaterialTimeScaleSeparation([2, 2, 2], velocity_every=1)
    o.set_timescales([2, 2, 2], 1)
    hb.iterate(10)
    o.step(10)
    xg, vg, _ = hb.read_vertices()
    xo, vo, _ = o.read_vertices()
    assert rel_l2(xg, xo) < RUN_TOL
    assert rel_l2(vg, vo) < RUN_TOL
    _, ug = hb.read_fluid()
    _, uo = o.read_fluid()
    assert rel_l2(ug, uo) < RUN_TOL
    hb.close()


def test_timescale_separation(built):
    case = mixed_periodic()
    o = _orc().apply_case(case)
    hc = case.build()
    hc.setMaterialTimeScaleSeparation([4, 2, 4], velocity_every=2)
    o.set_timescales([4, 2, 4], 2)
    hc.iterate(40)
    o.step(40)
    xg, vg, fg = hc.read_vertices()
    xo, vo, fo = o.read_vertices()
    assert rel_l2(xg, xo) < RUN_TOL
    assert rel_l2(vg, vo) < RUN_TOL
    assert rel_l2(fg, fo) < 1e-8
    hc.close()


def test_config0_shear_1000_steps(built):
    """The CPU-runnable configuration: 50^3 Couette at 100 1/s, one RBC of
    642 vertices, 1000 steps; plain FP64 within 1e-10 of the oracle."""
    C = _cases()
    case = C.shear_single_rbc(n=50, shear_rate=100.0, seed=1, min_triangles=600)
    hc = case.build()
    o = _orc().apply_case(case)
    hc.iterate(1000)
    o.step(1000)
    xg, vg, _ = hc.read_vertices()
    xo, vo, _ = o.read_vertices()
    rg, ug = hc.read_fluid()
    ro, uo = o.read_fluid()
    fluid = case.flags_array() == 0
    assert rel_l2(xg, xo) < RUN_TOL
    assert rel_l2(vg, vo) < RUN_TOL
    assert rel_l2(ug[:, fluid], uo[:, fluid]) < RUN_TOL
    assert rel_l2(rg[fluid], ro[fluid]) < RUN_TOL
    bg = hc.read_bins()
    bo = o.bins((8, 8, 8), xg, case.dims)  # binning of the same positions: bit-exact
    for k in bo:
        assert np.array_equal(bg[k], bo[k]), k
    hc.close()


def test_mixed_form_error_vs_fp64(built):
    """FP32 form (f_i - w_i storage) against the FP64 oracle: velocity and
    positions within 1e-4 relative L2 after 200 steps of a sheared RBC."""
    from hemocell_gb300 import _lib as L
    C = _cases()
    case = C.shear_single_rbc(n=24, shear_rate=20000.0, seed=7, min_triangles=320)
    hc = case.build(form=L.HC_FORM_MIXED_F32)
    o = _orc().apply_case(case)
    hc.iterate(200)
    o.step(200)
    _, ug = hc.read_fluid()
    _, uo = o.read_fluid()
    xg, vg, _ = hc.read_vertices()
    xo, vo, _ = o.read_vertices()
    assert rel_l2(ug, uo) < 1e-4
    assert rel_l2(vg, vo) < 1e-4
    assert rel_l2(xg, xo) < 1e-6
    hc.close()


def test_error_paths(built):
    from hemocell_gb300 import HemoCellError, _lib as L
    case = mixed_box()
    hc = case.build()
    with pytest.raises(HemoCellError):
        hc.setMaterialTimeScaleSeparation([3, 2, 4], velocity_every=2)
    with pytest.raises(HemoCellError):
        hc.set_wall_velocity(99, (0, 0, 0))
    with pytest.raises(HemoCellError):
        hc.stage(42)
    hc.close()


@pytest.mark.parametrize("form", [0, 1])
def test_programmatic_dependent_launch_same_results(built, form):
    """The step's kernels launched with programmatic dependent launch (tune[7]
    bit 10) give the results of ordinary launches, batched and graph-replayed."""
    from hemocell_gb300 import _lib as L
    case = mixed_box(wall=True)
    a = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    b = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    t = b.tuning()
    t[7] |= 0x400
    b.set_tuning(t)
    a.iterate(40)
    b.iterate(40)
    tol = RUN_TOL if form == 0 else 1e-5
    assert rel_l2(b.read_vertices()[0], a.read_vertices()[0]) < tol
    assert rel_l2(b.read_fluid()[1], a.read_fluid()[1]) < tol
    assert b.device_status() == a.device_status()
    a.close()
    b.close()


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("shape,var", [((32, 4), 0x1000), ((32, 4), 0x2000), ((8, 16), 0x3000), ((16, 8), 0x1000),
                                       ((64, 2), 0x2000), ((256, 1), 1 | 0x3000), ((128, 1), 1 | 0x2000)])
@pytest.mark.parametrize("walls", ["moving", "static", "odd"])
def test_collide_stream_variants_same_bits(built, form, shape, var, walls):
    """The direct collide-stream variants against the whole-row kernel: the
    interior pull (tune[7] bit 12), evict-last population stores (bit 13),
    warps shaped as 8 x 4 and 16 x 2 tiles, one thread per fluid node (kind 1)
    with the interior pull and evict-last stores, with moving walls (a sheared
    box with the moving-wall term), with walls at rest (a small pipe, the term
    compiled out) and on a 21 x 17 x 19 lattice (no size a multiple of a block
    or column length).  One collide-stream stage from the same random state
    gives the same bits; 30 graph-replayed steps with cells agree within the
    run tolerance (FP64 1e-12, FP32 1e-5) and delete the same cells: the
    spread's float atomics add the vertices of a node in whatever order they
    arrive, so two runs need not agree to the last bit once several vertices
    share a node."""
    from hemocell_gb300 import _lib as L
    C = _cases()
    if walls == "moving":
        case = mixed_box(wall=True)
    elif walls == "static":
        case = C.pipe_ht25(nx=24, ny=24, nz=32, radius=10.0, n_cells=4, seed=3)
    else:
        n = (21, 17, 19)
        flags, wl = C.shear_walls(n, 3000.0)
        t = C.plt_type(80, radius_m=1.0e-6, aspect=0.4)
        xyz = C.place_cells(t.mesh, np.array([[20.6, 8.0, 9.0]]), np.array([[0.4, -0.3, 0.2]]))
        case = C.Case("odd", n, (1, 1, 0), flags=flags, walls=wl, types=[t], cells=[(0, xyz)],
                      body_mode=L.HC_BODY_UNIFORM, body=(3e-6, -2e-6, 0.0))

    def pair():
        a = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
        b = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
        t = a.tuning()
        t[0], t[1] = 0, 1
        t[7] &= ~0xf0ff
        a.set_tuning(t)
        t[0], t[1] = shape
        t[7] |= var
        b.set_tuning(t)
        assert b.tuning()[7] & 0xf0ff == var
        return a, b

    a, b = pair()
    randomize(case, a, _orc().apply_case(case))
    randomize(case, b, _orc().apply_case(case))
    a.stage(1)
    b.stage(1)
    assert np.array_equal(b.read_populations(), a.read_populations())
    assert np.array_equal(b.read_force_field(0), a.read_force_field(0))
    a.close()
    b.close()
    a, b = pair()
    a.iterate(30)
    b.iterate(30)
    tol = 1e-12 if form == 0 else 1e-5
    fluid = case.flags_array() == 0
    assert rel_l2(b.read_vertices()[0], a.read_vertices()[0]) < tol
    assert rel_l2(b.read_fluid()[1][:, fluid], a.read_fluid()[1][:, fluid]) < tol
    assert np.array_equal(b.read_cells()[0], a.read_cells()[0])
    assert b.device_status() == a.device_status()
    a.close()
    b.close()


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("dims,periodic,fill", [((1, 1, 1), (1, 1, 1), 0), ((2, 3, 1), (1, 1, 1), 0),
                                               ((1, 5, 4), (1, 1, 1), 0), ((4, 3, 1), (1, 1, 0), 0),
                                               ((5, 2, 6), (1, 0, 1), 0), ((6, 5, 4), (1, 1, 1), 1)])
def test_degenerate_lattices_against_oracle(built, form, dims, periodic, fill):
    """Lattices of one or two nodes along an axis, periodic (every pull wraps
    onto the node itself or its one neighbour) and not (every link off a
    one-node axis bounces back), from random populations under a uniform body
    force: 20 graph-replayed steps against the oracle.  A lattice of wall
    nodes only steps without error."""
    from hemocell_gb300 import _lib as L
    C = _cases()
    n = dims[0] * dims[1] * dims[2]
    flags = np.full(n, fill, np.uint8)
    case = C.Case("tiny", dims, periodic, flags=flags, body_mode=L.HC_BODY_UNIFORM, body=(2e-5, -1e-5, 3e-5))
    hc = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    o = _orc().apply_case(case)
    randomize(case, hc, o)
    hc.iterate(20)
    o.step(20)
    assert hc.device_status() == 0
    rg, ug = hc.read_fluid()
    hc.close()
    if fill:
        return
    ro, uo = o.read_fluid()
    tol = RUN_TOL if form == 0 else 1e-5
    assert rel_l2(rg, ro) < tol
    assert rel_l2(ug, uo) < tol


@pytest.mark.parametrize("form", [0, 1])
def test_64bit_index_path_matches_tiles(built, form):
    """A lattice with 19 N >= 2^31 (512 x 512 x 432, 113.2 M nodes) runs the
    collide-stream's 64-bit index path (general pull, no fluid-node list),
    every other lattice here the 32-bit one.  Built as 8 x 8 periodic copies
    of a 64 x 64 x 432 cross-section holding a wall-bounded channel, with the
    Kolmogorov body force varying along z, every copy must hold the bits of
    the 32-bit run on one copy after 6 steps (density and velocity of every
    node)."""
    import torch
    from hemocell_gb300 import _lib as L
    free, _ = torch.cuda.mem_get_info()
    if free < 80 * 2 ** 30:
        pytest.skip("needs about 60 GB of free device memory")
    C = _cases()
    nx, ny, nz, k = 64, 64, 432, 8
    small_flags = C.cylinder_flags(nx, ny, nz, 24.0)
    big_flags = np.tile(small_flags.reshape(nz, ny, nx), (1, k, k)).reshape(-1)
    body = (2e-6, 0.0, 0.0)
    small = C.Case("tile", (nx, ny, nz), (1, 1, 1), flags=small_flags, body_mode=L.HC_BODY_KOLMOGOROV, body=body)
    big = C.Case("tiled", (k * nx, k * ny, nz), (1, 1, 1), flags=big_flags, body_mode=L.HC_BODY_KOLMOGOROV,
                 body=body)
    assert 19 * big.N >= 2 ** 31 > 19 * small.N
    a = small.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    a.iterate(6)
    ra, ua = a.read_fluid()
    a.close()
    b = big.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    b.iterate(6)
    rb, ub = b.read_fluid()
    assert b.device_status() == 0
    b.close()
    assert np.abs(ua).max() > 0          # the force has set the fluid moving
    ra = ra.reshape(nz, 1, ny, 1, nx)
    assert np.array_equal(rb.reshape(nz, k, ny, k, nx), np.broadcast_to(ra, (nz, k, ny, k, nx)))
    del rb
    ua = ua.reshape(3, nz, 1, ny, 1, nx)
    assert np.array_equal(ub.reshape(3, nz, k, ny, k, nx), np.broadcast_to(ua, (3, nz, k, ny, k, nx)))


@pytest.mark.parametrize("form", [0, 1])
def test_64bit_index_path_with_a_cell(built, form):
    """The cell stages' 64-bit index paths (tagged node velocity, spread,
    interpolation, force assembly on a lattice with 19 N >= 2^31): the tiled
    channels of the test above, with one RBC in copy (3, 5), against the same
    RBC in one copy (positions shifted by whole tiles, which changes their
    rounding: within the run tolerance) and an empty copy (every other copy
    of the big lattice, bit for bit), after 10 steps."""
    import torch
    from hemocell_gb300 import _lib as L
    free, _ = torch.cuda.mem_get_info()
    if free < 80 * 2 ** 30:
        pytest.skip("needs about 60 GB of free device memory")
    C = _cases()
    nx, ny, nz, k, tx, ty = 64, 64, 432, 8, 3, 5
    small_flags = C.cylinder_flags(nx, ny, nz, 24.0)
    big_flags = np.tile(small_flags.reshape(nz, ny, nx), (1, k, k)).reshape(-1)
    body = (2e-6, 0.0, 0.0)
    t = C.rbc_type(600)
    xyz = C.place_cells(t.mesh, np.array([[31.5, 31.5, 200.0]]), np.array([[0.3, -0.2, 0.5]]))
    offset = np.array([tx * nx, ty * ny, 0.0])
    kw = dict(periodic=(1, 1, 1), body_mode=L.HC_BODY_KOLMOGOROV, body=body)
    runs = {}
    for name, dims, flags, cells in (("cell", (nx, ny, nz), small_flags, [(0, xyz)]),
                                     ("empty", (nx, ny, nz), small_flags, []),
                                     ("big", (k * nx, k * ny, nz), big_flags, [(0, xyz + offset)])):
        case = C.Case(name, dims, kw["periodic"], flags=flags, body_mode=kw["body_mode"], body=kw["body"],
                      types=[t] if cells else [], cells=cells)
        h = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
        h.iterate(10)
        runs[name] = (h.read_vertices()[0] if cells else None, h.read_fluid(), h.device_status())
        h.close()
    tol = RUN_TOL if form == 0 else 1e-5
    xa, (ra, ua), sa = runs["cell"]
    _, (rc, uc), _ = runs["empty"]
    xb, (rb, ub), sb = runs["big"]
    assert sa == sb == 0
    assert rel_l2(xb - offset, xa) < tol
    assert np.abs(xa - xyz).max() > 0                 # the cell has moved
    rb = rb.reshape(nz, k, ny, k, nx)
    ub = ub.reshape(3, nz, k, ny, k, nx)
    assert rel_l2(ub[:, :, ty, :, tx, :].reshape(-1), ua.reshape(-1)) < tol
    assert rel_l2(rb[:, ty, :, tx, :].reshape(-1), ra) < tol
    rc = rc.reshape(nz, ny, nx)
    uc = uc.reshape(3, nz, ny, nx)
    for j in range(k):
        for i in range(k):
            if (i, j) != (tx, ty):
                assert np.array_equal(rb[:, j, :, i, :], rc)
                assert np.array_equal(ub[:, :, j, :, i, :], uc)


@pytest.mark.parametrize("form", [0, 1])
def test_autotune_restores_state_and_caches(built, tmp_path, form):
    """hc_autotune leaves the state as it found it, and a second handle of the
    same case reads its pick from the cache file.  The tuned and the default
    runs are each checked against the FP64 oracle at the form's run tolerance
    (FP64 1e-10, FP32 1e-4): two FP32 tunings need not agree to the last bits,
    since their force-assembly variants and spread atomics round in different
    orders."""
    from hemocell_gb300 import _lib as L
    case = mixed_box(wall=True)
    a = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    b = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    o = _orc().apply_case(case)
    a.iterate(5)
    b.iterate(5)
    o.step(5)
    x0 = b.read_vertices()[0]
    f0 = b.read_fluid()[1]
    cache = str(tmp_path / "tuning.txt")
    b.autotune(cache)
    assert np.array_equal(b.read_vertices()[0], x0)
    assert np.array_equal(b.read_fluid()[1], f0)
    t = b.tuning()
    b.set_tuning(t)
    a.iterate(20)
    b.iterate(20)
    o.step(20)
    tol = RUN_TOL if form == 0 else 1e-4
    xo, uo = o.read_vertices()[0], o.read_fluid()[1]
    alive = o.read_cells()[0]
    assert 0 < alive.sum() < alive.size        # cells crossing the walls are deleted
    # vertices of deleted cells are gone in the reference (deleteIncompleteCells),
    # so only the live cells' positions are compared
    keep = np.concatenate([np.full(xyz.shape[0], bool(alive[k])) for k, (_, xyz) in enumerate(case.cells)])
    for h in (a, b):
        assert np.array_equal(h.read_cells()[0], alive)
        assert rel_l2(h.read_vertices()[0][keep], xo[keep]) < tol
        assert rel_l2(h.read_fluid()[1], uo) < tol
    assert b.device_status() == a.device_status()
    assert a.device_status() & 5 == 0                 # finite, no wait ran out
    c = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    c.autotune(cache)
    assert c.tuning() == t
    for h in (a, b, c):
        h.close()


@pytest.mark.parametrize("form", [0, 1])
def test_profile_kernels_times_the_step(built, form):
    """hc_profile_kernels runs the step hc_step runs: the state it leaves is
    the state of as many plain steps (3 queued + nsteps), and its kernel
    times are positive and fit inside the whole-step time."""
    from hemocell_gb300 import _lib as L
    case = mixed_box(wall=True)
    a = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    b = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    a.iterate(5)
    b.iterate(5)
    k = b.profile_kernels(10)
    a.iterate(13)
    tol = RUN_TOL if form == 0 else 1e-5
    assert rel_l2(b.read_vertices()[0], a.read_vertices()[0]) < tol
    assert rel_l2(b.read_fluid()[1], a.read_fluid()[1]) < tol
    assert all(k[g] > 0 for g in ("collide_stream", "node_velocity", "mechanics", "step"))
    assert k["collide_stream"] + k["node_velocity"] + k["mechanics"] <= 1.05 * k["step"] + 1e-3
    with pytest.raises(Exception):
        b.profile_kernels(0)
    a.close()
    b.close()


@pytest.mark.parametrize("form,launch", [(0, 0), (0, 1), (1, 1)])
def test_kolmogorov_suspension_against_oracle(built, form, launch):
    """The 128^3 suspension's configuration at 36^3: fully periodic, the
    Kolmogorov body force F_x = A sin(2 pi z / n), packed RBC, PLT and a WBC
    (642-vertex), 60 steps against the oracle: FP64 within the run
    tolerance, the mixed form within 1e-4; alive cells identical."""
    C = _cases()
    case = C.kolmogorov_mix(n=36, rbc_fraction=0.15, n_wbc=1, plt_per_rbc=0.5, wbc_triangles=1280, seed=5)
    assert {t for t, _ in case.cells} == {0, 1, 2}
    hc = case.build(form=form, launch=launch)
    o = _orc().apply_case(case)
    hc.iterate(60)
    o.step(60)
    tol = RUN_TOL if form == 0 else 1e-4
    xg, vg, _ = hc.read_vertices()
    xo, vo, _ = o.read_vertices()
    assert rel_l2(xg, xo) < tol
    assert rel_l2(vg, vo) < (tol if form == 0 else 1e-3)
    assert rel_l2(hc.read_fluid()[1], o.read_fluid()[1]) < tol
    assert np.array_equal(hc.read_cells()[0], o.read_cells()[0])
    assert hc.device_status() & 1 == 0
    hc.close()


@pytest.mark.parametrize("form,launch", [(0, 0), (0, 1), (1, 1)])
def test_odd_lattice_against_oracle(built, form, launch):
    """A 21x17x19 lattice (no size a multiple of a block edge) with moving
    walls in z, periodic x and y, a body force and one platelet crossing the
    periodic x face: 60 steps against the oracle.  Exercises the pull's wrap
    corrections, partial blocks and the platelet path."""
    from hemocell_gb300 import _lib as L
    C = _cases()
    n = (21, 17, 19)
    flags, walls = C.shear_walls(n, 3000.0)
    t = C.plt_type(80, radius_m=1.0e-6, aspect=0.4)
    xyz = C.place_cells(t.mesh, np.array([[20.6, 8.0, 9.0]]), np.array([[0.4, -0.3, 0.2]]))
    case = C.Case("odd", n, (1, 1, 0), flags=flags, walls=walls, types=[t], cells=[(0, xyz)],
                  body_mode=L.HC_BODY_UNIFORM, body=(3e-6, -2e-6, 0.0))
    hc = case.build(form=form, launch=launch)
    o = _orc().apply_case(case)
    hc.iterate(60)
    o.step(60)
    tol = RUN_TOL if form == 0 else 1e-4
    fluid = case.flags_array() == 0
    assert rel_l2(hc.read_fluid()[1][:, fluid], o.read_fluid()[1][:, fluid]) < tol
    assert rel_l2(hc.read_vertices()[0], o.read_vertices()[0]) < tol
    assert np.array_equal(hc.read_cells()[0], o.read_cells()[0])
    hc.close()


def test_lattice_without_cells_batched(built):
    """Batched stepping (graph) of a lattice with no cells, both forms."""
    from hemocell_gb300 import _lib as L
    C = _cases()
    case = C.Case("empty", (24, 20, 16), (1, 1, 1), body_mode=L.HC_BODY_KOLMOGOROV, body=(1e-5, 0.0, 0.0))
    for form in (0, 1):
        hc = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
        o = _orc().apply_case(case)
        hc.iterate(50)
        o.step(50)
        assert rel_l2(hc.read_fluid()[1], o.read_fluid()[1]) < (RUN_TOL if form == 0 else 1e-4)
        hc.close()


@pytest.mark.parametrize("form", [0, 1])
def test_fused_advance_same_results(built, form):
    """Interpolation and advance inside the force assembly (the batched
    default) against their own kernel (tune[7] bit 11), over steps with a
    state change in between and a cell that reaches a wall."""
    from hemocell_gb300 import _lib as L
    case = mixed_box(wall=True)
    out = []
    for bit in (0, 0x800):
        hc = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
        t = hc.tuning()
        t[7] |= bit
        hc.set_tuning(t)
        hc.iterate(25)
        hc.setExternalVector(1, (1e-6, 2e-6, 0.0))     # undoes the fused spread
        hc.iterate(26)
        x, v, _ = hc.read_vertices()
        out.append((x, v, hc.read_fluid()[1], hc.read_cells()[0], hc.read_bins(), hc.device_status()))
        hc.close()
    tol = RUN_TOL if form == 0 else 1e-5
    a, b = out
    assert rel_l2(b[0], a[0]) < tol and rel_l2(b[1], a[1]) < max(tol, 1e-9) and rel_l2(b[2], a[2]) < tol
    assert np.array_equal(a[3], b[3]) and a[5] == b[5]
    for k in ("vertex_node", "tile_offsets", "tile_cells"):
        assert np.array_equal(a[4][k], b[4][k]), k


@pytest.mark.parametrize("form", [0, 1])
def test_node_tags_skipped_with_dense_node_velocity(built, form):
    """With the dense node velocity (tune[7] bits 8-9 = 3) the spreads write no
    node tags.  Switching to a tagged form in mid-run, while the next step's
    spread is already fused into the force field, spreads again with tags:
    every run matches the FP64 oracle at the form's run tolerance."""
    from hemocell_gb300 import _lib as L
    case = mixed_periodic()
    o = _orc().apply_case(case)
    runs = {}
    for name, first, second in (("dense", 0x300, 0x300), ("dense_then_tagged", 0x300, 0x000),
                                ("tagged_then_dense", 0x000, 0x300)):
        hc = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
        t = hc.tuning()
        t[7] = (t[7] & ~0x300) | first
        hc.set_tuning(t)
        hc.iterate(12)
        t[7] = (t[7] & ~0x300) | second
        hc.set_tuning(t)
        hc.iterate(13)
        runs[name] = (hc.read_vertices()[0], hc.read_fluid()[1], hc.device_status())
        hc.close()
    o.step(25)
    xo, uo = o.read_vertices()[0], o.read_fluid()[1]
    tol = RUN_TOL if form == 0 else 1e-4
    for name, (x, u, st) in runs.items():
        assert rel_l2(x, xo) < tol, name
        assert rel_l2(u, uo) < tol, name
        assert st & 5 == 0, name
