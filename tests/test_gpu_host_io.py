"""Per-step host traffic of the public API on the GPU: the asynchronous,
double-buffered position readback and setExternalVector's per-call upload
of the body-force profile, with the change of a body force added to a force
field that already holds the next step's fused spread."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _cases():
    from hemocell_gb300 import cases
    return cases


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("form", [0, 1])
def test_async_positions_match_synchronous_reads(built, form):
    """Positions read with read_positions_async into two alternating pinned
    buffers, one step after another, equal the positions a twin handle reads
    synchronously after each of the same steps (batched launch, one step per
    call, as the end-to-end loop runs)."""
    from hemocell_gb300 import _lib as L
    case = _cases().mixed_box(wall=True)
    a = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    b = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    V = a.stats().vertices
    bufs = [_pinned((V, 3)), _pinned((V, 3))]
    body = np.array(case.body, np.float64)
    ref = []
    got = []
    for k in range(8):
        for hc in (a, b):
            hc.setExternalVector(case.body_mode, body)
            hc.iterate(1)
        ref.append(b.read_positions())
        a.read_positions_async(bufs[k & 1], k & 1)
        if k >= 1:
            got.append(a.wait_positions((k - 1) & 1).copy())
    got.append(a.wait_positions(7 & 1).copy())
    # FP64 twins agree bit for bit; FP32 up to the order of the spread's float atomics
    for k in range(8):
        if form == 0:
            assert np.array_equal(got[k], ref[k]), k
        else:
            assert rel_l2(got[k], ref[k]) < 1e-9, k
    assert np.array_equal(got[-1], a.read_vertices()[0])
    with pytest.raises(Exception):
        a.read_positions_async(np.zeros((V, 2)), 0)
    a.close()
    b.close()


@pytest.mark.parametrize("form", [0, 1])
def test_changed_body_force_keeps_fused_spread(built, form):
    """A body force changed between batched steps (the next step's spread
    already fused into the force field, so the change is added to it) gives
    the run of the per-stage launch, which refills the force field with the
    new body force and spreads afterwards: FP64 within 1e-10, FP32 within
    1e-5; setting the same force again changes nothing."""
    from hemocell_gb300 import _lib as L
    case = _cases().mixed_box(wall=True)
    fused = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    staged = case.build(form=form, launch=L.HC_LAUNCH_PER_STAGE)
    same = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    for k in range(6):
        body = (2e-6 * (1.0 + 0.3 * np.sin(0.7 * k)), -1e-6, 5e-7 * k)
        for hc in (fused, staged):
            hc.setExternalVector(L.HC_BODY_UNIFORM, body)
            hc.iterate(4)
        same.setExternalVector(case.body_mode, case.body)
        same.iterate(4)
    tol = 1e-10 if form == 0 else 1e-5
    assert rel_l2(fused.read_vertices()[0], staged.read_vertices()[0]) < tol
    assert rel_l2(fused.read_fluid()[1], staged.read_fluid()[1]) < tol
    assert rel_l2(fused.read_force_field(1), staged.read_force_field(1)) < tol   # force of the last collision
    ref = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    ref.iterate(24)
    assert rel_l2(same.read_vertices()[0], ref.read_vertices()[0]) < (1e-13 if form == 0 else 1e-9)
    for hc in (fused, staged, same, ref):
        hc.close()


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("launch", [0, 1])
def test_single_steps_match_one_call(built, form, launch):
    """iterate(1) called 21 times (after the first step, the batched launch
    replays a one-step CUDA graph per buffer parity) ends in the state of one
    iterate(21), for both launch modes."""
    case = _cases().mixed_box(wall=True)
    a = case.build(form=form, launch=launch)
    b = case.build(form=form, launch=launch)
    for _ in range(21):
        a.iterate(1)
    b.iterate(21)
    # up to the order of the spread's atomic additions
    tol = 1e-14 if form == 0 else 1e-9
    assert rel_l2(a.read_vertices()[0], b.read_vertices()[0]) <= tol
    assert rel_l2(a.read_fluid()[1], b.read_fluid()[1]) <= tol
    assert a.stats().iter == b.stats().iter == 21
    assert a.device_status() == b.device_status()
    a.close()
    b.close()


@pytest.mark.parametrize("form", [0, 1])
def test_timescale_cycle_graph(built, form):
    """Materials every 6, 3 and 6 steps, velocity every 3 (a 6-step cycle):
    the batched launch replays whole cycles from one CUDA graph (after eager
    steps up to a cycle start) and ends where single eager steps end, and the
    FP64 form where the oracle ends."""
    from hemocell_gb300 import _lib as L
    from oracle import oracle as orc
    case = _cases().mixed_box(wall=True)
    a = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    b = case.build(form=form, launch=L.HC_LAUNCH_BATCHED)
    for hc in (a, b):
        hc.iterate(1)
        hc.setMaterialTimeScaleSeparation([6, 3, 6], velocity_every=3)
    a.iterate(40)
    for _ in range(40):
        b.iterate(1)
    # up to the order of the spread's atomic additions (FP32 rounding in the mixed form)
    tol = 1e-14 if form == 0 else 1e-6
    assert rel_l2(a.read_vertices()[0], b.read_vertices()[0]) <= tol
    assert rel_l2(a.read_fluid()[1], b.read_fluid()[1]) <= tol
    assert a.stats().iter == b.stats().iter == 41
    if form == 0:
        o = orc.apply_case(case)
        o.step(1)
        o.set_timescales([6, 3, 6], 3)
        o.step(40)
        assert rel_l2(a.read_vertices()[0], o.read_vertices()[0]) < 1e-10
    a.close()
    b.close()
