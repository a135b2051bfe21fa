"""Serving loop on the GPU: every solve gives the same result alone and in
the mix of a continuously batched stream, admission respects the memory
budget and the slots, and the C ABI's batch calls behave as declared.

Tolerance between a solve run alone and the same solve inside the batch
(relative L2 of vertex positions and fluid velocity): the kernels and launch
shapes are the same, only the order of floating-point atomic additions in
the force spread may differ, so FP64 <= 1e-10 and FP32 <= 1e-5.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = {0: 1e-10, 1: 1e-5}   # HC_FORM_PLAIN_F64, HC_FORM_MIXED_F32


def _requests():
    from hemocell_gb300.serving import Request
    spec = [(32, 1, 300.0, 1.0, 80), (32, 2, 120.0, 3.0, 131), (48, 1, 450.0, 0.6, 64), (32, 3, 75.0, 1.7, 101)]
    return [Request(id=i, arrival=0.0, n=n, n_rbc=k, shear_rate=g, stiffness=s, steps=st, seed=100 + i)
            for i, (n, k, g, s, st) in enumerate(spec)]


def _alone(solves, reqs, form):
    from hemocell_gb300 import _lib as L
    from hemocell_gb300.serving import read_result
    out = {}
    for r in reqs:
        hc = solves[r.id].build(form, L.HC_LAUNCH_BATCHED)
        hc.iterate(r.steps)
        out[r.id] = read_result(hc, fluid=True)
        hc.close()
    return out


def _compare(a, b, tol):
    for k in a:
        assert rel_l2(b[k]["x"], a[k]["x"]) <= tol, k
        assert rel_l2(b[k]["u"], a[k]["u"]) <= tol, k


@pytest.mark.parametrize("form", [0, 1])
def test_batched_solves_match_alone(built, form):
    """Two solves start, two more are admitted while those are on the GPU;
    each result equals the solve run alone."""
    from hemocell_gb300 import _lib as L
    from hemocell_gb300.hemocell import Batch
    from hemocell_gb300.serving import Solve, read_result
    reqs = _requests()
    solves = {r.id: Solve(r) for r in reqs}
    ref = _alone(solves, reqs, form)
    b = Batch(4 << 30, max_slots=8, chunk_steps=16)
    got = {}
    try:
        for r in reqs[:2]:
            assert b.admit(solves[r.id].build(form, L.HC_LAUNCH_BATCHED), r.steps, r.id)
        b.pump(0.0)
        st = b.stats()
        assert st["active"] == 2 and st["steps_enqueued"] > 0
        for r in reqs[2:]:
            assert b.admit(solves[r.id].build(form, L.HC_LAUNCH_BATCHED), r.steps, r.id)
        for _ in range(100000):
            b.pump(5.0)
            while True:
                x = b.pop()
                if x is None:
                    break
                tag, hc, status = x
                assert status == L.HC_OK
                got[tag] = read_result(hc, fluid=True)
                assert hc.stats().iter == reqs[tag].steps
                b.release(hc)
            if len(got) == len(reqs):
                break
        st = b.stats()
        assert st["completed"] == 4 and st["active"] == 0 and st["bytes_in_use"] == 0
        assert st["steps_enqueued"] == sum(r.steps for r in reqs)
    finally:
        b.close()
    _compare(ref, got, TOL[form])


def test_serve_stream_matches_alone(built):
    """The real-time server on staggered arrivals, FP32."""
    from hemocell_gb300 import _lib as L
    from hemocell_gb300.serving import Solve, serve, with_arrivals
    reqs = with_arrivals(_requests(), 400.0, 5)
    solves = {r.id: Solve(r) for r in reqs}
    ref = _alone(solves, reqs, L.HC_FORM_MIXED_F32)
    out = serve(reqs, L.HC_FORM_MIXED_F32, 4 << 30, max_slots=8, chunk_steps=16, keep_results=True, fluid=True,
                solves=solves)
    assert out["completed"] == len(reqs)
    assert out["p99_s"] >= out["p50_s"] > 0
    _compare(ref, out["results"], TOL[1])


def _finish_one(b):
    for _ in range(100000):
        if b.pump(5.0) > 0:
            break
    return b.pop()


def test_admission_by_memory_and_slots(built):
    from hemocell_gb300 import _lib as L
    from hemocell_gb300.hemocell import Batch
    from hemocell_gb300.serving import Solve
    r0, r1 = _requests()[:2]
    s0, s1 = Solve(r0), Solve(r1)
    h0 = s0.build(1, L.HC_LAUNCH_BATCHED)
    h1 = s1.build(1, L.HC_LAUNCH_BATCHED)
    need0, need1 = h0.stats().device_bytes, h1.stats().device_bytes
    assert need0 <= s0.bytes(1) and need1 <= s1.bytes(1)   # the estimate bounds the real footprint

    tight = Batch(need0 - 1, max_slots=4, chunk_steps=8)
    assert not tight.fits(need0)
    assert not tight.admit(h0, 10, 0)       # refused: the caller keeps the handle
    h0.iterate(2)
    assert h0.stats().iter == 2
    tight.close()

    # room for one of the two at a time
    b = Batch(max(need0, need1) + min(need0, need1) // 2, max_slots=4, chunk_steps=8)
    try:
        assert b.admit(h0, 10, 0)
        assert not b.admit(h1, 10, 1)       # over the budget while h0 is resident
        tag, hc, status = _finish_one(b)
        assert tag == 0 and status == L.HC_OK and hc.stats().iter == 12
        assert not b.admit(h1, 10, 1)       # a popped solve holds its bytes until released
        b.release(hc)
        assert b.admit(h1, 10, 1)
        tag, hc, status = _finish_one(b)
        assert tag == 1 and status == L.HC_OK
        b.release(hc)
        assert b.stats()["bytes_in_use"] == 0
    finally:
        b.close()

    one = Batch(1 << 30, max_slots=1, chunk_steps=8)
    try:
        assert one.admit(s0.build(1, L.HC_LAUNCH_BATCHED), 4, 0)
        h3 = s1.build(1, L.HC_LAUNCH_BATCHED)
        assert not one.admit(h3, 4, 1)      # no free slot
        h3.close()
    finally:
        one.close()                         # destroys the resident solve
