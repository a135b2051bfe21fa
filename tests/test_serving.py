"""Host side of the serving loop (no GPU): the seeded request stream, the
device-memory estimate used for admission, and the one-server queue replay
of the solo baseline."""
import numpy as np

from hemocell_gb300 import _lib as L
from hemocell_gb300 import serving as S
from hemocell_gb300.hemocell import estimate_device_bytes


def test_request_stream_is_seeded_and_in_range():
    a = S.request_stream(1, 200.0, 2000)
    b = S.request_stream(1, 200.0, 2000)
    c = S.request_stream(2, 200.0, 2000)
    assert a == b and a != c
    assert a[0].arrival == 0.0
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) >= 0)
    rate = (len(a) - 1) / arr[-1]
    assert 185.0 < rate < 215.0
    assert {r.n for r in a} == set(S.BOX_EDGES)
    assert {r.n_rbc for r in a} == set(range(1, 9))
    sr = np.array([r.shear_rate for r in a])
    assert sr.min() >= 50.0 and sr.max() <= 500.0
    k = np.log([r.stiffness for r in a])
    assert k.min() >= np.log(0.5) - 1e-12 and k.max() <= np.log(5.0) + 1e-12
    assert abs(k.mean() - 0.5 * (np.log(0.5) + np.log(5.0))) < 0.05   # log-uniform
    st = np.array([r.steps for r in a])
    assert st.min() >= 500 and st.max() <= 5000


def test_retimed_stream_keeps_requests():
    a = S.request_stream(3, 200.0, 50)
    b = S.with_arrivals(a, 20.0, 9)
    assert [r.id for r in a] == [r.id for r in b]
    assert all(x.steps == y.steps and x.n == y.n for x, y in zip(a, b))
    assert b[-1].arrival > a[-1].arrival


def test_device_bytes_estimate_bounds_the_lattice(built):
    f32 = estimate_device_bytes((32, 32, 32), L.HC_FORM_MIXED_F32, 642, 1)
    f64 = estimate_device_bytes((32, 32, 32), L.HC_FORM_PLAIN_F64, 642, 1)
    N = 32 ** 3
    # at least the two population buffers and two force fields
    assert f32 >= N * (2 * 19 * 4 + 2 * 4 * 4)
    assert f64 >= N * (2 * 19 * 8 + 2 * 3 * 8)
    assert f64 > f32
    assert estimate_device_bytes((64, 32, 32), L.HC_FORM_MIXED_F32, 642, 1) > f32
    assert estimate_device_bytes((32, 32, 32), L.HC_FORM_MIXED_F32, 8 * 642, 8) > f32


def test_fifo_replay():
    lat, end = S.fifo_latencies([0.0, 0.5, 3.0], [1.0, 1.0, 0.5])
    assert np.allclose(lat, [1.0, 1.5, 0.5]) and end == 3.5
