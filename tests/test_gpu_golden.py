"""The GPU plain FP64 form against the oracle's golden dumps (tests/golden/):
the 50^3 sheared RBC after 1000 steps, the 64x64x256 pipe with 279 RBC after
2000 steps and the 64^3 Kolmogorov suspension of RBC, PLT and a WBC after
300 steps.  Tile lists and cell ownership bit-exact; every vertex position
and velocity, sampled and averaged fluid velocity and density, centroids and
volumes within relative L2 1e-10.  The workloads are built with this
library's geometry, which equals the oracle's bit for bit
(tests/test_geometry_parity.py)."""
import os

import numpy as np
import pytest

from conftest import rel_l2
from test_golden import GOLD, check_against, _gen

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _summary(case, hc, positions=True):
    nx, ny, nz = case.dims
    x, v, _ = hc.read_vertices()
    alive, vol = hc.read_cells()
    rho, u = hc.read_fluid()
    fluid = case.flags_array() == 0
    uf = np.where(fluid[None, :], u, 0.0).reshape(3, nz, ny, nx)
    cnt = fluid.reshape(nz, ny, nx)
    nvs = [xyz.shape[0] for _, xyz in case.cells]
    offs = np.concatenate([[0], np.cumsum(nvs)])
    g = _gen()
    idx = g.sample_nodes(case.N, fluid)
    out = dict(alive=alive, volume=vol,
               centroids=np.array([x[offs[c]:offs[c + 1]].mean(axis=0) for c in range(len(nvs))]),
               u_plane=uf.sum(axis=(2, 3)) / np.maximum(cnt.sum(axis=(1, 2)), 1),
               u_column=uf.sum(axis=1) / np.maximum(cnt.sum(axis=0), 1),
               rho_sample=rho[idx], u_sample=u[:, idx], mass=np.array([rho[fluid].sum()]))
    b = hc.read_bins()
    for k in ("vertex_tile", "tile_offsets", "tile_cell_offsets", "tile_cells"):
        out[k] = b[k]
    if positions:
        out["x"], out["v"] = x, v
    return out


def test_gpu_shear_rbc_1000_steps_match_golden(built):
    from hemocell_gb300 import cases
    case = cases.shear_single_rbc(n=50, shear_rate=100.0, seed=1)
    hc = case.build()
    hc.iterate(1000)
    check_against(_summary(case, hc), _gen().SHEAR_FILE, TOL)
    hc.close()


@pytest.mark.parametrize("launch", [0, 1])
def test_gpu_pipe_2000_steps_match_golden(built, launch):
    from hemocell_gb300 import cases
    g = _gen()
    if not os.path.exists(g.PIPE_FILE):
        pytest.skip("pipe fixture not generated")
    case = cases.pipe_ht25(seed=1)
    hc = case.build(launch=launch)
    hc.iterate(2000)
    check_against(_summary(case, hc), g.PIPE_FILE, TOL)
    hc.close()


@pytest.mark.parametrize("launch", [0, 1])
def test_gpu_suspension_300_steps_match_golden(built, launch):
    from hemocell_gb300 import cases
    g = _gen()
    case = g.suspension_case(geo=cases.PRODUCT)
    assert {t for t, _ in case.cells} == {0, 1, 2}
    hc = case.build(launch=launch)
    hc.iterate(300)
    check_against(_summary(case, hc), g.SUSPENSION_FILE, TOL)
    hc.close()
