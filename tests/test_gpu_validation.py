"""The reference's own validation of the membrane model, run on the GB300
plain FP64 form: tests/validation/stretch_cell/test_stretch_cell.cpp
stretches one RBC with +-F spread over its 7 outermost vertices for 10,000
steps and bounds the axial and transverse diameters (published
force-displacement curves, doi 10.3389/fphys.2017.00563) and the volume
change (+-2%)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (force pN, transverse lower, upper, axial lower, upper) in um, test_stretch_cell.cpp:158-162
BOUNDS = [(25, 7.3, 7.9, 9.2, 9.7), (75, 7.0, 7.5, 11.0, 12.0), (125, 6.5, 7.0, 12.25, 12.75)]


@pytest.mark.parametrize("force,tlo,thi,alo,ahi", BOUNDS)
def test_stretch_cell_force_displacement(built, force, tlo, thi, alo, ahi):
    from hemocell_gb300 import cases
    case = cases.stretch_cell()
    hc = case.build()
    x0, _, _ = hc.read_vertices()
    ids, f = cases.stretch_forces(x0, force)
    hc.set_vertex_forces(ids, f)
    _, vol0 = hc.read_cells()
    hc.iterate(case.steps)
    x, _, _ = hc.read_vertices()
    alive, vol = hc.read_cells()
    hc.close()
    assert alive.tolist() == [1]
    to_um = cases.DX * 1e6
    axial = (x[:, 0].max() - x[:, 0].min()) * to_um
    transverse = (x[:, 1].max() - x[:, 1].min()) * to_um
    print(f"F={force} pN axial={axial:.3f} um transverse={transverse:.3f} um vol ratio={vol[0] / vol0[0]:.4f}")
    assert 0.98 < vol[0] / vol0[0] <= 1.02
    assert tlo <= transverse <= thi
    assert alo <= axial <= ahi
