"""Checkpoints, cell information and the cell CSV output on the GPU.

A run saved at step 25 and continued to step 50 is compared with a fresh
handle that loads the checkpoint and runs the same 25 steps, into a handle
that already holds the cells and into one that receives them from the
checkpoint: FP64 within 1e-11 (only the order of the spread's atomic
additions can differ), FP32 within 1e-5, and the iteration, alive flags and
tile lists identical."""
import dataclasses
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _case():
    from hemocell_gb300 import cases
    return cases.mixed_box()


def _state(hc):
    x, v, f = hc.read_vertices()
    rho, u = hc.read_fluid()
    alive, vol = hc.read_cells()
    return dict(x=x, v=v, u=u, rho=rho, alive=alive, iter=hc.stats().iter)


@pytest.mark.parametrize("form,launch", [(0, 0), (0, 1), (1, 1)])
def test_checkpoint_restart_continues_the_run(built, tmp_path, form, launch):
    from hemocell_gb300.hemocell import HemoCellError
    case = _case()
    tol = 1e-11 if form == 0 else 1e-5
    a = case.build(form=form, launch=launch)
    a.iterate(25)
    ck = str(tmp_path / "checkpoint")
    a.saveCheckPoint(ck)
    a.saveCheckPoint(ck)                                   # the first set becomes *.old
    assert os.path.exists(os.path.join(ck, "lattice.dat.old"))
    a.iterate(25)
    ref = _state(a)
    fluid = case.flags_array() == 0
    for with_cells in (True, False):
        c = case if with_cells else dataclasses.replace(case, cells=[])
        b = c.build(form=form, launch=launch)
        b.loadCheckPoint(ck)
        assert b.stats().iter == 25 and b.stats().cells == len(case.cells)
        b.iterate(25)
        got = _state(b)
        assert got["iter"] == ref["iter"] == 50
        assert np.array_equal(got["alive"], ref["alive"])
        assert rel_l2(got["x"], ref["x"]) <= tol
        assert rel_l2(got["v"], ref["v"]) <= max(tol, 1e-10)
        assert rel_l2(got["u"][:, fluid], ref["u"][:, fluid]) <= tol
        b.close()
    wrong = dataclasses.replace(case, dims=(20, 18, 17), flags=None, walls={}).build(form=form, launch=launch)
    with pytest.raises(HemoCellError):
        wrong.loadCheckPoint(ck)
    wrong.close()
    a.close()


def test_cell_info_and_csv(built, tmp_path):
    case = _case()
    hc = case.build()
    hc.iterate(10)
    info = hc.cell_info()
    x, v, _ = hc.read_vertices()
    alive, vol = hc.read_cells()
    off = 0
    for c, (t, xyz) in enumerate(case.cells):
        nv = xyz.shape[0]
        p, w = x[off:off + nv], v[off:off + nv]
        tris = case.types[t].mesh.tris
        r = p - p[0]
        a, b, cc = r[tris[:, 0]], r[tris[:, 1]], r[tris[:, 2]]
        area = 0.5 * np.linalg.norm(np.cross(b - a, cc - a), axis=1).sum()
        volume = np.einsum("ij,ij->i", a, np.cross(b, cc)).sum() / 6.0
        d = np.sqrt(((p[:, None, :] - p[None, :, :]) ** 2).sum(-1)).max()
        cen = p.mean(axis=0)
        for ax, n in enumerate(case.dims):
            if case.periodic[ax]:
                cen[ax] -= n * np.floor(cen[ax] / n)
        assert np.allclose(info[c, 0:3], cen, rtol=1e-12, atol=1e-12)
        assert np.allclose(info[c, 3:6], w.mean(axis=0), rtol=1e-12, atol=1e-15)
        assert info[c, 6] == pytest.approx(area, rel=1e-12)
        assert info[c, 7] == pytest.approx(volume, rel=1e-12)
        assert info[c, 7] == pytest.approx(vol[c], rel=1e-10)
        assert info[c, 8] == pytest.approx(d, rel=1e-12)
        assert np.allclose(info[c, 9:15], [p[:, 0].min(), p[:, 0].max(), p[:, 1].min(), p[:, 1].max(),
                                           p[:, 2].min(), p[:, 2].max()])
        assert info[c, 15] == (t if alive[c] else -1)
        off += nv
    out = str(tmp_path / "csv")
    hc.writeCellInfo_CSV(out, si_units=True)
    dx, dt = 0.5e-6, 1e-7
    for t, spec in enumerate(case.types):
        path = os.path.join(out, f"{spec.name}.{10:012d}.csv")
        lines = open(path).read().strip().splitlines()
        assert lines[0] == "X,Y,Z,area,volume,atomic_block,cellId,baseCellId,velocity_x,velocity_y,velocity_z"
        rows = [list(map(float, ln.split(","))) for ln in lines[1:]]
        mine = [c for c in range(len(case.cells)) if info[c, 15] == t]
        assert len(rows) == len(mine)
        for row, c in zip(rows, mine):
            assert row[6] == c
            assert row[0] == pytest.approx(info[c, 0] * dx, rel=1e-12)
            assert row[4] == pytest.approx(info[c, 7] * dx ** 3, rel=1e-12)
            assert row[8] == pytest.approx(info[c, 3] * dx / dt, rel=1e-12, abs=1e-300)
    hc.close()


def test_write_output_fields(built, tmp_path):
    """writeOutput: the XDMF descriptors name the reference's fields and the
    raw arrays hold exactly what the readback calls return."""
    import xml.etree.ElementTree as ET
    case = _case()
    hc = case.build()
    hc.iterate(5)
    out = str(tmp_path / "out")
    hc.writeOutput(out)
    d = os.path.join(out, "hdf5")
    nx, ny, nz = case.dims
    root = ET.parse(os.path.join(d, "Fluid.000000000005.xmf")).getroot()
    names = [a.get("Name") for a in root.iter("Attribute")]
    assert names == ["Velocity", "Density", "Force"]
    vel = np.fromfile(os.path.join(d, "Fluid.000000000005.Velocity.bin"), np.float32).reshape(nz * ny * nx, 3)
    rho, u = hc.read_fluid()
    assert np.allclose(vel, u.T.astype(np.float32))
    x, v, f = hc.read_vertices()
    alive, _ = hc.read_cells()
    written = 0
    for t, spec in enumerate(case.types):
        base = os.path.join(d, f"{spec.name}.000000000005")
        root = ET.parse(base + ".xmf").getroot()
        assert [a.get("Name") for a in root.iter("Attribute")] == ["Velocity", "Total force", "Cell Id"]
        pos = np.fromfile(base + ".Position.bin", np.float32).reshape(-1, 3)
        tri = np.fromfile(base + ".Triangles.bin", np.int32).reshape(-1, 3)
        cid = np.fromfile(base + ".CellId.bin", np.int32)
        nv = spec.mesh.nv
        cells = [c for c, (tt, _) in enumerate(case.cells) if tt == t and alive[c]]   # deleted cells are left out
        assert pos.shape[0] == nv * len(cells) and tri.shape[0] == spec.mesh.nf * len(cells)
        assert sorted(set(cid.tolist())) == cells
        for k, c in enumerate(cells):
            c0 = sum(case.cells[q][1].shape[0] for q in range(c))
            assert np.allclose(pos[k * nv:(k + 1) * nv], x[c0:c0 + nv].astype(np.float32))
        if cells:
            assert tri.max() == pos.shape[0] - 1
        written += len(cells)
    assert written == int(alive.sum()) > 0
    hc.close()
