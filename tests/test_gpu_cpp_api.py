"""The C++ mirror of the HemoCell case API (hemocell_gb300/cpp/hemocell.h):
the oneCellShear case program builds against it, reads config.xml, RBC.xml
and RBC.pos like the reference, and runs on the GPU."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(exe, case_dir, *args):
    r = subprocess.run([exe, "config.xml", *args], cwd=case_dir, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return [l for l in r.stdout.splitlines() if l.startswith("iter ")][-1].split()


def test_one_cell_shear_program(built, tmp_path):
    exe = os.path.join(ROOT, "hemocell_gb300", "_build", "oneCellShear")
    src = os.path.join(ROOT, "hemocell_gb300", "cpp", "examples", "oneCellShear")
    case_dir = str(tmp_path / "oneCellShear")
    shutil.copytree(src, case_dir)
    r = subprocess.run([exe, "config.xml", "200"], cwd=case_dir, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [l for l in r.stdout.splitlines() if l.startswith("iter ")][-1].split()
    assert int(line[1]) == 200
    vol_ratio = float(line[3])
    assert abs(vol_ratio - 1.0) < 0.02
    bbox = [float(v) for v in line[5:8]]
    assert 7.0 < max(bbox) < 9.0  # RBC diameter ~7.8 um stays a disc under weak shear
    # outputs at the configured intervals: cell CSV and checkpoints
    assert os.path.exists(os.path.join(case_dir, "tmp", "csv", "RBC.000000000100.csv"))
    assert os.path.exists(os.path.join(case_dir, "tmp", "checkpoint", "lattice.dat.old"))
    # resuming from the checkpoint at 200 reaches the same state as one run to 300
    straight = _run(exe, case_dir, "300")          # writes its own checkpoints (the last at 300)
    shutil.rmtree(os.path.join(case_dir, "tmp"))
    _run(exe, case_dir, "200")
    resumed = _run(exe, case_dir, "300", "resume")
    assert resumed[1] == straight[1] == "300"
    for a, b in zip(resumed[5:8], straight[5:8]):      # bounding box (the volume ratio is per run)
        assert abs(float(a) - float(b)) <= 1e-9 * abs(float(b))
