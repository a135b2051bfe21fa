"""The C++ mirror of the HemoCell case API (hemocell_gb300/cpp/hemocell.h):
the oneCellShear case program builds against it, reads config.xml, RBC.xml
and RBC.pos like the reference, and runs on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_one_cell_shear_program(built):
    exe = os.path.join(ROOT, "hemocell_gb300", "_build", "oneCellShear")
    case_dir = os.path.join(ROOT, "hemocell_gb300", "cpp", "examples", "oneCellShear")
    r = subprocess.run([exe, "config.xml", "200"], cwd=case_dir, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [l for l in r.stdout.splitlines() if l.startswith("iter ")][-1].split()
    assert int(line[1]) == 200
    vol_ratio = float(line[3])
    assert abs(vol_ratio - 1.0) < 0.02
    bbox = [float(v) for v in line[5:8]]
    assert 7.0 < max(bbox) < 9.0  # RBC diameter ~7.8 um stays a disc under weak shear
