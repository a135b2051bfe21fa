"""The integer floor/fraction of FP64 coordinates used by the mixed-form cell
kernels (hemocell_gb300/csrc/hc_posbits.h) against the FP64 operations it
replaces, compiled for the host with g++ (strict IEEE, no contraction)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_split_matches_fp64_operations(tmp_path):
    exe = str(tmp_path / "posbits_check")
    src = os.path.join(ROOT, "tests", "posbits_check.cpp")
    inc = os.path.join(ROOT, "hemocell_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", inc, src, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
    assert int(r.stdout.split()[1]) > 3_000_000
