"""The FP64 oracle against its committed golden dumps (tests/golden/), on the
CPU: the stage-by-stage mixed box and the 50^3 sheared RBC after 1000 steps
(the larger runs, minutes of oracle time, are checked on the GPU only).
Integer outputs (tile lists, cell ownership) must match exactly; floating
point within 1e-12 relative L2 (the oracle is deterministic; the margin
covers a last-bit difference of atan2 between the x86-64 and aarch64 C
libraries, which the platelet bending uses)."""
import os

import numpy as np
import pytest

from conftest import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
TOL = 1e-12


def _gen():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def check_against(got: dict, path: str, tol: float):
    ref = _gen().load(path)
    for k, b in ref.items():
        a = np.asarray(got[k])
        assert a.shape == b.shape, k
        if np.issubdtype(b.dtype, np.integer):
            assert np.array_equal(a, b), k
        else:
            assert rel_l2(a, b) <= tol, (k, rel_l2(a, b))


def test_oracle_stage_dumps_match_golden(built):
    g = _gen()
    check_against(g.stage_dumps(), g.STAGE_FILE, TOL)


def test_oracle_shear_rbc_1000_steps_match_golden(built):
    g = _gen()
    check_against(g.shear_run(), g.SHEAR_FILE, TOL)


def test_golden_files_are_small():
    """Small fixtures stay under 1 MB; the two full-field dumps (every vertex
    position and velocity of the pipe and of the 64^3 suspension) under 8 MB."""
    big = {"pipe_ht25_2000.npz", "kolmogorov_64_300.npz"}
    for f in os.listdir(GOLD):
        assert os.path.getsize(os.path.join(GOLD, f)) < (8_000_000 if f in big else 1_000_000), f
