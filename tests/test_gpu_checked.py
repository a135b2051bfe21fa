"""The bounds-checked build (libhcgpu_checked.so, -DHC_CHECKED): the
population pulls, the wall-class and IBM flag loads, the collision's stores
and each cell's vertex range compare their index with the array's length
first; a violation sets status bit 4 and skips the access, so nothing traps.
Small cases run on it in a child process (the checked library replaces the
product one there) against the FP64 oracle: moving and resting walls,
periodic faces crossed by cells, a lattice of one- and two-node axes, all
three cell types, per stage and batched, both forms.  Each must stay clean
(no index caught) and match the oracle as the product build does."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys, numpy as np
sys.path.insert(0, ROOT); sys.path.insert(0, ROOT + "/tests")
from hemocell_gb300 import _lib as L, cases as C
from oracle import oracle as orc
from conftest import rel_l2
assert L.LIB_PATH.endswith("libhcgpu_checked.so"), L.LIB_PATH
out = []
def run(name, case, form, launch, steps, tol):
    hc = case.build(form=form, launch=launch)
    o = orc.apply_case(case)
    hc.iterate(steps)
    o.step(steps)
    fluid = case.flags_array() == 0
    alive = o.read_cells()[0] if case.cells else np.zeros(0, np.int32)
    ex = 0.0
    if case.cells:
        keep = np.concatenate([np.full(x.shape[0], bool(alive[k])) for k, (_, x) in enumerate(case.cells)])
        ex = rel_l2(hc.read_vertices()[0][keep], o.read_vertices()[0][keep])
    eu = rel_l2(hc.read_fluid()[1][:, fluid], o.read_fluid()[1][:, fluid])
    st = hc.device_status()
    hc.close()
    print(name, form, launch, "%.2e %.2e" % (ex, eu), st, flush=True)
    assert st & 16 == 0, (name, "index check", st)
    assert ex < tol and eu < tol, (name, ex, eu)
mixed = C.mixed_box(wall=True)
kolm = C.kolmogorov_mix(n=36, rbc_fraction=0.15, n_wbc=1, plt_per_rbc=0.5, wbc_triangles=1280, seed=5)
pipe = C.pipe_ht25(nx=24, ny=24, nz=32, radius=10.0, n_cells=4, seed=3)
thin = C.Case("thin", (5, 2, 6), (1, 0, 1), body_mode=L.HC_BODY_UNIFORM, body=(1e-6, 0.0, 2e-6))
for form, tol in ((0, 1e-10), (1, 1e-4)):
    for launch in (0, 1):
        run("mixed", mixed, form, launch, 30, tol)
        run("kolmogorov", kolm, form, launch, 20, tol)
        run("pipe", pipe, form, launch, 20, tol)
        run("thin", thin, form, launch, 20, tol)
print("CLEAN")
'''


def test_checked_build_runs_clean(built):
    from hemocell_gb300 import build as B
    B.build(checked=True)
    env = dict(os.environ, HEMOCELL_GB300_CHECKED="1")
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + CHILD], env=env, capture_output=True,
                       text=True, timeout=1200)
    print(r.stdout[-4000:])
    assert r.returncode == 0 and "CLEAN" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]
