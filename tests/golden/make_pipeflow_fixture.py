"""Writes tests/golden/pipeflow_validation.npz from the reference's own inputs
of its pipe-flow validation (Validation.Pipeflow,
tests/validation/pipeflow/test_pipeflow.cpp of HemoCell):

  tests/validation/pipeflow/config_pipeflow.xml   domain, ibm and sim blocks
  tests/validation/pipeflow/RBC.pos, PLT.pos      cell centres [um] and angles [deg]
  tests/validation/pipeflow/RBC.xml, PLT.xml      MaterialModel blocks
  examples/pipeflow/tube.stl                      the ASCII STL tube

Only numbers are stored: the parsed configuration values, the .pos tables,
the material constants and the STL's triangle corners (as the doubles its
text parses to).  The reference tree exists only where this script runs; the
fixture is what the GPU test reads.

    python tests/golden/make_pipeflow_fixture.py [reference root]
"""
from __future__ import annotations

import os
import sys
import xml.etree.ElementTree as ET

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "pipeflow_validation.npz")


def read_pos(path: str) -> np.ndarray:
    with open(path) as fh:
        tok = fh.read().split()
    n = int(tok[0])
    return np.array([float(t) for t in tok[1:1 + 6 * n]], np.float64).reshape(n, 6)


def read_stl_ascii(path: str) -> np.ndarray:
    v = [[float(x) for x in line.split()[1:4]] for line in open(path) if line.strip().startswith("vertex")]
    return np.array(v, np.float64).reshape(-1, 3, 3)


def xml_value(root, *path) -> float:
    node = root
    for p in path:
        node = node.find(p)
    return float(node.text.strip())


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    vdir = os.path.join(ref, "tests", "validation", "pipeflow")
    cfg = ET.parse(os.path.join(vdir, "config_pipeflow.xml")).getroot()
    keys = {"dx": ("domain", "dx"), "dt": ("domain", "dt"), "nuP": ("domain", "nuP"), "rhoP": ("domain", "rhoP"),
            "kBT": ("domain", "kBT"), "Re": ("domain", "Re"), "refDir": ("domain", "refDir"),
            "refDirN": ("domain", "refDirN"), "fluidEnvelope": ("domain", "fluidEnvelope"),
            "stepMaterialEvery": ("ibm", "stepMaterialEvery"), "stepParticleEvery": ("ibm", "stepParticleEvery")}
    out = {f"cfg_{k}": np.array(xml_value(cfg, *p)) for k, p in keys.items()}
    for cell in ("RBC", "PLT"):
        mat = ET.parse(os.path.join(vdir, f"{cell}.xml")).getroot().find("MaterialModel")
        for k in ("kLink", "kBend", "kVolume", "kArea", "eta_m", "radius", "minNumTriangles"):
            out[f"{cell}_{k}"] = np.array(float(mat.find(k).text.strip()))
        out[f"{cell}_pos"] = read_pos(os.path.join(vdir, f"{cell}.pos"))
    plt = ET.parse(os.path.join(vdir, "PLT.xml")).getroot().find("MaterialModel")
    out["PLT_aspectRatio"] = np.array(float(plt.find("aspectRatio").text.strip()))
    out["stl_triangles"] = read_stl_ascii(os.path.join(ref, "examples", "pipeflow", "tube.stl"))
    np.savez_compressed(OUT, **out)
    print(OUT, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
