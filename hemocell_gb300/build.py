"""Build the in-tree CUDA library ``libhcgpu.so`` for sm_103a.

Each translation unit is compiled in parallel with nvcc (one ``-gencode``)
and linked with ``-shared``.  A unit is rebuilt only when its source or a
header is newer than its object, so repeated ``build()`` calls are cheap.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhcgpu.so")
# the bounds-checked build (-DHC_CHECKED): every guarded index is compared with
# its array's length before the access and a violation sets a status bit
# instead of faulting; built on demand by build(checked=True)
BUILD_CHECKED = os.path.join(BUILD, "checked")
LIB_CHECKED = os.path.join(HERE, "libhcgpu_checked.so")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
UNITS = ["hc_lattice.cu", "hc_cells.cu", "hc_api.cu", "hc_noalloc.cu", "hc_batch.cu", "hc_host.cpp"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _headers_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    paths += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(p) for p in paths)


def _compile(unit: str, hdr_mtime: float, verbose: bool, checked: bool = False) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD_CHECKED if checked else BUILD, unit + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_mtime):
        return obj
    cmd = [_nvcc(), GENCODE, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE,
           "-I", CSRC, "-c", src, "-o", obj] + (["-DHC_CHECKED"] if checked else [])
    if unit.endswith(".cpp"):
        # host geometry without fused multiply-adds: the same doubles on x86-64
        # and aarch64, and the same as the FP64 CPU restatement's
        cmd[1:1] = ["-x", "c++", "-Xcompiler", "-ffp-contract=off"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj


EXAMPLES = {"oneCellShear": os.path.join(HERE, "cpp", "examples", "oneCellShear", "oneCellShear.cpp")}


def build_examples(verbose: bool = False) -> dict:
    """Compile the C++ case programs written against cpp/hemocell.h."""
    out = {}
    for name, src in EXAMPLES.items():
        exe = os.path.join(BUILD, name)
        deps = [src, os.path.join(HERE, "cpp", "hemocell.h"), os.path.join(HERE, "cpp", "config.h"), LIB]
        if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(d) for d in deps):
            cmd = ["g++", "-std=c++17", "-O2", "-o", exe, src, "-I", os.path.join(_cuda_home(), "include"),
                   "-L", HERE, "-lhcgpu", f"-Wl,-rpath,{HERE}"]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"example {name} failed to build:\n{r.stdout}\n{r.stderr}")
        out[name] = exe
    return out


def _cuda_home() -> str:
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build(verbose: bool = False, checked: bool = False) -> str:
    """Compile every unit and link libhcgpu.so (with checked=True the
    bounds-checked libhcgpu_checked.so instead); returns the library path."""
    os.makedirs(BUILD_CHECKED if checked else BUILD, exist_ok=True)
    lib = LIB_CHECKED if checked else LIB
    hdr = _headers_mtime()
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u, hdr, verbose, checked), UNITS))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        cmd = [_nvcc(), GENCODE, "-shared", "-o", lib] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if not checked:
        build_examples(verbose)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
