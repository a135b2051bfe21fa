"""The benchmark's CPU-side contract: the reference arm's JSON line (it runs
the FP64 CPU restatement, so it needs no GPU), and the kernel names and
profiled DRAM traffic the GPU arm attaches to its roofline objects."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_arm_json_line():
    if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
        pytest.skip("oracle not built")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "MLUPS incl. IBM+cell forces" and d["unit"] == "MLUPS"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] >= 3 and d["n_gpus"] == 1
    assert d["dtype"] == "f64" and d["data"] == "synthetic"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the arm builds its workload with the oracle's geometry and loads no part of the GPU library
    assert d["native_libraries"] == ["liboracle.so"]
    cfg = d["config"]
    assert cfg["nodes"] == 64 * 64 * 256 and cfg["cells"] == 279 and cfg["vertices"] == 279 * 642


def test_step_kernel_names_follow_the_tuning():
    b = _bench()
    n = b.step_kernel_names([64, 2, 256, 256, 384, 0, 0, 9984])
    assert n == {"collide_stream": "k_collide_stream<float>", "node_velocity": "k_node_velocity_dense<float>",
                 "mechanics": "k_mechanics<float>"}
    n = b.step_kernel_names([32, 4, 64, 64, 384, 0, 2, 0x100 | 1])
    assert n == {"collide_stream": "k_collide_stream_fluid<float>", "node_velocity": "k_node_velocity_fluid<float>",
                 "mechanics": "k_mechanics_staged<float>"}
    assert b.step_kernel_names([0, 1, 64, 64, 256, 0, 1, 0x200 | 0x23])["collide_stream"] == \
        "k_collide_stream_bulk<float>"


def test_profiled_traffic_covers_the_step_kernels():
    """Every kernel the tuned FP32 step can launch on the pipe has a TRAFFIC
    line, with its bytes per launch and the commit of the capture."""
    b = _bench()
    for k in ("k_collide_stream<float>", "k_node_velocity_dense<float>", "k_mechanics<float>",
              "k_mechanics_staged<float>"):
        traffic, commit = b.profiled_traffic(k)
        assert traffic is not None and 1e6 < traffic < 1e9, k
        assert commit and len(commit) >= 7, k
    assert b.profiled_traffic("k_not_a_kernel<float>") == (None, None)
