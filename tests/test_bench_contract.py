"""bench.py prints the one JSON line its consumers read: the reference arm
on the CPU here, our arm (every leg, small sizes) on the GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
             "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def run_bench(*args, timeout=600):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                         timeout=timeout, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_line(built_lib):
    d = run_bench("--impl", "reference", "--steps", "3", "--warmup", "1", "--nx", "4", "--ny", "4", "--nz", "4",
                  "--p", "2")
    assert BASE_KEYS <= set(d)
    assert d["impl"] == "reference" and d["warmup"] == 3  # at least 3 warm-up steps
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["global_dofs"] == 9 ** 3 and d["value"] > 0


@pytest.mark.gpu
def test_our_arm_line(cuda):
    d = run_bench("--steps", "5", "--warmup", "3", "--nx", "6", "--ny", "6", "--nz", "6", "--p", "3",
                  "--batch-meshes", "8", "--served-requests", "400")
    assert BASE_KEYS <= set(d)
    assert {"roofline", "gpu_launches", "clocks", "batched", "served", "setup", "reference_device_equivalent",
            "partitioned"} <= set(d)
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and 0 < r["frac"] and r["peak"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == d["e2e"]["d2h_bytes_per_step"] == 8 * 6 ** 3 * 4 ** 3
    assert d["gpu_launches"] == 5 and d["steps"] == 5
    assert d["reference_device_equivalent"]["identical_results"]
    assert d["batched"]["identical_to_plain"]
    assert d["cpu_baseline"]["cores"] >= 1


@pytest.mark.parametrize("mode", ["gather", "scatter"])
def test_reference_arm_other_modes(built_lib, mode):
    d = run_bench("--impl", "reference", "--mode", mode, "--steps", "3", "--warmup", "1", "--nx", "4", "--ny", "4",
                  "--nz", "4", "--p", "2")
    assert BASE_KEYS <= set(d)
    assert d["metric"] == f"fp64 {mode.capitalize()} DOFS/s" and d["value"] > 0
    assert "Signed unique" in d["config"]["workload"]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["gather", "scatter"])
def test_our_arm_other_modes(cuda, mode):
    """Gather (Trans) and Scatter (NoTrans) on a Signed unique handle through
    the same harness; the GatherScatter-only legs are left out."""
    d = run_bench("--mode", mode, "--steps", "5", "--warmup", "3", "--nx", "6", "--ny", "6", "--nz", "6", "--p", "3")
    assert BASE_KEYS <= set(d)
    assert d["metric"] == f"fp64 {mode.capitalize()} DOFS/s"
    nl, ng = 6 ** 3 * 4 ** 3, 19 ** 3
    h2d, d2h = (8 * nl, 8 * ng) if mode == "gather" else (8 * ng, 8 * nl)
    assert (d["e2e"]["h2d_bytes_per_step"], d["e2e"]["d2h_bytes_per_step"]) == (h2d, d2h)
    assert d["batched"] is None and d["served"] is None and d["partitioned"] is None
    assert d["reference_device_equivalent"] is None and d["roofline"]["traffic"] is None
