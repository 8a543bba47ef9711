"""The one-line JSON contract of bench.py (the reference arm on the CPU, our arm
on a GPU), at small sizes."""
import json
import os
import subprocess
import sys

import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, timeout):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.strip().splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def test_reference_arm_line():
    d = _run(["--impl", "reference", "--n-side", "10", "--steps", "1", "--warmup", "0", "--ref-budget", "30"], 600)
    assert BASE_KEYS <= set(d)
    assert d["impl"] == "reference" and d["metric"] == "particle-steps/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0


@pytest.mark.gpu
def test_gpu_arm_line():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    d = _run(["--n-side", "30", "--steps", "3", "--warmup", "3", "--batch-scenes", "4", "--batch-steps", "2",
              "--cpu-budget", "2"], 900)
    assert BASE_KEYS | {"roofline", "alu_roofline", "gpu_launches", "clocks", "batched"} <= set(d)
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["value"] > 0
    assert d["config"]["workload"] and d["config"]["fluid_particles"] == 27000
    roof = d["roofline"]
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= set(roof)
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and roof["frac"] == pytest.approx(
        roof["achieved"] / roof["peak"])
    alu = d["alu_roofline"]
    assert alu["unit"] == "TFLOP/s" and alu["peak"] > 0 and 0 < alu["frac"] < 1
    assert {"value", "unit", "cores", "kind", "sample"} <= set(d["cpu_baseline"])
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    assert d["batched"]["n_scenes"] == 4 and d["batched"]["value"] > 0
    # the window ends the 500-substep run; the other workloads ride on the same line
    assert d["config"]["window"].startswith("substeps 498..500 ")
    for k in ("twophase3d", "dambreak2d", "dambreak3d_cs10"):
        assert d[k]["value"] > 0 and d[k]["unit"] == "particle-steps/s" and d[k]["mean_incom_iter"] >= 2
    assert d["twophase3d"]["fluid_particles"] == 2000000 and d["dambreak2d"]["fluid_particles"] == 5000
    assert d["dambreak3d_cs10"]["fluid_particles"] == 1000000
    assert d["adjoint"]["unit"] == "ratio" and 0 < d["adjoint"]["value"] < 3
