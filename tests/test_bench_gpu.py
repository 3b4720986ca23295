"""The benchmark's own arm on a small case: its JSON line carries every key the
benchmark contract asks for, with consistent values (the full 1M-particle run is
the benchmark itself)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_bench_json_contract_small_case():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--n", "65536", "--steps", "3",
                        "--warmup", "3", "--no-extras", "--no-cpu"],
                       capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "roofline", "e2e", "gpu_launches", "clocks", "accumulators"):
        assert key in d, key
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] >= 3
    assert d["value"] > 0 and d["unit"] == "pair-interactions/s" and d["dtype"] == "f32"
    assert d["value"] == pytest.approx(65536.0 ** 2 / (d["ms_per_step"] * 1e-3), rel=1e-6)
    rf = d["roofline"]
    assert rf["bound"] == "fp32" and rf["unit"] == "TFLOP/s"
    assert rf["frac"] == pytest.approx(rf["achieved"] / rf["peak"], rel=1e-9)
    assert 0.0 < rf["frac"] < 1.05 and 0.0 < rf["frac_of_measured"] < 1.1
    e2e = d["e2e"]
    assert e2e["unit"] == d["unit"] and 0 < e2e["value"] <= d["value"] * 1.05
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] == 3
    assert set(d["accumulators"]) == {"plain", "compensated", "reference_order"}
    assert d["config"]["accumulator"] in d["accumulators"]
    assert d["clocks"]["samples"] >= 0


def test_bench_split_mode_small_case():
    # --split: the one system over the job's GPUs (here a one-rank NCCL group);
    # the timed step includes the all-gather of positions.
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--split", "--n", "65536",
                        "--steps", "3", "--warmup", "3", "--no-extras", "--no-cpu"],
                       capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().splitlines()[-1].startswith("{")   # the JSON line comes last
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["scaling"] == "strong" and d["n_gpus"] == 1
    assert d["config"]["parallelism"].startswith("split1")
    assert d["value"] == pytest.approx(65536.0 ** 2 / (d["ms_per_step"] * 1e-3), rel=1e-6)
    assert d["e2e"]["value"] > 0 and d["gpu_launches"] == 3
