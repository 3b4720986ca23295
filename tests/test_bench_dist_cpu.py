"""The benchmark's multi-rank path on CPU: world size 2 over gloo (127.0.0.1).
With N GPUs the benchmark runs N independent replicas; the whole-job rate is
all ranks' pair interactions over the slowest rank's time."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), NB_BENCH_BACKEND="gloo")
    sys.path.insert(0, str(ROOT))
    import bench

    r, w = bench.dist_init()
    try:
        slowest = bench.max_over_ranks(1.0 + r, w)
        rate = bench.whole_job_rate(1000.0, 2.0 + 2 * r, w)
        bench.barrier(w)
        q.put((r, w, slowest, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_benchmark():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[:2] for o in out] == [(0, 2), (1, 2)]
    for _, _, slowest, rate in out:
        assert slowest == 2.0                     # max over ranks
        assert rate == pytest.approx(2 * 1000.0 / 4.0)


def test_reference_arm_json_contract():
    """`bench.py --impl reference` runs on host cores only, so its whole JSON line can
    be checked here: the keys and meanings the benchmark contract asks for."""
    import json
    import subprocess

    # Run the arm in a process that afterwards reports whether the library under
    # test was ever mapped: the reference arm must not load it.
    script = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3',\n"
        "            '--cpu-seconds', '0.5']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "except SystemExit as e:\n"
        "    assert not e.code, e.code\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('LIBRARY_MAPPED' if 'libnbody_gb300' in maps else 'LIBRARY_NOT_MAPPED',\n"
        "      file=sys.stderr)\n")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True,
                       timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    assert "LIBRARY_NOT_MAPPED" in r.stderr, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0 and line["unit"] == "pair-interactions/s"
    assert line["steps"] == 1 and line["warmup"] >= 3 and line["higher_is_better"] is True
    assert line["config"]["workload"].startswith("Plummer sphere N=1048576")
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
