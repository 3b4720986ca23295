"""The headless no_render driver (csrc/nbody_main.cpp over csrc/simulator.cpp):
the reference's argv and per-step stdout line (src/nbody.cpp:31-36, 83-123)."""
from __future__ import annotations

import re
import subprocess

import pytest

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu


def test_driver_prints_reference_lines():
    r = subprocess.run([str(nb.DRIVER_PATH), "4", "2", "0.999", "0.001", "1.0e-3", "2.0", "6"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 4                      # steps 3..6 after 2 warm steps
    pat = re.compile(r"^At step (\d+) kernel time is ([0-9.e+-]+) and mean is ([0-9.e+-]+) "
                     r"and stddev is: ([0-9.e+-]+)$")
    for k, ln in enumerate(lines):
        m = pat.match(ln)
        assert m, ln
        assert int(m.group(1)) == k + 3
        assert float(m.group(2)) > 0


def test_driver_rejects_unknown_method():
    r = subprocess.run([str(nb.DRIVER_PATH), "1", "1", "1", "1", "1", "1", "1", "64", "FOO"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "BRANCH or PREDICATED" in r.stderr


def test_driver_reference_order_state_is_the_reference_kernels(tmp_path):
    """Same argv as the reference's binary, reference-order accumulation: the final
    state equals the reference kernel's, run from the same initial disk
    (DiskGalaxySimulator's generator, simulator.cu:131-158), word for word."""
    import os

    import numpy as np

    import oracle_binding as orc

    if not orc.reference_available():
        pytest.skip("reference kernel cubin not built")
    batches, iters, frames = 4, 2, 6
    out = tmp_path / "state.f32"
    env = dict(os.environ, NBODY_GB300_ACCUMULATOR="reference_order",
               NBODY_GB300_STATE_OUT=str(out))
    r = subprocess.run([str(nb.DRIVER_PATH), str(batches), str(iters), "0.999", "0.001", "1.0e-3",
                        "2.0", str(frames)], capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stderr
    n = 256 * batches
    got = np.fromfile(out, dtype=np.float32).reshape(6, n)
    pos, vel = nb.reference_disk(n)
    ref, _ = orc.reference_run(pos, vel, 2.0, 0.001, 0.999, 1.0e-3, iters=iters * frames,
                               method=orc.BRANCH)
    assert all(np.array_equal(g.view(np.uint32), np.asarray(x, np.float32).view(np.uint32))
               for g, x in zip(got, ref))


def test_driver_rejects_unknown_accumulator():
    import os

    env = dict(os.environ, NBODY_GB300_ACCUMULATOR="kahan")
    r = subprocess.run([str(nb.DRIVER_PATH), "1", "1"], capture_output=True, text=True, timeout=60,
                       env=env)
    assert r.returncode == 1
    assert "reference_order" in r.stderr
