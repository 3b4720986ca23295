"""The headless no_render driver (csrc/nbody_main.cpp over csrc/simulator.cpp):
the reference's argv and per-step stdout line (src/nbody.cpp:138-248)."""
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
