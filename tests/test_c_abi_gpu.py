"""The C ABI from plain C99 on a GPU: the reference's main-loop calls run."""
from __future__ import annotations

import subprocess

import pytest

from c_abi_build import build_example

pytestmark = pytest.mark.gpu


def test_c_example_runs(tmp_path):
    exe = build_example(tmp_path)
    r = subprocess.run([str(exe), "4", "2", "0.999", "0.001", "1e-3", "2.0"], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("ok ") and "n=1024" in r.stdout
