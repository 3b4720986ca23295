"""The C ABI from plain C99: the header compiles as C, the library links, and
without a GPU the call reports NB_ERR_NO_DEVICE instead of aborting."""
from __future__ import annotations

import shutil
import subprocess

import pytest

from c_abi_build import build_example


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c_example_builds_and_reports_missing_device(tmp_path):
    torch = pytest.importorskip("torch")
    exe = build_example(tmp_path)
    r = subprocess.run([str(exe), "4", "2"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    if not torch.cuda.is_available():
        assert r.stdout.startswith("no device")
