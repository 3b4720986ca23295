"""Test configuration: markers, import paths, and an up-to-date native build.

`-m "not gpu"` runs on any machine (oracle, host logic, ABI loading);
`-m gpu` needs a GB300 and calls the CUDA path through the C ABI.

Before collection the session brings the native library (cuda-to-sycl-nbody_gb300/
build.py, nvcc) and the CPU oracle (oracle/Makefile) up to date.  Both builds are
incremental, so this costs a fraction of a second when nothing changed, and a
fresh checkout needs no separate build step before the tests.
"""
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "cuda-to-sycl-nbody_gb300", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    # Temporary files of the tests stay inside the repository (git-ignored).
    if not config.option.basetemp:
        config.option.basetemp = str(ROOT / ".pytest_tmp")
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: full-size workload (seconds of GPU time)")
    subprocess.run([sys.executable, str(ROOT / "cuda-to-sycl-nbody_gb300" / "build.py")],
                   check=True, stdout=subprocess.DEVNULL)
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "all"], check=True,
                   stdout=subprocess.DEVNULL)
