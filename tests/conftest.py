"""Test configuration: markers and import paths.

`-m "not gpu"` runs on any machine (oracle, host logic, ABI loading);
`-m gpu` needs a GB300 and calls the CUDA path through the C ABI.
"""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "cuda-to-sycl-nbody_gb300", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: full-size workload (seconds of GPU time)")
