"""Build tests/c_abi_example.c against the library (used by the C-ABI tests)."""
from __future__ import annotations

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
LIBDIR = ROOT / "cuda-to-sycl-nbody_gb300" / "nbody_gb300"


def build_example(tmp: Path) -> Path:
    exe = tmp / "c_abi_example"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-O1", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "c_abi_example.c"), "-o", str(exe), "-L", str(LIBDIR),
                    "-lnbody_gb300", f"-Wl,-rpath,{LIBDIR}"], check=True)
    return exe
