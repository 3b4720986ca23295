"""Generate the golden initial states of the reference's own generator.

    python tests/golden/initial_state/make_initial_state.py

Runs oracle/_ref/ref_ic_dump -- the reference's DiskGalaxySimulator constructor
(src/simulator.cu:24-34, randomParticlePos / initialParticleVel :131-158),
compiled unmodified from its sources by oracle/build_ref.sh with a host stand-in
for the CUDA runtime -- and writes reference_disk_n{N}.npz with its positions and
velocities.  tests/test_initial_state_cpu.py checks the library's
nb_ic_reference_disk against these files bit for bit.  Generated on x86-64 (glibc
libm), where the CPU tests run.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent.parent
DUMP = ROOT / "oracle" / "_ref" / "ref_ic_dump"
BATCHES = (1, 10)  # N = 256, 2560


def dump(batches: int, out: Path) -> dict:
    raw = out.with_suffix(".bin")
    subprocess.run([str(DUMP), str(raw), str(batches)], check=True)
    n = 256 * batches
    a = np.fromfile(raw, dtype=np.float32).reshape(6, n)
    raw.unlink()
    return dict(zip(("x", "y", "z", "vx", "vy", "vz"), a))


def main() -> int:
    if not DUMP.exists():
        print(f"{DUMP} missing: run oracle/build_ref.sh", file=sys.stderr)
        return 1
    for b in BATCHES:
        out = HERE / f"reference_disk_n{256 * b}.npz"
        np.savez_compressed(out, **dump(b, out))
        print("wrote", out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
