"""The reference-default initial state, pinned to the reference's own generator.

nb_ic_reference_disk (and so nb_sim_create_disk_galaxy / DiskGalaxySimulator with
no state given) must reproduce DiskGalaxySimulator::randomParticlePos and
initialParticleVel (src/simulator.cu:131-158) bit for bit.  The pins:
  * golden files written by the reference's own constructor
    (tests/golden/initial_state/, made by make_initial_state.py);
  * the same constructor run live (oracle/_ref/ref_ic_dump, built from the
    reference's unmodified sources by oracle/build_ref.sh) at more sizes, including
    the reference's default of 12,800 particles, where that binary exists."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

import nbody_gb300 as nb

HERE = Path(__file__).resolve().parent
GOLDEN = HERE / "golden" / "initial_state"
DUMP = HERE.parent / "oracle" / "_ref" / "ref_ic_dump"
COMPONENTS = ("x", "y", "z", "vx", "vy", "vz")


def library_state(n):
    (x, y, z), (vx, vy, vz) = nb.reference_disk(n)
    return dict(zip(COMPONENTS, (x, y, z, vx, vy, vz)))


@pytest.mark.parametrize("name", sorted(p.name for p in GOLDEN.glob("reference_disk_n*.npz")))
def test_library_matches_reference_generator_golden(name):
    d = np.load(GOLDEN / name)
    n = d["x"].size
    got = library_state(n)
    for c in COMPONENTS:
        assert np.array_equal(got[c], d[c]), (name, c, int(np.sum(got[c] != d[c])))


@pytest.mark.skipif(not DUMP.exists(), reason="oracle/_ref/ref_ic_dump not built "
                    "(oracle/build_ref.sh needs the reference checkout)")
@pytest.mark.parametrize("batches", [1, 3, 50])
def test_library_matches_reference_generator_live(batches, tmp_path):
    out = tmp_path / "state.bin"
    subprocess.run([str(DUMP), str(out), str(batches)], check=True, timeout=120)
    n = 256 * batches
    ref = np.fromfile(out, dtype=np.float32).reshape(6, n)
    got = library_state(n)
    for c, r in zip(COMPONENTS, ref):
        assert np.array_equal(got[c], r), (n, c, int(np.sum(got[c] != r)))
