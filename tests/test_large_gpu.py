"""Size-independent properties at a size the CPU oracle cannot finish quickly:
N = 4,194,304 (a Plummer sphere generated on the device).  Sampled rows agree with
FP64 all-pairs rows, and the pair forces cancel in the total (momentum)."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
from helpers import params

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_4m_particles_sampled_rows_and_momentum():
    n = 1 << 22
    zeros = [np.zeros(n, np.float32)] * 3
    with nb.Simulation(params(n, eps=1e-4, acc=nb.ACC_COMPENSATED), zeros, zeros, None) as sim:
        sim.generate(nb.IC_PLUMMER, 42)
        a = sim.accelerations()
        rows = np.linspace(0, n - 1, 256).astype(np.uint64)
        f64 = sim.fp64_accelerations(rows)
    g = np.stack([c[rows.astype(np.int64)].astype(np.float64) for c in a])
    r = np.stack(f64)
    err = np.linalg.norm(g - r, axis=0)
    mag = np.linalg.norm(r, axis=0)
    assert np.sqrt(np.mean(err ** 2) / np.mean(mag ** 2)) <= 1e-5
    # equal masses: sum_i a_i = 0 up to rounding (pairwise antisymmetric forces)
    A = np.stack([c.astype(np.float64) for c in a])
    assert np.linalg.norm(A.sum(axis=1)) <= 1e-6 * np.abs(A).sum()
