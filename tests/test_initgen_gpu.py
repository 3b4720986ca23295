"""Initial conditions generated on the GPU (nb_sim_generate) against the host
generators with the same seeds: same draws, values equal to within one float
rounding of the transcendental functions."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
from helpers import params

pytestmark = pytest.mark.gpu


def host(kind, seed, n, eps):
    if kind == nb.IC_THIN_DISK:
        return nb.thin_disk(seed, n, eps)
    if kind == nb.IC_PLUMMER:
        return nb.plummer(seed, n)
    return nb.two_disks(seed, n, eps)


def close(a, b):
    scale = max(1.0, float(np.max(np.abs(b))))
    assert np.max(np.abs(a - b)) <= 2e-6 * scale
    assert np.mean(a == b) > 0.95          # most values identical bit for bit


@pytest.mark.parametrize("kind", [nb.IC_THIN_DISK, nb.IC_PLUMMER, nb.IC_TWO_DISKS])
def test_device_generation_matches_host(kind):
    n, seed, eps = 20000, 123, float(np.float32(1e-3))
    (x, y, z), (vx, vy, vz), m = host(kind, seed, n, eps)
    zeros = [np.zeros(n, np.float32)] * 3
    with nb.Simulation(params(n, eps=eps), zeros, zeros, None) as sim:
        sim.generate(kind, seed)
        got = sim.get_state()
        acc_dev = sim.accelerations()
        sim.set_state((x, y, z), (vx, vy, vz), m)
        acc_host = sim.accelerations()
    for g, h in zip(got, (x, y, z, vx, vy, vz)):
        close(g, h)
    # masses came with the generation: same accelerations as the host state
    for a, b in zip(acc_dev, acc_host):
        assert np.allclose(a, b, rtol=1e-3, atol=1e-3 * np.max(np.abs(b)))


def test_ensemble_generation_uses_seed_plus_system_index():
    sizes = [64, 300, 1000]
    seed = 77
    zeros = [np.zeros(sum(sizes), np.float32)] * 3
    with nb.Simulation(params(sum(sizes)), zeros, zeros, None, sizes=sizes) as sim:
        sim.generate(nb.IC_PLUMMER, seed)
        got = sim.get_state()
    off = 0
    for k, s in enumerate(sizes):
        (x, y, z), (vx, vy, vz), _ = nb.plummer(seed + k, s)
        for g, h in zip(got, (x, y, z, vx, vy, vz)):
            close(g[off:off + s], h)
        off += s


def test_two_disks_need_even_sizes():
    zeros = [np.zeros(33, np.float32)] * 3
    with nb.Simulation(params(33), zeros, zeros, None) as sim:
        with pytest.raises(nb.NbError) as e:
            sim.generate(nb.IC_TWO_DISKS, 1)
        assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
