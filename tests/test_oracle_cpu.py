"""CPU checks of the oracle itself: known answers, conservation laws, agreement of
its FP32 restatement with its FP64 all-pairs sum, and the reference's PREDICATED
behaviour.  (The oracle is pinned to the reference kernel by
tests/test_golden_cpu.py and tests/test_parity_gpu.py.)"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_binding as orc
from helpers import disk_case, vec_errors


def test_two_body_known_answer():
    # Two unit masses at distance d: a = r / (d^2 + eps)^(3/2) towards each other.
    d, eps, G = 0.75, 1e-3, 2.0
    pos = [np.array([0.0, d], np.float32), np.zeros(2, np.float32), np.zeros(2, np.float32)]
    ax, ay, az = orc.accel_fp32(pos, None, G, eps)
    want = G * d / (d * d + eps) ** 1.5
    assert np.isclose(ax[0], want, rtol=1e-6) and np.isclose(ax[1], -want, rtol=1e-6)
    assert ay[0] == 0 and az[1] == 0
    bx, _, _ = orc.accel_fp64(pos, None, G, eps)
    assert np.isclose(bx[0], want, rtol=1e-12)


def test_single_particle_feels_no_force():
    pos = [np.array([0.3], np.float32)] * 3
    a = orc.accel_fp32(pos, None, 1.0, 1e-7)
    assert all(v[0] == 0 for v in a)


def test_fp32_restatement_agrees_with_fp64():
    pos, vel, m = disk_case(3000, seed=3)
    a32 = orc.accel_fp32(pos, None, float(np.float32(m[0])), 1e-3)
    a64 = orc.accel_fp64(pos, m, 1.0, 1e-3)
    rms, mx = vec_errors(a32, a64)
    assert rms < 1e-5 and mx < 1e-4


def test_momentum_conserved_without_damping():
    # With damping = 1 the step conserves total momentum up to FP32 rounding.
    pos, vel, m = disk_case(1500, seed=4)
    G = float(np.float32(m[0]))
    out = orc.run_fp32(pos, vel, None, G, 1e-3, 1.0, 1e-3, iters=5)
    p0 = np.array([np.sum(v.astype(np.float64)) for v in vel])
    p1 = np.array([np.sum(v.astype(np.float64)) for v in out[3:]])
    scale = np.sum(np.abs(vel[0].astype(np.float64)))
    assert np.all(np.abs(p1 - p0) < 1e-5 * scale)


def test_predicated_as_shipped_gives_zero_force():
    # src/simulator.cu:208-209 multiplies by (i == id): only the self term
    # survives, and it is 0 * rsqrt(eps^3) = 0.
    pos, vel, _ = disk_case(500, seed=5)
    a = orc.accel_fp32(pos, None, 1.0, 1e-3, method=orc.PREDICATED)
    assert all(np.all(v == 0) for v in a)
    out = orc.run_fp32(pos, vel, None, 1.0, 1e-3, 0.999, 1e-3, iters=1, method=orc.PREDICATED)
    for v0, v1 in zip(vel, out[3:]):
        assert np.array_equal(v1, v0 * np.float32(0.999))


def test_predicated_with_zero_softening_is_nan():
    # eps = 0: the self term is 0 * rsqrt(0) = NaN in the reference's arithmetic.
    pos, _, _ = disk_case(64, seed=6)
    a = orc.accel_fp32(pos, None, 1.0, 0.0, method=orc.PREDICATED)
    assert np.all(np.isnan(a[0]))
    b = orc.accel_fp32(pos, None, 1.0, 0.0, method=orc.BRANCH)
    assert np.all(np.isfinite(b[0]))


@pytest.mark.parametrize("n", [1, 2, 17])
def test_energy_of_small_systems(n):
    pos, vel, m = disk_case(n, seed=7)
    e = orc.energy_fp64(pos, vel, m, 1.0, 1e-3)
    x = np.stack([p.astype(np.float64) for p in pos], 1)
    v = np.stack([u.astype(np.float64) for u in vel], 1)
    mm = m.astype(np.float64)
    ke = 0.5 * np.sum(mm * np.sum(v * v, 1))
    pe = 0.0
    for i in range(n):
        for j in range(i + 1, n):
            pe -= mm[i] * mm[j] / np.sqrt(np.sum((x[i] - x[j]) ** 2) + 1e-3)
    assert np.isclose(e["kinetic"], ke, rtol=1e-12) and np.isclose(e["potential"], pe, rtol=1e-12,
                                                                     atol=1e-300)


def test_timed_cpu_port_agrees_with_oracle():
    # oracle/cpu_port.c: the same kernel body built -O3 -ffast-math for the timed
    # baseline; reordered sums (and possibly an rsqrt estimate) stay within 1e-4.
    pos, _, m = disk_case(3000, seed=5)
    G = float(np.float32(m[0]))
    rows = np.arange(0, 3000, 7)
    got = orc.port_accel(pos, G, 1e-3, rows=rows)
    ref = orc.accel_fp32(pos, None, G, 1e-3, rows=rows)
    rms, mx = vec_errors(got, ref)
    assert rms <= 1e-4 and mx <= 1e-4, (rms, mx)
    both = orc.port_accel(pos, G, 0.0, rows=np.array([0, 1]))   # eps = 0: j == i left out
    assert all(np.all(np.isfinite(a)) for a in both)


@pytest.mark.parametrize("seed,n", [(20261203, 4096), (7, 1), (11, 333)])
def test_workload_plummer_is_the_library_generator_bit_for_bit(seed, n):
    # The benchmark's reference arm makes its Plummer inputs with the oracle's
    # restatement (it never loads the library); both must give the same floats.
    import nbody_gb300 as nb

    a = orc.plummer(seed, n)
    b = nb.plummer(seed, n)
    for u, v in zip(list(a[0]) + list(a[1]) + [a[2]], list(b[0]) + list(b[1]) + [b[2]]):
        assert np.array_equal(u, v)
