"""Seeded randomized parity sweep: random sizes, distributions, softenings, masses
and kernel shapes, each checked against the CPU oracle (FP32 restatement).

Random inputs include ill-conditioned sums (tight clusters, tiny softening) where a
particle's net force is a small difference of large pair terms, so the per-particle
bound is the summation bound: |a_gpu - a_oracle| <= 1e-5 * G sum_j m_j |r_ij| /
(r_ij^2 + eps)^(3/2), alongside the relative RMS bound of the other tests."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import params, vec_errors

pytestmark = pytest.mark.gpu


def make_case(rng):
    n = int(rng.integers(1, 3000))
    kind = rng.choice(["cube", "gauss", "clustered", "line"])
    if kind == "cube":
        x = rng.uniform(-1, 1, (3, n))
    elif kind == "gauss":
        x = rng.normal(0, 1, (3, n))
    elif kind == "clustered":
        centres = rng.normal(0, 1, (3, 4))
        x = centres[:, rng.integers(0, 4, n)] + rng.normal(0, 1e-2, (3, n))
    else:
        x = np.zeros((3, n))
        x[0] = np.linspace(-1, 1, n)
    eps = float(np.float32(rng.choice([0.0, 1e-6, 1e-4, 1e-2])))
    equal = bool(rng.integers(0, 2))
    m = np.full(n, 1.0 / n) if equal else rng.uniform(0.1, 2.0, n) / n
    return [a.astype(np.float32) for a in x], m.astype(np.float32), eps


@pytest.mark.parametrize("seed", range(24))
def test_random_case_matches_oracle(seed):
    rng = np.random.default_rng(1000 + seed)
    pos, m, eps = make_case(rng)
    n = pos[0].size
    vel = [np.zeros(n, np.float32)] * 3
    acc = nb.ACC_COMPENSATED if seed % 2 else nb.ACC_PLAIN
    with nb.Simulation(params(n, eps=eps, acc=acc), pos, vel, m) as sim:
        sim.set_kernel_config(seed % nb.num_kernel_configs())
        got = sim.accelerations()
    equal = bool(np.all(m == m[0]))
    ref = orc.accel_fp32(pos, None if equal else m, float(np.float32(m[0])) if equal else 1.0, eps)
    assert all(np.all(np.isfinite(g)) for g in got)
    if n == 1:
        assert all(np.all(g == 0) for g in got)
        return
    rms, _ = vec_errors(got, ref)
    assert rms <= 1e-5, (seed, n, eps, rms)
    # per-particle error against the sum of pair-term magnitudes (FP64)
    X = np.stack([p.astype(np.float64) for p in pos], 1)
    mm = m.astype(np.float64)  # G = 1
    absum = np.zeros(n)
    for lo in range(0, n, 512):
        r = X[None, :, :] - X[lo:lo + 512, None, :]
        d2 = (r * r).sum(-1) + eps
        with np.errstate(divide="ignore", invalid="ignore"):
            t = mm[None, :] * np.sqrt((r * r).sum(-1)) / d2 ** 1.5
        t[~np.isfinite(t)] = 0.0
        absum[lo:lo + 512] = t.sum(1)
    err = np.linalg.norm(np.stack(got).astype(np.float64) - np.stack(ref).astype(np.float64), axis=0)
    assert np.all(err <= 1e-5 * absum + 1e-30), (seed, n, eps, float(np.max(err / absum)))
