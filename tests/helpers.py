"""Shared helpers for the tests: error metrics and seeded inputs."""
from __future__ import annotations

import numpy as np

import nbody_gb300 as nb


def vec_errors(got, ref):
    """(relative RMS, max per-particle relative error) of 3-vectors given as
    [x, y, z] arrays.  Per-particle errors are taken relative to the particle's
    reference magnitude, floored at 1% of the RMS magnitude so that particles
    whose net force nearly cancels do not dominate."""
    g = np.stack([np.asarray(a, dtype=np.float64) for a in got])
    r = np.stack([np.asarray(a, dtype=np.float64) for a in ref])
    d = np.linalg.norm(g - r, axis=0)
    mag = np.linalg.norm(r, axis=0)
    rms = np.sqrt(np.mean(mag ** 2))
    if rms == 0.0:
        return float(np.max(d)), float(np.max(d))
    rel_rms = float(np.sqrt(np.mean(d ** 2)) / rms)
    rel_max = float(np.max(d / np.maximum(mag, 0.01 * rms)))
    return rel_rms, rel_max


def disk_case(n: int, seed: int = 1, eps: float = 1e-3):
    """Config-0 style thin disk: positions, velocities, masses (all float32)."""
    (x, y, z), (vx, vy, vz), m = nb.thin_disk(seed, n, eps)
    return [x, y, z], [vx, vy, vz], m


def params(n: int, G=1.0, dt=1e-3, damping=0.999, eps=1e-3, method=nb.BRANCH,
           acc=nb.ACC_PLAIN, iters=1) -> nb.SimParam:
    return nb.SimParam(numParticles=n, G=G, dt=dt, damping=damping, distEps=eps,
                       calcMethod=method, accumulator=acc, simIterationsPerFrame=iters)


def g_eff(G: float, m: float) -> float:
    """G * m rounded as the library folds an equal mass into G (float32)."""
    return float(np.float32(G) * np.float32(m))


def displacement_errors(got, ref, start):
    """Position errors relative to how far the particles moved: (RMS of |x_got -
    x_ref| over the RMS of |x_ref - x_start|, max per-particle |x_got - x_ref| over
    that particle's |x_ref - x_start| floored at 10% of the RMS displacement).
    Positions are [x, y, z] arrays."""
    g = np.stack([np.asarray(a, dtype=np.float64) for a in got])
    r = np.stack([np.asarray(a, dtype=np.float64) for a in ref])
    s = np.stack([np.asarray(a, dtype=np.float64) for a in start])
    d = np.linalg.norm(g - r, axis=0)
    disp = np.linalg.norm(r - s, axis=0)
    rms_disp = float(np.sqrt(np.mean(disp ** 2)))
    if rms_disp == 0.0:
        return float(np.max(d)), float(np.max(d))
    return (float(np.sqrt(np.mean(d ** 2)) / rms_disp),
            float(np.max(d / np.maximum(disp, 0.1 * rms_disp))))
