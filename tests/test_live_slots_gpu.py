"""The force kernel's live-slot variant (csrc/force_kernel.cuh, kLive): in a system's
last, partly filled i-tile it runs only the register slots that hold a particle, on a
stream-K work list that charges each block by those slots (csrc/worklist.hpp).  The
host picks it where it saves at least 1 % of the slot work.  These tests check that
choice and compare the variant's accelerations and steps with the CPU oracle, system
by system, for both accumulators and both mass modes (reference semantics:
src/simulator.cu:193-228)."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import disk_case, displacement_errors, g_eff, params, vec_errors

pytestmark = pytest.mark.gpu

ACC_RMS, ACC_MAX = 1e-5, 1e-4
POS_REL, POS_REL_MAX = 1e-4, 1e-3
# Systems whose last i-tiles hold 1-3 slots' worth of particles for 256- and
# 128-thread shapes, between whole tiles and a single particle.
SIZES = [100, 300, 70, 2000, 1500, 33, 5000, 1, 640, 2048]


def _ensemble(mass_mode, seed=7):
    parts = [disk_case(s, seed=seed + k) for k, s in enumerate(SIZES)]
    pos = [np.concatenate([p[0][c] for p in parts]) for c in range(3)]
    vel = [np.concatenate([p[1][c] for p in parts]) for c in range(3)]
    m = np.concatenate([p[2] for p in parts])
    if mass_mode == "random":
        rng = np.random.default_rng(seed)
        m = (m * rng.uniform(0.5, 1.5, m.size)).astype(np.float32)
    return pos, vel, m


def test_variant_is_chosen_only_where_it_pays():
    pos, vel, m = _ensemble("equal")
    with nb.Simulation(params(int(sum(SIZES))), pos, vel, m, sizes=SIZES) as sim:
        sim.set_kernel_config(1)                 # 256 x 4: 1024-particle i-tiles
        assert sim.kernel_info()["live_slots"] == 1
    # one system of whole i-tiles keeps the full-slot kernel
    (x, y, z), (vx, vy, vz), mm = nb.plummer(3, 65536)
    with nb.Simulation(params(65536), (x, y, z), (vx, vy, vz), mm) as sim:
        sim.set_kernel_config(9)                 # 256 x 4 x 2048
        assert sim.kernel_info()["live_slots"] == 0


@pytest.mark.parametrize("cfg", [1, 8, 9, 12])
@pytest.mark.parametrize("acc", [nb.ACC_PLAIN, nb.ACC_COMPENSATED])
@pytest.mark.parametrize("mass_mode", ["equal", "random"])
def test_live_variant_matches_oracle(cfg, acc, mass_mode):
    pos, vel, m = _ensemble(mass_mode)
    n = int(sum(SIZES))
    with nb.Simulation(params(n, acc=acc), pos, vel, m, sizes=SIZES) as sim:
        sim.set_kernel_config(cfg)
        assert sim.kernel_info()["live_slots"] == 1
        a = sim.accelerations()
        sim.advance(3)
        st = sim.get_state()
    off = 0
    for k, s in enumerate(SIZES):
        sl = slice(off, off + s)
        ps, vs, ms = [c[sl] for c in pos], [c[sl] for c in vel], m[sl]
        if mass_mode == "equal":
            G, om = g_eff(1.0, ms[0]), None
        else:
            G, om = 1.0, ms
        if s > 1:
            ref = orc.accel_fp32(ps, om, G, 1e-3)
            rms, mx = vec_errors([c[sl] for c in a], ref)
            assert rms <= ACC_RMS and mx <= ACC_MAX, (cfg, k, s, rms, mx)
        r3 = orc.run_fp32(ps, vs, om, G, 1e-3, 0.999, 1e-3, iters=3)
        if s > 1:
            rms, mx = displacement_errors([c[sl] for c in st[:3]], r3[:3], ps)
            assert rms <= POS_REL and mx <= POS_REL_MAX, (cfg, k, s, rms, mx)
        else:
            for g, r in zip(st[:3], r3[:3]):
                assert g[sl][0] == r[0]
        off += s
