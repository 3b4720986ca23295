"""GPU parity of the reference-order accumulator (NB_ACC_REFERENCE_ORDER): bit for
bit against the reference kernel particle_interaction<BRANCH>
(src/simulator.cu:186-229) -- its golden fixtures and live runs of the kernel
itself, built from the reference's source -- on the same inputs.

Tolerance: none.  Every output word (x, y, z, vx, vy, vz) must be identical.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import disk_case, params, vec_errors

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
BRANCH_CASES = sorted(p.stem for p in GOLDEN.glob("*.npz")
                      if json.loads(str(np.load(p)["params"]))["method"] == nb.BRANCH)
needs_reference = pytest.mark.skipif(not orc.reference_available(),
                                     reason="reference kernel cubin not built")


def same_bits(got, ref):
    return all(np.array_equal(np.asarray(g, np.float32).view(np.uint32),
                              np.asarray(r, np.float32).view(np.uint32))
               for g, r in zip(got, ref))


def ro_params(n, **kw):
    return params(n, acc=nb.ACC_REFERENCE_ORDER, **kw)


def test_branch_golden_cases_present():
    assert {"thin_disk_n2048", "force_sum_n1000", "perf_args_n1280", "ragged_n333",
            "reference_default_n1024"} <= set(BRANCH_CASES)


@pytest.mark.parametrize("name", BRANCH_CASES)
def test_bitwise_equal_to_golden_fixtures(name):
    d = np.load(GOLDEN / f"{name}.npz")
    prm = json.loads(str(d["params"]))
    pos = [d["x"], d["y"], d["z"]]
    vel = [d["vx"], d["vy"], d["vz"]]
    out = [d[f"out_{c}"] for c in ("x", "y", "z", "vx", "vy", "vz")]
    n = pos[0].size
    p = nb.SimParam(numParticles=n, G=prm["G"], dt=prm["dt"], damping=prm["damping"],
                    distEps=prm["eps"], calcMethod=nb.BRANCH, accumulator=nb.ACC_REFERENCE_ORDER)
    with nb.Simulation(p, pos, vel, None) as sim:
        sim.advance(prm["iters"])
        got = sim.get_state()
    assert same_bits(got, out), name


@needs_reference
@pytest.mark.parametrize("n,eps,iters", [(1, 1e-3, 2), (2, 1e-3, 2), (17, 1e-3, 3),
                                         (333, 0.0, 3), (1000, 1e-3, 5), (4099, 1e-3, 2),
                                         (25600, 1e-3, 10)])
def test_bitwise_equal_to_reference_kernel(n, eps, iters):
    pos, vel, _ = disk_case(n, seed=n + 7, eps=max(eps, 1e-6))
    ref, _ = orc.reference_run(pos, vel, 1.0, 1e-3, 0.999, eps, iters=iters, method=orc.BRANCH)
    with nb.Simulation(ro_params(n, eps=eps), pos, vel, None) as sim:
        sim.advance(iters)
        got = sim.get_state()
    assert same_bits(got, ref)


@needs_reference
def test_ensemble_systems_each_equal_to_reference_kernel():
    sizes = [333, 17, 1000, 2048, 1]
    rng = np.random.default_rng(5)
    pos = [rng.uniform(-1, 1, sum(sizes)).astype(np.float32) for _ in range(3)]
    vel = [rng.uniform(-0.1, 0.1, sum(sizes)).astype(np.float32) for _ in range(3)]
    p = ro_params(sum(sizes), eps=1e-3)
    with nb.Simulation(p, pos, vel, None, sizes=sizes) as sim:
        sim.advance(3)
        got = sim.get_state()
    start = 0
    for n in sizes:
        sl = slice(start, start + n)
        ref, _ = orc.reference_run([a[sl] for a in pos], [a[sl] for a in vel], 1.0, 1e-3, 0.999,
                                   1e-3, iters=3, method=orc.BRANCH)
        assert same_bits([g[sl] for g in got], ref), n
        start += n


def test_per_system_launches_and_graph_match_one_launch():
    sizes = [700, 64, 1500]
    rng = np.random.default_rng(9)
    pos = [rng.uniform(-1, 1, sum(sizes)).astype(np.float32) for _ in range(3)]
    vel = [np.zeros(sum(sizes), np.float32) for _ in range(3)]
    p = ro_params(sum(sizes))
    outs = []
    for how in ("advance", "per_system", "graph"):
        with nb.Simulation(p, pos, vel, None, sizes=sizes) as sim:
            if how == "advance":
                sim.advance(4)
            elif how == "per_system":
                sim.advance_per_system(4)
            else:
                sim.graph_capture(4)
                sim.graph_launch()
            outs.append(sim.get_state())
    assert same_bits(outs[1], outs[0]) and same_bits(outs[2], outs[0])


def test_accelerations_agree_with_oracle():
    n = 3000
    pos, vel, m = disk_case(n, seed=3)
    with nb.Simulation(ro_params(n), pos, vel, None) as sim:
        got = sim.accelerations()
    rms, mx = vec_errors(got, orc.accel_fp32(pos, None, 1.0, 1e-3))
    assert rms <= 1e-5 and mx <= 1e-4


def test_unequal_masses_are_rejected():
    """At creation, and by set_state (which then leaves the state untouched)."""
    n = 64
    pos, vel, _ = disk_case(n, seed=4)
    m = np.linspace(1.0, 2.0, n).astype(np.float32)
    with pytest.raises(nb.NbError) as e:
        nb.Simulation(ro_params(n), pos, vel, m)
    assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
    with nb.Simulation(ro_params(n), pos, vel, None) as sim:
        before = sim.get_state()
        with pytest.raises(nb.NbError) as e:
            sim.set_state(pos, vel, m)
        assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
        assert same_bits(sim.get_state(), before)
        sim.set_state(pos, vel, np.full(n, 0.5, np.float32))   # equal masses: accepted
        sim.advance(1)


@needs_reference
@pytest.mark.parametrize("eps", [1e-3, 0.0])
def test_coincident_particles_match_reference_kernel(eps):
    """Particles at identical positions: with eps > 0 their mutual term is exactly
    zero; with eps = 0 it is 0 * rsqrt(0) = NaN in the reference, and NaN must appear
    in the same words here (NaN payloads aside)."""
    n = 600
    pos, vel, _ = disk_case(n, seed=21)
    for a in pos:
        a[300:310] = a[0]           # ten copies of particle 0's position
        a[500] = a[499]
    iters = 1 if eps == 0.0 else 2   # NaN positions would reach every particle in step 2
    ref, _ = orc.reference_run(pos, vel, 1.0, 1e-3, 0.999, eps, iters=iters, method=orc.BRANCH)
    with nb.Simulation(ro_params(n, eps=eps), pos, vel, None) as sim:
        sim.advance(iters)
        got = sim.get_state()
    for g, r in zip(got, ref):
        assert np.array_equal(np.isnan(g), np.isnan(r))
        fin = ~np.isnan(r)
        assert np.array_equal(g[fin].view(np.uint32), r[fin].view(np.uint32))
    if eps == 0.0:
        assert np.isnan(ref[3][0]) and np.isnan(ref[3][300]) and np.isnan(ref[3][500])
        assert not np.isnan(ref[3][1])
    else:
        assert all(np.all(np.isfinite(r)) for r in ref)


@needs_reference
@pytest.mark.parametrize("seed", range(24))
def test_random_cases_bitwise_equal_to_reference_kernel(seed):
    """Seeded random sizes, softenings (zero included), G, dt, damping, iteration
    counts and position scales: every output word equals the reference kernel's."""
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.choice([1, 2, 3, 31, 32, 33, 255, 256, 257, 511, 1023, 1025]) if seed < 8
            else rng.integers(1, 6000))
    eps = float(np.float32([0.0, 1e-6, 1e-4, 1e-3, 1e-2, 0.1][seed % 6]))
    G = float(np.float32(10 ** rng.uniform(-3, 1)))
    dt = float(np.float32(10 ** rng.uniform(-4, -2)))
    damping = float(np.float32(rng.choice([1.0, 0.999, 0.9])))
    iters = int(rng.integers(1, 5))
    scale = 10 ** rng.uniform(-1, 2)
    pos = [(rng.standard_normal(n) * scale).astype(np.float32) for _ in range(3)]
    vel = [(rng.standard_normal(n) * 0.1).astype(np.float32) for _ in range(3)]
    ref, _ = orc.reference_run(pos, vel, G, dt, damping, eps, iters=iters, method=orc.BRANCH)
    p = nb.SimParam(numParticles=n, G=G, dt=dt, damping=damping, distEps=eps,
                    calcMethod=nb.BRANCH, accumulator=nb.ACC_REFERENCE_ORDER)
    with nb.Simulation(p, pos, vel, None) as sim:
        sim.advance(iters)
        got = sim.get_state()
    assert same_bits(got, ref), (n, eps, G, dt, damping, iters)


@needs_reference
def test_thousand_steps_bitwise_equal_to_reference_kernel():
    """1000 iterations of the 25,600-particle thin disk (N = 25,600, unit masses with G = 1/N):
    the trajectories are chaotic, so any single rounding difference would have
    grown into visible divergence; every word still matches."""
    n, iters = 25600, 1000
    pos, vel, _ = disk_case(n, seed=2024)
    G = float(np.float32(1.0 / n))
    ref, _ = orc.reference_run(pos, vel, G, 1e-3, 0.999, 1e-3, iters=iters, method=orc.BRANCH)
    p = nb.SimParam(numParticles=n, G=G, dt=1e-3, damping=0.999, distEps=1e-3,
                    calcMethod=nb.BRANCH, accumulator=nb.ACC_REFERENCE_ORDER)
    with nb.Simulation(p, pos, vel, None) as sim:
        sim.advance(iters)
        got = sim.get_state()
    assert same_bits(got, ref)
    # the tuned kernel follows a different rounding path and ends elsewhere
    p.accumulator = nb.ACC_PLAIN
    with nb.Simulation(p, pos, vel, None) as sim:
        sim.advance(iters)
        fast = sim.get_state()
    assert not same_bits(fast, ref)


@needs_reference
@pytest.mark.parametrize("n", [25600, 150000, 200000, 300000, 1 << 20])
def test_every_shape_and_autotune_stay_bitwise(n):
    """The default shape depends on the size: the largest i-tiles that still fill the
    GPU (the stream-K grid hands split i-tiles over between CTAs); the autotuner
    picks among all shapes; every choice gives the reference's bits."""
    pos, vel, _ = disk_case(n, seed=31)
    G = float(np.float32(1.0 / n))
    ref, _ = orc.reference_run(pos, vel, G, 1e-3, 0.999, 1e-3, iters=2, method=orc.BRANCH)
    p = nb.SimParam(numParticles=n, G=G, dt=1e-3, damping=0.999, distEps=1e-3,
                    calcMethod=nb.BRANCH, accumulator=nb.ACC_REFERENCE_ORDER)
    with nb.Simulation(p, pos, vel, None) as sim:
        default = sim.kernel_info()["config_index"]
        chosen = sim.autotune()
        assert chosen <= -1 and sim.kernel_info()["config_index"] == chosen
        sim.advance(2)
        got = sim.get_state()
    # the largest i-tiles that give every SM two CTAs (one for 384 x 2, where only one
    # fits): 384 x 2 (1536 particles) from 233,472 up; 256 x 1 (512) from 155,648;
    # 128 x 1 (256) from 77,824; below that 64 x 1 (128)
    want = {25600: -4, 150000: -3, 200000: -2, 300000: -1, 1 << 20: -1}[n]
    assert default == want, (n, default)
    assert same_bits(got, ref)


@needs_reference
def test_shape_selection_by_index_stays_bitwise():
    # nb_sim_set_kernel_config selects the reference-order kernel's shapes by index in
    # this mode (reported back as -1 - index); every shape gives the reference's bits.
    n = 40000
    pos, vel, _ = disk_case(n, seed=37)
    G = float(np.float32(1.0 / n))
    ref, _ = orc.reference_run(pos, vel, G, 1e-3, 0.999, 1e-3, iters=2, method=orc.BRANCH)
    p = nb.SimParam(numParticles=n, G=G, dt=1e-3, damping=0.999, distEps=1e-3,
                    calcMethod=nb.BRANCH, accumulator=nb.ACC_REFERENCE_ORDER)
    with nb.Simulation(p, pos, vel, None) as sim:
        shapes = 0
        while True:
            try:
                sim.set_kernel_config(shapes)
            except nb.NbError as e:
                assert e.status == nb.NB_ERR_INVALID_ARGUMENT
                break
            assert sim.kernel_info()["config_index"] == -1 - shapes
            sim.set_state(pos, vel)
            sim.advance(2)
            assert same_bits(sim.get_state(), ref), shapes
            shapes += 1
        assert shapes == 4
        sim.set_kernel_config(-1)                     # back to the default
        assert sim.kernel_info()["config_index"] <= -1
