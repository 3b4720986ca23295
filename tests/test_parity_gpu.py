"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle, the FP64
all-pairs sum and the reference's own kernel, on the same seeded inputs.

Tolerances (FP32 pair arithmetic; rsqrt is MUFU on the GPU, correctly rounded in
the oracle):
  accelerations   relative RMS <= 1e-5, per-particle max <= 1e-4 (helpers.vec_errors)
  positions       after 10 iterations, relative to the displacement over those
                  iterations: RMS <= 1e-4, per particle <= 1e-3 with the displacement
                  floored at 10% of its RMS (helpers.displacement_errors)
  velocities      max |dv| <= 1e-4 * max |v|
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import disk_case, displacement_errors, g_eff, params, vec_errors

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"

ACC_RMS = 1e-5
ACC_MAX = 1e-4
POS_REL = 1e-4       # of the RMS displacement
POS_REL_MAX = 1e-3   # per particle, displacement floored at 10% of its RMS
EPS32 = float(np.float32(1e-3))  # the softening as the library stores it


def make_sim(n, seed=1, eps=1e-3, method=nb.BRANCH, acc=nb.ACC_PLAIN, mass="equal", cfg=None,
             **kw):
    pos, vel, m = disk_case(n, seed=seed, eps=max(eps, 1e-6))
    if mass == "random":
        rng = np.random.default_rng(seed)
        m = (rng.uniform(0.5, 1.5, n) / n).astype(np.float32)
    elif mass == "unit":
        m = None
    p = params(n, eps=eps, method=method, acc=acc, **kw)
    sim = nb.Simulation(p, pos, vel, m)
    if cfg is not None:
        sim.set_kernel_config(cfg)
    return sim, pos, vel, m


def assert_positions(got, ref, start):
    rms, mx = displacement_errors(got, ref, start)
    assert rms <= POS_REL and mx <= POS_REL_MAX, (rms, mx)


def oracle_G(m, G=1.0):
    """Oracle call arguments equivalent to the library's mass handling."""
    if m is None:
        return None, G
    if np.all(m == m[0]):
        return None, g_eff(G, m[0])
    return m, G


@pytest.mark.parametrize("n", [1, 2, 3, 15, 16, 17, 255, 256, 257, 1000, 4099])
def test_accelerations_match_oracle(n):
    sim, pos, vel, m = make_sim(n, seed=n)
    with sim:
        got = sim.accelerations()
    om, G = oracle_G(m)
    ref32 = orc.accel_fp32(pos, om, G, 1e-3)
    ref64 = orc.accel_fp64(pos, m, 1.0, EPS32)
    if n == 1:
        assert all(np.all(g == 0) for g in got)
        return
    for ref in (ref32, ref64):
        rms, mx = vec_errors(got, ref)
        assert rms <= ACC_RMS and mx <= ACC_MAX, (n, rms, mx)


@pytest.mark.parametrize("cfg", range(nb.num_kernel_configs()))
def test_every_kernel_shape_matches_oracle(cfg):
    n = 5000
    sim, pos, vel, m = make_sim(n, seed=11, cfg=cfg)
    with sim:
        got = sim.accelerations()
    om, G = oracle_G(m)
    rms, mx = vec_errors(got, orc.accel_fp32(pos, om, G, 1e-3))
    assert rms <= ACC_RMS and mx <= ACC_MAX


@pytest.mark.parametrize("acc", [nb.ACC_PLAIN, nb.ACC_COMPENSATED])
@pytest.mark.parametrize("mass", ["equal", "random", "unit"])
def test_ten_steps_match_oracle(acc, mass):
    n = 2048
    sim, pos, vel, m = make_sim(n, seed=21, acc=acc, mass=mass)
    with sim:
        sim.advance(10)
        got = sim.get_state()
    om, G = oracle_G(m)
    ref = orc.run_fp32(pos, vel, om, G, 1e-3, 0.999, 1e-3, iters=10)
    assert_positions(got[:3], ref[:3], pos)
    vscale = max(float(np.max(np.abs(r))) for r in ref[3:])
    dv = max(float(np.max(np.abs(g - r))) for g, r in zip(got[3:], ref[3:]))
    assert dv <= POS_REL * vscale


def test_thin_disk_25600_accelerations_against_fp64():
    # N = 25,600 thin disk, eps2 = 1e-3, m = 1/N, G = 1 (the CPU-runnable case).
    n = 25600
    sim, pos, vel, m = make_sim(n, seed=2024)
    with sim:
        got = sim.accelerations()
        rows = np.arange(0, n, 7)
        f64 = sim.fp64_accelerations(rows)
    ref = orc.accel_fp64(pos, m, 1.0, EPS32)
    rms, mx = vec_errors(got, ref)
    assert rms <= ACC_RMS and mx <= ACC_MAX
    # the GPU FP64 rows agree with the CPU FP64 oracle (same float32 softening)
    for a, b in zip(f64, ref):
        assert np.allclose(a, b[rows], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("acc", [nb.ACC_PLAIN, nb.ACC_COMPENSATED, nb.ACC_REFERENCE_ORDER])
def test_two_body_known_answer(acc):
    # Two unit masses a distance d apart along a direction u: each accelerates
    # towards the other with G d / (d^2 + eps)^(3/2) (simulator.cu:200-206), equal
    # and opposite to the last bit; one step from rest with damping 1 moves each by
    # a dt^2 (:214-228).
    d, eps, G, dt = 0.75, 1e-3, 2.0, 1e-2
    u = np.array([2.0, -1.0, 2.0]) / 3.0
    p0, p1 = -0.5 * d * u, 0.5 * d * u
    pos = [np.array([p0[c], p1[c]], np.float32) for c in range(3)]
    vel = [np.zeros(2, np.float32)] * 3
    m = np.ones(2, np.float32)
    with nb.Simulation(params(2, G=G, dt=dt, damping=1.0, eps=eps, acc=acc), pos, vel, m) as sim:
        a = sim.accelerations()
        sim.advance(1)
        st = sim.get_state()
    r = np.array([pos[c][1] - pos[c][0] for c in range(3)], np.float64)
    want = G * r / (float(r @ r) + eps) ** 1.5
    for c in range(3):
        assert np.isclose(a[c][0], want[c], rtol=2e-6, atol=1e-7), (c, a[c][0], want[c])
        assert a[c][1] == -a[c][0]
        assert np.isclose(st[3 + c][0], want[c] * dt, rtol=2e-6, atol=1e-9)
        assert np.isclose(st[c][0], pos[c][0] + want[c] * dt * dt, rtol=1e-6, atol=1e-9)


def test_zero_softening_excludes_self_pair():
    # eps = 0: the self term would be 0 * inf; the reference skips it (:206).
    n = 700
    sim, pos, vel, m = make_sim(n, seed=31, eps=0.0)
    with sim:
        got = sim.accelerations()
    assert all(np.all(np.isfinite(g)) for g in got)
    om, G = oracle_G(m)
    rms, mx = vec_errors(got, orc.accel_fp32(pos, om, G, 0.0))
    assert rms <= ACC_RMS and mx <= ACC_MAX


def test_predicated_matches_oracle_bitwise():
    n = 1000
    sim, pos, vel, m = make_sim(n, seed=41, method=nb.PREDICATED, mass="unit", G=2.0)
    with sim:
        sim.advance(3)
        got = sim.get_state()
    ref = orc.run_fp32(pos, vel, None, 2.0, 1e-3, 0.999, 1e-3, iters=3, method=orc.PREDICATED)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


def _same_words(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32),
                          np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("mass", ["random", "equal"])
def test_predicated_both_kernels_match_oracle_bitwise(mass):
    # Equal masses run the sequential-order kernel with the PREDICATED pair term;
    # per-particle masses keep the one-thread-per-particle kernel.  Both give the
    # oracle's words, here with a coincident pair (0 * rsqrt(...) of a finite term).
    n = 3001
    sim, pos, vel, m = make_sim(n, seed=43, method=nb.PREDICATED, mass=mass)
    with sim:
        sim.advance(2)
        got = sim.get_state()
    om, G = oracle_G(m)
    ref = orc.run_fp32(pos, vel, om, G, 1e-3, 0.999, 1e-3, iters=2, method=orc.PREDICATED)
    for g, r in zip(got, ref):
        assert _same_words(g, r)


def test_predicated_zero_softening_gives_nan_like_reference():
    n = 64
    sim, pos, vel, m = make_sim(n, seed=42, eps=0.0, method=nb.PREDICATED, mass="unit")
    with sim:
        a = sim.accelerations()
    assert np.all(np.isnan(a[0]))


def test_deterministic_and_graph_equivalent():
    n = 30000  # several split i-tiles per CTA
    sim, pos, vel, m = make_sim(n, seed=51)
    with sim:
        sim.advance(4)
        a = sim.get_state()
        sim.set_state(pos, vel)
        sim.advance(4)
        b = sim.get_state()
        sim.set_state(pos, vel)
        sim.graph_capture(4)
        sim.graph_launch()
        c = sim.get_state()
        sim.set_state(pos, vel)
        sim.advance(1)                 # start the graph from the other buffer
        sim.graph_capture(3)
        sim.graph_launch()
        d = sim.get_state()
    for u, v, w, q in zip(a, b, c, d):
        assert np.array_equal(u, v) and np.array_equal(u, w) and np.array_equal(u, q)


def test_step_matches_stepsim_contract():
    # stepSim runs simIterationsPerFrame iterations and records the time.
    n = 4096
    sim, pos, vel, m = make_sim(n, seed=61, iters=5)
    with sim:
        sim.step()
        assert sim.last_step_ms() > 0
        got = sim.get_state()
    om, G = oracle_G(m)
    ref = orc.run_fp32(pos, vel, om, G, 1e-3, 0.999, 1e-3, iters=5)
    assert_positions(got[:3], ref[:3], pos)


def test_ensemble_matches_per_system_oracle():
    sizes = [1, 17, 64, 300, 1000, 2500, 16, 4097]
    parts = [disk_case(s, seed=100 + k) for k, s in enumerate(sizes)]
    pos = [np.concatenate([p[0][c] for p in parts]) for c in range(3)]
    vel = [np.concatenate([p[1][c] for p in parts]) for c in range(3)]
    m = np.concatenate([p[2] for p in parts])
    p = params(int(sum(sizes)))
    with nb.Simulation(p, pos, vel, m, sizes=sizes) as sim:
        assert sim.num_systems() == len(sizes)
        acc = sim.accelerations()
        sim.advance(3)
        st = sim.get_state()
        sim.set_state(pos, vel)
        sim.advance_per_system(3)
        st2 = sim.get_state()
    off = 0
    for k, s in enumerate(sizes):
        sl = slice(off, off + s)
        ps = [a[sl] for a in pos]
        ref = orc.accel_fp32(ps, None, g_eff(1.0, m[off]), 1e-3)
        if s > 1:
            rms, mx = vec_errors([a[sl] for a in acc], ref)
            assert rms <= ACC_RMS and mx <= ACC_MAX, (k, s, rms, mx)
        r3 = orc.run_fp32(ps, [v[sl] for v in vel], None, g_eff(1.0, m[off]), 1e-3, 0.999, 1e-3,
                          iters=3)
        if s > 1:
            assert_positions([g[sl] for g in st[:3]], r3[:3], ps)
            assert_positions([g[sl] for g in st2[:3]], r3[:3], ps)
        else:
            for g, g2, r in zip(st[:3], st2[:3], r3[:3]):
                assert g[sl][0] == r[0] and g2[sl][0] == r[0]
        off += s


def test_reference_disk_runs_like_reference_defaults():
    p = nb.SimParam(numParticles=2560)  # reference defaults: G=2, dt=0.005, eps=1e-7, unit mass
    sim = nb.DiskGalaxySimulator(p)
    (x, y, z), (vx, vy, vz) = nb.reference_disk(2560)
    assert np.array_equal(sim.getParticlePos()[0], x)
    sim.stepSim()
    ref = orc.run_fp32([x, y, z], [vx, vy, vz], None, 2.0, np.float32(0.005),
                       np.float32(0.999998), np.float32(1e-7), iters=4)
    assert_positions(sim.getParticlePos(), ref[:3], [x, y, z])
    assert sim.getLastStepTime() > 0
    assert sim.getNumParticles() == 2560 and sim.getGwSize() == 64 and sim.getCM() == nb.BRANCH
    assert "GB300" in sim.getDeviceName()


# ----------------------------------------------------------- the reference's own kernel
needs_ref = pytest.mark.skipif(not orc.reference_available(),
                               reason="reference cubin not built (oracle/build_ref.sh)")


@needs_ref
@pytest.mark.parametrize("n", [256, 1000, 25600])
def test_accelerations_match_reference_kernel(n):
    # With damping = 0, dt = 1, G = 1 the reference kernel's velocity output is its
    # force sum: v' = 0 * v + (F * 1) * 1 (simulator.cu:214-216).
    pos, vel, m = disk_case(n, seed=7 * n)
    zeros = [np.zeros(n, np.float32)] * 3
    out, _ = orc.reference_run(pos, zeros, 1.0, 1.0, 0.0, 1e-3, iters=1)
    p = params(n, G=1.0)
    with nb.Simulation(p, pos, zeros, None) as sim:
        got = sim.accelerations()
    rms, mx = vec_errors(got, out[3:])
    assert rms <= ACC_RMS and mx <= ACC_MAX
    # and the oracle against the reference kernel
    rms, mx = vec_errors(orc.accel_fp32(pos, None, 1.0, 1e-3), out[3:])
    assert rms <= ACC_RMS and mx <= ACC_MAX


@needs_ref
@pytest.mark.parametrize("n,eps", [(300000, 1e-3), (5000, 0.0)])
def test_predicated_stream_k_matches_reference_kernel_bitwise(n, eps):
    # At N = 300,000 the PREDICATED mode runs the sequential-order kernel with split
    # i-tiles handed over between CTAs; eps = 0 turns every particle's sum to NaN
    # through its own 0 * rsqrt(0) term, as in the reference.
    pos, vel, _ = disk_case(n, seed=3 * n + 1)
    ref, _ = orc.reference_run(pos, vel, 2.0, 1e-3, 0.999, eps, iters=2, method=nb.PREDICATED,
                               gw_size=128)
    with nb.Simulation(params(n, G=2.0, eps=eps, method=nb.PREDICATED), pos, vel, None) as sim:
        info = sim.kernel_info()
        sim.advance(2)
        got = sim.get_state()
    assert info["config_index"] <= -1
    if n == 300000:
        assert info["split_tiles"] > 0
    for g, r in zip(got, ref):
        assert _same_words(g, r)


@needs_ref
@pytest.mark.parametrize("method", [nb.BRANCH, nb.PREDICATED])
def test_ten_steps_match_reference_kernel(method):
    # Config-0 parameters: G_eff = G * m with the reference's unit-mass kernel.
    n = 25600
    pos, vel, m = disk_case(n, seed=99)
    G = g_eff(1.0, m[0])
    ref, _ = orc.reference_run(pos, vel, G, 1e-3, 0.999, 1e-3, iters=10, method=method)
    p = params(n, method=method)
    with nb.Simulation(p, pos, vel, m) as sim:
        sim.advance(10)
        got = sim.get_state()
    if method == nb.BRANCH:
        assert_positions(got[:3], ref[:3], pos)
    else:
        # PREDICATED moves the particles by their velocities only (zero force).
        scale = max(float(np.max(np.abs(r))) for r in ref[:3])
        assert max(float(np.max(np.abs(g - r))) for g, r in zip(got[:3], ref[:3])) <= 1e-6 * scale
    if method == nb.PREDICATED:
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("*.npz")))
def test_library_matches_golden_fixtures(name):
    d = np.load(GOLDEN / f"{name}.npz")
    prm = json.loads(str(d["params"]))
    pos = [d["x"], d["y"], d["z"]]
    vel = [d["vx"], d["vy"], d["vz"]]
    out = [d[f"out_{c}"] for c in ("x", "y", "z", "vx", "vy", "vz")]
    n = pos[0].size
    p = nb.SimParam(numParticles=n, G=prm["G"], dt=prm["dt"], damping=prm["damping"],
                    distEps=prm["eps"], calcMethod=prm["method"])
    with nb.Simulation(p, pos, vel, None) as sim:
        sim.advance(prm["iters"])
        got = sim.get_state()
    if prm["method"] == nb.PREDICATED:
        for g, r in zip(got, out):
            assert np.array_equal(g, r)
    elif prm["damping"] == 0.0 and prm["dt"] == 1.0:
        rms, mx = vec_errors(got[3:], out[3:])
        assert rms <= ACC_RMS and mx <= ACC_MAX
    else:
        assert_positions(got[:3], out[:3], pos)


@pytest.mark.parametrize("acc", [nb.ACC_PLAIN, nb.ACC_COMPENSATED])
def test_coincident_particles_like_reference(acc):
    """Tuned kernel on particles at identical positions: finite and within tolerance
    of the oracle for eps > 0; NaN exactly for the coincident particles for eps = 0,
    as the reference's 0 * rsqrt(0) gives."""
    n = 600
    pos, vel, m = disk_case(n, seed=21)
    for a in pos:
        a[300:310] = a[0]
        a[500] = a[499]
    with nb.Simulation(params(n, acc=acc), pos, vel, None) as sim:
        got = sim.accelerations()
    assert all(np.all(np.isfinite(g)) for g in got)
    rms, mx = vec_errors(got, orc.accel_fp64(pos, None, 1.0, EPS32))
    assert rms <= ACC_RMS and mx <= ACC_MAX
    with nb.Simulation(params(n, eps=0.0, acc=acc), pos, vel, None) as sim:
        got = sim.accelerations()
    bad = np.isnan(got[0])
    expect = np.zeros(n, bool)
    expect[[0, *range(300, 310), 499, 500]] = True
    assert np.array_equal(bad, expect)
