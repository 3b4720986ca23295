"""Parity at the workloads' own sizes: the 1,048,576-particle Plummer sphere (eps2 =
1e-4) and the 262,144-particle two-disk collision (eps2 = 1e-3), both from the
library's seeded generators.

At these sizes the reference kernel's own FP32 running sum (src/simulator.cu:196-207)
is itself about 2e-5 (sphere) and 2e-4 (collision) relative RMS away from the FP64
all-pairs sum, so no FP32 result can lie within 1e-5 of both.  The tests pin the
resolution:
  * the library's default accumulator (compensated) is within 1e-5 relative RMS
    and 1e-4 per-particle max of FP64;
  * its distance from the reference kernel equals the reference kernel's own
    distance from FP64 to within 1e-5 (what separates them is the reference's
    rounding, not the library's);
  * the reference-order accumulator reproduces the reference kernel bit for bit,
    accelerations and two full iterations;
  * the plain FP32 accumulator meets 1e-5 on the sphere and stays well inside the
    reference's own error on the collision (where it misses 1e-5).
FP64 rows come from the GPU (nb_sim_fp64_accelerations), checked here against the
CPU FP64 oracle on a subset."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import g_eff, params, vec_errors

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

SEED = 20261203
ACC_RMS = 1e-5
ACC_MAX = 1e-4
ROWS = 1024

needs_ref = pytest.mark.skipif(not orc.reference_available(),
                               reason="reference cubin not built (oracle/build_ref.sh)")


def _case(name):
    if name == "plummer_1m":
        (x, y, z), (vx, vy, vz), m = nb.plummer(SEED, 1 << 20)
        return [x, y, z], [vx, vy, vz], m, float(np.float32(1e-4))
    (x, y, z), (vx, vy, vz), m = nb.two_disks(SEED, 262144, 1e-3)
    return [x, y, z], [vx, vy, vz], m, float(np.float32(1e-3))


@pytest.fixture(scope="module", params=["plummer_1m", "two_disks_262k"])
def case(request):
    pos, vel, m, eps = _case(request.param)
    n = pos[0].size
    rows = np.linspace(0, n - 1, ROWS).astype(np.int64)
    with nb.Simulation(params(n, eps=eps, acc=nb.ACC_COMPENSATED), pos, vel, m) as sim:
        f64 = sim.fp64_accelerations(rows.astype(np.uint64))
    # the GPU FP64 rows against the CPU FP64 oracle on every 16th row
    sub = rows[::16]
    cpu = orc.accel_fp64(pos, m, 1.0, eps, rows=sub)
    for a, b in zip(f64, cpu):
        assert np.allclose(a[::16], b, rtol=1e-10, atol=1e-12)
    return request.param, pos, vel, m, eps, rows, f64


def _accelerations(pos, vel, m, eps, acc):
    n = pos[0].size
    with nb.Simulation(params(n, eps=eps, acc=acc), pos, vel, m) as sim:
        return sim.accelerations()


def _rows(a, rows):
    return [c[rows] for c in a]


@pytest.fixture(scope="module")
def reference_sum(case):
    """The reference kernel's acceleration: one launch with dt = 1 and damping = 0,
    whose velocity output is (F * 1) * G_eff (simulator.cu:214-216)."""
    if not orc.reference_available():
        pytest.skip("reference cubin not built (oracle/build_ref.sh)")
    name, pos, vel, m, eps, rows, f64 = case
    zeros = [np.zeros(pos[0].size, np.float32)] * 3
    out, _ = orc.reference_run(pos, zeros, g_eff(1.0, m[0]), 1.0, 0.0, eps, iters=1,
                               gw_size=128)
    return out[3:]


def test_compensated_meets_the_fp64_target(case):
    name, pos, vel, m, eps, rows, f64 = case
    got = _accelerations(pos, vel, m, eps, nb.ACC_COMPENSATED)
    rms, mx = vec_errors(_rows(got, rows), f64)
    print(f"{name}: compensated vs FP64 rel RMS {rms:.3g}, max {mx:.3g}")
    assert rms <= ACC_RMS and mx <= ACC_MAX, (name, rms, mx)


def test_plain_accumulator_error_is_bounded(case):
    name, pos, vel, m, eps, rows, f64 = case
    got = _accelerations(pos, vel, m, eps, nb.ACC_PLAIN)
    rms, mx = vec_errors(_rows(got, rows), f64)
    print(f"{name}: plain vs FP64 rel RMS {rms:.3g}, max {mx:.3g}")
    if name == "plummer_1m":
        assert rms <= ACC_RMS and mx <= ACC_MAX, (name, rms, mx)
    else:
        # The collision's close encounters: the plain FP32 sum misses 1e-5 (about
        # 2e-5), a tenth of the reference's own sequential sum (about 2.3e-4).
        assert rms <= 5e-5, (name, rms, mx)


@needs_ref
def test_distance_from_reference_kernel_is_the_reference_rounding(case, reference_sum):
    name, pos, vel, m, eps, rows, f64 = case
    ref_rms, _ = vec_errors(_rows(reference_sum, rows), f64)
    assert ref_rms > ACC_RMS / 4          # the reference itself is far from FP64 here
    for acc in (nb.ACC_COMPENSATED, nb.ACC_PLAIN):
        got = _accelerations(pos, vel, m, eps, acc)
        ours_rms, _ = vec_errors(_rows(got, rows), f64)
        d_rms, _ = vec_errors(_rows(got, rows), _rows(reference_sum, rows))
        assert abs(d_rms - ref_rms) <= ours_rms + ACC_RMS, (name, acc, d_rms, ref_rms, ours_rms)
        # and over every particle, not only the sampled rows
        d_all, _ = vec_errors(got, reference_sum)
        print(f"{name}: reference kernel vs FP64 {ref_rms:.3g}; accumulator {acc} vs FP64 "
              f"{ours_rms:.3g}, vs the reference kernel {d_rms:.3g} (rows), {d_all:.3g} (all)")
        assert d_all <= 2 * ref_rms + ACC_RMS, (name, acc, d_all, ref_rms)


@needs_ref
def test_reference_order_is_the_reference_kernel_bit_for_bit(case, reference_sum):
    name, pos, vel, m, eps, rows, f64 = case
    got = _accelerations(pos, vel, m, eps, nb.ACC_REFERENCE_ORDER)
    for g, r in zip(got, reference_sum):
        assert np.array_equal(g, r), name
    # two iterations of the workload's own step (dt = 1e-4 or 1e-3, damping 1)
    dt = 1e-4 if name == "plummer_1m" else 1e-3
    G = g_eff(1.0, m[0])
    ref, _ = orc.reference_run(pos, vel, G, dt, 1.0, eps, iters=2, gw_size=128)
    n = pos[0].size
    with nb.Simulation(params(n, dt=dt, damping=1.0, eps=eps, acc=nb.ACC_REFERENCE_ORDER),
                       pos, vel, m) as sim:
        sim.advance(2)
        st = sim.get_state()
    for g, r in zip(st, ref):
        assert np.array_equal(g, r), name


def test_ensemble_workload_against_fp64_rows():
    # The 4,096-system ensemble (sizes log-uniform in [64, 8192], about 6.6M particles,
    # eps2 = 1e-3): FP32 accelerations of one persistent launch against FP64 rows
    # spread over every system, for the default accumulator and the plain one.
    sizes = nb.ensemble_sizes(SEED, 4096, 64, 8192)
    parts = [nb.plummer(SEED + 1 + k, int(s)) for k, s in enumerate(sizes)]
    pos = [np.concatenate([q[0][c] for q in parts]) for c in range(3)]
    vel = [np.concatenate([q[1][c] for q in parts]) for c in range(3)]
    m = np.concatenate([q[2] for q in parts])
    n = pos[0].size
    rows = np.linspace(0, n - 1, 2048).astype(np.int64)
    eps = float(np.float32(1e-3))
    for acc, bound in ((nb.ACC_COMPENSATED, ACC_RMS), (nb.ACC_PLAIN, ACC_RMS)):
        with nb.Simulation(params(n, eps=eps, acc=acc), pos, vel, m, sizes=sizes) as sim:
            got = sim.accelerations()
            f64 = sim.fp64_accelerations(rows.astype(np.uint64))
        rms, mx = vec_errors(_rows(got, rows), f64)
        print(f"ensemble_4096_systems: accumulator {acc} vs FP64 rel RMS {rms:.3g}, max {mx:.3g}")
        assert rms <= bound and mx <= ACC_MAX, (acc, rms, mx)
