"""Failure detection without a GPU fault: every device-side wait of the force
kernel is bounded; when one runs out (here: a tile that is never copied, via
the one-shot test hook) the launch reports NB_ERR_DEVICE_TIMEOUT to the host and
the simulation and the CUDA context stay usable."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import disk_case, g_eff, params

pytestmark = pytest.mark.gpu


def test_bounded_wait_timeout_is_reported_and_recoverable():
    n = 20000  # several CTAs with split i-tiles
    pos, vel, m = disk_case(n, seed=77)
    with nb.Simulation(params(n), pos, vel, m) as sim:
        sim.inject_wait_timeout()
        sim.advance(1)
        with pytest.raises(nb.NbError) as e:
            sim.synchronize()
        assert e.value.status == nb.NB_ERR_DEVICE_TIMEOUT
        # the context and the simulation remain usable
        sim.set_state(pos, vel)
        sim.advance(2)
        got = sim.get_state()
    ref = orc.run_fp32(pos, vel, None, g_eff(1.0, m[0]), 1e-3, 0.999, 1e-3, iters=2)
    scale = max(float(np.max(np.abs(r))) for r in ref[:3])
    assert max(float(np.max(np.abs(g - r))) for g, r in zip(got[:3], ref[:3])) <= 1e-4 * scale


def test_withheld_hand_over_times_out_and_is_recoverable():
    # NB_ACC_REFERENCE_ORDER at N = 300,000: 196 i-tiles of 1536 on 152 CTAs, so split
    # i-tiles are handed over between CTAs.  With the hand-overs withheld, each CTA
    # that continues one gives up after its bounded wait (no fault, no hang).
    n = 300000
    pos, vel, m = disk_case(n, seed=79)
    p = params(n, acc=nb.ACC_REFERENCE_ORDER)
    with nb.Simulation(p, pos, vel, m) as ref:
        ref.advance(2)
        want = ref.get_state()
    with nb.Simulation(p, pos, vel, m) as sim:
        assert sim.kernel_info()["split_tiles"] > 0
        sim.inject_failure(nb.INJECT_HAND_OVER_WITHHELD)
        sim.advance(1)
        with pytest.raises(nb.NbError) as e:
            sim.synchronize()
        assert e.value.status == nb.NB_ERR_DEVICE_TIMEOUT
        sim.set_state(pos, vel)                      # usable again, same bits as before
        sim.advance(2)
        got = sim.get_state()
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_failure_hook_arguments():
    pos, vel, m = disk_case(256, seed=80)
    with nb.Simulation(params(256), pos, vel, m) as sim:
        for kind, status in ((3, nb.NB_ERR_INVALID_ARGUMENT),
                             (nb.INJECT_HAND_OVER_WITHHELD, nb.NB_ERR_STATE)):
            with pytest.raises(nb.NbError) as e:
                sim.inject_failure(kind)
            assert e.value.status == status


def test_errors_do_not_cross_the_abi_as_exceptions():
    n = 64
    pos, vel, m = disk_case(n, seed=78)
    with nb.Simulation(params(n), pos, vel, m) as sim:
        with pytest.raises(nb.NbError) as e:
            sim.graph_launch()                       # nothing captured
        assert e.value.status == nb.NB_ERR_STATE
        with pytest.raises(nb.NbError) as e:
            sim.fp64_accelerations([n + 5])          # row out of range
        assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
        with pytest.raises(nb.NbError) as e:
            sim.adjoint_backward(np.zeros(3 * n, np.float32))
        assert e.value.status == nb.NB_ERR_STATE
        sim.advance(1)
        sim.synchronize()


def test_every_allocation_failure_is_reported_and_cleaned_up():
    """Fail the k-th device allocation of a simulation's creation and first use
    (state, work list, reference-order tiles, accelerations, diagnostics, render
    buffers) for every k: each failure surfaces as NB_ERR_OUT_OF_MEMORY, nothing
    leaks into the next attempt, and once k passes the last allocation everything
    works and matches the oracle."""
    n = 3000
    pos, vel, m = disk_case(n, seed=79)

    import torch

    img = torch.empty((64, 64, 4), dtype=torch.float32, device="cuda")
    view, proj = nb.camera_matrices(0.0, 0.5, 8.0, 64, 64)

    def use(acc):
        with nb.Simulation(params(n, acc=acc), pos, vel, m) as sim:
            sim.advance(1)
            sim.accelerations()
            sim.diagnostics()
            sim.render(view, proj, 64, 64, img.data_ptr())
            return sim.get_state()

    for acc in (nb.ACC_PLAIN, nb.ACC_REFERENCE_ORDER):
        failures = 0
        for k in range(1, 200):
            nb.inject_alloc_failure(k)
            try:
                got = use(acc)
            except nb.NbError as e:
                assert e.status == nb.NB_ERR_OUT_OF_MEMORY, (k, e)
                failures += 1
                continue
            finally:
                nb.inject_alloc_failure(0)
            break
        assert failures >= 5, failures           # creation alone makes several allocations
        ref = orc.run_fp32(pos, vel, None, g_eff(1.0, m[0]), 1e-3, 0.999, 1e-3, iters=1)
        scale = max(float(np.max(np.abs(r))) for r in ref[:3])
        assert max(float(np.max(np.abs(g - r))) for g, r in zip(got[:3], ref[:3])) <= 1e-4 * scale
