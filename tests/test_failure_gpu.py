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
