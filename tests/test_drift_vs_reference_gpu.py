"""Energy and momentum drift against the reference's own kernel: the same
thin disk (N = 25,600, m = 1/N, G = 1, eps2 = 1e-3, dt = 1e-3, damping 1
so both are conserved) advanced 300 iterations by the reference kernel
(src/simulator.cu:186-229, built unmodified for sm_103a) and by this library; the
FP64 diagnostics of each final state.  The library's drift must be no worse."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import disk_case, g_eff, params

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not orc.reference_available(),
                                 reason="reference cubin not built (oracle/build_ref.sh)")]

N, STEPS = 25600, 300


def drifts(sim_for_diag, state, m, e0, p0, scale):
    sim_for_diag.set_state(state[:3], state[3:], m)
    d = sim_for_diag.diagnostics()
    return (abs(d["total"] - e0) / abs(e0),
            float(np.linalg.norm(np.array(d["momentum"]) - p0)) / scale)


def test_energy_and_momentum_drift_no_worse_than_reference():
    pos, vel, m = disk_case(N, seed=2027)
    p = params(N, damping=1.0)
    with nb.Simulation(p, pos, vel, m) as diag:
        d0 = diag.diagnostics()
        e0, p0 = d0["total"], np.array(d0["momentum"])
        scale = float(np.sum(m.astype(np.float64) * np.sqrt(sum(v.astype(np.float64) ** 2
                                                                 for v in vel))))
        ref, _ = orc.reference_run(pos, vel, g_eff(1.0, m[0]), 1e-3, 1.0, 1e-3, STEPS)
        de_ref, dp_ref = drifts(diag, ref, m, e0, p0, scale)
        results = {}
        for name, acc in (("plain", nb.ACC_PLAIN), ("compensated", nb.ACC_COMPENSATED),
                          ("reference order", nb.ACC_REFERENCE_ORDER)):
            with nb.Simulation(params(N, damping=1.0, acc=acc), pos, vel, m) as sim:
                sim.advance(STEPS)
                st = sim.get_state()
            if acc == nb.ACC_REFERENCE_ORDER:   # the reference's own trajectory, bit for bit
                assert all(np.array_equal(a.view(np.uint32), b.view(np.uint32))
                           for a, b in zip(st, ref))
            results[name] = drifts(diag, st, m, e0, p0, scale)
    print(f"reference kernel: energy drift {de_ref:.3e}, momentum drift {dp_ref:.3e}")
    for name, (de, dp) in results.items():
        print(f"library {name}: energy drift {de:.3e}, momentum drift {dp:.3e}")
        # energy drift is integration error: the same within a few percent
        assert de <= 1.05 * de_ref + 1e-9, (name, de, de_ref)
        # momentum drift comes from rounding: no worse than the reference
        assert dp <= 1.5 * dp_ref + 1e-9, (name, dp, dp_ref)
