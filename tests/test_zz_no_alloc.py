"""nb_accelerations_noalloc: accelerations for callers that cannot allocate GPU
memory (they bring their own input and output buffers; the library's scratch is
a fixed device array).  Collected last on purpose.  Checks, through the C ABI,
that two calls in a row agree with the allocating entry point
(nb_sim_accelerations) within the parity tolerance of the other tests, and that
sizes beyond the fixed scratch are refused."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
from helpers import disk_case, params, vec_errors

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ACC_RMS = 1e-5
ACC_MAX = 1e-4


def reference_accelerations(pos, vel, m, G, eps):
    p = params(pos[0].size, G=G, eps=eps)
    with nb.Simulation(p, pos, vel, m) as sim:
        return sim.accelerations()


def noalloc_accelerations(pos, m, G, eps):
    n = pos[0].size
    xyzm = torch.from_numpy(np.stack([pos[0], pos[1], pos[2], m], 1).astype(np.float32)).cuda()
    out = torch.full((n, 4), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = nb.lib.nb_accelerations_noalloc(xyzm.data_ptr(), n, G, eps, out.data_ptr(),
                                         stream.cuda_stream or None)
    assert rc == nb.NB_OK, nb.lib.nb_last_error().decode()
    a = out.cpu().numpy()
    return [a[:, 0], a[:, 1], a[:, 2]], a[:, 3]


def test_two_calls_in_a_row_match_allocating_entry_point():
    cases = []
    pos, vel, m = disk_case(20000, seed=91)                       # equal masses
    cases.append((pos, vel, m, 1.0, float(np.float32(1e-3))))
    pos, vel, _ = disk_case(5003, seed=92)                        # ragged size, unequal masses
    m = (np.random.default_rng(92).uniform(0.5, 1.5, 5003) / 5003).astype(np.float32)
    cases.append((pos, vel, m, 2.0, float(np.float32(1e-4))))
    for pos, vel, m, G, eps in cases:                             # two calls, one after the other
        got, w = noalloc_accelerations(pos, m, G, eps)
        ref = reference_accelerations(pos, vel, m, G, eps)
        rms, mx = vec_errors(got, ref)
        assert rms <= ACC_RMS and mx <= ACC_MAX, (rms, mx)
        assert np.all(w == 0.0)


def test_sizes_beyond_the_fixed_scratch_are_refused():
    big = 262144 + 1
    xyzm = torch.zeros((big, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros((big, 4), dtype=torch.float32, device="cuda")
    rc = nb.lib.nb_accelerations_noalloc(xyzm.data_ptr(), big, 1.0, 1e-3, out.data_ptr(), None)
    assert rc == nb.NB_ERR_INVALID_ARGUMENT
    assert "262144" in nb.lib.nb_last_error().decode()
