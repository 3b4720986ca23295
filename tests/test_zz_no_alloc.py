"""nb_accelerations_noalloc: accelerations for callers that cannot allocate GPU
memory -- an engine or plugin host that hands out every device buffer from its own
pools, or a frame loop that must not stall on cudaMalloc.  They bring their own
input and output buffers; the library's scratch is a fixed device array, which
caps the size at 262,144 particles.

Collected last on purpose (a failure here leaves every other test already run).
Checks, through the C ABI:
  * two calls in a row agree with the allocating entry point (nb_sim_accelerations)
    within the parity tolerance of the other tests;
  * the output agrees with the CPU oracle (FP32 restatement of the reference's
    force sum, and FP64) at the maximum size, on strided rows;
  * zero softening (the self pair is then excluded by index), n = 1, a ragged size;
  * sizes beyond the fixed scratch are refused."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
import oracle_binding as orc
from helpers import disk_case, g_eff, params, vec_errors

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ACC_RMS = 1e-5
ACC_MAX = 1e-4
MAX_N = 262144


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


def test_maximum_size_matches_oracle_on_strided_rows():
    # The largest plan the fixed tables hold: 512 i-tiles on the full persistent grid.
    (x, y, z), _, m = nb.plummer(2026, MAX_N)
    pos = [x, y, z]
    eps = float(np.float32(1e-4))
    for _ in range(2):                                            # the array keeps old contents
        got, w = noalloc_accelerations(pos, m, 1.0, eps)
        rows = np.linspace(0, MAX_N - 1, 384).astype(np.int64)
        g = [a[rows] for a in got]
        ref32 = orc.accel_fp32(pos, None, g_eff(1.0, m[0]), eps, rows=rows)
        ref64 = orc.accel_fp64(pos, m, 1.0, eps, rows=rows)
        for ref in (ref32, ref64):
            rms, mx = vec_errors(g, ref)
            assert rms <= ACC_RMS and mx <= ACC_MAX, (rms, mx)
        assert np.all(w == 0.0)


def test_zero_softening_single_particle_and_ragged_size_match_oracle():
    # eps = 0: the self pair would be 0 * rsqrt(0); it is left out by index, as the
    # reference's `if (i == id) continue;` does.
    pos, _, m = disk_case(700, seed=93)
    got, _ = noalloc_accelerations(pos, m, 1.0, 0.0)
    assert all(np.all(np.isfinite(a)) for a in got)
    rms, mx = vec_errors(got, orc.accel_fp32(pos, None, g_eff(1.0, m[0]), 0.0))
    assert rms <= ACC_RMS and mx <= ACC_MAX, (rms, mx)
    pos, _, m = disk_case(1, seed=94)                             # no other particle: zero
    got, _ = noalloc_accelerations(pos, m, 1.0, 1e-3)
    assert all(float(a[0]) == 0.0 for a in got)
    pos, _, _ = disk_case(4099, seed=95)                          # per-particle masses, ragged
    m = (np.random.default_rng(95).uniform(0.5, 1.5, 4099) / 4099).astype(np.float32)
    eps = float(np.float32(1e-3))
    got, _ = noalloc_accelerations(pos, m, 1.0, eps)
    rms, mx = vec_errors(got, orc.accel_fp64(pos, m, 1.0, eps))
    assert rms <= ACC_RMS and mx <= ACC_MAX, (rms, mx)


def test_sizes_beyond_the_fixed_scratch_are_refused():
    big = MAX_N + 1
    xyzm = torch.zeros((big, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros((big, 4), dtype=torch.float32, device="cuda")
    rc = nb.lib.nb_accelerations_noalloc(xyzm.data_ptr(), big, 1.0, 1e-3, out.data_ptr(), None)
    assert rc == nb.NB_ERR_INVALID_ARGUMENT
    assert "262144" in nb.lib.nb_last_error().decode()
