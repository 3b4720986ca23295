"""Device hand-off and stream use: nb_sim_export_device (the renderer's per-frame
copy, src/renderer_gl.cpp:111-114 / 156-172, made device-to-device) and running a
simulation on the caller's CUDA stream."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
from helpers import disk_case, params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_export_matches_host_state():
    sizes = [100, 33, 1000]
    parts = [disk_case(s, seed=300 + k) for k, s in enumerate(sizes)]
    pos = [np.concatenate([p[0][c] for p in parts]) for c in range(3)]
    vel = [np.concatenate([p[1][c] for p in parts]) for c in range(3)]
    m = np.concatenate([p[2] for p in parts])
    n = sum(sizes)
    with nb.Simulation(params(n), pos, vel, m, sizes=sizes) as sim:
        sim.advance(3)
        x, y, z, vx, vy, vz = sim.get_state()
        P = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        V = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        sim.export_device(P.data_ptr(), V.data_ptr())
        sim.synchronize()
        pos_only = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        sim.export_device(pos_only.data_ptr())
        sim.synchronize()
    P, V, Q = P.cpu().numpy(), V.cpu().numpy(), pos_only.cpu().numpy()
    assert np.array_equal(P[:, 0], x) and np.array_equal(P[:, 1], y) and np.array_equal(P[:, 2], z)
    assert np.array_equal(P[:, 3], m)
    assert np.array_equal(V[:, 0], vx) and np.array_equal(V[:, 1], vy) and np.array_equal(V[:, 2], vz)
    assert np.array_equal(Q, P)


def test_runs_on_callers_stream():
    n = 5000
    pos, vel, m = disk_case(n, seed=310)
    with nb.Simulation(params(n), pos, vel, m) as a:
        a.advance(5)
        ref = a.get_state()
    s = torch.cuda.Stream()
    with nb.Simulation(params(n), pos, vel, m) as b:
        b.set_stream(s.cuda_stream)
        with torch.cuda.stream(s):
            b.advance(5)
            ev = torch.cuda.Event()
            ev.record(s)
        ev.synchronize()
        got = b.get_state()
    for u, v in zip(ref, got):
        assert np.array_equal(u, v)


def test_export_rejects_misaligned_buffer():
    n = 64
    pos, vel, m = disk_case(n, seed=311)
    buf = torch.empty(4 * n + 1, dtype=torch.float32, device="cuda")
    with nb.Simulation(params(n), pos, vel, m) as sim:
        with pytest.raises(nb.NbError) as e:
            sim.export_device(buf.data_ptr() + 4)
        assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
