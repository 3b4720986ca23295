"""One system split over ranks (nbody_gb300.shard) on CPU: world size 2 over gloo
(127.0.0.1).  Each rank drives a host stand-in of the simulation whose step is the
CPU oracle's (the reference kernel restated, oracle/nbody_oracle.c) restricted to
the rank's shard, with the library's state-block rules; the real partition and
all-gather code of ShardedSimulation moves the blocks.  After several steps every
rank's copy must equal the unsharded oracle run bit for bit: the partition covers
every particle once and the exchange assembles the blocks in the right places."""
from __future__ import annotations

import ctypes
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent
N, STEPS, G, DT, DAMP, EPS = 1000, 3, 2.0, 1e-3, 0.999, 1e-3


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class HostShardSim:
    """The state-block interface of nbody_gb300.Simulation on host arrays: 16 bytes
    per particle (x, y, z, m) / (vx, vy, vz, 0), padded to 16 particles; a step
    writes only the shard's particles, like nb_sim_set_shard."""

    def __init__(self, pos, vel):
        self.n = pos[0].size
        self.npad = -(-self.n // 16) * 16
        self.pos = np.zeros((self.npad, 4), np.float32)
        self.vel = np.zeros((self.npad, 4), np.float32)
        self.pos[: self.n, :3] = np.stack(pos, 1)
        self.vel[: self.n, :3] = np.stack(vel, 1)
        self.first, self.count = 0, self.n

    def set_shard(self, first, count):
        assert first % 16 == 0 and 0 < count <= self.n - first
        assert first + count == self.n or count % 16 == 0
        self.first, self.count = first, count

    def advance(self, iterations):
        import oracle_binding as orc

        for _ in range(iterations):
            n = self.n
            out = orc.run_fp32([self.pos[:n, c] for c in range(3)],
                               [self.vel[:n, c] for c in range(3)], None, G, DT, DAMP, EPS,
                               iters=1)
            sl = slice(self.first, self.first + self.count)
            for c in range(3):
                self.pos[sl, c] = out[c][sl]
                self.vel[sl, c] = out[3 + c][sl]

    def _range(self, first, count):
        end = self.npad if first + count == self.n else first + count
        assert first % 16 == 0 and end % 16 == 0
        return first, end

    def state_block_bytes(self, first, count, what=1):
        f, e = self._range(first, count)
        return 16 * (e - f)

    def _array(self, what):
        return self.pos if what == 1 else self.vel

    def copy_state_block(self, first, count, what, dst_ptr):
        f, e = self._range(first, count)
        a = self._array(what)
        ctypes.memmove(dst_ptr, a[f:e].ctypes.data, 16 * (e - f))

    def load_state_block(self, first, count, what, src_ptr):
        f, e = self._range(first, count)
        a = self._array(what)
        ctypes.memmove(a[f:e].ctypes.data, src_ptr, 16 * (e - f))


def _inputs():
    rng = np.random.default_rng(5)
    pos = [rng.normal(size=N).astype(np.float32) for _ in range(3)]
    vel = [(0.1 * rng.normal(size=N)).astype(np.float32) for _ in range(3)]
    return pos, vel


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    for p in (ROOT / "cuda-to-sycl-nbody_gb300", ROOT / "tests"):
        sys.path.insert(0, str(p))
    from nbody_gb300.shard import ShardedSimulation

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pos, vel = _inputs()
        sim = HostShardSim(pos, vel)
        sharded = ShardedSimulation(sim, rank, world, device="cpu")
        sharded.step(STEPS)
        sharded.gather_velocities()
        q.put((rank, sharded.shard, sim.pos[:N, :3].copy(), sim.vel[:N, :3].copy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_match_the_unsharded_run_bit_for_bit():
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding as orc

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=180) for _ in procs), key=lambda o: o[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [(0, 512), (512, N - 512)]
    pos, vel = _inputs()
    ref = orc.run_fp32(pos, vel, None, G, DT, DAMP, EPS, iters=STEPS)
    for _, _, p_, v_ in out:
        for c in range(3):
            assert np.array_equal(p_[:, c], ref[c])
            assert np.array_equal(v_[:, c], ref[3 + c])


def test_shard_bounds():
    sys.path.insert(0, str(ROOT / "cuda-to-sycl-nbody_gb300"))
    from nbody_gb300.shard import shard_bounds

    assert shard_bounds(1 << 20, 8) == [(k << 17, 1 << 17) for k in range(8)]
    assert shard_bounds(1000, 2) == [(0, 512), (512, 488)]
    assert shard_bounds(17, 1) == [(0, 17)]
    b = shard_bounds(25600, 3)
    assert sum(c for _, c in b) == 25600 and all(f % 16 == 0 for f, _ in b)
    with pytest.raises(ValueError):
        shard_bounds(20, 3)
