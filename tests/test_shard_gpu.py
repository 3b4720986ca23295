"""One system split into shards (nb_sim_set_shard + state blocks), on one GPU.

Two simulations of the same system each integrate one shard, and between steps
swap their shards' position blocks through device buffers -- what the ranks of a
multi-GPU run do with an all-gather.  After several steps both copies must hold
the unsharded run's state: bit for bit with the reference-order accumulator (the
same sequence of roundings per particle whatever the work list), within the
parity tolerance with the tuned kernel (its split points differ)."""
from __future__ import annotations

import numpy as np
import pytest

import nbody_gb300 as nb
from helpers import disk_case, displacement_errors, params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N, STEPS = 20000, 4


def _run_two_shards(acc, pos, vel, m, steps):
    bounds = [(0, 10240), (10240, N - 10240)]
    stream = torch.cuda.current_stream()
    sims = [nb.Simulation(params(N, acc=acc), pos, vel, m) for _ in bounds]
    bufs = []
    for sim, (f, c) in zip(sims, bounds):
        sim.set_stream(stream.cuda_stream)
        sim.set_shard(f, c)
        bufs.append(torch.empty(sim.state_block_bytes(f, c), dtype=torch.uint8, device="cuda"))
    for _ in range(steps):
        for sim in sims:
            sim.advance(1)
        for k, (f, c) in enumerate(bounds):          # each shard's block to the other copy
            sims[k].copy_state_block(f, c, nb.BLOCK_POSITIONS, bufs[k].data_ptr())
            sims[1 - k].load_state_block(f, c, nb.BLOCK_POSITIONS, bufs[k].data_ptr())
    for k, (f, c) in enumerate(bounds):              # and the velocities once at the end
        sims[k].copy_state_block(f, c, nb.BLOCK_VELOCITIES, bufs[k].data_ptr())
        sims[1 - k].load_state_block(f, c, nb.BLOCK_VELOCITIES, bufs[k].data_ptr())
    states = [sim.get_state() for sim in sims]
    for sim in sims:
        sim.close()
    return states


@pytest.mark.parametrize("acc", [nb.ACC_REFERENCE_ORDER, nb.ACC_COMPENSATED])
def test_two_shards_reproduce_the_whole_system(acc):
    pos, vel, m = disk_case(N, seed=77)
    with nb.Simulation(params(N, acc=acc), pos, vel, m) as whole:
        whole.advance(STEPS)
        ref = whole.get_state()
    for st in _run_two_shards(acc, pos, vel, m, STEPS):
        if acc == nb.ACC_REFERENCE_ORDER:
            for g, r in zip(st, ref):
                assert np.array_equal(g, r)
        else:
            rms, mx = displacement_errors(st[:3], ref[:3], pos)
            assert rms <= 1e-4 and mx <= 1e-3, (rms, mx)


def test_sharded_simulation_over_a_one_rank_nccl_group():
    import os

    import torch.distributed as dist

    from nbody_gb300.shard import ShardedSimulation

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    os.environ.setdefault("MASTER_PORT", "29531")
    dist.init_process_group("nccl", rank=0, world_size=1)
    try:
        pos, vel, m = disk_case(4096, seed=78)
        p = params(4096, acc=nb.ACC_REFERENCE_ORDER)
        with nb.Simulation(p, pos, vel, m) as whole:
            whole.advance(3)
            ref = whole.get_state()
        with nb.Simulation(p, pos, vel, m) as sim:
            sharded = ShardedSimulation(sim, 0, 1, device="cuda")
            assert sharded.shard == (0, 4096)
            sharded.step(3)
            got = sim.get_state()
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)
    finally:
        dist.destroy_process_group()


def test_shard_arguments_and_what_they_invalidate():
    pos, vel, m = disk_case(1000, seed=79)
    with nb.Simulation(params(1000), pos, vel, m) as sim:
        for first, count in ((3, 100), (0, 1001), (992, 16), (16, 20)):
            with pytest.raises(nb.NbError) as e:
                sim.set_shard(first, count)
            assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
        sim.set_shard(992, 8)                         # the last shard may be ragged
        assert sim.state_block_bytes(992, 8) == 16 * 16
        with pytest.raises(nb.NbError):
            sim.copy_state_block(0, 16, 3, 1)         # unknown block kind
        side = torch.cuda.Stream()                    # graphs are captured on a non-default stream
        sim.set_stream(side.cuda_stream)
        sim.graph_capture(2)
        sim.set_shard(0, 512)                         # new work list: the graph is dropped
        with pytest.raises(nb.NbError) as e:
            sim.graph_launch()
        assert e.value.status == nb.NB_ERR_STATE
        with pytest.raises(nb.NbError) as e:
            sim.adjoint_forward(4, 2)                 # the adjoint needs the whole system
        assert e.value.status == nb.NB_ERR_STATE
        sim.set_shard(0, 0)                           # whole system again
        sim.adjoint_forward(4, 2)
    sizes = [100, 200]
    parts = [disk_case(s, seed=80 + k) for k, s in enumerate(sizes)]
    pos = [np.concatenate([q[0][c] for q in parts]) for c in range(3)]
    vel = [np.concatenate([q[1][c] for q in parts]) for c in range(3)]
    with nb.Simulation(params(300), pos, vel, None, sizes=sizes) as ens:
        with pytest.raises(nb.NbError):
            ens.set_shard(0, 96)                      # ensembles are not sharded
