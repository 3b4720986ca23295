"""One system split over the ranks of a torch.distributed group.

The reference runs its one system on device 0 (src/simulator.cu:40).  Here a
system of n particles splits into equal shards, one per rank: every rank keeps a
whole copy of the system (nb_sim), integrates only its own particles, each against
all n (nb_sim_set_shard), and after every step the ranks all-gather the position
blocks of their shards (nb_sim_copy_state_block / nb_sim_load_state_block), so that
each starts the next step with every particle's new position.  Per step and rank
that is n^2 / world pair interactions and one all-gather of 16 bytes per particle.

The collective runs on the group's backend: NCCL for CUDA tensors, gloo for the
host tensors of the CPU tests.  On a GPU the simulation is moved onto torch's
current stream, so the step, the block copies and the all-gather are ordered on one
stream without host synchronisation.  No kernel waits on another rank.
"""
from __future__ import annotations

PAD = 16  # particles; shard boundaries are multiples of it


def shard_bounds(n: int, world: int) -> list[tuple[int, int]]:
    """(first, count) of each rank's shard: equal shards whose boundaries are
    multiples of 16 particles, the last one taking the rest."""
    if world < 1:
        raise ValueError("world must be >= 1")
    per = -(-(-(-n // world)) // PAD) * PAD          # ceil(ceil(n / world) / 16) * 16
    out = []
    for r in range(world):
        first = r * per
        count = min(per, n - first)
        if count <= 0:
            raise ValueError(f"{n} particles cannot be split into {world} shards of "
                             f"multiples of {PAD}")
        out.append((first, count))
    return out


class ShardedSimulation:
    """Rank `rank`'s shard of a system split over `world` ranks.

    `sim` is this rank's whole copy of the system: a Simulation of one system (or
    an object with its n, set_shard, advance, state_block_bytes, copy_state_block
    and load_state_block).  `device` is where the exchange buffers live: a CUDA
    device for the library (NCCL), "cpu" for host-side stand-ins (gloo).  Every
    rank constructs it with the same system and world size."""

    def __init__(self, sim, rank: int, world: int, device="cuda", group=None):
        import torch

        self.sim = sim
        self.rank = rank
        self.world = world
        self.group = group
        self.device = torch.device(device)
        self.bounds = shard_bounds(sim.n, world)
        first, count = self.bounds[rank]
        sim.set_shard(first, count)
        if self.device.type == "cuda":
            sim.set_stream(torch.cuda.current_stream(self.device).cuda_stream)
        # all_gather_into_tensor wants equal pieces: every rank sends a buffer as
        # large as the largest block, and each loads only the bytes of its peers'.
        self.block_bytes = max(sim.state_block_bytes(f, c) for f, c in self.bounds)
        self._mine = torch.empty(self.block_bytes, dtype=torch.uint8, device=self.device)
        self._all = torch.empty(self.block_bytes * world, dtype=torch.uint8, device=self.device)

    @property
    def shard(self) -> tuple[int, int]:
        return self.bounds[self.rank]

    def exchange(self, what: int | None = None) -> None:
        """All-gather the shards' position (or velocity) blocks into every rank's copy."""
        import torch.distributed as dist

        from . import BLOCK_POSITIONS

        what = BLOCK_POSITIONS if what is None else what
        first, count = self.shard
        self.sim.copy_state_block(first, count, what, self._mine.data_ptr())
        dist.all_gather_into_tensor(self._all, self._mine, group=self.group)
        base = self._all.data_ptr()
        for r, (f, c) in enumerate(self.bounds):
            if r != self.rank:
                self.sim.load_state_block(f, c, what, base + r * self.block_bytes)

    def step(self, iterations: int = 1) -> None:
        """`iterations` steps: advance this shard, then exchange positions."""
        for _ in range(iterations):
            self.sim.advance(1)
            self.exchange()

    def gather_velocities(self) -> None:
        """Bring every rank's copy of the velocities up to date (the steps keep only
        each rank's own shard current)."""
        from . import BLOCK_VELOCITIES

        self.exchange(BLOCK_VELOCITIES)
