"""Bunch sharding across ranks (one process per GPU).

The bunches of a current scan or an uneven batch are independent: each
rank advances a contiguous range of them in its own BunchBatch, with no
exchange during the steps; results (densities, profiles, fillings) are
gathered to rank 0 when the caller asks for them.  Ranges are balanced by
cost (cells per step, times the interpolation taps of the bunch's chain).

Ranks talk through torch.distributed (NCCL between GPUs, gloo for the
host-side tests); nothing here runs on the device except the batches.
"""
import numpy as np


def bunch_cost(desc):
    """Relative cost of one solver step of a bunch: its cells, weighted by
    the taps of its chain (chain 1 interpolates it^2 taps per cell)."""
    n = int(desc.n)
    it = int(desc.it)
    taps = it * it if int(desc.chain) == 1 else 3 * it + 5
    return float(n) * n * taps


def partition(costs, world):
    """Contiguous ranges [(start, end)] of the bunch list, one per rank,
    each as close as possible to an equal share of the total cost.  Every
    bunch belongs to exactly one range; a rank may get an empty range when
    there are fewer bunches than ranks."""
    costs = np.asarray(costs, np.float64)
    nb = costs.size
    if world < 1:
        raise ValueError("world must be >= 1")
    cum = np.concatenate([[0.0], np.cumsum(costs)])
    total = cum[-1]
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        # first index whose prefix cost reaches the target, kept monotone
        k = int(np.searchsorted(cum, target, side="left"))
        if k > 0 and abs(cum[k - 1] - target) <= abs(cum[min(k, nb)] - target):
            k -= 1
        bounds.append(min(max(k, bounds[-1]), nb))
    bounds.append(nb)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def gather_to_root(local, ranges, rank, world, dist=None, group=None):
    """Concatenate per-rank float32 arrays on rank 0 in bunch order.

    local: this rank's 1-D array (its bunches' values, in order).  Returns
    the concatenation on rank 0 and None elsewhere.  With world == 1 (or no
    process group) the local array is returned as is."""
    local = np.ascontiguousarray(local, np.float32)
    if world == 1 or dist is None:
        return local
    import torch
    sizes = [None] * world
    dist.all_gather_object(sizes, int(local.size), group=group)
    width = max(max(sizes), 1)
    buf = torch.zeros(width, dtype=torch.float32)
    buf[:local.size] = torch.from_numpy(local)
    if rank == 0:
        parts = [torch.zeros(width, dtype=torch.float32) for _ in range(world)]
        dist.gather(buf, parts, dst=0, group=group)
        return np.concatenate([parts[r][:sizes[r]].numpy()
                               for r in range(world)])
    dist.gather(buf, None, dst=0, group=group)
    return None


class ShardedScan:
    """This rank's share of a batch of independent bunches.

    descs: the bunch descriptors of the whole scan (every rank passes the
    same list); impedances: the tables they name.  make_batch(descs, imps)
    builds the local batch (a vfps.BunchBatch on this rank's GPU)."""

    def __init__(self, descs, impedances, rank, world, make_batch, dist=None,
                 group=None):
        self.rank, self.world = rank, world
        self.dist, self.group = dist, group
        self.ranges = partition([bunch_cost(d) for d in descs], world)
        lo, hi = self.ranges[rank]
        self.local = list(descs[lo:hi])
        self.batch = make_batch(self.local, impedances) if self.local else None

    def step(self, nsteps):
        if self.batch is not None:
            self.batch.step(nsteps)

    def profiles(self):
        """All bunches' profiles on rank 0 (None on the other ranks)."""
        if self.batch is None:
            local = np.zeros(0, np.float32)
        else:
            local = np.concatenate([self.batch.profile(i)
                                    for i in range(len(self.local))])
        return gather_to_root(local, self.ranges, self.rank, self.world,
                              self.dist, self.group)

    def fillings(self):
        local = (np.zeros(0, np.float32) if self.batch is None
                 else np.asarray(self.batch.filling(), np.float32))
        return gather_to_root(local, self.ranges, self.rank, self.world,
                              self.dist, self.group)
