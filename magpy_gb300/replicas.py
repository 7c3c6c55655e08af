"""Ensemble members split over processes, one GPU each.

Members of an ensemble are independent: the reference runs each one as its
own joblib job (magpy/model.py:204-207) and only the statistics of
magpy/results.py:134-217 combine them.  A world of W processes therefore
takes contiguous member ranges, every rank integrates its range in one
launch, and the one exchange is the sum of the per-rank cluster
magnetisations (max_samples x 3 doubles).  Seeds are derived for the whole
ensemble on every rank (magpy/model.py:202-203) and sliced, so member e gets
the same seed, and the same trajectory, at any world size.

The exchange goes through ``torch.distributed`` on CPU tensors (gloo, or any
backend that reduces host tensors); partial sums are gathered and added in
rank order, so every rank holds the same bits whatever the backend's
reduction order.
"""
from __future__ import annotations

import numpy as np

from .results import MU0, _trapezoid


def member_range(n_members: int, world: int, rank: int) -> tuple[int, int]:
    """[start, stop) of rank's members: sizes differ by at most one, the
    larger shares first."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    q, r = divmod(int(n_members), world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def _world(group):
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return 1, 0
    return dist.get_world_size(group), dist.get_rank(group)


def _gather_sum(local: np.ndarray, group) -> np.ndarray:
    """Sum of ``local`` over ranks, added in rank order on every rank."""
    import torch
    import torch.distributed as dist
    world, _ = _world(group)
    if world == 1:
        return np.array(local, dtype=np.float64)
    t = torch.from_numpy(np.ascontiguousarray(local, dtype=np.float64))
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    total = parts[0].numpy().copy()
    for p in parts[1:]:
        total += p.numpy()
    return total


def max_over_ranks(x: float, group=None) -> float:
    """The largest value of a per-rank scalar (e.g. a step time)."""
    import torch
    import torch.distributed as dist
    world, _ = _world(group)
    if world == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


class ShardResults:
    """One rank's members and the ensemble statistics of all ranks.

    ``local`` is the rank's ``EnsembleResults``; ``ensemble_magnetisation``
    and ``energy_dissipated`` are the whole ensemble's, identical on every
    rank.
    """

    def __init__(self, local, start, stop, n_members, M_sum):
        self.local = local
        self.start, self.stop, self.n_members = start, stop, n_members
        self.time = local.time if local is not None else None
        self.field = local.field if local is not None else None
        self._M = M_sum / n_members

    def ensemble_magnetisation(self, direction="z"):
        """magpy/results.py:134-151 over the members of every rank."""
        return self._M["xyz".index(direction)]

    def energy_dissipated(self, start_time=None, end_time=None):
        """magpy/results.py:167-191 on the ensemble magnetisation of every rank."""
        before = (self.time >= start_time) if start_time is not None else True
        after = (self.time <= end_time) if end_time is not None else True
        mask = np.ones_like(self.time, dtype=bool) & before & after
        return -MU0 * _trapezoid(self.field[mask], self.ensemble_magnetisation()[mask])

    def final_cycle_energy_dissipated(self, field_frequency):
        """magpy/results.py:193-217."""
        return self.energy_dissipated(start_time=self.time[-1] - 1.0 / field_frequency)


def simulate_shard(model, end_time, time_step, max_samples, random_state, group=None,
                   simulate_members=None, **kwargs) -> ShardResults:
    """``EnsembleModel.simulate`` with the members split over the ranks of
    ``group`` (the default process group when None; one process = the whole
    ensemble).  ``simulate_members(members, seeds, end_time, time_step,
    max_samples, **kwargs)`` integrates a member range; it defaults to the
    model's GPU path."""
    world, rank = _world(group)
    E = model.ensemble_size
    start, stop = member_range(E, world, rank)
    seeds = model.seeds(random_state)[start:stop]
    run = simulate_members or model.simulate_members
    local = None
    S = int(max_samples)
    M_local = np.zeros((3, S))
    if stop > start:
        local = run(range(start, stop), seeds, end_time, time_step, max_samples, **kwargs)
        n_local = stop - start
        for c, d in enumerate("xyz"):
            M_local[c] = local.ensemble_magnetisation(d) * n_local
    M_sum = _gather_sum(M_local, group)
    res = ShardResults(local, start, stop, E, M_sum)
    if local is None:
        # a rank without members still reports the common time and field axes
        res.time, res.field = _broadcast_axes(group)
    else:
        _broadcast_axes(group, local.time, local.field)
    return res


def _broadcast_axes(group, time=None, field=None):
    """Time and field samples from rank 0 (which always has members)."""
    import torch
    import torch.distributed as dist
    world, rank = _world(group)
    if world == 1:
        return time, field
    S = torch.tensor([0 if time is None else len(time)], dtype=torch.int64)
    dist.broadcast(S, src=dist.get_global_rank(group, 0) if group is not None else 0,
                   group=group)
    buf = torch.zeros(2, int(S.item()), dtype=torch.float64)
    if rank == 0:
        buf[0] = torch.from_numpy(np.asarray(time, dtype=np.float64))
        buf[1] = torch.from_numpy(np.asarray(field, dtype=np.float64))
    dist.broadcast(buf, src=dist.get_global_rank(group, 0) if group is not None else 0,
                   group=group)
    return buf[0].numpy(), buf[1].numpy()
