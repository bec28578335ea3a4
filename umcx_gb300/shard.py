"""Photon-range sharding across ranks (one process per GPU), torch.distributed for the final reduction.

Photon i's random stream depends only on (session seeds, i), so a simulation of N photons splits into disjoint
index ranges that ranks run independently; the results of the whole run are the sums of the ranks' output volumes
and energy tallies (a single reduction at the end, no exchange on the data path) and the concatenation of their
detected-photon rows.
"""
from __future__ import annotations

import numpy as np


def shard_range(nphoton: int, rank: int, world: int, offset: int = 0) -> tuple[int, int]:
    """(first photon index, photon count) of `rank` when nphoton photons are split across `world` ranks."""
    base, extra = divmod(int(nphoton), int(world))
    start = rank * base + min(rank, extra)
    count = base + (1 if rank < extra else 0)
    return offset + start, count


def shard_sim(sim, rank: int, world: int):
    """A copy of sim restricted to this rank's photon range (strong scaling: the total photon count is fixed)."""
    s = sim.copy()
    s.photon_offset, s.nphoton = shard_range(sim.nphoton, rank, world, sim.photon_offset)
    return s


def reduce_results(fluence, energy_escape: float, energy_total: float, detp=None, group=None):
    """Sum output volumes and energies over ranks and gather detected-photon rows (on every rank)."""
    import torch
    import torch.distributed as dist

    f = torch.from_numpy(np.ascontiguousarray(fluence, np.float32)) if fluence is not None else None
    if f is not None:
        dist.all_reduce(f, op=dist.ReduceOp.SUM, group=group)
    e = torch.tensor([energy_escape, energy_total], dtype=torch.float64)
    dist.all_reduce(e, op=dist.ReduceOp.SUM, group=group)
    rows = None
    if detp is not None:
        gathered = [None] * dist.get_world_size(group)
        dist.all_gather_object(gathered, np.asarray(detp), group=group)
        rows = np.concatenate([g for g in gathered if g is not None and len(g)], axis=0) if any(
            g is not None and len(g) for g in gathered) else np.zeros((0, detp.shape[1] if detp.ndim == 2 else 0),
                                                                       np.float32)
    return (None if f is None else f.numpy()), float(e[0]), float(e[1]), rows
