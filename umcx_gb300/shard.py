"""Photon-range sharding across ranks (one process per GPU), torch.distributed for the final reduction.

Photon i's random stream depends only on (session seeds, i) (fangq/umcx src/umcx.cpp:752, 761), so a simulation of
N photons splits into disjoint index ranges that ranks run independently; the results of the whole run are the sums
of the ranks' output volumes and energy tallies (a single reduction at the end, no exchange on the data path) and the
concatenation of their detected-photon rows.

The reduction takes the outputs where they are: numpy arrays or CPU tensors through any backend, CUDA tensors in
place on the GPU through NCCL.  Under gloo a CUDA tensor is reduced through a host copy.
"""
from __future__ import annotations

import os

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


def _backend(group=None) -> str:
    import torch.distributed as dist

    return str(dist.get_backend(group)).lower()


def _all_reduce_sum(t, group=None):
    """In-place sum over ranks of tensor t; a CUDA tensor under a CPU-only backend goes through a host copy."""
    import torch.distributed as dist

    if t.is_cuda and _backend(group) != "nccl":
        h = t.cpu()
        dist.all_reduce(h, op=dist.ReduceOp.SUM, group=group)
        t.copy_(h)
    else:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


def _gather_rows(rows, group=None):
    """Concatenation over ranks (in rank order) of each rank's [n_r, cols] detected rows."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    if not isinstance(rows, torch.Tensor):
        gathered = [None] * world
        dist.all_gather_object(gathered, np.asarray(rows), group=group)
        nonempty = [g for g in gathered if g is not None and len(g)]
        return np.concatenate(nonempty, axis=0) if nonempty else np.zeros((0, rows.shape[1]), np.float32)
    cols = rows.shape[1]
    dev = rows.device if (rows.is_cuda and _backend(group) == "nccl") else torch.device("cpu")
    n = torch.tensor([rows.shape[0]], dtype=torch.int64, device=dev)
    counts = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    counts = [int(c.item()) for c in counts]
    most = max(counts)
    pad = torch.zeros((most, cols), dtype=rows.dtype, device=dev)
    pad[: rows.shape[0]] = rows.to(dev)
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    out = torch.cat([p[:c] for p, c in zip(parts, counts)], dim=0)
    return out.to(rows.device)


def reduce_results(fluence, energy_escape: float, energy_total: float, detp=None, group=None):
    """Sum output volumes and energies over ranks and gather detected-photon rows (on every rank).

    fluence / detp: numpy arrays (returned as numpy) or torch tensors (fluence reduced in place on its device,
    rows gathered on it).  Returns (fluence, energy_escape, energy_total, rows)."""
    import torch

    if fluence is None:
        f = None
    elif isinstance(fluence, torch.Tensor):
        f = _all_reduce_sum(fluence, group)
    else:
        f = _all_reduce_sum(torch.from_numpy(np.ascontiguousarray(fluence, np.float32)), group).numpy()
    dev = fluence.device if isinstance(fluence, torch.Tensor) and fluence.is_cuda and _backend(group) == "nccl" \
        else torch.device("cpu")
    e = torch.tensor([energy_escape, energy_total], dtype=torch.float64, device=dev)
    _all_reduce_sum(e, group)
    rows = None if detp is None else _gather_rows(detp, group)
    return f, float(e[0]), float(e[1]), rows


class Shard:
    """One rank of a photon-range-sharded simulation: its photon range and the end-of-step reduction."""

    def __init__(self, rank: int, world: int, group=None):
        self.rank, self.world, self.group = rank, world, group

    @classmethod
    def init(cls, backend: str = "nccl") -> "Shard":
        """Join the process group from the torchrun environment (RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT)."""
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if not dist.is_initialized():
            dist.init_process_group(backend)
        return cls(dist.get_rank(), dist.get_world_size())

    def photon_range(self, photons_per_rank: int) -> tuple[int, int]:
        """(first photon index, count) of this rank when every rank simulates photons_per_rank photons of one
        world x photons_per_rank simulation (weak scaling)."""
        return self.rank * int(photons_per_rank), int(photons_per_rank)

    def reduce_device(self, d_fluence, d_rows, result) -> dict:
        """The end of a sharded step: sums the output volume in place and the tallies over ranks, gathers the
        detected rows; returns the whole simulation's energies, event counts and rows."""
        import torch

        f, esc, tot, rows = reduce_results(d_fluence, result.energy_escape, result.energy_total, d_rows, self.group)
        dev = d_fluence.device if d_fluence is not None and d_fluence.is_cuda and _backend(self.group) == "nccl" \
            else torch.device("cpu")
        counts = torch.tensor([result.launched, result.steps, result.crossings, result.scatters, result.detected],
                              dtype=torch.float64, device=dev)
        _all_reduce_sum(counts, self.group)
        c = [int(x) for x in counts.tolist()]
        return {"energy_escape": esc, "energy_total": tot, "rows": rows, "launched": c[0], "steps": c[1],
                "crossings": c[2], "scatters": c[3], "detected": c[4]}

    def barrier(self):
        import torch.distributed as dist

        dist.barrier(group=self.group)

    def max_over_ranks(self, values):
        import torch
        import torch.distributed as dist

        dev = torch.device("cuda", torch.cuda.current_device()) if _backend(self.group) == "nccl" else "cpu"
        t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=self.group)
        return t.tolist()

    def close(self):
        import torch.distributed as dist

        if dist.is_initialized():
            dist.destroy_process_group()
