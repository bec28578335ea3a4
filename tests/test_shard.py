"""Photon-range sharding across ranks (no GPU): two gloo ranks on the CPU, each simulating its share of the photon
index range with the CPU oracle, reduce to exactly the single-process run (up to FP32 summation order)."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_shard_range_partitions():
    from umcx_gb300.shard import shard_range

    for n in (0, 1, 7, 1000, 1000003):
        for world in (1, 2, 3, 8):
            spans = [shard_range(n, r, world, offset=5) for r in range(world)]
            assert sum(c for _, c in spans) == n
            pos = 5
            for start, count in spans:
                assert start == pos
                pos += count


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, outdir):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import oracle
    from umcx_gb300 import Job
    from umcx_gb300.shard import reduce_results, shard_sim

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    job = Job.from_args(["--bench", "cubesph60b", "-n", "6000"])
    s = shard_sim(job.sim, rank, world)
    flu, dp, res, _ = oracle.forward(s, job.labels, job.media, job.detpos, nthreads=1)
    f, esc, tot, rows = reduce_results(flu, res.energy_escape, res.energy_total, dp)
    if rank == 0:
        np.savez(os.path.join(outdir, "sharded.npz"), f=f, esc=esc, tot=tot, rows=rows)
    dist.destroy_process_group()


def test_two_ranks_equal_single_run(tmp_path):
    import torch.multiprocessing as mp

    import oracle
    from umcx_gb300 import Job

    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    got = np.load(tmp_path / "sharded.npz")
    job = Job.from_args(["--bench", "cubesph60b", "-n", "6000"])
    f, dp, res, _ = oracle.forward(job.sim, job.labels, job.media, job.detpos, nthreads=1)
    assert abs(float(got["tot"]) - res.energy_total) <= 1e-9 * res.energy_total
    assert abs(float(got["esc"]) - res.energy_escape) <= 1e-9 * res.energy_total
    np.testing.assert_allclose(got["f"], f, rtol=1e-5, atol=1e-7)
    a = got["rows"]
    assert a.shape == dp.shape
    np.testing.assert_array_equal(a[np.lexsort(a.T[::-1])], dp[np.lexsort(dp.T[::-1])])
