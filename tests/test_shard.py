"""Photon-range sharding across ranks: two gloo ranks, each simulating its share of the photon index range (with
the CPU oracle, or -- marked gpu -- through the CUDA library with both ranks on cuda:0), reduce to exactly the
single-process run (up to FP32 summation order)."""
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


def _worker_tensors(rank, world, port, outdir):
    """Torch-tensor outputs through Shard.reduce_device (gloo, CPU tensors), as bench.py reduces a sharded step."""
    sys.path.insert(0, str(ROOT))
    import torch

    import oracle
    from umcx_gb300 import Job
    from umcx_gb300.shard import Shard

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sh = Shard.init("gloo")
    job = Job.from_args(["--bench", "cubesph60b", "-n", "6000"])
    s = job.sim.copy()
    s.photon_offset, s.nphoton = sh.photon_range(3000)
    flu, dp, res, _ = oracle.forward(s, job.labels, job.media, job.detpos, nthreads=1)
    t_flu = torch.from_numpy(flu.ravel().copy())
    out = sh.reduce_device(t_flu, torch.from_numpy(dp.copy()), res)
    mx = sh.max_over_ranks([float(rank), 10.0 - rank])
    if rank == 0:
        np.savez(os.path.join(outdir, "tensors.npz"), f=t_flu.numpy(), esc=out["energy_escape"],
                 tot=out["energy_total"], rows=out["rows"].numpy(), launched=out["launched"], steps=out["steps"],
                 detected=out["detected"], mx=np.array(mx))
    sh.close()


def test_two_ranks_torch_tensors_equal_single_run(tmp_path):
    import torch.multiprocessing as mp

    import oracle
    from umcx_gb300 import Job

    port = _free_port()
    mp.start_processes(_worker_tensors, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    got = np.load(tmp_path / "tensors.npz")
    job = Job.from_args(["--bench", "cubesph60b", "-n", "6000"])
    f, dp, res, _ = oracle.forward(job.sim, job.labels, job.media, job.detpos, nthreads=1)
    assert int(got["launched"]) == 6000 and int(got["steps"]) == res.steps and int(got["detected"]) == res.detected
    assert abs(float(got["tot"]) - res.energy_total) <= 1e-9 * res.energy_total
    assert abs(float(got["esc"]) - res.energy_escape) <= 1e-9 * res.energy_total
    np.testing.assert_allclose(got["f"], f.ravel(), rtol=1e-5, atol=1e-7)
    a = got["rows"]
    np.testing.assert_array_equal(a[np.lexsort(a.T[::-1])], dp[np.lexsort(dp.T[::-1])])
    assert list(got["mx"]) == [1.0, 10.0]


def _worker_gpu(rank, world, port, outdir, backend="gloo"):
    """Each rank runs its photon range through the CUDA library on cuda:0, then the ranks reduce (gloo when two
    processes share one GPU: no kernel of one waits for the other, the exchange is on the host; nccl with one rank)."""
    sys.path.insert(0, str(ROOT))
    import torch

    from umcx_gb300 import Context, Job, detp_columns
    from umcx_gb300.shard import Shard, shard_sim

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sh = Shard.init(backend)
    job = Job.from_args(["--bench", "cubesph60b", "-n", "200000"])
    s = shard_sim(job.sim, rank, world)
    torch.cuda.set_device(0)
    with Context(0) as ctx:
        d_lab = torch.from_numpy(job.labels.ravel().copy()).cuda()
        cols = detp_columns(s)
        d_flu = torch.zeros(s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3], dtype=torch.float32, device="cuda")
        d_det = torch.zeros(s.maxdetphotons * cols, dtype=torch.float32, device="cuda")
        r = ctx.forward_device(s, d_lab, job.media, job.detpos, d_flu, d_det, torch.cuda.current_stream())
        out = sh.reduce_device(d_flu, d_det[: r.saved * cols].view(-1, cols), r)
        out["max_ms"] = sh.max_over_ranks([r.kernel_ms])[0]
        sh.barrier()
        if rank == 0:
            np.savez(os.path.join(outdir, "gpu.npz"), f=d_flu.cpu().numpy(), esc=out["energy_escape"],
                     tot=out["energy_total"], rows=out["rows"].cpu().numpy(), launched=out["launched"],
                     steps=out["steps"], crossings=out["crossings"], detected=out["detected"], max_ms=out["max_ms"],
                     kernel_ms=r.kernel_ms)
    sh.close()


@pytest.mark.gpu
def test_two_ranks_on_the_cuda_path_equal_single_run(tmp_path):
    """Two ranks each simulate half of the photon range through the CUDA library and reduce: the same event counts
    and detected rows as one run of all photons, energies to 1e-9, the volume to FP32 summation order."""
    import torch
    import torch.multiprocessing as mp

    from umcx_gb300 import Context, Job

    port = _free_port()
    mp.start_processes(_worker_gpu, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    got = np.load(tmp_path / "gpu.npz")
    job = Job.from_args(["--bench", "cubesph60b", "-n", "200000"])
    with Context(0) as ctx:
        one = ctx.forward(job.sim, job.labels, job.media, job.detpos)
    r = one.result
    assert (int(got["launched"]), int(got["steps"]), int(got["crossings"]), int(got["detected"])) == (
        r.launched, r.steps, r.crossings, r.detected)
    assert abs(float(got["tot"]) - r.energy_total) <= 1e-9 * r.energy_total
    assert abs(float(got["esc"]) - r.energy_escape) <= 1e-9 * r.energy_total
    np.testing.assert_allclose(got["f"], one.fluence.ravel(), rtol=2e-5, atol=1e-6)
    a, b = got["rows"], one.detp
    np.testing.assert_array_equal(a[np.lexsort(a.T[::-1])], b[np.lexsort(b.T[::-1])])


@pytest.mark.gpu
def test_one_nccl_rank_on_the_cuda_path_equals_single_run(tmp_path):
    """The reduction that bench.py --gpus N performs under NCCL (in-place all-reduce of the device volume, all-gather
    of the detected rows with padded counts, tallies and the max over ranks), run by one NCCL rank on the device
    tensors of its own run (one GPU cannot hold two NCCL ranks): counts and detected rows equal the single run, energies
    and the volume to their summation order."""
    import torch.multiprocessing as mp

    from umcx_gb300 import Context, Job

    port = _free_port()
    mp.start_processes(_worker_gpu, args=(1, port, str(tmp_path), "nccl"), nprocs=1, start_method="spawn", join=True)
    got = np.load(tmp_path / "gpu.npz")
    job = Job.from_args(["--bench", "cubesph60b", "-n", "200000"])
    with Context(0) as ctx:
        one = ctx.forward(job.sim, job.labels, job.media, job.detpos)
    r = one.result
    assert (int(got["launched"]), int(got["steps"]), int(got["crossings"]), int(got["detected"])) == (
        r.launched, r.steps, r.crossings, r.detected)
    # (the FP64 tallies are sums of per-warp atomics: their order, and so their last bits, varies between runs)
    assert abs(float(got["tot"]) - r.energy_total) <= 1e-12 * r.energy_total
    assert abs(float(got["esc"]) - r.energy_escape) <= 1e-12 * r.energy_total
    assert float(got["max_ms"]) == float(got["kernel_ms"])
    np.testing.assert_allclose(got["f"], one.fluence.ravel(), rtol=2e-6, atol=1e-7)
    a, b = got["rows"], one.detp
    np.testing.assert_array_equal(a[np.lexsort(a.T[::-1])], b[np.lexsort(b.T[::-1])])
