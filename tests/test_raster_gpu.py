"""Device label builder (umcx_gpu_build_labels / umcx_job_build_labels) against the host front end (GPU required).

The host rasteriser and detector masking are pinned byte-for-byte to the reference's --dumpmask output
(tests/test_frontend.py); here the GPU-built uint8 labels must equal the host-built ones exactly, for every
built-in benchmark, the benchmark configurations, the batched workload's random domains, a JData volume and edge
cases (single-voxel and one-voxel-thick grids, detectors at corners, outside the grid, of radius 0), and the
errors must match (a shape value read from a missing key, a label without a medium)."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import C1, C2, C3, SHAPES  # noqa: E402

pytestmark = pytest.mark.gpu

BENCHES = ["cube60", "cube60b", "cube60planar", "cubesph60b", "sphshells", "spherebox", "skinvessel"]


def device_labels(ctx, job):
    import torch

    s = job.sim
    d = torch.full((s.dim[0] * s.dim[1] * s.dim[2],), 0xAB, dtype=torch.uint8, device="cuda")
    job.build_labels(ctx, d)
    return d.cpu().numpy().reshape(s.dim[0], s.dim[1], s.dim[2])


def check_same(ctx, args):
    from umcx_gb300 import Job

    host = Job.from_args(args)
    dev = Job.from_args(args, device_labels=True)
    assert dev.labels is None
    ref = host.labels
    np.testing.assert_array_equal(device_labels(ctx, dev), ref)
    # a host-built job rebuilt on the device gives the same bytes too
    np.testing.assert_array_equal(device_labels(ctx, host), ref)
    return ref


@pytest.mark.parametrize("bench", BENCHES)
def test_benchmarks(ctx, bench):
    check_same(ctx, ["--bench", bench])


@pytest.mark.parametrize("name,cfg", [("c1", C1), ("c2", C2), ("c3", C3), ("shapes", SHAPES)])
def test_configurations(ctx, name, cfg):
    lab = check_same(ctx, ["--json", json.dumps(cfg)])
    if name in ("c2", "shapes"):
        assert (lab & 0x80).any()  # detectors were masked


def test_batched_workload_domains(ctx):
    from umcx_gb300.workloads import config5

    for i in range(24):
        check_same(ctx, ["--json", json.dumps(config5(i))])


def test_jdata_volume_with_detectors(ctx):
    rng = np.random.default_rng(5)
    vol = rng.integers(0, 3, size=(12, 10, 8)).astype(np.int64)
    vol[:, :, 2:] = np.maximum(vol[:, :, 2:], 1)
    cfg = dict(C2)
    cfg = json.loads(json.dumps(cfg))
    cfg["Shapes"] = {"_ArraySize_": [12, 10, 8], "_ArrayType_": "uint8", "_ArrayData_": vol.ravel().tolist()}
    cfg["Domain"]["Dim"] = [12, 10, 8]
    cfg["Optode"]["Source"]["Pos"] = [5, 5, 0]
    cfg["Optode"]["Detector"] = [{"Pos": [3, 3, 2], "R": 2}, {"Pos": [11, 9, 7], "R": 1.5}]
    lab = check_same(ctx, ["--json", json.dumps(cfg)])
    assert (lab & 0x80).any()


@pytest.mark.parametrize("dim,dets", [
    ([1, 1, 1], [{"Pos": [0, 0, 0], "R": 1}]),
    ([1, 7, 5], [{"Pos": [0, 3, 2], "R": 2}]),
    ([9, 1, 6], [{"Pos": [4, 0, 3], "R": 0}, {"Pos": [8.5, 0.5, 5.5], "R": 0.7}]),
    ([16, 16, 16], [{"Pos": [0, 0, 0], "R": 3}, {"Pos": [15.9, 15.9, 15.9], "R": 2.5}, {"Pos": [-3, 8, 8], "R": 2},
                    {"Pos": [8, 8, 30], "R": 1}, {"Pos": [7.25, 8.5, 8.75], "R": 4.3}]),
])
def test_edge_grids_and_detectors(ctx, dim, dets):
    cfg = json.loads(json.dumps(SHAPES))
    cfg["Domain"]["Dim"] = dim
    cfg["Shapes"] = [{"Grid": {"Tag": 1, "Size": dim}}, {"Sphere": {"O": [d / 2 for d in dim], "R": 2, "Tag": 2}},
                     {"ZLayers": [[0, 1, 0], [2, 3, 3]]}]
    cfg["Optode"]["Source"]["Pos"] = [0, 0, 0]
    cfg["Optode"]["Detector"] = dets
    check_same(ctx, ["--json", json.dumps(cfg)])


def test_missing_shape_value_reported_on_device(ctx):
    from umcx_gb300 import Job

    cfg = json.loads(json.dumps(C1))
    cfg["Shapes"].append({"Box": {"O": [10, 10, 10], "Tag": 2}})  # no "Sip.ze": read once a voxel passes O
    args = ["--json", json.dumps(cfg)]
    with pytest.raises(ValueError, match="type must be number, but is null"):
        Job.from_args(args)
    dev = Job.from_args(args, device_labels=True)
    with pytest.raises(RuntimeError, match="type must be number, but is null"):
        device_labels(ctx, dev)


def test_label_without_medium_reported_on_device(ctx):
    from umcx_gb300 import Job

    cfg = json.loads(json.dumps(C1))
    cfg["Shapes"].append({"Sphere": {"O": [30, 30, 30], "R": 5, "Tag": 7}})
    args = ["--json", json.dumps(cfg)]
    with pytest.raises(ValueError, match="label 7 has no entry in Domain.Media") as host_err:
        Job.from_args(args)
    dev = Job.from_args(args, device_labels=True)
    with pytest.raises(RuntimeError, match="label 7 has no entry in Domain.Media"):
        device_labels(ctx, dev)
    assert "label 7" in str(host_err.value)


def test_batch_with_device_labels_matches_host_labels(ctx):
    from umcx_gb300 import Batch
    from umcx_gb300.workloads import batch5

    host_jobs = batch5(12, photon_scale=0.01, max_edge=64)
    dev_jobs = batch5(12, photon_scale=0.01, max_edge=64, device_labels=True)
    a = Batch.from_jobs(ctx, host_jobs)
    b = Batch.from_jobs(ctx, dev_jobs, device_labels=True)
    ra, rb = a.run(), b.run()
    assert ra.launched == rb.launched and ra.steps == rb.steps and ra.crossings == rb.crossings
    for i in range(12):
        fa, xa = a.get(i)
        fb, xb = b.get(i)
        assert xa.launched == xb.launched
        assert abs(xa.energy_escape - xb.energy_escape) <= 1e-9 * xa.energy_total
        np.testing.assert_allclose(fb, fa, rtol=1e-6, atol=0)
