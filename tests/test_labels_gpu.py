"""Palette-packed shared-memory labels (GPU required).

The fast forward kernel can read voxel labels from a 2- or 4-bit palette-packed copy of the label volume held in
shared memory instead of the uint8 volume in global memory.  The label bytes it sees are the same, so every photon
follows the same path: the same step / crossing / scatter counts, the same detected-photon records (compared
exactly, as sorted rows) and the same output volume up to the order of FP64 atomic additions."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import C2, SHAPES  # noqa: E402

pytestmark = pytest.mark.gpu


def job_for(cfg, photons):
    from umcx_gb300 import Job

    cfg = json.loads(json.dumps(cfg))
    cfg["Session"]["Photons"] = int(photons)
    return Job.from_args(["-j", json.dumps(cfg)])


def run(ctx, sim, labels, media, detpos, pack, block=512):
    ctx.set_tuning(block_size=block, aggregation=1, label_pack=pack)
    try:
        return ctx.forward(sim, labels, media, detpos)
    finally:
        ctx.set_tuning()


def sorted_rows(detp):
    if detp is None:
        return np.zeros((0, 0), np.float32)
    d = np.asarray(detp)
    return d[np.lexsort(d.T[::-1])] if len(d) else d


def assert_same_photons(a, b):
    ra, rb = a.result, b.result
    for k in ("launched", "steps", "crossings", "scatters", "reflections", "detected", "saved", "capped"):
        assert getattr(ra, k) == getattr(rb, k), k
    assert abs(ra.energy_total - rb.energy_total) <= 1e-12 * ra.energy_total
    assert abs(ra.energy_escape - rb.energy_escape) <= 1e-12 * ra.energy_total
    np.testing.assert_array_equal(sorted_rows(a.detp), sorted_rows(b.detp))
    np.testing.assert_allclose(a.fluence, b.fluence, rtol=1e-6, atol=0)


def test_two_bit_palette_same_photons(ctx):
    job = job_for(C2, 100000)  # labels 1, 2 and detector-flagged copies: at most 4 bytes, 2 bits per voxel
    g = run(ctx, job.sim, job.labels, job.media, job.detpos, pack=1)
    p = run(ctx, job.sim, job.labels, job.media, job.detpos, pack=2)
    assert g.result.label_bits == 0 and p.result.label_bits == 2
    assert_same_photons(g, p)


def test_four_bit_palette_same_photons(ctx):
    job = job_for(SHAPES, 50000)
    nbytes = len(np.unique(job.labels))
    assert 4 < nbytes <= 16
    g = run(ctx, job.sim, job.labels, job.media, job.detpos, pack=1)
    p = run(ctx, job.sim, job.labels, job.media, job.detpos, pack=2, block=1024)
    assert g.result.label_bits == 0 and p.result.label_bits == 4
    assert_same_photons(g, p)


def test_too_many_label_bytes_reads_global(ctx):
    job = job_for(C2, 20000)
    s = job.sim
    lab = job.labels.copy()
    nmed = 20
    # 19 tissue labels in x slabs: 19 label bytes + the detector-flagged copies, more than 16
    x = np.arange(s.dim[0])[:, None, None]
    lab = np.where(lab & 0x7F, ((x * (nmed - 1)) // s.dim[0] + 1) | (lab & 0x80), lab).astype(np.uint8)
    assert len(np.unique(lab)) > 16
    media = np.tile(np.asarray(job.media)[1:2], (nmed, 1))
    media[0] = job.media[0]
    s.mediumnum = nmed
    out = run(ctx, s, lab, media, job.detpos, pack=2)
    assert out.result.label_bits == 0 and out.result.launched == s.nphoton


def test_label_source_selection(ctx):
    job = job_for(C2, 20000)
    # automatic mode reads global memory (no measured gain from the copy)
    out = run(ctx, job.sim, job.labels, job.media, job.detpos, pack=0, block=1024)
    assert out.result.label_bits == 0
    # strict math keeps the reference's label reads
    s = job.sim
    s.flags |= 1
    out = run(ctx, s, job.labels, job.media, job.detpos, pack=2, block=1024)
    assert out.result.label_bits == 0


def test_device_api_packs_device_labels(ctx):
    import torch

    job = job_for(C2, 50000)
    s = job.sim
    host = run(ctx, s, job.labels, job.media, job.detpos, pack=1)
    d_lab = torch.from_numpy(job.labels.ravel().copy()).cuda()
    d_flu = torch.zeros(host.fluence.size, dtype=torch.float32, device="cuda")
    d_det = torch.zeros(s.maxdetphotons * host.detp.shape[1], dtype=torch.float32, device="cuda")
    ctx.set_tuning(block_size=512, aggregation=1, label_pack=2)
    try:
        r = ctx.forward_device(s, d_lab, job.media, job.detpos, d_flu, d_det, torch.cuda.current_stream())
    finally:
        ctx.set_tuning()
    assert r.label_bits == 2
    assert r.steps == host.result.steps and r.detected == host.result.detected
    np.testing.assert_allclose(d_flu.cpu().numpy().reshape(host.fluence.shape), host.fluence, rtol=1e-6, atol=0)
