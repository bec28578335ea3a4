"""Edge cases of the CUDA forward path (GPU required): no photons, single photons, a full detected-photon buffer,
more media than the reference's fixed partial-path scratch holds, and a domain with no tissue."""
import json
import math
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import C1, C2  # noqa: E402
from statcheck import det_stats, run_batches, z_of_means  # noqa: E402

pytestmark = pytest.mark.gpu

# 16 tissue labels (17 media with the background): one-voxel layers of labels 2..16 between label-1 layers, a
# refractive-index change at every layer boundary, four detectors on the source face and partial paths saved.
# The reference keeps partial paths in a fixed 10-float scratch per photon (src/umcx.cpp:757), so it overflows
# beyond 11 media; here every medium has its column.
L16 = {"Session": {"ID": "l16", "Photons": 1000, "RNGSeed": 12345, "DoMismatch": 1, "DoPartialPath": 1,
                   "SaveDetFlag": 5, "OutputType": "x"},
       "Forward": {"T0": 0, "T1": 5e-9, "Dt": 5e-10},
       "Domain": {"Dim": [40, 40, 40], "LengthUnit": 1,
                  "Media": [{"mua": 0, "mus": 0, "g": 1, "n": 1}] + [
                      {"mua": round(0.002 + 0.001 * k, 4), "mus": round(0.6 + 0.25 * k, 3),
                       "g": round(0.5 + 0.025 * k, 3), "n": round(1.33 + 0.02 * (k % 5), 2)} for k in range(16)]},
       "Optode": {"Source": {"Type": "pencil", "Pos": [20, 20, 0], "Dir": [0, 0, 1]},
                  "Detector": [{"Pos": [20, 14, 0], "R": 2}, {"Pos": [14, 20, 0], "R": 2},
                               {"Pos": [20, 26, 0], "R": 2}, {"Pos": [26, 20, 0], "R": 2}]},
       "Shapes": [{"Grid": {"Tag": 1, "Size": [40, 40, 40]}},
                  {"ZLayers": [[2 * k + 3, 2 * k + 4, k + 2] for k in range(15)]}]}


def job_for(cfg, photons):
    from umcx_gb300 import Job

    cfg = json.loads(json.dumps(cfg))
    cfg["Session"]["Photons"] = int(photons)
    return Job.from_json(cfg)


def test_zero_photons(ctx):
    job = job_for(C2, 1000)
    s = job.sim
    s.nphoton = 0
    out = ctx.forward(s, job.labels, job.media, job.detpos)
    r = out.result
    assert r.status == 0 and r.launched == 0 and r.steps == 0 and r.detected == 0 and r.saved == 0
    assert r.energy_total == 0.0 and r.energy_escape == 0.0
    assert not out.fluence.any()


def test_single_photons_follow_the_oracle(ctx):
    """One photon per launch (one CTA, one busy lane): the strict kernel reproduces the oracle's event counts and
    deposits for most photon indices (the rest differ by a last-ulp difference of a math function at a boundary)."""
    import oracle
    from umcx_gb300._lib import SIM_STRICT_MATH

    job = job_for(C1, 1)
    same = 0
    for i in range(10):
        s = job.sim
        s.nphoton = 1
        s.photon_offset = i
        c_flu, _, c, _ = oracle.forward(s, job.labels, job.media, job.detpos)
        s.flags = SIM_STRICT_MATH
        out = ctx.forward(s, job.labels, job.media, job.detpos)
        g = out.result
        assert g.launched == 1 and g.status == 0
        if (g.steps, g.crossings, g.scatters, g.reflections) == (c.steps, c.crossings, c.scatters, c.reflections):
            same += 1
            np.testing.assert_allclose(out.fluence, c_flu, rtol=1e-4, atol=1e-7)
            assert abs(g.energy_escape - c.energy_escape) <= 1e-4 * max(c.energy_total, 1e-30) + 1e-6
    assert same >= 7, same


def test_detected_buffer_overflow(ctx):
    """With fewer record slots than detected photons, every detection is still counted, only the first
    maxdetphotons records are stored (MCX_detect::addphoton, src/umcx.cpp:164-176), and the physics is unchanged."""
    job = job_for(C2, 200000)
    s = job.sim
    full = ctx.forward(s, job.labels, job.media, job.detpos)
    assert full.result.detected > 200 and full.result.saved == full.result.detected
    s.maxdetphotons = 64
    small = ctx.forward(s, job.labels, job.media, job.detpos)
    r = small.result
    assert r.status == 0 and r.detected == full.result.detected and r.saved == 64
    assert small.detp.shape == (64, full.detp.shape[1])
    assert r.steps == full.result.steps and r.scatters == full.result.scatters
    np.testing.assert_allclose(small.fluence, full.fluence, rtol=1e-5, atol=1e-7)
    rows = {tuple(x) for x in full.detp.tolist()}
    assert all(tuple(x) in rows for x in small.detp.tolist())


def test_many_media_partial_paths_match_oracle(ctx):
    """17 media with partial paths and a refractive-index change at every layer: detected counts and per-detector
    mean partial paths of every medium agree with the oracle within 3 standard errors."""
    job = job_for(L16, 200000)
    sim = job.sim
    assert sim.mediumnum == 17 and len(np.unique(job.labels & 0x7F)) == 16

    def gpu(s):
        out = ctx.forward(s, job.labels, job.media, job.detpos)
        return out.fluence, out.detp, out.result

    def cpu(s):
        import oracle

        f, d, r, _ = oracle.forward(s, job.labels, job.media, job.detpos)
        return f, d, r

    g = run_batches(gpu, sim, 20)
    c = run_batches(cpu, sim, 20)
    assert all(r.status == 0 and r.capped == 0 for r in g.results)
    za = z_of_means(g.absorbed, c.absorbed)
    assert abs(za) < 3, (g.absorbed.mean(), c.absorbed.mean(), za)
    ng = sum(r.detected for r in g.results)
    nc = sum(r.detected for r in c.results)
    assert ng > 1000 and abs(ng - nc) <= 3 * math.sqrt(ng + nc) + 1, (ng, nc)
    assert all(d.shape[1] == 1 + sim.mediumnum for d in g.detp if d is not None and len(d))
    cols = slice(1, 1 + sim.mediumnum)
    for (n1, m1, s1), (n2, m2, s2) in zip(det_stats(g.detp, sim.detnum, cols), det_stats(c.detp, sim.detnum, cols)):
        assert abs(n1 - n2) <= 3 * math.sqrt(n1 + n2) + 1
        if n1 > 30 and n2 > 30:
            z = (m1 - m2) / np.sqrt(s1 ** 2 + s2 ** 2 + 1e-30)
            assert np.all(np.abs(z[np.isfinite(z)]) < 3.5), (m1, m2, z)
    gm = sum(r.reflections for r in g.results) / sim.nphoton
    cm = sum(r.reflections for r in c.results) / sim.nphoton
    assert abs(gm - cm) < 0.02 * cm, (gm, cm)


def test_domain_without_tissue(ctx):
    """A grid of background only: photons cross it in straight lines and are never counted in the energy totals
    (final label 0, src/umcx.cpp:765); the path-length deposits of the mua = 0 background match the oracle."""
    import oracle

    cfg = json.loads(json.dumps(C1))
    cfg["Shapes"] = [{"Grid": {"Tag": 0, "Size": [60, 60, 60]}}]
    job = job_for(cfg, 5000)
    s = job.sim
    out = ctx.forward(s, job.labels, job.media, job.detpos)
    c_flu, _, c, _ = oracle.forward(s, job.labels, job.media, job.detpos)
    r = out.result
    assert r.status == 0 and r.launched == 5000
    assert r.energy_total == 0.0 and c.energy_total == 0.0
    assert r.steps == c.steps and r.crossings == c.crossings and r.scatters == 0
    np.testing.assert_allclose(out.fluence, c_flu, rtol=1e-5, atol=1e-6)
