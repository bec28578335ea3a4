"""Batched simulations (one persistent, graph-captured launch) against single runs of the same simulations and
against the CPU oracle (GPU).

Every photon of simulation i is seeded exactly as in a single run of i, so photon histories are the same up to the
last bits of single-precision arithmetic (the batched and single kernels are separate compilations, which may
contract multiply-adds differently, so an occasional photon drifts by an ulp and then diverges): launched energy
agrees exactly, escaped energy and output volumes to ~1e-6.  The single-run path itself is checked against the CPU
oracle in test_forward_gpu.py."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_batch(n=12, scale=0.02, max_edge=64):
    from umcx_gb300.workloads import batch5

    return batch5(n, photon_scale=scale, max_edge=max_edge)


def test_batch_matches_single_runs(ctx):
    from umcx_gb300.api import Batch

    jobs = small_batch()
    b = Batch.from_jobs(ctx, jobs)
    tot = b.run()
    assert tot.status == 0
    assert tot.launched == sum(j.sim.nphoton for j in jobs)
    for i, j in enumerate(jobs):
        flu, r = b.get(i)
        single = ctx.forward(j.sim, j.labels, j.media, j.detpos)
        assert abs(r.energy_total - single.result.energy_total) <= 1e-9 * single.result.energy_total
        # a diverging photon moves its whole remaining weight (<= 1) between escape and absorption
        assert abs(r.energy_escape - single.result.energy_escape) <= max(5.0, 1e-5 * single.result.energy_total)
        a, s = flu.astype(np.float64), single.fluence.astype(np.float64)
        assert abs(a.sum() - s.sum()) <= 1e-4 * s.sum()
        assert np.linalg.norm(a - s) <= 1e-2 * np.linalg.norm(s)
    b.close()


def test_batch_graph_replay_is_repeatable(ctx):
    from umcx_gb300.api import Batch

    jobs = small_batch(6, scale=0.01)
    b = Batch.from_jobs(ctx, jobs)
    r1 = b.run()
    f1, _ = b.get(3)
    r2 = b.run()
    f2, _ = b.get(3)
    assert (r1.steps, r1.crossings, r1.scatters) == (r2.steps, r2.crossings, r2.scatters)
    np.testing.assert_allclose(f1, f2, rtol=1e-6, atol=1e-9)
    b.set_tuning(256, 0, 2)  # re-captured with aggregation on
    r3 = b.run()
    assert r3.steps == r1.steps
    b.close()


def test_zero_progress_guard_on_batched_workload(ctx):
    """The 256-simulation workload at 30 % of its photon budgets contains photons that would bounce in place
    forever at a grid face (a zero direction component with a stale inverse direction, reflected back onto the
    face).  They are stopped by the zero-progress guard and counted in `capped`; the launch finishes quickly."""
    from umcx_gb300.api import Batch
    from umcx_gb300.workloads import batch5

    jobs = batch5(256, photon_scale=0.3)
    b = Batch.from_jobs(ctx, jobs)
    b.set_tuning(1024, 0, 1, 60000)
    r = b.run()
    print(f"scale 0.3 batch: {r.launched} photons in {r.kernel_ms:.1f} ms, capped {r.capped}")
    assert r.status == 0 and r.launched == sum(j.sim.nphoton for j in jobs)
    assert r.capped >= 1 and r.capped <= 100
    assert r.kernel_ms < 30000
    b.close()


def test_batch_requires_detector_positions(ctx):
    from umcx_gb300 import Job
    from umcx_gb300.api import Batch

    j = Job.from_args(["--bench", "cube60b", "-n", "1000"])
    assert j.sim.issavedet and j.sim.detnum > 0
    with pytest.raises(RuntimeError, match="detpos is NULL"):
        Batch(ctx, [j.sim], [j.labels], [j.media], None)


def detector_rows_by_id(rows, detnum):
    return [rows[rows[:, 0] == d] for d in range(1, detnum + 1)]


def test_batch_detected_photons_match_single_runs(ctx):
    """Simulations that save detected photons keep their own records inside a batch, next to simulations that save
    none: per simulation the detection count and the per-detector record count and mean partial paths equal a single
    run's (up to the rare photon that drifts by an ulp between the two compilations); a simulation whose row capacity
    is below its detections counts them all and keeps exactly its capacity."""
    from umcx_gb300 import Job
    from umcx_gb300.api import Batch

    det_jobs = [Job.from_args(["--bench", "cube60b", "-n", "40000"]),
                Job.from_args(["--bench", "cubesph60b", "-n", "60000"]),
                Job.from_args(["--bench", "cube60b", "-n", "30000", "-E", "7"])]
    plain = small_batch(3, scale=0.01)
    jobs = [plain[0], det_jobs[0], plain[1], det_jobs[1], det_jobs[2], plain[2]]
    sims = [j.sim for j in jobs]
    sims[4].maxdetphotons = 50  # fewer rows than detections
    b = Batch.from_jobs(ctx, jobs, sims=sims)
    tot = b.run()
    assert tot.status == 0 and tot.launched == sum(s.nphoton for s in sims)
    assert tot.detected >= tot.saved > 0
    detected = saved = 0
    for i, (j, s) in enumerate(zip(jobs, sims)):
        _, r = b.get(i)
        rows = b.detp(i)
        detected += r.detected
        saved += r.saved
        if not s.issavedet:
            assert r.detected == 0 and r.saved == 0 and rows.shape[0] == 0
            continue
        single = ctx.forward(s, j.labels, j.media, j.detpos)
        n1, n2 = r.detected, single.result.detected
        assert abs(n1 - n2) <= max(3, n2 // 500), (i, n1, n2)
        assert r.saved == min(r.detected, s.maxdetphotons) == rows.shape[0]
        assert rows.shape[1] == single.detp.shape[1]
        if s.maxdetphotons < n2:
            continue
        assert np.all((rows[:, 0] >= 1) & (rows[:, 0] <= s.detnum))
        for d, (a, c) in enumerate(zip(detector_rows_by_id(rows, s.detnum),
                                       detector_rows_by_id(single.detp, s.detnum))):
            assert abs(len(a) - len(c)) <= max(3, len(c) // 500), (i, d, len(a), len(c))
            if len(c) > 20:
                pa, pc = a[:, 1:1 + s.mediumnum].mean(0), c[:, 1:1 + s.mediumnum].mean(0)
                np.testing.assert_allclose(pa, pc, rtol=2e-2, atol=1e-3 * max(1.0, float(pc.max())))
    assert (detected, saved) == (tot.detected, tot.saved)
    b.close()


def test_batched_detected_photons_match_oracle(ctx):
    """Detected-photon records of the batched kernel against the CPU oracle on the same seeds: the heterogeneous
    60^3 + sphere geometry with reflection and 4 detectors (4e5 photons) and cube60b (2e5 photons), each entering
    the batch as 10 photon-index ranges between simulations that save no records.  Criteria of the
    single-simulation parity test: detection counts (in all and per detector) within 3 standard errors, every
    per-detector mean partial path within 3 standard errors, absorbed fraction within 3 standard errors."""
    import oracle
    from statcheck import det_stats, run_batches, z_of_means

    from umcx_gb300 import Job
    from umcx_gb300.api import Batch

    specs = [(["--bench", "cubesph60b"], 400000), (["--bench", "cube60b"], 200000)]
    nb = 10
    fillers = small_batch(nb * len(specs), scale=0.005)
    entries, sims, base = [], [], []
    for q, (args, n) in enumerate(specs):
        j = Job.from_args([*args, "-n", str(n)])
        base.append(j)
        per = n // nb
        for k in range(nb):
            t = j.sim.copy()
            t.photon_offset = k * per
            t.nphoton = per
            entries.append(j)
            sims.append(t)
            f = fillers[q * nb + k]
            entries.append(f)
            sims.append(f.sim)
    b = Batch.from_jobs(ctx, entries, sims=sims)
    tot = b.run()
    assert tot.status == 0 and tot.launched == sum(s.nphoton for s in sims)
    for q, j in enumerate(base):
        s = j.sim
        it = iter(range(2 * q * nb, 2 * (q + 1) * nb, 2))

        def gpu(_s):
            i = next(it)
            flu, r = b.get(i)
            return flu, b.detp(i), r

        g = run_batches(gpu, s, nb)
        c = run_batches(lambda _s: oracle.forward(_s, j.labels, j.media, j.detpos), s, nb)
        za = z_of_means(g.absorbed, c.absorbed)
        ng = sum(r.detected for r in g.results)
        nc = sum(r.detected for r in c.results)
        zd = (ng - nc) / math.sqrt(ng + nc)
        line = f"{s.dim[0]}^3, {s.detnum} detectors: absorbed z={za:.2f}; detected gpu {ng} cpu {nc} z={zd:.2f}"
        assert abs(za) < 3 and abs(zd) < 3 and ng > 100, line
        cols = slice(1, 1 + s.mediumnum)
        zmax = 0.0
        for (n1, m1, s1), (n2, m2, s2) in zip(det_stats(g.detp, s.detnum, cols), det_stats(c.detp, s.detnum, cols)):
            zn = (n1 - n2) / math.sqrt(n1 + n2) if n1 + n2 else 0.0
            assert abs(zn) < 3, (line, n1, n2)
            if n1 > 30 and n2 > 30:
                z = (m1 - m2) / np.sqrt(s1 ** 2 + s2 ** 2 + 1e-30)
                z = z[np.isfinite(z)]
                zmax = max(zmax, float(np.abs(z).max()) if z.size else 0.0)
                assert np.all(np.abs(z) < 3), (line, m1, m2, z)
        print(line + f"; per-detector mean partial path max |z| {zmax:.2f}")
    for i in range(1, len(sims), 2):  # the fillers save no records
        _, r = b.get(i)
        assert r.detected == 0 and b.detp(i).shape[0] == 0
    b.close()


def test_autotuners(ctx):
    import torch

    from umcx_gb300 import Job
    from umcx_gb300.api import autotune_batch

    job = Job.from_args(["--bench", "cubesph60b", "-n", "2e5"])
    s = job.sim
    d_lab = torch.from_numpy(job.labels.ravel().copy()).cuda()
    d_flu = torch.zeros(s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3], dtype=torch.float32, device="cuda")
    d_det = torch.zeros(s.maxdetphotons * 4, dtype=torch.float32, device="cuda")
    best = ctx.autotune(s, d_lab, job.media, job.detpos, d_flu, d_det, fraction=0.2)
    assert best["block_size"] in (128, 256, 512, 1024) and best["probe_ms"] > 0
    ctx.set_tuning()
    bb = autotune_batch(ctx, small_batch(4, scale=0.01), fraction=1.0, candidates=((256, 1), (512, 2)))
    assert bb["block_size"] in (256, 512)


def test_batch_outputs_into_caller_buffer(ctx):
    from umcx_gb300.api import Batch

    jobs = small_batch(4, scale=0.01)
    b = Batch.from_jobs(ctx, jobs)
    b.run()
    biggest = max(j.sim.dim[0] * j.sim.dim[1] * j.sim.dim[2] * j.sim.dim[3] for j in jobs)
    out = np.full(biggest, -1.0, np.float32)
    for i in range(len(jobs)):
        ref, r_ref = b.get(i)
        got, r_got = b.get(i, out=out)
        assert got.base is not None and np.shares_memory(got, out)
        np.testing.assert_array_equal(got, ref)
        assert r_got.energy_total == r_ref.energy_total
    with pytest.raises(ValueError):
        b.get(0, out=np.zeros(10, np.float32))
    b.close()


def test_batch_budget_stops_kernel_and_context_survives(ctx):
    """A batch whose launch outlives its wall-clock budget stops with status 3 (no hang, no fault); the batch can be
    re-tuned with a normal budget and run to completion, and the context stays usable."""
    from umcx_gb300.api import Batch

    jobs = small_batch(8, scale=0.5)
    b = Batch.from_jobs(ctx, jobs)
    b.set_tuning(1024, 0, 1, 1)  # 1 ms
    with pytest.raises(RuntimeError, match="status 3.*budget"):
        b.run()
    b.set_tuning(1024, 0, 1, 0)
    r = b.run()
    assert r.status == 0 and r.launched == sum(j.sim.nphoton for j in jobs)
    b.close()


def stratified_subset():
    """Indices of the 256-simulation workload covering every (edge, source type) stratum, alternating 2 and 5
    tissue labels, plus one simulation with 3 and one with 4 labels."""
    from umcx_gb300.workloads import EDGES, config5

    cfgs = [config5(i) for i in range(256)]
    info = [(c["Domain"]["Dim"][0], c["Optode"]["Source"]["Type"], len(c["Domain"]["Media"]) - 1) for c in cfgs]
    picked = []
    for k, (edge, stype) in enumerate((e, t) for e in EDGES for t in ("pencil", "isotropic")):
        want = 2 if k % 2 == 0 else 5
        cands = [i for i, (e, t, n) in enumerate(info) if e == edge and t == stype]
        exact = [i for i in cands if info[i][2] == want]
        picked.append((exact or cands)[0])
    for nlab in (3, 4):
        picked.append(next(i for i, (e, t, n) in enumerate(info) if n == nlab and i not in picked and e <= 64))
    return picked


def test_batched_form_matches_oracle(ctx):
    """The batched kernel against the CPU oracle on the same seeds, for a stratified subset of the 256-simulation
    workload (every domain edge, pencil and isotropic sources, 2 to 5 labels) at 1e5 photons each.  Each
    simulation enters the batch as 10 photon-index ranges, so that both sides have batch standard errors; the
    criteria are those of the single-simulation parity test: absorbed fraction within 3 standard errors, and over
    voxels with at least 100 deposits at most frac_over3_limit(10) (2.3 %) beyond 3 standard errors, mean z^2 below
    1.5, |mean z| below 0.2."""
    import oracle
    from statcheck import compare_fluence, run_batches, z_of_means
    from test_forward_gpu import frac_over3_limit

    from umcx_gb300.api import Batch
    from umcx_gb300.workloads import batch5

    idx = stratified_subset()
    all_jobs = batch5(max(idx) + 1)
    jobs = [all_jobs[i] for i in idx]
    nb, photons = 10, 100000
    per = photons // nb
    entries, sims = [], []
    for j in jobs:
        s = j.sim
        s.nphoton = photons
        for k in range(nb):
            t = s.copy()
            t.photon_offset = k * per
            t.nphoton = per
            entries.append(j)
            sims.append(t)
    b = Batch.from_jobs(ctx, entries, sims=sims)
    tot = b.run()
    assert tot.status == 0 and tot.launched == nb * per * len(jobs)
    for q, (i, j) in enumerate(zip(idx, jobs)):
        s = j.sim
        s.nphoton = photons
        it = iter(range(q * nb, (q + 1) * nb))
        g = run_batches(lambda _s: (lambda fr: (fr[0], None, fr[1]))(b.get(next(it))), s, nb)
        c = run_batches(lambda _s: oracle.forward(_s, j.labels, j.media, None, depcount=True), s, nb)
        zt = z_of_means(g.total, c.total)
        assert abs(zt) < 3 or abs(g.total.sum() - c.total.sum()) <= 1e-6 * c.total.sum(), (i, zt)
        za = z_of_means(g.absorbed, c.absorbed)
        fc = compare_fluence(g, c, c.depcount)
        line = (f"sim {i} (edge {s.dim[0]}, {s.mediumnum - 1} labels, src {s.srctype}): absorbed gpu "
                f"{g.absorbed.mean():.5f} cpu {c.absorbed.mean():.5f} z={za:.2f}; voxels {fc.tested}, |z|>3 "
                f"{fc.frac_over3:.4f}, max |z| {fc.max_abs_z:.2f}, mean z^2 {fc.mean_z2:.3f}, rel L2 {fc.rel_l2:.2e}")
        print(line)
        assert abs(za) < 3, line
        if fc.tested:
            assert fc.frac_over3 <= frac_over3_limit(nb) and fc.mean_z2 < 1.5 and abs(fc.mean_z) < 0.2, line
    b.close()
