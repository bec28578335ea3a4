"""Parity of the CUDA forward path with the CPU oracle on the same inputs and seeds (GPU required).

Parity tolerances, as asserted below:
  * energy: absorbed (the summed energy volume) + escaped = launched, to 1e-5 relative;
  * absorbed fraction, launched energy, detected-photon count: within 3 standard errors (photon-index batches);
  * per-detector mean partial pathlength of every label: within 3 standard errors (pooled detected rows);
  * voxel fluence, over voxels with at least 100 deposits: the fraction beyond 3 standard errors at most three times
    what chance gives for independent samples with batch standard errors (Student's t, frac_over3_limit: 1.4 % at 20
    batches; the oracle and the GPU share photon seeds, which makes the differences smaller still), mean z^2 below
    1.5 and |mean z| below 0.2; the normalised L2 difference and the largest |z| are printed for every case.
Standard errors come from photon-index batches of each run.  The benchmark configurations run at their own photon
counts (configuration 1 at 1e6, configuration 2 at 1e7, configuration 3 at 1e7 against its 1e8)."""
import json
import math
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import C1, C2, C3, SHAPES  # noqa: E402
from statcheck import compare_fluence, det_stats, run_batches, z_of_means  # noqa: E402

pytestmark = pytest.mark.gpu


def job_for(spec, photons):
    from umcx_gb300 import Job

    if isinstance(spec, dict):
        cfg = json.loads(json.dumps(spec))
        cfg["Session"]["Photons"] = int(photons)
        return Job.from_args(["-j", json.dumps(cfg)])
    return Job.from_args([*spec, "-n", str(int(photons))])


def gpu_runner(ctx, job):
    def fn(s):
        out = ctx.forward(s, job.labels, job.media, job.detpos)
        return out.fluence, out.detp, out.result
    return fn


def cpu_runner(job, depcount=False):
    import oracle

    def fn(s):
        return oracle.forward(s, job.labels, job.media, job.detpos, depcount=depcount)
    return fn


def frac_over3_limit(nbatch: int) -> float:
    """Largest accepted fraction of tested voxels beyond 3 standard errors: three times what chance gives for
    independent samples, whose z follows Student's t with 2 (nbatch - 1) degrees of freedom when both standard
    errors come from nbatch batches (0.47 % at 20 batches, 0.77 % at 10), and at least 1 %."""
    from scipy.stats import t

    return max(0.01, 3 * 2 * float(t.sf(3.0, 2 * (nbatch - 1))))


def with_output(spec, otype):
    cfg = json.loads(json.dumps(spec))
    cfg["Session"]["OutputType"] = otype
    return cfg


def with_window(spec, t0, t1, dt):
    """The same simulation with another time window: with t0 > 0 the deposits of the first nanoseconds fall before
    the first gate and are skipped by both sides (the reference writes them before its array)."""
    cfg = json.loads(json.dumps(spec))
    cfg["Forward"] = {"T0": t0, "T1": t1, "Dt": dt}
    return cfg


CASES = {
    "c1": (C1, 1000000, 20),
    "c2": (C2, 10000000, 20),
    "c3": (C3, 10000000, 10),
    "c1_fluence": (with_output(C1, "f"), 1000000, 20),
    "c2_fluence": (with_output(C2, "f"), 1000000, 20),
    "c2_late_window": (with_window(C2, 1e-9, 5e-9, 1e-10), 1000000, 20),
    "cube60b": (["--bench", "cube60b"], 200000, 20),
    "spherebox": (["--bench", "spherebox"], 100000, 20),
    "sphshells": (["--bench", "sphshells"], 50000, 10),
    "planar": (["--bench", "cube60planar"], 100000, 20),
    "isotropic": (["--bench", "cube60", "--json", '{"Optode":{"Source":{"Type":"isotropic","Pos":[29,29,29]}}}'],
                  20000, 10),
    "cone": (["--bench", "cube60b", "--json", '{"Optode":{"Source":{"Type":"cone","Param1":[0.5,0,0,0]}}}'],
             100000, 20),
    "fourier": (["--bench", "cube60planar", "--json",
                 '{"Optode":{"Source":{"Type":"fourier","Param1":[40,0,0,2.25],"Param2":[0,40,0,1.5]}}}'],
                100000, 20),
    "shapes": (SHAPES, 50000, 10),
    # sources outside the grid: every photon is moved onto it first (MCX_photon::skip, L339-358, weight reset to 1),
    # and most of the wide cone's photons miss it (counted as launched, nothing else, L263-266)
    "outside_pencil": (["--bench", "cube60", "--json", '{"Optode":{"Source":{"Pos":[29.5,29.5,-10]}}}'], 100000, 20),
    "outside_cone": (["--bench", "cube60", "--json",
                      '{"Optode":{"Source":{"Type":"cone","Pos":[29.5,29.5,-20],"Param1":[0.9,0,0,0]}}}'], 200000, 20),
}


@pytest.mark.parametrize("name", list(CASES))
def test_forward_parity(ctx, name):
    spec, n, nb = CASES[name]
    job = job_for(spec, n)
    sim = job.sim
    g = run_batches(gpu_runner(ctx, job), sim, nb)
    c = run_batches(cpu_runner(job, depcount=bool(sim.issavevol)), sim, nb)
    # every launched photon is processed exactly once
    assert sum(r.launched for r in g.results) == sim.nphoton
    assert all(r.status == 0 and r.capped == 0 for r in g.results)
    # launch weights depend only on the photon streams
    zt = z_of_means(g.total, c.total)
    assert abs(zt) < 3 or abs(g.total.sum() - c.total.sum()) <= 1e-6 * c.total.sum(), (g.total.sum(), c.total.sum())
    za = z_of_means(g.absorbed, c.absorbed)
    line = f"{name} ({sim.nphoton} photons): absorbed gpu {g.absorbed.mean():.6f} cpu {c.absorbed.mean():.6f} z={za:.2f}"
    assert abs(za) < 3, line
    if sim.issavevol:
        fc = compare_fluence(g, c, c.depcount)
        line += (f"; fluence voxels tested {fc.tested}, |z|>3 {fc.frac_over3:.4f}, max |z| {fc.max_abs_z:.2f}, "
                 f"mean z {fc.mean_z:.3f}, mean z^2 {fc.mean_z2:.3f}, rel L2 {fc.rel_l2:.2e}")
        if fc.tested:
            assert fc.frac_over3 <= frac_over3_limit(nb) and fc.mean_z2 < 1.5 and abs(fc.mean_z) < 0.2, line
    if sim.issavedet and sim.detnum:
        ng = sum(r.detected for r in g.results)
        nc = sum(r.detected for r in c.results)
        zd = (ng - nc) / math.sqrt(ng + nc) if ng + nc else 0.0
        line += f"; detected gpu {ng} cpu {nc} z={zd:.2f}"
        assert abs(zd) < 3, line
        if sim.savedetflag & 4 and sim.savedetflag & 1:
            cols = slice(1, 1 + sim.mediumnum)
            zmax = 0.0
            for (n1, m1, s1), (n2, m2, s2) in zip(det_stats(g.detp, sim.detnum, cols),
                                                  det_stats(c.detp, sim.detnum, cols)):
                zn = (n1 - n2) / math.sqrt(n1 + n2) if n1 + n2 else 0.0
                assert abs(zn) < 3, (name, n1, n2)
                if n1 > 30 and n2 > 30:
                    z = (m1 - m2) / np.sqrt(s1 ** 2 + s2 ** 2 + 1e-30)
                    z = z[np.isfinite(z)]
                    zmax = max(zmax, float(np.abs(z).max()) if z.size else 0.0)
                    assert np.all(np.abs(z) < 3), (name, m1, m2, z)
            line += f"; per-detector mean partial path max |z| {zmax:.2f}"
    print(line)


def test_detected_exit_records_match_oracle(ctx):
    """Detected-photon rows with every SaveDetFlag column -- detector id, partial paths, exit position and exit
    direction (MCX_photon::savedetector, src/umcx.cpp:429-435; row layout L171-174): per detector the count and the
    mean of every partial-path, position and direction column agree with the oracle within 3 standard errors, or to
    within 1e-5 (voxel units, direction components) for a column without spread -- the exit coordinate of the z = 0
    face, which both sides reach within a float rounding of 0; every exit point lies within its detector's radius (the
    detection test, L430-431) and every exit direction is a unit vector leaving through the z = 0 face that holds the
    detectors."""
    cfg = json.loads(json.dumps(C2))
    cfg["Session"]["SaveDetFlag"] = 1 + 4 + 16 + 32
    job = job_for(cfg, 1000000)
    sim = job.sim
    g = run_batches(gpu_runner(ctx, job), sim, 20)
    c = run_batches(cpu_runner(job), sim, 20)
    k = sim.mediumnum
    groups = {"partial path": slice(1, 1 + k), "exit position": slice(1 + k, 4 + k),
              "exit direction": slice(4 + k, 7 + k)}
    line = "exit records:"
    for name, cols in groups.items():
        zmax = 0.0
        for d, ((n1, m1, s1), (n2, m2, s2)) in enumerate(zip(det_stats(g.detp, sim.detnum, cols),
                                                             det_stats(c.detp, sim.detnum, cols))):
            zn = (n1 - n2) / math.sqrt(n1 + n2) if n1 + n2 else 0.0
            assert abs(zn) < 3, (name, d, n1, n2)
            if n1 > 30 and n2 > 30:
                z = (m1 - m2) / np.sqrt(s1 ** 2 + s2 ** 2 + 1e-30)
                keep = np.isfinite(z) & (np.abs(m1 - m2) >= 1e-5)  # a spread-free column only has to agree to 1e-5
                assert np.all(np.abs(z[keep]) < 3), (name, d, m1, m2, z)
                zmax = max(zmax, float(np.abs(z[keep]).max()) if keep.any() else 0.0)
        line += f" {name} max |z| {zmax:.2f};"
    rows = np.concatenate([r for r in g.detp if r is not None and len(r)], axis=0)
    assert rows.shape[1] == 7 + k and len(rows) > 1000
    det = np.asarray(job.detpos, dtype=np.float64).reshape(-1, 4)
    centre = det[rows[:, 0].astype(int) - 1]
    dist = np.linalg.norm(rows[:, 1 + k:4 + k] - centre[:, :3], axis=1)
    assert np.all(dist < centre[:, 3] + 1e-4), dist.max()
    v = rows[:, 4 + k:7 + k]
    assert np.all(np.abs(np.linalg.norm(v, axis=1) - 1.0) < 1e-4) and np.all(v[:, 2] < 0.0)
    print(line + f" {len(rows)} rows, largest distance to the detector centre {dist.max():.3f} (radius 1)")


@pytest.mark.parametrize("name,spec,photons", [
    ("c1", C1, 10000000),    # configuration 1 geometry at 10x its photon count
    ("c2", C2, 1000000),
    ("c3", C3, 100000000),   # configuration 3 at its own photon count: 8 M voxels, ~2.7e10 deposits
])
def test_energy_conservation(ctx, name, spec, photons):
    """Absorbed (the summed FP32 energy volume) + escaped = launched, to 1e-5 relative."""
    cfg = json.loads(json.dumps(spec))
    cfg["Session"].update({"OutputType": "e", "Photons": photons})
    job = job_for(cfg, photons)
    out = ctx.forward(job.sim, job.labels, job.media, job.detpos)
    r = out.result
    absorbed = float(out.fluence.astype(np.float64).sum())
    rel = abs(absorbed + r.energy_escape - r.energy_total) / r.energy_total
    print(f"energy {name}: launched {r.energy_total:.3f} absorbed {absorbed:.3f} escaped {r.energy_escape:.3f} "
          f"rel {rel:.2e}")
    assert r.status == 0 and r.launched == photons
    assert rel < 1e-5


def test_launch_shape_flags_on_gpu(ctx):
    """-T 256 -t 25600 (BlockSize / ThreadNum, src/umcx.cpp:739-741) launch 100 CTAs of 256 threads; every photon's
    history depends only on its index, so the event counts equal those of the default launch exactly."""
    job = job_for(["--bench", "cubesph60b", "-T", "256", "-t", "25600"], 200000)
    assert job.tuning == {"block_size": 256, "grid_size": 100}
    base = ctx.forward(job.sim, job.labels, job.media, job.detpos).result
    ctx.set_tuning(**job.tuning)
    try:
        r = ctx.forward(job.sim, job.labels, job.media, job.detpos).result
    finally:
        ctx.set_tuning()
    assert (r.block_size, r.grid_size) == (256, 100)
    assert base.block_size == 1024 and base.grid_size > 100
    assert (r.launched, r.steps, r.crossings, r.scatters, r.reflections, r.detected) == (
        base.launched, base.steps, base.crossings, base.scatters, base.reflections, base.detected)
    assert abs(r.energy_escape - base.energy_escape) <= 1e-9 * base.energy_total


def test_fp32_accumulation_mode(ctx):
    """Reference-style FP32 atomic accumulation (UMCX_SIM_FP32_ACCUM) gives the same volume within FP32 rounding
    at a small photon count, and loses energy only at the level the reference does."""
    from umcx_gb300._lib import SIM_FP32_ACCUM

    cfg = json.loads(json.dumps(C2))
    cfg["Session"].update({"OutputType": "e"})
    job = job_for(cfg, 100000)
    s64 = job.sim
    s32 = job.sim
    s32.flags = SIM_FP32_ACCUM
    a = ctx.forward(s64, job.labels, job.media, job.detpos)
    b = ctx.forward(s32, job.labels, job.media, job.detpos)
    assert a.result.steps == b.result.steps and a.result.detected == b.result.detected
    np.testing.assert_allclose(b.fluence, a.fluence, rtol=1e-3, atol=1e-6)
    r = b.result
    rel = abs(float(b.fluence.astype(np.float64).sum()) + r.energy_escape - r.energy_total) / r.energy_total
    assert rel < 1e-4


def test_rng_bit_exact(ctx):
    import oracle

    seeds = oracle.seeds(1648335518)
    base = (1 << 32) - 64  # crosses the 32-bit truncation of the photon index
    gpu = ctx.rng_dump(seeds, base, 128, 40)
    for k in range(128):
        assert np.array_equal(gpu[k], oracle.rng_dump(seeds, base + k, 40)), k
    gpu0 = ctx.rng_dump(seeds, 0, 1000, 8)
    for k in (0, 1, 2, 31, 32, 999):
        assert np.array_equal(gpu0[k], oracle.rng_dump(seeds, k, 8))


def test_strict_math_tracks_oracle(ctx):
    """The strict kernel (reference expression forms, no FMA contraction) reproduces most photons' outcomes:
    its absorbed fraction agrees with the oracle far inside the statistical error."""
    import oracle
    from umcx_gb300._lib import SIM_STRICT_MATH

    job = job_for(["--bench", "cube60b"], 100000)
    s = job.sim
    s.flags = SIM_STRICT_MATH
    g = ctx.forward(s, job.labels, job.media, job.detpos)
    _, _, r, _ = oracle.forward(job.sim, job.labels, job.media, job.detpos)
    a_g = g.absorbed_fraction
    a_c = (r.energy_total - r.energy_escape) / r.energy_total
    se = math.sqrt(a_c * (1 - a_c) / s.nphoton)
    print(f"strict: gpu {a_g:.7f} cpu {a_c:.7f} diff/se {(a_g - a_c) / se:.4f}")
    assert abs(a_g - a_c) < 0.5 * se


def test_device_buffers_match_host_api(ctx):
    import torch

    job = job_for(C2, 50000)
    s = job.sim
    host = ctx.forward(s, job.labels, job.media, job.detpos)
    d_lab = torch.from_numpy(job.labels.ravel().copy()).cuda()
    d_flu = torch.zeros(host.fluence.size, dtype=torch.float32, device="cuda")
    d_det = torch.zeros(s.maxdetphotons * 4, dtype=torch.float32, device="cuda")
    r = ctx.forward_device(s, d_lab, job.media, job.detpos, d_flu, d_det, torch.cuda.current_stream())
    assert r.detected == host.result.detected and r.steps == host.result.steps
    assert abs(r.energy_escape - host.result.energy_escape) < 1e-9 * host.result.energy_total
    np.testing.assert_allclose(d_flu.cpu().numpy().reshape(host.fluence.shape), host.fluence, rtol=2e-5, atol=1e-6)


def test_budget_stops_kernel_and_context_survives(ctx):
    job = job_for(["--bench", "cube60b"], 200000000)
    ctx.set_tuning(budget_ms=20)
    try:
        with pytest.raises(RuntimeError, match="status 3.*budget"):
            ctx.forward(job.sim, job.labels, job.media, job.detpos)
    finally:
        ctx.set_tuning()
    small = job_for(["--bench", "cube60b"], 10000)
    out = ctx.forward(small.sim, small.labels, small.media, small.detpos)
    assert out.result.status == 0 and out.result.launched == 10000


@pytest.mark.parametrize("args,lo,hi,det", [
    (["--bench", "cube60", "-S", "0"], 17, 18, None),                        # test/testumcx.sh:60-62
    (["--bench", "cube60b", "-S", "0"], 27, 28, None),                       # :64-66
    (["--bench", "cube60", "-b", "1", "-S", "0"], 27, 28, None),             # :68-70
    (["--bench", "cube60b"], 0, 100, (4000, 4999)),                          # :80-82 detected 4xxx
    (["--bench", "cube60planar"], 25, 26, None),                             # :84-86
    (["--bench", "cube60", "--json", '{"Optode":{"Source":{"Type":"isotropic","Pos":[29,29,29]}}}', "-d", "0",
      "-S", "0"], 88, 89, None),                                             # :88-90
    (["--bench", "cube60", "--json",
      '{"Domain":{"Media":[[0,0,1,1],[0.001,0.001,0,1]]},"Optode":{"Source":{"Type":"cone","Param1":[0.5,0,0,0]}}}',
      "-d", "0", "-S", "0"], 6, 7, None),                                    # :92-94
    (["--bench", "skinvessel", "-S", "0", "-n", "1e5"], 39, 40, None),      # :112-114
    (["--bench", "spherebox", "-S", "0"], 10, 12, None),                     # :130-132
])
def test_reference_known_answers_on_gpu(args, lo, hi, det, tmp_path):
    """The reference's own regression checks (test/testumcx.sh), run through the GPU CLI."""
    import oracle

    cli = ROOT / "umcx_gb300" / "_build" / "umcx"
    p = subprocess.run([str(cli), *args], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    line = oracle.parse_line(p.stdout)
    assert line is not None, p.stdout
    assert lo <= line["absorbed"] < hi, line
    if det:
        assert det[0] <= line["detected"] <= det[1], line


def test_cli_outputs_have_reference_layout(tmp_path):
    import oracle

    cli = ROOT / "umcx_gb300" / "_build" / "umcx"
    p = subprocess.run([str(cli), "--bench", "cubesph60b", "-n", "1e5", "-s", "o"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout
    line = oracle.parse_line(p.stdout)
    vol = oracle.read_bjdata(tmp_path / "o.bnii")
    assert vol["NIFTIHeader"]["Dim"] == [60, 60, 60, 1]
    assert vol["NIFTIData"].shape == (60, 60, 60, 1) and vol["NIFTIData"].dtype == np.float32
    det = oracle.read_bjdata(tmp_path / "o_detp.jdb")
    info = det["MCXData"]["Info"]
    assert info["ColumnNum"] == 4 and info["TotalPhoton"] == 4 and info["SavedPhoton"] == line["detected"]
    rows = det["MCXData"]["PhotonRawData"]
    assert rows.shape == (line["detected"], 4)
    assert set(np.unique(rows[:, 0])) <= {1.0, 2.0, 3.0, 4.0}
    assert np.all(rows[:, 3] == 0)  # the last partial-path column is always zero (ppath index = label - 1)


def test_mcx_run_json_entry(tmp_path, monkeypatch):
    import ctypes as C

    from umcx_gb300 import load

    cfg = json.loads(json.dumps(C2))
    cfg["Session"].update({"ID": "rj", "Photons": 20000})
    monkeypatch.chdir(tmp_path)
    assert load().MCX_run_json(json.dumps(cfg).encode()) == 0
    assert (tmp_path / "rj.bnii").exists() and (tmp_path / "rj_detp.jdb").exists()
    assert load().MCX_run_json(b'{"Session":{}}') != 0


def test_caller_owned_output_arrays(ctx):
    """Context.forward writes into output arrays the caller reuses from call to call (stale contents overwritten)."""
    job = job_for(C2, 20000)
    s = job.sim
    ref = ctx.forward(s, job.labels, job.media, job.detpos)
    nout = s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3]
    flu = np.full(nout, 7.0, np.float32)
    dp = np.full(s.maxdetphotons * ref.detp.shape[1], 7.0, np.float32)
    for _ in range(2):
        out = ctx.forward(s, job.labels, job.media, job.detpos, fluence=flu, detp=dp)
        assert np.shares_memory(out.fluence, flu)
        assert out.result.steps == ref.result.steps and out.result.detected == ref.result.detected
        np.testing.assert_allclose(out.fluence, ref.fluence, rtol=1e-5, atol=1e-7)
    with pytest.raises(ValueError):
        ctx.forward(s, job.labels, job.media, job.detpos, fluence=np.zeros(10, np.float32))
