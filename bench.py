"""Benchmark of the umcx photon-transport hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--photons P] [--forms LIST]

Headline workload (configuration 2): the heterogeneous forward configuration with refractive mismatch and
detectors -- 60x60x60 voxels of 1 mm, background label 1 (mua 0.005/mm, mus 1/mm, g 0.01, n 1.37), a radius-15
sphere of label 2 (mua 0.002, mus 5, g 0.9, n 1.0) centred at (30,30,30), pencil source at (29,29,0) along +z,
boundary reflection on, 1e7 photons per step, 50 time gates over 0-5 ns, four disk detectors of radius 1 mm at
z = 0 with partial pathlengths saved.  Synthetic input (the configuration is generated, not read from a dataset).

One step = one full simulation of P photons.  `value` is photons/ms of the propagation kernel with the inputs
resident in HBM (CUDA events on the launching stream; the output volume is cleared inside the step and the L2 is
flushed by writing a 256 MB buffer between steps).  `e2e` is the same metric through the C ABI call with host
buffers in page-locked memory (umcx_gpu_forward: label upload, simulation, fluence + detected-photon download),
timed on the host.  Under torchrun (N > 1) every rank simulates its own photon range of one N x P-photon
simulation and the ranks sum the output volume and the tallies on the GPU and gather the detected rows inside the
timed step (umcx_gb300.shard): weak scaling.

`forms` (rank 0, N = 1 sizes) measures the other configurations the same way, each with its device time, end-to-end
time and roofline fractions: configuration 1 at its 1e6 photons, the reference's own published benchmark cube60
(configuration 1 plus four saved detectors, 1e8 photons), configuration 3 at 1e8 photons, the forward + adjoint form
(configuration 4) and the batched form (configuration 5, 256 simulations at their full photon budgets, against the
same simulations as sequential single launches).

--impl reference times the reference's own CPU implementation (the unmodified reference program built from its
sources, oracle/_ref/umcx, with all host threads; else the C restatement in oracle/) on a bounded photon sample of
the same configuration.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from umcx_gb300.workloads import config1, config2, config3  # noqa: E402

CONFIG = config2()
WORKLOAD = "heterogeneous forward, 60^3 grid, sphere R15, reflection on, 50 gates, 4 detectors (ppath saved)"
METRIC = "photons/ms (forward, heterogeneous 60^3 + sphere, reflection, 50 gates, 4 detectors)"

# per workload: the input, its photons per step, timed steps of a `forms` entry, and what an ncu capture of the
# propagation kernel on the same build measured (profiles/): warp instructions issued per voxel step
# (smsp__inst_executed.sum / steps) and DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch at
# that photon count.  None where no capture exists; the line then reports null for those fractions.
FORWARD = {
    "c2": {"json": CONFIG, "photons": 10000000, "workload": WORKLOAD,
           # profiles/k_forward_workloads.md: 3.7381e10 warp instructions / 3.4359e9 steps; 93.3 MB + 3.065 GB
           "warp_inst_per_step": 10.88, "dram_bytes": 93255680 + 3065493760},
    "c1": {"json": config1(), "photons": 1000000, "steps": 20,
           "workload": "homogeneous 60^3 cube, pencil beam, one 5 ns gate, no reflection (configuration 1)",
           # 3.8693e9 / 1.9618e8 steps (at 1e6 photons the launch's drain is a large share); 13.9 MB read
           "warp_inst_per_step": 19.72, "dram_bytes": 13939968},
    "cube60": {"args": ["--bench", "cube60"], "photons": 100000000, "steps": 5,
               "workload": "the reference's cube60 benchmark: configuration 1 plus four saved detectors, 1e8 photons "
                           "(published: 175 075 photons/ms on an RTX 5090)",
               # 1.7139e11 / 1.9626e10 steps; 14.1 MB read (the 1.7 MB FP64 volume stays in L2)
               "warp_inst_per_step": 8.733, "dram_bytes": 14073856 + 1536},
    "c3": {"json": config3(), "photons": 100000000, "steps": 5,
           "workload": "200^3 layered domain of 0.005 mm voxels with a cylinder, disk source, 1 ns gate (configuration 3)",
           # 2.6523e11 / 2.9111e10 steps; 69.4 MB read + 10.9 GB of FP64 accumulator lines written back
           "warp_inst_per_step": 9.111, "dram_bytes": 69378560 + 10894940160},
}

# per-event FP32 and SFU-class operation counts (FMA = 1 op), fixed from the reference's formulas:
# step L316-337, scatter L364-380, voxel crossing / deposit L285-310, reflect L381-417
OPS_FP32 = {"steps": 26, "scatters": 45, "crossings": 8, "reflections": 25}
OPS_SFU = {"steps": 2, "scatters": 9, "crossings": 1, "reflections": 2}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region.  nvidia-smi writes its samples straight into a
    temporary file (no reader thread in this process, so sampling never competes with the timed loop for the
    interpreter)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.out = None

    def start(self):
        try:
            self.out = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.out, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.seek(0)
        self.lines = [ln.strip() for ln in self.out]
        self.out.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference_run(photons: int, threads: int) -> dict:
    """Run the reference's CPU implementation on the benchmark configuration; returns photons/ms and details."""
    import oracle

    cfg = json.loads(json.dumps(CONFIG))
    cfg["Session"]["Photons"] = int(photons)
    cfg["Session"]["DoSaveVolume"] = 1
    if oracle.have_reference():
        with tempfile.TemporaryDirectory() as d:
            t0 = time.perf_counter()
            r = oracle.run_reference(["-j", json.dumps(cfg)], d, threads=threads, timeout=900)
            wall = time.perf_counter() - t0
        if r.get("returncode") == 0 and "speed" in r:
            return {"value": r["speed"], "kind": "reference", "wall_s": wall, "duration_ms": r["duration_ms"],
                    "absorbed": r["absorbed"], "detected": r["detected"]}
    from umcx_gb300 import Job

    job = Job.from_json(cfg)
    t0 = time.perf_counter()
    _, _, res, _ = oracle.forward(job.sim, job.labels, job.media, job.detpos, nthreads=threads)
    ms = (time.perf_counter() - t0) * 1e3
    return {"value": photons / ms, "kind": "port", "wall_s": ms / 1e3, "duration_ms": ms,
            "absorbed": (res.energy_total - res.energy_escape) / res.energy_total * 100, "detected": int(res.saved)}


def run_reference_arm(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle

    try:
        oracle.build(reference_root=None)  # rebuilds the reference program from its staged sources when needed
    except Exception:
        pass
    threads = os.cpu_count() or 1
    photons = args.cpu_photons
    for _ in range(args.warmup):
        cpu_reference_run(max(photons // 10, 10000), threads)
    vals, walls, info = [], [], None
    for _ in range(args.steps):
        info = cpu_reference_run(photons, threads)
        vals.append(info["value"])
        walls.append(info["wall_s"])
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "photons/ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(walls),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (generated configuration)",
        "config": {"workload": WORKLOAD, "photons_per_step": photons, "threads": threads,
                   "photons_per_step_of_the_gpu_arm": int(CONFIG["Session"]["Photons"]),
                   "sample": "a bounded sample of the same simulation per step: at the CPU's rate the GPU arm's "
                             "1e7 photons would take about 15 s per step; photons/ms does not depend on the count "
                             "(1e6 photons gave the same rate)",
                   "program": "reference umcx CPU OpenMP build" if info["kind"] == "reference" else "oracle C port"},
        "cpu_baseline": {"value": value, "unit": "photons/ms", "cores": threads, "kind": info["kind"],
                         "sample": f"{photons} photons of the benchmark configuration per step"},
        "e2e": {"value": value, "unit": "photons/ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
        "absorbed_percent": info["absorbed"], "detected": info["detected"],
    }
    print(json.dumps(line), flush=True)


def job_of(spec: dict, photons: int):
    from umcx_gb300 import Job

    if "json" in spec:
        cfg = json.loads(json.dumps(spec["json"]))
        cfg["Session"]["Photons"] = int(photons)
        return Job.from_json(cfg)
    return Job.from_args([*spec["args"], "-n", str(int(photons))])


def roofline(r, kms: float, peaks: dict, hbm_peak: float, spec: dict) -> dict:
    """Fractions of the propagation kernel: the formula FP32 operations (per-event counts x the launch's events)
    against the live FMA rate and against SMs x 128 lanes x clock; SFU operations; fluence atomics against the
    scattered-atomic rate; warp instructions issued (ncu count per step x live steps) against 4 issue slots per SM
    and cycle; algorithmic bytes against HBM."""
    fp32_ops = sum(getattr(r, k) * v for k, v in OPS_FP32.items())
    sfu_ops = sum(getattr(r, k) * v for k, v in OPS_SFU.items())
    sec = kms * 1e-3
    achieved = fp32_ops / sec / 1e12
    peak = peaks["fp32_fma_per_s"] / 1e12
    spec_peak = peaks["sm_count"] * 128 * peaks["sm_clock_khz"] * 1e3 / 1e12
    issue_peak = peaks["sm_count"] * 4 * peaks["sm_clock_khz"] * 1e3
    wips = spec.get("warp_inst_per_step")
    issue = None
    if wips:
        issue = {"achieved_warp_inst_per_s": r.steps * wips / sec, "peak_warp_inst_per_s": issue_peak,
                 "frac": r.steps * wips / sec / issue_peak, "warp_inst_per_step": wips,
                 "source": "instructions per step from an ncu capture of this build (profiles/)"}
    return {"bound": "fp32", "achieved": achieved, "peak": peak,
            "unit": "Top/s (FP32 instructions, FMA = 1 op; peak measured live by an FMA loop)",
            "frac": achieved / peak,
            "frac_of_spec_rate": achieved / spec_peak, "spec_rate": spec_peak,
            "traffic": spec.get("dram_bytes"),
            "ops_per_launch": fp32_ops,
            "events_per_launch": {k: int(getattr(r, k)) for k in OPS_FP32},
            "sfu": {"achieved": sfu_ops / sec / 1e12, "peak": peaks["sfu_per_s"] / 1e12,
                    "frac": sfu_ops / sec / peaks["sfu_per_s"], "unit": "Top/s"},
            "l2_atomics": {"achieved_per_s": r.crossings / sec, "peak_per_s": peaks["l2_atomic_per_s"],
                           "frac": r.crossings / sec / peaks["l2_atomic_per_s"]},
            "hbm": {"algorithmic_gbs": r.crossings * 9.0 / sec / 1e9, "peak_gbs": hbm_peak},
            "issue": issue}


def time_forward(ctx, job, photons: int, steps: int, warmup: int, device: int, flush, shard=None):
    """Device-timed steps (kernel + output rounding; plus, with a shard, the cross-rank reduction) and the results."""
    import torch

    from umcx_gb300 import detp_columns

    sim = job.sim
    if shard is not None:
        sim.photon_offset, sim.nphoton = shard.photon_range(photons)
    nvox = sim.dim[0] * sim.dim[1] * sim.dim[2]
    nout = nvox * sim.dim[3]
    d_lab = torch.from_numpy(job.labels.ravel().copy()).to(f"cuda:{device}")
    d_flu = torch.empty(nout, dtype=torch.float32, device=f"cuda:{device}")
    d_det = torch.empty(max(1, sim.maxdetphotons * detp_columns(sim)), dtype=torch.float32, device=f"cuda:{device}")
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        ctx.forward_device(sim, d_lab, job.media, job.detpos, d_flu, d_det, stream)
    step_ms, kernel_ms, results = [], [], []
    if shard is not None:
        shard.barrier()
    torch.cuda.synchronize()
    gc.disable()  # no collector pause between a step's start event and its launches
    try:
        _timed_steps(ctx, job, sim, d_lab, d_flu, d_det, stream, flush, shard, steps, step_ms, kernel_ms, results)
    finally:
        gc.enable()
    if shard is not None:
        shard.barrier()
    torch.cuda.synchronize()
    return step_ms, kernel_ms, results


def _timed_steps(ctx, job, sim, d_lab, d_flu, d_det, stream, flush, shard, steps, step_ms, kernel_ms, results):
    """The timed steps of time_forward: each bracketed by CUDA events on the launching stream."""
    import torch

    from umcx_gb300 import detp_columns

    for _ in range(steps):
        flush.fill_(1)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        r = ctx.forward_device(sim, d_lab, job.media, job.detpos, d_flu, d_det, stream)
        if shard is not None:
            shard.reduce_device(d_flu, d_det[: r.saved * detp_columns(sim)].view(-1, detp_columns(sim))
                                if sim.issavedet and detp_columns(sim) else None, r)
        ev1.record(stream)
        ev1.synchronize()
        step_ms.append(ev0.elapsed_time(ev1))
        kernel_ms.append(r.kernel_ms)
        results.append(r)


def time_e2e(ctx, job, photons: int, reps: int, flush) -> dict:
    """photons/ms through umcx_gpu_forward with host buffers (caller-owned, page-locked, reused)."""
    import torch

    from umcx_gb300 import detp_columns

    sim = job.sim
    nvox = sim.dim[0] * sim.dim[1] * sim.dim[2]
    nout = nvox * sim.dim[3]

    def pinned(n, dtype):
        return torch.ones(n, dtype=dtype, pin_memory=True).numpy()

    h_lab = pinned(nvox, torch.uint8)
    h_lab[:] = job.labels.reshape(-1)
    h_flu = pinned(nout, torch.float32) if sim.issavevol else None
    h_dp = pinned(max(1, sim.maxdetphotons * detp_columns(sim)), torch.float32) if sim.issavedet else None
    ms = []
    for _ in range(max(1, reps)):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = ctx.forward(sim, h_lab, job.media, job.detpos, fluence=h_flu, detp=h_dp)
        ms.append((time.perf_counter() - t0) * 1e3)
    r = out.result
    h2d = nvox + 4 * 4 * sim.mediumnum + 4 * 4 * sim.detnum
    d2h = (nout * 4 if sim.issavevol else 0) + int(r.saved) * detp_columns(sim) * 4 + 96
    m = statistics.mean(ms)
    return {"value": photons / m, "unit": "photons/ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": m}


def measure_form(ctx, name: str, args, device: int, flush, peaks: dict, hbm_peak: float) -> dict:
    """One single-simulation configuration: device-timed photons/ms, end-to-end photons/ms, roofline fractions."""
    from umcx_gb300._lib import SIM_FP32_ACCUM

    spec = FORWARD[name]
    photons = int(spec["photons"])
    job = job_of(spec, photons)
    steps = spec.get("steps", 10)
    step_ms, kernel_ms, results = time_forward(ctx, job, photons, steps, 3, device, flush)
    r = results[-1]
    kms = statistics.mean(kernel_ms)
    launches_per_step = 2 if (job.sim.issavevol and not (job.sim.flags & SIM_FP32_ACCUM)) else 1
    return {"workload": spec["workload"], "photons": photons, "steps": steps,
            "photons_per_ms": photons * steps / sum(step_ms), "ms_per_step": sum(step_ms) / steps, "kernel_ms": kms,
            "e2e": time_e2e(ctx, job_of(spec, photons), photons, 3, flush),
            "gpu_launches_per_step": launches_per_step,
            "roofline": roofline(r, kms, peaks, hbm_peak, spec),
            "physics": {"absorbed_percent": (r.energy_total - r.energy_escape) / r.energy_total * 100,
                        "detected": int(r.detected), "steps_per_photon": r.steps / r.launched,
                        "scatters_per_photon": r.scatters / r.launched}}


def measure_adjoint(ctx, args) -> dict:
    """Forward + adjoint form (configuration 4: the configuration-1 grid and medium, 1e7 photons, four detectors,
    50 gates): photons/ms of the adjoint forward kernel plus the backward pass (record reduction and replay of every
    detected photon for the voxel Jacobians), device time."""
    from umcx_gb300 import Job

    cfg = json.loads(json.dumps(CONFIG))
    cfg["Session"].update({"ID": "c4", "Photons": 10000000, "DoMismatch": 0})
    cfg["Domain"]["Media"] = cfg["Domain"]["Media"][:2]
    cfg["Shapes"] = cfg["Shapes"][:1]
    job = Job.from_json(cfg)
    sim = job.sim
    fwd_ms, bwd_ms, recs = [], [], 0
    for rep in range(4):  # the first run warms up
        out = ctx.forward_adjoint(sim, job.labels, job.media, job.detpos)
        adj = ctx.backward(jacobian=True)
        if rep:
            fwd_ms.append(out.result.kernel_ms)
            bwd_ms.append(adj["replay_ms"])
        recs = adj["records"]
    f, b = statistics.mean(fwd_ms), statistics.mean(bwd_ms)
    return {"workload": "configuration 1 grid/medium + 4 detectors, 50 gates, 1e7 photons; per-label mua/mus "
                        "gradients of 200 detector readings and the summed volume + voxel Jacobians of 4 detectors",
            "photons_per_ms": sim.nphoton / (f + b), "forward_adjoint_ms": f, "replay_ms": b,
            "detected_records": int(recs), "replay_mismatch": int(adj["replay_mismatch"])}


def measure_batched(ctx, args, device) -> dict:
    """Batched form (configuration 5): 256 independent simulations in one persistent, graph-captured launch,
    autotuned, versus the same simulations as sequential single launches on the same GPU."""
    import torch

    from umcx_gb300.api import Batch, autotune_batch
    from umcx_gb300.workloads import batch5

    # set-up cost: JSON -> jobs -> batch, with the label volumes painted on the host or built on the GPU
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = Batch.from_jobs(ctx, batch5(args.batch_sims, photon_scale=args.batch_scale))
    torch.cuda.synchronize()
    setup_host = time.perf_counter() - t0
    b.close()
    t0 = time.perf_counter()
    jobs = batch5(args.batch_sims, photon_scale=args.batch_scale, device_labels=True)
    b = Batch.from_jobs(ctx, jobs, device_labels=True)
    torch.cuda.synchronize()
    setup_device = time.perf_counter() - t0
    n = sum(j.sim.nphoton for j in jobs)
    if args.no_autotune:
        tune = {"block_size": 1024, "blocks_per_sm": 0, "aggregation": 1, "source": "fixed"}
    else:
        tune = autotune_batch(ctx, jobs, fraction=0.1 if args.batch_scale >= 0.5 else 0.2, min_photons=500,
                              candidates=((512, 1), (1024, 1), (512, 2), (1024, 2)))
    b.set_tuning(tune["block_size"], tune["blocks_per_sm"], tune["aggregation"])
    b.run()
    runs = [b.run() for _ in range(2)]
    ms = statistics.mean(r.kernel_ms for r in runs)
    steps_per_photon = runs[-1].steps / max(1, runs[-1].launched)
    # end to end: one more run plus every simulation's output volume read back to the host, into one caller-owned
    # page-locked buffer of the largest volume that is reused (allocated and touched outside the timed region)
    host_out = torch.ones(max(j.sim.dim[0] * j.sim.dim[1] * j.sim.dim[2] * j.sim.dim[3] for j in jobs),
                          dtype=torch.float32, pin_memory=True).numpy()
    t0 = time.perf_counter()
    b.run()
    out_bytes = 0
    for i in range(len(jobs)):
        flu, _ = b.get(i, out=host_out)
        out_bytes += 0 if flu is None else flu.nbytes
    run_get = time.perf_counter() - t0
    b.close()
    # the same simulations one launch each (device buffers, same tuning)
    ctx.set_tuning(tune["block_size"], tune["blocks_per_sm"], tune["aggregation"])
    biggest = max(j.sim.dim[0] * j.sim.dim[1] * j.sim.dim[2] * j.sim.dim[3] for j in jobs)
    d_flu = torch.empty(biggest, dtype=torch.float32, device=f"cuda:{device}")
    d_lab = torch.empty(max(j.sim.dim[0] * j.sim.dim[1] * j.sim.dim[2] for j in jobs), dtype=torch.uint8,
                        device=f"cuda:{device}")
    stream = torch.cuda.current_stream()
    seq = 0.0
    for j in jobs:
        j.build_labels(ctx, d_lab)
        seq += ctx.forward_device(j.sim, d_lab, j.media, None, d_flu, None, stream).kernel_ms
    ctx.set_tuning()
    return {"workload": f"{len(jobs)} simulations, edges 32-128, 2-5 labels, log-uniform 1e5-1e7 photons "
                        f"(x{args.batch_scale}), 10 gates",
            "photons": n, "steps_per_photon": steps_per_photon,
            "photons_per_ms": n / ms, "graph_ms": ms, "sequential_photons_per_ms": n / seq,
            "sequential_kernel_ms": seq, "speedup_vs_sequential": seq / ms, "tuning": tune,
            "setup_s": {"labels_on_host": setup_host, "labels_on_gpu": setup_device},
            "e2e": {"photons_per_ms": n / ((setup_device + run_get) * 1e3), "setup_s": setup_device,
                    "run_and_readback_s": run_get, "d2h_bytes": out_bytes}}


def run_gpu_arm(args) -> None:
    import torch

    from umcx_gb300 import Context, measure_peaks
    from umcx_gb300._lib import SIM_FP32_ACCUM

    ws, rank, local = dist_env()
    shard = None
    if ws > 1:
        from umcx_gb300.shard import Shard

        torch.cuda.set_device(local)
        shard = Shard.init("nccl")
    device = local if ws > 1 else 0
    torch.cuda.set_device(device)

    spec = FORWARD[args.workload]
    photons = int(args.photons) if args.photons else int(spec["photons"])
    job = job_of(spec, photons)
    ctx = Context(device)
    if args.block or args.blocks_per_sm or args.aggregation:
        ctx.set_tuning(args.block, args.blocks_per_sm, args.aggregation)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{device}")
    tuning = {"block_size": args.block, "blocks_per_sm": args.blocks_per_sm, "aggregation": args.aggregation,
              "source": "command line"}
    if not (args.block or args.blocks_per_sm or args.aggregation) and not args.no_autotune:
        # the project's autotuner: timed runs at half the photons over block sizes and aggregation modes.  A probe
        # must be long against the launch's drain (the last, longest photons: ~5 ms here), or the drain's noise
        # decides the choice
        import numpy as np  # noqa: F401

        from umcx_gb300 import detp_columns

        s = job.sim
        d_lab = torch.from_numpy(job.labels.ravel().copy()).to(f"cuda:{device}")
        d_flu = torch.empty(s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3], dtype=torch.float32, device=f"cuda:{device}")
        d_det = torch.empty(max(1, s.maxdetphotons * detp_columns(s)), dtype=torch.float32, device=f"cuda:{device}")
        tuning = dict(ctx.autotune(s, d_lab, job.media, job.detpos, d_flu, d_det, fraction=0.5),
                      source="autotune (50 % photon probes)")
        del d_lab, d_flu, d_det

    sampler = ClockSampler(device)
    sampler.start()
    t_all = time.perf_counter()
    step_ms, kernel_ms, results = time_forward(ctx, job, photons, args.steps, args.warmup, device, flush, shard)
    wall_all = time.perf_counter() - t_all
    clocks = sampler.stop()
    e2e = time_e2e(ctx, job_of(spec, photons), photons, args.e2e_steps, flush)

    # max over ranks
    total_step_ms = sum(step_ms)
    e2e_ms = e2e["ms_per_step"]
    if shard is not None:
        total_step_ms, e2e_ms = shard.max_over_ranks([total_step_ms, e2e_ms])
    photons_all = photons * ws
    value = photons_all * args.steps / total_step_ms
    e2e["value"] = photons_all / e2e_ms
    e2e["ms_per_step"] = e2e_ms
    r0 = results[-1]
    kms = statistics.mean(kernel_ms)
    peaks = measure_peaks(device)
    peaks_file = ROOT / "MEASURED_PEAKS.json"
    hbm_peak = json.loads(peaks_file.read_text()).get("hbm_gbs") if peaks_file.exists() else 6800.0
    # the other forms first, while the GPU is still busy (the CPU baseline leaves it idle for seconds)
    forms = {}
    wanted = set() if args.no_forms else {f.strip() for f in args.forms.split(",") if f.strip()}
    if rank == 0:
        ctx.set_tuning(tuning["block_size"], tuning["blocks_per_sm"], tuning["aggregation"])
        for name in ("c1", "cube60", "c3"):
            if name in wanted:
                forms[name] = measure_form(ctx, name, args, device, flush, peaks, hbm_peak)
        if "adjoint" in wanted:
            forms["adjoint"] = measure_adjoint(ctx, args)
        if "batched" in wanted:
            forms["batched"] = measure_batched(ctx, args, device)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_reference_run(args.cpu_photons, os.cpu_count() or 1)

    if rank == 0:
        sim = job.sim
        launches = 2 if (sim.issavevol and not (sim.flags & SIM_FP32_ACCUM)) else 1
        line = {
            "metric": METRIC if args.workload == "c2" else f"photons/ms ({spec['workload']})", "value": value,
            "unit": "photons/ms", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_step_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (generated configuration)",
            "config": {"workload": spec["workload"], "photons_per_step_per_gpu": photons, "grid": list(sim.dim[:3]),
                       "gates": int(sim.dim[3]), "detectors": int(sim.detnum),
                       "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"photon ranges x{ws}" + (" + GPU sum of volumes and tallies" if ws > 1 else ""),
                       "tuning": tuning},
            "e2e": e2e,
            # per step: the propagation kernel and the FP64 -> FP32 rounding of the output volume
            "gpu_launches": args.steps * launches,
            "kernel_ms": kms,
            "roofline": roofline(r0, kms, peaks, hbm_peak, spec if photons == spec["photons"] else {}),
            "clocks": clocks,
            "physics": {"absorbed_percent": (r0.energy_total - r0.energy_escape) / r0.energy_total * 100,
                        "detected": int(r0.detected), "steps_per_photon": r0.steps / r0.launched,
                        "scatters_per_photon": r0.scatters / r0.launched},
            "wall_s_timed": wall_all,
        }
        if cpu:
            line["cpu_baseline"] = {"value": cpu["value"], "unit": "photons/ms", "cores": os.cpu_count() or 1,
                                    "kind": cpu["kind"],
                                    "sample": f"{args.cpu_photons} photons of the same configuration"}
        if forms:
            line["forms"] = forms
        print(json.dumps(line), flush=True)
    if shard is not None:
        shard.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--photons", type=float, default=0, help="photons per step (default: the workload's own)")
    ap.add_argument("--workload", default="c2", choices=sorted(FORWARD),
                    help="the timed configuration (default: configuration 2, the headline; the others for profiling)")
    ap.add_argument("--cpu-photons", type=int, default=1000000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--aggregation", type=int, default=0)
    ap.add_argument("--no-forms", action="store_true", help="skip the other configurations and forms")
    ap.add_argument("--forms", default="c1,cube60,c3,adjoint,batched", help="comma list of the extra forms to measure")
    ap.add_argument("--no-autotune", action="store_true", help="use the built-in launch defaults (forms: fixed)")
    ap.add_argument("--batch-sims", type=int, default=256)
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="photon-budget scale of the batched form (1.0 = the full 5.4e8-photon batch, ~3.5 s/run)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":
        if args.cpu_photons == 1000000:
            args.cpu_photons = 300000
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
