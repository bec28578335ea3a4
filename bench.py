"""Benchmark of the umcx photon-transport hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--photons P]

Workload: the heterogeneous forward configuration with refractive mismatch and detectors -- 60x60x60 voxels of
1 mm, background label 1 (mua 0.005/mm, mus 1/mm, g 0.01, n 1.37), a radius-15 sphere of label 2 (mua 0.002,
mus 5, g 0.9, n 1.0) centred at (30,30,30), pencil source at (29,29,0) along +z, boundary reflection on, 1e7
photons per step, 50 time gates over 0-5 ns, four disk detectors of radius 1 mm at z = 0 with partial
pathlengths saved.  Synthetic input (the configuration is generated, not read from a dataset).

One step = one full simulation of P photons.  `value` is photons/ms of the propagation kernel with the inputs
resident in HBM (CUDA events on the launching stream; the fluence output, 43 MB, is cleared inside the step and the
L2 is flushed by writing a 256 MB buffer between steps).  `e2e` is the same metric through the C ABI call with host
buffers in page-locked memory (umcx_gpu_forward: label upload, simulation, fluence + detected-photon download),
timed on the host.

--impl reference times the reference's own CPU implementation (the unmodified reference program built from its
sources, oracle/_ref/umcx, with all host threads; else the C restatement in oracle/) on a bounded photon sample of
the same configuration.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

CONFIG = {
    "Session": {"ID": "bench_c2", "Photons": 10000000, "RNGSeed": 1648335518, "DoMismatch": 1, "DoPartialPath": 1,
                "SaveDetFlag": 5, "OutputType": "x"},
    "Forward": {"T0": 0, "T1": 5e-9, "Dt": 1e-10},
    "Domain": {"Dim": [60, 60, 60], "LengthUnit": 1,
               "Media": [{"mua": 0, "mus": 0, "g": 1, "n": 1}, {"mua": 0.005, "mus": 1.0, "g": 0.01, "n": 1.37},
                         {"mua": 0.002, "mus": 5.0, "g": 0.9, "n": 1.0}]},
    "Optode": {"Source": {"Type": "pencil", "Pos": [29, 29, 0], "Dir": [0, 0, 1]},
               "Detector": [{"Pos": [29, 19, 0], "R": 1}, {"Pos": [19, 29, 0], "R": 1},
                            {"Pos": [29, 39, 0], "R": 1}, {"Pos": [39, 29, 0], "R": 1}]},
    "Shapes": [{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}, {"Sphere": {"O": [30, 30, 30], "R": 15, "Tag": 2}}],
}
WORKLOAD = "heterogeneous forward, 60^3 grid, sphere R15, reflection on, 50 gates, 4 detectors (ppath saved)"
METRIC = "photons/ms (forward, heterogeneous 60^3 + sphere, reflection, 50 gates, 4 detectors)"

# DRAM bytes (read + write) of one propagation launch of the default workload (1e7 photons), from an ncu capture
# of the same command (dram__bytes_read.sum + dram__bytes_write.sum: 93.5 MB of label and table reads, 3.06 GB of
# FP64-accumulator lines, the volume and the copies of its first gates, written back as L2 evicts them); not
# measured live, reported only for the default size
DRAM_BYTES_DEFAULT_LAUNCH = 93_477_376 + 3_064_464_000

# warp instructions issued per voxel step by the propagation kernel, from an ncu capture of the default launch
# (smsp__inst_executed.sum 4.37e10 over 3.436e9 steps; block 1024, plain atomics), captured before the copies of
# the output volume took 32-bit offsets (a few instructions fewer per deposit, so a slight overestimate); with the
# live step count and kernel time it gives the issue rate against the SMs' 4 issue slots per cycle
WARP_INST_PER_STEP = 12.72

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
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
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
                   "program": "reference umcx CPU OpenMP build" if info["kind"] == "reference" else "oracle C port"},
        "cpu_baseline": {"value": value, "unit": "photons/ms", "cores": threads, "kind": info["kind"],
                         "sample": f"{photons} photons of the benchmark configuration per step"},
        "e2e": {"value": value, "unit": "photons/ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
        "absorbed_percent": info["absorbed"], "detected": info["detected"],
    }
    print(json.dumps(line), flush=True)


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
        tune = autotune_batch(ctx, jobs, fraction=0.2, min_photons=500,
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
    import numpy as np
    import torch

    from umcx_gb300 import Context, Job, detp_columns, measure_peaks
    from umcx_gb300._lib import SIM_FP32_ACCUM

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if ws > 1 else 0
    torch.cuda.set_device(device)

    cfg = json.loads(json.dumps(CONFIG))
    cfg["Session"]["Photons"] = int(args.photons)
    job = Job.from_json(cfg)
    sim = job.sim
    sim.photon_offset = rank * int(args.photons)  # weak scaling: each rank simulates its own photon range
    ctx = Context(device)
    if args.block or args.blocks_per_sm or args.aggregation:
        ctx.set_tuning(args.block, args.blocks_per_sm, args.aggregation)
    nvox = sim.dim[0] * sim.dim[1] * sim.dim[2]
    nout = nvox * sim.dim[3]
    d_lab = torch.from_numpy(job.labels.ravel().copy()).to(f"cuda:{device}")
    d_flu = torch.empty(nout, dtype=torch.float32, device=f"cuda:{device}")
    d_det = torch.empty(sim.maxdetphotons * detp_columns(sim), dtype=torch.float32, device=f"cuda:{device}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{device}")
    stream = torch.cuda.current_stream()
    tuning = {"block_size": args.block, "blocks_per_sm": args.blocks_per_sm, "aggregation": args.aggregation,
              "source": "command line"}
    if not (args.block or args.blocks_per_sm or args.aggregation) and not args.no_autotune:
        # the project's autotuner: timed runs at half the photons over block sizes and aggregation modes.  A probe
        # must be long against the launch's drain (the last, longest photons: ~7 ms here), or the drain's noise
        # decides the choice
        tuning = dict(ctx.autotune(sim, d_lab, job.media, job.detpos, d_flu, d_det, fraction=0.5),
                      source="autotune (50 % photon probes)")

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        ctx.forward_device(sim, d_lab, job.media, job.detpos, d_flu, d_det, stream)
    sampler = ClockSampler(device)
    sampler.start()
    kernel_ms, step_ms, results = [], [], []
    barrier()
    t_all = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(1)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        r = ctx.forward_device(sim, d_lab, job.media, job.detpos, d_flu, d_det, stream)
        ev1.record(stream)
        ev1.synchronize()
        step_ms.append(ev0.elapsed_time(ev1))
        kernel_ms.append(r.kernel_ms)
        results.append(r)
    barrier()
    wall_all = time.perf_counter() - t_all
    clocks = sampler.stop()

    # end to end through the C ABI with host buffers: the caller's label volume in, the fluence and detected-photon
    # rows out into output arrays it reuses from call to call (page-locked host memory, allocated and touched once
    # outside the timed region)
    def pinned(n, dtype):
        return torch.ones(n, dtype=dtype, pin_memory=True).numpy()

    h_lab = pinned(nvox, torch.uint8)
    h_lab[:] = job.labels.reshape(-1)
    h_med, h_det = job.media, job.detpos
    h_flu = pinned(nout, torch.float32)
    h_dp = pinned(max(1, sim.maxdetphotons * detp_columns(sim)), torch.float32)
    e2e_ms = []
    for _ in range(max(1, args.e2e_steps)):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = ctx.forward(sim, h_lab, h_med, h_det, fluence=h_flu, detp=h_dp)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    r_host = out.result
    h2d = nvox + 4 * 4 * sim.mediumnum + 4 * 4 * sim.detnum
    d2h = nout * 4 + int(r_host.saved) * detp_columns(sim) * 4 + 96

    # max over ranks
    total_step_ms = sum(step_ms)
    if ws > 1:
        import torch.distributed as dist

        t = torch.tensor([total_step_ms, statistics.mean(e2e_ms)], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_step_ms, e2e_mean = t.tolist()
    else:
        e2e_mean = statistics.mean(e2e_ms)

    photons_all = int(args.photons) * ws
    value = photons_all * args.steps / total_step_ms
    e2e_value = photons_all / e2e_mean
    r0 = results[-1]
    kms = statistics.mean(kernel_ms)
    fp32_ops = sum(getattr(r0, k) * v for k, v in OPS_FP32.items())
    sfu_ops = sum(getattr(r0, k) * v for k, v in OPS_SFU.items())
    peaks = measure_peaks(device)
    achieved_fp32 = fp32_ops / (kms * 1e-3) / 1e12
    peak_fp32 = peaks["fp32_fma_per_s"] / 1e12
    achieved_sfu = sfu_ops / (kms * 1e-3) / 1e12
    peak_sfu = peaks["sfu_per_s"] / 1e12
    atomics_per_s = r0.crossings / (kms * 1e-3)
    issue_per_s = r0.steps * WARP_INST_PER_STEP / (kms * 1e-3)
    issue_peak = peaks["sm_count"] * 4 * peaks["sm_clock_khz"] * 1e3
    peaks_file = ROOT / "MEASURED_PEAKS.json"
    hbm_peak = json.loads(peaks_file.read_text()).get("hbm_gbs") if peaks_file.exists() else 6800.0
    traffic_alg = r0.crossings * 9.0  # label byte + fluence read-modify-write per crossing
    # the other forms first, while the GPU is still busy (the CPU baseline leaves it idle for seconds)
    forms = {}
    wanted = set() if args.no_forms else {f.strip() for f in args.forms.split(",") if f.strip()}
    if rank == 0 and "adjoint" in wanted:
        forms["adjoint"] = measure_adjoint(ctx, args)
    if rank == 0 and "batched" in wanted:
        forms["batched"] = measure_batched(ctx, args, device)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_reference_run(args.cpu_photons, os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "photons/ms", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_step_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (generated configuration)",
            "config": {"workload": WORKLOAD, "photons_per_step_per_gpu": int(args.photons), "grid": [60, 60, 60],
                       "gates": int(sim.dim[3]), "detectors": int(sim.detnum),
                       "l2": "flushed between steps (256 MB write)", "parallelism": f"photon ranges x{ws}",
                       "tuning": tuning},
            "e2e": {"value": e2e_value, "unit": "photons/ms", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_mean},
            # per step: the propagation kernel and the FP64 -> FP32 rounding of the output volume
            "gpu_launches": args.steps * (2 if (sim.issavevol and not (sim.flags & SIM_FP32_ACCUM)) else 1),
            "kernel_ms": kms,
            "roofline": {"bound": "fp32", "achieved": achieved_fp32, "peak": peak_fp32,
                         "unit": "Top/s (FP32 instructions, FMA = 1 op; peak measured live by an FMA loop)",
                         "frac": achieved_fp32 / peak_fp32,
                         "traffic": DRAM_BYTES_DEFAULT_LAUNCH if int(args.photons) == 10000000 else None,
                         "ops_per_launch": fp32_ops,
                         "events_per_launch": {k: int(getattr(r0, k)) for k in OPS_FP32},
                         "sfu": {"achieved": achieved_sfu, "peak": peak_sfu, "frac": achieved_sfu / peak_sfu,
                                 "unit": "Top/s"},
                         "l2_atomics": {"achieved_per_s": atomics_per_s, "peak_per_s": peaks["l2_atomic_per_s"],
                                        "frac": atomics_per_s / peaks["l2_atomic_per_s"]},
                         "hbm": {"algorithmic_gbs": traffic_alg / (kms * 1e-3) / 1e9, "peak_gbs": hbm_peak},
                         "issue": {"achieved_warp_inst_per_s": issue_per_s, "peak_warp_inst_per_s": issue_peak,
                                   "frac": issue_per_s / issue_peak, "warp_inst_per_step": WARP_INST_PER_STEP,
                                   "source": "instructions per step from the ncu capture of the default launch"}},
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
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--photons", type=float, default=1e7)
    ap.add_argument("--cpu-photons", type=int, default=1000000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--aggregation", type=int, default=0)
    ap.add_argument("--no-forms", action="store_true", help="skip the adjoint and batched forms")
    ap.add_argument("--forms", default="adjoint,batched", help="comma list of the extra forms to measure")
    ap.add_argument("--no-autotune", action="store_true", help="use the built-in launch defaults (forms: fixed)")
    ap.add_argument("--batch-sims", type=int, default=256)
    ap.add_argument("--batch-scale", type=float, default=0.1,
                    help="photon-budget scale of the batched form (1.0 = the full 5.4e8-photon batch, ~5 s/run)")
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
