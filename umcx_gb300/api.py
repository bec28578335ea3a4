"""Python side of the library: jobs (reference-style inputs) and GPU contexts, over the C ABI.

    from umcx_gb300 import Job, Context
    job = Job.from_args(["--bench", "cube60", "-n", "1e6"])
    with Context(0) as ctx:
        out = ctx.forward(job.sim, job.labels, job.media, job.detpos)
    out.fluence  # float32 [maxgate, nx, ny, nz], not normalised; job.normalizer(out.energy_total) gives L820's factor
"""
from __future__ import annotations

import ctypes as C
import json
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import Result, Sim, Tuning, check, load


def _argv(args: list[str]):
    arr = (C.c_char_p * (len(args) + 1))()
    arr[0] = b"umcx"
    for k, a in enumerate(args):
        arr[k + 1] = a.encode()
    return arr


class Job:
    """A parsed reference-style input (MCX_userio + MCX_run_simulation set-up)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_args(cls, args: list[str], device_labels: bool = False) -> "Job":
        """Parse a reference command line.  device_labels=True leaves the shapes unpainted and the detectors
        unmasked on the host: the label volume is then built on the GPU by build_labels (job.labels is None)."""
        lib = load()
        h = C.c_void_p()
        flags = _lib.UMCX_JOB_DEVICE_LABELS if device_labels else 0
        rc = lib.umcx_job_from_args_ex(C.byref(h), len(args) + 1, _argv(args), flags)
        job = cls(h)
        if rc != _lib.UMCX_OK:
            msg = lib.umcx_job_error(h).decode()
            lib.umcx_job_free(h)
            job._h = None
            raise ValueError(msg)
        return job

    @classmethod
    def from_json(cls, cfg, device_labels: bool = False) -> "Job":
        text = cfg if isinstance(cfg, str) else json.dumps(cfg)
        return cls.from_args(["--json", text], device_labels)

    def __del__(self):
        if getattr(self, "_h", None):
            load().umcx_job_free(self._h)
            self._h = None

    @property
    def action(self) -> int:
        return load().umcx_job_action(self._h)

    @property
    def console(self) -> str:
        return load().umcx_job_console(self._h).decode()

    @property
    def config(self) -> dict:
        return json.loads(load().umcx_job_config_json(self._h, -1).decode())

    @property
    def sim(self) -> Sim:
        return load().umcx_job_sim(self._h).contents.copy()

    @property
    def labels(self) -> np.ndarray | None:
        """uint8 labels [nx, ny, nz] built on the host (None for a job parsed with device_labels=True)."""
        s = self.sim
        n = s.dim[0] * s.dim[1] * s.dim[2]
        p = load().umcx_job_labels(self._h)
        if not p:
            return None
        return np.ctypeslib.as_array(p, shape=(n,)).copy().reshape(s.dim[0], s.dim[1], s.dim[2])

    @property
    def has_host_labels(self) -> bool:
        return bool(load().umcx_job_labels(self._h))

    def build_labels(self, ctx: "Context", d_labels) -> None:
        """Build this job's uint8 label volume on the GPU (umcx_job_build_labels) into d_labels: a CUDA tensor of
        nx*ny*nz bytes, or a device address (int)."""
        ptr = d_labels if isinstance(d_labels, int) else d_labels.data_ptr()
        check(load().umcx_job_build_labels(self._h, ctx.handle, C.c_void_p(ptr)), ctx.handle, "umcx_job_build_labels")

    @property
    def media(self) -> np.ndarray:
        s = self.sim
        p = load().umcx_job_media(self._h)
        return np.ctypeslib.as_array(p, shape=(s.mediumnum * 4,)).copy().reshape(s.mediumnum, 4)

    @property
    def detpos(self) -> np.ndarray:
        s = self.sim
        if s.detnum == 0:
            return np.zeros((0, 4), np.float32)
        p = load().umcx_job_detpos(self._h)
        return np.ctypeslib.as_array(p, shape=(s.detnum * 4,)).copy().reshape(s.detnum, 4)

    @property
    def isnormalized(self) -> bool:
        return bool(load().umcx_job_isnormalized(self._h))

    @property
    def tuning(self) -> dict:
        """Launch shape the input asks for (Session.BlockSize / ThreadNum, the -T / -t flags), as keyword arguments
        of Context.set_tuning; empty when the input names neither."""
        t = _lib.Tuning()
        check(load().umcx_job_tuning(self._h, C.byref(t)), None, "umcx_job_tuning")
        return {"block_size": t.block_size, "grid_size": t.grid_size} if (t.block_size or t.grid_size) else {}

    def normalizer(self, energytotal: float) -> float:
        return float(load().umcx_job_normalizer(self._h, energytotal))

    def domain_int32(self) -> np.ndarray:
        lib = load()
        dims = (C.c_uint32 * 3)()
        check(lib.umcx_job_domain_dims(self._h, dims), None, "umcx_job_domain_dims")
        out = np.zeros(dims[0] * dims[1] * dims[2], np.int32)
        check(lib.umcx_job_domain_int32(self._h, out.ctypes.data, out.size), None, "umcx_job_domain_int32")
        return out.reshape(dims[0], dims[1], dims[2])

    def dump_mask(self, path: str) -> None:
        check(load().umcx_job_dump_mask(self._h, path.encode()), None, "umcx_job_dump_mask")

    def write_outputs(self, fluence, detp, res: Result, normalize: bool = True) -> None:
        f = None if fluence is None else np.ascontiguousarray(fluence, np.float32)
        d = None if detp is None else np.ascontiguousarray(detp, np.float32)
        check(load().umcx_job_write_outputs(self._h, None if f is None else f.ctypes.data,
                                            None if d is None else d.ctypes.data, C.byref(res), int(normalize)),
              None, "umcx_job_write_outputs")


def detp_columns(sim: Sim) -> int:
    """Floats per detected-photon row for sim's SaveDetFlag (umcx_detp_columns, the reference's L157)."""
    return load().umcx_detp_columns(C.byref(sim))


def measure_peaks(device: int = 0) -> dict:
    """FP32 FMA/s, SFU op/s and scattered L2 float-atomic/s of the device (roofline denominators)."""
    p = _lib.Peaks()
    check(load().umcx_measure_peaks(int(device), C.byref(p)), None, "umcx_measure_peaks")
    return {"fp32_fma_per_s": p.fp32_fma_per_s, "sfu_per_s": p.sfu_per_s, "l2_atomic_per_s": p.l2_atomic_per_s,
            "sm_count": p.sm_count, "sm_clock_khz": p.sm_clock_khz}


def seeds_from_rngseed(seed: int) -> np.ndarray:
    """The four session seeds the reference derives from RNGSeed (srand + four rand() calls, L724-727)."""
    out = (C.c_uint32 * 4)()
    check(load().umcx_seeds_from_rngseed(int(seed), out), None, "umcx_seeds_from_rngseed")
    return np.array(list(out), np.uint32)


@dataclass
class Forward:
    """Outputs of one forward simulation: fluence [maxgate, nx, ny, nz] (not normalised), detected-photon rows
    [saved, columns] and the tallies (energies, event counts, kernel time)."""

    fluence: np.ndarray | None
    detp: np.ndarray | None
    result: Result
    extra: dict = field(default_factory=dict)

    @property
    def energy_total(self) -> float:
        return self.result.energy_total

    @property
    def energy_escape(self) -> float:
        return self.result.energy_escape

    @property
    def absorbed_fraction(self) -> float:
        r = self.result
        return (r.energy_total - r.energy_escape) / r.energy_total


class Context:
    """A CUDA device context of the library (umcx_create / umcx_destroy)."""

    def __init__(self, device: int = 0):
        lib = load()
        self._h = C.c_void_p()
        rc = lib.umcx_create(C.byref(self._h), int(device))
        if rc != _lib.UMCX_OK:
            raise RuntimeError(f"umcx_create({device}) failed with status {rc}")

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().umcx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def last_error(self) -> str:
        return load().umcx_last_error(self._h).decode()

    def set_tuning(self, block_size: int = 0, blocks_per_sm: int = 0, aggregation: int = 0,
                   budget_ms: int = 0, grid_size: int = 0) -> None:
        """Launch tuning for later calls (0 = automatic).  grid_size: CTAs of the launch (0 = one persistent wave of
        resident CTAs), as the reference's ThreadNum / BlockSize give it (Job.tuning)."""
        t = Tuning(block_size, blocks_per_sm, aggregation, budget_ms, grid_size)
        check(load().umcx_set_tuning(self._h, C.byref(t)), self._h, "umcx_set_tuning")

    def forward(self, sim: Sim, labels, media, detpos=None, fluence=None, detp=None) -> Forward:
        """Host-buffer forward simulation (umcx_gpu_forward).  fluence / detp: optional caller-owned float32 output
        arrays (nx*ny*nz*maxgate and maxdetphotons*columns elements) reused across calls instead of new ones."""
        lab = np.ascontiguousarray(labels, np.uint8)
        med = np.ascontiguousarray(media, np.float32)
        det = np.ascontiguousarray(detpos if detpos is not None else np.zeros((0, 4)), np.float32)
        nout = sim.dim[0] * sim.dim[1] * sim.dim[2] * sim.dim[3]
        cols = detp_columns(sim)
        ndp = max(1, sim.maxdetphotons * cols)
        flu = dp = None
        if sim.issavevol:
            flu = np.zeros(nout, np.float32) if fluence is None else fluence.reshape(-1)
            if flu.dtype != np.float32 or flu.size < nout or not flu.flags.c_contiguous:
                raise ValueError("fluence must be a contiguous float32 array of nx*ny*nz*maxgate elements")
        if sim.issavedet:
            dp = np.zeros(ndp, np.float32) if detp is None else detp.reshape(-1)
            if dp.dtype != np.float32 or dp.size < ndp or not dp.flags.c_contiguous:
                raise ValueError("detp must be a contiguous float32 array of maxdetphotons*columns elements")
        res = Result()
        rc = load().umcx_gpu_forward(self._h, C.byref(sim), lab.ctypes.data, med.ctypes.data,
                                     det.ctypes.data if det.size else None,
                                     None if flu is None else flu.ctypes.data,
                                     None if dp is None else dp.ctypes.data, C.byref(res))
        check(rc, self._h, "umcx_gpu_forward")
        if flu is not None:
            flu = flu[:nout].reshape(sim.dim[3], sim.dim[0], sim.dim[1], sim.dim[2])
        if dp is not None:
            dp = dp[: res.saved * cols].reshape(res.saved, cols)
        return Forward(flu, dp, res)

    def forward_adjoint(self, sim: Sim, labels, media, detpos=None) -> Forward:
        """Forward pass that keeps what umcx_gpu_backward needs (umcx_gpu_forward_adjoint)."""
        lab = np.ascontiguousarray(labels, np.uint8)
        med = np.ascontiguousarray(media, np.float32)
        det = np.ascontiguousarray(detpos if detpos is not None else np.zeros((0, 4)), np.float32)
        nout = sim.dim[0] * sim.dim[1] * sim.dim[2] * sim.dim[3]
        flu = np.zeros(nout, np.float32) if sim.issavevol else None
        cols = detp_columns(sim)
        dp = np.zeros(max(1, sim.maxdetphotons * cols), np.float32) if sim.issavedet else None
        res = Result()
        rc = load().umcx_gpu_forward_adjoint(self._h, C.byref(sim), lab.ctypes.data, med.ctypes.data,
                                             det.ctypes.data if det.size else None,
                                             None if flu is None else flu.ctypes.data,
                                             None if dp is None else dp.ctypes.data, C.byref(res))
        check(rc, self._h, "umcx_gpu_forward_adjoint")
        self._adj_sim = sim.copy()
        if flu is not None:
            flu = flu.reshape(sim.dim[3], sim.dim[0], sim.dim[1], sim.dim[2])
        if dp is not None:
            dp = dp[: res.saved * cols].reshape(res.saved, cols)
        return Forward(flu, dp, res)

    def backward(self, jacobian: bool = False) -> dict:
        """Derivatives of the last forward_adjoint's detector readings and summed output (umcx_gpu_backward)."""
        s = self._adj_sim
        d, t, k = s.detnum, s.dim[3], s.mediumnum
        out = {"readings": np.zeros((d, t)), "dread_dmua": np.zeros((d, t, k)), "dread_dmus": np.zeros((d, t, k)),
               "dflu_dmua": np.zeros(k), "dflu_dmus": np.zeros(k)}
        jac = np.zeros((d, s.dim[0], s.dim[1], s.dim[2]), np.float32) if jacobian and d else None
        a = _lib.Adjoint()
        a.readings = out["readings"].ctypes.data
        a.dread_dmua = out["dread_dmua"].ctypes.data
        a.dread_dmus = out["dread_dmus"].ctypes.data
        a.dflu_dmua = out["dflu_dmua"].ctypes.data
        a.dflu_dmus = out["dflu_dmus"].ctypes.data
        a.jacobian = None if jac is None else jac.ctypes.data
        check(load().umcx_gpu_backward(self._h, C.byref(a)), self._h, "umcx_gpu_backward")
        out.update({"jacobian": jac, "records": a.records, "replay_mismatch": a.replay_mismatch,
                    "replay_ms": a.replay_ms})
        return out

    def forward_device(self, sim: Sim, d_labels, media, detpos, d_fluence, d_detp, stream=None) -> Result:
        """Device-buffer forward simulation (umcx_gpu_forward_device); d_* are torch CUDA tensors."""
        med = np.ascontiguousarray(media, np.float32)
        det = np.ascontiguousarray(detpos if detpos is not None else np.zeros((0, 4)), np.float32)
        res = Result()
        st = None if stream is None else C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))
        rc = load().umcx_gpu_forward_device(self._h, C.byref(sim), C.c_void_p(d_labels.data_ptr()), med.ctypes.data,
                                            det.ctypes.data if det.size else None,
                                            None if d_fluence is None else C.c_void_p(d_fluence.data_ptr()),
                                            None if d_detp is None else C.c_void_p(d_detp.data_ptr()), st,
                                            C.byref(res))
        check(rc, self._h, "umcx_gpu_forward_device")
        return res

    def autotune(self, sim: Sim, d_labels, media, detpos, d_fluence, d_detp, fraction: float = 0.05) -> dict:
        """Pick block size / CTAs per SM / aggregation for this simulation from short timed runs (umcx_autotune)."""
        med = np.ascontiguousarray(media, np.float32)
        det = np.ascontiguousarray(detpos if detpos is not None else np.zeros((0, 4)), np.float32)
        best = Tuning()
        ms = C.c_float()
        rc = load().umcx_autotune(self._h, C.byref(sim), C.c_void_p(d_labels.data_ptr()), med.ctypes.data,
                                  det.ctypes.data if det.size else None,
                                  None if d_fluence is None else C.c_void_p(d_fluence.data_ptr()),
                                  None if d_detp is None else C.c_void_p(d_detp.data_ptr()), float(fraction),
                                  C.byref(best), C.byref(ms))
        check(rc, self._h, "umcx_autotune")
        return {"block_size": best.block_size, "blocks_per_sm": best.blocks_per_sm, "aggregation": best.aggregation,
                "probe_ms": ms.value}

    def rng_dump(self, seeds, photon_offset: int, nphoton: int, ndraw: int) -> np.ndarray:
        """rand01() draws [nphoton, ndraw] of photons photon_offset.. computed on the device (known-answer hook)."""
        s = (C.c_uint32 * 4)(*[int(x) for x in seeds])
        out = np.zeros(nphoton * ndraw, np.float32)
        check(load().umcx_gpu_rng_dump(self._h, s, int(photon_offset), int(nphoton), int(ndraw), out.ctypes.data),
              self._h, "umcx_gpu_rng_dump")
        return out.reshape(nphoton, ndraw)


class Batch:
    """Many independent simulations in one persistent, graph-captured launch (umcx_batch_*)."""

    def __init__(self, ctx: Context, sims, labels, media, detpos=None):
        """labels: one host uint8 volume per simulation, or None to write them in place afterwards (label_ptr).
        detpos: per simulation its detectors ([detnum, 4] {x, y, z, r}) or None; needed by the simulations that
        save detected photons (issavedet)."""
        lib = load()
        n = len(sims)
        arr = (Sim * n)(*[s.copy() for s in sims])
        keep_lab = [] if labels is None else [np.ascontiguousarray(x, np.uint8) for x in labels]
        keep_med = [np.ascontiguousarray(m, np.float32) for m in media]
        keep_det = [None if d is None or len(d) == 0 else np.ascontiguousarray(d, np.float32)
                    for d in (detpos if detpos is not None else [None] * n)]
        lab = None if labels is None else (C.c_void_p * n)(*[x.ctypes.data for x in keep_lab])
        med = (C.c_void_p * n)(*[m.ctypes.data for m in keep_med])
        det = (C.c_void_p * n)(*[None if d is None else d.ctypes.data for d in keep_det])
        self._ctx = ctx
        self._h = C.c_void_p()
        check(lib.umcx_batch_create(ctx.handle, n, arr, lab, med, det, C.byref(self._h)), ctx.handle,
              "umcx_batch_create")
        self.sims = [s.copy() for s in sims]

    @classmethod
    def from_jobs(cls, ctx: Context, jobs, device_labels: bool = False, sims=None) -> "Batch":
        """Batch of parsed jobs (sims: replacement simulation descriptions, e.g. with scaled photon counts).
        device_labels=True builds every label volume on the GPU straight into the batch's label pool
        (umcx_job_build_labels at umcx_batch_labels), with no host volume at all."""
        sims = [j.sim for j in jobs] if sims is None else sims
        detpos = [j.detpos for j in jobs]
        if not device_labels:
            return cls(ctx, sims, [j.labels for j in jobs], [j.media for j in jobs], detpos)
        b = cls(ctx, sims, None, [j.media for j in jobs], detpos)
        for i, j in enumerate(jobs):
            j.build_labels(ctx, b.label_ptr(i))
        return b

    def label_ptr(self, i: int) -> int:
        """Device address of simulation i's uint8 labels in the batch's pool (umcx_batch_labels)."""
        p = load().umcx_batch_labels(self._h, int(i))
        if not p:
            raise IndexError(i)
        return int(p)

    def run(self) -> Result:
        """Run the whole batch once (graph launch); returns the summed tallies and the graph's device time."""
        r = Result()
        check(load().umcx_batch_run(self._h, C.byref(r)), self._ctx.handle, "umcx_batch_run")
        return r

    def get(self, i: int, out=None):
        """Simulation i's output volume [maxgate, nx, ny, nz] and tallies of the last run; out: an optional
        caller-owned contiguous float32 array of at least that many elements, reused instead of a new one."""
        s = self.sims[i]
        n = s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3]
        flu = None
        if s.issavevol:
            flu = np.zeros(n, np.float32) if out is None else out.reshape(-1)[:n]
            if flu.dtype != np.float32 or flu.size < n or not flu.flags.c_contiguous:
                raise ValueError("out must be a contiguous float32 array of nx*ny*nz*maxgate elements")
        r = Result()
        check(load().umcx_batch_get(self._h, int(i), None if flu is None else flu.ctypes.data, None, C.byref(r)),
              self._ctx.handle, "umcx_batch_get")
        if flu is not None:
            flu = flu.reshape(s.dim[3], s.dim[0], s.dim[1], s.dim[2])
        return flu, r

    def detp(self, i: int) -> np.ndarray:
        """Simulation i's detected-photon records of the last run, [saved, umcx_detp_columns] (L164-176)."""
        lib = load()
        r = Result()
        check(lib.umcx_batch_get(self._h, int(i), None, None, C.byref(r)), self._ctx.handle, "umcx_batch_get")
        cols = lib.umcx_detp_columns(C.byref(self.sims[i]))
        rows = np.zeros((int(r.saved), cols), np.float32)
        if rows.size:
            check(lib.umcx_batch_get(self._h, int(i), None, rows.ctypes.data, None), self._ctx.handle,
                  "umcx_batch_get")
        return rows

    def set_tuning(self, block_size: int = 0, blocks_per_sm: int = 0, aggregation: int = 0, budget_ms: int = 0):
        t = Tuning(block_size, blocks_per_sm, aggregation, budget_ms)
        check(load().umcx_batch_set_tuning(self._h, C.byref(t)), self._ctx.handle, "umcx_batch_set_tuning")

    def close(self):
        if getattr(self, "_h", None):
            load().umcx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def autotune_batch(ctx: Context, jobs, fraction: float = 0.05,
                   candidates=((256, 1), (512, 1), (1024, 1), (256, 2), (512, 2), (1024, 2)),
                   min_photons: int = 2000) -> dict:
    """Autotuner for batches: times a photon-scaled copy of the batch for each (block size, aggregation) candidate
    and returns the fastest configuration (apply it with Batch.set_tuning)."""
    sims = []
    for j in jobs:
        s = j.sim
        s.nphoton = min(s.nphoton, max(min_photons, int(s.nphoton * fraction)))
        sims.append(s)
    probe = Batch.from_jobs(ctx, jobs, device_labels=not all(j.has_host_labels for j in jobs), sims=sims)
    best = None
    for block, agg in candidates:
        probe.set_tuning(block, 0, agg)
        probe.run()
        ms = min(probe.run().kernel_ms for _ in range(3))  # fastest of three after a warm-up run
        if best is None or ms < best["probe_ms"]:
            best = {"block_size": block, "blocks_per_sm": 0, "aggregation": agg, "probe_ms": ms}
    probe.close()
    return best
