"""Statistical parity helpers: run the CUDA path and the CPU oracle on the same seeds, split into photon-index
batches, and compare means with batch standard errors (parity tolerance: 3 standard errors).

Per-voxel batch statistics are accumulated as running means and sums of squared deviations (Welford), so that a
50-gate 60^3 volume over 20 batches needs three volumes of memory per side, not twenty."""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Batched:
    nbatch: int
    flu_mean: np.ndarray | None   # [gates, nx, ny, nz] mean over batches of each batch's output volume
    flu_m2: np.ndarray | None     # sum of squared deviations from the running mean
    absorbed: np.ndarray          # [B] absorbed fraction per batch
    total: np.ndarray             # [B]
    escape: np.ndarray            # [B]
    detp: list                    # per batch detected rows
    results: list
    depcount: np.ndarray | None = field(default=None)  # deposits per voxel summed over batches (oracle only)


def run_batches(fn, sim, nbatch: int) -> Batched:
    """fn(sim) -> (fluence, detp, result[, depcount]); photons [0, sim.nphoton) split into nbatch equal index
    ranges."""
    n = sim.nphoton
    per = n // nbatch
    mean = m2 = dep = None
    ab, tot, esc, dps, res = [], [], [], [], []
    for b in range(nbatch):
        s = sim.copy()
        s.photon_offset = sim.photon_offset + b * per
        s.nphoton = per
        out = fn(s)
        f, d, r = out[0], out[1], out[2]
        if f is not None:
            x = np.asarray(f, np.float64)
            if mean is None:
                mean = np.zeros_like(x)
                m2 = np.zeros_like(x)
            delta = x - mean
            mean += delta / (b + 1)
            m2 += delta * (x - mean)
        if len(out) > 3 and out[3] is not None:
            dep = out[3].astype(np.uint64) if dep is None else dep + out[3]
        tot.append(r.energy_total)
        esc.append(r.energy_escape)
        ab.append((r.energy_total - r.energy_escape) / r.energy_total)
        dps.append(d)
        res.append(r)
    return Batched(nbatch, mean, m2, np.array(ab), np.array(tot), np.array(esc), dps, res, dep)


def mean_se(x: np.ndarray, axis=0):
    b = x.shape[axis]
    return x.mean(axis), x.std(axis, ddof=1) / math.sqrt(b)


@dataclass
class FluenceCompare:
    tested: int          # voxels with at least min_deposits deposits (and a nonzero standard error)
    frac_over3: float    # fraction of them whose |z| exceeds 3
    max_abs_z: float
    mean_z: float
    mean_z2: float
    rel_l2: float        # ||mean_a - mean_b|| / ||mean_b|| over the whole volume


def compare_fluence(a: Batched, b: Batched, deposits: np.ndarray, min_deposits: int = 100) -> FluenceCompare:
    """z = (mean_a - mean_b) / sqrt(se_a^2 + se_b^2) per voxel, over voxels with >= min_deposits deposits."""
    sa = np.sqrt(a.flu_m2 / (a.nbatch - 1) / a.nbatch)
    sb = np.sqrt(b.flu_m2 / (b.nbatch - 1) / b.nbatch)
    mask = (deposits >= min_deposits) & ((sa > 0) | (sb > 0))
    z = (a.flu_mean[mask] - b.flu_mean[mask]) / np.sqrt(sa[mask] ** 2 + sb[mask] ** 2)
    rel_l2 = float(np.linalg.norm(a.flu_mean - b.flu_mean) / max(np.linalg.norm(b.flu_mean), 1e-300))
    if not z.size:
        return FluenceCompare(0, 0.0, 0.0, 0.0, 0.0, rel_l2)
    return FluenceCompare(int(mask.sum()), float((np.abs(z) > 3).mean()), float(np.abs(z).max()), float(z.mean()),
                          float((z ** 2).mean()), rel_l2)


def z_of_means(xa: np.ndarray, xb: np.ndarray) -> float:
    ma, sa = mean_se(xa)
    mb, sb = mean_se(xb)
    den = math.sqrt(sa * sa + sb * sb)
    return float((ma - mb) / den) if den > 0 else (0.0 if ma == mb else float("inf"))


def det_stats(rows_list, detnum: int, ppath_cols: slice):
    """Per detector: photon count, mean partial paths and their standard errors from the pooled rows."""
    rows = np.concatenate([r for r in rows_list if r is not None and len(r)], axis=0) if any(
        r is not None and len(r) for r in rows_list) else np.zeros((0, 1))
    out = []
    for d in range(1, detnum + 1):
        sel = rows[rows[:, 0] == d] if len(rows) else rows
        pp = sel[:, ppath_cols] if len(sel) else np.zeros((0, 1))
        n = len(sel)
        mean = pp.mean(0) if n else np.zeros(pp.shape[1])
        se = pp.std(0, ddof=1) / math.sqrt(n) if n > 1 else np.full(pp.shape[1], np.inf)
        out.append((n, mean, se))
    return out
