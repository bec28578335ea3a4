"""Statistical parity helpers: run the CUDA path and the CPU oracle on the same seeds, split into photon-index
batches, and compare means with batch standard errors (parity tolerance: 3 standard errors)."""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Batched:
    fluence: np.ndarray       # [B, gates, nx, ny, nz]
    absorbed: np.ndarray      # [B] absorbed fraction per batch
    total: np.ndarray         # [B]
    escape: np.ndarray        # [B]
    detp: list                # per batch detected rows
    results: list


def run_batches(fn, sim, nbatch: int) -> Batched:
    """fn(sim) -> (fluence, detp, result); photons [0, sim.nphoton) split into nbatch equal index ranges."""
    n = sim.nphoton
    per = n // nbatch
    flu, ab, tot, esc, dps, res = [], [], [], [], [], []
    for b in range(nbatch):
        s = sim.copy()
        s.photon_offset = sim.photon_offset + b * per
        s.nphoton = per
        f, d, r = fn(s)
        flu.append(np.asarray(f, np.float64))
        tot.append(r.energy_total)
        esc.append(r.energy_escape)
        ab.append((r.energy_total - r.energy_escape) / r.energy_total)
        dps.append(d)
        res.append(r)
    return Batched(np.stack(flu), np.array(ab), np.array(tot), np.array(esc), dps, res)


def mean_se(x: np.ndarray, axis=0):
    b = x.shape[axis]
    return x.mean(axis), x.std(axis, ddof=1) / math.sqrt(b)


@dataclass
class FluenceCompare:
    tested: int
    frac_over3: float
    mean_z: float
    mean_z2: float
    rel_l2: float


def compare_fluence(a: Batched, b: Batched, deposits: np.ndarray, min_deposits: int = 100) -> FluenceCompare:
    ma, sa = mean_se(a.fluence)
    mb, sb = mean_se(b.fluence)
    mask = (deposits >= min_deposits) & ((sa > 0) | (sb > 0))
    z = (ma[mask] - mb[mask]) / np.sqrt(sa[mask] ** 2 + sb[mask] ** 2)
    rel_l2 = float(np.linalg.norm(ma - mb) / max(np.linalg.norm(mb), 1e-300))
    return FluenceCompare(int(mask.sum()), float((np.abs(z) > 3).mean()) if z.size else 0.0,
                          float(z.mean()) if z.size else 0.0, float((z ** 2).mean()) if z.size else 0.0, rel_l2)


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
