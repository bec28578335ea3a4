"""Synthetic benchmark configurations (reference-style JSON inputs), generated -- no dataset is read.

config5(i): simulation i of the batched benchmark -- cubic domain with edge drawn from {32, 48, 64, 96, 128} voxels
of 1 mm, 2-5 tissue labels made of a random background plus random spheres (radius 5-30 % of the edge) and
z-slabs, per-label mua U[0.001, 0.05]/mm, mus U[0.5, 20]/mm, g U[0, 0.95], n U[1.33, 1.45], a photon budget
log-uniform in [1e5, 1e7], a pencil or isotropic source at a random point of a random face pointing inwards,
10 time gates over 0-5 ns, fluence output, boundary reflection on.  Everything is drawn from
numpy.random.default_rng(i); the RNG seed of simulation i is derived from i.
"""
from __future__ import annotations

import numpy as np

EDGES = (32, 48, 64, 96, 128)


def config5(i: int, photon_scale: float = 1.0, max_edge: int | None = None) -> dict:
    rng = np.random.default_rng(i)
    edges = [e for e in EDGES if max_edge is None or e <= max_edge]
    edge = int(rng.choice(edges))
    nlab = int(rng.integers(2, 6))  # tissue labels 1..nlab
    media = [{"mua": 0.0, "mus": 0.0, "g": 1.0, "n": 1.0}]
    for _ in range(nlab):
        media.append({"mua": float(rng.uniform(0.001, 0.05)), "mus": float(rng.uniform(0.5, 20.0)),
                      "g": float(rng.uniform(0.0, 0.95)), "n": float(rng.uniform(1.33, 1.45))})
    shapes = [{"Grid": {"Tag": 1, "Size": [edge, edge, edge]}}]
    for tag in range(2, nlab + 1):
        if rng.random() < 0.6:
            r = float(rng.uniform(0.05, 0.30)) * edge
            o = [float(rng.uniform(r, edge - r)) for _ in range(3)]
            shapes.append({"Sphere": {"O": o, "R": r, "Tag": tag}})
        else:
            z0 = float(rng.uniform(0, edge * 0.8))
            z1 = float(min(edge, z0 + rng.uniform(0.05, 0.3) * edge))
            shapes.append({"ZLayers": [[z0, z1, tag]]})
    photons = int(10 ** rng.uniform(5, 7) * photon_scale)
    face = int(rng.integers(0, 6))
    axis, side = face // 2, face % 2
    pos = [float(rng.uniform(0.5, edge - 0.5)) for _ in range(3)]
    pos[axis] = 0.0 if side == 0 else float(edge) - 1e-3
    direction = [0.0, 0.0, 0.0]
    direction[axis] = 1.0 if side == 0 else -1.0
    stype = "pencil" if rng.random() < 0.5 else "isotropic"
    return {
        "Session": {"ID": f"c5_{i}", "Photons": max(photons, 1000), "RNGSeed": int(1 + (1648335518 + 7919 * i) % 2147483646),
                    "DoMismatch": 1, "DoPartialPath": 0, "OutputType": "x"},
        "Forward": {"T0": 0.0, "T1": 5e-9, "Dt": 5e-10},
        "Domain": {"Dim": [edge, edge, edge], "LengthUnit": 1.0, "Media": media},
        "Optode": {"Source": {"Type": stype, "Pos": pos, "Dir": direction}},
        "Shapes": shapes,
    }


def batch5(n: int = 256, photon_scale: float = 1.0, max_edge: int | None = None, device_labels: bool = False):
    """Jobs of the batched benchmark (umcx_gb300.Job objects); device_labels=True leaves the label volumes to be
    built on the GPU (Batch.from_jobs(..., device_labels=True))."""
    from .api import Job

    return [Job.from_json(config5(i, photon_scale, max_edge), device_labels) for i in range(n)]
