"""Synthetic benchmark configurations (reference-style JSON inputs), generated -- no dataset is read.

config1(), config2(), config3(): the three single-simulation benchmark configurations --
  1. homogeneous 60^3 cube of 1 mm voxels (label 1: mua 0.005/mm, mus 1/mm, g 0.01, n 1.37), pencil source at
     (29,29,0) along +z, 1e6 photons, one 0-5 ns gate, no boundary reflection;
  2. the same cube with a radius-15 sphere of label 2 (mua 0.002, mus 5, g 0.9, n 1.0) at (30,30,30), boundary
     reflection, 1e7 photons, 50 gates over 0-5 ns, four radius-1 disk detectors at z = 0 with partial paths saved;
  3. 200^3 voxels of 0.005 mm: 20 layers of air, 8 of label 1 (mua 3.56, mus 19.3, g 0.81, n 1.34), the rest label 2
     (mua 0.022, same scattering), a radius-20 cylinder along x of label 3 (mua 19.0, mus 64.5, g 0.9, n 1.36),
     a 0.3 mm disk source at the top-face centre along +z, 1e8 photons, one 0-1 ns gate, energy output.

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

_C1_MEDIA = [{"mua": 0, "mus": 0, "g": 1, "n": 1}, {"mua": 0.005, "mus": 1.0, "g": 0.01, "n": 1.37}]


def config1(photons: int = 1000000) -> dict:
    return {"Session": {"ID": "c1", "Photons": int(photons), "RNGSeed": 1648335518, "DoMismatch": 0,
                        "DoPartialPath": 0, "OutputType": "x"},
            "Forward": {"T0": 0, "T1": 5e-9, "Dt": 5e-9},
            "Domain": {"Dim": [60, 60, 60], "LengthUnit": 1, "Media": list(_C1_MEDIA)},
            "Optode": {"Source": {"Type": "pencil", "Pos": [29, 29, 0], "Dir": [0, 0, 1]}},
            "Shapes": [{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}]}


def config2(photons: int = 10000000) -> dict:
    return {"Session": {"ID": "c2", "Photons": int(photons), "RNGSeed": 1648335518, "DoMismatch": 1,
                        "DoPartialPath": 1, "SaveDetFlag": 5, "OutputType": "x"},
            "Forward": {"T0": 0, "T1": 5e-9, "Dt": 1e-10},
            "Domain": {"Dim": [60, 60, 60], "LengthUnit": 1,
                       "Media": list(_C1_MEDIA) + [{"mua": 0.002, "mus": 5.0, "g": 0.9, "n": 1.0}]},
            "Optode": {"Source": {"Type": "pencil", "Pos": [29, 29, 0], "Dir": [0, 0, 1]},
                       "Detector": [{"Pos": [29, 19, 0], "R": 1}, {"Pos": [19, 29, 0], "R": 1},
                                    {"Pos": [29, 39, 0], "R": 1}, {"Pos": [39, 29, 0], "R": 1}]},
            "Shapes": [{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}, {"Sphere": {"O": [30, 30, 30], "R": 15, "Tag": 2}}]}


def config3(photons: int = 100000000) -> dict:
    return {"Session": {"ID": "c3", "Photons": int(photons), "RNGSeed": 1648335518, "DoMismatch": 1,
                        "DoPartialPath": 0, "OutputType": "e"},
            "Forward": {"T0": 0, "T1": 1e-9, "Dt": 1e-9},
            "Domain": {"Dim": [200, 200, 200], "LengthUnit": 0.005,
                       "Media": [{"mua": 0, "mus": 0, "g": 1, "n": 1},
                                 {"mua": 3.56, "mus": 19.3, "g": 0.81, "n": 1.34},
                                 {"mua": 0.022, "mus": 19.3, "g": 0.81, "n": 1.34},
                                 {"mua": 19.0, "mus": 64.5, "g": 0.90, "n": 1.36}]},
            "Optode": {"Source": {"Type": "disk", "Pos": [100, 100, 0], "Dir": [0, 0, 1], "Param1": [60, 0, 0, 0]}},
            "Shapes": [{"Grid": {"Tag": 0, "Size": [200, 200, 200]}}, {"ZLayers": [[20, 28, 1], [28.5, 200, 2]]},
                       {"Cylinder": {"Tag": 3, "C0": [0, 100, 100], "C1": [200, 100, 100], "R": 20}}]}


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
