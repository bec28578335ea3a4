"""Generates tests/golden/reference_runs.json from the UNMODIFIED reference program (oracle/_ref/umcx, built from
the reference sources by oracle/build_ref.sh).

    python tests/golden/make_golden.py

For every case it records what the reference printed (absorbed %, detected count, normaliser, simulated energy)
and the SHA-256 of the files it wrote (--dumpmask label volumes, .bnii fluence, _detp.jdb detected photons).  The
reference runs single-threaded (OMP_NUM_THREADS=1), which makes its outputs deterministic.  The tests then check
that this repository's front end writes byte-identical label volumes and that the C oracle plus the repository's
writers reproduce the simulation outputs byte for byte.
"""
from __future__ import annotations

import base64
import hashlib
import json
import sys
import tempfile
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

C1 = {"Session": {"ID": "c1", "Photons": 20000, "RNGSeed": 1648335518, "DoMismatch": 0, "DoPartialPath": 0,
                  "OutputType": "x"},
      "Forward": {"T0": 0, "T1": 5e-9, "Dt": 5e-9},
      "Domain": {"Dim": [60, 60, 60], "LengthUnit": 1,
                 "Media": [{"mua": 0, "mus": 0, "g": 1, "n": 1}, {"mua": 0.005, "mus": 1.0, "g": 0.01, "n": 1.37}]},
      "Optode": {"Source": {"Type": "pencil", "Pos": [29, 29, 0], "Dir": [0, 0, 1]}},
      "Shapes": [{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}]}

C2 = {"Session": {"ID": "c2", "Photons": 20000, "RNGSeed": 1648335518, "DoMismatch": 1, "DoPartialPath": 1,
                  "SaveDetFlag": 5, "OutputType": "x"},
      "Forward": {"T0": 0, "T1": 5e-9, "Dt": 1e-10},
      "Domain": {"Dim": [60, 60, 60], "LengthUnit": 1,
                 "Media": [{"mua": 0, "mus": 0, "g": 1, "n": 1}, {"mua": 0.005, "mus": 1.0, "g": 0.01, "n": 1.37},
                           {"mua": 0.002, "mus": 5.0, "g": 0.9, "n": 1.0}]},
      "Optode": {"Source": {"Type": "pencil", "Pos": [29, 29, 0], "Dir": [0, 0, 1]},
                 "Detector": [{"Pos": [29, 19, 0], "R": 1}, {"Pos": [19, 29, 0], "R": 1},
                              {"Pos": [29, 39, 0], "R": 1}, {"Pos": [39, 29, 0], "R": 1}]},
      "Shapes": [{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}, {"Sphere": {"O": [30, 30, 30], "R": 15, "Tag": 2}}]}

C3 = {"Session": {"ID": "c3", "Photons": 2000, "RNGSeed": 1648335518, "DoMismatch": 1, "DoPartialPath": 0,
                  "OutputType": "e"},
      "Forward": {"T0": 0, "T1": 1e-9, "Dt": 1e-9},
      "Domain": {"Dim": [200, 200, 200], "LengthUnit": 0.005,
                 "Media": [{"mua": 0, "mus": 0, "g": 1, "n": 1}, {"mua": 3.56, "mus": 19.3, "g": 0.81, "n": 1.34},
                           {"mua": 0.022, "mus": 19.3, "g": 0.81, "n": 1.34},
                           {"mua": 19.0, "mus": 64.5, "g": 0.90, "n": 1.36}]},
      "Optode": {"Source": {"Type": "disk", "Pos": [100, 100, 0], "Dir": [0, 0, 1], "Param1": [60, 0, 0, 0]}},
      "Shapes": [{"Grid": {"Tag": 0, "Size": [200, 200, 200]}}, {"ZLayers": [[20, 28, 1], [28.5, 200, 2]]},
                 {"Cylinder": {"Tag": 3, "C0": [0, 100, 100], "C1": [200, 100, 100], "R": 20}}]}

# a small domain exercising every shape construct, an oblique cylinder and an interior detector
SHAPES = {"Session": {"ID": "shapes", "Photons": 5000, "DoMismatch": 1},
          "Forward": {"T0": 0, "T1": 5e-9, "Dt": 5e-10},
          "Domain": {"Dim": [40, 36, 32],
                     "Media": [[0, 0, 1, 1], [0.01, 1.0, 0.5, 1.37], [0.02, 2.0, 0.8, 1.4], [0.005, 0.5, 0.0, 1.33],
                               [0.03, 4.0, 0.9, 1.45]]},
          "Optode": {"Source": {"Type": "isotropic", "Pos": [20, 18, 16], "Dir": [0, 0, 1]},
                     "Detector": [{"Pos": [20, 18, 6], "R": 2}, {"Pos": [0, 10, 10], "R": 3},
                                  {"Pos": [39, 35, 31], "R": 2.5}]},
          "Shapes": [{"Grid": {"Tag": 0, "Size": [40, 36, 32]}},
                     {"Sphere": {"O": [20, 18, 16], "R": 10, "Tag": 1}},
                     {"XLayers": [[2, 6, 2], [30.5, 33, 3]]},
                     {"YLayers": [[0, 3, 4]]},
                     {"ZLayers": [[28, 32, 2]]},
                     {"Cylinder": {"Tag": 3, "C0": [5, 5, 5], "C1": [30, 25, 20], "R": 3.5}},
                     {"Name": "all shapes"}]}


def jdata_volume(compressed: bool):
    rng = np.random.default_rng(7)
    vol = rng.integers(0, 3, size=(12, 10, 8)).astype(np.uint8)
    vol[3:9, 3:7, 2:6] = 1
    cfg = json.loads(json.dumps(C1))
    cfg["Session"].update({"ID": "jdz" if compressed else "jd", "Photons": 5000, "DoMismatch": 1})
    cfg["Domain"]["Dim"] = [12, 10, 8]
    cfg["Domain"]["Media"] = [[0, 0, 1, 1], [0.01, 1.0, 0.5, 1.37], [0.02, 2.0, 0.7, 1.45]]
    cfg["Optode"]["Source"] = {"Type": "pencil", "Pos": [5.5, 5, 0], "Dir": [0, 0, 1]}
    cfg["Optode"]["Detector"] = [{"Pos": [5, 3, 0], "R": 2}]
    if compressed:
        cfg["Shapes"] = {"_ArraySize_": [12, 10, 8], "_ArrayType_": "uint8", "_ArrayZipType_": "zlib",
                         "_ArrayZipSize_": [1, 960],
                         "_ArrayZipData_": base64.b64encode(zlib.compress(vol.tobytes())).decode()}
    else:
        cfg["Shapes"] = {"_ArraySize_": [12, 10, 8], "_ArrayType_": "int32", "_ArrayData_": vol.ravel().tolist()}
    return cfg


def cases():
    """(name, kind, args-or-json).  kind 'mask' = --dumpmask, 'json' = --dumpjson, 'run' = simulation."""
    out = []
    benches = ["cube60", "cube60b", "cube60planar", "cubesph60b", "sphshells", "spherebox", "skinvessel"]
    for b in benches:
        out.append((f"mask_{b}", "mask", ["--bench", b]))
        out.append((f"json_{b}", "json", ["--bench", b]))
    for name, cfg in [("c1", C1), ("c2", C2), ("c3", C3), ("shapes", SHAPES), ("jd", jdata_volume(False)),
                      ("jdz", jdata_volume(True))]:
        out.append((f"mask_{name}", "mask", cfg))
    runs = [
        ("cube60", ["--bench", "cube60", "-n", "2e4"]),
        ("cube60b", ["--bench", "cube60b", "-n", "2e4"]),
        ("cube60planar", ["--bench", "cube60planar", "-n", "1e4"]),
        ("cubesph60b", ["--bench", "cubesph60b", "-n", "2e4"]),
        ("sphshells", ["--bench", "sphshells", "-n", "1e4"]),
        ("spherebox", ["--bench", "spherebox", "-n", "2e4"]),
        ("isotropic", ["--bench", "cube60", "--json", '{"Optode":{"Source":{"Type":"isotropic","Pos":[29,29,29]}}}',
                       "-n", "5e3"]),
        ("cone", ["--bench", "cube60", "--json",
                  '{"Domain":{"Media":[[0,0,1,1],[0.001,0.001,0,1]]},"Optode":{"Source":{"Type":"cone","Param1":[0.5,0,0,0]}}}',
                  "-n", "1e4"]),
        ("fourier", ["--bench", "cube60planar", "--json",
                     '{"Optode":{"Source":{"Type":"fourier","Param1":[40,0,0,2.25],"Param2":[0,40,0,1.5]}}}',
                     "-n", "1e4"]),
        ("outf", ["--bench", "cube60b", "-O", "f", "-n", "1e4"]),
        ("oute", ["--bench", "cube60b", "-O", "e", "-n", "1e4"]),
        ("nonorm", ["--bench", "cube60b", "-U", "0", "-n", "1e4"]),
        ("detflags", ["--bench", "cubesph60b", "-w", "53", "-n", "1e4"]),
        ("maxdet", ["--bench", "cube60b", "-H", "10", "-n", "1e4"]),
        ("nosave", ["--bench", "cube60b", "-S", "0", "-n", "1e4"]),
        ("seed", ["--bench", "cube60b", "-E", "12345", "-n", "1e4"]),
        ("unit", ["--bench", "cubesph60b", "-u", "0.5", "-n", "1e4"]),
    ]
    for name, args in runs:
        out.append((f"run_{name}", "run", args))
    for name, cfg in [("c1", C1), ("c2", C2), ("c3", C3), ("shapes", SHAPES), ("jd", jdata_volume(False)),
                      ("jdz", jdata_volume(True))]:
        out.append((f"run_{name}", "run", cfg))
    return out


def args_of(spec, sid: str) -> list[str]:
    if isinstance(spec, dict):
        cfg = json.loads(json.dumps(spec))
        cfg["Session"]["ID"] = sid
        return ["-j", json.dumps(cfg)]
    return [*spec, "-s", sid]


def sha(path: Path) -> str | None:
    return hashlib.sha256(path.read_bytes()).hexdigest() if path.exists() else None


def main() -> None:
    if not oracle.have_reference():
        raise SystemExit("oracle/_ref/umcx is missing: run `sh oracle/build_ref.sh` first")
    results = {}
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        for name, kind, spec in cases():
            sid = name
            args = args_of(spec, sid)
            if kind == "mask":
                r = oracle.run_reference([*args, "--dumpmask"], d)
                results[name] = {"kind": kind, "spec": spec, "sha_vol": sha(d / f"{sid}_vol.bnii")}
            elif kind == "json":
                r = oracle.run_reference([*args[:-2], "--dumpjson"], d)
                results[name] = {"kind": kind, "spec": spec,
                                 "sha_stdout": hashlib.sha256(r["stdout"].encode()).hexdigest()}
            else:
                r = oracle.run_reference(args, d, threads=1)
                results[name] = {"kind": kind, "spec": spec, "absorbed": r.get("absorbed"),
                                 "detected": r.get("detected"), "normalizer": r.get("normalizer"),
                                 "energy": r.get("energy"), "sha_bnii": sha(d / f"{sid}.bnii"),
                                 "sha_detp": sha(d / f"{sid}_detp.jdb")}
            print(name, {k: v for k, v in results[name].items() if k != "spec"}, flush=True)
    (HERE / "reference_runs.json").write_text(json.dumps(results, indent=1) + "\n")


if __name__ == "__main__":
    main()
