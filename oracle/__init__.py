"""CPU oracle of the umcx photon-transport hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may use this package, and only
as the reference results that GPU outputs are compared with, or as the timed CPU baseline.  The product (umcx_gb300/) never imports it.

Two reference implementations live here:
  * libumcx_oracle.so, a plain-C restatement of the reference's photon loop (umcx_oracle.c), pinned bit-for-bit
    against the reference's own outputs (tests/test_oracle_pin.py);
  * oracle/_ref/umcx, the UNMODIFIED reference program built from its sources by build_ref.sh (git-ignored).
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB_PATH = BUILD / "libumcx_oracle.so"
REF_DIR = HERE / "_ref"
REF_BIN = REF_DIR / "umcx"

_lib = None


def reference_root() -> Path | None:
    """Checkout of the reference project: $UMCX_REFERENCE_ROOT, else a `reference` directory beside this repository;
    None when neither holds src/umcx.cpp (on a host that only has the staged copy under oracle/_ref/)."""
    for cand in (os.environ.get("UMCX_REFERENCE_ROOT"), str(HERE.parent.parent / "reference")):
        if cand and Path(cand, "src", "umcx.cpp").exists():
            return Path(cand)
    return None


def _ref_root_arg(root: str | None) -> str:
    if root is None:
        found = reference_root()
        return str(found) if found else ""
    return root


def build(reference_root: str | None = None) -> None:
    """Compile the C oracle and (when its sources are reachable) the reference program.  reference_root None looks
    the checkout up (see reference_root()); "" uses only the staged copy."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "umcx_oracle.c"
    hdr = HERE.parent / "include" / "umcx_gpu.h"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", str(LIB_PATH),
                        str(src), "-lm"], check=True)
    root = _ref_root_arg(reference_root)
    if (root and Path(root, "src", "umcx.cpp").exists()) or (REF_DIR / "src" / "umcx.cpp").exists():
        subprocess.run(["sh", str(HERE / "build_ref.sh"), root], check=True, stdout=subprocess.DEVNULL)


def start_build_ref(reference_root: str | None = None):
    """Start building the reference program in the background; returns the Popen (or None)."""
    root = _ref_root_arg(reference_root)
    if (root and Path(root, "src", "umcx.cpp").exists()) or (REF_DIR / "src" / "umcx.cpp").exists():
        return subprocess.Popen(["sh", str(HERE / "build_ref.sh"), root], stdout=subprocess.DEVNULL)
    return None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        from umcx_gb300._lib import Result, Sim

        lib = C.CDLL(str(LIB_PATH))
        lib.oracle_forward.restype = C.c_int
        lib.oracle_forward.argtypes = [C.POINTER(Sim), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.POINTER(Result), C.c_int]
        lib.oracle_seeds.restype = C.c_int
        lib.oracle_seeds.argtypes = [C.c_int32, C.POINTER(C.c_uint32)]
        lib.oracle_rng_dump.restype = None
        lib.oracle_rng_dump.argtypes = [C.POINTER(C.c_uint32), C.c_uint64, C.c_int, C.c_void_p]
        lib.oracle_trace_photon.restype = C.c_int
        lib.oracle_trace_photon.argtypes = [C.POINTER(Sim), C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                            C.c_void_p, C.c_void_p, C.c_int]
        lib.oracle_detp_columns.restype = C.c_int
        lib.oracle_detp_columns.argtypes = [C.POINTER(Sim)]
        _lib = lib
    return _lib


def forward(sim, labels, media, detpos=None, nthreads: int = 0, depcount: bool = False):
    """Run photons [sim.photon_offset, +sim.nphoton) on the CPU. Returns (fluence, detp, result, depcount)."""
    from umcx_gb300._lib import Result

    lib = load()
    lab = np.ascontiguousarray(labels, np.uint8)
    med = np.ascontiguousarray(media, np.float32)
    det = np.ascontiguousarray(detpos if detpos is not None else np.zeros((0, 4)), np.float32)
    nout = sim.dim[0] * sim.dim[1] * sim.dim[2] * sim.dim[3]
    flu = np.zeros(nout, np.float32)
    cols = lib.oracle_detp_columns(C.byref(sim))
    dp = np.zeros(max(1, sim.maxdetphotons * cols), np.float32) if sim.issavedet else None
    dc = np.zeros(nout, np.uint32) if depcount else None
    res = Result()
    rc = lib.oracle_forward(C.byref(sim), lab.ctypes.data, med.ctypes.data, det.ctypes.data if det.size else None,
                            flu.ctypes.data, None if dp is None else dp.ctypes.data,
                            None if dc is None else dc.ctypes.data, C.byref(res), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle_forward failed: {rc}")
    shape = (sim.dim[3], sim.dim[0], sim.dim[1], sim.dim[2])
    if dp is not None:
        dp = dp[: res.saved * cols].reshape(res.saved, cols)
    return flu.reshape(shape), dp, res, (None if dc is None else dc.reshape(shape))


def seeds(rngseed: int) -> np.ndarray:
    out = (C.c_uint32 * 4)()
    load().oracle_seeds(int(rngseed), out)
    return np.array(list(out), np.uint32)


def rng_dump(seed4, photon: int, ndraw: int) -> np.ndarray:
    s = (C.c_uint32 * 4)(*[int(x) for x in seed4])
    out = np.zeros(ndraw, np.float32)
    load().oracle_rng_dump(s, int(photon), int(ndraw), out.ctypes.data)
    return out


def trace(sim, labels, media, detpos, photon: int, maxrows: int = 4096) -> np.ndarray:
    """Event rows {kind, x, y, z, w, vx, vy, vz} of one photon (kind 0 launch, 1 crossing, 2 scatter)."""
    lab = np.ascontiguousarray(labels, np.uint8)
    med = np.ascontiguousarray(media, np.float32)
    det = np.ascontiguousarray(detpos if detpos is not None else np.zeros((0, 4)), np.float32)
    scratch = np.zeros(sim.dim[0] * sim.dim[1] * sim.dim[2] * sim.dim[3], np.float32)
    rows = np.zeros((maxrows, 8), np.float32)
    n = load().oracle_trace_photon(C.byref(sim), lab.ctypes.data, med.ctypes.data, det.ctypes.data if det.size else None,
                                   int(photon), scratch.ctypes.data, rows.ctypes.data, maxrows)
    return rows[:n]


# ---------------------------------------------------------------------------------------------- reference program
LINE_RE = re.compile(
    r"simulated energy ([0-9.eE+-]+), speed ([0-9.eE+-]+) photon/ms, duration ([0-9.eE+-]+) ms, "
    r"normalizer ([0-9.eE+-]+), detected (-?\d+), absorbed ([0-9.eE+-]+)%")


def parse_line(text: str) -> dict | None:
    m = LINE_RE.search(text)
    if not m:
        return None
    return {"energy": float(m.group(1)), "speed": float(m.group(2)), "duration_ms": float(m.group(3)),
            "normalizer": float(m.group(4)), "detected": int(m.group(5)), "absorbed": float(m.group(6))}


def have_reference() -> bool:
    return REF_BIN.exists() and os.access(REF_BIN, os.X_OK)


def run_reference(args: list[str], cwd: str | Path, threads: int = 1, timeout: float = 600) -> dict:
    """Run the unmodified reference program; returns the parsed console line plus raw stdout."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    p = subprocess.run([str(REF_BIN), *args], cwd=str(cwd), env=env, capture_output=True, text=True, timeout=timeout)
    out = parse_line(p.stdout) or {}
    out["stdout"] = p.stdout
    out["returncode"] = p.returncode
    return out


# ---------------------------------------------------------------------------------------------- BJData reader
def read_bjdata(path_or_bytes) -> object:
    """Minimal BJData Draft-2 reader for the .bnii / _detp.jdb files (containers, numbers, strings, ND-arrays)."""
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else Path(path_or_bytes).read_bytes()
    pos = 0
    ints = {"i": "<i1", "U": "<u1", "I": "<i2", "u": "<u2", "l": "<i4", "m": "<u4", "L": "<i8", "M": "<u8",
            "d": "<f4", "D": "<f8", "C": "<u1"}

    def num(m):
        nonlocal pos
        dt = np.dtype(ints[m])
        v = np.frombuffer(data, dt, 1, pos)[0]
        pos += dt.itemsize
        return v.item()

    def count():
        nonlocal pos
        m = chr(data[pos])
        pos += 1
        return int(num(m))

    def string_body():
        nonlocal pos
        n = count()
        s = data[pos:pos + n].decode()
        pos += n
        return s

    def value(m=None):
        nonlocal pos
        if m is None:
            m = chr(data[pos])
            pos += 1
        if m in ints:
            return num(m)
        if m == "S":
            return string_body()
        if m == "T":
            return True
        if m == "F":
            return False
        if m == "Z":
            return None
        if m == "[":
            typ = None
            if chr(data[pos]) == "$":
                typ = chr(data[pos + 1])
                pos += 2
            if chr(data[pos]) == "#":
                pos += 1
                if chr(data[pos]) == "[":  # ND-array dims
                    pos += 1
                    dims = value("[")
                    dt = np.dtype(ints[typ])
                    n = int(np.prod(dims)) if len(dims) else 0
                    arr = np.frombuffer(data, dt, n, pos).copy().reshape(dims)
                    pos += n * dt.itemsize
                    return arr
                n = count()
                if typ is not None and typ in ints:
                    dt = np.dtype(ints[typ])
                    arr = np.frombuffer(data, dt, n, pos).copy()
                    pos += n * dt.itemsize
                    return arr.tolist()
                return [value(typ) for _ in range(n)]
            out = []
            while chr(data[pos]) != "]":
                out.append(value())
            pos += 1
            return out
        if m == "{":
            typ = None
            if chr(data[pos]) == "$":
                typ = chr(data[pos + 1])
                pos += 2
            out = {}
            if chr(data[pos]) == "#":
                pos += 1
                n = count()
                for _ in range(n):
                    k = string_body()
                    out[k] = value(typ)
                return out
            while chr(data[pos]) != "}":
                k = string_body()
                out[k] = value(typ)
            pos += 1
            return out
        raise ValueError(f"unsupported BJData marker {m!r} at {pos - 1}")

    return value()
