"""Builds libumcx_gb300.so (CUDA kernels for sm_103a + C ABI + host front end) and the `umcx` program in-tree.

    python -m umcx_gb300.build            # or: from umcx_gb300.build import build; build()

Plain nvcc / g++ invocations run in parallel, no cmake.  Outputs go to umcx_gb300/_build/ (git-ignored).
Objects are rebuilt only when a source or header is newer than the object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INC = ROOT / "include"
OUT = PKG / "_build"
LIB = OUT / "libumcx_gb300.so"
CLI = OUT / "umcx"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]

# The production (fast-math) propagation kernels are compiled with --use_fast_math: single-precision denormals
# flushed to zero and the approximate division, square root and transcendentals (6-7 % faster on the benchmark
# configuration; the photon statistics are unchanged).  The strict instances keep IEEE arithmetic and no FMA
# contraction; the label builder (raster.cu) keeps IEEE arithmetic so that voxel-centre ties resolve as on the host.
FAST = ["--use_fast_math"]
CU_UNITS = {
    "capi.cu": [],
    "kernels_fast.cu": FAST,
    "kernels_fast_agg.cu": FAST,
    "kernels_strict.cu": ["--fmad=false"],
    "kernels_adjoint.cu": FAST,
    "kernels_batch.cu": FAST,
    "kernels_batch_det.cu": FAST,
    "peaks.cu": [],
    "noalloc.cu": [],
    "raster.cu": [],
}
CPP_UNITS = ["jsonlite.cpp", "frontend.cpp", "run.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _extra_defs() -> list[str]:
    """Extra -D definitions for nvcc from UMCX_NVCC_DEFS (space separated), for build variants."""
    return [f"-D{d}" for d in os.environ.get("UMCX_NVCC_DEFS", "").split() if d]


def _have_zlib() -> bool:
    return Path("/usr/include/zlib.h").exists() and any(
        Path(d, n).exists()
        for d in ("/usr/lib/x86_64-linux-gnu", "/usr/lib/aarch64-linux-gnu", "/usr/lib64", "/usr/lib", "/lib/x86_64-linux-gnu", "/lib/aarch64-linux-gnu")
        for n in ("libz.so", "libz.a"))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INC.glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str], log: Path) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    log.write_text(" ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}{proc.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    zlib = _have_zlib()
    hdrs = _headers()
    defs = ["-DUMCX_HAVE_ZLIB"] if zlib else []
    # the CUDA objects of another build variant (different UMCX_NVCC_DEFS) are rebuilt
    stamp = OUT / "nvcc_defs.txt"
    variant = " ".join(_extra_defs())
    rebuild_cu = not stamp.exists() or stamp.read_text() != variant
    steps = []
    objs = []
    for unit, extra in CU_UNITS.items():
        src = CSRC / unit
        obj = OUT / (unit + ".o")
        objs.append(obj)
        if rebuild_cu or _stale(obj, [src, *hdrs]):
            steps.append(([nvcc, *NVCC_FLAGS, *ARCH, *extra, *_extra_defs(), "-c", str(src), "-o", str(obj)],
                          OUT / (unit + ".log")))
    for unit in CPP_UNITS:
        src = CSRC / unit
        obj = OUT / (unit + ".o")
        objs.append(obj)
        if _stale(obj, [src, *hdrs]):
            steps.append((["g++", *CXX_FLAGS, *defs, "-c", str(src), "-o", str(obj)], OUT / (unit + ".log")))
    main_obj = OUT / "main.cpp.o"
    if _stale(main_obj, [CSRC / "main.cpp", *hdrs]):
        steps.append((["g++", *CXX_FLAGS, "-c", str(CSRC / "main.cpp"), "-o", str(main_obj)], OUT / "main.cpp.log"))
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_run, c, l) for c, l in steps]:
            f.result()
    if rebuild_cu:
        stamp.write_text(variant)
    if _stale(LIB, objs):
        libs = ["-lz"] if zlib else []
        _run([nvcc, "-shared", *ARCH, "-o", str(LIB), *map(str, objs), *libs], OUT / "link.log")
    if _stale(CLI, [LIB, main_obj]):
        _run(["g++", "-o", str(CLI), str(main_obj), f"-L{OUT}", "-lumcx_gb300", "-Wl,-rpath,$ORIGIN"], OUT / "cli.log")
    if verbose:
        for log in sorted(OUT.glob("*.log")):
            sys.stdout.write(log.read_text())
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
