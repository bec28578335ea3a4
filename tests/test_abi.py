"""The C ABI library loads and exports every entry point declared in include/*.h (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "while", "return", "sizeof"):
                names.append(name)
    return sorted(set(names))


def test_header_lists_entry_points():
    names = declared_functions()
    for must in ("umcx_gpu_forward", "umcx_gpu_forward_device", "umcx_create", "MCX_run_cmd", "MCX_run_json",
                 "umcx_job_from_args", "umcx_seeds_from_rngseed"):
        assert must in names


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(name):
    from umcx_gb300 import load

    lib = load()
    assert hasattr(lib, name), f"{name} is declared in include/ but not exported by libumcx_gb300.so"


def test_production_build_has_no_device_checks():
    """The default build compiles the device bounds checks out (UMCX_DEVICE_CHECKS builds report 1)."""
    import os

    from umcx_gb300 import load

    expect = 1 if "UMCX_DEVICE_CHECKS=1" in os.environ.get("UMCX_NVCC_DEFS", "") else 0
    assert load().umcx_device_checks() == expect


def test_python_signatures_cover_header():
    from umcx_gb300._lib import SIGNATURES

    bound = {n for n, _, _ in SIGNATURES}
    missing = set(declared_functions()) - bound
    assert not missing, f"no ctypes signature for {sorted(missing)}"


def test_struct_layouts():
    from umcx_gb300._lib import Domain, Result, ShapeOp, Sim, Tuning

    assert C.sizeof(Sim) == 168
    assert C.sizeof(Result) == 104
    assert C.sizeof(Tuning) == 24
    assert C.sizeof(ShapeOp) == 48
    assert C.sizeof(Domain) == 56


def test_no_device_is_an_error_not_a_crash():
    import torch

    from umcx_gb300 import load

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = load()
    h = C.c_void_p()
    assert lib.umcx_create(C.byref(h), 0) != 0
    assert not h.value


def test_detp_columns():
    from umcx_gb300 import Sim, detp_columns

    s = Sim()
    s.mediumnum = 3
    for flag, cols in [(1, 1), (4, 3), (5, 4), (16, 3), (32, 3), (53, 10), (0, 0)]:
        s.savedetflag = flag
        assert detp_columns(s) == cols
