"""A plain-C program against the C ABI (tests/native/capi_forward.c): the headers compile as C and the program links
against libumcx_gb300.so (CPU); on a GPU it reproduces the reference's known answer for cube60 (17.x % absorbed)."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
BUILD = ROOT / "umcx_gb300" / "_build"


def build_program(tmp_path) -> Path:
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    exe = tmp_path / "capi_forward"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "native" / "capi_forward.c"), "-o", str(exe), f"-L{BUILD}", "-lumcx_gb300",
                    f"-Wl,-rpath,{BUILD}"], check=True)
    return exe


def test_c_program_builds_against_the_abi(tmp_path):
    assert build_program(tmp_path).exists()


@pytest.mark.gpu
def test_c_program_runs_cube60(tmp_path):
    exe = build_program(tmp_path)
    out = subprocess.run([str(exe), "--bench", "cube60", "-n", "1e6"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    m = re.search(r"absorbed (\S+) detected (\d+) launched (\d+)", out.stdout)
    assert m and int(m.group(3)) == 1000000
    assert 0.17 <= float(m.group(1)) < 0.18  # test/testumcx.sh: cube60 absorbs 17.x %
