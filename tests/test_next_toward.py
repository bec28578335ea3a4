"""The fast path's nextafterf restatement (umcx_gb300/csrc/next_toward.h) against the C library's nextafterf, on the
host (the same header compiles for the device)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_next_toward_matches_nextafterf(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = tmp_path / "next_toward_test"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(ROOT / "tests" / "native" / "next_toward_test.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout
