"""The C++ front end under AddressSanitizer and UndefinedBehaviorSanitizer (no GPU).

tests/native/frontend_check.cpp drives frontend.cpp and jsonlite.cpp -- command-line and JSON parsing, built-in
benchmarks, shape rasterisation, JData volumes (plain and zipped), detector masking, job set-up and the .bnii /
_detp.jdb / --dumpmask writers -- over every input of the golden set plus invalid inputs.  A sanitizer report, a
leak or an uncaught exception fails the test; the label volumes built by the sanitizer build must equal the
library's."""
import json
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import args_of  # noqa: E402

GOLD = json.loads((ROOT / "tests" / "golden" / "reference_runs.json").read_text())
CSRC = ROOT / "umcx_gb300" / "csrc"

ERRORS = [
    (["--bench", "nosuch"], "benchmark nosuch is not found"),
    (["--bench", "cube60", "-n"], "incomplete input parameter: -n"),
    (["cube60", "extra"], "must use -flag or --flag"),
    (["--bench", "cube60", "--json", '{"Shapes":[{"Grid":{"Tag":1,"Size":[4,4,4]}},{"Torus":{}}]}'],
     "shape constructTorus is not supported"),
    (["--bench", "cube60", "--json", '{"Domain":{"Media":[[0,0,1,1],[0.01,1,0,1]]},'
                                     '"Shapes":[{"Grid":{"Tag":2,"Size":[8,8,8]}}]}'], "label 2 has no entry"),
    (["--json", '{"Session":'], ""),
    (["-f", "/nonexistent/input.json"], ""),
]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("asan") / "frontend_check"
    zlib = subprocess.run([gxx, "-x", "c", "-", "-lz", "-o", str(out) + ".probe"], input="int main(){return 0;}",
                          capture_output=True, text=True).returncode == 0
    cmd = [gxx, "-std=c++17", "-g", "-O1", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-ffp-contract=off", *(["-DUMCX_HAVE_ZLIB"] if zlib else []), str(CSRC / "frontend.cpp"),
           str(CSRC / "jsonlite.cpp"), str(ROOT / "tests" / "native" / "frontend_check.cpp"),
           *(["-lz"] if zlib else []), "-o", str(out)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0 and "sanitize" in p.stderr:
        pytest.skip("sanitizer runtime not available: " + p.stderr[-200:])
    assert p.returncode == 0, p.stderr[-2000:]
    return out, zlib


def run_checker(exe, inputs, cwd):
    text = "\n".join(json.dumps(x) for x in inputs) + "\n"
    env = {"ASAN_OPTIONS": "detect_leaks=1:abort_on_error=0", "UBSAN_OPTIONS": "print_stacktrace=1", "PATH": "/usr/bin:/bin"}
    p = subprocess.run([str(exe)], input=text, capture_output=True, text=True, cwd=cwd, env=env, timeout=600)
    assert p.returncode == 0, (p.returncode, p.stderr[-4000:])
    for marker in ("AddressSanitizer", "LeakSanitizer", "runtime error:"):
        assert marker not in p.stderr, p.stderr[-4000:]
    lines = p.stdout.splitlines()
    assert len(lines) == len(inputs), p.stdout[-2000:]
    return lines


def test_golden_inputs_clean_under_sanitizers(checker, tmp_path):
    exe, zlib = checker
    names = [k for k, v in GOLD.items() if zlib or not k.endswith("jdz")]
    inputs = []
    for k in names:
        args = args_of(GOLD[k]["spec"], k)
        if GOLD[k]["kind"] == "mask":
            args = [*args, "--dumpmask"]
        elif GOLD[k]["kind"] == "json":
            args = [*args[:-2], "--dumpjson"]
        inputs.append(args)
    inputs.append(["-h"])
    lines = run_checker(exe, inputs, tmp_path)
    bad = [(k, ln) for k, ln in zip(names, lines) if not ln.startswith("ok ")]
    assert not bad, bad
    # outputs were written: one volume per run with a saved volume, one mask per --dumpmask
    assert len(list(tmp_path.glob("*_vol.bnii"))) == sum(GOLD[k]["kind"] == "mask" for k in names)
    assert list(tmp_path.glob("*.bnii")) and list(tmp_path.glob("*_detp.jdb"))

    # the sanitizer build's label volumes are the library's
    from umcx_gb300 import Job

    for k, ln in zip(names, lines):
        if GOLD[k]["kind"] != "run":
            continue
        job = Job.from_args(args_of(GOLD[k]["spec"], k))
        _, _, nvox, labelsum, mediumnum, detnum = ln.split()
        assert int(nvox) == job.labels.size and int(labelsum) == int(job.labels.astype(np.uint64).sum()), k
        assert int(mediumnum) == job.sim.mediumnum and int(detnum) == job.sim.detnum, k


def test_invalid_inputs_clean_under_sanitizers(checker, tmp_path):
    exe, _ = checker
    json_obj = {"Session": {"ID": "j", "Photons": 10}, "Forward": {"T0": 0, "T1": 1e-9, "Dt": 1e-9},
                "Domain": {"Dim": [8, 8, 8], "Media": [[0, 0, 1, 1], [0.01, 1, 0.5, 1.37]]},
                "Optode": {"Source": {"Pos": [4, 4, 0], "Dir": [0, 0, 1]}},
                "Shapes": [{"Grid": {"Tag": 1, "Size": [8, 8, 8]}}]}
    inputs = [a for a, _ in ERRORS] + [json_obj]
    lines = run_checker(exe, inputs, tmp_path)
    for (args, msg), ln in zip(ERRORS, lines):
        assert ln.startswith("error "), (args, ln)
        assert msg in ln, (args, ln)
    assert lines[-1].startswith("ok run 512"), lines[-1]
