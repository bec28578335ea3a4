"""Front-end parity with the reference's MCX_userio (no GPU): command lines, --dumpjson text, --dumpmask label
volumes (byte-identical .bnii files), job set-up and error messages.  Golden values come from the reference
program (tests/golden/make_golden.py)."""
import hashlib
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import args_of  # noqa: E402

GOLD = json.loads((ROOT / "tests" / "golden" / "reference_runs.json").read_text())
CLI = ROOT / "umcx_gb300" / "_build" / "umcx"


def cases(kind):
    return [k for k, v in GOLD.items() if v["kind"] == kind]


@pytest.mark.parametrize("name", cases("mask"))
def test_dumpmask_matches_reference(name, tmp_path):
    from umcx_gb300 import Job

    job = Job.from_args([*args_of(GOLD[name]["spec"], name), "--dumpmask"])
    assert job.action == 2
    path = tmp_path / f"{name}_vol.bnii"
    job.dump_mask(str(path))
    assert hashlib.sha256(path.read_bytes()).hexdigest() == GOLD[name]["sha_vol"]


@pytest.mark.parametrize("name", cases("json"))
def test_dumpjson_matches_reference(name):
    from umcx_gb300 import Job

    args = args_of(GOLD[name]["spec"], name)[:-2]
    job = Job.from_args([*args, "--dumpjson"])
    assert job.action == 1
    assert hashlib.sha256(job.console.encode()).hexdigest() == GOLD[name]["sha_stdout"]


def test_cli_dumpmask_and_help(tmp_path):
    p = subprocess.run([str(CLI), "--bench", "cubesph60b", "-s", "x", "--dumpmask"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert p.returncode == 0
    assert hashlib.sha256((tmp_path / "x_vol.bnii").read_bytes()).hexdigest() == GOLD["mask_cubesph60b"]["sha_vol"]
    h = subprocess.run([str(CLI)], capture_output=True, text=True)
    assert h.returncode == 0
    flags = set(__import__("re").findall(r"--[a-z]+", h.stdout))
    assert len(flags) >= 5 and "cube60" in h.stdout  # test/testumcx.sh:28-38
    j = subprocess.run([str(CLI), "--bench", "cube60", "--json",
                        '{"Optode":{"Source":{"Type":"isotropic","Pos":[29,29,29]}}}', "--dumpjson"],
                       capture_output=True, text=True)
    assert '"ID": "cube60"' in j.stdout and "isotropic" in j.stdout  # test/testumcx.sh:40-58


@pytest.mark.parametrize("args,msg", [
    (["--bench", "nosuch"], "benchmark nosuch is not found"),
    (["--bench", "cube60", "-n"], "incomplete input parameter: -n"),
    (["cube60", "extra"], "must use -flag or --flag to use more than 1 input"),
    (["--bench", "cube60", "--json", '{"Shapes":[{"Grid":{"Tag":1,"Size":[4,4,4]}},{"Torus":{}}]}'],
     "shape constructTorus is not supported"),
    (["--bench", "cube60", "--json", '{"Shapes":[{"Box":{"O":[0,0,0],"Size":[2,2,2],"Tag":1}}]}'],
     "type must be number, but is null"),
    (["--json", '{"Domain":{"Dim":[4,4,4],"Media":[[0,0,1,1]]},"Forward":{"T0":0,"T1":1e-9,"Dt":1e-9},'
                '"Optode":{"Source":{"Pos":[1,1,0],"Dir":[0,0,1]}},"Session":{"ID":"x"}}'],
     "type must be number, but is null"),
])
def test_input_errors(args, msg):
    from umcx_gb300 import Job

    with pytest.raises(ValueError) as e:
        Job.from_args(args)
    assert msg in str(e.value)


def test_cli_error_exit_code(tmp_path):
    p = subprocess.run([str(CLI), "--bench", "nosuch"], cwd=tmp_path, capture_output=True, text=True)
    assert p.returncode == 1
    assert "umcx encounters an error:" in p.stdout and "benchmark nosuch is not found" in p.stdout


def test_job_setup_matches_reference_rules():
    from umcx_gb300 import Job, seeds_from_rngseed

    job = Job.from_args(["--bench", "cubesph60b", "-n", "1e5", "-u", "0.5"])
    s = job.sim
    assert (s.dim[0], s.dim[1], s.dim[2], s.dim[3]) == (60, 60, 60, 1)
    assert s.nphoton == 100000 and s.isreflect == 1 and s.issavedet == 1 and s.savedetflag == 5
    assert s.mediumnum == 3 and s.detnum == 4 and s.srctype == 0 and s.maxdetphotons == 1000000
    # object media scale mua/mus by LengthUnit (L804)
    assert np.allclose(job.media[1], [0.005 * 0.5, 1.0 * 0.5, 0.01, 1.37])
    assert list(s.seeds) == list(seeds_from_rngseed(1648335518))
    lab = job.labels
    assert lab.shape == (60, 60, 60)
    assert set(np.unique(lab & 0x7F)) == {1, 2}
    det = (lab & 0x80) != 0
    assert det.sum() == 4 * 17 and det[:, :, 0].sum() == det.sum()  # boundary detector voxels on z=0 (L621)
    # array media are taken verbatim
    job2 = Job.from_args(["--bench", "cube60", "--json", '{"Domain":{"Media":[[0,0,1,1],[0.001,0.001,0,1]]}}'])
    assert np.allclose(job2.media[1], [0.001, 0.001, 0, 1])
    # normaliser (L820): fluence rate = rtstep / (total * u^2)
    assert abs(job.normalizer(1e5) - (1 / 5e-9) / (1e5 * 0.25)) < 1e-3
    # flags given before --bench are replaced by the benchmark (the reference applies arguments in order)
    job3 = Job.from_args(["-n", "5", "--bench", "cube60"])
    assert job3.sim.nphoton == 1000000


def test_label_out_of_media_is_rejected():
    from umcx_gb300 import Job

    with pytest.raises(ValueError, match="label 2 has no entry"):
        Job.from_args(["--bench", "cube60", "--json",
                       '{"Domain":{"Media":[[0,0,1,1],[0.01,1,0,1]]},"Shapes":[{"Grid":{"Tag":2,"Size":[8,8,8]}}]}'])


def test_config_roundtrip():
    from umcx_gb300 import Job

    cfg = Job.from_args(["--bench", "skinvessel"]).config
    assert cfg["Domain"]["LengthUnit"] == 0.005 and cfg["Optode"]["Source"]["Type"] == "disk"
    assert list(cfg["Shapes"][2]["Cylinder"].keys()) == ["C0", "C1", "R", "Tag"]  # key-sorted literal (L647)


@pytest.mark.parametrize("args,expect", [
    ([], {}),                                                        # neither key: the library's own launch
    (["-T", "256", "-t", "25600"], {"block_size": 256, "grid_size": 100}),
    (["-T", "256"], {"block_size": 256, "grid_size": 390}),          # ThreadNum defaults to 100000 (L739)
    (["-t", "6400"], {"block_size": 64, "grid_size": 100}),          # BlockSize defaults to 64 (L741)
    (["-T", "100", "-t", "1000"], {"block_size": 128, "grid_size": 10}),  # rounded up to whole warps
    (["--json", '{"Session":{"BlockSize":512,"ThreadNum":1000000}}'], {"block_size": 512, "grid_size": 1953}),
])
def test_launch_shape_flags(args, expect):
    """-T/--blocksize and -t/--thread (Session.BlockSize / ThreadNum) set the launch shape as the reference's GPU
    build does (src/umcx.cpp:739-741): CTAs of BlockSize threads, ThreadNum / BlockSize of them."""
    from umcx_gb300 import Job

    job = Job.from_args(["--bench", "cube60", "-n", "1000", *args])
    assert job.tuning == expect


def test_launch_shape_rejects_bad_block():
    from umcx_gb300 import Job

    with pytest.raises(ValueError, match="BlockSize"):
        Job.from_args(["--bench", "cube60", "-n", "1000", "-T", "2048"])
