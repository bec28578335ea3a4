"""The allocation-free entry point (umcx_gpu_forward_noalloc), called through the C ABI.

It serves callers that may not allocate device memory themselves or through the library (an application that owns
the GPU memory pool, a plugin inside another framework's allocator): they pass their own input and output buffers
and the kernel's working state lives in a fixed array inside the library.  This test checks that two calls in a
row both reproduce the allocating entry point (umcx_gpu_forward_device with the same FP32 accumulation), so the
shared scratch array is correctly cleared between calls.  It sits in its own file, collected last."""
import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import C2  # noqa: E402

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point_twice():
    import torch

    from umcx_gb300 import Context, Job, Result, load
    from umcx_gb300._lib import SIM_FP32_ACCUM

    cfg = json.loads(json.dumps(C2))
    cfg["Session"]["Photons"] = 200000
    job = Job.from_json(cfg)
    sim = job.sim
    sim.flags = SIM_FP32_ACCUM
    nout = sim.dim[0] * sim.dim[1] * sim.dim[2] * sim.dim[3]
    cols = 4
    d_lab = torch.from_numpy(job.labels.ravel().copy()).cuda()
    media = np.ascontiguousarray(job.media, np.float32)
    det = np.ascontiguousarray(job.detpos, np.float32)

    ref_flu = torch.zeros(nout, dtype=torch.float32, device="cuda")
    ref_det = torch.zeros(sim.maxdetphotons * cols, dtype=torch.float32, device="cuda")
    with Context(0) as ctx:
        ref = ctx.forward_device(sim, d_lab, media, det, ref_flu, ref_det, torch.cuda.current_stream())
    ref_flu_h = ref_flu.cpu().numpy()

    lib = load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        flu = torch.full((nout,), 7.0, dtype=torch.float32, device="cuda")  # stale contents must be overwritten
        dp = torch.zeros(sim.maxdetphotons * cols, dtype=torch.float32, device="cuda")
        res = Result()
        rc = lib.umcx_gpu_forward_noalloc(0, C.byref(sim), C.c_void_p(d_lab.data_ptr()), media.ctypes.data,
                                          det.ctypes.data, C.c_void_p(flu.data_ptr()), C.c_void_p(dp.data_ptr()),
                                          stream, C.byref(res))
        assert rc == 0 and res.status == 0, (call, rc)
        assert res.launched == sim.nphoton
        # every photon's history is deterministic: counts match exactly
        assert (res.steps, res.crossings, res.scatters, res.detected) == (ref.steps, ref.crossings, ref.scatters,
                                                                          ref.detected), call
        assert abs(res.energy_total - ref.energy_total) <= 1e-9 * ref.energy_total
        assert abs(res.energy_escape - ref.energy_escape) <= 1e-9 * ref.energy_total
        # atomic accumulation order differs between runs: FP32 rounding of long sums (the source voxel collects
        # ~1e5 deposits into a value near 2e5, whose ulp is 1/64, so the order alone moves it by up to ~2e-4)
        np.testing.assert_allclose(flu.cpu().numpy(), ref_flu_h, rtol=1e-3, atol=1e-6)
        rows = dp.cpu().numpy()[: res.saved * cols].reshape(-1, cols)
        ref_rows = ref_det.cpu().numpy()[: ref.saved * cols].reshape(-1, cols)
        order = np.lexsort(rows.T[::-1])
        ref_order = np.lexsort(ref_rows.T[::-1])
        np.testing.assert_allclose(rows[order], ref_rows[ref_order], rtol=1e-5, atol=1e-5)


def test_noalloc_rejects_too_many_media():
    import torch

    from umcx_gb300 import Job, Result, load

    job = Job.from_args(["--bench", "cube60", "-n", "1000"])
    sim = job.sim
    sim.mediumnum = 129  # beyond the fixed scratch array's table
    d = torch.zeros(8, dtype=torch.uint8, device="cuda")
    media = np.zeros(129 * 4, np.float32)
    det = np.ascontiguousarray(job.detpos, np.float32)
    res = Result()
    rc = load().umcx_gpu_forward_noalloc(0, C.byref(sim), C.c_void_p(d.data_ptr()), media.ctypes.data,
                                         det.ctypes.data, C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()),
                                         None, C.byref(res))
    assert rc == 1
