"""The allocation-free entry point (umcx_gpu_forward_noalloc), called through the C ABI.

It serves callers that may not allocate device memory themselves or through the library (an application that owns
the GPU memory pool, a plugin inside another framework's allocator): they pass their own input and output buffers
and the kernel's working state lives in a fixed array inside the library.  The GPU tests check that two calls in a
row both reproduce the allocating entry point (umcx_gpu_forward_device with the same FP32 accumulation), so the
shared scratch array is correctly cleared between calls, for the fast and strict kernels, with the volume or the
detected photons switched off, and on a non-default stream.  The input checks (the same rules as the allocating
entry points, plus the fixed table size) run without a GPU: a rejected call returns before any CUDA call.  The file
sits on its own, collected last."""
import ctypes as C
import json
import math
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import C2  # noqa: E402

VARIANTS = {
    "fast": {},
    "strict": {"strict": True},
    "no_volume": {"issavevol": 0},
    "no_detectors": {"issavedet": 0},
    "side_stream": {"side_stream": True},
}


@pytest.mark.gpu
@pytest.mark.parametrize("variant", list(VARIANTS))
def test_noalloc_matches_allocating_entry_point_twice(variant):
    import torch

    from umcx_gb300 import Context, Job, Result, detp_columns, load
    from umcx_gb300._lib import SIM_FP32_ACCUM, SIM_STRICT_MATH

    opt = VARIANTS[variant]
    cfg = json.loads(json.dumps(C2))
    cfg["Session"]["Photons"] = 200000
    job = Job.from_json(cfg)
    sim = job.sim
    sim.flags = SIM_FP32_ACCUM | (SIM_STRICT_MATH if opt.get("strict") else 0)
    if "issavevol" in opt:
        sim.issavevol = opt["issavevol"]
    if "issavedet" in opt:
        sim.issavedet = opt["issavedet"]
        sim.maxdetphotons = 0
    nout = sim.dim[0] * sim.dim[1] * sim.dim[2] * sim.dim[3]
    cols = detp_columns(sim)
    ndet = max(1, sim.maxdetphotons * cols) if sim.issavedet else 1
    d_lab = torch.from_numpy(job.labels.ravel().copy()).cuda()
    media = np.ascontiguousarray(job.media, np.float32)
    det = np.ascontiguousarray(job.detpos, np.float32)
    stream = torch.cuda.Stream() if opt.get("side_stream") else torch.cuda.current_stream()

    ref_flu = torch.zeros(nout, dtype=torch.float32, device="cuda")
    ref_det = torch.zeros(ndet, dtype=torch.float32, device="cuda")
    with Context(0) as ctx:
        ref = ctx.forward_device(sim, d_lab, media, det, ref_flu if sim.issavevol else None,
                                 ref_det if sim.issavedet else None, stream)
    ref_flu_h = ref_flu.cpu().numpy()

    lib = load()
    for call in range(2):
        flu = torch.full((nout,), 7.0, dtype=torch.float32, device="cuda")  # stale contents must be overwritten
        dp = torch.zeros(ndet, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        res = Result()
        rc = lib.umcx_gpu_forward_noalloc(0, C.byref(sim), C.c_void_p(d_lab.data_ptr()), media.ctypes.data,
                                          det.ctypes.data, C.c_void_p(flu.data_ptr()) if sim.issavevol else None,
                                          C.c_void_p(dp.data_ptr()) if sim.issavedet else None,
                                          C.c_void_p(stream.cuda_stream), C.byref(res))
        assert rc == 0 and res.status == 0, (variant, call, rc)
        assert res.launched == sim.nphoton
        assert res.block_size > 0 and res.grid_size > 0
        # every photon's history is deterministic: counts match exactly
        assert (res.steps, res.crossings, res.scatters, res.detected) == (ref.steps, ref.crossings, ref.scatters,
                                                                          ref.detected), (variant, call)
        assert abs(res.energy_total - ref.energy_total) <= 1e-9 * ref.energy_total
        assert abs(res.energy_escape - ref.energy_escape) <= 1e-9 * ref.energy_total
        if sim.issavevol:
            # atomic accumulation order differs between runs: FP32 rounding of long sums (the source voxel collects
            # ~1e5 deposits into a value near 2e5, whose ulp is 1/64, so the order alone moves it by up to ~2e-4)
            np.testing.assert_allclose(flu.cpu().numpy(), ref_flu_h, rtol=1e-3, atol=1e-6)
        else:
            assert np.all(flu.cpu().numpy() == 7.0)  # no volume requested: the caller's buffer is left alone
        if sim.issavedet:
            rows = dp.cpu().numpy()[: res.saved * cols].reshape(-1, cols)
            ref_rows = ref_det.cpu().numpy()[: ref.saved * cols].reshape(-1, cols)
            order = np.lexsort(rows.T[::-1])
            ref_order = np.lexsort(ref_rows.T[::-1])
            np.testing.assert_allclose(rows[order], ref_rows[ref_order], rtol=1e-5, atol=1e-5)
        else:
            assert res.saved == 0


def _call_rejected(mutate, media_rows=None):
    """Calls the entry point with a description changed by `mutate`; the pointers are placeholders that a rejected
    call never touches (it returns before any CUDA call)."""
    from umcx_gb300 import Job, Result, load

    job = Job.from_args(["--bench", "cubesph60b", "-n", "1000"])
    sim = job.sim
    mutate(sim)
    rows = media_rows or max(sim.mediumnum, 1)
    media = np.zeros(rows * 4, np.float32)
    det = np.zeros(max(1, sim.detnum) * 4, np.float32)
    fake = C.c_void_p(0x1000)
    res = Result()
    rc = load().umcx_gpu_forward_noalloc(0, C.byref(sim), fake, media.ctypes.data, det.ctypes.data, fake, fake,
                                         None, C.byref(res))
    return rc, res


@pytest.mark.parametrize("what,mutate", [
    ("too many media", lambda s: setattr(s, "mediumnum", 129)),
    ("NaN end time", lambda s: setattr(s, "tend", math.nan)),
    ("infinite end time", lambda s: setattr(s, "tend", math.inf)),
    ("zero gate rate", lambda s: setattr(s, "rtstep", 0.0)),
    ("empty grid", lambda s: s.dim.__setitem__(0, 0)),
    ("no gates", lambda s: s.dim.__setitem__(3, 0)),
    ("negative detectors", lambda s: setattr(s, "detnum", -1)),
    ("too many detectors", lambda s: setattr(s, "detnum", 65)),
    ("unknown flags", lambda s: setattr(s, "flags", 0x80)),
    ("unknown source", lambda s: setattr(s, "srctype", 9)),
])
def test_noalloc_rejects_invalid_input(what, mutate):
    rc, res = _call_rejected(mutate)
    assert rc == 1 and res.status == 1, what
