"""torch.autograd harness around the C-ABI forward/backward pair (used by the tests only).

PhotonTransport.apply(mua, mus, context, job) returns
  readings  [detnum, maxgate]  detected exit weight per launched photon, per detector and time gate
  total     []                 sum of the raw (un-normalised) output volume
as differentiable functions of the per-label mua and mus (per-voxel units, the media table's).  Gradients come
from umcx_gpu_backward: per-label derivatives from the detected photons' partial paths and scatter counts, and the
summed-volume derivatives tallied during the forward pass.
"""
from __future__ import annotations

import numpy as np
import torch


class PhotonTransport(torch.autograd.Function):
    @staticmethod
    def forward(fctx, mua, mus, context, job, sim=None):
        sim = (sim or job.sim).copy()
        media = job.media.copy()
        media[:, 0] = mua.detach().cpu().numpy().astype(np.float32)
        media[:, 1] = mus.detach().cpu().numpy().astype(np.float32)
        out = context.forward_adjoint(sim, job.labels, media, job.detpos)
        adj = context.backward()
        n = float(sim.nphoton)
        fctx.save_for_backward(torch.from_numpy(adj["dread_dmua"] / n), torch.from_numpy(adj["dread_dmus"] / n),
                               torch.from_numpy(adj["dflu_dmua"]), torch.from_numpy(adj["dflu_dmus"]))
        readings = torch.from_numpy(adj["readings"] / n)
        total = torch.tensor(float(out.fluence.astype(np.float64).sum()) if out.fluence is not None else 0.0,
                             dtype=torch.float64)
        return readings, total

    @staticmethod
    def backward(fctx, g_read, g_total):
        d_mua, d_mus, f_mua, f_mus = fctx.saved_tensors
        g_read = g_read.to(torch.float64)
        g_total = g_total.to(torch.float64)
        gmua = torch.einsum("dt,dtk->k", g_read, d_mua) + g_total * f_mua
        gmus = torch.einsum("dt,dtk->k", g_read, d_mus) + g_total * f_mus
        return gmua, gmus, None, None, None
