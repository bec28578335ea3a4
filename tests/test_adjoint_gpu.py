"""Adjoint / replay parity (GPU required).

Configuration 4: the configuration-1 medium and grid (60^3 homogeneous label 1, pencil beam, no reflection) with
configuration 2's four detectors and 50 gates.  Checks:
  * mua gradients of detector readings and of the summed output against central finite differences (1 % steps)
    under common random numbers -- changing mua leaves every path unchanged, so the agreement is tight;
  * mus gradients (path-score estimator) against central finite differences under common random numbers, within
    their combined statistical error;
  * the reference's own pathlength-derived sensitivities (-sum w L_k / N with w = exp(-sum mua_k L_k), from the
    oracle's detected-photon partial paths) within 3 standard errors;
  * the replay Jacobian: every recorded photon replays to the same exit, and the Jacobian summed over each label's
    voxels equals that label's mua derivative of the readings;
  * the torch.autograd harness delivers the same vector-Jacobian products."""
import json
import math
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import C1, C2  # noqa: E402

pytestmark = pytest.mark.gpu


def config4(photons: int, output="x"):
    cfg = json.loads(json.dumps(C1))
    cfg["Session"].update({"ID": "c4", "Photons": int(photons), "DoPartialPath": 1, "SaveDetFlag": 5,
                           "OutputType": output})
    cfg["Forward"] = dict(C2["Forward"])
    cfg["Optode"]["Detector"] = json.loads(json.dumps(C2["Optode"]["Detector"]))
    return cfg


def job4(photons, output="x"):
    from umcx_gb300 import Job

    return Job.from_json(config4(photons, output))


def run(ctx, job, media, sim=None):
    s = (sim or job.sim).copy()
    out = ctx.forward_adjoint(s, job.labels, media, job.detpos)
    adj = ctx.backward()
    return out, adj


def test_mua_gradients_match_finite_differences(ctx):
    job = job4(200000)
    media = job.media
    out, adj = run(ctx, job, media)
    assert adj["records"] == out.result.saved > 100
    k = 1
    h = 0.01 * media[k, 0]
    mp, mm = media.copy(), media.copy()
    mp[k, 0] += h
    mm[k, 0] -= h
    op, ap = run(ctx, job, mp)
    om, am = run(ctx, job, mm)
    # identical paths: the detected set and the step counts do not change with mua
    assert op.result.steps == om.result.steps == out.result.steps
    fd_read = (ap["readings"] - am["readings"]) / (2 * h)
    grad = adj["dread_dmua"][:, :, k]
    tot_fd, tot_ad = fd_read.sum(), grad.sum()
    print(f"readings d/dmua: adjoint {tot_ad:.6e} FD {tot_fd:.6e}")
    assert abs(tot_ad - tot_fd) <= 1e-3 * abs(tot_fd)
    big = np.abs(fd_read) > 1e-3 * np.abs(fd_read).max()
    np.testing.assert_allclose(grad[big], fd_read[big], rtol=2e-3)
    fd_flu = (op.fluence.astype(np.float64).sum() - om.fluence.astype(np.float64).sum()) / (2 * h)
    print(f"sum(volume) d/dmua: adjoint {adj['dflu_dmua'][k]:.6e} FD {fd_flu:.6e}")
    assert abs(adj["dflu_dmua"][k] - fd_flu) <= 2e-3 * abs(fd_flu)


def test_mua_gradient_energy_output(ctx):
    job = job4(100000, output="e")
    media = job.media
    out, adj = run(ctx, job, media)
    k = 1
    h = 0.01 * media[k, 0]
    mp, mm = media.copy(), media.copy()
    mp[k, 0] += h
    mm[k, 0] -= h
    op, _ = run(ctx, job, mp)
    om, _ = run(ctx, job, mm)
    fd = (op.fluence.astype(np.float64).sum() - om.fluence.astype(np.float64).sum()) / (2 * h)
    assert abs(adj["dflu_dmua"][k] - fd) <= 2e-3 * abs(fd)


def test_mus_gradients_match_finite_differences(ctx):
    """Score-function (adjoint) vs common-random-number finite differences, batch statistics."""
    nb, per = 8, 250000
    job = job4(per)
    media = job.media
    k = 1
    h = 0.01 * media[k, 1]
    mp, mm = media.copy(), media.copy()
    mp[k, 1] += h
    mm[k, 1] -= h
    ad_r, fd_r, ad_f, fd_f = [], [], [], []
    for b in range(nb):
        s = job.sim
        s.photon_offset = b * per
        o, a = run(ctx, job, media, s)
        op, ap = run(ctx, job, mp, s)
        om, am = run(ctx, job, mm, s)
        ad_r.append(a["dread_dmus"][:, :, k].sum())
        fd_r.append((ap["readings"].sum() - am["readings"].sum()) / (2 * h))
        ad_f.append(a["dflu_dmus"][k])
        fd_f.append((op.fluence.astype(np.float64).sum() - om.fluence.astype(np.float64).sum()) / (2 * h))
    for name, x, y in [("readings", ad_r, fd_r), ("volume", ad_f, fd_f)]:
        x, y = np.array(x), np.array(y)
        se = math.sqrt(x.var(ddof=1) / nb + y.var(ddof=1) / nb)
        print(f"d/dmus {name}: adjoint {x.mean():.5e} +- {x.std(ddof=1) / math.sqrt(nb):.2e}, "
              f"FD {y.mean():.5e} +- {y.std(ddof=1) / math.sqrt(nb):.2e}")
        assert abs(x.mean() - y.mean()) < 3 * se + 1e-12


def test_matches_reference_pathlength_sensitivities(ctx):
    """-sum_p w_p L_pk per detector from the oracle's partial paths (the reference's own detected-photon data)."""
    import oracle

    nb, per = 10, 200000
    job = job4(per)
    media = job.media
    g, c = [], []
    for b in range(nb):
        s = job.sim
        s.photon_offset = b * per
        _, adj = run(ctx, job, media, s)
        g.append(adj["dread_dmua"][:, :, 1].sum(axis=1))
        _, dp, _, _ = oracle.forward(s, job.labels, media, job.detpos)
        # partial-path column k holds label k + 1 (the last column is always zero)
        L = dp[:, 1:s.mediumnum].astype(np.float64)
        w = np.exp(-(L * media[1:, 0][None, :].astype(np.float64)).sum(1))
        sens = np.zeros(s.detnum)
        for d in range(s.detnum):
            sel = dp[:, 0] == d + 1
            sens[d] = -(w[sel] * L[sel, 0]).sum()  # ppath column k holds label k+1: label 1 is column 0
        c.append(sens)
    g, c = np.array(g), np.array(c)
    se = np.sqrt(g.var(0, ddof=1) / nb + c.var(0, ddof=1) / nb)
    z = (g.mean(0) - c.mean(0)) / se
    print("per-detector d/dmua_1: adjoint", g.mean(0), "reference pathlengths", c.mean(0), "z", z)
    assert np.all(np.abs(z) < 3)


def test_replay_jacobian_consistent(ctx):
    job = job4(300000)
    s = job.sim
    out = ctx.forward_adjoint(s, job.labels, job.media, job.detpos)
    adj = ctx.backward(jacobian=True)
    assert adj["records"] > 100
    assert adj["replay_mismatch"] <= max(1, adj["records"] // 1000), adj["replay_mismatch"]
    J = adj["jacobian"].astype(np.float64)
    lab = job.labels & 0x7F
    for d in range(s.detnum):
        for k in range(s.mediumnum):
            js = J[d][lab == k].sum()
            ad = adj["dread_dmua"][d, :, k].sum()
            if abs(ad) > 0:
                assert abs(js - ad) <= 1e-4 * abs(ad), (d, k, js, ad)
    assert (J <= 0).all()
    print(f"replay: {adj['records']} photons in {adj['replay_ms']:.2f} ms, mismatches {adj['replay_mismatch']}")


def test_autograd_harness(ctx):
    import torch

    from umcx_gb300.autograd import PhotonTransport

    job = job4(100000)
    media = job.media
    mua = torch.tensor(media[:, 0].astype(np.float64), requires_grad=True)
    mus = torch.tensor(media[:, 1].astype(np.float64), requires_grad=True)
    readings, total = PhotonTransport.apply(mua, mus, ctx, job)
    weights = torch.linspace(0.5, 1.5, readings.shape[1], dtype=torch.float64)
    loss = (readings * weights).sum() + 1e-6 * total
    loss.backward()
    # finite-difference check of the same scalar along mua_1
    k = 1
    h = 0.01 * float(media[k, 0])

    def L(m):
        with torch.no_grad():
            r, t = PhotonTransport.apply(m, mus.detach(), ctx, job)
            return float((r * weights).sum() + 1e-6 * t)
    mp = mua.detach().clone()
    mm = mua.detach().clone()
    mp[k] += h
    mm[k] -= h
    fd = (L(mp) - L(mm)) / (2 * h)
    assert abs(mua.grad[k].item() - fd) <= 2e-3 * abs(fd)
    assert mus.grad is not None and torch.isfinite(mus.grad).all()


def test_adjoint_budget_stops_kernel_and_context_survives(ctx):
    """The adjoint forward kernel honours the launch budget too (status 3), and the context stays usable."""
    from umcx_gb300 import Job

    job = Job.from_args(["--bench", "cube60", "-n", "100000000"])
    ctx.set_tuning(budget_ms=10)
    try:
        with pytest.raises(RuntimeError, match="status 3"):
            ctx.forward_adjoint(job.sim, job.labels, job.media, job.detpos)
    finally:
        ctx.set_tuning()
    small = Job.from_args(["--bench", "cube60", "-n", "10000"])
    out = ctx.forward(small.sim, small.labels, small.media, small.detpos)
    assert out.result.status == 0 and out.result.launched == 10000
