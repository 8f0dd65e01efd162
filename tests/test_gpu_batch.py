"""(channel, polarisation) batches through libwstack_gb300.so.

A batch of C channels x Pol polarisations is C*Pol jobs; job (c, p) must equal
the single-image path run on channel c's measurements with polarisation p's
values and weights alone (freq_per_chan = polarizations = 1).

Tolerances:
  batch vs single-image FP32C plan    normwise max 1e-6 (same kernels and
                                      records; bins are never split here, so
                                      the fixed-point tile sums are exact)
  batch vs FP64 oracle per job        rms 1e-5 over the image (the FP32C target)
  graph replay vs direct forward      identical
  adjoint vs single-image adjoint     normwise max 1e-6
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NX, PLANES, SUPPORT = 256, 4, 7


def _nrm_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _nrm_rms(a, b):
    return float(np.sqrt(np.mean(np.abs(a - b) ** 2)) / max(np.sqrt(np.mean(np.abs(b) ** 2)), 1e-300))


@pytest.fixture(scope="module")
def obs(gpu):
    from lofar_gb300 import synth
    b = synth.observe_batch(n_channels=3, pols=4, n_per_channel=24_000, n_stations=30,
                            diameter_m=3000.0, hours=4.0)
    chans = list(b.channels)
    # an empty channel (everything flagged) between two others
    empty = (np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0, np.float32),
             np.zeros(0, np.float32), np.zeros(0, np.float32))
    chans.insert(1, empty)
    # NaN-flag a few entries of one polarisation (the reference skips them)
    vr = chans[0][3].copy()
    vr[5 * 4 + 2] = np.nan
    vr[77 * 4 + 2] = np.nan
    chans[0] = chans[0][:3] + (vr,) + chans[0][4:]
    return dict(chans=chans, pols=4, res=b.resolution, wmin=b.wmin, wmax=b.wmax)


def _batch(o):
    from lofar_gb300 import Batch
    B = Batch(NX, NX, PLANES, SUPPORT, channels=len(o["chans"]), pols=o["pols"])
    B.set_wcorrection(o["res"], o["wmin"], o["wmax"])
    B.bind(o["chans"])
    return B


def _job(o, c, p):
    uu, vv, ww, vr, vi, wt = o["chans"][c]
    P = o["pols"]
    return (uu, vv, ww, np.ascontiguousarray(vr[p::P]), np.ascontiguousarray(vi[p::P]),
            np.ascontiguousarray(wt[p::P]))


def _plan(o):
    from lofar_gb300 import Plan
    pl = Plan(NX, NX, PLANES, SUPPORT, precision="fp32c")
    pl.set_wcorrection(o["res"], o["wmin"], o["wmax"])
    return pl


def test_forward_matches_single_image_jobs(obs):
    B = _batch(obs)
    imgs = B.forward(graph=True).cpu().numpy()
    pl = _plan(obs)
    for c in range(len(obs["chans"])):
        for p in range(obs["pols"]):
            job = _job(obs, c, p)
            if job[0].shape[0] == 0:
                assert np.all(imgs[c, p] == 0), (c, p)
                continue
            ref = pl.image_forward(*job).cpu().numpy()
            assert _nrm_max(imgs[c, p], ref) <= 1e-6, (c, p)


def test_forward_matches_fp64_oracle(obs):
    B = _batch(obs)
    imgs = B.forward(graph=False).cpu().numpy()
    for c in (0, 2, 3):
        for p in range(obs["pols"]):
            uu, vv, ww, vr, vi, wt = _job(obs, c, p)
            re, im = O.image_forward(uu, vv, ww, vr, vi, wt, num_w_planes=PLANES, dx=1 / NX,
                                     dw=1 / PLANES, w_support=SUPPORT, nx=NX, ny=NX,
                                     resolution=obs["res"], wmin=obs["wmin"], wmax=obs["wmax"])
            assert _nrm_rms(imgs[c, p], re + 1j * im) <= 1e-5, (c, p)


def test_graph_replay_reads_current_inputs(obs):
    import torch
    B = _batch(obs)
    a = B.forward(graph=False).clone()
    g1 = B.forward(graph=True).clone()
    out = B.new_images()
    B.forward(out, graph=True)
    B.forward(out, graph=True)   # replay of the captured graph
    assert torch.equal(a, g1) and torch.equal(a, out)
    # scale channel 0's values in place: the replayed graph must see it
    B._bound[0][3].mul_(2.0)
    B._bound[0][4].mul_(2.0)
    B.forward(out, graph=True)
    ref = B.forward(graph=False)
    assert torch.equal(out, ref)
    assert torch.allclose(out[0], 2.0 * a[0], rtol=1e-5, atol=1e-6 * float(a[0].abs().max()))
    assert torch.equal(out[2:], a[2:])


def test_adjoint_matches_single_image_jobs(obs):
    import torch
    B = _batch(obs)
    B.forward()
    rng = np.random.default_rng(3)
    shape = (len(obs["chans"]), obs["pols"], NX, NX)
    y = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    yt = torch.as_tensor(y).cuda()
    out = B.adjoint(yt).cpu().numpy()
    assert out.shape[0] == B.n_vis() == sum(ch[0].shape[0] for ch in obs["chans"]) * obs["pols"]
    pl = _plan(obs)
    P = obs["pols"]
    for c in range(len(obs["chans"])):
        n = obs["chans"][c][0].shape[0]
        off = B.vis_offset(c)
        if n == 0:
            assert B.vis_offset(c + 1) == off
            continue
        mine = out[off:off + n * P].reshape(n, P)
        for p in range(P):
            pl.bin(*_job(obs, c, p))
            ref = pl.image_adjoint(yt[c, p]).cpu().numpy()
            assert _nrm_max(mine[:, p], ref) <= 1e-6, (c, p)


def test_adjoint_matches_fp64_oracle(obs):
    import torch
    B = _batch(obs)
    B.forward()
    rng = np.random.default_rng(5)
    shape = (len(obs["chans"]), obs["pols"], NX, NX)
    y = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    out = B.adjoint(torch.as_tensor(y.astype(np.complex64)).cuda()).cpu().numpy()
    c, P = 2, obs["pols"]
    uu, vv, ww = obs["chans"][c][:3]
    off, n = B.vis_offset(c), uu.shape[0]
    mine = out[off:off + n * P].reshape(n, P)
    for p in range(P):
        g = O.image_adjoint(y[c, p].real, y[c, p].imag, uu, vv, ww, num_w_planes=PLANES,
                            dx=1 / NX, dw=1 / PLANES, w_support=SUPPORT, nx=NX, ny=NX,
                            resolution=obs["res"], wmin=obs["wmin"], wmax=obs["wmax"])
        assert _nrm_rms(mine[:, p], g[:, 0] + 1j * g[:, 1]) <= 1e-5, p


def test_stats_count_records_of_every_job(obs):
    B = _batch(obs)
    B.forward()
    st = B.stats()
    pl = _plan(obs)
    total = 0
    for c in range(len(obs["chans"])):
        for p in range(obs["pols"]):
            job = _job(obs, c, p)
            pl.bin(*job)
            total += pl.stats()["records"]
    assert st["records"] == total
    assert st["points_in"] == B.n_vis()
    assert st["bins"] == len(obs["chans"]) * obs["pols"] * PLANES * (NX // st["tile"]) ** 2


def test_autotune_keeps_fastest_and_stays_correct(obs):
    import torch
    B = _batch(obs)
    ref = B.forward(graph=False).clone()
    best, tried = B.autotune(iters=2)
    assert tried and best["ms"] == min(t["ms"] for t in tried)
    assert any(t["tile"] == 32 for t in tried) and any(t["tile"] == 64 for t in tried)
    assert B.stats()["tile"] == best["tile"]
    out = B.forward(graph=True)
    scale = float(ref.abs().max())
    assert float((out - ref).abs().max()) <= 1e-6 * scale


def test_small_split_sizes_agree(obs):
    """Bins cut into work items (split partial tiles) give the same images."""
    B = _batch(obs)
    ref = B.forward(graph=False).clone()
    B.set_tuning(chunk=512)
    out = B.forward(graph=True)
    scale = float(ref.abs().max())
    assert float((out - ref).abs().max()) <= 2e-6 * scale
