"""The FP32C per-plane FFTs (shared-memory Stockham kernels) and their fusion
with the w-correction, against NumPy in FP64.

Tolerances: plain transforms 2e-6 relative rms (FP32 arithmetic, log2 N
rounding steps); the pruned/fused pipeline against the dense one 2e-6.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rel_rms(a, b):
    return float(np.sqrt(np.mean(np.abs(a - b) ** 2) / np.mean(np.abs(b) ** 2)))


@pytest.mark.parametrize("nx,ny", [(256, 256), (512, 1024), (1024, 512), (2048, 2048),
                                   (4096, 256), (256, 8192)])
@pytest.mark.parametrize("sign", [+1, -1])
def test_plain_fft_matches_numpy(gpu, nx, ny, sign):
    import torch
    from lofar_gb300 import Plan
    planes = 2
    p = Plan(nx, ny, planes, 7, precision="fp32c")
    rng = np.random.default_rng(nx + ny + sign)
    z = (rng.standard_normal((planes, ny, nx)) + 1j * rng.standard_normal((planes, ny, nx)))
    g = torch.as_tensor(z.astype(np.complex64)).cuda()
    p.fft(g, sign)
    got = g.cpu().numpy().astype(np.complex128)
    if sign > 0:
        ref = np.fft.ifft2(z.astype(np.complex64).astype(np.complex128), axes=(-2, -1)) * (nx * ny)
    else:
        ref = np.fft.fft2(z.astype(np.complex64).astype(np.complex128), axes=(-2, -1))
    assert _rel_rms(got, ref) <= 2e-6


def _gridded_plan(precision, nx=512, planes=8):
    from lofar_gb300 import Plan, synth
    obs = synth.observe(n_stations=30, diameter_m=3000.0, hours=3.0, n_vis=100_000, sky_seed=8)
    p = Plan(nx, nx, planes, 7, precision=precision)
    p.set_wcorrection(1.0 / 900.0, obs.wmin, obs.wmax)
    p.bin(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight)
    return p, obs


def test_pruned_fused_forward_equals_dense(gpu):
    p, obs = _gridded_plan("fp32c")
    g1 = p.grid()
    g2 = g1.clone()
    a = p.fft_wcorrect(g1, prune=True).cpu().numpy()
    b = p.fft_wcorrect(g2, prune=False).cpu().numpy()
    assert np.isfinite(b).all()
    assert _rel_rms(a, b) <= 2e-6


def test_occupied_tiles_grid_feeds_the_pruned_forward(gpu):
    """wsg_grid_occupied writes the occupied tiles exactly as wsg_grid does and
    leaves the others untouched; with pruning the forward reads no others."""
    import torch
    p, obs = _gridded_plan("fp32c")
    dense = p.grid()
    poisoned = torch.full_like(dense, complex(float("nan"), float("nan")))
    occ = p.grid(poisoned, occupied_only=True)
    assert torch.isnan(occ.real).any()            # empty tiles left as they were
    finite = ~torch.isnan(occ.real)
    assert torch.equal(occ[finite], dense[finite])
    assert float(dense[~finite].abs().max()) == 0.0
    a = p.fft_wcorrect(occ, prune=True).cpu().numpy()
    b = p.fft_wcorrect(dense.clone(), prune=True).cpu().numpy()
    assert np.array_equal(a, b)


def test_pruned_fused_adjoint_equals_dense_on_degridded_cells(gpu):
    import torch
    p, obs = _gridded_plan("fp32c")
    rng = np.random.default_rng(4)
    img = torch.as_tensor((rng.standard_normal((512, 512)) + 1j * rng.standard_normal((512, 512)))
                          .astype(np.complex64)).cuda()
    ga = p.wcorrect_adjoint_fft(img, prune=True)
    da = p.degrid(ga).cpu().numpy()
    gb = p.wcorrect_adjoint_fft(img, prune=False)
    db = p.degrid(gb).cpu().numpy()
    assert _rel_rms(da, db) <= 2e-6


def test_fused_forward_matches_oracle_image(gpu):
    import torch
    p, obs = _gridded_plan("fp32c")
    img = p.image_forward(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight)
    re, im = O.image_forward(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight,
                             num_w_planes=8, dx=1 / 512, dw=1 / 8, w_support=7, nx=512, ny=512,
                             resolution=1.0 / 900.0, wmin=obs.wmin, wmax=obs.wmax)
    z = img.cpu().numpy().astype(np.complex128)
    ref = re + 1j * im
    ok = np.isfinite(ref)
    assert np.array_equal(np.isfinite(z), ok)
    assert _rel_rms(z[ok], ref[ok]) <= 1e-5


def test_fused_adjoint_excludes_nan_pixels(gpu):
    """Pixels where the forward is NaN (r^2 > 1) are excluded from the adjoint:
    their image value (NaN here: the forward image itself is fed back) and
    their NaN w-screen phase must not reach the transforms."""
    import torch
    from lofar_gb300 import Plan, synth
    obs = synth.observe(n_stations=24, diameter_m=2000.0, hours=2.0, n_vis=30_000)
    nx, planes, res = 256, 8, 1.0 / 150.0
    outs = {}
    for prec in ("fp64", "fp32c"):
        p = Plan(nx, nx, planes, 7, precision=prec)
        p.set_wcorrection(res, obs.wmin, obs.wmax)
        img = p.image_forward(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight)
        nan = torch.isnan(img.real)
        assert 0 < int(nan.sum()) < nx * nx * 9 // 10
        outs[prec] = p.image_adjoint(img).to(torch.complex128).cpu().numpy()
        p.close()
    assert np.isfinite(outs["fp32c"]).all() and np.isfinite(outs["fp64"]).all()
    assert _rel_rms(outs["fp32c"], outs["fp64"]) <= 1e-5
