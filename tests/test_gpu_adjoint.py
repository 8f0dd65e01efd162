"""Adjoint (degridding) and gradients through libwstack_gb300.so.

Checks, all in FP64 unless stated:
  * degrid vs the oracle's transpose of the gridder (1e-12 normwise)
  * dot-product test <A x, y> = <x, A^H y> to 1e-10 (image operator)
  * autograd gradient vs the FP64 CPU gradient (oracle adjoint) to 1e-10
  * central differences on 64 random entries: the loss is exactly quadratic
    in each visibility, so the central difference equals the derivative up to
    FP64 rounding; agreement to 1e-6 relative
  * FP32C: dot-product test to 1e-5 and gradient to 1e-4 of the FP64 one
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _dot(a, b):
    return float(np.sum(a.real * b.real + a.imag * b.imag))


@pytest.fixture(scope="module")
def case(gpu):
    from lofar_gb300 import synth
    obs = synth.observe(n_stations=30, diameter_m=3000.0, hours=3.0, n_vis=60_000, sky_seed=4)
    nx, planes = 128, 8
    res = 1.0 / 1500.0  # no NaN pixels: the dot test needs a finite image
    return dict(obs=obs, nx=nx, planes=planes, support=7, res=res)


def _plan(c, precision):
    from lofar_gb300 import Plan
    p = Plan(c["nx"], c["nx"], c["planes"], c["support"], precision=precision)
    p.set_wcorrection(c["res"], c["obs"].wmin, c["obs"].wmax)
    return p


def test_degrid_matches_oracle_transpose(case):
    import torch
    o = case["obs"]
    nx, planes = case["nx"], case["planes"]
    rng = np.random.default_rng(0)
    g = rng.standard_normal((planes, nx, nx, 2))
    for prec, tol in (("fp64", 1e-12), ("fp32c", 2e-6)):
        p = _plan(case, prec)
        p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
        gt = torch.view_as_complex(torch.as_tensor(g).cuda().contiguous()).to(p.cdtype)
        d = p.degrid(gt)
        got = torch.view_as_real(d).cpu().numpy().astype(np.float64)
        ref = O.degrid(o.uu, o.vv, o.ww, g, num_w_planes=planes, dx=1 / nx, dw=1 / planes,
                       w_support=7, nx=nx, ny=nx)
        assert np.abs(got - ref).max() <= tol * np.abs(ref).max(), prec


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32c", 1e-5)])
def test_dot_product(case, precision, tol):
    import torch
    o = case["obs"]
    p = _plan(case, precision)
    nx = case["nx"]
    x = torch.complex(torch.as_tensor(o.vis_real, dtype=torch.float64),
                      torch.as_tensor(o.vis_img, dtype=torch.float64))
    img = p.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    rng = np.random.default_rng(1)
    y = torch.complex(torch.as_tensor(rng.standard_normal((nx, nx))),
                      torch.as_tensor(rng.standard_normal((nx, nx))))
    aty = p.image_adjoint(y.cuda())
    lhs = _dot(img.cpu().to(torch.complex128).numpy(), y.numpy())
    rhs = _dot(x.numpy(), aty.cpu().to(torch.complex128).numpy())
    assert abs(lhs - rhs) <= tol * abs(lhs)


def _loss_and_grad(case, precision, target):
    # float64 leaves holding float32 values: the library reads them as float32
    # (the reference's layout) and autograd returns float64 gradients
    import torch
    from lofar_gb300.autograd import dirty_image
    o = case["obs"]
    p = _plan(case, precision)
    vr = torch.as_tensor(o.vis_real, dtype=torch.float64).cuda().requires_grad_(True)
    vi = torch.as_tensor(o.vis_img, dtype=torch.float64).cuda().requires_grad_(True)
    wt = torch.as_tensor(o.weight, dtype=torch.float64).cuda().requires_grad_(True)
    img = dirty_image(p, o.uu, o.vv, o.ww, vr, vi, wt)
    loss = 0.5 * ((img.to(torch.float64) - target) ** 2).sum()
    loss.backward()
    return p, loss.item(), vr.grad.double().cpu().numpy(), vi.grad.double().cpu().numpy(), \
        wt.grad.double().cpu().numpy()


@pytest.fixture(scope="module")
def target(case):
    import torch
    from lofar_gb300 import synth
    o = case["obs"]
    other = synth.observe(n_stations=30, diameter_m=3000.0, hours=3.0, n_vis=60_000, sky_seed=77)
    re, im = O.image_forward(other.uu, other.vv, other.ww, other.vis_real, other.vis_img,
                             other.weight, num_w_planes=case["planes"], dx=1 / case["nx"],
                             dw=1 / case["planes"], w_support=7, nx=case["nx"], ny=case["nx"],
                             resolution=case["res"], wmin=o.wmin, wmax=o.wmax)
    return torch.as_tensor(np.stack([re, im], -1)).cuda()


def test_gradient_matches_cpu_fp64(case, target):
    o = case["obs"]
    nx, planes = case["nx"], case["planes"]
    _, loss, gvr, gvi, gwt = _loss_and_grad(case, "fp64", target)
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=7, nx=nx, ny=nx,
              resolution=case["res"], wmin=o.wmin, wmax=o.wmax)
    re, im = O.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, **kw)
    t = target.cpu().numpy()
    r = np.stack([re - t[..., 0], im - t[..., 1]], -1)
    g = O.image_adjoint(r[..., 0], r[..., 1], o.uu, o.vv, o.ww, **kw)
    wt = o.weight.astype(np.float64)
    ref_vr = wt * g[:, 0]
    ref_vi = wt * g[:, 1]
    ref_wt = g[:, 0] * o.vis_real + g[:, 1] * o.vis_img
    for a, b in ((gvr, ref_vr), (gvi, ref_vi), (gwt, ref_wt)):
        assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()


def test_central_differences(case, target):
    import torch
    from lofar_gb300.autograd import dirty_image
    o = case["obs"]
    p, loss0, gvr, gvi, _ = _loss_and_grad(case, "fp64", target)
    rng = np.random.default_rng(7)
    idx = rng.choice(o.n, 64, replace=False)
    vr0 = torch.as_tensor(o.vis_real).cuda()
    vi0 = torch.as_tensor(o.vis_img).cuda()
    wt = torch.as_tensor(o.weight).cuda()

    def loss(vr):
        with torch.no_grad():
            img = dirty_image(p, o.uu, o.vv, o.ww, vr, vi0, wt)
            return 0.5 * ((img.double() - target) ** 2).sum().item()
    for m in idx:
        v = float(o.vis_real[m])
        h = np.float32(max(abs(v), 1.0) * 2.0 ** -6)
        up, dn = vr0.clone(), vr0.clone()
        up[m] = float(np.float32(v) + h)
        dn[m] = float(np.float32(v) - h)
        step = float(np.float32(v) + h) - float(np.float32(v) - h)
        fd = (loss(up) - loss(dn)) / step
        assert abs(fd - gvr[m]) <= 1e-6 * max(abs(gvr[m]), 1e-3 * np.abs(gvr).max()), m


def test_fp32c_gradient_close_to_fp64(case, target):
    _, _, a, b, c = _loss_and_grad(case, "fp64", target)
    _, _, a32, b32, c32 = _loss_and_grad(case, "fp32c", target)
    for x, y in ((a32, a), (b32, b), (c32, c)):
        assert np.sqrt(np.mean((x - y) ** 2)) <= 1e-4 * np.sqrt(np.mean(y ** 2))
