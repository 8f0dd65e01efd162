"""Parity at the workload configurations themselves, against the FP64 oracle.

Every comparison here is GPU path vs oracle (never the GPU path vs itself),
at the configurations the throughput figures are quoted on:

  c1_512x8_1M        the reference's own CPU configuration in full: 512^2 grid,
                     8 w-planes, support 7, 1,048,576 measurements (48
                     stations, 3 km, 4 h).  FP64 grid <= 1e-12 (normwise max),
                     FP64 image <= 1e-11 (relative rms over finite pixels),
                     FP32C image <= 1e-5; NaN masks identical.
  c2_4096x32_1M      the precision configuration's geometry (4096^2, 32 planes,
                     support 7, 62 stations, 8 km, 8 h) on 1M measurements:
                     every w-plane of the FP64 grid against the oracle's plane
                     (<= 1e-12 normwise max) and of the FP32C grid (<= 2e-6
                     relative rms per plane); a 256^2 image window against the
                     windowed oracle (FP64 <= 1e-11 relative rms, FP32C <= 1e-5
                     of the image rms); FP32C vs FP64 over the whole image
                     <= 1e-5 with identical NaN masks.
  c3_2048x16_10M     the differentiation configuration: 2048^2, 16 planes, 10M
                     measurements.  Dot-product test <Ax, y> = <x, A^H y> to
                     1e-10 (FP64) and 1e-5 (FP32C); the autograd gradient of
                     1/2 ||I(vis) - I_target||^2 (I_target imaged from a
                     different sky seed) against the FP64 CPU gradient from the
                     oracle's adjoint to 1e-10 (FP64) and 1e-4 (FP32C forward +
                     adjoint, relative rms); central differences on 64 random
                     entries (see the test for the step).
  offsets_8192x36_200k
                     P*Nx*Ny = 2.4e9 > 2^31 cells (the reference's int offset
                     j + k*Nx + w*Nx*Ny overflows there, w-stacking.cu:90):
                     forward and adjoint in both precisions, a 256^2 window
                     against the windowed oracle, with measurements in the
                     planes above the 2^31-cell mark.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nrm_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _rel_rms(a, b):
    return float(np.sqrt(np.mean(np.abs(a - b) ** 2) / max(np.mean(np.abs(b) ** 2), 1e-300)))


def _observe(name, n_vis=None, sky_seed=2, backend="torch"):
    from lofar_gb300 import synth
    gen = dict(synth.CONFIGS[name]["gen"])
    if n_vis is not None:
        gen["n_vis"] = n_vis
    return synth.observe(backend=backend, sky_seed=sky_seed, **gen)


def _plan(nx, planes, support, precision, obs, resolution=None):
    from lofar_gb300 import Plan
    p = Plan(nx, nx, planes, support, precision=precision)
    p.set_wcorrection(obs.resolution if resolution is None else resolution, obs.wmin, obs.wmax)
    return p


def _free(*plans):
    import torch
    for p in plans:
        p.close()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


# ---------------------------------------------------------------------------
# c1: the reference's CPU configuration in full
# ---------------------------------------------------------------------------

def test_c1_512x8_1M_full_against_oracle(gpu):
    import torch
    from lofar_gb300 import synth
    cfg = synth.CONFIGS["c1"]
    o = _observe("c1")
    assert o.n == 1_048_576
    nx, planes, support = cfg["nx"], cfg["planes"], cfg["support"]
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=support, nx=nx, ny=nx)
    grid = O.wstack(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, **kw)
    re, im = O.phase_correction(O.fft_planes(grid), nx=nx, ny=nx, num_w_planes=planes,
                                resolution=o.resolution, wmin=o.wmin, wmax=o.wmax)
    ref = re + 1j * im
    fin = np.isfinite(re)

    imgs = {}
    for prec in ("fp64", "fp32c"):
        p = _plan(nx, planes, support, prec, o)
        p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
        g = torch.view_as_real(p.grid()).double().cpu().numpy()
        if prec == "fp64":
            assert _nrm_max(g, grid) <= 1e-12
        else:
            assert _rel_rms(g, grid) <= 1e-6
        img = p.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
        imgs[prec] = img.to(torch.complex128).cpu().numpy()
        _free(p)
    for prec, tol in (("fp64", 1e-11), ("fp32c", 1e-5)):
        z = imgs[prec]
        assert np.array_equal(np.isfinite(z.real), fin), prec
        assert _rel_rms(z[fin], ref[fin]) <= tol, prec


# ---------------------------------------------------------------------------
# c2: the precision configuration's geometry on 1M measurements
# ---------------------------------------------------------------------------

def test_c2_4096x32_1M_planes_and_window_against_oracle(gpu):
    import torch
    from lofar_gb300 import synth
    cfg = synth.CONFIGS["c2"]
    nx, planes, support, win = cfg["nx"], cfg["planes"], cfg["support"], 256
    o = _observe("c2", n_vis=1_000_000)
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=support, nx=nx, ny=nx)
    x0 = y0 = 13 * nx // 16 - win // 2

    p64 = _plan(nx, planes, support, "fp64", o)
    p32 = _plan(nx, planes, support, "fp32c", o)
    p64.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    p32.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    g64 = p64.grid()
    g32 = p32.grid()
    plane = np.zeros((nx, nx, 2))
    worst64, worst32 = 0.0, 0.0
    for w in range(planes):
        O.grid_plane(w, o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, out=plane, **kw)
        if not plane.any():
            assert float(g64[w].abs().max()) == 0.0 and float(g32[w].abs().max()) == 0.0
            continue
        a = torch.view_as_real(g64[w]).cpu().numpy()
        b = torch.view_as_real(g32[w]).double().cpu().numpy()
        worst64 = max(worst64, _nrm_max(a, plane))
        worst32 = max(worst32, _rel_rms(b, plane))
    assert worst64 <= 1e-12
    assert worst32 <= 2e-6
    del g64, g32
    _free(p64, p32)

    re, im = O.image_window(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, x0=x0, y0=y0,
                            wx=win, wy=win, resolution=o.resolution, wmin=o.wmin, wmax=o.wmax,
                            **kw)
    ref = re + 1j * im
    assert np.isfinite(ref).all()
    imgs = {}
    for prec in ("fp64", "fp32c"):
        p = _plan(nx, planes, support, prec, o)
        imgs[prec] = p.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img,
                                     o.weight).to(torch.complex128)
        _free(p)
    a64, a32 = imgs["fp64"], imgs["fp32c"]
    fin = torch.isfinite(a64.real)
    assert torch.equal(fin, torch.isfinite(a32.real))
    rms = float(torch.sqrt((a64[fin].abs() ** 2).mean()))
    assert float(torch.sqrt(((a32 - a64)[fin].abs() ** 2).mean())) <= 1e-5 * rms
    w64 = a64[y0:y0 + win, x0:x0 + win].cpu().numpy()
    w32 = a32[y0:y0 + win, x0:x0 + win].cpu().numpy()
    assert _rel_rms(w64, ref) <= 1e-11
    assert float(np.sqrt(np.mean(np.abs(w32 - ref) ** 2))) <= 1e-5 * rms


# ---------------------------------------------------------------------------
# c3: the differentiation configuration
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def c3(gpu):
    import torch
    from lofar_gb300 import synth
    cfg = synth.CONFIGS["c3"]
    nx, planes, support = cfg["nx"], cfg["planes"], cfg["support"]
    o = _observe("c3")
    other = _observe("c3", sky_seed=11)
    assert o.n == 10_000_000
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=support, nx=nx, ny=nx,
              resolution=o.resolution, wmin=o.wmin, wmax=o.wmax)
    tre, tim = O.image_forward(other.uu, other.vv, other.ww, other.vis_real, other.vis_img,
                               other.weight, **kw)
    assert np.isfinite(tre).all()   # the dot test needs a finite image
    target = torch.as_tensor(np.stack([tre, tim], -1)).cuda()
    return dict(obs=o, nx=nx, planes=planes, support=support, kw=kw, target=target)


def _dot(a, b):
    return float(np.sum(a.real * b.real + a.imag * b.imag))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32c", 1e-5)])
def test_c3_2048x16_10M_dot_product(c3, precision, tol):
    import torch
    o, nx = c3["obs"], c3["nx"]
    p = _plan(nx, c3["planes"], c3["support"], precision, o)
    img = p.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    rng = np.random.default_rng(1)
    y = rng.standard_normal((nx, nx)) + 1j * rng.standard_normal((nx, nx))
    aty = p.image_adjoint(torch.as_tensor(y).cuda())
    x = o.vis_real.astype(np.float64) + 1j * o.vis_img.astype(np.float64)
    lhs = _dot(img.to(torch.complex128).cpu().numpy(), y)
    rhs = _dot(x, aty.to(torch.complex128).cpu().numpy())
    _free(p)
    assert abs(lhs - rhs) <= tol * abs(lhs)


def _loss_grad(c3, precision):
    import torch
    from lofar_gb300.autograd import dirty_image
    o = c3["obs"]
    p = _plan(c3["nx"], c3["planes"], c3["support"], precision, o)
    vr = torch.as_tensor(o.vis_real, dtype=torch.float64).cuda().requires_grad_(True)
    vi = torch.as_tensor(o.vis_img, dtype=torch.float64).cuda().requires_grad_(True)
    wt = torch.as_tensor(o.weight, dtype=torch.float64).cuda().requires_grad_(True)
    img = dirty_image(p, o.uu, o.vv, o.ww, vr, vi, wt)
    loss = 0.5 * ((img.to(torch.float64) - c3["target"]) ** 2).sum()
    loss.backward()
    return p, (vr.grad.cpu().numpy(), vi.grad.cpu().numpy(), wt.grad.cpu().numpy())


@pytest.fixture(scope="module")
def c3_cpu_gradient(c3):
    """The FP64 CPU gradient: oracle forward, residual, oracle adjoint."""
    o, kw = c3["obs"], c3["kw"]
    re, im = O.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, **kw)
    t = c3["target"].cpu().numpy()
    g = O.image_adjoint(re - t[..., 0], im - t[..., 1], o.uu, o.vv, o.ww, **kw)
    wt = o.weight.astype(np.float64)
    return (wt * g[:, 0], wt * g[:, 1], g[:, 0] * o.vis_real + g[:, 1] * o.vis_img)


def test_c3_2048x16_10M_gradient_against_cpu_fp64(c3, c3_cpu_gradient):
    p, got = _loss_grad(c3, "fp64")
    _free(p)
    for a, b in zip(got, c3_cpu_gradient):
        assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()
    p, got32 = _loss_grad(c3, "fp32c")
    _free(p)
    for a, b in zip(got32, c3_cpu_gradient):
        assert _rel_rms(a, b) <= 1e-4


def test_c3_2048x16_10M_central_differences(c3):
    """Central differences of the FP64 loss on 64 random vis_real entries.

    The library reads the values as float32 (the reference's input layout), so
    a perturbed entry must be a float32 value: the step is
    h = 2^-6 * max(|v|, 1) and the divisor is the float32 difference
    f32(v + h) - f32(v - h) exactly.  The loss is exactly quadratic in each
    entry, so this central difference has no truncation error at any step;
    the configuration's epsilon of 1e-6 is below the float32 spacing of most
    values (it would round to 0-8 ulps of v), while the larger step keeps the
    perturbation exact and the image difference far above FP64 rounding.  The
    loss difference is summed as 1/2 sum (I_up - I_dn)(I_up + I_dn - 2 T)
    rather than as the difference of two loss sums over 8M pixel terms, whose
    rounding would swamp the entries with small gradients.  Agreement: 1e-6
    relative (floor 1e-3 of the largest gradient)."""
    import torch
    from lofar_gb300.autograd import dirty_image
    o = c3["obs"]
    p, (gvr, _, _) = _loss_grad(c3, "fp64")
    target = c3["target"]
    rng = np.random.default_rng(7)
    idx = rng.choice(o.n, 64, replace=False)
    vr0 = torch.as_tensor(o.vis_real).cuda()
    vi0 = torch.as_tensor(o.vis_img).cuda()
    wt = torch.as_tensor(o.weight).cuda()

    def image(vr):
        with torch.no_grad():
            return dirty_image(p, o.uu, o.vv, o.ww, vr, vi0, wt).double()
    scale = np.abs(gvr).max()
    for m in idx:
        v = float(o.vis_real[m])
        h = np.float32(max(abs(v), 1.0) * 2.0 ** -6)
        up, dn = vr0.clone(), vr0.clone()
        up[m] = float(np.float32(v) + h)
        dn[m] = float(np.float32(v) - h)
        step = float(np.float32(v) + h) - float(np.float32(v) - h)
        # loss(up) - loss(dn) = 1/2 sum (I_up - I_dn)(I_up + I_dn - 2 T), summed
        # in this form so that the two ~8M-term loss sums need not cancel
        iu, idn = image(up), image(dn)
        fd = 0.5 * float(((iu - idn) * (iu + idn - 2.0 * target)).sum()) / step
        assert abs(fd - gvr[m]) <= 1e-6 * max(abs(gvr[m]), 1e-3 * scale), m
    _free(p)


# ---------------------------------------------------------------------------
# more than 2^31 cells in the cube
# ---------------------------------------------------------------------------

def test_offsets_8192x36_200k_above_2_31_cells(gpu):
    import torch
    nx, planes, support, win = 8192, 36, 9, 256
    assert planes * nx * nx > 2 ** 31
    o = _observe("c5", n_vis=200_000)
    # measurements in the planes whose cells lie beyond the 2^31-cell mark
    high = (o.ww / (1.0 / planes)).astype(np.int64) * nx * nx >= 2 ** 31
    assert high.sum() > 200
    x0 = y0 = 13 * nx // 16 - win // 2
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=support, nx=nx, ny=nx,
              resolution=o.resolution, wmin=o.wmin, wmax=o.wmax)
    re, im = O.image_window(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, x0=x0, y0=y0,
                            wx=win, wy=win, **kw)
    ref = re + 1j * im
    rng = np.random.default_rng(2)
    yw = rng.standard_normal((win, win)) + 1j * rng.standard_normal((win, win))
    aw = O.adjoint_window(yw.real, yw.imag, o.uu, o.vv, o.ww, x0=x0, y0=y0, **kw)
    aref = aw[:, 0] + 1j * aw[:, 1]
    # the planes above the mark must contribute to the window image
    assert np.abs(aref[high]).max() > 0.0

    imgs, adjs = {}, {}
    for prec in ("fp64", "fp32c"):
        p = _plan(nx, planes, support, prec, o)
        imgs[prec] = p.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img,
                                     o.weight).to(torch.complex128)
        full = torch.zeros((nx, nx), dtype=p.cdtype, device="cuda")
        full[y0:y0 + win, x0:x0 + win] = torch.as_tensor(yw, device="cuda").to(p.cdtype)
        adjs[prec] = p.image_adjoint(full).cpu().numpy().astype(np.complex128)
        del full
        _free(p)

    w64 = imgs["fp64"][y0:y0 + win, x0:x0 + win].cpu().numpy()
    w32 = imgs["fp32c"][y0:y0 + win, x0:x0 + win].cpu().numpy()
    assert np.isfinite(ref).all() and np.isfinite(w32).all()
    assert _rel_rms(w64, ref) <= 1e-11
    assert _rel_rms(adjs["fp64"], aref) <= 1e-11
    assert _rel_rms(adjs["fp64"][high], aref[high]) <= 1e-11
    a64, a32 = imgs["fp64"], imgs["fp32c"]
    fin = torch.isfinite(a64.real)
    assert torch.equal(fin, torch.isfinite(a32.real))
    rms = float(torch.sqrt((a64[fin].abs() ** 2).mean()))
    assert float(torch.sqrt(((a32 - a64)[fin].abs() ** 2).mean())) <= 1e-5 * rms
    assert float(np.sqrt(np.mean(np.abs(w32 - ref) ** 2))) <= 1e-5 * rms
    assert _rel_rms(adjs["fp32c"], aref) <= 1e-5
