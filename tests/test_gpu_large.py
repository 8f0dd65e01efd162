"""The large-image path (8192-point FFT kernels, support 9) against the FP64
oracle's windowed forms, at a size the oracle finishes in seconds.

The full configuration (8192^2 x 128 planes, 400M visibilities) runs in
`bench.py --workload c5`, validated the same way on a 1M-visibility subset and
a 512^2 window.  Here: 8192^2 x 8 planes, 200k visibilities, a 256^2 window at
pixel coordinate 0 (where the w-correction is finite).

Tolerance: relative rms 1e-5 over the window (forward) and over the
visibilities (adjoint of an image supported on the window).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NX, PLANES, SUPPORT, WIN = 8192, 8, 9, 256


@pytest.fixture(scope="module")
def case(gpu):
    from lofar_gb300 import synth
    obs = synth.observe(n_stations=62, diameter_m=8000.0, hours=12.0, n_vis=200_000)
    return obs


def _rel_rms(a, b):
    return float(np.sqrt(np.mean(np.abs(a - b) ** 2) / np.mean(np.abs(b) ** 2)))


def test_large_image_window_and_adjoint(case):
    import torch
    from lofar_gb300 import Plan
    o = case
    p = Plan(NX, NX, PLANES, SUPPORT, precision="fp32c")
    p.set_wcorrection(o.resolution, o.wmin, o.wmax)
    img = p.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    x0 = y0 = NX // 2
    kw = dict(num_w_planes=PLANES, dx=1 / NX, dw=1 / PLANES, w_support=SUPPORT, nx=NX, ny=NX,
              resolution=o.resolution, wmin=o.wmin, wmax=o.wmax)
    re, im = O.image_window(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, x0=x0, y0=y0,
                            wx=WIN, wy=WIN, **kw)
    ref = re + 1j * im
    win = img[y0:y0 + WIN, x0:x0 + WIN].cpu().numpy().astype(np.complex128)
    assert np.isfinite(ref).all() and np.isfinite(win).all()
    assert _rel_rms(win, ref) <= 1e-5
    # NaN rule far from pixel coordinate 0: the image corner (0, 0) is NaN at this size
    assert torch.isnan(img[0, 0].real) == (np.sin((NX // 2) * o.resolution) ** 2 * 2 > 1)

    rng = np.random.default_rng(2)
    yw = rng.standard_normal((WIN, WIN)) + 1j * rng.standard_normal((WIN, WIN))
    full = torch.zeros((NX, NX), dtype=torch.complex64, device="cuda")
    full[y0:y0 + WIN, x0:x0 + WIN] = torch.as_tensor(yw.astype(np.complex64), device="cuda")
    g = p.image_adjoint(full).cpu().numpy().astype(np.complex128)
    a = O.adjoint_window(yw.real, yw.imag, o.uu, o.vv, o.ww, x0=x0, y0=y0, **kw)
    assert _rel_rms(g, a[:, 0] + 1j * a[:, 1]) <= 1e-5
