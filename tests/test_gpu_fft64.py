"""The FP64 form's per-plane 2D FFT on the integer pipe (fft64.cu).

Power-of-two grids of edge 256..8192 take a block-floating-point FFT on
signed 64-bit integers; other grids, and any grid with
WSTACK_GB300_FFT=cufft, take the Z2Z library FFT.  The reference's
fftw_data (fourier_transform.c:25-59) is FFTW_BACKWARD per plane, the
oracle's stand-in is NumPy's FFT.

Tolerances:
  integer FFT vs NumPy, per plane      max |diff| <= 1e-13 * max |ref|
  integer FFT vs the library FFT       max |diff| <= 1e-13 * max |ref|
  a plane holding a NaN                every output NaN (as every output of
                                       a DFT of such an input is non-finite)
  an all-zero column or plane          exactly zero
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _nrm(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _cube(rng, p, ny, nx):
    x = rng.standard_normal((p, ny, nx)) + 1j * rng.standard_normal((p, ny, nx))
    x[0, :, nx // 3: nx // 2] = 0          # zero columns
    x[0, ny // 4: ny // 2, :] = 0          # zero rows
    return x


def _plan_fft(x, sign, env=None):
    import torch
    from lofar_gb300 import Plan
    p, ny, nx = x.shape
    old = os.environ.pop("WSTACK_GB300_FFT", None)
    if env:
        os.environ["WSTACK_GB300_FFT"] = env
    try:
        plan = Plan(nx, ny, p, 7, precision="fp64")
    finally:
        os.environ.pop("WSTACK_GB300_FFT", None)
        if old is not None:
            os.environ["WSTACK_GB300_FFT"] = old
    g = torch.as_tensor(x).cuda()
    plan.fft(g, sign)
    torch.cuda.synchronize()
    out = g.cpu().numpy()
    plan.close()
    return out


@pytest.mark.parametrize("shape", [(3, 256, 256), (2, 2048, 512), (2, 512, 2048),
                                   (1, 256, 8192), (1, 8192, 256), (1, 4096, 4096)])
@pytest.mark.parametrize("sign", [1, -1])
def test_integer_fft_matches_numpy(gpu, shape, sign):
    rng = np.random.default_rng(sum(shape) + sign)
    x = _cube(rng, *shape)
    got = _plan_fft(x, sign)
    ref = np.fft.ifft2(x) * (shape[1] * shape[2]) if sign > 0 else np.fft.fft2(x)
    for p in range(shape[0]):
        assert _nrm(got[p], ref[p]) <= TOL, p


def test_integer_fft_spike_nan_and_zero_planes(gpu):
    rng = np.random.default_rng(3)
    x = _cube(rng, 4, 512, 512)
    x[1] = 0
    x[1, 5, 7] = 2.5 - 1.0j                 # one point: a pure phase ramp
    x[2, 3, 4] = np.nan
    x[3] = 0
    got = _plan_fft(x, 1)
    ref = np.fft.ifft2(x) * 512 * 512
    assert _nrm(got[0], ref[0]) <= TOL
    assert _nrm(got[1], ref[1]) <= TOL
    assert np.isnan(got[2]).all()
    assert np.array_equal(got[3], np.zeros_like(got[3]))


def test_integer_fft_matches_library_fft(gpu):
    rng = np.random.default_rng(5)
    x = _cube(rng, 2, 1024, 1024)
    a = _plan_fft(x, 1)
    b = _plan_fft(x, 1, env="cufft")
    for p in range(2):
        assert _nrm(a[p], b[p]) <= TOL


def test_non_power_of_two_takes_the_library_fft(gpu):
    rng = np.random.default_rng(7)
    x = _cube(rng, 2, 300, 250)
    got = _plan_fft(x, -1)
    ref = np.fft.fft2(x)
    for p in range(2):
        assert _nrm(got[p], ref[p]) <= 1e-14


@pytest.mark.parametrize("shape", [(3, 512, 512), (2, 300, 256)])
def test_dropin_fft_planes(gpu, shape):
    """wstack_fft_planes: FFTW_BACKWARD per plane times 1/(nx ny), host
    buffers in and out (the exact power of two rides on the integer FFT's
    output exponent)."""
    from lofar_gb300 import api
    p, ny, nx = shape
    rng = np.random.default_rng(11)
    x = _cube(rng, p, ny, nx)
    inp = np.ascontiguousarray(np.stack([x.real, x.imag], -1))
    out = np.zeros_like(inp)
    api.fft_planes(inp, out, nx, ny, p)
    got = out[..., 0] + 1j * out[..., 1]
    ref = np.fft.ifft2(x)
    for w in range(p):
        assert _nrm(got[w], ref[w]) <= TOL
