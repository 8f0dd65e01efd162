"""The CPU oracle, pinned against the reference's own build and fixtures."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _grid_args(d):
    nx, ny, planes, support, nf, np_ = (int(x) for x in d["params"])
    dx, dw = (float(x) for x in d["dxdw"])
    return dict(num_w_planes=planes, freq_per_chan=nf, polarizations=np_, dx=dx, dw=dw,
                w_support=support, nx=nx, ny=ny)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_bit_identical_to_reference_fixtures(path):
    d = np.load(path)
    g = O.wstack(d["uu"], d["vv"], d["ww"], d["vis_real"], d["vis_img"], d["weight"],
                 num_threads=1, **_grid_args(d))
    assert np.array_equal(g, d["grid"])
    if "image_real" in d:
        res, wmin, wmax = (float(x) for x in d["wc"])
        a = _grid_args(d)
        re, im = O.phase_correction(d["gridss"], nx=a["nx"], ny=a["ny"],
                                    num_w_planes=a["num_w_planes"], resolution=res, wmin=wmin,
                                    wmax=wmax, num_threads=1)
        assert np.array_equal(re, d["image_real"], equal_nan=True)
        assert np.array_equal(im, d["image_imag"], equal_nan=True)


def test_fixtures_present():
    names = {os.path.basename(p) for p in GOLDEN}
    assert {"obs_48x40_p4_s7.npz", "edges_40x36_p3_s5.npz", "fold_f2p2_nan_32_p2_s7.npz",
            "single_16_p1_s7.npz", "p1_32_s9.npz", "nanfield_32_p4_s3.npz"} <= names


def test_oracle_matches_reference_build_live():
    if O.load_ref() is None:
        pytest.skip("reference CPU build not available on this host")
    rng = np.random.default_rng(5)
    n = 4000
    uu, vv, ww = rng.random(n), rng.random(n), rng.random(n) * 0.999
    vr = rng.standard_normal(n).astype(np.float32)
    vi = rng.standard_normal(n).astype(np.float32)
    wt = rng.uniform(0.1, 1, n).astype(np.float32)
    kw = dict(num_w_planes=8, dx=1 / 64, dw=1 / 8, w_support=7, nx=64, ny=64, num_threads=1)
    a = O.wstack(uu, vv, ww, vr, vi, wt, lib="oracle", **kw)
    b = O.wstack(uu, vv, ww, vr, vi, wt, lib="ref", **kw)
    assert np.array_equal(a, b)
    gs = O.fft_planes(a)
    pa = O.phase_correction(gs, nx=64, ny=64, num_w_planes=8, resolution=1 / 50, wmin=-30,
                            wmax=45, num_threads=1)
    pb = O.phase_correction(gs, nx=64, ny=64, num_w_planes=8, resolution=1 / 50, wmin=-30,
                            wmax=45, num_threads=1, lib="ref")
    assert np.array_equal(pa[0], pb[0], equal_nan=True)
    assert np.array_equal(pa[1], pb[1], equal_nan=True)


def test_oracle_threads_agree():
    d = np.load(GOLDEN[0])
    g1 = O.wstack(d["uu"], d["vv"], d["ww"], d["vis_real"], d["vis_img"], d["weight"],
                  num_threads=1, **_grid_args(d))
    g4 = O.wstack(d["uu"], d["vv"], d["ww"], d["vis_real"], d["vis_img"], d["weight"],
                  num_threads=4, **_grid_args(d))
    assert np.abs(g4 - g1).max() <= 1e-13 * np.abs(g1).max()


def test_single_measurement_is_the_gaussian():
    # w-stacking.cu:17-22 with std22 = 0.5, norm = std22/PI (PI = 3.14159265359)
    g = O.wstack([10.25 / 32], [9.75 / 32], [0.0], [2.0], [0.5], [1.0], num_w_planes=1, dx=1 / 32,
                 dw=1.0, w_support=7, nx=32, ny=32, num_threads=1)
    k, j = np.mgrid[0:32, 0:32]
    du = j + 0.5 - 10.25
    dv = k + 0.5 - 9.75
    win = (np.abs(j - 10) <= 3) & (np.abs(k - 9) <= 3)
    expect = np.where(win, 0.5 / 3.14159265359 * np.exp(-(du * du + dv * dv) * 0.5), 0.0)
    np.testing.assert_allclose(g[0, :, :, 0], 2.0 * expect, rtol=1e-15, atol=0)
    np.testing.assert_allclose(g[0, :, :, 1], 0.5 * expect, rtol=1e-15, atol=0)


def test_out_of_range_plane_is_skipped():
    # the reference writes outside the grid here (w-stacking.cu:69,90); the
    # oracle and the library skip such measurements
    g = O.wstack([0.5, 0.5], [0.5, 0.5], [1.0, -0.6], [1.0, 1.0], [0.0, 0.0], [1.0, 1.0],
                 num_w_planes=2, dx=1 / 16, dw=0.5, w_support=3, nx=16, ny=16, num_threads=1)
    assert not g.any()


def test_nan_flag_skips_the_entry():
    base = dict(num_w_planes=1, freq_per_chan=2, polarizations=1, dx=1 / 16, dw=1.0,
                w_support=3, nx=16, ny=16, num_threads=1)
    a = O.wstack([0.5], [0.5], [0.0], [np.nan, 3.0], [7.0, 1.0], [1.0], **base)
    b = O.wstack([0.5], [0.5], [0.0], [3.0], [1.0], [1.0], **dict(base, freq_per_chan=1))
    assert np.array_equal(a, b)


def test_fft_stage_is_fftw_backward_scaled():
    rng = np.random.default_rng(1)
    g = rng.standard_normal((2, 8, 6, 2))
    out = O.fft_planes(g)
    z = g[..., 0] + 1j * g[..., 1]
    k = np.arange(8)[:, None, None, None]
    j = np.arange(6)[None, :, None, None]
    y = np.arange(8)[None, None, :, None]
    x = np.arange(6)[None, None, None, :]
    ph = np.exp(2j * np.pi * (k * y / 8 + j * x / 6))
    ref = np.einsum("pkj,kjyx->pyx", z, ph) / 48
    np.testing.assert_allclose(out[..., 0] + 1j * out[..., 1], ref, atol=1e-13)


def _dot(a, b):
    return float(np.sum(a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]))


def test_oracle_adjoint_dot_product():
    rng = np.random.default_rng(3)
    n, nx, planes = 500, 32, 4
    uu, vv, ww = rng.random(n), rng.random(n), rng.random(n) * 0.999
    vr = rng.standard_normal(n).astype(np.float32)
    vi = rng.standard_normal(n).astype(np.float32)
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=7, nx=nx, ny=nx,
              resolution=1 / 40, wmin=-50.0, wmax=80.0, num_threads=1)
    re, im = O.image_forward(uu, vv, ww, vr, vi, np.ones(n, np.float32), **kw)
    assert np.isfinite(re).all()
    y = rng.standard_normal((nx, nx, 2))
    ax_y = _dot(np.stack([re, im], -1), y)
    aty = O.image_adjoint(y[..., 0], y[..., 1], uu, vv, ww, **kw)
    x_aty = _dot(np.stack([vr.astype(np.float64), vi.astype(np.float64)], -1), aty)
    assert abs(ax_y - x_aty) <= 1e-12 * max(abs(ax_y), 1.0)


def test_resolution_rule_truncates_like_c_int_abs():
    assert O.resolution(-1499.9, 1428.6) == 1.0 / 1499
    assert O.resolution(-3.7, 1500.2) == 1.0 / 1500


@pytest.mark.parametrize("nx,ny,planes,win", [(64, 64, 4, (20, 8, 16, 12)),
                                              (48, 40, 3, (30, 25, 18, 15)),
                                              (32, 32, 1, (0, 0, 32, 32))])
def test_window_oracle_equals_full_chain(nx, ny, planes, win):
    """The plane-by-plane windowed forms (used where the FP64 cube does not fit
    in memory) equal the full oracle chain on the window."""
    from lofar_gb300 import synth
    obs = synth.observe(n_stations=16, diameter_m=1500.0, hours=2.0, n_vis=3000, sky_seed=9)
    x0, y0, wx, wy = win
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=7, nx=nx, ny=ny,
              resolution=1 / 400.0, wmin=obs.wmin, wmax=obs.wmax)
    re, im = O.image_forward(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight, **kw)
    wr, wi = O.image_window(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight,
                            x0=x0, y0=y0, wx=wx, wy=wy, **kw)
    ref = re[y0:y0 + wy, x0:x0 + wx] + 1j * im[y0:y0 + wy, x0:x0 + wx]
    assert np.abs(wr + 1j * wi - ref).max() <= 1e-13 * np.abs(ref).max()
    rng = np.random.default_rng(1)
    y = rng.standard_normal((wy, wx)) + 1j * rng.standard_normal((wy, wx))
    full = np.zeros((ny, nx), np.complex128)
    full[y0:y0 + wy, x0:x0 + wx] = y
    a_ref = O.image_adjoint(full.real, full.imag, obs.uu, obs.vv, obs.ww, **{
        k: v for k, v in kw.items()})
    a = O.adjoint_window(y.real, y.imag, obs.uu, obs.vv, obs.ww, x0=x0, y0=y0, **kw)
    assert np.abs(a - a_ref).max() <= 1e-13 * np.abs(a_ref).max()
