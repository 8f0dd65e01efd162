"""Parity of the CUDA path against the oracle and the reference fixtures.

Every call goes through libwstack_gb300.so (the C ABI), either through the
drop-in entry points with host NumPy buffers or through the plan API with
device tensors.

Tolerances (stated per form):
  FP64 grid         max |diff| <= 1e-12 * max |ref|      (normwise)
  FP64 image        rms |diff| <= 1e-11 * rms |ref| over finite pixels; NaN
                    mask identical.  (The phase 2*PI*w*(sqrt(1-r2)-1) reaches
                    ~1e3 rad, whose FP64 rounding alone is ~1e-13 rad.)
  FP32C grid        rms <= 1e-6, max <= 1e-5 (normwise)
  FP32C image       rms <= 1e-5 over finite pixels (the precision target)
  cell/plane index  bit-exact (checked through single-measurement footprints)
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _args(d):
    nx, ny, planes, support, nf, np_ = (int(x) for x in d["params"])
    dx, dw = (float(x) for x in d["dxdw"])
    return nx, ny, planes, support, nf, np_, dx, dw


def _nrm_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _nrm_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


@pytest.fixture(autouse=True)
def _fp64_default(gpu):
    import lofar_gb300 as L
    L.set_precision("fp64")
    yield
    L.set_precision("fp64")


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_dropin_wstack_matches_reference_fixture(path):
    import lofar_gb300 as L
    d = np.load(path)
    nx, ny, planes, support, nf, np_, dx, dw = _args(d)
    grid = np.full((planes, ny, nx, 2), 7.0)  # overwritten, like the reference's CUDA build
    n = d["uu"].shape[0]
    L.wstack(planes, n, nf, np_, d["uu"], d["vv"], d["ww"], d["vis_real"], d["vis_img"],
             d["weight"], dx, dw, support, nx, ny, grid, 1)
    assert _nrm_max(grid, d["grid"]) <= 1e-12


@pytest.mark.parametrize("path", [p for p in GOLDEN if "image_real" in np.load(p)],
                         ids=lambda p: os.path.basename(p)[:-4])
def test_dropin_phase_correction_matches_reference_fixture(path):
    import lofar_gb300 as L
    d = np.load(path)
    nx, ny, planes, *_ = _args(d)
    res, wmin, wmax = (float(x) for x in d["wc"])
    re = np.full((ny, nx), 3.0)
    im = np.full((ny, nx), 3.0)
    L.phase_correction(np.ascontiguousarray(d["gridss"]), re, im, nx, ny, planes, nx, ny, res,
                       wmin, wmax, 1)
    ref_re, ref_im = d["image_real"], d["image_imag"]
    assert np.array_equal(np.isnan(re), np.isnan(ref_re))
    assert np.array_equal(np.isnan(im), np.isnan(ref_im))
    ok = np.isfinite(ref_re)
    z = np.stack([re[ok], im[ok]])
    zr = np.stack([ref_re[ok], ref_im[ok]])
    assert _nrm_rms(z, zr) <= 1e-11
    assert _nrm_max(z, zr) <= 1e-10


def test_dropin_fft_planes_matches_fftw_backward():
    import lofar_gb300 as L
    rng = np.random.default_rng(2)
    g = rng.standard_normal((3, 24, 40, 2))
    out = np.zeros_like(g)
    L.fft_planes(g, out, 40, 24, 3)
    ref = O.fft_planes(g)
    assert _nrm_max(out, ref) <= 1e-13
    # in place
    h = g.copy()
    L.fft_planes(h, h, 40, 24, 3)
    assert _nrm_max(h, ref) <= 1e-13


def test_dropin_accepts_device_pointers():
    import torch
    import lofar_gb300 as L
    d = np.load(GOLDEN[0])
    nx, ny, planes, support, nf, np_, dx, dw = _args(d)
    t = {k: torch.as_tensor(d[k]).cuda() for k in ("uu", "vv", "ww", "vis_real", "vis_img", "weight")}
    grid = torch.zeros((planes, ny, nx, 2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    L.wstack(planes, t["uu"].numel(), nf, np_, t["uu"], t["vv"], t["ww"], t["vis_real"],
             t["vis_img"], t["weight"], dx, dw, support, nx, ny, grid, 1)
    assert _nrm_max(grid.cpu().numpy(), d["grid"]) <= 1e-12


def _obs(n=200_000, nx=256, planes=8, seed=2, stations=48, diameter=3000.0):
    from lofar_gb300 import synth
    obs = synth.observe(n_stations=stations, diameter_m=diameter, hours=4.0, n_vis=n,
                        sky_seed=seed)
    return obs


@pytest.fixture(scope="module")
def medium():
    """256^2 x 8 planes, 200k measurements, support 7: oracle outputs in FP64."""
    obs = _obs()
    nx, planes, support = 256, 8, 7
    kw = dict(num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=support, nx=nx, ny=nx)
    grid = O.wstack(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight,
                    num_threads=0, **kw)
    res = 1.0 / 150.0   # wide field: NaN corners in the reference image
    gs = O.fft_planes(grid)
    re, im = O.phase_correction(gs, nx=nx, ny=nx, num_w_planes=planes, resolution=res,
                                wmin=obs.wmin, wmax=obs.wmax, num_threads=0)
    return dict(obs=obs, nx=nx, planes=planes, support=support, grid=grid, re=re, im=im,
                res=res)


def _plan(m, precision):
    from lofar_gb300 import Plan
    p = Plan(m["nx"], m["nx"], m["planes"], m["support"], precision=precision)
    p.set_wcorrection(m["res"], m["obs"].wmin, m["obs"].wmax)
    return p


@pytest.mark.parametrize("tile", [32, 64])
def test_plan_grid_fp64(medium, tile):
    import torch
    o = medium["obs"]
    p = _plan(medium, "fp64")
    p.set_tuning(tile=tile)
    p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    g = torch.view_as_real(p.grid()).cpu().numpy()
    assert _nrm_max(g, medium["grid"]) <= 1e-12
    st = p.stats()
    assert st["dropped_plane"] == 0 and st["points_in"] == o.n


@pytest.mark.parametrize("tile,chunk", [(64, 4096), (32, 512)])
def test_plan_grid_fp32c(medium, tile, chunk):
    import torch
    o = medium["obs"]
    p = _plan(medium, "fp32c")
    p.set_tuning(tile=tile, chunk=chunk)
    p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    g = torch.view_as_real(p.grid()).cpu().numpy().astype(np.float64)
    assert _nrm_rms(g, medium["grid"]) <= 1e-6
    assert _nrm_max(g, medium["grid"]) <= 1e-5


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32c", 1e-5)])
def test_plan_image_forward(medium, precision, tol):
    import torch
    o = medium["obs"]
    p = _plan(medium, precision)
    img = p.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    z = torch.view_as_real(img).cpu().numpy().astype(np.float64)
    re, im = medium["re"], medium["im"]
    assert np.array_equal(np.isnan(z[..., 0]), np.isnan(re))
    assert np.isnan(re).any()
    ok = np.isfinite(re)
    got = np.stack([z[..., 0][ok], z[..., 1][ok]])
    ref = np.stack([re[ok], im[ok]])
    assert _nrm_rms(got, ref) <= tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32c", 2e-6)])
def test_concentrated_bins_are_split_and_combined(precision, tol):
    """150k measurements inside a few cells: bins far above the split size are
    cut into work items whose partial tiles are combined (FP32C), or gridded
    whole (FP64); both must match the oracle."""
    import torch
    from lofar_gb300 import Plan
    rng = np.random.default_rng(21)
    n, nx, planes = 150_000, 128, 2
    uu = 0.5 + rng.normal(0, 1.5 / nx, n)
    vv = 0.37 + rng.normal(0, 1.5 / nx, n)
    ww = rng.random(n) * 0.999
    vr = rng.standard_normal(n).astype(np.float32)
    vi = rng.standard_normal(n).astype(np.float32)
    wt = np.ones(n, np.float32)
    ref = O.wstack(uu, vv, ww, vr, vi, wt, num_w_planes=planes, dx=1 / nx, dw=1 / planes,
                   w_support=7, nx=nx, ny=nx)
    p = Plan(nx, nx, planes, 7, precision=precision)
    p.set_tuning(chunk=512)
    p.bin(uu, vv, ww, vr, vi, wt)
    g = torch.view_as_real(p.grid()).double().cpu().numpy()
    assert p.stats()["max_bin_records"] > 20 * 512
    assert _nrm_rms(g, ref) <= tol
    assert _nrm_max(g, ref) <= 10 * tol


def test_single_measurement_indices_bit_exact():
    """Footprints of single measurements at awkward positions equal the oracle's
    to FP64 rounding: same cell, same plane, same clipped window."""
    import lofar_gb300 as L
    rng = np.random.default_rng(9)
    nx, ny, planes = 64, 48, 4
    us = [0.0, 1e-300, 3.0 / 64, 3.0 / 64 - 1e-17, np.nextafter(3.0 / 64, 0), 0.5,
          np.nextafter(1.0, 0.0), -0.2 / 64, -1.5 / 64, 63.999999 / 64, 65.0 / 64]
    for u in us:
        for v in (0.0, 0.37, (ny - 1e-9) / nx, -0.01 / 64):
            w = float(rng.random() * 0.999)
            args = ([u], [v], [w], np.array([1.0], np.float32), np.array([-0.5], np.float32),
                    np.array([1.0], np.float32))
            ref = O.wstack(*args, num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=7,
                           nx=nx, ny=ny, num_threads=1)
            got = np.zeros_like(ref)
            L.wstack(planes, 1, 1, 1, np.array([u]), np.array([v]), np.array([w]), *args[3:],
                     1 / nx, 1 / planes, 7, nx, ny, got, 1)
            assert np.array_equal(got != 0, ref != 0), (u, v)
            assert np.abs(got - ref).max() <= 4e-15 * max(np.abs(ref).max(), 1e-300), (u, v)


def test_out_of_range_plane_dropped_and_counted():
    from lofar_gb300 import Plan
    p = Plan(32, 32, 2, 3, precision="fp64")
    p.bin([0.5, 0.5, 0.5], [0.5, 0.5, 0.5], [1.0, -0.6, 0.2], [1.0] * 3, [0.0] * 3, [1.0] * 3)
    g = p.grid().cpu().numpy()
    st = p.stats()
    assert st["dropped_plane"] == 2
    ref = O.wstack([0.5], [0.5], [0.2], [1.0], [0.0], [1.0], num_w_planes=2, dx=1 / 32, dw=0.5,
                   w_support=3, nx=32, ny=32)
    assert np.abs(np.stack([g.real, g.imag], -1) - ref).max() <= 1e-15


def test_empty_input():
    import torch
    from lofar_gb300 import Plan
    p = Plan(64, 64, 4, 7, precision="fp32c")
    p.bin(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0, np.float32), np.zeros(0, np.float32),
          np.zeros(0, np.float32))
    g = p.grid()
    torch.cuda.synchronize()
    assert g.abs().max().item() == 0.0


def test_fp32c_grid_is_deterministic_without_split_bins(gpu):
    """Integer tile sums and an order-independent scale: two runs grid to the
    same bits although the binning's atomics order the records differently."""
    import torch
    from lofar_gb300 import Plan, synth
    o = synth.observe(n_stations=40, diameter_m=4000.0, hours=6.0, n_vis=1_500_000)
    grids = []
    for _ in range(2):
        p = Plan(1024, 1024, 8, 7, precision="fp32c")
        p.set_tuning(chunk=1 << 22)   # no bin is split
        p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
        assert p.stats()["max_bin_records"] < (1 << 22)
        grids.append(p.grid().cpu())
        p.close()
    assert torch.equal(torch.view_as_real(grids[0]), torch.view_as_real(grids[1]))


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_layout_hint_changes_only_the_walk(medium, precision):
    """The [dump][baseline] walk of the binning (wsg_plan_set_layout) with the
    observation's true baseline count, and with a wrong one, grids what the
    index-order walk grids: FP64 (which keeps the index-order walk) against the
    oracle at 1e-12, FP32C at the FP32C grid tolerances (split bins' chunks
    hold other records, so their per-item scales and roundings differ)."""
    import torch
    o = medium["obs"]
    for rows in (0, o.meta["n_baselines"], 1000, 7):
        p = _plan(medium, precision)
        p.set_layout(rows)
        p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
        g = torch.view_as_real(p.grid()).double().cpu().numpy()
        st = p.stats()
        assert st["points_in"] == o.n and st["dropped_plane"] == 0
        p.close()
        if precision == "fp64":
            assert _nrm_max(g, medium["grid"]) <= 1e-12, rows
        else:
            assert _nrm_rms(g, medium["grid"]) <= 1e-6, rows
            assert _nrm_max(g, medium["grid"]) <= 1e-5, rows


@pytest.mark.parametrize("support", [7, 9])
def test_layout_walk_grids_the_same_bits_and_counts(support):
    """The [dump][baseline] walk bins the same records as the index-order walk.
    Without split bins the FP32C grid is then bit-identical (integer tile sums
    at an order-independent scale), whatever rows count the plan is given: the
    true one (n not a multiple of it), a wrong one, n - 1 (two dumps, the last
    of one row) or more than n (index order).  The dropped-measurement counts
    agree.  The inputs hold measurements outside the planes and outside the
    grid, and NaN values; the walk's grid matches the oracle (FP32C grid
    tolerances: rms 1e-6 and max 1e-5 at support 7, twice that at 9)."""
    import torch
    from lofar_gb300 import Plan, synth
    o = synth.observe(n_stations=20, diameter_m=3000.0, hours=3.0, n_vis=190_001)
    uu, vv, ww = o.uu.copy(), o.vv.copy(), o.ww.copy()
    vr, vi, wt = o.vis_real.copy(), o.vis_img.copy(), o.weight.copy()
    n, nb = uu.shape[0], o.meta["n_baselines"]
    assert n % nb != 0
    ww[::997] = 1.5          # past the last plane
    uu[5::1009] = 3.0        # window entirely outside the grid
    vr[7::1013] = np.nan     # contributes zero (w-stacking.cu:98-112)
    nx, planes = 256, 8
    first = None
    for rows in (nb, 0, 3, n - 1, n + 5):
        p = Plan(nx, nx, planes, support, precision="fp32c")
        p.set_tuning(chunk=1 << 22)   # no bin is split
        p.set_layout(rows)
        p.bin(uu, vv, ww, vr, vi, wt)
        g = torch.view_as_real(p.grid()).cpu()
        st = p.stats()
        p.close()
        assert st["max_bin_records"] < (1 << 22)
        if first is None:
            first = (g, st)
            keep = ww < 1.0   # the oracle, like the reference, takes in-range planes only
            ref = O.wstack(uu[keep], vv[keep], ww[keep], vr[keep], vi[keep], wt[keep],
                           num_w_planes=planes, dx=1 / nx, dw=1 / planes, w_support=support,
                           nx=nx, ny=nx)
            # a support-9 window puts 81 rounded taps in a cell: twice the
            # FP32C grid tolerance of support 7
            tol = 1e-6 if support == 7 else 2e-6
            assert _nrm_rms(g.double().numpy(), ref) <= tol
            assert _nrm_max(g.double().numpy(), ref) <= 10 * tol
            assert st["dropped_plane"] == len(range(0, n, 997))
            assert st["dropped_window"] > 0
            continue
        assert torch.equal(g, first[0]), rows
        for k in ("points_in", "records", "dropped_plane", "dropped_window"):
            assert st[k] == first[1][k], (rows, k)


def test_layout_walk_folds_frequencies_and_polarisations():
    """The walk's scatter folds sum_{f,p} weight*vis with NaN flags
    (w-stacking.cu:98-112) for F, Pol > 1 like the index-order walk: the FP32C
    grid matches the oracle and, without split bins, is bit-identical to the
    index-order walk's."""
    import torch
    from lofar_gb300 import Plan, synth
    o = synth.observe(n_stations=16, diameter_m=3000.0, hours=3.0, n_vis=60_007)
    n, nb, nf, npol = o.n, o.meta["n_baselines"], 2, 2
    rng = np.random.default_rng(17)
    # the sky's visibilities, a different gain per (frequency, polarisation)
    gain = np.array([1.0, 0.9, 1.1, 0.8], np.float32).reshape(1, nf, npol)
    vr = (o.vis_real.reshape(n, 1, 1) * gain).reshape(-1)
    vi = (o.vis_img.reshape(n, 1, 1) * gain).reshape(-1)
    wt = (0.5 + 0.5 * rng.random(n * npol)).astype(np.float32)
    vr[5::97] = np.nan
    nx, planes = 128, 4
    ref = O.wstack(o.uu, o.vv, o.ww, vr, vi, wt, num_w_planes=planes, freq_per_chan=nf,
                   polarizations=npol, dx=1 / nx, dw=1 / planes, w_support=7, nx=nx, ny=nx)
    grids = []
    for rows in (nb, 0):
        p = Plan(nx, nx, planes, 7, precision="fp32c")
        p.set_tuning(chunk=1 << 22)
        p.set_layout(rows)
        p.bin(o.uu, o.vv, o.ww, vr, vi, wt, freq_per_chan=nf, polarizations=npol)
        grids.append(torch.view_as_real(p.grid()).cpu())
        p.close()
    assert torch.equal(grids[0], grids[1])
    g = grids[0].double().numpy()
    assert _nrm_rms(g, ref) <= 1e-6
    assert _nrm_max(g, ref) <= 1e-5


@pytest.mark.parametrize("support", [7, 9])
def test_layout_walk_degrid_matches_the_index_walk(support):
    """The walk's adjoint (values in record order, gathered back to measurement
    order) gives what the index-order walk's scattered stores give, with zeros
    for dropped measurements, and matches the oracle's transpose."""
    import torch
    from lofar_gb300 import Plan, synth
    o = synth.observe(n_stations=16, diameter_m=3000.0, hours=3.0, n_vis=50_011)
    uu, ww = o.uu.copy(), o.ww.copy()
    ww[::331] = 1.5   # past the last plane: no record, degridded as zero
    nx, planes = 128, 4
    gnp = np.random.default_rng(3).standard_normal((planes, nx, nx, 2))
    g = torch.view_as_complex(torch.as_tensor(gnp).contiguous()).to(torch.complex64).cuda()
    outs = []
    for rows in (o.meta["n_baselines"], 0):
        p = Plan(nx, nx, planes, support, precision="fp32c")
        p.set_layout(rows)
        p.bin(uu, o.vv, ww, o.vis_real, o.vis_img, o.weight)
        outs.append(p.degrid(g).cpu())
        p.close()
    assert torch.equal(outs[0], outs[1])
    assert bool((outs[0][::331] == 0).all())
    keep = ww < 1.0
    ref = O.degrid(uu[keep], o.vv[keep], ww[keep], gnp, num_w_planes=planes, dx=1 / nx,
                   dw=1 / planes, w_support=support, nx=nx, ny=nx)
    got = torch.view_as_real(outs[0][torch.as_tensor(keep)]).double().numpy()
    assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max()
