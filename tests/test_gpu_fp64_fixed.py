"""The FP64 form's fixed-point taps (grid.cu k_grid_f64, degrid.cu
k_degrid_f64, fixed64.cuh).

The FP64 gridder sums each work item's taps (a bin, or a chunk of at most
4096 records of a split bin) as 64-bit integers at a power-of-two scale fixed
by the largest exponent of the item's values; the degridder
converts each staged tile to 64-bit integers at the tile's own scale.  Bins
and tiles holding a NaN or an infinity take FP64 arithmetic instead, so that
non-finite values propagate as in the reference (w-stacking.cu:103-112: a
finite real part with a NaN imaginary part is gridded, and the NaN spreads
over the measurement's window).

Tolerances:
  grid, degrid vs the oracle        max |diff| <= 1e-12 * max |ref| over the
                                    finite cells; NaN masks identical
  two FP64 gridding runs            bit-identical when no bin is split
                                    (integer sums, bounds that do not depend
                                    on the records' order)
  split bins, gridded twice         rms 1e-12 (FP64), 2e-6 (FP32C) both times
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NX, PLANES, SUPPORT = 256, 8, 7
KW = dict(num_w_planes=PLANES, dx=1 / NX, dw=1 / PLANES, w_support=SUPPORT, nx=NX, ny=NX)


def _obs(n=150_000, seed=4):
    from lofar_gb300 import synth
    return synth.observe(n_stations=40, diameter_m=3000.0, hours=4.0, n_vis=n, sky_seed=seed)


def _grid_gpu(o, vr, vi):
    import torch
    from lofar_gb300 import Plan
    p = Plan(NX, NX, PLANES, SUPPORT, precision="fp64")
    p.bin(o.uu, o.vv, o.ww, vr, vi, o.weight)
    g = torch.view_as_real(p.grid()).cpu().numpy()
    p.close()
    return g


def _cmp_finite(got, ref):
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = np.isfinite(ref)
    return float(np.abs(got[ok] - ref[ok]).max() / np.abs(ref[ok]).max())


def test_fp64_grid_is_deterministic(gpu):
    """Bins of at most 4096 records sum in fixed point at a scale that does not
    depend on the records' order: two runs grid to the same bits although
    the binning's atomics order the records differently."""
    import torch
    from lofar_gb300 import Plan, synth
    o = synth.observe(n_stations=40, diameter_m=4000.0, hours=6.0, n_vis=200_000)
    grids = []
    for _ in range(2):
        p = Plan(1024, 1024, 8, 7, precision="fp64")
        p.set_tuning(tile=32, chunk=1 << 22)   # no bin is split
        p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
        assert p.stats()["max_bin_records"] <= 4096
        grids.append(p.grid().cpu())
        p.close()
    assert torch.equal(torch.view_as_real(grids[0]), torch.view_as_real(grids[1]))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32c", 2e-6)])
def test_split_bins_grid_again_after_one_binning(gpu, precision, tol):
    """A second wsg_grid after one wsg_bin combines the split bins' partial
    tiles again (the combining CTA rearms the bin's counter)."""
    import torch
    from lofar_gb300 import Plan
    o = _obs(seed=12)
    ref = O.wstack(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, **KW)
    p = Plan(NX, NX, PLANES, SUPPORT, precision=precision)
    p.set_tuning(chunk=512)
    p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    assert p.stats()["max_bin_records"] > 4 * 512
    for _ in range(2):
        g = torch.view_as_real(p.grid()).double().cpu().numpy()
        assert float(np.sqrt(((g - ref) ** 2).mean() / (ref ** 2).mean())) <= tol
    p.close()


def test_fp64_grid_nan_imaginary_part_propagates(gpu):
    o = _obs()
    vr, vi = o.vis_real.copy(), o.vis_img.copy()
    rng = np.random.default_rng(9)
    bad = rng.choice(o.n, 3, replace=False)
    vi[bad] = np.nan                      # unflagged: the real part is finite
    vr[rng.choice(o.n, 50, replace=False)] = np.nan   # flagged: skipped
    ref = O.wstack(o.uu, o.vv, o.ww, vr, vi, o.weight, **KW)
    got = _grid_gpu(o, vr, vi)
    assert np.isnan(ref[..., 1]).any() and not np.isnan(ref[..., 0]).any()
    assert _cmp_finite(got, ref) <= 1e-12


@pytest.mark.parametrize("scale", [1e-30, 1e30])
def test_fp64_grid_extreme_scales(gpu, scale):
    o = _obs(seed=6)
    vr = (o.vis_real.astype(np.float64) * scale).astype(np.float32)
    vi = (o.vis_img.astype(np.float64) * scale).astype(np.float32)
    ref = O.wstack(o.uu, o.vv, o.ww, vr, vi, o.weight, **KW)
    got = _grid_gpu(o, vr, vi)
    assert _cmp_finite(got, ref) <= 1e-12


def test_fp64_degrid_nan_cell_propagates(gpu):
    import torch
    from lofar_gb300 import Plan
    o = _obs(seed=8)
    rng = np.random.default_rng(10)
    g = rng.standard_normal((PLANES, NX, NX, 2))
    g[:, NX // 2 + 2, :, 1] = np.nan      # a row near v = 0 in every plane
    ref = O.degrid(o.uu, o.vv, o.ww, g, **KW)
    p = Plan(NX, NX, PLANES, SUPPORT, precision="fp64")
    p.bin(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
    gt = torch.view_as_complex(torch.as_tensor(np.ascontiguousarray(g))).cuda()
    out = torch.view_as_real(p.degrid(gt)).cpu().numpy()
    p.close()
    # the weights are real: a NaN imaginary part of a cell makes the
    # imaginary part of every output whose window holds the cell NaN
    assert np.isnan(ref[:, 1]).any() and not np.isnan(ref[:, 0]).any()
    assert _cmp_finite(out, ref) <= 1e-12


def test_fp64_negative_coordinates(gpu):
    """The reference's cell is pos truncated toward zero, so a measurement just
    below u = 0 or v = 0 has a fraction in (-1, 0] and its window reaches onto
    the grid from outside: the factorised weights then take exp(c) up to
    e^1.5.  Grid and degrid match the oracle."""
    import torch
    from lofar_gb300 import Plan
    o = _obs(seed=14)
    rng = np.random.default_rng(15)
    k = 3000
    uu = np.concatenate([o.uu, rng.uniform(-3.0 / NX, 0.0, k), rng.uniform(0.2, 0.8, k)])
    vv = np.concatenate([o.vv, rng.uniform(0.2, 0.8, k), rng.uniform(-3.0 / NX, 0.0, k)])
    ww = np.concatenate([o.ww, rng.uniform(0.0, 0.99, 2 * k)])
    vr = np.concatenate([o.vis_real, rng.standard_normal(2 * k).astype(np.float32)])
    vi = np.concatenate([o.vis_img, rng.standard_normal(2 * k).astype(np.float32)])
    wt = np.concatenate([o.weight, np.ones(2 * k, np.float32)])
    ref = O.wstack(uu, vv, ww, vr, vi, wt, **KW)
    p = Plan(NX, NX, PLANES, SUPPORT, precision="fp64")
    p.bin(uu, vv, ww, vr, vi, wt)
    g = torch.view_as_real(p.grid()).cpu().numpy()
    assert _cmp_finite(g, ref) <= 1e-12
    gin = np.random.default_rng(16).standard_normal((PLANES, NX, NX, 2))
    dref = O.degrid(uu, vv, ww, gin, **KW)
    gt = torch.view_as_complex(torch.as_tensor(np.ascontiguousarray(gin))).cuda()
    out = torch.view_as_real(p.degrid(gt)).cpu().numpy()
    p.close()
    assert _cmp_finite(out, dref) <= 1e-12
