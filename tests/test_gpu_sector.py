"""v-slab sectoring on the GPU (wsg_sector_*, wsg_initialize_array) against the
restatement of initialize_array (oracle/binms_oracle.py), itself pinned to the
reference's own initialize_array on the fixtures (tests/test_binms.py).

Bars:
  histo_send, slab lists, gathered rows      bit-exact (integer and copy work;
                                             the v shift is one IEEE subtract)
  the decomposition (every rank, every slab, summed) vs the same
  decomposition run by the oracle             max |diff| <= 1e-12 * max |ref|

The decomposition does not reproduce the single-rank grid exactly, in the
reference as here: a row less than one cell below a slab edge is also listed
in the slab above, where its shifted v lies in (-dx, 0), and the reference's
(int) conversion (w-stacking.cu:66-71) truncates that to cell 0 instead of
-1, so its footprint there lands one row too high.  The test pins that
behaviour against the oracle and bounds it against the single-rank grid.
"""
import json
import os

import numpy as np
import pytest

from oracle import binms_oracle as B

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "binms")


def _edge_v(n, nsectors, yaxis, dx, wsh, seed):
    """Random v in [0, 1) with a tenth of the rows on or beside slab edges and
    the edges of the w_supporth bands (one ulp either side)."""
    rng = np.random.default_rng(seed)
    v = rng.random(n)
    k = rng.integers(1, nsectors, size=n // 10) if nsectors > 1 else np.ones(n // 10, int)
    base = (k * yaxis).astype(np.float64) * dx
    off = rng.choice(np.array([0.0, wsh, -wsh, 0.5 * wsh]), size=n // 10)
    e = base + off
    ulp = rng.integers(-1, 2, size=n // 10)
    e = np.where(ulp < 0, np.nextafter(e, 0.0), np.where(ulp > 0, np.nextafter(e, 1.0), e))
    v[rng.choice(n, size=n // 10, replace=False)] = np.clip(e, 0.0, np.nextafter(1.0, 0.0))
    return v


@pytest.mark.parametrize("nsectors,n", [(1, 100_000), (2, 1_000_003), (7, 777_777), (64, 2_000_000),
                                        (1023, 3_000_001)])
def test_sector_lists_bit_exact(gpu, nsectors, n):
    import torch
    from lofar_gb300 import sectors
    ny = 1024 * ((nsectors + 1023) // 1024) if nsectors > 1024 else 2048
    yaxis = ny // nsectors
    dx = 1.0 / ny
    wsh = sectors.w_supporth(7, dx)
    v = _edge_v(n, nsectors, yaxis, dx, wsh, seed=nsectors)
    histo, lists = B.initialize_array(v, nsectors, yaxis, dx, wsh)
    off_dev, off, index = sectors.sector_lists(torch.from_numpy(v).cuda(), nsectors, yaxis, dx,
                                               wsh)
    assert np.array_equal(np.diff(off), histo)
    assert np.array_equal(index.cpu().numpy(), np.concatenate(lists))
    assert histo.sum() > n   # the edge rows were duplicated


def test_initialize_array_drop_in_matches_the_reference_fixtures(gpu):
    """wsg_initialize_array on the rows of every recorded case, against the
    reference's histo_send (the lists are checked through the restatement)."""
    from lofar_gb300 import sectors
    cases = json.load(open(os.path.join(GOLD, "expected.json")))
    done = 0
    for c in cases:
        if c["short_read"]:
            continue
        p = B.parse_parameter_file(open(os.path.join(GOLD, c["paramfile"])).read())
        d = os.path.join(GOLD, p["datapath"][c["dataset"]])
        meta, start = B.partition(B.parse_metadata(open(os.path.join(d, p["metafile"])).read()),
                                  c["rank"], c["size"])
        vv = B.read_measurements(d + "/", p, meta, start)["vv"]
        dx = 1.0 / p["grid_size_x"]
        geom = (c["size"], p["grid_size_y"] // c["size"], dx,
                float((p["w_support"] - 1) // 2) * dx)
        histo, lists = sectors.initialize_array(vv, *geom)
        assert histo.tolist() == c["histo"]
        _, ref_lists = B.initialize_array(vv, *geom)
        assert all(np.array_equal(a, b) for a, b in zip(lists, ref_lists))
        done += 1
    assert done >= 20


def test_gather_bit_exact(gpu):
    import torch
    from lofar_gb300 import sectors
    rng = np.random.default_rng(5)
    n, nf, npol, S, ny = 300_000, 3, 2, 5, 1000
    yaxis, dx = ny // S, 1.0 / 1024
    wsh = sectors.w_supporth(9, dx)
    host = {"uu": rng.random(n), "vv": rng.random(n) * (S * yaxis * dx), "ww": rng.random(n),
            "weights": rng.random(n * npol).astype(np.float32),
            "vis_real": rng.standard_normal(n * nf * npol).astype(np.float32),
            "vis_img": rng.standard_normal(n * nf * npol).astype(np.float32)}
    dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
    _, off, index = sectors.sector_lists(dev["vv"], S, yaxis, dx, wsh)
    _, lists = B.initialize_array(host["vv"], S, yaxis, dx, wsh)
    for s in range(S + 1):
        got = sectors.sector_gather(index, off, s, yaxis, dx, nf, npol, **dev)
        want = B.sector_compose(lists[s], s, yaxis, dx, host["uu"], host["vv"], host["ww"],
                                host["weights"], host["vis_real"], host["vis_img"], nf, npol)
        for k in want:
            assert np.array_equal(got[k].cpu().numpy(), want[k]), (s, k)


def _oracle_by_slabs(ranks, *, nx, ny, planes, w_support, nf, npol, uu, vv, ww, weights,
                     vis_real, vis_img):
    from oracle import oracle as O
    yaxis, dx = ny // ranks, 1.0 / nx
    wsh = float((w_support - 1) // 2) * dx
    full = np.zeros((planes, ny, nx, 2))
    n = uu.shape[0]
    per, rem = divmod(n, ranks)
    for r in range(ranks):
        a = r * per
        b = a + per + (rem if r == ranks - 1 else 0)
        _, lists = B.initialize_array(vv[a:b], ranks, yaxis, dx, wsh)
        for s in range(ranks):
            c = B.sector_compose(lists[s], s, yaxis, dx, uu[a:b], vv[a:b], ww[a:b],
                                 weights[a * npol:b * npol], vis_real[a * nf * npol:b * nf * npol],
                                 vis_img[a * nf * npol:b * nf * npol], nf, npol)
            if len(c["uu"]):
                full[:, s * yaxis:(s + 1) * yaxis] += O.wstack(
                    c["uu"], c["vv"], c["ww"], c["vis_real"], c["vis_img"], c["weights"],
                    num_w_planes=planes, freq_per_chan=nf, polarizations=npol, dx=dx,
                    dw=1.0 / planes, w_support=w_support, nx=nx, ny=yaxis)
    return full


def test_slab_decomposition_matches_the_oracle(gpu):
    """The reference's multi-rank decomposition (row shares, slab lists with
    edge duplicates, per-slab gather and gridding, the reduction) on one GPU,
    against the same decomposition run by the oracle; with one rank it is the
    single-rank grid."""
    import torch
    from lofar_gb300 import sectors, synth
    from oracle import oracle as O
    nx = ny = 256
    planes, support, nf, npol = 8, 7, 2, 2
    obs = synth.observe(n_stations=24, diameter_m=3000.0, hours=4.0, n_vis=60_000)
    rng = np.random.default_rng(9)
    n = obs.uu.shape[0]
    vr = rng.standard_normal(n * nf * npol).astype(np.float32)
    vi = rng.standard_normal(n * nf * npol).astype(np.float32)
    wt = rng.random(n * npol).astype(np.float32)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
           (("uu", obs.uu), ("vv", obs.vv), ("ww", obs.ww), ("weights", wt), ("vis_real", vr),
            ("vis_img", vi))}
    single = O.wstack(obs.uu, obs.vv, obs.ww, vr, vi, wt, num_w_planes=planes,
                      freq_per_chan=nf, polarizations=npol, dx=1 / nx, dw=1 / planes,
                      w_support=support, nx=nx, ny=ny)
    geo = dict(nx=nx, ny=ny, planes=planes, w_support=support, nf=nf, npol=npol)
    for ranks in (1, 4):
        g = sectors.grid_by_slabs(ranks, **geo, **dev).cpu().numpy()
        ref = single if ranks == 1 else _oracle_by_slabs(
            ranks, **geo, uu=obs.uu, vv=obs.vv, ww=obs.ww, weights=wt, vis_real=vr, vis_img=vi)
        err = np.abs(g - ref).max() / np.abs(ref).max()
        assert err <= 1e-12, (ranks, err)
        if ranks > 1:
            # the truncation at the slab edges: rows just above each edge only
            dev_rows = np.nonzero(np.abs(g - single).max(axis=(0, 2, 3)) >
                                  1e-12 * np.abs(single).max())[0]
            assert set(dev_rows % (ny // ranks)) <= {1, 2, 3}, dev_rows


def test_sector_errors(gpu):
    import torch
    from lofar_gb300 import _lib, sectors
    from lofar_gb300._lib import WstackError
    v = torch.tensor([0.1, 0.5, 2.5], dtype=torch.float64, device="cuda")
    with pytest.raises(WstackError) as e:
        sectors.sector_lists(v, 1, 64, 1 / 64, 3 / 64)
    assert e.value.status == _lib.WSG_ERR_ARG
    v = torch.tensor([0.1, float("nan")], dtype=torch.float64, device="cuda")
    with pytest.raises(WstackError):
        sectors.sector_lists(v, 4, 16, 1 / 64, 3 / 64)
    lib = _lib.load()
    v = torch.rand(1000, dtype=torch.float64, device="cuda")
    off = torch.empty(6, dtype=torch.int64, device="cuda")
    idx = torch.empty(10, dtype=torch.int64, device="cuda")
    assert lib.wsg_sector_lists(v.data_ptr(), 1000, 4, 16, 1 / 64, 3 / 64, off.data_ptr(),
                                idx.data_ptr(), 10, None) == _lib.WSG_ERR_CAPACITY
