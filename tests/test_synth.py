"""Synthetic observation generator: layout, ranges, determinism."""
import numpy as np

from lofar_gb300 import synth


def test_layout_and_ranges():
    obs = synth.observe(n_stations=10, diameter_m=1000.0, hours=1.0, n_vis=1000)
    assert obs.n == 1000 and obs.n_vis == 1000
    for a in (obs.uu, obs.vv, obs.ww):
        assert a.dtype == np.float64 and a.min() >= 0.0 and a.max() < 1.0
    assert obs.vis_real.dtype == np.float32 and obs.weight.dtype == np.float32
    assert (obs.weight == 1).all()
    assert obs.meta["n_baselines"] == 45
    # time-major: the first n_baselines rows are dump 0
    assert obs.meta["n_dumps"] == -(-1000 // 45)


def test_deterministic():
    a = synth.observe(n_stations=8, diameter_m=500.0, hours=1.0, n_vis=200)
    b = synth.observe(n_stations=8, diameter_m=500.0, hours=1.0, n_vis=200)
    for k in ("uu", "vv", "ww", "vis_real", "vis_img"):
        assert np.array_equal(getattr(a, k), getattr(b, k))


def test_uv_origin_maps_to_grid_centre():
    obs = synth.observe(n_stations=12, diameter_m=1000.0, hours=2.0, n_vis=2000)
    u = (obs.uu - 0.5) * 2 * obs.meta["U"]
    assert abs(np.abs(u).max() - obs.meta["U"]) / obs.meta["U"] < 1e-9 or np.abs(u).max() <= obs.meta["U"]


def test_point_source_visibility_model():
    sky = (np.array([2.0]), np.array([0.01]), np.array([-0.005]),
           np.array([np.sqrt(1 - 0.01 ** 2 - 0.005 ** 2)]))
    u, v, w = np.array([100.0]), np.array([-50.0]), np.array([20.0])
    vis = synth.point_source_vis(u, v, w, sky)
    ph = -2 * np.pi * (100 * 0.01 + 50 * 0.005 + 20 * (sky[3][0] - 1))
    np.testing.assert_allclose(vis[0], 2.0 * np.exp(1j * ph), rtol=1e-14)


def test_reference_resolution_rule():
    assert synth.reference_resolution(-1499.9, 1428.6) == 1.0 / 1499


def test_batch_generator_is_seeded_and_shares_one_grid():
    a = synth.observe_batch(n_channels=4, pols=4, n_per_channel=3000, n_stations=20,
                            diameter_m=2000.0, hours=2.0)
    b = synth.observe_batch(n_channels=4, pols=4, n_per_channel=3000, n_stations=20,
                            diameter_m=2000.0, hours=2.0)
    assert len(a.channels) == 4
    for ca, cb in zip(a.channels, b.channels):
        for x, y in zip(ca, cb):
            assert np.array_equal(x, y)
    counts = [c[0].shape[0] for c in a.channels]
    # per-channel flagging: uneven counts, each between 40% and 100% of 3000
    assert len(set(counts)) == 4 and all(0.35 * 3000 < n <= 3000 for n in counts)
    for c in a.channels:
        n = c[0].shape[0]
        assert all(x.shape == (n,) for x in c[:3])
        assert all(x.shape == (n * 4,) and x.dtype == np.float32 for x in c[3:])
        for x in c[:3]:
            assert x.min() >= 0.0 and x.max() < 1.0
    # uv extent grows with frequency on the shared grid
    spread = [np.abs(c[0] - 0.5).max() for c in a.channels]
    assert spread == sorted(spread)
    assert a.n_vis == sum(counts) * 4
    assert 0.0 <= a.flag_fraction.min() and a.flag_fraction.max() <= 0.6


def test_device_generator_matches_host_geometry():
    """The chunked generator (for workloads too large for host memory) gives
    observe()'s coordinates and metadata exactly, whatever the chunking."""
    o = synth.observe(n_stations=20, diameter_m=2000.0, hours=2.0, n_vis=50_000)
    for chunk in (7, 1000):
        d = synth.observe_device(n_stations=20, diameter_m=2000.0, hours=2.0, n_vis=50_000,
                                 device="cpu", chunk_dumps=chunk)
        for k in ("uu", "vv", "ww"):
            assert np.array_equal(d[k].numpy(), getattr(o, k))
        assert (d["wmin"], d["wmax"], d["resolution"]) == (o.wmin, o.wmax, o.resolution)
        assert d["vis_real"].dtype.is_floating_point and d["weight"].numpy().min() == 1.0
        # same sky, noise of the same level
        diff = d["vis_real"].numpy().astype(np.float64) - o.vis_real
        assert 0.05 < diff.std() < 0.3
