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
