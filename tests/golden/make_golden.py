"""Generate the golden fixtures in this directory from the reference itself.

The outputs come from the reference's own CPU code (w-stacking.cu and
phase_correction.cu compiled as C with -DPHASE_ON by oracle/build.py into
oracle/_ref/libref.so), run single-threaded so that the results are
deterministic.  Inputs are seeded and stored in the fixtures next to the
outputs, so the fixtures are self-contained and the tests never need the
reference tree.

Run from the repository root where the reference tree is available:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lofar_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _save(name, **arrays):
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **arrays)
    print(f"{path}: {os.path.getsize(path)} bytes")


def grid_case(name, *, uu, vv, ww, vr, vi, wt, nf, np_, nx, ny, planes, support, dx=None,
              dw=None, phase=None):
    dx = 1.0 / nx if dx is None else dx
    dw = 1.0 / planes if dw is None else dw
    g = O.wstack(uu, vv, ww, vr, vi, wt, num_w_planes=planes, freq_per_chan=nf,
                 polarizations=np_, dx=dx, dw=dw, w_support=support, nx=nx, ny=ny,
                 num_threads=1, lib="ref")
    out = dict(uu=uu, vv=vv, ww=ww, vis_real=vr, vis_img=vi, weight=wt,
               params=np.array([nx, ny, planes, support, nf, np_], np.int64),
               dxdw=np.array([dx, dw], np.float64), grid=g)
    if phase is not None:
        res, wmin, wmax = phase
        gs = O.fft_planes(g)
        re, im = O.phase_correction(gs, nx=nx, ny=ny, num_w_planes=planes, resolution=res,
                                    wmin=wmin, wmax=wmax, num_threads=1, lib="ref")
        out.update(gridss=gs, image_real=re, image_imag=im,
                   wc=np.array([res, wmin, wmax], np.float64))
    _save(name, **out)


def main():
    if O.load_ref() is None:
        print("reference tree not available: cannot regenerate fixtures", file=sys.stderr)
        return 1

    # 1. synthetic LOFAR-like observation, 48 stations / 3 km / 4 h, small grid
    obs = synth.observe(n_stations=48, diameter_m=3000.0, hours=4.0, n_vis=6000)
    grid_case("obs_48x40_p4_s7", uu=obs.uu, vv=obs.vv, ww=obs.ww, vr=obs.vis_real,
              vi=obs.vis_img, wt=obs.weight, nf=1, np_=1, nx=48, ny=40, planes=4, support=7,
              phase=(1.0 / 60.0, obs.wmin, obs.wmax))

    rng = np.random.default_rng(11)

    # 2. frequency x polarisation fold with NaN flags and non-unit weights
    n = 300
    nf, np_ = 2, 2
    uu = rng.random(n)
    vv = rng.random(n)
    ww = rng.random(n) * np.nextafter(1.0, 0.0)
    vr = rng.standard_normal(n * nf * np_).astype(np.float32)
    vi = rng.standard_normal(n * nf * np_).astype(np.float32)
    vr[rng.random(vr.size) < 0.1] = np.nan
    wt = rng.uniform(0.5, 2.0, n * np_).astype(np.float32)
    grid_case("fold_f2p2_nan_32_p2_s7", uu=uu, vv=vv, ww=ww, vr=vr, vi=vi, wt=wt, nf=nf,
              np_=np_, nx=32, ny=32, planes=2, support=7)

    # 3. edges: cells on every border, coordinates in (-1/N, 0) (truncation
    #    toward zero), non-power-of-two grid and plane count (IEEE division path)
    nx, ny, planes = 40, 36, 3
    pts = []
    for u in (0.0, 0.5 / nx, 1.0 / nx, 0.5, 1.0 - 1.0 / nx, np.nextafter(1.0, 0.0), -0.3 / nx,
              -0.99 / nx):
        for v in (0.0, 0.2 / nx, 0.5, 1.0 - 0.5 / nx, -0.5 / nx, (ny - 0.5) / nx):
            pts.append((u, v))
    pts = np.array(pts)
    n = pts.shape[0]
    # (ww = nextafter(1, 0) would give plane index 3 == P here, because
    # 0.99999999999999989 / fl(1/3) rounds to 3.0: the reference then writes
    # past the end of the grid, so the largest w kept is 1 - 1e-9)
    ww = np.concatenate([rng.random(n - 4) * (1.0 - 1e-9),
                         [0.0, 1.0 / planes, 1.0 - 1e-9, -0.1 / planes]])
    vr = rng.standard_normal(n).astype(np.float32)
    vi = rng.standard_normal(n).astype(np.float32)
    wt = np.ones(n, np.float32)
    grid_case("edges_40x36_p3_s5", uu=pts[:, 0].copy(), vv=pts[:, 1].copy(), ww=ww, vr=vr, vi=vi,
              wt=wt, nf=1, np_=1, nx=nx, ny=ny, planes=planes, support=5,
              phase=(1.0 / 30.0, -20.0, 35.0))

    # 4. one measurement at a cell centre: the analytic Gaussian footprint
    grid_case("single_16_p1_s7", uu=np.array([8.5 / 16]), vv=np.array([7.5 / 16]),
              ww=np.array([0.0]), vr=np.array([1.0], np.float32),
              vi=np.array([0.0], np.float32), wt=np.array([1.0], np.float32), nf=1, np_=1,
              nx=16, ny=16, planes=1, support=7)

    # 5. single plane (phase correction reduces to the plain sum) and a wide
    #    field where sin^2+sin^2 > 1 (NaN pixels in the reference image)
    obs2 = synth.observe(n_stations=20, diameter_m=2000.0, hours=2.0, n_vis=2000, sky_seed=5)
    grid_case("p1_32_s9", uu=obs2.uu, vv=obs2.vv, ww=obs2.ww, vr=obs2.vis_real,
              vi=obs2.vis_img, wt=obs2.weight, nf=1, np_=1, nx=32, ny=32, planes=1, support=9,
              phase=(1.0 / 40.0, obs2.wmin, obs2.wmax))
    grid_case("nanfield_32_p4_s3", uu=obs2.uu, vv=obs2.vv, ww=obs2.ww, vr=obs2.vis_real,
              vi=obs2.vis_img, wt=obs2.weight, nf=1, np_=1, nx=32, ny=32, planes=4, support=3,
              phase=(1.0 / 12.0, obs2.wmin, obs2.wmax))
    return 0


if __name__ == "__main__":
    sys.exit(main())
