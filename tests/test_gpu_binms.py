"""The reference's main() end to end on the GPU: files in, dump files out.

Datasets are written in the reference's input layout (lofar_gb300.binms.
write_dataset): meta.txt, float64 uvw, float32 weights and values, with the
1000 trailing rows that the reader drops set to values that would land
outside the grid, and two rows off the reference's single v-slab (|vv| >= 1,
gridding.c:42-56) that must not be gridded.  The driver (wsg_run_paramfile,
and its executable) reads them, grids, transforms and w-corrects on the GPU
and writes the reference's dump files; these are compared with the oracle run
on the rows the reference grids.

Tolerances (as in the parity tests):
  FP64 grid dump, fft dump     max |diff| <= 1e-12 * max |ref|
  FP64 image dump              relative rms 1e-11 over finite pixels, NaN mask
                               identical
  FP32C image dump             relative rms 1e-5 over finite pixels
  device cube dump             bit-exact (widening and a power-of-two scale)
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NX, PLANES, SUPPORT = 256, 8, 7


def _nrm_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _rel_rms_finite(re, im, ref_re, ref_im):
    assert np.array_equal(np.isnan(re), np.isnan(ref_re))
    assert np.array_equal(np.isnan(im), np.isnan(ref_im))
    ok = np.isfinite(ref_re) & np.isfinite(ref_im)
    d = (re[ok] - ref_re[ok]) ** 2 + (im[ok] - ref_im[ok]) ** 2
    r = ref_re[ok] ** 2 + ref_im[ok] ** 2
    return float(np.sqrt(d.mean() / r.mean()))


def _write(directory, seed, n, nf, npol, stations):
    from lofar_gb300 import binms, synth
    obs = synth.observe(n_stations=stations, diameter_m=3000.0, hours=4.0, n_vis=n,
                        sky_seed=seed, noise_seed=seed + 1)
    rng = np.random.default_rng(seed)
    uu, vv, ww = obs.uu.copy(), obs.vv.copy(), obs.ww.copy()
    vv[5], vv[17] = 1.25, -1.5
    gains = (rng.standard_normal(nf * npol) + 1j * rng.standard_normal(nf * npol)) * 0.5 + 1.0
    vis = (obs.vis_real + 1j * obs.vis_img)[:, None] * gains[None, :]
    vr, vi = vis.real.astype(np.float32), vis.imag.astype(np.float32)
    vr[rng.random(vr.shape) < 0.01] = np.nan          # flagged (w-stacking.cu:104)
    wt = rng.random((n, npol)).astype(np.float32) + 0.5
    junk = 1000
    full = dict(
        uu=np.concatenate([uu, np.full(junk, 0.5)]),
        vv=np.concatenate([vv, np.full(junk, 0.5)]),
        ww=np.concatenate([ww, np.full(junk, 7.0)]),          # w-plane 56: outside the cube
        weights=np.concatenate([wt.reshape(-1), np.full(junk * npol, 1e6, np.float32)]),
        vis_real=np.concatenate([vr.reshape(-1), np.full(junk * nf * npol, 1e6, np.float32)]),
        vis_img=np.concatenate([vi.reshape(-1), np.full(junk * nf * npol, 1e6, np.float32)]))
    binms.write_dataset(directory, freq_per_chan=nf, polarisations=npol, uvmin=obs.uvmin,
                        uvmax=obs.uvmax, wmin=obs.wmin, wmax=obs.wmax, **full)
    keep = np.abs(vv) < 1.0
    rows = dict(uu=uu[keep], vv=vv[keep], ww=ww[keep], vis_real=vr[keep].reshape(-1),
                vis_img=vi[keep].reshape(-1), weight=wt[keep].reshape(-1))
    return rows, obs, nf, npol, int((~keep).sum())


def _oracle(rows, obs, nf, npol):
    grid = O.wstack(rows["uu"], rows["vv"], rows["ww"], rows["vis_real"], rows["vis_img"],
                    rows["weight"], num_w_planes=PLANES, freq_per_chan=nf, polarizations=npol,
                    dx=1 / NX, dw=1 / PLANES, w_support=SUPPORT, nx=NX, ny=NX)
    fft = O.fft_planes(grid)
    res = O.resolution(obs.uvmin, obs.uvmax)
    re, im = O.phase_correction(fft, nx=NX, ny=NX, num_w_planes=PLANES, resolution=res,
                                wmin=obs.wmin, wmax=obs.wmax)
    return grid, fft, re, im, res


@pytest.fixture(scope="module")
def run_dir(gpu, tmp_path_factory):
    d = tmp_path_factory.mktemp("binms_run")
    ds = [_write(str(d / "ds0") + "/", 21, 20000, 2, 2, 24),
          _write(str(d / "ds1") + "/", 31, 12000, 1, 1, 20)]
    (d / "paramfile.txt").write_text(
        f"ndatasets 2\nDatapath1 {d}/ds0/\nDatapath2 {d}/ds1/\nnum_threads 1\n"
        f"w_support {SUPPORT}\ngrid_size_x {NX}\ngrid_size_y {NX}\nnum_w_planes {PLANES}\n"
        "ufile ucoord.bin\nvfile vcoord.bin\nwfile wcoord.bin\nweightsfile weights.bin\n"
        "visrealfile visibilities_real.bin\nvisimgfile visibilities_img.bin\nmetafile meta.txt\n"
        "outfile2 grid_real.bin\noutfile3 grid_img.bin\nfftfile2 fft_real.bin\n"
        "fftfile3 fft_img.bin\ntimingfile timings.dat\n")
    return d, ds, [_oracle(*x[:4]) for x in ds]


def test_driver_grid_and_fft_dumps_match_the_oracle(run_dir):
    from lofar_gb300 import binms
    d, ds, ref = run_dir
    out = d / "out_data"
    out.mkdir()
    rep = binms.run(d / "paramfile.txt", write_data=True, outdir=out)
    assert rep["datasets"] == 2
    assert rep["dropped"] == ds[0][4] + ds[1][4] == 4
    assert rep["Nmeasures"] == len(ds[1][0]["uu"])
    for k, (grid, fft, _, _, res) in enumerate(ref):
        g = binms.read_dump(out / f"{k}grid_real.bin", out / f"{k}grid_img.bin", (PLANES, NX, NX))
        assert _nrm_max(np.stack([g.real, g.imag], -1), grid) <= 1e-12
        f = binms.read_dump(out / f"{k}fft_real.bin", out / f"{k}fft_img.bin", (PLANES, NX, NX))
        assert _nrm_max(np.stack([f.real, f.imag], -1), fft) <= 1e-12
        t = (out / f"{k}timings.dat").read_text().split()
        assert len(t) == 7 and all(float(x) >= 0 for x in t)
    assert rep["resolution"] == ref[1][4]


def test_driver_image_dump_matches_the_oracle(run_dir):
    from lofar_gb300 import binms
    d, ds, ref = run_dir
    out = d / "out_image"
    out.mkdir()
    binms.run(d / "paramfile.txt", write_image=True, outdir=out)
    for k, (_, _, ref_re, ref_im, _) in enumerate(ref):
        # WRITE_IMAGE reuses the fft dump's names (fourier_transform.c:186-187)
        re = np.fromfile(out / f"{k}fft_real.bin", dtype=np.float64).reshape(NX, NX)
        im = np.fromfile(out / f"{k}fft_img.bin", dtype=np.float64).reshape(NX, NX)
        assert _rel_rms_finite(re, im, ref_re, ref_im) <= 1e-11
        assert not (out / f"{k}grid_real.bin").exists()


def test_driver_fp32c_image(run_dir):
    from lofar_gb300 import binms
    d, ds, ref = run_dir
    out = d / "out_fp32c"
    out.mkdir()
    binms.run(d / "paramfile.txt", write_image=True, precision="fp32c", outdir=out)
    for k, (_, _, ref_re, ref_im, _) in enumerate(ref):
        re = np.fromfile(out / f"{k}fft_real.bin", dtype=np.float64).reshape(NX, NX)
        im = np.fromfile(out / f"{k}fft_img.bin", dtype=np.float64).reshape(NX, NX)
        assert _rel_rms_finite(re, im, ref_re, ref_im) <= 1e-5


def test_runner_executable(run_dir):
    from lofar_gb300 import build
    d, ds, ref = run_dir
    out = d / "out_exe"
    out.mkdir()
    r = subprocess.run([build.RUNNER, str(d / "paramfile.txt"), "--write-image", "--outdir",
                        str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for line in ("Dataset 0", "Dataset 1", "Subtracting last 1000 measurements",
                 f"N. measurements {20000}", "PERFORMING FFT", "PHASE CORRECTION", "WRITING IMAGE",
                 "TOTAL time"):
        assert line in r.stdout, line
    re = np.fromfile(out / "1fft_real.bin", dtype=np.float64).reshape(NX, NX)
    im = np.fromfile(out / "1fft_img.bin", dtype=np.float64).reshape(NX, NX)
    assert _rel_rms_finite(re, im, ref[1][2], ref[1][3]) <= 1e-11


@pytest.mark.parametrize("precision,shape,scale", [("fp32c", (3, 2048, 4096), 0.5),
                                                   ("fp64", (2, 512, 384), 1.0 / 1024)])
def test_device_cube_dump(gpu, tmp_path, precision, shape, scale):
    """The chunked, double-buffered device dump (8M values a chunk: the first
    case spans three chunks and reuses a staging slot)."""
    import torch
    from lofar_gb300 import Plan, binms
    p, ny, nx = shape
    plan = Plan(nx, ny, p, 7, precision=precision)
    g = torch.Generator(device="cuda").manual_seed(3)
    dt = torch.complex64 if precision == "fp32c" else torch.complex128
    cube = torch.randn((p, ny, nx), dtype=dt, device="cuda", generator=g)
    binms.plan_dump_cube(plan, cube, tmp_path / "re.bin", tmp_path / "im.bin", scale=scale)
    c = cube.cpu().numpy().astype(np.complex128)
    assert np.array_equal(np.fromfile(tmp_path / "re.bin", dtype=np.float64),
                          (c.real * scale).reshape(-1))
    assert np.array_equal(np.fromfile(tmp_path / "im.bin", dtype=np.float64),
                          (c.imag * scale).reshape(-1))
    plan.close()
    os.remove(tmp_path / "re.bin")
    os.remove(tmp_path / "im.bin")


def test_driver_grid_dump_matches_the_reference_own_dump(gpu, tmp_path, monkeypatch):
    """The reference's own single-rank run (init.c reader, gridding.c sector
    loop and WRITE_DATA dump, recorded in tests/golden/binms/ref_grid/) and
    wsg_run_paramfile on the GPU read the same files with the same parameter
    file; their grid dumps agree to FP64 summation order."""
    from lofar_gb300 import binms
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "binms")
    monkeypatch.chdir(gold)
    p = binms.read_parameter_file("paramfile_grid.txt")
    out = tmp_path / "out"
    out.mkdir()
    binms.run("paramfile_grid.txt", write_data=True, outdir=out, write_timings=False)
    shape = (p["num_w_planes"], p["grid_size_y"], p["grid_size_x"])
    got = binms.read_dump(out / f"0{p['outfile2']}", out / f"0{p['outfile3']}", shape)
    ref = binms.read_dump(os.path.join(gold, "ref_grid", "0grid_real.bin"),
                          os.path.join(gold, "ref_grid", "0grid_img.bin"), shape)
    assert np.abs(ref).max() > 0
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
