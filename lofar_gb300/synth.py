"""Seeded synthetic interferometer observations in the reference's input layout.

The reference reads measurement sets written as raw binaries (``init.c:390-501``):
``uu, vv, ww`` float64 per measurement, ``weight`` float32 as ``[m][pol]`` and
``vis_real, vis_img`` float32 as ``[m][freq][pol]``.  Its gridder takes
coordinates already normalised so that ``cell = (int)(uu/dx)`` with
``dx = 1/Nx`` and ``plane = (int)(ww/dw)`` with ``dw = 1/P``
(``w-stacking.cu:66-71``, ``init.c:16-17``); so ``uu, vv, ww`` must lie in
``[0, 1)``.  Its own dataset is not available, so this module synthesises one:

* stations uniform in a disk of the given diameter (seeded);
* every station pair once (no autocorrelations, no conjugates), time-major
  rows (all baselines of dump 0, then dump 1, ...), truncated to ``n_vis``;
* earth-rotation uvw tracks (Thompson, Moran & Swenson, eq. 4.1) over the given
  hours at declination +45 deg from latitude 52.9 deg, in wavelengths;
* values ``sum_s S_s exp(-2 pi i (u l_s + v m_s + w (n_s - 1)))`` for 20 point
  sources (flux log-uniform 0.1-10 Jy, l, m uniform in +-0.02 rad) plus complex
  Gaussian noise, sigma 0.1 per component; weights 1.

Normalisation: ``u / (2 U)`` lies in ``[-0.5, 0.5]`` with ``U = max(|u|, |v|)``;
the reference indexes from the grid corner, so ``uu = 0.5 + u/(2U)`` is passed
(uv origin at cell ``Nx/2``), clamped below 1 with ``nextafter``.  ``w`` is mapped
to ``(w - wmin)/(wmax - wmin)``, also clamped below 1.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

C_LIGHT = 299_792_458.0
LOFAR_LATITUDE_DEG = 52.9


@dataclass
class Observation:
    uu: np.ndarray          # float64 [n], in [0, 1)
    vv: np.ndarray          # float64 [n], in [0, 1)
    ww: np.ndarray          # float64 [n], in [0, 1)
    vis_real: np.ndarray    # float32 [n*F*Pol], [m][f][p]
    vis_img: np.ndarray     # float32 [n*F*Pol]
    weight: np.ndarray      # float32 [n*Pol], [m][p]
    freq_per_chan: int
    polarizations: int
    uvmin: float            # metadata fields of meta.txt (init.c:293-296), wavelengths
    uvmax: float
    wmin: float
    wmax: float
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.uu.shape[0])

    @property
    def n_vis(self) -> int:
        return self.n * self.freq_per_chan * self.polarizations

    @property
    def resolution(self) -> float:
        return reference_resolution(self.uvmin, self.uvmax)


def reference_resolution(uvmin: float, uvmax: float) -> float:
    """gridding.c:160: 1/MAX(abs(uvmin), abs(uvmax)) with C int abs (truncation)."""
    a = abs(int(math.trunc(uvmin)))
    b = abs(int(math.trunc(uvmax)))
    return 1.0 / float(max(a, b))


def stations(n_stations: int, diameter_m: float, seed: int) -> np.ndarray:
    """East/north positions [n, 2] in metres, uniform in a disk."""
    rng = np.random.default_rng(seed)
    r = 0.5 * diameter_m * np.sqrt(rng.random(n_stations))
    th = 2.0 * np.pi * rng.random(n_stations)
    return np.stack([r * np.cos(th), r * np.sin(th)], axis=1)


def baselines_xyz(pos_en: np.ndarray, lat_deg: float = LOFAR_LATITUDE_DEG) -> np.ndarray:
    """Equatorial (X, Y, Z) baseline vectors [n_bl, 3] in metres, pairs i<j."""
    lat = math.radians(lat_deg)
    e, nn = pos_en[:, 0], pos_en[:, 1]
    x = -nn * math.sin(lat)
    y = e
    z = nn * math.cos(lat)
    i, j = np.triu_indices(pos_en.shape[0], k=1)
    return np.stack([x[j] - x[i], y[j] - y[i], z[j] - z[i]], axis=1)


def uvw_tracks(bl_xyz: np.ndarray, n_dumps: int, hours: float, dec_deg: float,
               freq_hz: float) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """uvw in wavelengths, [n_dumps, n_bl] each (TMS eq. 4.1)."""
    h = np.deg2rad(np.linspace(-hours / 2, hours / 2, n_dumps) * 15.0)[:, None]
    d = math.radians(dec_deg)
    lx, ly, lz = bl_xyz[None, :, 0], bl_xyz[None, :, 1], bl_xyz[None, :, 2]
    sh, ch = np.sin(h), np.cos(h)
    scale = freq_hz / C_LIGHT
    u = (sh * lx + ch * ly) * scale
    v = (-math.sin(d) * ch * lx + math.sin(d) * sh * ly + math.cos(d) * lz) * scale
    w = (math.cos(d) * ch * lx - math.cos(d) * sh * ly + math.sin(d) * lz) * scale
    return u, v, w


def sky_model(seed: int, n_sources: int = 20, flux=(0.1, 10.0), lm_max: float = 0.02):
    rng = np.random.default_rng(seed)
    s = np.exp(rng.uniform(math.log(flux[0]), math.log(flux[1]), n_sources))
    l = rng.uniform(-lm_max, lm_max, n_sources)
    m = rng.uniform(-lm_max, lm_max, n_sources)
    n = np.sqrt(1.0 - l * l - m * m)
    return s, l, m, n


def point_source_vis(u, v, w, sky, chunk: int = 1 << 20):
    """Complex128 visibilities of a point-source sky at (u, v, w) wavelengths."""
    s, l, m, n = sky
    out = np.zeros(u.shape[0], np.complex128)
    for a in range(0, u.shape[0], chunk):
        b = min(a + chunk, u.shape[0])
        ph = -2.0 * np.pi * (np.outer(u[a:b], l) + np.outer(v[a:b], m) + np.outer(w[a:b], n - 1.0))
        out[a:b] = (s[None, :] * np.exp(1j * ph)).sum(axis=1)
    return out


def point_source_vis_torch(u, v, w, sky, device="cuda", chunk: int = 1 << 22):
    """Same as point_source_vis, evaluated with torch on `device` (float64)."""
    import torch
    s, l, m, n = (torch.as_tensor(x, dtype=torch.float64, device=device) for x in sky)
    re = np.empty(u.shape[0], np.float64)
    im = np.empty(u.shape[0], np.float64)
    for a in range(0, u.shape[0], chunk):
        b = min(a + chunk, u.shape[0])
        tu = torch.as_tensor(u[a:b], device=device)[:, None]
        tv = torch.as_tensor(v[a:b], device=device)[:, None]
        tw = torch.as_tensor(w[a:b], device=device)[:, None]
        ph = -2.0 * math.pi * (tu * l + tv * m + tw * (n - 1.0))
        re[a:b] = (s * torch.cos(ph)).sum(1).cpu().numpy()
        im[a:b] = (s * torch.sin(ph)).sum(1).cpu().numpy()
    return re + 1j * im


def _below_one(x: np.ndarray) -> np.ndarray:
    return np.minimum(x, np.nextafter(1.0, 0.0))


def observe(*, n_stations: int, diameter_m: float, hours: float, n_vis: int,
            freq_hz: float = 150e6, dec_deg: float = 45.0, station_seed: int = 1,
            sky_seed: int = 2, noise_seed: int = 3, noise_sigma: float = 0.1,
            backend: str = "numpy", device: str = "cuda", uv_scale: float | None = None,
            w_range: tuple[float, float] | None = None) -> Observation:
    """One channel, one polarisation, time-major measurements in reference layout.

    ``uv_scale`` (= U, wavelengths) and ``w_range`` override the normalisation,
    so several channels can share one grid.
    """
    bl = baselines_xyz(stations(n_stations, diameter_m, station_seed))
    n_bl = bl.shape[0]
    n_dumps = -(-n_vis // n_bl)
    u, v, w = uvw_tracks(bl, n_dumps, hours, dec_deg, freq_hz)
    u = u.reshape(-1)[:n_vis]
    v = v.reshape(-1)[:n_vis]
    w = w.reshape(-1)[:n_vis]
    sky = sky_model(sky_seed)
    if backend == "torch":
        vis = point_source_vis_torch(u, v, w, sky, device=device)
    else:
        vis = point_source_vis(u, v, w, sky)
    rng = np.random.default_rng(noise_seed)
    vis = vis + noise_sigma * (rng.standard_normal(n_vis) + 1j * rng.standard_normal(n_vis))

    big_u = float(max(np.abs(u).max(), np.abs(v).max())) if uv_scale is None else float(uv_scale)
    wmin, wmax = (float(w.min()), float(w.max())) if w_range is None else w_range
    uu = _below_one(0.5 + u / (2.0 * big_u))
    vv = _below_one(0.5 + v / (2.0 * big_u))
    ww = _below_one((w - wmin) / (wmax - wmin))
    return Observation(
        uu=np.ascontiguousarray(uu), vv=np.ascontiguousarray(vv), ww=np.ascontiguousarray(ww),
        vis_real=vis.real.astype(np.float32), vis_img=vis.imag.astype(np.float32),
        weight=np.ones(n_vis, np.float32), freq_per_chan=1, polarizations=1,
        uvmin=float(min(u.min(), v.min())), uvmax=float(max(u.max(), v.max())),
        wmin=wmin, wmax=wmax,
        meta=dict(n_stations=n_stations, n_baselines=n_bl, n_dumps=n_dumps, hours=hours,
                  freq_hz=freq_hz, dec_deg=dec_deg, diameter_m=diameter_m, U=big_u,
                  seeds=(station_seed, sky_seed, noise_seed)))


def observe_device(*, n_stations: int, diameter_m: float, hours: float, n_vis: int,
                   freq_hz: float = 150e6, dec_deg: float = 45.0, station_seed: int = 1,
                   sky_seed: int = 2, noise_seed: int = 3, noise_sigma: float = 0.1,
                   device: str = "cuda", chunk_dumps: int = 2048) -> dict:
    """observe() for workloads too large for host memory: the same stations,
    tracks, sky and normalisation, generated dump-chunk by dump-chunk straight
    into device tensors (uu, vv, ww float64; vis_real, vis_img, weight float32).
    The noise comes from a seeded torch generator on the device, so its values
    differ from observe()'s.  Returns a dict with the tensors and the metadata
    (wmin, wmax, uvmin, uvmax, resolution)."""
    import torch
    bl = baselines_xyz(stations(n_stations, diameter_m, station_seed))
    n_bl = bl.shape[0]
    n_dumps = -(-n_vis // n_bl)
    hours_all = np.linspace(-hours / 2, hours / 2, n_dumps)

    def tracks(d0, d1):
        h = np.deg2rad(hours_all[d0:d1] * 15.0)[:, None]
        d = math.radians(dec_deg)
        lx, ly, lz = bl[None, :, 0], bl[None, :, 1], bl[None, :, 2]
        sh, ch = np.sin(h), np.cos(h)
        scale = freq_hz / C_LIGHT
        u = (sh * lx + ch * ly) * scale
        v = (-math.sin(d) * ch * lx + math.sin(d) * sh * ly + math.cos(d) * lz) * scale
        w = (math.cos(d) * ch * lx - math.cos(d) * sh * ly + math.sin(d) * lz) * scale
        rows = min((d1 - d0) * n_bl, n_vis - d0 * n_bl)
        return (u.reshape(-1)[:rows], v.reshape(-1)[:rows], w.reshape(-1)[:rows])

    big_u, wmin, wmax = 0.0, math.inf, -math.inf
    umin, umax = math.inf, -math.inf
    for d0 in range(0, n_dumps, chunk_dumps):
        u, v, w = tracks(d0, min(d0 + chunk_dumps, n_dumps))
        big_u = max(big_u, float(np.abs(u).max()), float(np.abs(v).max()))
        wmin, wmax = min(wmin, float(w.min())), max(wmax, float(w.max()))
        umin = min(umin, float(u.min()), float(v.min()))
        umax = max(umax, float(u.max()), float(v.max()))
    out = {k: torch.empty(n_vis, dtype=torch.float64, device=device) for k in ("uu", "vv", "ww")}
    for k in ("vis_real", "vis_img"):
        out[k] = torch.empty(n_vis, dtype=torch.float32, device=device)
    out["weight"] = torch.ones(n_vis, dtype=torch.float32, device=device)
    s, l, m, nn = (torch.as_tensor(x, dtype=torch.float64, device=device) for x in sky_model(sky_seed))
    gen = torch.Generator(device=device)
    gen.manual_seed(int(noise_seed))
    below = float(np.nextafter(1.0, 0.0))
    for d0 in range(0, n_dumps, chunk_dumps):
        u, v, w = (torch.as_tensor(x, device=device) for x in tracks(d0, min(d0 + chunk_dumps, n_dumps)))
        a, b = d0 * n_bl, d0 * n_bl + u.shape[0]
        ph = -2.0 * math.pi * (u[:, None] * l + v[:, None] * m + w[:, None] * (nn - 1.0))
        re = (s * torch.cos(ph)).sum(1) + noise_sigma * torch.randn(b - a, generator=gen, device=device, dtype=torch.float64)
        im = (s * torch.sin(ph)).sum(1) + noise_sigma * torch.randn(b - a, generator=gen, device=device, dtype=torch.float64)
        out["uu"][a:b] = torch.clamp_max(0.5 + u / (2.0 * big_u), below)
        out["vv"][a:b] = torch.clamp_max(0.5 + v / (2.0 * big_u), below)
        out["ww"][a:b] = torch.clamp_max((w - wmin) / (wmax - wmin), below)
        out["vis_real"][a:b] = re.float()
        out["vis_img"][a:b] = im.float()
    out.update(wmin=wmin, wmax=wmax, uvmin=umin, uvmax=umax,
               resolution=reference_resolution(umin, umax), n=n_vis, n_baselines=n_bl,
               n_dumps=n_dumps)
    return out


# Polarisation responses of the batch generator: XX, XY, YX, YY of a weakly
# polarised sky (Stokes Q = 0.05 I, U + iV leakage 0.05 at 0.3 rad);
# fewer polarisations take XX (and YY).
POL_GAINS = {1: (1.0,), 2: (1.0, 0.9),
             4: (1.0, 0.05 * np.exp(0.3j), 0.05 * np.exp(-0.3j), 0.9)}


@dataclass
class BatchObservation:
    """Per-channel inputs of a (channel, polarisation) batch.

    channels[c] = (uu, vv, ww, vis_real, vis_img, weight): uvw float64 [n_c]
    normalised on one grid shared by all channels (uvw in wavelengths scale
    with frequency), values and weights float32 [n_c][pols].
    """
    channels: list
    pols: int
    freqs: np.ndarray
    flag_fraction: np.ndarray
    uvmin: float
    uvmax: float
    wmin: float
    wmax: float

    @property
    def resolution(self) -> float:
        return reference_resolution(self.uvmin, self.uvmax)

    @property
    def n_vis(self) -> int:
        return sum(int(ch[0].shape[0]) for ch in self.channels) * self.pols


def observe_batch(*, n_channels: int = 16, f_lo: float = 120e6, f_hi: float = 180e6,
                  pols: int = 4, n_per_channel: int = 8_000_000, flag_max: float = 0.6,
                  n_stations: int = 62, diameter_m: float = 8000.0, hours: float = 8.0,
                  dec_deg: float = 45.0, station_seed: int = 1, sky_seed: int = 2,
                  noise_seed: int = 3, flag_seed: int = 4, noise_sigma: float = 0.1,
                  backend: str = "numpy", device: str = "cuda") -> BatchObservation:
    """Channels uniform in [f_lo, f_hi]; each starts from the same n_per_channel
    time-major measurements and drops a fraction U(0, flag_max) of them
    (per channel, each measurement independently, seeded).  Every polarisation
    of a channel carries the sky times its POL_GAINS entry plus its own noise."""
    if pols not in POL_GAINS:
        raise ValueError(f"pols must be one of {sorted(POL_GAINS)}")
    bl = baselines_xyz(stations(n_stations, diameter_m, station_seed))
    n_dumps = -(-n_per_channel // bl.shape[0])
    um, vm, wm = (x.reshape(-1)[:n_per_channel] for x in
                  uvw_tracks(bl, n_dumps, hours, dec_deg, C_LIGHT))   # metres
    freqs = np.linspace(f_lo, f_hi, n_channels)
    s_lo, s_hi = f_lo / C_LIGHT, f_hi / C_LIGHT
    big_u = float(max(np.abs(um).max(), np.abs(vm).max())) * s_hi
    lo_w, hi_w = float(wm.min()), float(wm.max())
    wmin = lo_w * (s_hi if lo_w < 0 else s_lo)
    wmax = hi_w * (s_hi if hi_w > 0 else s_lo)
    frng = np.random.default_rng(flag_seed)
    frac = frng.uniform(0.0, flag_max, n_channels)
    sky = sky_model(sky_seed)
    gains = np.asarray(POL_GAINS[pols], np.complex128)
    chans = []
    for c in range(n_channels):
        keep = frng.random(n_per_channel) >= frac[c]
        sc = freqs[c] / C_LIGHT
        u, v, w = um[keep] * sc, vm[keep] * sc, wm[keep] * sc
        if backend == "torch":
            base = point_source_vis_torch(u, v, w, sky, device=device)
        else:
            base = point_source_vis(u, v, w, sky)
        n = u.shape[0]
        nrng = np.random.default_rng((noise_seed, c))
        vis = base[:, None] * gains[None, :] + noise_sigma * (
            nrng.standard_normal((n, pols)) + 1j * nrng.standard_normal((n, pols)))
        chans.append((
            np.ascontiguousarray(_below_one(0.5 + u / (2.0 * big_u))),
            np.ascontiguousarray(_below_one(0.5 + v / (2.0 * big_u))),
            np.ascontiguousarray(_below_one((w - wmin) / (wmax - wmin))),
            np.ascontiguousarray(vis.real.astype(np.float32).reshape(-1)),
            np.ascontiguousarray(vis.imag.astype(np.float32).reshape(-1)),
            np.ones(n * pols, np.float32)))
    return BatchObservation(channels=chans, pols=pols, freqs=freqs, flag_fraction=frac,
                            uvmin=-big_u, uvmax=big_u, wmin=wmin, wmax=wmax)


# Workload definitions (grid, planes, support, visibility generator).
CONFIGS = {
    # plain FP64 w-stacking, runnable on the reference's OpenMP CPU path
    "c1": dict(nx=512, ny=512, planes=8, support=7,
               gen=dict(n_stations=48, diameter_m=3000.0, hours=4.0, n_vis=1_048_576)),
    # precision form: FP32-compensated beside FP64
    "c2": dict(nx=4096, ny=4096, planes=32, support=7,
               gen=dict(n_stations=62, diameter_m=8000.0, hours=8.0, n_vis=50_000_000)),
    # differentiation
    "c3": dict(nx=2048, ny=2048, planes=16, support=7,
               gen=dict(n_stations=62, diameter_m=8000.0, hours=8.0, n_vis=10_000_000)),
    # batching: 16 channels x 4 polarisations, one grid each
    "c4": dict(nx=2048, ny=2048, planes=16, support=7,
               gen=dict(n_channels=16, f_lo=120e6, f_hi=180e6, pols=4, n_per_channel=8_000_000,
                        flag_max=0.6, n_stations=62, diameter_m=8000.0, hours=8.0)),
    # large single image
    "c5": dict(nx=8192, ny=8192, planes=128, support=9,
               gen=dict(n_stations=62, diameter_m=8000.0, hours=12.0, n_vis=400_000_000)),
}


def scaled_config(name: str, n_vis: int | None = None, nx: int | None = None,
                  planes: int | None = None) -> dict:
    c = {k: (dict(v) if isinstance(v, dict) else v) for k, v in CONFIGS[name].items()}
    if n_vis is not None:
        c["gen"]["n_vis"] = n_vis
    if nx is not None:
        c["nx"] = c["ny"] = nx
    if planes is not None:
        c["planes"] = planes
    return c
