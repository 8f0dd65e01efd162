"""Python front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker or as the timed CPU
baseline.  The product library never routes through it.

It wraps two shared libraries built by ``oracle/build.py``:

* ``liboracle.so``: the C restatement (``wstack_oracle.c``), FP64;
* ``libref.so`` (optional): the reference's own CPU code compiled from the
  reference tree, used to pin the restatement.

The FFT stage of the reference (``fourier_transform.c:25-59``: FFTW_BACKWARD,
unnormalised, then scaled by 1/(Nx*Ny)) calls FFTW, which is not installed;
``numpy.fft.ifft2`` computes exactly that transform (exponent +i, 1/(Nx*Ny)),
so it stands in for FFTW here.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_float_p = ctypes.POINTER(ctypes.c_float)

_WSTACK_ARGS = [ctypes.c_int, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                _c_double_p, _c_double_p, _c_double_p, _c_float_p, _c_float_p, _c_float_p,
                ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                _c_double_p, ctypes.c_int]
_PHASE_ARGS = [_c_double_p, _c_double_p, _c_double_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
               ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
               ctypes.c_int]

_libs: dict[str, ctypes.CDLL] = {}


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_c_double_p)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_c_float_p)


def load_oracle() -> ctypes.CDLL:
    if "oracle" not in _libs:
        so = _build.build_oracle()
        lib = ctypes.CDLL(so)
        lib.oracle_wstack.argtypes = _WSTACK_ARGS
        lib.oracle_wstack.restype = None
        lib.oracle_phase_correction.argtypes = _PHASE_ARGS + [ctypes.c_int]
        lib.oracle_phase_correction.restype = None
        lib.oracle_degrid.argtypes = [ctypes.c_int, ctypes.c_long, _c_double_p, _c_double_p,
                                      _c_double_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, _c_double_p, _c_double_p,
                                      ctypes.c_int]
        lib.oracle_degrid.restype = None
        lib.oracle_phase_adjoint.argtypes = [_c_double_p, _c_double_p, _c_double_p,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_int]
        lib.oracle_phase_adjoint.restype = None
        lib.oracle_resolution.argtypes = [ctypes.c_double, ctypes.c_double]
        lib.oracle_resolution.restype = ctypes.c_double
        _i, _l, _d, _p = ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_void_p
        lib.oracle_grid_plane.argtypes = [_i, _i, _l, _l, _l, _c_double_p, _c_double_p,
                                          _c_double_p, _c_float_p, _c_float_p, _c_float_p, _d,
                                          _d, _i, _i, _i, _c_double_p, _p, _i]
        lib.oracle_grid_plane.restype = None
        lib.oracle_degrid_plane.argtypes = [_i, _i, _l, _c_double_p, _c_double_p, _c_double_p,
                                            _d, _d, _i, _i, _i, _p, _p, _p, _i]
        lib.oracle_degrid_plane.restype = None
        lib.oracle_phase_window.argtypes = [_c_double_p, _c_double_p, _c_double_p, _i, _i, _i,
                                            _i, _i, _i, _i, _i, _d, _d, _d, _i, _i]
        lib.oracle_phase_window.restype = None
        _libs["oracle"] = lib
    return _libs["oracle"]


def load_ref() -> ctypes.CDLL | None:
    """The reference's own CPU build, or None where it cannot be built."""
    if "ref" not in _libs:
        so = _build.build_ref()
        if so is None or not os.path.exists(so):
            return None
        try:
            lib = ctypes.CDLL(so)
        except OSError:
            return None
        lib.wstack.argtypes = _WSTACK_ARGS
        lib.wstack.restype = None
        lib.phase_correction.argtypes = _PHASE_ARGS
        lib.phase_correction.restype = None
        _libs["ref"] = lib
    return _libs["ref"]


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def wstack(uu, vv, ww, vis_real, vis_img, weight, *, num_w_planes, freq_per_chan=1,
           polarizations=1, dx, dw, w_support, nx, ny, num_threads=0, lib="oracle", grid=None):
    """Grid measurements; returns grid [P][ny][nx][2] float64 (accumulated into `grid`)."""
    uu, vv, ww = _c(uu, np.float64), _c(vv, np.float64), _c(ww, np.float64)
    vr, vi, wt = _c(vis_real, np.float32), _c(vis_img, np.float32), _c(weight, np.float32)
    n = uu.shape[0]
    assert vr.size == n * freq_per_chan * polarizations and wt.size == n * polarizations
    if grid is None:
        grid = np.zeros((num_w_planes, ny, nx, 2), np.float64)
    if lib == "ref":
        L = load_ref()
        if L is None:
            raise RuntimeError("reference CPU build unavailable")
        fn = L.wstack
    else:
        fn = load_oracle().oracle_wstack
    fn(num_w_planes, n, freq_per_chan, polarizations, _dp(uu), _dp(vv), _dp(ww), _fp(vr),
       _fp(vi), _fp(wt), dx, dw, w_support, nx, ny, _dp(grid), num_threads)
    return grid


def phase_correction(gridss, *, nx, ny, num_w_planes, resolution, wmin, wmax,
                     num_threads=0, lib="oracle", phase_on=True, xaxistot=None, yaxistot=None):
    """W-correct and sum planes; returns (image_real, image_imag) [ny][nx] float64."""
    g = _c(gridss, np.float64)
    re = np.zeros((ny, nx), np.float64)
    im = np.zeros((ny, nx), np.float64)
    xt = nx if xaxistot is None else xaxistot
    yt = ny if yaxistot is None else yaxistot
    if lib == "ref":
        L = load_ref()
        if L is None:
            raise RuntimeError("reference CPU build unavailable")
        L.phase_correction(_dp(g), _dp(re), _dp(im), nx, ny, num_w_planes, xt, yt,
                           resolution, wmin, wmax, num_threads)
    else:
        load_oracle().oracle_phase_correction(_dp(g), _dp(re), _dp(im), nx, ny, num_w_planes,
                                              xt, yt, resolution, wmin, wmax, num_threads,
                                              1 if phase_on else 0)
    return re, im


def fft_planes(grid, workers=None):
    """FFTW_BACKWARD per plane scaled by 1/(nx*ny) (fourier_transform.c:25-59)."""
    z = grid[..., 0] + 1j * grid[..., 1]
    try:
        import scipy.fft as sfft
        out = sfft.ifft2(z, axes=(-2, -1), workers=workers)
    except ImportError:  # pragma: no cover
        out = np.fft.ifft2(z, axes=(-2, -1))
    return np.stack([out.real, out.imag], axis=-1)


def fft_planes_adjoint(planes, workers=None):
    """Adjoint of fft_planes: unnormalised forward DFT (exponent -i) times 1/(nx*ny)."""
    z = planes[..., 0] + 1j * planes[..., 1]
    n = z.shape[-1] * z.shape[-2]
    try:
        import scipy.fft as sfft
        out = sfft.fft2(z, axes=(-2, -1), workers=workers) / n
    except ImportError:  # pragma: no cover
        out = np.fft.fft2(z, axes=(-2, -1)) / n
    return np.stack([out.real, out.imag], axis=-1)


def degrid(uu, vv, ww, grid, *, num_w_planes, dx, dw, w_support, nx, ny, num_threads=0):
    """Transpose of the gridding map: per-measurement complex [N][2] float64."""
    uu, vv, ww = _c(uu, np.float64), _c(vv, np.float64), _c(ww, np.float64)
    g = _c(grid, np.float64)
    out = np.zeros((uu.shape[0], 2), np.float64)
    load_oracle().oracle_degrid(num_w_planes, uu.shape[0], _dp(uu), _dp(vv), _dp(ww), dx, dw,
                                w_support, nx, ny, _dp(g), _dp(out), num_threads)
    return out


def phase_adjoint(image_real, image_imag, *, nx, ny, num_w_planes, resolution, wmin, wmax,
                  num_threads=0, phase_on=True):
    """Adjoint of phase_correction: planes [P][ny][nx][2] float64."""
    re, im = _c(image_real, np.float64), _c(image_imag, np.float64)
    planes = np.zeros((num_w_planes, ny, nx, 2), np.float64)
    load_oracle().oracle_phase_adjoint(_dp(re), _dp(im), _dp(planes), nx, ny, num_w_planes, nx,
                                       ny, resolution, wmin, wmax, num_threads,
                                       1 if phase_on else 0)
    return planes


def resolution(uvmin, uvmax):
    """The reference's resolution rule, gridding.c:160 (int abs of truncated values)."""
    return load_oracle().oracle_resolution(uvmin, uvmax)


def fold_measurements(vis_real, vis_img, weight, freq_per_chan, polarizations):
    """V_m = sum_{f,p} (double)(float)(weight*vis), NaN-flagged entries skipped
    (the fold inside w-stacking.cu:279-298, taken out of the tap loop)."""
    n = weight.size // polarizations
    vr = np.asarray(vis_real, np.float32).reshape(n, freq_per_chan, polarizations)
    vi = np.asarray(vis_img, np.float32).reshape(n, freq_per_chan, polarizations)
    wt = np.asarray(weight, np.float32).reshape(n, 1, polarizations)
    ok = ~np.isnan(vr)
    pr = np.where(ok, (wt * vr).astype(np.float32), 0).astype(np.float64).sum(axis=(1, 2))
    pi = np.where(ok, (wt * vi).astype(np.float32), 0).astype(np.float64).sum(axis=(1, 2))
    return pr, pi


def image_forward(uu, vv, ww, vis_real, vis_img, weight, *, num_w_planes, freq_per_chan=1,
                  polarizations=1, dx, dw, w_support, nx, ny, resolution, wmin, wmax,
                  num_threads=0, lib="oracle"):
    """grid -> per-plane FFT -> w-correction: the reference's hot path end to end."""
    g = wstack(uu, vv, ww, vis_real, vis_img, weight, num_w_planes=num_w_planes,
               freq_per_chan=freq_per_chan, polarizations=polarizations, dx=dx, dw=dw,
               w_support=w_support, nx=nx, ny=ny, num_threads=num_threads, lib=lib)
    gs = fft_planes(g)
    return phase_correction(gs, nx=nx, ny=ny, num_w_planes=num_w_planes, resolution=resolution,
                            wmin=wmin, wmax=wmax, num_threads=num_threads, lib=lib)


def image_adjoint(image_real, image_imag, uu, vv, ww, *, num_w_planes, dx, dw, w_support, nx,
                  ny, resolution, wmin, wmax, num_threads=0):
    """Adjoint of image_forward with respect to the folded measurement values."""
    planes = phase_adjoint(image_real, image_imag, nx=nx, ny=ny, num_w_planes=num_w_planes,
                           resolution=resolution, wmin=wmin, wmax=wmax, num_threads=num_threads)
    g = fft_planes_adjoint(planes)
    return degrid(uu, vv, ww, g, num_w_planes=num_w_planes, dx=dx, dw=dw, w_support=w_support,
                  nx=nx, ny=ny, num_threads=num_threads)



def grid_plane(w, uu, vv, ww, vis_real, vis_img, weight, *, num_w_planes, freq_per_chan=1,
               polarizations=1, dx, dw, w_support, nx, ny, num_threads=0, out=None):
    """Plane w of wstack(...) alone: [ny][nx][2] float64 (the reference's
    gridding arithmetic, w-stacking.cu:243-306, restricted to the measurements
    whose plane index is w), without the whole FP64 cube in memory."""
    uu, vv, ww = _c(uu, np.float64), _c(vv, np.float64), _c(ww, np.float64)
    vr, vi, wt = _c(vis_real, np.float32), _c(vis_img, np.float32), _c(weight, np.float32)
    if out is None:
        out = np.zeros((ny, nx, 2), np.float64)
    else:
        out[...] = 0.0
    rows = np.zeros(ny, np.uint8)
    load_oracle().oracle_grid_plane(w, num_w_planes, uu.shape[0], freq_per_chan, polarizations,
                                    _dp(uu), _dp(vv), _dp(ww), _fp(vr), _fp(vi), _fp(wt), dx, dw,
                                    w_support, nx, ny, _dp(out), rows.ctypes.data, num_threads)
    return out


def _ifft_rows(g, workers):
    try:
        import scipy.fft as sfft
        return sfft.ifft(g, axis=1, workers=workers)
    except ImportError:  # pragma: no cover
        return np.fft.ifft(g, axis=1)


def _fft_rows(g, workers):
    try:
        import scipy.fft as sfft
        return sfft.fft(g, axis=1, workers=workers)
    except ImportError:  # pragma: no cover
        return np.fft.fft(g, axis=1)


def image_window(uu, vv, ww, vis_real, vis_img, weight, *, num_w_planes, freq_per_chan=1,
                 polarizations=1, dx, dw, w_support, nx, ny, resolution, wmin, wmax, x0, y0,
                 wx, wy, num_threads=0):
    """Pixels [y0, y0+wy) x [x0, x0+wx) of image_forward(...), one plane at a time
    (no FP64 cube in memory): returns (image_real, image_imag) [wy][wx] float64.

    Per plane: oracle_grid_plane (the reference's gridding arithmetic), then the
    plane's inverse DFT on the window: an FFT along u of the rows that hold
    taps (the FFTW_BACKWARD stand-in, as in fft_planes), a direct DFT along v
    from those rows to the window's rows, the 1/(nx*ny) scale, and the
    w-correction of the window's pixels (oracle_phase_window)."""
    uu, vv, ww = _c(uu, np.float64), _c(vv, np.float64), _c(ww, np.float64)
    vr, vi, wt = _c(vis_real, np.float32), _c(vis_img, np.float32), _c(weight, np.float32)
    n = uu.shape[0]
    L = load_oracle()
    assert 0 <= x0 and x0 + wx <= nx and 0 <= y0 and y0 + wy <= ny
    workers = num_threads if num_threads > 0 else -1
    buf = np.zeros((ny, nx, 2), np.float64)
    bufc = buf.view(np.complex128).reshape(ny, nx)
    rows = np.zeros(ny, np.uint8)
    re = np.zeros((wy, wx), np.float64)
    im = np.zeros((wy, wx), np.float64)
    ys = np.arange(y0, y0 + wy)
    tw = np.exp(2j * np.pi * np.arange(ny) / ny)
    for w in range(num_w_planes):
        rows[:] = 0
        L.oracle_grid_plane(w, num_w_planes, n, freq_per_chan, polarizations, _dp(uu), _dp(vv),
                            _dp(ww), _fp(vr), _fp(vi), _fp(wt), dx, dw, w_support, nx, ny,
                            _dp(buf), rows.ctypes.data, num_threads)
        ks = np.nonzero(rows)[0]
        if ks.size == 0:
            continue
        g = bufc[ks]
        bufc[ks] = 0.0
        r = _ifft_rows(g, workers)[:, x0:x0 + wx]            # includes 1/nx
        ey = tw[np.outer(ys, ks) % ny]
        plane = (ey @ r) / ny
        pl = np.ascontiguousarray(np.stack([plane.real, plane.imag], -1))
        L.oracle_phase_window(_dp(pl), _dp(re), _dp(im), w, num_w_planes, x0, y0, wx, wy, nx,
                              ny, resolution, wmin, wmax, 0, num_threads)
    return re, im


def adjoint_window(image_real, image_imag, uu, vv, ww, *, x0, y0, num_w_planes, dx, dw,
                   w_support, nx, ny, resolution, wmin, wmax, num_threads=0):
    """image_adjoint(...) for an image that is zero outside the window whose
    [wy][wx] values are given at offset (x0, y0): per-measurement [N][2].

    Per plane: the w-correction adjoint on the window (oracle_phase_window),
    the forward DFT scaled by 1/(nx*ny) evaluated on the grid rows the plane's
    measurements read (a direct DFT along v, then an FFT along u), and
    oracle_degrid_plane."""
    re, im = _c(image_real, np.float64), _c(image_imag, np.float64)
    wy, wx = re.shape
    uu, vv, ww = _c(uu, np.float64), _c(vv, np.float64), _c(ww, np.float64)
    n = uu.shape[0]
    L = load_oracle()
    assert 0 <= x0 and x0 + wx <= nx and 0 <= y0 and y0 + wy <= ny
    workers = num_threads if num_threads > 0 else -1
    buf = np.zeros((ny, nx, 2), np.float64)
    bufc = buf.view(np.complex128).reshape(ny, nx)
    rows = np.zeros(ny, np.uint8)
    out = np.zeros((n, 2), np.float64)
    pl = np.zeros((wy, wx, 2), np.float64)
    ys = np.arange(y0, y0 + wy)
    tw = np.exp(-2j * np.pi * np.arange(ny) / ny)
    for w in range(num_w_planes):
        rows[:] = 0
        L.oracle_degrid_plane(w, num_w_planes, n, _dp(uu), _dp(vv), _dp(ww), dx, dw, w_support,
                              nx, ny, None, None, rows.ctypes.data, num_threads)
        ks = np.nonzero(rows)[0]
        if ks.size == 0:
            continue
        L.oracle_phase_window(_dp(pl), _dp(re), _dp(im), w, num_w_planes, x0, y0, wx, wy, nx,
                              ny, resolution, wmin, wmax, 1, num_threads)
        p = pl[..., 0] + 1j * pl[..., 1]
        ey = tw[np.outer(ks, ys) % ny]
        t = np.zeros((ks.size, nx), np.complex128)
        t[:, x0:x0 + wx] = ey @ p
        bufc[ks] = _fft_rows(t, workers) / (float(nx) * float(ny))
        L.oracle_degrid_plane(w, num_w_planes, n, _dp(uu), _dp(vv), _dp(ww), dx, dw, w_support,
                              nx, ny, buf.ctypes.data, out.ctypes.data, rows.ctypes.data,
                              num_threads)
        bufc[ks] = 0.0
    return out
