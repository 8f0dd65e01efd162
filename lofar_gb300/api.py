"""Python front end of libwstack_gb300.so.

Two layers, mirroring the C ABI:

* ``wstack``, ``phase_correction``, ``fft_planes``: the reference's entry
  points (w-stacking.h:12-51, fourier_transform.c:25-59) with the same argument
  names and meaning, over NumPy host arrays or CUDA tensors.  They raise
  ``WstackError`` where the reference would print and carry on.
* ``Plan``: the device-resident pipeline (bin -> grid -> FFT -> w-correct and
  its adjoint) over torch CUDA tensors; calls are ordered on torch's current
  stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import WSG_FP32C, WSG_FP64, WstackError, check

PRECISIONS = {"fp64": WSG_FP64, "fp32c": WSG_FP32C, WSG_FP64: WSG_FP64, WSG_FP32C: WSG_FP32C}


def _ptr(a):
    """Raw address of a NumPy array or torch tensor (contiguous)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported buffer type {type(a)!r}")


def _check_legacy():
    status, msg = _lib.last_error()
    if status != _lib.WSG_OK:
        raise WstackError(status, msg)


# ---------------------------------------------------------------------------
# reference entry points
# ---------------------------------------------------------------------------

def wstack(num_w_planes, num_points, freq_per_chan, polarizations, uu, vv, ww, vis_real,
           vis_img, weight, dx, dw, w_support, grid_size_x, grid_size_y, grid, num_threads=1):
    """The reference's wstack() (w-stacking.h:12-29): grid is overwritten."""
    lib = _lib.load()
    lib.wstack(int(num_w_planes), int(num_points), int(freq_per_chan), int(polarizations),
               _ptr(uu), _ptr(vv), _ptr(ww), _ptr(vis_real), _ptr(vis_img), _ptr(weight),
               float(dx), float(dw), int(w_support), int(grid_size_x), int(grid_size_y),
               _ptr(grid), int(num_threads))
    _check_legacy()
    return grid


def phase_correction(gridss, image_real, image_imag, xaxis, yaxis, num_w_planes, xaxistot,
                     yaxistot, resolution, wmin, wmax, num_threads=1):
    """The reference's phase_correction() (w-stacking.h:39-51): images overwritten."""
    lib = _lib.load()
    lib.phase_correction(_ptr(gridss), _ptr(image_real), _ptr(image_imag), int(xaxis),
                         int(yaxis), int(num_w_planes), int(xaxistot), int(yaxistot),
                         float(resolution), float(wmin), float(wmax), int(num_threads))
    _check_legacy()
    return image_real, image_imag


def fft_planes(grid_in, grid_out, nx, ny, nplanes):
    """FFTW_BACKWARD per plane scaled by 1/(nx*ny) (fourier_transform.c:25-59)."""
    check(_lib.load().wstack_fft_planes(_ptr(grid_in), _ptr(grid_out), int(nx), int(ny),
                                        int(nplanes)))
    return grid_out


def set_precision(precision) -> int:
    """Precision of the drop-in wstack(): 'fp64' (default) or 'fp32c'."""
    old = _lib.load().wstack_gb300_set_precision(PRECISIONS[precision])
    if old < 0:
        raise ValueError(f"invalid precision {precision!r}")
    return old


def release() -> None:
    """Free the device state kept between drop-in calls."""
    _lib.load().wstack_gb300_release()


# ---------------------------------------------------------------------------
# device-resident plan
# ---------------------------------------------------------------------------

class Plan:
    """A [planes][ny][nx] w-stacking plan resident on the current CUDA device.

    precision: 'fp64' (complex128, the reference's arithmetic) or 'fp32c'
    (complex64 with compensated tile accumulation).
    """

    def __init__(self, nx: int, ny: int, planes: int, support: int, dx: float | None = None,
                 dw: float | None = None, precision="fp32c"):
        import torch
        self._torch = torch
        self.nx, self.ny, self.planes, self.support = int(nx), int(ny), int(planes), int(support)
        self.dx = 1.0 / nx if dx is None else float(dx)
        self.dw = 1.0 / planes if dw is None else float(dw)
        self.precision = PRECISIONS[precision]
        self.cdtype = torch.complex128 if self.precision == WSG_FP64 else torch.complex64
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.wsg_plan_create(ctypes.byref(h), self.nx, self.ny, self.planes,
                                       self.support, self.dx, self.dw, self.precision,
                                       self._stream()))
        self._h = h
        self.n_binned = None

    def _stream(self):
        return ctypes.c_void_p(self._torch.cuda.current_stream().cuda_stream)

    def _sync_stream(self):
        check(self.lib.wsg_plan_set_stream(self._h, self._stream()))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.wsg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration ------------------------------------------------------
    def set_tuning(self, tile: int = 0, ctas: int = 0, chunk: int = 0):
        check(self.lib.wsg_plan_set_tuning(self._h, int(tile), int(ctas), int(chunk)))

    def set_layout(self, rows_per_dump: int):
        """Measurements come as [dump][baseline] with rows_per_dump rows per
        dump (the reference's measurement sets): a speed hint for the binning
        of FP32C plans; 0 = unknown."""
        check(self.lib.wsg_plan_set_layout(self._h, int(rows_per_dump)))

    def reserve(self, max_points: int):
        self._sync_stream()
        check(self.lib.wsg_plan_reserve(self._h, int(max_points)))

    def set_wcorrection(self, resolution: float, wmin: float, wmax: float):
        check(self.lib.wsg_plan_set_wcorrection(self._h, float(resolution), float(wmin),
                                                float(wmax)))

    def stats(self) -> dict:
        self._sync_stream()
        s = _lib.Stats()
        check(self.lib.wsg_plan_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in _lib.Stats._fields_}

    def device_bytes(self) -> int:
        return int(self.lib.wsg_plan_device_bytes(self._h))

    # -- stages -------------------------------------------------------------
    def _inputs(self, uu, vv, ww, vis_real, vis_img, weight):
        t = self._torch
        dev = t.device("cuda", t.cuda.current_device())

        def prep(x, dt):
            x = t.as_tensor(x, dtype=dt, device=dev)
            return x.contiguous()
        return (prep(uu, t.float64), prep(vv, t.float64), prep(ww, t.float64),
                prep(vis_real, t.float32), prep(vis_img, t.float32), prep(weight, t.float32))

    def bin(self, uu, vv, ww, vis_real, vis_img, weight, freq_per_chan=1, polarizations=1):
        ins = self._inputs(uu, vv, ww, vis_real, vis_img, weight)
        n = ins[0].numel()
        self._sync_stream()
        check(self.lib.wsg_bin(self._h, n, int(freq_per_chan), int(polarizations),
                               *[x.data_ptr() for x in ins]))
        self._keep = ins
        self.n_binned = n
        return self

    def new_grid(self):
        return self._torch.empty((self.planes, self.ny, self.nx), dtype=self.cdtype, device="cuda")

    def grid(self, out=None, occupied_only: bool = False):
        """Grid the binned measurements.  occupied_only: write only the tiles
        that hold measurements (the input fft_wcorrect reads with pruning)."""
        out = self.new_grid() if out is None else out
        assert out.dtype == self.cdtype and out.is_contiguous() and out.numel() == self.planes * self.ny * self.nx
        self._sync_stream()
        fn = self.lib.wsg_grid_occupied if occupied_only else self.lib.wsg_grid
        check(fn(self._h, out.data_ptr()))
        return out

    def fft(self, grid, sign: int = +1):
        self._sync_stream()
        check(self.lib.wsg_fft(self._h, grid.data_ptr(), int(sign)))
        return grid

    def wcorrect(self, planes, scale: float = 1.0, out=None):
        out = self._torch.empty((self.ny, self.nx), dtype=self.cdtype, device="cuda") if out is None else out
        self._sync_stream()
        check(self.lib.wsg_wcorrect(self._h, planes.data_ptr(), out.data_ptr(), float(scale)))
        return out

    def wcorrect_adjoint(self, image, scale: float = 1.0, out=None):
        out = self.new_grid() if out is None else out
        image = image.to(self.cdtype).contiguous()
        self._sync_stream()
        check(self.lib.wsg_wcorrect_adjoint(self._h, image.data_ptr(), out.data_ptr(),
                                            float(scale)))
        return out

    def fft_wcorrect(self, grid, out=None, prune=True):
        """Inverse per-plane FFT of `grid` (overwritten) + w-correction -> image."""
        out = self._torch.empty((self.ny, self.nx), dtype=self.cdtype, device="cuda") if out is None else out
        self._sync_stream()
        check(self.lib.wsg_fft_wcorrect(self._h, grid.data_ptr(), out.data_ptr(), int(bool(prune))))
        return out

    def wcorrect_adjoint_fft(self, image, out=None, prune=True):
        """Adjoint of fft_wcorrect -> grid (with prune, only the degridded cells)."""
        out = self.new_grid() if out is None else out
        image = image.to(self.cdtype).contiguous()
        self._sync_stream()
        check(self.lib.wsg_wcorrect_adjoint_fft(self._h, image.data_ptr(), out.data_ptr(),
                                                int(bool(prune))))
        return out

    def degrid(self, grid, out=None):
        if self.n_binned is None:
            raise WstackError(_lib.WSG_ERR_STATE, "degrid before bin")
        out = self._torch.empty(self.n_binned, dtype=self.cdtype, device="cuda") if out is None else out
        self._sync_stream()
        check(self.lib.wsg_degrid(self._h, grid.data_ptr(), out.data_ptr()))
        return out

    # -- composite ----------------------------------------------------------
    def image_forward(self, uu, vv, ww, vis_real, vis_img, weight, freq_per_chan=1,
                      polarizations=1, out=None):
        ins = self._inputs(uu, vv, ww, vis_real, vis_img, weight)
        n = ins[0].numel()
        out = self._torch.empty((self.ny, self.nx), dtype=self.cdtype, device="cuda") if out is None else out
        self._sync_stream()
        check(self.lib.wsg_image_forward(self._h, n, int(freq_per_chan), int(polarizations),
                                         *[x.data_ptr() for x in ins], out.data_ptr()))
        self._keep = ins
        self.n_binned = n
        return out

    def image_adjoint(self, image, out=None):
        if self.n_binned is None:
            raise WstackError(_lib.WSG_ERR_STATE, "adjoint before a forward call")
        image = image.to(self.cdtype).contiguous()
        out = self._torch.empty(self.n_binned, dtype=self.cdtype, device="cuda") if out is None else out
        self._sync_stream()
        check(self.lib.wsg_image_adjoint(self._h, image.data_ptr(), out.data_ptr()))
        return out

    def image_forward_host(self, uu, vv, ww, vis_real, vis_img, weight, image_out,
                           freq_per_chan=1, polarizations=1):
        """HOST buffers in and out (copies included); returns when done."""
        n = int(uu.shape[0])
        self._sync_stream()
        check(self.lib.wsg_image_forward_host(self._h, n, int(freq_per_chan), int(polarizations),
                                              _ptr(uu), _ptr(vv), _ptr(ww), _ptr(vis_real),
                                              _ptr(vis_img), _ptr(weight), _ptr(image_out)))
        self.n_binned = n
        return image_out

    def image_adjoint_host(self, image, out):
        self._sync_stream()
        check(self.lib.wsg_image_adjoint_host(self._h, _ptr(image), _ptr(out)))
        return out

    def image_forward_host_async(self, uu, vv, ww, vis_real, vis_img, weight, image_out,
                                 freq_per_chan=1, polarizations=1):
        """Asynchronous image_forward_host: returns at once; the host buffers
        must stay untouched until synchronize()."""
        n = int(uu.shape[0])
        self._sync_stream()
        check(self.lib.wsg_image_forward_host_async(
            self._h, n, int(freq_per_chan), int(polarizations), _ptr(uu), _ptr(vv), _ptr(ww),
            _ptr(vis_real), _ptr(vis_img), _ptr(weight), _ptr(image_out)))
        self.n_binned = n
        return image_out

    def image_adjoint_host_async(self, image, out):
        """Asynchronous image_adjoint_host (see image_forward_host_async)."""
        self._sync_stream()
        check(self.lib.wsg_image_adjoint_host_async(self._h, _ptr(image), _ptr(out)))
        return out

    def synchronize(self):
        """Wait for every call submitted to the plan."""
        check(self.lib.wsg_plan_synchronize(self._h))

    # -- tuning ---------------------------------------------------------------
    def autotune(self, uu, vv, ww, vis_real, vis_img, weight, iters: int = 3, freq_per_chan=1,
                 polarizations=1, image=None):
        """Time tile/split/CTA candidates on these inputs (forward imaging) and
        keep the fastest; returns (best, tried) as dicts."""
        ins = self._inputs(uu, vv, ww, vis_real, vis_img, weight)
        n = ins[0].numel()
        image = self._torch.empty((self.ny, self.nx), dtype=self.cdtype, device="cuda") if image is None else image
        best = _lib.Tuning()
        tried = (_lib.Tuning * 64)()
        nt = ctypes.c_int(0)
        self._sync_stream()
        check(self.lib.wsg_plan_autotune(self._h, n, int(freq_per_chan), int(polarizations),
                                         *[x.data_ptr() for x in ins], image.data_ptr(), int(iters),
                                         ctypes.byref(best), tried, 64, ctypes.byref(nt)))
        self._keep = ins
        self.n_binned = n
        return _tuning_dict(best), [_tuning_dict(tried[i]) for i in range(min(nt.value, 64))]


def _tuning_dict(t) -> dict:
    return {"tile": t.tile, "ctas": t.ctas, "chunk": t.chunk, "ms": t.ms}


class Batch:
    """Many (channel, polarisation) jobs imaged together (FP32C).

    Each job is what wstack() + FFT + phase_correction() give for one channel
    and one polarisation alone.  Channels share the grid geometry and the
    w-correction; each has its own uvw and measurement count.  Inputs per
    channel c: uu, vv, ww float64 [n_c]; vis_real, vis_img, weight float32
    [n_c][pols].  Outputs: images [channels][pols][ny][nx] complex64; the
    adjoint gives one complex64 per visibility, channel after channel.
    """

    def __init__(self, nx: int, ny: int, planes: int, support: int, channels: int, pols: int,
                 dx: float | None = None, dw: float | None = None):
        import torch
        self._torch = torch
        self.nx, self.ny, self.planes, self.support = int(nx), int(ny), int(planes), int(support)
        self.channels, self.pols = int(channels), int(pols)
        self.dx = 1.0 / nx if dx is None else float(dx)
        self.dw = 1.0 / planes if dw is None else float(dw)
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.wsg_batch_create(ctypes.byref(h), self.nx, self.ny, self.planes,
                                        self.support, self.dx, self.dw, self.channels, self.pols,
                                        self._stream()))
        self._h = h
        self._bound = None

    def _stream(self):
        return ctypes.c_void_p(self._torch.cuda.current_stream().cuda_stream)

    def _sync_stream(self):
        check(self.lib.wsg_batch_set_stream(self._h, self._stream()))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.wsg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_wcorrection(self, resolution: float, wmin: float, wmax: float):
        check(self.lib.wsg_batch_set_wcorrection(self._h, float(resolution), float(wmin),
                                                 float(wmax)))

    def set_tuning(self, tile: int = 0, ctas: int = 0, chunk: int = 0):
        check(self.lib.wsg_batch_set_tuning(self._h, int(tile), int(ctas), int(chunk)))

    def bind(self, channels):
        """channels: sequence of (uu, vv, ww, vis_real, vis_img, weight) per channel."""
        if len(channels) != self.channels:
            raise ValueError(f"expected {self.channels} channels, got {len(channels)}")
        t = self._torch
        dev = t.device("cuda", t.cuda.current_device())
        keep = []
        table = (_lib.Channel * self.channels)()
        for c, (uu, vv, ww, vr, vi, wt) in enumerate(channels):
            ins = [t.as_tensor(x, dtype=dt, device=dev).contiguous()
                   for x, dt in ((uu, t.float64), (vv, t.float64), (ww, t.float64),
                                 (vr, t.float32), (vi, t.float32), (wt, t.float32))]
            n = ins[0].numel()
            for x in ins[3:]:
                if x.numel() != n * self.pols:
                    raise ValueError(f"channel {c}: vis/weight need {n}x{self.pols} entries")
            table[c] = _lib.Channel(n, *[x.data_ptr() for x in ins])
            keep.append(ins)
        self._sync_stream()
        check(self.lib.wsg_batch_bind(self._h, table))
        self._bound = keep
        return self

    def new_images(self):
        return self._torch.empty((self.channels, self.pols, self.ny, self.nx),
                                 dtype=self._torch.complex64, device="cuda")

    def forward(self, images=None, graph: bool = True):
        images = self.new_images() if images is None else images
        assert images.dtype == self._torch.complex64 and images.is_contiguous()
        assert images.numel() == self.channels * self.pols * self.ny * self.nx
        self._sync_stream()
        check(self.lib.wsg_batch_forward(self._h, images.data_ptr(), int(bool(graph))))
        return images

    def n_vis(self) -> int:
        return int(self.lib.wsg_batch_vis_offset(self._h, self.channels))

    def vis_offset(self, channel: int) -> int:
        return int(self.lib.wsg_batch_vis_offset(self._h, int(channel)))

    def adjoint(self, images, out=None):
        images = images.to(self._torch.complex64).contiguous()
        out = self._torch.empty(self.n_vis(), dtype=self._torch.complex64, device="cuda") if out is None else out
        self._sync_stream()
        check(self.lib.wsg_batch_adjoint(self._h, images.data_ptr(), out.data_ptr()))
        return out

    def grids(self):
        """View of the resident grids [channels][pols][P][ny][nx] (complex64)."""
        ptr = self.lib.wsg_batch_grids(self._h)
        return _wrap_device(ptr, (self.channels, self.pols, self.planes, self.ny, self.nx),
                            self._torch.complex64)

    def autotune(self, images=None, iters: int = 3):
        images = self.new_images() if images is None else images
        best = _lib.Tuning()
        tried = (_lib.Tuning * 64)()
        nt = ctypes.c_int(0)
        self._sync_stream()
        check(self.lib.wsg_batch_autotune(self._h, images.data_ptr(), int(iters),
                                          ctypes.byref(best), tried, 64, ctypes.byref(nt)))
        return _tuning_dict(best), [_tuning_dict(tried[i]) for i in range(min(nt.value, 64))]

    def stats(self) -> dict:
        self._sync_stream()
        s = _lib.Stats()
        check(self.lib.wsg_batch_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in _lib.Stats._fields_}

    def device_bytes(self) -> int:
        return int(self.lib.wsg_batch_device_bytes(self._h))


class _DevArray:
    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def _wrap_device(ptr, shape, dtype):
    """A torch tensor viewing library-owned device memory (valid while the owner lives)."""
    import torch
    if not ptr:
        raise WstackError(_lib.WSG_ERR_STATE, "no device buffer")
    typestr = {torch.complex64: "<f4", torch.complex128: "<f8"}[dtype]
    real = torch.as_tensor(_DevArray(ptr, tuple(shape) + (2,), typestr), device="cuda")
    return torch.view_as_complex(real)
