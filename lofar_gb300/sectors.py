"""v-slab sectoring through libwstack_gb300.so (include/wstack_gb300.h, section 4).

A rank of the reference grids its rows slab by slab (gridding.c:35-263):
``initialize_array`` lists each slab's rows (a row near a slab edge is listed
in the neighbouring slab too), and for each slab the rows are gathered in
reverse list order with v shifted to the slab and gridded onto a
``grid_size_y / nsectors``-row grid, which MPI then reduces to the slab's
owner.  Here the lists and the gather run on the GPU:

* ``sector_lists``      device offsets and concatenated lists
* ``sector_gather``     one slab's rows, ready for ``wstack`` on the slab grid
* ``initialize_array``  the host drop-in: histo_send and per-slab NumPy lists
* ``grid_by_slabs``     a run of the reference's multi-rank decomposition on one
                        GPU (every rank, every slab, the reduction summed into
                        the full grid)
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check


def w_supporth(w_support: int, dx: float) -> float:
    """init.c:18."""
    return float((w_support - 1) // 2) * dx


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def sector_lists(vv, nsectors: int, yaxis: int, dx: float, wsh: float):
    """Device float64 vv -> (offsets int64 [nsectors+2] on the device, the same
    on the host as NumPy, index int64 [total] on the device)."""
    import torch
    lib = _lib.load()
    vv = vv.contiguous()
    n = vv.numel()
    off = torch.empty(nsectors + 2, dtype=torch.int64, device=vv.device)
    check(lib.wsg_sector_count(vv.data_ptr(), n, nsectors, yaxis, dx, wsh, off.data_ptr(),
                               _stream()))
    total = int(off[-1].item())
    index = torch.empty(max(total, 1), dtype=torch.int64, device=vv.device)
    check(lib.wsg_sector_lists(vv.data_ptr(), n, nsectors, yaxis, dx, wsh, off.data_ptr(),
                               index.data_ptr(), index.numel(), _stream()))
    return off, off.cpu().numpy(), index[:total]


def sector_gather(index, offsets_host, isector: int, yaxis: int, dx: float, nf: int, npol: int,
                  uu, vv, ww, weights, vis_real, vis_img) -> dict:
    """Slab isector's rows (reverse list order, v shifted) as device tensors."""
    import torch
    lo, hi = int(offsets_host[isector]), int(offsets_host[isector + 1])
    nsec = hi - lo
    dev = uu.device
    out = {"uu": torch.empty(nsec, dtype=torch.float64, device=dev),
           "vv": torch.empty(nsec, dtype=torch.float64, device=dev),
           "ww": torch.empty(nsec, dtype=torch.float64, device=dev),
           "weights": torch.empty(nsec * npol, dtype=torch.float32, device=dev),
           "vis_real": torch.empty(nsec * nf * npol, dtype=torch.float32, device=dev),
           "vis_img": torch.empty(nsec * nf * npol, dtype=torch.float32, device=dev)}
    if nsec == 0:
        return out
    lst = index[lo:hi]
    check(_lib.load().wsg_sector_gather(
        lst.data_ptr(), nsec, isector, yaxis, dx, nf, npol, uu.data_ptr(), vv.data_ptr(),
        ww.data_ptr(), weights.data_ptr(), vis_real.data_ptr(), vis_img.data_ptr(),
        *[out[k].data_ptr() for k in ("uu", "vv", "ww", "weights", "vis_real", "vis_img")],
        _stream()))
    return out


def initialize_array(vv, nsectors: int, yaxis: int, dx: float, wsh: float):
    """Host drop-in (wsg_initialize_array) -> (histo_send, [list per slab]) as NumPy."""
    lib = _lib.load()
    v = np.ascontiguousarray(vv, dtype=np.float64)
    histo = np.zeros(nsectors + 1, dtype=np.int64)
    ptrs = (ctypes.c_void_p * (nsectors + 1))()
    check(lib.wsg_initialize_array(v.ctypes.data, v.size, nsectors, yaxis, dx, wsh,
                                   histo.ctypes.data, ptrs))
    libc = ctypes.CDLL(None)
    lists = []
    for s in range(nsectors + 1):
        n = int(histo[s])
        if n:
            buf = (ctypes.c_int64 * n).from_address(ptrs[s])
            lists.append(np.frombuffer(buf, dtype=np.int64).copy())
        else:
            lists.append(np.zeros(0, dtype=np.int64))
        libc.free(ctypes.c_void_p(ptrs[s]))
    return histo, lists


def grid_by_slabs(nranks: int, *, nx: int, ny: int, planes: int, w_support: int, nf: int,
                  npol: int, uu, vv, ww, weights, vis_real, vis_img):
    """The reference's decomposition for ``nranks`` ranks on one GPU: rank r
    takes its contiguous share of the rows (init.c:327-333), sectors them into
    nranks slabs of ny // nranks rows, and grids each slab's rows onto a slab
    grid with the drop-in wstack; the slab grids of all ranks are summed into
    their slab of a [planes][ny][nx][2] float64 grid (MPI_Reduce to the slab's
    owner, gridding.c:296-322).  Inputs are device tensors; returns the grid on
    the device."""
    import torch
    from .api import wstack
    n = uu.numel()
    yaxis = ny // nranks
    dx, dw = 1.0 / nx, 1.0 / planes
    wsh = w_supporth(w_support, dx)
    full = torch.zeros((planes, ny, nx, 2), dtype=torch.float64, device=uu.device)
    slab = torch.empty((planes, yaxis, nx, 2), dtype=torch.float64, device=uu.device)
    per, rem = divmod(n, nranks)
    for r in range(nranks):
        a = r * per
        b = a + per + (rem if r == nranks - 1 else 0)
        mine = {"uu": uu[a:b], "vv": vv[a:b], "ww": ww[a:b],
                "weights": weights[a * npol:b * npol],
                "vis_real": vis_real[a * nf * npol:b * nf * npol],
                "vis_img": vis_img[a * nf * npol:b * nf * npol]}
        _, off, index = sector_lists(mine["vv"], nranks, yaxis, dx, wsh)
        for s in range(nranks):
            rows = sector_gather(index, off, s, yaxis, dx, nf, npol, **mine)
            m = rows["uu"].numel()
            if m == 0:
                continue
            wstack(planes, m, nf, npol, rows["uu"], rows["vv"], rows["ww"], rows["vis_real"],
                   rows["vis_img"], rows["weights"], dx, dw, w_support, nx, yaxis, slab, 1)
            full[:, s * yaxis:(s + 1) * yaxis] += slab
    return full


__all__ = ["w_supporth", "sector_lists", "sector_gather", "initialize_array", "grid_by_slabs"]
