"""Plane-sharded imaging across ranks: one process per GPU, one image.

The reference spreads one image over MPI ranks by v-slabs of the grid and
reduces each slab's grid to its owner (``gridding.c:35-86``, ``gridding.c:
308-322``), then transforms with the slab-distributed FFTW-MPI
(``fourier_transform.c:25``).  Here the w-stack is cut along its plane axis
instead: rank r owns a contiguous range of w-planes [p0, p1) and the
measurements whose plane index ``(int)(ww/dw)`` (the reference's own step,
``w-stacking.cu:69``) falls in it.  Gridding, the per-plane FFTs and the
w-correction of those planes are all local to the rank; the w-corrected image
is a sum over planes (``phase_correction.cu:152-207``), so the ranks' partial
images add up to the whole image with one sum-reduction of Nx*Ny complex
values -- the only exchange, instead of the grid's P*Nx*Ny.

The adjoint goes the other way: every rank holds the same image (the
reduction above leaves it on every rank), applies the adjoint of its planes
and degrids its own measurements; each measurement belongs to exactly one
rank, so a sum-reduction of the per-measurement outputs (zero outside a
rank's measurements) assembles the full result.

Nothing here depends on the imager: ``forward`` and ``adjoint`` take the
per-rank imaging function, so the same partition and reductions run with the
library's GPU plans (NCCL) or any other imager (gloo on CPU).  Only loads of
each rank's own memory are involved; no peer memory is read.
"""
from __future__ import annotations

import numpy as np


def plane_index(ww, dw):
    """(int)(ww/dw) per measurement, as the reference computes it
    (w-stacking.cu:69): IEEE division, truncation toward zero."""
    if isinstance(ww, np.ndarray):
        return np.trunc(np.asarray(ww, np.float64) / dw).astype(np.int64)
    import torch
    return torch.trunc(ww.to(torch.float64) / dw).to(torch.int64)


def plane_ranges(counts, world: int, balance: bool = True):
    """Contiguous plane ranges [(p0, p1)] for `world` ranks.

    counts: measurements per plane (length P).  With `balance`, the cuts put
    about the same number of measurements on every rank (earth-rotation data
    crowd the middle planes); otherwise the planes are split evenly."""
    counts = np.asarray(counts, np.int64)
    planes = counts.size
    if world < 1 or world > planes:
        raise ValueError(f"{world} ranks for {planes} planes")
    if not balance or counts.sum() == 0:
        cuts = [(planes * r) // world for r in range(world + 1)]
    else:
        cum = np.concatenate([[0], np.cumsum(counts)])
        total = cum[-1]
        cuts = [0]
        for r in range(1, world):
            # the cut whose measurement count is nearest r/world of the total,
            # after the previous cut and leaving at least one plane per later rank
            t = total * r / world
            c = int(np.searchsorted(cum, t, side="left"))
            if c > 0 and (c > planes or t - cum[c - 1] <= cum[c] - t):
                c -= 1
            c = min(max(c, cuts[-1] + 1), planes - (world - r))
            cuts.append(c)
        cuts.append(planes)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


class PlaneShard:
    """This rank's share of a plane-sharded image.

    planes, dw: the w-stack (P planes of width dw, as passed to wstack()).
    counts: measurements per plane, the same on every rank (e.g. from
    ``plane_counts``), used to balance the ranges; None splits planes evenly.
    group: a torch.distributed process group (None = the default group, or a
    single process when torch.distributed is not initialised)."""

    def __init__(self, planes: int, dw: float, counts=None, rank=None, world=None, group=None):
        import torch.distributed as dist
        self.group = group
        if rank is None or world is None:
            if dist.is_available() and dist.is_initialized():
                rank, world = dist.get_rank(group), dist.get_world_size(group)
            else:
                rank, world = 0, 1
        self.rank, self.world = int(rank), int(world)
        self.planes, self.dw = int(planes), float(dw)
        c = np.ones(self.planes, np.int64) if counts is None else np.asarray(counts)
        self.ranges = plane_ranges(c, self.world, balance=counts is not None)
        self.p0, self.p1 = self.ranges[self.rank]

    def mask(self, ww):
        """Measurements this rank grids: plane index in [p0, p1)."""
        p = plane_index(ww, self.dw)
        return (p >= self.p0) & (p < self.p1)

    def select(self, uu, vv, ww, vis_real, vis_img, weight, freq_per_chan=1, polarizations=1):
        """This rank's measurements (the reference's layouts: values [m][f][p],
        weights [m][p]) and their indices in the full set."""
        m = self.mask(ww)
        n = uu.shape[0]
        nfp = freq_per_chan * polarizations
        if isinstance(uu, np.ndarray):
            idx = np.nonzero(m)[0]
        else:
            import torch
            idx = torch.nonzero(m).reshape(-1)
        return idx, (uu[idx], vv[idx], ww[idx],
                     vis_real.reshape(n, nfp)[idx].reshape(-1),
                     vis_img.reshape(n, nfp)[idx].reshape(-1),
                     weight.reshape(n, polarizations)[idx].reshape(-1))

    def _all_reduce(self, t):
        import torch.distributed as dist
        if self.world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
        return t

    def forward(self, imager, uu, vv, ww, vis_real, vis_img, weight, freq_per_chan=1,
                polarizations=1):
        """Sum over ranks of imager(<this rank's measurements>): the image of
        every measurement, on every rank.  imager returns a torch tensor (an
        image of this rank's planes); it is reduced in place."""
        _, sub = self.select(uu, vv, ww, vis_real, vis_img, weight, freq_per_chan, polarizations)
        return self._all_reduce(imager(*sub))

    def adjoint(self, adjoint_fn, image, ww, n_total):
        """Sum over ranks of the adjoint outputs of each rank's measurements,
        scattered to their places among all n_total measurements.
        adjoint_fn(image, idx) returns a torch tensor [len(idx), ...] for this
        rank's measurements."""
        import torch
        m = self.mask(ww)
        idx = np.nonzero(m)[0] if isinstance(m, np.ndarray) else torch.nonzero(m).reshape(-1)
        local = adjoint_fn(image, idx)
        out = torch.zeros((n_total,) + tuple(local.shape[1:]), dtype=local.dtype,
                          device=local.device)
        out[torch.as_tensor(idx, device=local.device)] = local
        return self._all_reduce(out)


def plane_counts(ww, dw, planes):
    """Measurements per plane (plane indices outside [0, P) are not counted:
    no rank grids them, as a single rank drops them)."""
    p = plane_index(ww, dw)
    if not isinstance(p, np.ndarray):
        p = p.cpu().numpy()
    p = p[(p >= 0) & (p < planes)]
    return np.bincount(p, minlength=planes)
