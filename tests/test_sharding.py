"""Plane-sharded imaging (lofar_gb300.sharding) on CPU: the partition of the
measurements by w-plane and the two sum-reductions, with two gloo ranks as
torchrun launches them.  The per-rank imager is the FP64 oracle, so the
reduced results are compared with the single-rank oracle directly:

  * partition: each rank's measurements grid (oracle, one thread) to exactly
    the single-rank grid's planes [p0, p1) and to zeros elsewhere -- the
    plane assignment is the reference's (int)(ww/dw), bit for bit;
  * forward: the reduced image equals the single-rank image to 1e-12;
  * adjoint: the reduced per-measurement outputs equal the single-rank
    adjoint to 1e-12.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NX, PLANES, SUPPORT, N = 128, 8, 7, 20_000
RES = 1.0 / 1500.0


def _case():
    from lofar_gb300 import synth
    return synth.observe(n_stations=24, diameter_m=3000.0, hours=4.0, n_vis=N, sky_seed=5)


def _kw(o):
    return dict(num_w_planes=PLANES, dx=1 / NX, dw=1 / PLANES, w_support=SUPPORT, nx=NX, ny=NX,
                resolution=RES, wmin=o.wmin, wmax=o.wmax)


def test_plane_ranges_are_contiguous_and_cover_the_stack():
    from lofar_gb300.sharding import plane_ranges
    counts = np.array([5, 50, 400, 900, 1000, 380, 40, 3])
    for world in range(1, 9):
        for bal in (True, False):
            r = plane_ranges(counts, world, balance=bal)
            assert r[0][0] == 0 and r[-1][1] == PLANES
            assert all(a < b for a, b in r)
            assert all(r[i][1] == r[i + 1][0] for i in range(world - 1))
    # balanced cuts put about half the measurements on each of two ranks
    (a0, a1), (b0, b1) = plane_ranges(counts, 2)
    share = counts[a0:a1].sum() / counts.sum()
    assert 0.3 < share < 0.7
    with pytest.raises(ValueError):
        plane_ranges(counts, 9)


def test_partition_matches_the_reference_plane_step():
    from oracle import oracle as O
    from lofar_gb300.sharding import PlaneShard, plane_counts
    o = _case()
    kw = _kw(o)
    g = {k: kw[k] for k in ("num_w_planes", "dx", "dw", "w_support", "nx", "ny")}
    full = O.wstack(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, num_threads=1, **g)
    counts = plane_counts(o.ww, 1 / PLANES, PLANES)
    for world in (2, 3):
        seen = np.zeros(N, np.int64)
        for rank in range(world):
            sh = PlaneShard(PLANES, 1 / PLANES, counts, rank=rank, world=world)
            idx, sub = sh.select(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
            seen[idx] += 1
            part = O.wstack(*sub, num_threads=1, **g)
            assert np.array_equal(part[sh.p0:sh.p1], full[sh.p0:sh.p1])
            assert not part[:sh.p0].any() and not part[sh.p1:].any()
        assert np.array_equal(seen, np.ones(N, np.int64))   # disjoint and complete


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    from lofar_gb300.sharding import PlaneShard, plane_counts
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        o = _case()
        kw = _kw(o)
        sh = PlaneShard(PLANES, 1 / PLANES, plane_counts(o.ww, 1 / PLANES, PLANES))

        def imager(uu, vv, ww, vr, vi, wt):
            re, im = O.image_forward(uu, vv, ww, vr, vi, wt, num_threads=1, **kw)
            return torch.as_tensor(np.stack([re, im], -1))

        img = sh.forward(imager, o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight)
        y = np.random.default_rng(3).standard_normal((NX, NX, 2))

        def adjoint_fn(image, idx):
            a = O.image_adjoint(image[..., 0], image[..., 1], o.uu[idx], o.vv[idx], o.ww[idx],
                                num_threads=1, **kw)
            return torch.as_tensor(a)

        adj = sh.adjoint(adjoint_fn, y, o.ww, N)
        q.put((rank, (sh.p0, sh.p1), img.numpy(), adj.numpy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_single_rank_image_and_adjoint():
    import torch.multiprocessing as mp
    from oracle import oracle as O
    O.load_oracle()   # built once, before the ranks start
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    o = _case()
    kw = _kw(o)
    re, im = O.image_forward(o.uu, o.vv, o.ww, o.vis_real, o.vis_img, o.weight, **kw)
    ref = np.stack([re, im], -1)
    assert np.isfinite(ref).all()
    y = np.random.default_rng(3).standard_normal((NX, NX, 2))
    aref = O.image_adjoint(y[..., 0], y[..., 1], o.uu, o.vv, o.ww, **kw)
    (r0, rng0, img0, adj0), (r1, rng1, img1, adj1) = out
    assert rng0[1] == rng1[0] and rng0[0] == 0 and rng1[1] == PLANES
    for img, adj in ((img0, adj0), (img1, adj1)):
        assert np.abs(img - ref).max() <= 1e-12 * np.abs(ref).max()
        assert np.abs(adj - aref).max() <= 1e-12 * np.abs(aref).max()
