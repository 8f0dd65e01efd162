"""bench.py's multi-rank path on CPU: two gloo ranks, as torchrun launches them.

The w-stacking path runs as replicas (one whole image per GPU, no exchange
step), so the only cross-rank logic is the timing: the job's time is the
slowest rank's, and the reported throughput counts every rank's visibilities.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    v = bench.whole_job_mvis(1_000_000, world, ms)

    class A:
        steps, warmup, gpus = 1, 0, world
    ref = bench.bench_reference(A, rank, world) if rank != 0 else "rank0"
    q.put((rank, ms, v, ref))
    dist.destroy_process_group()


def test_two_ranks_report_the_slowest_rank_and_all_visibilities():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert out[0][2] == pytest.approx(2_000_000 / 15e-3 / 1e6)
    assert out[0][2] == out[1][2]
    # the reference arm: rank 1 does no work and prints nothing
    assert out[1][3] is None


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.whole_job_mvis(50_000_000, 1, 20.0) == pytest.approx(2500.0)


def test_stage_roofline_arithmetic():
    """bench.py's per-stage GB/s: algorithmic bytes over the median time, as a
    fraction of the peak (complex64 and complex128 cubes)."""
    import bench
    per = {"bin": [1.0, 1.0, 9.0], "grid": [2.0], "fft_wcorrect": [4.0],
           "wcorrect_adj_fft": [4.0], "degrid": [2.0]}
    n, nx, planes = 1_000_000, 1024, 4
    for sc in (8, 16):
        st = bench.roofline(per, n, nx, planes, sc, 1000.0, "measured")
        ab = bench.algorithmic_bytes(n, nx, nx, planes, sc)
        g = st["gridding(bin+grid)"]
        assert g["ms"] == 3.0 and g["bytes"] == ab["grid"]
        assert g["gbs"] == pytest.approx(ab["grid"] / 3e-3 / 1e9)
        assert st["degrid"]["frac"] == pytest.approx(ab["degrid"] / 2e-3 / 1e9 / 1000.0)
    assert bench.algorithmic_bytes(n, nx, nx, planes, 16)["fft_wcorrect"] == \
        2 * bench.algorithmic_bytes(n, nx, nx, planes, 8)["fft_wcorrect"]


def test_fft_fp64_equivalent_rate():
    import bench
    r = bench.fft_fp64_equivalent(4096, 32, 25.0)
    flop = 5.0 * 4096 * 4096 * 24 * 32
    assert r["tflops"] == pytest.approx(flop / 25e-3 / 1e12)
    assert r["of_nominal_fp64"] == pytest.approx(r["tflops"] / 1.25)
