"""bench.py's host-side arithmetic (no GPU): the roofline traffic read from the
committed ncu launch-list summary, and the replica aggregation."""
import os

import pytest

import bench


def test_profiled_traffic_reads_the_committed_launch_list():
    assert os.path.exists(bench.PROFILE_MD)
    t = bench.profiled_traffic(bench.PROFILE_RECORDS)
    assert t is not None
    # the gridding stage's kernels move a few GB per step at the profiled size,
    # more than the algorithmic bytes (the sort re-reads the inputs)
    algo = bench.algorithmic_bytes(50_000_000, 4096, 4096, 32, 8)["grid"]
    assert algo < t < 3 * algo
    # scaled linearly by the records binned
    assert bench.profiled_traffic(2 * bench.PROFILE_RECORDS) == pytest.approx(2 * t)


def test_whole_job_rate_counts_every_rank():
    assert bench.whole_job_mvis(1_000_000, 4, 10.0) == pytest.approx(400.0)
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_l2_flush_only_for_workloads_that_fit_the_l2():
    # C1: 1M measurements, 512^2 x 8 complex64: the working set fits the L2 twice
    c1 = 1_048_576 * 36 + 8 * 512 * 512 * 8
    assert bench.l2_flush_bytes(c1) == 256 << 20
    assert "flushed" in bench.l2_note(bench.l2_flush_bytes(c1))
    # C2: 50M measurements, 4096^2 x 32: no flush needed
    c2 = 50_000_000 * 36 + 32 * 4096 * 4096 * 8
    assert bench.l2_flush_bytes(c2) == 0
    assert "no flush" in bench.l2_note(0)
