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
