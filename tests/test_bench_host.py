"""bench.py's host-side helpers, without a GPU: the CPU legs' thread count,
the roofline denominator and the single-rank reductions."""
from __future__ import annotations

import argparse
import os

import bench


def test_host_threads():
    assert bench.host_threads(argparse.Namespace(ref_threads=3)) == 3
    n = bench.host_threads(argparse.Namespace(ref_threads=0))
    assert 1 <= n <= (os.cpu_count() or 1)


def test_measured_peak():
    peak, kind = bench.measured_peak()
    assert peak > 0 and kind in ("measured", "fallback")


def test_single_rank_reductions():
    import torch
    dev = torch.device("cpu")
    assert bench.dist_max(2.5, 1, dev) == 2.5
    assert bench.dist_sum(7.0, 1, dev) == 7.0
