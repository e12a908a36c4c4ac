"""Host-side helpers of bench.py that need no GPU: the committed ncu summary's
machine-readable traffic line is found for the headline configuration, and the
peaks file is read."""
import argparse
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_step_traffic_line_is_found_for_the_headline_configuration():
    args = argparse.Namespace(precision="mixed", pre_iters=2, refine_iters=2, refactor_every=50)
    t = bench.step_traffic(4096, args)
    assert t is not None and 1e6 < t < 1e10
    args.pre_iters = 7
    assert bench.step_traffic(4096, args) is None


def test_peaks_are_read():
    hbm, bf16, bf16s, kind = bench.peaks()
    assert hbm > 1000 and bf16 > 100 and bf16s > 100 and kind in ("measured", "fallback")
