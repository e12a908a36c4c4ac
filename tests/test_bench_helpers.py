"""Host-side helpers of bench.py that need no GPU: the per-class roofline
arithmetic, the lookup of committed ncu traffic lines, and the peaks file."""
import math
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_class_roofline_counts_the_work_actually_run():
    n, steps = 4096, 10
    # 16 FP32 passes and 4 double-float passes per step, 16 transform jobs, 20 products
    prof = {"boundary_sums_fp32": (16 * steps * 0.02, 16 * steps), "boundary_sums_df": (4 * steps * 0.06, 4 * steps),
            "spectral_deriv": (8 * steps * 0.034, 8 * steps), "gemv": (20 * steps * 0.009, 20 * steps),
            "other": (0.0, 0)}
    pk = {"fp64_tflops": 1.2, "fp32_tflops": 60.0, "hbm_gbs": 6792.7}
    c = bench.class_roofline(prof, steps, n, {"boundary_sums_fp32": 16, "boundary_sums_df": 4}, 16, 20, pk)
    assert "other" not in c
    s32 = c["boundary_sums_fp32"]
    assert math.isclose(s32["work_per_step"], 16 * n * (n - 1) * 15.0)
    assert math.isclose(s32["achieved"], s32["work_per_step"] / (16 * 0.02e-3) / 1e12)
    assert math.isclose(s32["frac"], s32["achieved"] / 60.0) and s32["bound"] == "fp32"
    sp = c["spectral_deriv"]
    assert math.isclose(sp["work_per_step"], 16 * 10.0 * n * 12) and sp["bound"] == "fp64"
    assert c["gemv"]["bound"] == "hbm" and math.isclose(c["gemv"]["work_per_step"], 20 * 2.0 * n * n)


def test_fft4_work_counts_five_n_log_n_per_transform():
    # N2 = 64: per stage, z and phi: 2 forward column sets, 5 row sets, 3 inverse column sets of
    # 64 FFTs of 64 points; a': 1 forward column set, 2 row sets, 1 inverse column set
    n = 4096
    per_fft = 5.0 * 64 * 6
    assert math.isclose(bench.fft4_work_per_step("fft4_columns", n), 4 * 2 * 64 * per_fft)
    assert math.isclose(bench.fft4_work_per_step("fft4_rows", n), 4 * 5 * 64 * per_fft)
    assert math.isclose(bench.fft4_work_per_step("fft4_inverse_columns", n), 4 * 3 * 64 * per_fft)
    assert math.isclose(bench.fft4_work_per_step("ap_transform", n), 4 * 4 * 64 * per_fft)


def test_traffic_lookup_misses_cleanly():
    assert bench.kernel_traffic("no_such_kernel", 4096) is None


def test_peaks_are_read():
    hbm, bf16, bf16s, kind = bench.peaks()
    assert hbm > 1000 and bf16 > 100 and bf16s > 100 and kind in ("measured", "fallback")
