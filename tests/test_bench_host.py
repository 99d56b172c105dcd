"""bench.py's host logic on the CPU: the clock record it attaches to every
line (median SM clock under load, throttle reasons), the dB error statistics,
the roofline object and the algorithmic work counts it divides by."""
import math
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import bench  # noqa: E402


def _clock_rows(tmp_path, rows):
    p = tmp_path / "clocks.csv"
    p.write_text("\n".join(rows) + "\n")
    c = bench.ClockSampler()
    c.proc, c.path = object(), str(p)          # as if nvidia-smi had written the file
    return c.summary()


def test_clock_summary_median_under_load_and_reasons(tmp_path):
    idle = "0, 345, 2070, 120.5, 0x0, Not Active, Not Active, Not Active, Not Active"
    rows = [idle] + [f"0, {mhz}, 2070, 1100.0, 0x4, Not Active, Not Active, Not Active, Active"
                     for mhz in (1950, 1965, 1980)] + ["garbage line"]
    s = _clock_rows(tmp_path, rows)
    assert s["sm_mhz"] == 1965.0                 # the idle sample is not "under load"
    assert s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 4


def test_clock_summary_flags_thermal_slowdown(tmp_path):
    rows = ["0, 1500, 2070, 1300.0, 0x40, Not Active, Active, Not Active, Not Active"] * 3
    s = _clock_rows(tmp_path, rows)
    assert s["reasons"] == ["hw_thermal_slowdown"]


def test_clock_summary_without_nvidia_smi():
    c = bench.ClockSampler()
    assert c.summary()["reasons"] == ["nvidia-smi unavailable"]


def test_db_stats():
    F64 = np.array([[1.0, 0.5, 1e-4], [2.0, 1.0, 0.1]], dtype=complex)
    F32 = F64 * np.array([[1.0, 1.0 + 1e-4, 1.1], [1.0, 1.0, 1.0 - 1e-3]])
    s = bench.db_stats(F32, F64)
    worst = 20 * math.log10(1.1)
    assert s["depth_db_at_max_err"] == pytest.approx(-80.0)
    # the -80 dB sample is excluded from the within-60-dB maximum
    assert s["max_db_err_within_60db_of_peak"] == pytest.approx(abs(20 * math.log10(1.0 - 1e-3)))
    assert s["max_db_err_within_60db_of_peak"] < worst


class _Near:
    pairs = np.array([[0, 0, 0, 10], [0, 1, 10, 5]])
    tails = np.array([[0, 64], [64, 100]])


class _Prob:
    n, m_max, nrhs, N, n_xi = 10, 3, 4, 6, 128
    near = _Near()


def test_kernel_work_counts():
    p = _Prob()
    assert bench.kernel_work(p, "residual") == 8.0 * 10 * 10 * 4 * 4
    assert bench.kernel_work(p, "far_fill") == 4.0 * 24 * 24 * 65 * 5
    assert bench.kernel_work(p, "near_fill") == 4.0 * (10 * 112 + 5 * 148) * 5


def _res(name, work, secs):
    return {"kernel_s": {name: [secs, secs], "lu": [secs / 10]}, "kernel_work": {name: [work, work]},
            "steps": 2, "dev_s": 4 * secs, "prob": _Prob()}


def test_roofline_tensor_and_fill_objects():
    peaks = {"hbm_gbs": 6794.1, "bf16_tflops": 1900.4, "sm_max_mhz": 2070.0, "source": "measured"}
    r = bench.roofline(_res("residual", 2e12, 1.0), peaks, "cone_sphere_ka40")
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["achieved"] == 2.0 and r["frac"] == round(2.0 / 1900.4, 5)
    assert r["kernel"] == "residual" and r["launches_per_step"] == 1.0
    f = bench.roofline(_res("far_fill", 5e12, 0.5), peaks, "cone_sphere_ka40")
    assert f["achieved"] == 10.0
    assert f["fp32_pipe"]["nominal_peak_tflops"] == round(152 * 128 * 2 * 2070e6 / 1e12, 1)
    assert f["traffic"] == bench.TRAFFIC.get(("far_fill", "cone_sphere_ka40"))
    samples = (4.0 * _Prob.N) ** 2 * (_Prob.n_xi // 2 + 1)
    assert f["fp32_pipe"]["samples_per_s"] == float(f"{samples * 2 / 1.0:.4g}")
    assert bench.roofline(_res("near_fill", 1e12, 1.0), peaks, "x")["traffic"] is None


def test_load_peaks_prefers_the_measured_file():
    p = bench.load_peaks()
    if os.path.exists(os.path.join(REPO, "MEASURED_PEAKS.json")):
        assert p["source"] == "measured" and p["hbm_gbs"] and p["bf16_tflops"]
    else:
        assert p == {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}
