"""bench.py's host-side pieces (no GPU): the algorithmic bytes it divides by, the peak it
reads, the traffic it takes from the committed ncu summaries, and the workload it names."""

import json
import types

import numpy as np

import bench
from tests import cases


def test_algorithmic_bytes_of_the_headline_workload():
    """8 values per cell-step, 4 per strip cell-step, 4 per accumulator entry (fp32 at 2024²:
    132.65 MB per step, 32.4 B per cell-update)."""
    p = cases.config2("single", n_steps=10)
    nx, ny, L = p.grid.nx, p.grid.ny, p.grid.pml_layers
    dft = sum(s.flat_index.size * s.wavelengths.size for s in p.samplings)
    b = bench.algorithmic_bytes_per_step(p)
    assert b == 4 * (8 * nx * ny + 8 * L * (nx + ny)) + 16 * dft
    assert (nx, ny) == (2024, 2024)
    assert abs(b / 1e6 - 132.65) < 0.01 and abs(b / (nx * ny) - 32.4) < 0.05


def test_peak_is_the_measured_copy_bandwidth_or_the_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "PEAKS", tmp_path / "peaks.json")
    assert bench.hbm_peak() == (bench.FALLBACK_HBM_GBS, "fallback")
    (tmp_path / "peaks.json").write_text(json.dumps({"hbm_gbs": 6771.8}))
    assert bench.hbm_peak() == (6771.8, "measured")


def test_traffic_of_the_default_kernels_comes_from_committed_summaries():
    for tag in ("k_tb_step_interior_40x128", "k_tb_step_interior_48x128", "k_tb_step_interior_40x128_k8",
                "k_tb_seg_interior_40x128_k8"):
        traffic, source = bench.ncu_traffic(tag)
        assert traffic is not None and 70e6 < traffic < 100e6 and source.endswith(".md"), tag
        if tag != "k_tb_step_interior_48x128":  # an earlier form, kept for its traffic only
            limiter, _ = bench.profile_entry("limiter", tag)
            assert limiter, tag
    assert bench.ncu_traffic("no_such_kernel") == (None, None)
    # the 3D stencil kernels: DRAM bytes per cell (the algorithmic 36 and 48 plus a little)
    for tag, lo, hi in (("k3_update_h_f32", 36, 48), ("k3_update_e_f32", 48, 60)):
        text, source = bench.profile_entry("traffic_bytes_per_cell", tag)
        assert text and lo <= float(text.split()[0]) <= hi and source.endswith(".md"), tag


def test_workload_description_names_the_headline_configuration():
    p = bench.workload("single", 10)
    d = bench.config_dict(p, types.SimpleNamespace(precision="single"))
    assert d["grid"] == [2024, 2024] and d["time_steps_per_step"] == 10
    assert "2000^2" in d["workload"] and "16 wavelengths" in d["workload"] and "l2" in d
    assert np.dtype(p.real) == np.float32


def test_clock_summary_takes_the_median_and_the_active_reasons():
    """The samples nvidia-smi prints during the timed region (csv, noheader, nounits): the median
    SM clock, the maximum, and which throttle reasons were ever active; unreadable lines skipped."""
    c = bench.ClockSampler(0)
    c.lines = [
        "0, 2070, 2070, 812.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1965, 2070, 1390.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 820.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]",
        "",
    ]
    assert c.summary() == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    c.lines = ["0, 1200, 2070, 900.0, 0x0000000000000008, Active, Not Active, Active, Not Active"]
    assert c.summary()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    c.lines = []
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
