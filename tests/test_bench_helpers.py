"""bench.py's host helpers: the roofline denominators come from the measured-peaks
file when it exists (marked "measured") and from the stated fallback otherwise; the
per-launch DRAM bytes and DFMA counts are read from the committed profile summaries
by key. No GPU."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_peaks_measured_and_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench._peaks() == (6800.0, "fallback")
    assert bench._bf16_peak() == (1900.0, 1700.0, "fallback")
    assert bench._max_sm_mhz() == 2070.0
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps(
        {"hbm_gbs": 6765.7, "bf16_tflops": 1921.3, "bf16_tflops_sustained": 1712.4,
         "sm_max_mhz": 2032.0}))
    assert bench._peaks() == (6765.7, "measured")
    assert bench._bf16_peak() == (1921.3, 1712.4, "measured")
    assert bench._max_sm_mhz() == 2032.0


def test_profile_figures_by_key(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench._traffic_from_profiles("acoustic2d_f64") is None      # no profiles folder
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "a.md").write_text("text\ntraffic_bytes_per_launch[acoustic2d_f64]: 232526080\n"
                               "dfma_per_launch[acoustic2d_f64]: 34206000\n")
    (prof / "b.md").write_text("traffic_bytes_per_launch[acoustic2d_f64_tb2]: 1.5e8\n")
    assert bench._traffic_from_profiles("acoustic2d_f64") == 232526080.0
    assert bench._traffic_from_profiles("acoustic2d_f64", "dfma_per_launch") == 34206000.0
    assert bench._traffic_from_profiles("acoustic2d_f64_tb2") == 1.5e8   # no prefix match
    assert bench._traffic_from_profiles("acoustic2d_f32") is None


def test_committed_profiles_carry_the_default_line_figures():
    """The default line's roofline traffic and FP64 figure resolve from the committed
    summaries (so a bench run reports them without a capture of its own)."""
    assert bench._traffic_from_profiles("acoustic2d_f64") > 0
    assert bench._traffic_from_profiles("acoustic2d_f64", "dfma_per_launch") > 0
    for key in ("acoustic2d_dw_tb2", "acoustic2d_f32_tb2", "batched_f64_tb2",
                "batched_f32_tb2", "batched_dw_tb2"):
        assert bench._traffic_from_profiles(key) > 0, key
