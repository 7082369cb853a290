"""Host-side helpers of bench.py (no GPU): the L1 data-pipe bound reported
beside the HBM roofline, and the L2 note of the workload description."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_l1_bound_arithmetic(monkeypatch):
    monkeypatch.setattr(bench, "sm_count", lambda dev: 152)
    w = bench.l1_wavefronts_for("tet_quality_tma_kernel")
    assert w and w > 0
    r = bench.l1_bound("tet_quality_tma_kernel", 70e-6, 0, {"sm_mhz": 2070.0})
    # one wavefront per SM per cycle: w / 152 cycles at 2070 MHz
    bound_s = w / 152 / 2070e6
    assert abs(r["bound_us"] - bound_s * 1e6) < 0.01
    assert abs(r["frac"] - bound_s / 70e-6) < 1e-4
    # without a clock sample the maximum SM clock is assumed
    assert bench.l1_bound("tet_quality_tma_kernel", 70e-6, 0, None)["sm_mhz"] == 2070.0


def test_l1_bound_needs_counts_and_device(monkeypatch):
    monkeypatch.setattr(bench, "sm_count", lambda dev: None)
    assert bench.l1_bound("tet_quality_tma_kernel", 70e-6, 0, None) is None
    monkeypatch.setattr(bench, "sm_count", lambda dev: 152)
    assert bench.l1_bound("no_such_kernel", 70e-6, 0, None) is None


def test_workload_l2_note():
    big = bench.workload_config(128, 2146689, 12582912, 385.0)["l2"]
    small = bench.workload_config(16, 4913, 24576, 1.0)["l2"]
    assert big.startswith("inputs larger than L2")
    assert small.startswith("inputs fit in L2")
