"""bench.py's arithmetic that needs no GPU: the rooflines' formulas and constants."""

import types

import pytest

import bench


def test_alu_roofline_formulas(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "get_device_properties", lambda i: types.SimpleNamespace(multi_processor_count=152))
    r = bench.alu_roofline(2.0e9, 4.0e7, 2070.0)
    fp32, fp64, issue = r["fp32"], r["fp64"], r["issue_fp32"]
    assert fp32["peak_tflops"] == pytest.approx(152 * 128 * 2 * 2.07e9 / 1e12)
    assert fp64["peak_tflops"] == pytest.approx(152 * 2 * 2 * 2.07e9 / 1e12)
    assert fp32["achieved_tflops"] == pytest.approx(bench.FLOPS_FP32_PER_CELL_UPDATE * 2.0e9 / 1e12)
    assert fp64["frac"] == pytest.approx(bench.FLOPS_FP64_PER_CELL_UPDATE * 4.0e7 / (fp64["peak_tflops"] * 1e12))
    assert issue["peak_per_s"] == pytest.approx(152 * 4 * 2.07e9)
    assert issue["frac"] == pytest.approx(bench.WARP_INSTR_FP32_PER_CELL_UPDATE * 2.0e9 / issue["peak_per_s"])
    # a missing FP64 rate leaves the FP64 entry out
    assert "fp64" not in bench.alu_roofline(2.0e9, None, 2070.0)


def test_minimum_traffic_and_constants_are_consistent():
    # SSPRK3: 8 state passes of C = 4 FP32 variables per cell-update = 128 bytes; a step is six
    # sweep launches, so the roofline's algorithmic bytes per launch at 2048^2 are 89.5 MB
    assert 8 * 4 * 4 == 128
    assert 128 * 2048 * 2048 / 6 == pytest.approx(89.48e6, rel=1e-3)
    # the measured sweep traffic per launch sits near what a launch must touch: the cell averages
    # in and a divergence or stage result out, averaged over a step (201 MB at 2048^2)
    touched = 2048 * 2048 * 4 * 4 * (2 + 2 + (2 + 5) + (2 + 5)) / 6
    assert 0.9 * touched < bench.SWEEP_DRAM_BYTES < 1.2 * touched
    assert bench.FLOPS_FP64_PER_CELL_UPDATE > bench.FLOPS_FP32_PER_CELL_UPDATE > 0


def test_batched_cpu_worker_runs_the_workload_methods():
    # one oracle step of a small four-quadrant grid with each of the batched workload's methods
    for ppm in (False, True):
        assert bench.batched_cpu_worker((16, ppm, 7)) > 0
