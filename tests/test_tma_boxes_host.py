"""The sweep tiles' bulk-copy boxes, checked on the host for every tile of a set
of grid sizes (tests/native/tma_boxes_check.cu): 16-byte x origins, boxes inside
the grid, and every element a tile reads from its box inside the box."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_tma_boxes(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "tma_boxes_check")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-diag-suppress", "177", "-gencode",
                    "arch=compute_103a,code=sm_103a", "-o", exe, os.path.join(HERE, "native", "tma_boxes_check.cu")],
                   check=True, capture_output=True, timeout=600)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
