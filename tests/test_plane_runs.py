"""The operand passes' run layout (momms_gb300/csrc/planes.cuh: run_grid,
run_lanes_log2, run_place, run_col) covers every element of the planes once
and stays inside the padded rows, on the CPU: tests/cpp/test_plane_runs.cu is
compiled by nvcc for the host and run (no kernel is launched)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_plane_runs.cu")


@pytest.mark.skipif(shutil.which(os.environ.get("NVCC", "nvcc")) is None, reason="nvcc not found")
def test_run_layout_covers_planes_once(tmp_path):
    exe = str(tmp_path / "test_plane_runs")
    cmd = [os.environ.get("NVCC", "nvcc"), "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
           "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "momms_gb300", "csrc"), "-I",
           os.path.join(ROOT, "include"), SRC, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "OK"
