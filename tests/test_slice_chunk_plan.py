"""The slice kernels' TMEM chunk plan (sp::plan_chunks in
momms_gb300/csrc/slicegemm.cuh) against the MMA issuer's step-by-step rule,
on the CPU: tests/cpp/test_slice_chunks.cu is compiled by nvcc for the host
and run (no kernel is launched)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_slice_chunks.cu")


@pytest.mark.skipif(shutil.which(os.environ.get("NVCC", "nvcc")) is None, reason="nvcc not found")
def test_plan_chunks_matches_issuer(tmp_path):
    exe = str(tmp_path / "test_slice_chunks")
    cmd = [os.environ.get("NVCC", "nvcc"), "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
           "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "momms_gb300", "csrc"), "-I",
           os.path.join(ROOT, "include"), SRC, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "OK"
