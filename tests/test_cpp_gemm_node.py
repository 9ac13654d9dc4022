"""The C++ node API in include/momms/gemm_node.hpp (the reference's GemmNode
composition layer: Matrix views, PartM/PartN/PartK, SpawnThreads) with the
GPU leaf GpuGemm.

* CPU: tests/cpp/test_gemm_node.cpp's own checks of view arithmetic, call
  sequences, beta handling per k slab and thread teams.
* GPU: composed algorithms (blocked in m, n and k, on a thread team, with
  the plain, Ozaki and split-TF32 leaves) whose results are checked here
  against the double-double oracle with the componentwise bound
  |C - C_exact| <= 2(k+2) u (|alpha||A||B| + |beta||C0|).
"""
import os
import subprocess

import numpy as np
import pytest

import momms_gb300 as mg
from tests import oracle_util as ou

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_gemm_node.cpp")
HDR = os.path.join(ROOT, "include", "momms", "gemm_node.hpp")


@pytest.fixture(scope="module")
def node_exe(tmp_path_factory):
    if not os.path.exists(mg.LIB_PATH):
        from momms_gb300 import build as b
        b.build()
    out = str(tmp_path_factory.mktemp("node") / "test_gemm_node")
    libdir = os.path.dirname(mg.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o",
           out, "-L", libdir, "-lmomms_gpu", "-Wl,-rpath," + libdir, "-pthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_header_is_self_contained(tmp_path):
    src = tmp_path / "only.cpp"
    src.write_text("#include <momms/gemm_node.hpp>\nint main() { return 0; }\n")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I",
                    os.path.join(ROOT, "include"), str(src)], check=True, capture_output=True, text=True)


def test_node_composition_cpu(node_exe):
    r = subprocess.run([node_exe, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "OK"


def _read_case(path):
    with open(path, "rb") as f:
        hdr = np.frombuffer(f.read(40), dtype=np.int64)
        alpha, beta = np.frombuffer(f.read(16), dtype=np.float64)
        dt = np.float64 if hdr[0] == 0 else np.float32
        m, n, k = (int(x) for x in hdr[2:5])

        def mat(h, w):
            a = np.frombuffer(f.read(h * w * np.dtype(dt).itemsize), dtype=dt)
            return np.asfortranarray(a.reshape(w, h).T)

        A, B, C0, C = mat(m, k), mat(k, n), mat(m, n), mat(m, n)
    return dt, int(hdr[1]), float(alpha), float(beta), A, B, C0, C


@pytest.mark.gpu
def test_node_composition_gpu(gpu, node_exe, tmp_path):
    r = subprocess.run([node_exe, "gpu", str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    names = sorted(p for p in os.listdir(tmp_path) if p.endswith(".bin"))
    assert names == ["f32_mn.bin", "f32_tf32_k.bin", "f64_nkm.bin", "f64_ozaki_k.bin", "f64_spawn_mn.bin"]
    for name in names:
        dt, prec, alpha, beta, A, B, C0, C = _read_case(os.path.join(tmp_path, name))
        k = A.shape[1]
        u = 2.0**-53 if dt == np.float64 else 2.0**-24
        ref, mag = ou.dd_gemm(A.astype(np.float64), B.astype(np.float64), C0.astype(np.float64), alpha=alpha,
                              beta=beta)
        ratio = ou.bound_ratio(C.astype(np.float64), ref, mag, k, u)
        assert ratio <= 1.0, (name, ratio)
        # every entry was written (C0 differs from the result everywhere it can)
        assert np.all(np.isfinite(C)), name
