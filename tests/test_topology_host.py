"""The host hierarchy builders (csrc/bvh.cu: binned SAH over every
triangle, and the two-level build for instanced scenes) checked on the CPU:
a small harness compiled with nvcc runs them on 300 random scenes of
instanced meshes and validates every tree (tests/native/topology_check.cu).
No GPU is used."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "diffrender_tutorials_gb300", "csrc")


def test_host_topologies_are_valid_trees(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "topology_check")
    src = os.path.join(HERE, "native", "topology_check.cu")
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-I", CSRC, "-I", os.path.join(os.path.dirname(HERE), "include"),
                        "-gencode", "arch=compute_103a,code=sm_103a", src, "-o", exe],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-2000:]
    assert "0 failed" in out.stdout
