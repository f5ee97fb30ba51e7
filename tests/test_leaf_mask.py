"""The edit kernels' leaf rule (classify, then shape_mask for partial leaves)
against a per-voxel brute force, on the CPU: tests/leaf_mask_check.cu compiles
the kernels' own __host__ __device__ functions into a host program (nvcc, no
GPU needed) and checks every combination of the box mask's per-axis masks plus
sampled boxes and spheres in both the 32-bit and the 64-bit paths."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_leaf_rule_equals_per_voxel_predicates(tmp_path):
    from vkhashdag_gb300 import _build
    try:
        nvcc = _build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "leaf_mask_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                        os.path.join(HERE, "leaf_mask_check.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    counts = dict(zip(r.stdout.split()[1::2], map(int, r.stdout.split()[2::2])))
    assert counts["partial"] > 100000 and counts["none"] > 10000 and counts["full"] > 10000, r.stdout
