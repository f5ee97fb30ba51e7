"""The edit kernels' per-node rules on the CPU: tests/edit_rule_check.cu compiles
the kernels' own __host__ __device__ functions into a host program (nvcc, no GPU
needed) and checks the leaf rule (classify, then shape_mask for partial leaves)
against a per-voxel brute force, and the expand kernel's classify_children
against classify of each child, for sampled boxes and spheres in both the 32-bit
and the 64-bit paths and every combination of the box mask's per-axis masks."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_node_rules_equal_the_reference_predicates(tmp_path):
    from vkhashdag_gb300 import _build
    try:
        nvcc = _build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "edit_rule_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                        os.path.join(HERE, "edit_rule_check.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    counts = dict(zip(r.stdout.split()[1::2], map(int, r.stdout.split()[2::2])))
    assert counts["partial"] > 100000 and counts["none"] > 10000 and counts["full"] > 10000, r.stdout
    assert min(counts["child_none"], counts["child_partial"], counts["child_full"]) > 10000, r.stdout
