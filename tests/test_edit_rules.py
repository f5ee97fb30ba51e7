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


def build_check(tmp_path):
    from vkhashdag_gb300 import _build
    try:
        nvcc = _build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "edit_rule_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                        os.path.join(HERE, "edit_rule_check.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_node_rules_equal_the_reference_predicates(tmp_path):
    exe = build_check(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    counts = dict(zip(r.stdout.split()[1::2], map(int, r.stdout.split()[2::2])))
    assert counts["partial"] > 100000 and counts["none"] > 10000 and counts["full"] > 10000, r.stdout
    assert min(counts["child_none"], counts["child_partial"], counts["child_full"]) > 10000, r.stdout


def test_node_hashes_equal_the_oracle(orc, tmp_path):
    """The dedup kernel's node hashes (MurmurHash3 body over an inner node's
    words finished with its length; the 64-bit finaliser of a leaf), compiled
    for the host, against the oracle's restatement of Hasher.hpp on random inner
    nodes of every length and random leaves."""
    import numpy as np
    exe = build_check(tmp_path)
    rng = np.random.default_rng(7)
    recs, want = [], []
    for _ in range(4000):
        mask = int(rng.integers(1, 256))
        words = [mask] + [int(x) for x in rng.integers(0, 2 ** 32, bin(mask).count("1"), dtype=np.uint64)]
        recs += [0, len(words)] + words
        w = np.array(words, np.uint32)
        want.append(orc.lib().orc_hash_inner(w.ctypes.data, len(w)))
    for _ in range(4000):
        w0, w1 = (int(x) for x in rng.integers(0, 2 ** 32, 2, dtype=np.uint64))
        recs += [1, 2, w0, w1]
        want.append(orc.lib().orc_hash_leaf(w0, w1))
    src, out = str(tmp_path / "nodes.bin"), str(tmp_path / "hashes.bin")
    np.array(recs, np.uint32).tofile(src)
    r = subprocess.run([exe, "hashes", src, out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(out, np.uint32)
    assert np.array_equal(got, np.array(want, np.uint32))
