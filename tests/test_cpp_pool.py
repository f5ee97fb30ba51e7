"""The C++ host side of the pool (include/hashdag_gpu_pool.hpp, GpuNodePool over
the C ABI, and include/hashdag_host_mirror.hpp, the host mirror with the
reference's storage hooks): tests/gpu_pool_check.cpp is compiled with g++ and
linked against libhashdag_gb300.so.

That the mirror satisfies the reference's NodePool / ThreadedNodePool /
GCNodePool concepts, and that the reference's own Edit, ThreadedEdit,
ThreadedGC and Traversal give the reference's golden pools on it, is checked
where the reference compiles: oracle/ref_driver.cpp runs them on the mirror
(static_asserts of the concepts; tests/test_oracle.py compares its output with
the golden fixtures)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_check(hd, tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "gpu_pool_check")
    libdir = os.path.dirname(hd.library_path)
    r = subprocess.run([gxx, "-std=c++20", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "gpu_pool_check.cpp"), "-L", libdir, "-lhashdag_gb300",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def run_check(exe, mode):
    r = subprocess.run([exe, mode], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok " + mode), r.stdout + r.stderr


def test_host_mirror_hooks(hd, tmp_path):
    run_check(build_check(hd, tmp_path), "mirror")


def test_create_without_a_device_returns_null(hd, tmp_path):
    if hd.lib().hd_device_available():
        pytest.skip("a CUDA device is present")
    run_check(build_check(hd, tmp_path), "nodevice")


@pytest.mark.gpu
def test_device_pool_download_upload_round_trip(hd, tmp_path):
    """Edits on the device, Download into the mirror, Upload of the mirror into
    a second pool (the same words, the same filled pointers), the same further
    edits on both, occupancy against the edits' predicates, GC through the
    class."""
    run_check(build_check(hd, tmp_path), "device")
