"""The C++ host side of the pool (include/hashdag_gpu_pool.hpp, GpuNodePool over
the C ABI, and include/hashdag_host_mirror.hpp, the host mirror with the
reference's storage hooks): tests/gpu_pool_check.cpp is compiled with g++,
linked against libhashdag_gb300.so, or with -DHD_FAKE_DEVICE against an
in-memory pool that serves the entry points GpuNodePool calls (the incremental
publish and the dump format, on the CPU).

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


def build_fake(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "gpu_pool_check_fake")
    r = subprocess.run([gxx, "-std=c++20", "-O1", "-Wall", "-DHD_FAKE_DEVICE", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "gpu_pool_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def run_check(exe, mode, *args):
    r = subprocess.run([exe, mode, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok " + mode), r.stdout + r.stderr


def test_host_mirror_hooks(hd, tmp_path):
    run_check(build_check(hd, tmp_path), "mirror")


def test_create_without_a_device_returns_null(hd, tmp_path):
    if hd.lib().hd_device_available():
        pytest.skip("a CUDA device is present")
    run_check(build_check(hd, tmp_path), "nodevice")


def test_incremental_publish_on_an_appending_pool(tmp_path):
    """Publish reads everything on the first sync and after an epoch change
    (freed pages reported), otherwise exactly the appended words of each
    bucket, recorded as the pages' written ranges (the dirty ranges the
    application's Flush sends)."""
    run_check(build_fake(tmp_path), "fake_publish")


def test_pool_dump_save_load(tmp_path):
    run_check(build_fake(tmp_path), "dump", str(tmp_path))


def test_pool_dump_same_bytes_in_python_and_cpp(orc, tmp_path):
    """A dump written by vkhashdag_gb300.write_pool_dump from the oracle's pool
    (the reference's words) is read by HostPoolMirror::Load and written again
    by HostPoolMirror::Save byte for byte; read_pool_dump gives the words back."""
    import numpy as np
    from vkhashdag_gb300 import read_pool_dump, write_pool_dump, workloads as W
    cfg = W.config_for_resolution(256)
    pool = orc.OraclePool.from_config(cfg)
    root = pool.edit(orc.NULL, W.sphere_scene(256, 8, seed=3))
    bw, ids, pages = pool.dump()
    src, out = str(tmp_path / "a.hdmp"), str(tmp_path / "b.hdmp")
    write_pool_dump(src, cfg, bw, ids, pages)
    run_check(build_fake(tmp_path), "dump_copy", src, out)
    assert open(src, "rb").read() == open(out, "rb").read()
    c2, bw2, ids2, pages2 = read_pool_dump(out)
    assert c2 == cfg and np.array_equal(bw2, bw) and np.array_equal(ids2, ids) and np.array_equal(pages2, pages)
    again = orc.OraclePool.from_config(c2)
    again.load(bw2, ids2, pages2)
    assert again.canonical(root)[2] == pool.canonical(root)[2]
    with pytest.raises(ValueError):
        write_pool_dump(src, cfg, bw[:-1], ids, pages)
    open(src, "wb").write(open(out, "rb").read()[:-4])
    with pytest.raises(ValueError):
        read_pool_dump(src)


@pytest.mark.gpu
def test_incremental_publish_equals_device_words(hd, tmp_path):
    """On the device: after edits, Publish reads only appended pages and the
    mirror equals the device's words; after a GC it reads everything."""
    run_check(build_check(hd, tmp_path), "publish")


@pytest.mark.gpu
def test_node_pool_save_load(hd, tmp_path):
    """NodePool.save / load: a device pool written to a dump and loaded into
    another pool answers point queries the same way."""
    import numpy as np
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(256)
    a = hd.NodePool(cfg, heap_pages=cfg.get_total_pages())
    root = a.edit(hd.NULL, W.sphere_scene(256, 8, seed=4))
    path = str(tmp_path / "p.hdmp")
    a.save(path)
    b = hd.NodePool(cfg, heap_pages=cfg.get_total_pages())
    b.load(path)
    q = W.point_queries(256, 1 << 14, seed=2)
    assert np.array_equal(a.query(root, q), b.query(root, q))
    bw, ids, pages = a.download()
    bw2, ids2, pages2 = b.download()
    assert np.array_equal(bw, bw2) and np.array_equal(ids, ids2) and np.array_equal(pages, pages2)


@pytest.mark.gpu
def test_device_pool_download_upload_round_trip(hd, tmp_path):
    """Edits on the device, Download into the mirror, Upload of the mirror into
    a second pool (the same words, the same filled pointers), the same further
    edits on both, occupancy against the edits' predicates, GC through the
    class."""
    run_check(build_check(hd, tmp_path), "device")


@pytest.mark.gpu
def test_colour_pool_class(hd, tmp_path):
    """GpuColorPool over the colour entry points: one edit per call and all in
    one call give the same octree words and roots; digs keep the colour root."""
    run_check(build_check(hd, tmp_path), "color")
