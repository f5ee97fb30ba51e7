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


def test_editor_objects_lower_to_descriptors(tmp_path):
    """LowerEditor / LowerColorEditor turn the application's editor objects
    (SphereEditor<kFill/kDig/kPaint>, AABBEditor, a box dig) into the
    descriptors the device applies; the concepts accept exactly those."""
    run_check(build_fake(tmp_path), "lowering")


@pytest.mark.parametrize("body", [
    "struct Weird { int q; }; auto d = hashdag_gb300::LowerEditor(Weird{1});",
    "struct Weird { int q; }; uint32_t r; auto p = hashdag_gb300::GpuNodePool::Create(hd_config{}); "
    "p->Edit(0u, Weird{1}, &r);",
    "enum class EditMode { kFill, kDig, kPaint }; struct V { unsigned x, y, z; }; "
    "template <EditMode M> struct SphereEditor { V center; unsigned long long r2; }; uint32_t r; "
    "auto p = hashdag_gb300::GpuNodePool::Create(hd_config{}); "
    "p->Edit(0u, SphereEditor<EditMode::kPaint>{{1, 2, 3}, 4}, &r);",
])
def test_other_editors_do_not_compile(tmp_path, body):
    """An editor the device cannot apply (no sphere or box members, or a paint
    as a geometry edit) is a compile error, not a CPU fallback."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    src = tmp_path / "bad.cpp"
    src.write_text('#include "hashdag_gpu_pool.hpp"\nint main() { ' + body + ' return 0; }\n')
    r = subprocess.run([gxx, "-std=c++20", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode != 0
    ok = tmp_path / "ok.cpp"
    ok.write_text('#include "hashdag_gpu_pool.hpp"\nint main() { return 0; }\n')
    r = subprocess.run([gxx, "-std=c++20", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(ok)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["full_then_dig", "scene64", "aabb_kat"])
def test_reference_editor_objects_on_device(hd, orc, golden, tmp_path, name):
    """The application's editor objects through the reference's call forms
    (ThreadedEdit(&busy_pool, root, editor, max_task_level) and
    Edit(root, editor), src/main.cpp:214-223) on the device: the DAG equals the
    reference's (canonical digests of the golden scenario) and one batched pass
    of the same edits ends on the same root."""
    import numpy as np
    from helpers import config_from, scenario, scenario_edits
    from vkhashdag_gb300 import read_pool_dump
    s = scenario(golden, name)
    cfg = config_from(s["config"])
    edits = np.ascontiguousarray(scenario_edits(s))
    path = tmp_path / "edits.bin"
    path.write_bytes(edits.tobytes())
    (tmp_path / "edits.bin.cfg").write_bytes(bytes(cfg.to_c()))
    exe = build_check(hd, tmp_path)
    dump = str(tmp_path / "pool.hdmp")
    r = subprocess.run([exe, "editors", str(path), dump], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok editors"), r.stdout + r.stderr
    root = int(next(ln for ln in r.stdout.splitlines() if ln.startswith("root "))[5:])
    c2, bw, ids, pages = read_pool_dump(dump)
    mirror = orc.OraclePool.from_config(c2)
    mirror.load(bw, ids, pages)
    ok, counts, digests = mirror.canonical(root)
    assert ok and counts == s["canonical_counts"] and [str(d) for d in digests] == s["canonical_digests"]
