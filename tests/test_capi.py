"""The C ABI library and the host-side logic, without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "hashdag_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(hd_[a-z_0-9]+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(hd):
    syms = declared_symbols()
    assert len(syms) >= 24
    lib = ctypes.CDLL(hd.library_path)
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_edit_desc_layout_matches_header(hd):
    assert hd.EDIT_DTYPE.itemsize == 40 and hd.HIT_DTYPE.itemsize == 40
    assert hd.EDIT_DTYPE.fields["r2"][1] == 32


def test_config_mirror(hd):
    """DefaultConfig / Config derived quantities (include/hashdag/Config.hpp)."""
    c = hd.DefaultConfig()()
    assert c.get_node_levels() == 16 and c.get_voxel_level() == 17 and c.get_resolution() == 1 << 17
    assert c.get_words_per_bucket() == 2048
    assert c.get_level_base_bucket_indices()[9] == 9 * 1024
    assert c.validate()
    big = hd.Config(9, 2, [21] * 3)
    assert not big.validate()
    lib = hd.lib()
    assert lib.hd_config_validate(ctypes.byref(c.to_c())) == 1
    assert lib.hd_config_validate(ctypes.byref(big.to_c())) == 0
    out = hd._Config()
    lib.hd_config_default(17, 9, 9, 2, 10, 16, ctypes.byref(out))
    assert out.node_levels == 16 and list(out.bucket_bits_each_level[:16]) == [10] * 9 + [16] * 7


def test_status_strings(hd):
    lib = hd.lib()
    assert lib.hd_status_string(2) == b"bucket full"


def test_pool_create_fails_loudly_without_device(hd):
    if hd.device_available():
        pytest.skip("device present")
    with pytest.raises(hd.HashDagError) as e:
        hd.NodePool(hd.DefaultConfig(level_count=6)(), heap_pages=64)
    assert e.value.status == 8  # HD_ERR_NO_DEVICE: no CPU fallback


def test_count_voxel_edits_matches_brute_force(hd):
    from vkhashdag_gb300 import workloads as W
    res = 64
    e = W.mixed_batch(res, 60, seed=5, r_max=20, side_max=30)
    e = np.concatenate([e, W.sphere_scene(res, 4, seed=1)])
    g = np.stack(np.meshgrid(np.arange(res), np.arange(res), np.arange(res), indexing="ij"), -1).reshape(-1, 3)
    want = 0
    for x in e:
        if x["shape"] == 0:
            d = g.astype(np.int64) - x["p0"].astype(np.int64)
            want += int(((d * d).sum(1) <= int(x["r2"])).sum())
        else:
            want += int(np.all((g >= x["p0"]) & (g < x["p1"]), 1).sum())
    assert hd.count_voxel_edits(e, res) == want


def test_workloads_deterministic_and_in_range():
    from vkhashdag_gb300 import workloads as W
    a = W.mixed_batch(32768, 1000, seed=1)
    b = W.mixed_batch(32768, 1000, seed=1)
    assert a.tobytes() == b.tobytes()
    sph = a[a["shape"] == 0]
    r = np.sqrt(sph["r2"].astype(np.float64))
    assert r.min() >= 1 and r.max() <= 512
    box = a[a["shape"] == 1]
    side = box["p1"].astype(np.int64) - box["p0"].astype(np.int64)
    assert side.min() >= 1 and side.max() <= 1024
    assert 0.6 < len(sph) / len(a) < 0.8
    assert 0.4 < (a["op"] == 1).mean() < 0.6
    t = W.terrain_columns(256, 8, seed=0)
    assert len(t) == 32 * 32 and t["p1"][:, 1].min() >= 1


def test_struct_layouts_match_the_header(hd, tmp_path):
    """sizeof/offsetof of every ABI struct, compiled from the header, equals the
    Python mirrors (ctypes structures and numpy dtypes)."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    structs = {
        "hd_config": hd._Config, "hd_pool_stats": hd._Stats, "hd_server_config": hd._ServerConfig,
        "hd_request_result": hd._RequestResult, "hd_server_stats": hd._ServerStats,
        "hd_color_config": hd._ColorConfig,
    }
    dtypes = {"hd_edit_desc": hd.EDIT_DTYPE, "hd_hit": hd.HIT_DTYPE, "hd_camera": hd.CAMERA_DTYPE,
              "hd_vbr_edit_desc": hd.VBR_EDIT_DTYPE, "hd_vbr_color": hd.COLOR_DTYPE}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "hashdag_gpu.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{name}.{field} %zu\\n", offsetof({name}, {field}));')
    for name, dt in dtypes.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for field in dt.names:
            lines.append(f'printf("{name}.{field} %zu\\n", offsetof({name}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                   text=True).stdout.splitlines())
    for name, cls in structs.items():
        assert int(got[name]) == ctypes.sizeof(cls), name
        for field, _ in cls._fields_:
            assert int(got[f"{name}.{field}"]) == getattr(cls, field).offset, (name, field)
    for name, dt in dtypes.items():
        assert int(got[name]) == dt.itemsize, name
        for field in dt.names:
            assert int(got[f"{name}.{field}"]) == dt.fields[field][1], (name, field)


def test_server_entry_points_reject_bad_arguments(hd):
    lib = hd.lib()
    out = ctypes.c_void_p()
    assert lib.hd_server_create(None, None, 0, None, ctypes.byref(out)) == 1 and not out.value
    rid = ctypes.c_uint64()
    assert lib.hd_server_submit_edits(None, 0, None, 0, ctypes.byref(rid)) == 1
    assert lib.hd_server_submit_camera(None, 0, None, 1, 1, 1, None, ctypes.byref(rid)) == 1
    r = hd._RequestResult()
    assert lib.hd_server_wait(None, 1, 0.0, ctypes.byref(r)) == 1
    assert lib.hd_server_drain(None) == 1 and lib.hd_server_pause(None, 1) == 1
    lib.hd_server_destroy(None)


def test_tuning_entry_points_reject_bad_arguments(hd):
    lib = hd.lib()
    t = hd._Tuning(8, 8, 8, 4, 16)
    assert lib.hd_edit_set_tuning(None, ctypes.byref(t)) == 1
    assert lib.hd_edit_get_tuning(None, ctypes.byref(t)) == 1
    assert lib.hd_edit_autotune(None, 0, None, 0, None, None, None) == 1


def test_colour_entry_points_reject_bad_arguments(hd):
    lib = hd.lib()
    out = ctypes.c_void_p()
    cfg = hd._ColorConfig(3, 0, 1 << 10, 1 << 10)
    assert lib.hd_color_pool_create(None, ctypes.byref(cfg), ctypes.byref(out)) == 1 and not out.value
    r, c = ctypes.c_uint32(), ctypes.c_uint32()
    assert lib.hd_vbr_edit(None, None, 0, 0, None, 0, ctypes.byref(r), ctypes.byref(c)) == 1
    n1, n2 = ctypes.c_uint64(), ctypes.c_uint64()
    assert lib.hd_color_pool_read(None, None, ctypes.byref(n1), None, ctypes.byref(n2)) == 1
    assert lib.hd_color_fetch(None, 0, None, 1, None, None) == 1
    lib.hd_color_pool_destroy(None)


def test_colour_editors_to_descriptors(hd):
    e = hd.vbr_edits_to_array([
        hd.SphereEditor((5, 6, 7), 16, hd.EditMode.kPaint, hd.VBRColor.rgb8(1, 2, 3)),
        hd.AABBEditor((0, 0, 0), (4, 4, 4), hd.EditMode.kFill, hd.VBRColor.weighted(0x1234, 0xABCD, 2, 2)),
        hd.SphereEditor((1, 1, 1), 4, hd.EditMode.kDig)])
    assert e["edit"]["op"].tolist() == [hd.OP_PAINT, hd.OP_FILL, hd.OP_DIG]
    assert e["colors"].tolist() == [0x030201, 0xABCD1234, 0] and e["bits_per_weight"].tolist() == [0, 2, 0]
    with pytest.raises(ValueError):
        hd.vbr_edits_to_array([hd.SphereEditor((1, 1, 1), 4, hd.EditMode.kFill)])


def test_headers_compile_standalone(tmp_path):
    """The C ABI header is plain C99; the C++ host headers compile on their own
    with every warning on (they depend on nothing but hashdag_gpu.h)."""
    import shutil
    import subprocess
    inc = os.path.join(ROOT, "include")
    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if not gcc or not gxx:
        pytest.skip("gcc / g++ not found")
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-x", "c",
                        os.path.join(inc, "hashdag_gpu.h")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for h in ("hashdag_host_mirror.hpp", "hashdag_gpu_pool.hpp"):
        src = tmp_path / (h + ".cpp")
        src.write_text(f'#include "{h}"\nint main() {{ return 0; }}\n')
        r = subprocess.run([gxx, "-std=c++20", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-I", inc,
                            str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_oracle_and_engine_count_the_same_voxel_edits(hd, orc):
    """The reference arm of the benchmark counts voxel-edits with the oracle,
    the engine's arm with hd_count_voxel_edits: equal on the benchmark's own
    batch (65,536 mixed edits on 32768^3) and on the terrain spheres."""
    from vkhashdag_gb300 import workloads as W
    e = W.mixed_batch(32768, 65536, seed=5)
    assert orc.count_voxel_edits(e, 32768) == hd.count_voxel_edits(e, 32768)
    s = W.surface_spheres(16384, 512, seed=0, band=64, block=32)
    assert orc.count_voxel_edits(s, 16384) == hd.count_voxel_edits(s, 16384)
