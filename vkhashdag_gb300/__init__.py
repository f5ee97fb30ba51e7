"""vkhashdag_gb300 -- GB300 HashDAG edit engine (Python host mirror of the C ABI).

The names follow the reference's hashdag API (include/hashdag/): ``Config`` and
``DefaultConfig`` (Config.hpp:15-75), ``NodePointer`` values as plain ints with
``NULL`` = 0xFFFFFFFF (NodePointer.hpp:13-31), ``EditType``/editors
(Editor.hpp:18-55, src/main.cpp:32-150) and ``NodePool`` with ``edit``
(NodePool.hpp:405-417), ``upsert_inner_node``/``upsert_leaf``
(NodePool.hpp:228-238) and ``traversal`` (NodePoolTraversal.hpp:93-256).

Every call goes through ``libhashdag_gb300.so`` (CUDA, sm_103a).  There is no
CPU fallback: constructing a ``NodePool`` without the built library or without a
CUDA device raises.
"""
from __future__ import annotations

import ctypes
import enum
import os
import weakref
from dataclasses import dataclass, field
from typing import Iterable, List, Optional, Sequence

import numpy as np

__all__ = [
    "NULL", "Config", "DefaultConfig", "EditMode", "SphereEditor", "AABBEditor", "NodePool",
    "HashDagError", "EDIT_DTYPE", "HIT_DTYPE", "CAMERA_DTYPE", "edits_to_array", "lib", "library_path",
    "count_voxel_edits", "device_available", "Server", "REQ_EDIT", "REQ_CAMERA", "projection_factor",
    "write_pool_dump", "read_pool_dump",
]

NULL = 0xFFFFFFFF
MAX_LEVELS = 24
_HERE = os.path.dirname(os.path.abspath(__file__))
library_path = os.path.join(_HERE, "libhashdag_gb300.so")

# hd_edit_desc (include/hashdag_gpu.h): 40 bytes
EDIT_DTYPE = np.dtype([("shape", "<u4"), ("op", "<u4"), ("p0", "<u4", (3,)), ("p1", "<u4", (3,)), ("r2", "<u8")],
                      align=True)
assert EDIT_DTYPE.itemsize == 40
HIT_DTYPE = np.dtype([("voxel", "<u4", (3,)), ("size", "<u4"), ("level", "<u4"), ("hit", "<u4"), ("t", "<f4"),
                      ("pos", "<f4", (3,))])
assert HIT_DTYPE.itemsize == 40
CAMERA_DTYPE = np.dtype([("position", "<f4", (3,)), ("look", "<f4", (3,)), ("side", "<f4", (3,)),
                         ("up", "<f4", (3,))])

SHAPE_SPHERE, SHAPE_AABB = 0, 1
OP_FILL, OP_DIG, OP_PAINT = 0, 1, 2
# hd_vbr_edit_desc: a colour edit (op FILL = coloured fill, PAINT = paint without
# geometry change, DIG = stateless dig that leaves the colours) and its colour
# (VBRColor: RGB8 in colors when bits_per_weight is 0, else two R5G6B5 end
# points, low half first, and a weight below 2^bits_per_weight)
VBR_EDIT_DTYPE = np.dtype([("edit", EDIT_DTYPE), ("colors", "<u4"), ("weight", "<u4"), ("bits_per_weight", "<u4"),
                           ("pad", "<u4")], align=True)
# hd_vbr_color: one voxel's colour (has_value, the VBRColor fields) and its RGB
# as trace.frag computes it
COLOR_DTYPE = np.dtype([("has_value", "<u4"), ("colors", "<u4"), ("weight", "<u4"), ("bits_per_weight", "<u4"),
                        ("rgb", "<f4", (3,))])

STATUS = {0: "ok", 1: "invalid argument", 2: "bucket full", 3: "device page heap exhausted", 4: "dedup index full",
          5: "edit workspace capacity exceeded", 6: "CUDA error", 7: "device wait timed out", 8: "no CUDA device",
          9: "device consistency check failed"}


class HashDagError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)} (status {status})")


class _Config(ctypes.Structure):
    _fields_ = [("word_bits_per_page", ctypes.c_uint32), ("page_bits_per_bucket", ctypes.c_uint32),
                ("node_levels", ctypes.c_uint32), ("hasher", ctypes.c_uint32),
                ("bucket_bits_each_level", ctypes.c_uint32 * MAX_LEVELS)]


class _Stats(ctypes.Structure):
    _fields_ = [("heap_pages", ctypes.c_uint64), ("used_pages", ctypes.c_uint64), ("total_buckets", ctypes.c_uint64),
                ("total_pages", ctypes.c_uint64), ("index_slots", ctypes.c_uint64), ("index_used", ctypes.c_uint64),
                ("max_bucket_words", ctypes.c_uint32), ("words_per_bucket", ctypes.c_uint32)]


class _Tuning(ctypes.Structure):
    _fields_ = [("expand_blocks_per_sm", ctypes.c_uint32), ("leaf_blocks_per_sm", ctypes.c_uint32),
                ("dedup_blocks_per_sm", ctypes.c_uint32), ("long_blocks_per_sm", ctypes.c_uint32),
                ("long_threshold", ctypes.c_uint32), ("leaf_compact", ctypes.c_uint32)]


class _GcStats(ctypes.Structure):
    _fields_ = [("live_nodes", ctypes.c_uint64), ("words_before", ctypes.c_uint64), ("words_after", ctypes.c_uint64),
                ("pages_before", ctypes.c_uint64), ("pages_after", ctypes.c_uint64)]


class _ServerConfig(ctypes.Structure):
    _fields_ = [("max_pass_edits", ctypes.c_uint32), ("ray_slots", ctypes.c_uint32),
                ("max_rays_per_request", ctypes.c_uint32), ("reserve_pages", ctypes.c_uint32),
                ("pages_per_edit_hint", ctypes.c_double), ("gc_free_fraction", ctypes.c_double)]


class _RequestResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("kind", ctypes.c_uint32), ("scene", ctypes.c_uint32),
                ("status", ctypes.c_int32), ("admitted", ctypes.c_uint32), ("root_in", ctypes.c_uint32),
                ("root", ctypes.c_uint32), ("pass_id", ctypes.c_uint64), ("pass_requests", ctypes.c_uint32),
                ("pass_edits", ctypes.c_uint32), ("rays", ctypes.c_uint64), ("hits", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("node_words", ctypes.c_uint64), ("t_submit_ms", ctypes.c_double),
                ("t_start_ms", ctypes.c_double), ("t_done_ms", ctypes.c_double), ("gc_epoch", ctypes.c_uint64)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("edit_requests", ctypes.c_uint64), ("camera_requests", ctypes.c_uint64),
                ("refused", ctypes.c_uint64), ("failed", ctypes.c_uint64), ("edit_passes", ctypes.c_uint64),
                ("edits_applied", ctypes.c_uint64), ("rays_traced", ctypes.c_uint64),
                ("max_pass_requests", ctypes.c_uint32), ("queued", ctypes.c_uint32),
                ("edit_p50_ms", ctypes.c_double), ("edit_p99_ms", ctypes.c_double),
                ("camera_p50_ms", ctypes.c_double), ("camera_p99_ms", ctypes.c_double),
                ("gc_runs", ctypes.c_uint64), ("gc_ms", ctypes.c_double)]


class _ColorConfig(ctypes.Structure):
    _fields_ = [("leaf_level", ctypes.c_uint32), ("keep_history", ctypes.c_uint32), ("max_nodes", ctypes.c_uint64),
                ("max_leaf_words", ctypes.c_uint64)]


_lib = None


def lib():
    """The loaded C ABI library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(library_path):
        raise RuntimeError(f"{library_path} is missing: build it with vkhashdag_gb300._build.build()")
    L = ctypes.CDLL(library_path)
    P, U32, U64, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    sig = {
        "hd_pool_create": (I, [ctypes.POINTER(_Config), U64, U32, I, ctypes.POINTER(P)]),
        "hd_pool_destroy": (None, [P]),
        "hd_config_validate": (I, [ctypes.POINTER(_Config)]),
        "hd_config_default": (None, [U32, U32, U32, U32, U32, U32, ctypes.POINTER(_Config)]),
        "hd_pool_filled_pointers": (I, [P, P]),
        "hd_pool_get_stats": (I, [P, ctypes.POINTER(_Stats)]),
        "hd_pool_get_error": (I, [P, P]),
        "hd_pool_clear_error": (I, [P]),
        "hd_edit": (I, [P, U32, P, U32, P, P]),
        "hd_edit_async": (I, [P, U32, P, U32, P, P]),
        "hd_edit_async_droot": (I, [P, P, P, U32, P, P]),
        "hd_edit_async_droot_hinted": (I, [P, P, P, P, U32, P, P]),
        "hd_edit_last_leaf_work": (I, [P, P]),
        "hd_edit_reserve": (I, [P, U64, U64, U32]),
        "hd_edit_last_counters": (I, [P, P, P, P, P, P]),
        "hd_edit_last_probe_stats": (I, [P, P, P, P]),
        "hd_pool_checkpoint": (I, [P]),
        "hd_pool_rollback": (I, [P, P]),
        "hd_upsert": (I, [P, U32, P, P, U32, P]),
        "hd_upsert_noalloc": (I, [P, U32, P, U32, P, P]),
        "hd_gc": (I, [P, P, U32, ctypes.POINTER(_GcStats)]),
        "hd_edit_get_tuning": (I, [P, ctypes.POINTER(_Tuning)]),
        "hd_edit_set_tuning": (I, [P, ctypes.POINTER(_Tuning)]),
        "hd_edit_autotune": (I, [P, U32, P, U32, ctypes.POINTER(_Tuning), P, P]),
        "hd_edit_profile_begin": (I, [P, U32]),
        "hd_edit_profile_end": (I, [P, P, P]),
        "hd_pool_kernel_launches": (U64, [P]),
        "hd_pool_read_bucket_words": (I, [P, U32, U32, P]),
        "hd_pool_read_page_map": (I, [P, P]),
        "hd_pool_read_pages": (I, [P, P, U32, P]),
        "hd_pool_upload": (I, [P, P, P, U32, P, P]),
        "hd_pool_epoch": (I, [P, P]),
        "hd_query": (I, [P, U32, P, U32, P, P]),
        "hd_trace": (I, [P, U32, P, P, U32, P, P]),
        "hd_trace_pinhole_async": (I, [P, U32, P, U32, U32, U32, P, P, P]),
        "hd_trace_pinhole_stackless_async": (I, [P, U32, P, U32, U32, U32, P, P, P]),
        "hd_trace_pinhole_lod_async": (I, [P, U32, P, U32, U32, U32, ctypes.c_float, ctypes.c_float, P, P, P]),
        "hd_projection_factor": (ctypes.c_float, [ctypes.c_float, U32, U32]),
        "hd_server_create": (I, [P, P, U32, ctypes.POINTER(_ServerConfig), ctypes.POINTER(P)]),
        "hd_server_destroy": (None, [P]),
        "hd_server_submit_edits": (I, [P, U32, P, U32, ctypes.POINTER(U64)]),
        "hd_server_submit_camera": (I, [P, U32, P, U32, U32, U32, P, ctypes.POINTER(U64)]),
        "hd_server_wait": (I, [P, U64, ctypes.c_double, ctypes.POINTER(_RequestResult)]),
        "hd_server_drain": (I, [P]),
        "hd_server_pause": (I, [P, I]),
        "hd_server_scene_root": (I, [P, U32, ctypes.POINTER(U32)]),
        "hd_server_get_stats": (I, [P, ctypes.POINTER(_ServerStats)]),
        "hd_count_voxel_edits": (U64, [P, U32, U32]),
        "hd_color_pool_create": (I, [P, ctypes.POINTER(_ColorConfig), ctypes.POINTER(P)]),
        "hd_color_pool_destroy": (None, [P]),
        "hd_color_pool_read": (I, [P, P, ctypes.POINTER(U64), P, ctypes.POINTER(U64)]),
        "hd_vbr_edit": (I, [P, P, U32, U32, P, U32, ctypes.POINTER(U32), ctypes.POINTER(U32)]),
        "hd_color_fetch": (I, [P, U32, P, U32, P, P]),
        "hd_status_string": (ctypes.c_char_p, [I]),
        "hd_device_available": (I, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def device_available() -> bool:
    return bool(lib().hd_device_available())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(status: int, what: str):
    if status != 0:
        raise HashDagError(status, what)


@dataclass
class Config:
    """hashdag::Config<uint32_t> (include/hashdag/Config.hpp:15-57)."""
    word_bits_per_page: int
    page_bits_per_bucket: int
    bucket_bits_each_level: List[int]
    hasher: int = 0  # 0 MurmurHasher32, 1 all nodes to bucket 0 of their level (test ZeroHasher)

    def get_node_levels(self) -> int:
        return len(self.bucket_bits_each_level)

    def get_leaf_level(self) -> int:
        return self.get_node_levels()

    def get_voxel_level(self) -> int:
        return self.get_node_levels() + 1

    def get_resolution(self) -> int:
        return 1 << self.get_voxel_level()

    def get_words_per_page(self) -> int:
        return 1 << self.word_bits_per_page

    def get_pages_per_bucket(self) -> int:
        return 1 << self.page_bits_per_bucket

    def get_words_per_bucket(self) -> int:
        return 1 << (self.word_bits_per_page + self.page_bits_per_bucket)

    def get_buckets_at_level(self, level: int) -> int:
        return 1 << self.bucket_bits_each_level[level]

    def get_level_base_bucket_indices(self) -> List[int]:
        out, b = [], 0
        for bits in self.bucket_bits_each_level:
            out.append(b)
            b += 1 << bits
        return out

    def get_total_buckets(self) -> int:
        return sum(1 << b for b in self.bucket_bits_each_level)

    def get_total_pages(self) -> int:
        return self.get_total_buckets() << self.page_bits_per_bucket

    def get_total_words(self) -> int:
        return self.get_total_buckets() << (self.word_bits_per_page + self.page_bits_per_bucket)

    def to_c(self) -> _Config:
        c = _Config()
        c.word_bits_per_page = self.word_bits_per_page
        c.page_bits_per_bucket = self.page_bits_per_bucket
        c.node_levels = len(self.bucket_bits_each_level)
        c.hasher = self.hasher
        for i, b in enumerate(self.bucket_bits_each_level):
            c.bucket_bits_each_level[i] = b
        return c

    def validate(self) -> bool:
        """Config::Validate (include/hashdag/Config.hpp:48-56)."""
        if self.word_bits_per_page < 4:
            return False
        total = sum(1 << b for b in self.bucket_bits_each_level) << (self.word_bits_per_page + self.page_bits_per_bucket)
        return total - 1 <= 0xFFFFFFFE


@dataclass
class DefaultConfig:
    """hashdag::DefaultConfig<uint32_t> (include/hashdag/Config.hpp:59-75)."""
    level_count: int = 17
    top_level_count: int = 9
    word_bits_per_page: int = 9
    page_bits_per_bucket: int = 2
    bucket_bits_per_top_level: int = 10
    bucket_bits_per_bottom_level: int = 16

    def __call__(self) -> Config:
        bits = [self.bucket_bits_per_top_level if l < self.top_level_count else self.bucket_bits_per_bottom_level
                for l in range(self.level_count - 1)]
        return Config(self.word_bits_per_page, self.page_bits_per_bucket, bits)


class EditMode(enum.IntEnum):
    """EditMode of src/main.cpp:72 (kPaint recolours only: colour edits)."""
    kFill = OP_FILL
    kDig = OP_DIG
    kPaint = OP_PAINT


@dataclass
class VBRColor:
    """hashdag::VBRColor (include/hashdag/VBRColor.hpp:18-43): an RGB8 colour
    (bits_per_weight 0, colors = r | g << 8 | b << 16) or two R5G6B5 end
    points (low 16 bits first) mixed by weight / (2^bits_per_weight - 1)."""
    colors: int = 0
    weight: int = 0
    bits_per_weight: int = 0

    @staticmethod
    def rgb8(r: int, g: int, b: int) -> "VBRColor":
        return VBRColor(int(r) | int(g) << 8 | int(b) << 16)

    @staticmethod
    def weighted(left_r5g6b5: int, right_r5g6b5: int, weight: int, bits_per_weight: int) -> "VBRColor":
        return VBRColor(int(left_r5g6b5) | int(right_r5g6b5) << 16, int(weight), int(bits_per_weight))


@dataclass
class SphereEditor:
    """SphereEditor<Mode> (src/main.cpp:73-150): voxel p inside iff |p-center|^2 <= r2.
    With a colour it is the colour editor (kFill, kPaint) for hd_vbr_edit."""
    center: Sequence[int]
    r2: int
    mode: EditMode = EditMode.kFill
    color: Optional[VBRColor] = None

    def desc(self):
        return (SHAPE_SPHERE, int(self.mode), tuple(int(c) for c in self.center), (0, 0, 0), int(self.r2))


@dataclass
class AABBEditor:
    """AABBEditor (src/main.cpp:32-63): voxel p inside iff aabb_min <= p < aabb_max; kDig by symmetry.
    With a colour it is the colour editor (kFill; kPaint by symmetry) for hd_vbr_edit."""
    aabb_min: Sequence[int]
    aabb_max: Sequence[int]
    mode: EditMode = EditMode.kFill
    color: Optional[VBRColor] = None

    def desc(self):
        return (SHAPE_AABB, int(self.mode), tuple(int(c) for c in self.aabb_min), tuple(int(c) for c in self.aabb_max), 0)


def edits_to_array(editors: Iterable) -> np.ndarray:
    items = [e.desc() for e in editors]
    return np.array(items, dtype=EDIT_DTYPE)


def vbr_edits_to_array(editors: Iterable) -> np.ndarray:
    """Colour edits (VBR_EDIT_DTYPE) from editors; an editor without a colour
    must dig (the application's stateless digs)."""
    editors = list(editors)
    out = np.zeros(len(editors), VBR_EDIT_DTYPE)
    for i, e in enumerate(editors):
        out[i]["edit"] = np.array(e.desc(), dtype=EDIT_DTYPE)
        c = e.color
        if c is None:
            if e.mode != EditMode.kDig:
                raise ValueError("a colour edit that fills or paints needs a colour")
            continue
        out[i]["colors"], out[i]["weight"], out[i]["bits_per_weight"] = c.colors, c.weight, c.bits_per_weight
    return out


def projection_factor(fov_y: float, height: int, divisor: int = 1) -> float:
    """Pixel-tolerance projection factor of the renderer (src/rg/TracePass.cpp:114-118,
    divisor 1; src/rg/BeamPass.cpp:90-94, divisor 8)."""
    return float(lib().hd_projection_factor(float(fov_y), int(height), int(divisor)))


def count_voxel_edits(edits: np.ndarray, resolution: int) -> int:
    edits = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
    return int(lib().hd_count_voxel_edits(_ptr(edits), len(edits), resolution))


_DUMP_MAGIC = b"HDMP"
_DUMP_VERSION = 1


def write_pool_dump(path: str, config: Config, bucket_words, page_ids, pages):
    """Writes a pool dump, byte for byte the file HostPoolMirror::Save writes
    (include/hashdag_host_mirror.hpp): "HDMP", version 1, the hd_config, total
    buckets, the bucket word counts, the number of pages, then per page its id
    and words; little-endian uint32.  Pages in ascending id order."""
    bw = np.ascontiguousarray(bucket_words, dtype="<u4")
    ids = np.ascontiguousarray(page_ids, dtype="<u4")
    pg = np.ascontiguousarray(pages, dtype="<u4").reshape(len(ids), config.get_words_per_page())
    if len(bw) != config.get_total_buckets() or (len(ids) > 1 and np.any(np.diff(ids.astype(np.int64)) <= 0)):
        raise ValueError("bucket words of another configuration, or page ids not ascending")
    rec = np.empty((len(ids), 1 + pg.shape[1]), dtype="<u4")
    rec[:, 0] = ids
    rec[:, 1:] = pg
    with open(path, "wb") as f:
        f.write(_DUMP_MAGIC)
        f.write(np.array([_DUMP_VERSION], "<u4").tobytes())
        f.write(bytes(config.to_c()))
        f.write(np.array([len(bw)], "<u4").tobytes())
        f.write(bw.tobytes())
        f.write(np.array([len(ids)], "<u4").tobytes())
        f.write(rec.tobytes())


def read_pool_dump(path: str):
    """(config, bucket_words, page_ids, pages) of a pool dump (write_pool_dump,
    HostPoolMirror::Save); ValueError on a malformed file."""
    raw = open(path, "rb").read()
    csize = ctypes.sizeof(_Config)
    if raw[:4] != _DUMP_MAGIC or len(raw) < 8 + csize + 4:
        raise ValueError("not a pool dump")
    if int(np.frombuffer(raw, "<u4", 1, 4)[0]) != _DUMP_VERSION:
        raise ValueError("unknown pool dump version")
    c = _Config.from_buffer_copy(raw[8:8 + csize])
    if not 1 <= c.node_levels <= MAX_LEVELS:
        raise ValueError("malformed pool dump")
    config = Config(c.word_bits_per_page, c.page_bits_per_bucket, list(c.bucket_bits_each_level[:c.node_levels]),
                    c.hasher)
    off = 8 + csize
    nb = int(np.frombuffer(raw, "<u4", 1, off)[0])
    if nb != config.get_total_buckets() or len(raw) < off + 4 * (nb + 2):
        raise ValueError("malformed pool dump")
    bw = np.frombuffer(raw, "<u4", nb, off + 4).copy()
    off += 4 * (nb + 1)
    n_pages = int(np.frombuffer(raw, "<u4", 1, off)[0])
    wpp = config.get_words_per_page()
    if len(raw) != off + 4 + 4 * n_pages * (1 + wpp):
        raise ValueError("malformed pool dump")
    rec = np.frombuffer(raw, "<u4", n_pages * (1 + wpp), off + 4).reshape(n_pages, 1 + wpp)
    return config, bw, rec[:, 0].copy(), rec[:, 1:].copy()


class NodePool:
    """A device-resident node pool (NodePoolBase + DAGNodePool storage, on the GPU).

    ``heap_pages`` is the number of physical pages reserved on the device
    (``heap_pages << word_bits_per_page`` 32-bit words).
    """

    def __init__(self, config: Config, heap_pages: int = 1 << 16, index_log2: int = 0, device: int = 0):
        L = lib()
        self.config = config
        self._cfg = config.to_c()
        h = ctypes.c_void_p()
        _check(L.hd_pool_create(ctypes.byref(self._cfg), heap_pages, index_log2, device, ctypes.byref(h)),
               "hd_pool_create")
        self._h = h
        self.device = device
        self.root = NULL
        self._color_pools = weakref.WeakSet()  # closed before this pool

    # -- lifecycle -------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            for cp in list(getattr(self, "_color_pools", ())):
                cp.close()
            lib().hd_pool_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def get_config(self) -> Config:
        return self.config

    def filled_node_pointers(self) -> List[int]:
        out = np.zeros(self.config.get_node_levels(), np.uint32)
        _check(lib().hd_pool_filled_pointers(self._h, _ptr(out)), "hd_pool_filled_pointers")
        return [int(x) for x in out]

    def stats(self) -> dict:
        s = _Stats()
        _check(lib().hd_pool_get_stats(self._h, ctypes.byref(s)), "hd_pool_get_stats")
        return {k: getattr(s, k) for k, _ in _Stats._fields_}

    # -- edit path ---------------------------------------------------------
    def edit_async(self, root: int, d_edits: int, n: int, d_out_root: int, stream: int = 0):
        """Device edits (pointer to n hd_edit_desc) -> device root; no host sync."""
        _check(lib().hd_edit_async(self._h, root & 0xFFFFFFFF, ctypes.c_void_p(d_edits), n,
                                   ctypes.c_void_p(d_out_root), ctypes.c_void_p(stream)), "hd_edit_async")

    def edit_async_droot(self, d_root: int, d_edits: int, n: int, d_out_root: int, stream: int = 0):
        """Like edit_async, with the input root read from device memory."""
        _check(lib().hd_edit_async_droot(self._h, ctypes.c_void_p(d_root), ctypes.c_void_p(d_edits), n,
                                         ctypes.c_void_p(d_out_root), ctypes.c_void_p(stream)), "hd_edit_async_droot")

    def edit_async_droot_hinted(self, d_root: int, d_edits: int, h_edits: np.ndarray, d_out_root: int,
                                stream: int = 0):
        """edit_async_droot with a host copy of the same edits sizing the launch
        (bounding-box grids, one-CTA small passes) as edit() does."""
        h = np.ascontiguousarray(h_edits, dtype=EDIT_DTYPE)
        _check(lib().hd_edit_async_droot_hinted(self._h, ctypes.c_void_p(d_root), ctypes.c_void_p(d_edits), _ptr(h),
                                                len(h), ctypes.c_void_p(d_out_root), ctypes.c_void_p(stream)),
               "hd_edit_async_droot_hinted")

    def error(self) -> int:
        e = ctypes.c_uint32(0)
        _check(lib().hd_pool_get_error(self._h, ctypes.byref(e)), "hd_pool_get_error")
        return e.value

    def clear_error(self):
        _check(lib().hd_pool_clear_error(self._h), "hd_pool_clear_error")

    def edit(self, root: int, editors, stream: int = 0) -> int:
        """Apply one editor or an ordered list of editors / an EDIT_DTYPE array to root."""
        if isinstance(editors, np.ndarray):
            arr = np.ascontiguousarray(editors, dtype=EDIT_DTYPE)
        elif isinstance(editors, (SphereEditor, AABBEditor)):
            arr = edits_to_array([editors])
        else:
            arr = edits_to_array(editors)
        out = ctypes.c_uint32(NULL)
        _check(lib().hd_edit(self._h, root & 0xFFFFFFFF, _ptr(arr), len(arr), ctypes.byref(out),
                             ctypes.c_void_p(stream)), "hd_edit")
        return out.value

    def last_counters(self):
        """Per-level (items, candidates, inserted) of the last pass."""
        c = self.last_counters_full()
        return c["items"], c["candidates"], c["inserted"]

    def last_counters_full(self) -> dict:
        n = self.config.get_node_levels()
        names = ["items", "candidates", "candidate_words", "inserted", "inserted_words"]
        arrs = {k: np.zeros(n, np.uint64) for k in names}
        _check(lib().hd_edit_last_counters(self._h, *[_ptr(arrs[k]) for k in names]), "hd_edit_last_counters")
        return arrs

    def last_leaf_work(self) -> dict:
        """Work of the last pass's level-(L-2) leaf kernels."""
        v = np.zeros(7, np.uint64)
        _check(lib().hd_edit_last_leaf_work(self._h, _ptr(v)), "hd_edit_last_leaf_work")
        return dict(zip(["nodes", "pairs", "base_words", "old_leaves", "lookups", "cache_hits", "inner_lookups"],
                        (int(x) for x in v)))

    def last_probe_stats(self) -> dict:
        """Index slots visited by the last pass's probes, longest probe, bucket CAS retries."""
        v = np.zeros(3, np.uint64)
        _check(lib().hd_edit_last_probe_stats(self._h, _ptr(v[0:1]), _ptr(v[1:2]), _ptr(v[2:3])),
               "hd_edit_last_probe_stats")
        return {"probe_steps": int(v[0]), "max_probe": int(v[1]), "cas_retries": int(v[2])}

    def vbr_edit(self, root: int, color_pool: "DAGColorPool", color_root: int, edits) -> tuple:
        """Colour edits one after another (NodePoolBase::Edit with a
        VBREditorWrapper into the colour octree, src/main.cpp:224-242; digs are
        stateless): VBR_EDIT_DTYPE array or colour editors.  Returns (root,
        colour root)."""
        if not isinstance(edits, np.ndarray):
            edits = vbr_edits_to_array(edits)
        edits = np.ascontiguousarray(edits, dtype=VBR_EDIT_DTYPE)
        r, c = ctypes.c_uint32(0), ctypes.c_uint32(0)
        _check(lib().hd_vbr_edit(self._h, color_pool._h, root & 0xFFFFFFFF, color_root & 0xFFFFFFFF,
                                 _ptr(edits) if len(edits) else None, len(edits), ctypes.byref(r), ctypes.byref(c)),
               "hd_vbr_edit")
        return int(r.value), int(c.value)

    def gc(self, roots) -> tuple:
        """NodePoolThreadedGC::ThreadedGC: keeps what `roots` (and the filled nodes)
        reach, compacts the pool; returns (remapped roots, statistics)."""
        r = np.ascontiguousarray([int(x) & 0xFFFFFFFF for x in roots], np.uint32)
        st = _GcStats()
        _check(lib().hd_gc(self._h, _ptr(r) if len(r) else None, len(r), ctypes.byref(st)), "hd_gc")
        return [int(x) for x in r], {name: int(getattr(st, name)) for name, _ in _GcStats._fields_}

    def tuning(self) -> dict:
        t = _Tuning()
        _check(lib().hd_edit_get_tuning(self._h, ctypes.byref(t)), "hd_edit_get_tuning")
        return {name: getattr(t, name) for name, _ in _Tuning._fields_}

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        t = _Tuning(**cur)
        _check(lib().hd_edit_set_tuning(self._h, ctypes.byref(t)), "hd_edit_set_tuning")

    def autotune(self, root: int, edits: np.ndarray) -> dict:
        """Times the batched pass of `edits` on `root` for candidate launch shapes
        (the pool ends unchanged; its checkpoint slot is reused) and installs the
        fastest; returns the shape and the pass times before / after."""
        e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        t = _Tuning()
        before, after = ctypes.c_float(), ctypes.c_float()
        _check(lib().hd_edit_autotune(self._h, root & 0xFFFFFFFF, _ptr(e), len(e), ctypes.byref(t),
                                      ctypes.byref(before), ctypes.byref(after)), "hd_edit_autotune")
        out = {name: getattr(t, name) for name, _ in _Tuning._fields_}
        out["ms_before"], out["ms_after"] = before.value, after.value
        return out

    def checkpoint(self):
        _check(lib().hd_pool_checkpoint(self._h), "hd_pool_checkpoint")

    def rollback(self, stream: int = 0):
        _check(lib().hd_pool_rollback(self._h, ctypes.c_void_p(stream)), "hd_pool_rollback")

    def profile_begin(self, max_passes: int):
        _check(lib().hd_edit_profile_begin(self._h, max_passes), "hd_edit_profile_begin")

    def profile_end(self):
        """(phase times in ms summed over the profiled passes, number of passes).
        Phases: [0] root+expand, [1] leaf voxels, then the dedup launch of
        level L-1 down to 0, [last] finish."""
        n = self.config.get_node_levels() + 3
        out = np.zeros(n, np.float32)
        passes = ctypes.c_uint32(0)
        _check(lib().hd_edit_profile_end(self._h, _ptr(out), ctypes.byref(passes)), "hd_edit_profile_end")
        return out, passes.value

    def kernel_launches(self) -> int:
        return int(lib().hd_pool_kernel_launches(self._h))

    def epoch(self) -> int:
        """Generation of the committed words (hd_pool_epoch): changes with every
        GC, rollback or upload; between equal values the pool only appended."""
        e = ctypes.c_uint64(0)
        _check(lib().hd_pool_epoch(self._h, ctypes.byref(e)), "hd_pool_epoch")
        return int(e.value)

    def reserve(self, max_items: int, max_list_entries: int, max_edits: int):
        _check(lib().hd_edit_reserve(self._h, max_items, max_list_entries, max_edits), "hd_edit_reserve")

    # -- upsert ------------------------------------------------------------
    def upsert_nodes(self, level: int, nodes: Sequence[Sequence[int]]) -> List[int]:
        words = np.array([w for n in nodes for w in n], dtype=np.uint32)
        lens = np.array([len(n) for n in nodes], dtype=np.uint32)
        out = np.zeros(len(nodes), np.uint32)
        _check(lib().hd_upsert(self._h, level, _ptr(words), _ptr(lens), len(nodes), _ptr(out)), "hd_upsert")
        return [int(x) for x in out]

    def upsert_inner_node(self, level: int, node: Sequence[int]) -> int:
        return self.upsert_nodes(level, [node])[0]

    def upsert_leaf(self, level: int, leaf: Sequence[int]) -> int:
        return self.upsert_nodes(level, [leaf])[0]

    # -- host mirror -------------------------------------------------------
    def bucket_words(self) -> np.ndarray:
        n = self.config.get_total_buckets()
        out = np.zeros(n, np.uint32)
        _check(lib().hd_pool_read_bucket_words(self._h, 0, n, _ptr(out)), "hd_pool_read_bucket_words")
        return out

    def page_map(self) -> np.ndarray:
        out = np.zeros(self.config.get_total_pages(), np.uint8)
        _check(lib().hd_pool_read_page_map(self._h, _ptr(out)), "hd_pool_read_page_map")
        return out

    def read_pages(self, page_ids) -> np.ndarray:
        ids = np.ascontiguousarray(page_ids, dtype=np.uint32)
        out = np.zeros((len(ids), self.config.get_words_per_page()), np.uint32)
        _check(lib().hd_pool_read_pages(self._h, _ptr(ids), len(ids), _ptr(out)), "hd_pool_read_pages")
        return out

    def download(self):
        """(bucket_words, page_ids, pages) of the whole pool."""
        pm = self.page_map()
        ids = np.nonzero(pm)[0].astype(np.uint32)
        return self.bucket_words(), ids, self.read_pages(ids)

    def save(self, path: str):
        """The pool as a dump file (write_pool_dump; HostPoolMirror::Load reads it)."""
        bw, ids, pages = self.download()
        write_pool_dump(path, self.config, bw, ids, pages)

    def load(self, path: str):
        """Replaces the pool with a dump of a pool of the same configuration."""
        config, bw, ids, pages = read_pool_dump(path)
        if bytes(config.to_c()) != bytes(self.config.to_c()):
            raise ValueError("the dump holds a pool of another configuration")
        self.upload(bw, ids, pages)

    def upload(self, bucket_words, page_ids, pages, filled=None):
        bw = np.ascontiguousarray(bucket_words, dtype=np.uint32)
        ids = np.ascontiguousarray(page_ids, dtype=np.uint32)
        pg = np.ascontiguousarray(pages, dtype=np.uint32)
        fl = None if filled is None else np.ascontiguousarray(filled, dtype=np.uint32)
        _check(lib().hd_pool_upload(self._h, _ptr(bw), _ptr(ids), len(ids), _ptr(pg),
                                    None if fl is None else _ptr(fl)), "hd_pool_upload")

    # -- read path ---------------------------------------------------------
    def query(self, root: int, xyz) -> np.ndarray:
        pts = np.ascontiguousarray(xyz, dtype=np.uint32).reshape(-1, 3)
        out = np.zeros(len(pts), np.uint8)
        _check(lib().hd_query(self._h, root & 0xFFFFFFFF, _ptr(pts), len(pts), _ptr(out), None), "hd_query")
        return out

    def trace_pinhole_async(self, root: int, cameras: np.ndarray, width: int, height: int, d_out: int,
                            d_counters: int = 0, stream: int = 0):
        """Primary rays of pinhole cameras (CAMERA_DTYPE array, host) into a device buffer of hits."""
        cams = np.ascontiguousarray(cameras, dtype=CAMERA_DTYPE)
        _check(lib().hd_trace_pinhole_async(self._h, root & 0xFFFFFFFF, _ptr(cams), len(cams), width, height,
                                            ctypes.c_void_p(d_out), ctypes.c_void_p(d_counters or None),
                                            ctypes.c_void_p(stream)), "hd_trace_pinhole_async")

    def trace_pinhole_stackless_async(self, root: int, cameras: np.ndarray, width: int, height: int, d_out: int,
                                      d_counters: int = 0, stream: int = 0):
        """trace_pinhole_async through the stackless warp-coherent kernel (same hits)."""
        cams = np.ascontiguousarray(cameras, dtype=CAMERA_DTYPE)
        _check(lib().hd_trace_pinhole_stackless_async(self._h, root & 0xFFFFFFFF, _ptr(cams), len(cams), width, height,
                                                      ctypes.c_void_p(d_out), ctypes.c_void_p(d_counters or None),
                                                      ctypes.c_void_p(stream)), "hd_trace_pinhole_stackless_async")

    def trace_pinhole_lod_async(self, root: int, cameras: np.ndarray, width: int, height: int, proj_factor: float,
                                beam_proj_factor: float, d_out: int, d_counters: int = 0, stream: int = 0):
        """Renderer traversal with level of detail (trace.frag) and, when
        beam_proj_factor > 0, the 8x8 beam prepass (beam.frag) into device hits."""
        cams = np.ascontiguousarray(cameras, dtype=CAMERA_DTYPE)
        _check(lib().hd_trace_pinhole_lod_async(self._h, root & 0xFFFFFFFF, _ptr(cams), len(cams), width, height,
                                                float(proj_factor), float(beam_proj_factor), ctypes.c_void_p(d_out),
                                                ctypes.c_void_p(d_counters or None), ctypes.c_void_p(stream)),
               "hd_trace_pinhole_lod_async")

    def traversal(self, root: int, origins, dirs) -> np.ndarray:
        o = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 3)
        out = np.zeros(len(o), HIT_DTYPE)
        _check(lib().hd_trace(self._h, root & 0xFFFFFFFF, _ptr(o), _ptr(d), len(o), _ptr(out), None), "hd_trace")
        return out


REQ_EDIT, REQ_CAMERA = 0, 1


class DAGColorPool:
    """The colour octree of a node pool (the application's DAGColorPool,
    src/DAGColorPool.hpp:20-218, on the device): tagged 32-bit pointers,
    8-pointer nodes and VBR leaf chunks at ``leaf_level``.  Edited through
    ``NodePool.vbr_edit``; ``read`` gives back the reference's words."""

    NULL = 0xC0000000

    def __init__(self, pool: "NodePool", leaf_level: int, keep_history: bool = False, max_nodes: int = 1 << 20,
                 max_leaf_words: int = 1 << 24):
        self.pool = pool
        self.leaf_level = leaf_level
        cfg = _ColorConfig(leaf_level, int(keep_history), max_nodes, max_leaf_words)
        h = ctypes.c_void_p()
        _check(lib().hd_color_pool_create(pool._h, ctypes.byref(cfg), ctypes.byref(h)), "hd_color_pool_create")
        self._h = h
        pool._color_pools.add(self)

    def close(self):
        if getattr(self, "_h", None):
            lib().hd_color_pool_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def read(self):
        """(nodes (n, 8) uint32, leaf words uint32): the host mirror."""
        nn, nl = ctypes.c_uint64(0), ctypes.c_uint64(0)
        _check(lib().hd_color_pool_read(self._h, None, ctypes.byref(nn), None, ctypes.byref(nl)), "hd_color_pool_read")
        nodes = np.zeros((nn.value, 8), np.uint32)
        leaves = np.zeros(nl.value, np.uint32)
        _check(lib().hd_color_pool_read(self._h, _ptr(nodes), ctypes.byref(nn), _ptr(leaves), ctypes.byref(nl)),
               "hd_color_pool_read")
        return nodes[:nn.value], leaves[:nl.value]

    def fetch(self, color_root: int, xyz) -> np.ndarray:
        """Colours of voxels (n, 3) under color_root (trace.frag Color_Fetch): COLOR_DTYPE."""
        import torch
        pts = np.ascontiguousarray(xyz, dtype=np.uint32).reshape(-1, 3)
        dev = torch.device("cuda", self.pool.device)
        d_in = torch.from_numpy(pts.view(np.int32).copy()).to(dev)
        d_out = torch.zeros(len(pts) * COLOR_DTYPE.itemsize // 4, dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _check(lib().hd_color_fetch(self._h, color_root & 0xFFFFFFFF, ctypes.c_void_p(d_in.data_ptr()), len(pts),
                                    ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream)), "hd_color_fetch")
        torch.cuda.synchronize(dev)
        return d_out.cpu().numpy().view(COLOR_DTYPE).copy()


class Server:
    """Serving loop over resident scenes (hd_server_* of the C ABI).

    ``scenes`` is a list of (NodePool, root).  Edit requests of a scene are
    merged into one batched pass whenever the scene's previous pass has
    finished; camera requests are traced on their own streams against the
    scene's last finished root.  ``wait`` returns a result dict once per id.
    The pools must outlive the server and must not be edited around it while it
    runs.
    """

    def __init__(self, scenes, max_pass_edits: int = 0, ray_slots: int = 0, max_rays_per_request: int = 0,
                 reserve_pages: int = 0, pages_per_edit_hint: float = 0.0, gc_free_fraction: float = 0.0):
        self._pools = [p for p, _ in scenes]  # keep the pools alive
        handles = (ctypes.c_void_p * len(scenes))(*[p.handle for p, _ in scenes])
        roots = np.array([r & 0xFFFFFFFF for _, r in scenes], np.uint32)
        cfg = _ServerConfig(max_pass_edits, ray_slots, max_rays_per_request, reserve_pages, pages_per_edit_hint,
                            gc_free_fraction)
        h = ctypes.c_void_p()
        _check(lib().hd_server_create(handles, _ptr(roots), len(scenes), ctypes.byref(cfg), ctypes.byref(h)),
               "hd_server_create")
        self._h = h
        self._keep = {}

    def submit_edits(self, scene: int, edits: np.ndarray) -> int:
        e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        rid = ctypes.c_uint64()
        _check(lib().hd_server_submit_edits(self._h, scene, _ptr(e), len(e), ctypes.byref(rid)),
               "hd_server_submit_edits")
        return rid.value

    def submit_camera(self, scene: int, cameras: np.ndarray, width: int, height: int, out=None) -> int:
        """out: None (hits stay on the device), a HIT_DTYPE numpy array, or an
        object with data_ptr() (e.g. a pinned torch byte tensor) of
        n_cameras*width*height*40 bytes; kept alive until the result is taken."""
        cams = np.ascontiguousarray(cameras, dtype=CAMERA_DTYPE)
        n = len(cams) * width * height
        if out is None:
            ptr = None
        elif isinstance(out, np.ndarray):
            if out.nbytes < n * HIT_DTYPE.itemsize or not out.flags.c_contiguous:
                raise ValueError("output buffer too small or not contiguous")
            ptr = out.ctypes.data
        else:
            if out.numel() * out.element_size() < n * HIT_DTYPE.itemsize:
                raise ValueError("output buffer too small")
            ptr = out.data_ptr()
        rid = ctypes.c_uint64()
        _check(lib().hd_server_submit_camera(self._h, scene, _ptr(cams), len(cams), width, height,
                                             ctypes.c_void_p(ptr), ctypes.byref(rid)), "hd_server_submit_camera")
        if out is not None:
            self._keep[rid.value] = out
        return rid.value

    def wait(self, rid: int, timeout_ms: float = -1.0) -> Optional[dict]:
        """Result of request rid as a dict, or None if timeout_ms ran out."""
        r = _RequestResult()
        st = lib().hd_server_wait(self._h, rid, float(timeout_ms), ctypes.byref(r))
        if st == 7:
            return None
        _check(st, "hd_server_wait")
        self._keep.pop(rid, None)
        return {name: getattr(r, name) for name, _ in _RequestResult._fields_}

    def drain(self):
        _check(lib().hd_server_drain(self._h), "hd_server_drain")

    def pause(self, paused: bool = True):
        """While paused no new pass or ray request starts; submissions queue."""
        _check(lib().hd_server_pause(self._h, 1 if paused else 0), "hd_server_pause")

    def scene_root(self, scene: int) -> int:
        r = ctypes.c_uint32()
        _check(lib().hd_server_scene_root(self._h, scene, ctypes.byref(r)), "hd_server_scene_root")
        return r.value

    def stats(self) -> dict:
        s = _ServerStats()
        _check(lib().hd_server_get_stats(self._h, ctypes.byref(s)), "hd_server_get_stats")
        return {name: getattr(s, name) for name, _ in _ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().hd_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
