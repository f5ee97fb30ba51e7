"""The oracle: CPU restatement of the reference edit path, and a runner for the
reference's own header library.

TEST INFRASTRUCTURE ONLY -- imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, as the checker or the timed CPU baseline.  The
engine (vkhashdag_gb300) never imports it.

* ``OraclePool`` wraps liboracle.so (hashdag_oracle.cpp), a plain C++
  restatement of include/hashdag/NodePool.hpp + NodePoolThreadedEdit.hpp +
  NodePoolTraversal.hpp with the stateless editors of src/main.cpp.
* ``run_reference`` executes oracle/_ref/ref_driver, built from the reference's
  own headers by build_ref.sh where the reference tree exists (this is how the
  restatement is pinned and the golden fixtures under tests/golden/ are made).
"""
from __future__ import annotations

import ctypes
import os
import shutil
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")
# where the reference tree is read from when the reference driver is built
REFERENCE_ROOT = os.environ.get("HASHDAG_REFERENCE_ROOT", "/root/reference")

EDIT_DTYPE = np.dtype([("shape", "<u4"), ("op", "<u4"), ("p0", "<u4", (3,)), ("p1", "<u4", (3,)), ("r2", "<u8")],
                      align=True)
HIT_DTYPE = np.dtype([("voxel", "<u4", (3,)), ("size", "<u4"), ("level", "<u4"), ("hit", "<u4"), ("t", "<f4"),
                      ("pos", "<f4", (3,))])
NULL = 0xFFFFFFFF


def build(force: bool = False) -> str:
    """Compile the restatement into liboracle.so (OpenMP for the threaded edit)."""
    src = os.path.join(HERE, "hashdag_oracle.cpp")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cxx = shutil.which("g++") or "g++"
    tmp = LIB + ".tmp"
    cmd = [cxx, "-std=c++20", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_ref(reference_root: str = REFERENCE_ROOT) -> str | None:
    """Build oracle/_ref/ref_driver from the reference headers; None where the tree is absent."""
    if not os.path.exists(os.path.join(reference_root, "include", "hashdag", "NodePool.hpp")):
        return None
    drv = os.path.join(HERE, "ref_driver.cpp")
    if os.path.exists(REF_DRIVER) and os.path.getmtime(REF_DRIVER) >= os.path.getmtime(drv):
        return REF_DRIVER
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), reference_root], check=True)
    return REF_DRIVER


def reference_available() -> bool:
    return os.path.exists(REF_DRIVER)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P, U32, U64, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        sig = {
            "orc_pool_create": (P, [U32, U32, U32, P, U32]),
            "orc_pool_destroy": (None, [P]),
            "orc_pool_ok": (I, [P]),
            "orc_make_filled": (None, [P, P]),
            "orc_edit": (U32, [P, U32, P, U32]),
            "orc_threaded_edit": (U32, [P, U32, P, U32, U32, I]),
            "orc_max_threads": (I, []),
            "orc_upsert": (U32, [P, U32, P, U32]),
            "orc_bucket_words": (U32, [P, U32]),
            "orc_total_buckets": (U64, [P]),
            "orc_total_pages": (U64, [P]),
            "orc_read_page": (I, [P, U32, P]),
            "orc_pool_load": (None, [P, P, P, U32, P, P]),
            "orc_canonical": (I, [P, U32, P, P]),
            "orc_canonical_simple": (I, [P, U32, P, P]),
            "orc_count_voxel_edits": (U64, [P, U32, U32]),
            "orc_query": (None, [P, U32, P, U32, P]),
            "orc_dense": (None, [P, U32, P]),
            "orc_trace": (None, [P, U32, P, P, U32, P]),
            "orc_trace_threads": (None, [P, U32, P, P, U32, P, I]),
            "orc_gc": (None, [P, P, U32, I]),
            "orc_gc_serial": (None, [P, P, U32]),
            "orc_trace_pinhole_lod": (None, [P, U32, P, U32, U32, U32, ctypes.c_float, ctypes.c_float, P, I]),
            "orc_color_pool_create": (P, [U32, I]),
            "orc_color_pool_destroy": (None, [P]),
            "orc_color_nodes": (U64, [P, P]),
            "orc_color_leaves": (U64, [P, P]),
            "orc_color_pool_load": (None, [P, P, U64, P, U64]),
            "orc_vbr_edit": (None, [P, P, U32, U32, P, U32, U32, U32, U32, P, P]),
            "orc_color_fetch": (None, [P, P, U32, P, U32, P]),
            "orc_vbr_set_per_voxel": (None, [I]),
            "orc_hash_inner": (U32, [P, U32]),
            "orc_hash_leaf": (U32, [U32, U32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleColorPool:
    """Colour octree of the application's DAGColorPool (restated)."""

    NULL = 3 << 30

    def __init__(self, leaf_level, keep_history=False):
        self._h = lib().orc_color_pool_create(leaf_level, int(keep_history))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_color_pool_destroy(self._h)
            self._h = None

    def nodes(self):
        n = lib().orc_color_nodes(self._h, None)
        out = np.zeros((n, 8), np.uint32)
        lib().orc_color_nodes(self._h, _p(out))
        return out

    def load(self, nodes, leaves):
        """Replace the octree with (n, 8) nodes and leaf words (a device pool's mirror)."""
        n = np.ascontiguousarray(nodes, np.uint32).reshape(-1, 8)
        w = np.ascontiguousarray(leaves, np.uint32)
        lib().orc_color_pool_load(self._h, _p(n), len(n), _p(w), len(w))

    def leaves(self):
        n = lib().orc_color_leaves(self._h, None)
        out = np.zeros(n, np.uint32)
        lib().orc_color_leaves(self._h, _p(out))
        return out


class OraclePool:
    """Host pool of the restatement (vector-backed pages, like DAGNodePool's hooks)."""

    def __init__(self, word_bits_per_page, page_bits_per_bucket, bucket_bits_each_level, hasher=0):
        self.wbpp, self.pbpb = word_bits_per_page, page_bits_per_bucket
        self.bits = list(bucket_bits_each_level)
        self.L = len(self.bits)
        b = np.array(self.bits, np.uint32)
        self._h = lib().orc_pool_create(self.wbpp, self.pbpb, self.L, _p(b), hasher)

    @classmethod
    def from_config(cls, cfg):
        return cls(cfg.word_bits_per_page, cfg.page_bits_per_bucket, cfg.bucket_bits_each_level, cfg.hasher)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_pool_destroy(self._h)
            self._h = None

    @property
    def ok(self) -> bool:
        """False once a bucket overflowed (the reference then silently keeps the stale node)."""
        return bool(lib().orc_pool_ok(self._h))

    def make_filled(self):
        out = np.zeros(self.L, np.uint32)
        lib().orc_make_filled(self._h, _p(out))
        return [int(x) for x in out]

    def edit(self, root, edits) -> int:
        e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        return int(lib().orc_edit(self._h, root, _p(e), len(e)))

    def threaded_edit(self, root, edits, max_task_level, threads=0) -> int:
        e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        t = threads or lib().orc_max_threads()
        return int(lib().orc_threaded_edit(self._h, root, _p(e), len(e), max_task_level, t))

    def upsert(self, level, words) -> int:
        w = np.ascontiguousarray(words, dtype=np.uint32)
        return int(lib().orc_upsert(self._h, level, _p(w), len(w)))

    def bucket_words(self) -> np.ndarray:
        n = int(lib().orc_total_buckets(self._h))
        return np.array([lib().orc_bucket_words(self._h, i) for i in range(n)], np.uint32) if n < 4096 else \
            self._bucket_words_fast(n)

    def _bucket_words_fast(self, n):
        return np.fromiter((lib().orc_bucket_words(self._h, i) for i in range(n)), np.uint32, n)

    def dump(self):
        """(bucket_words, page_ids, pages) of all existing pages."""
        n_pages = int(lib().orc_total_pages(self._h))
        wpp = 1 << self.wbpp
        ids, pages = [], []
        buf = np.zeros(wpp, np.uint32)
        for i in range(n_pages):
            if lib().orc_read_page(self._h, i, _p(buf)):
                ids.append(i)
                pages.append(buf.copy())
        pg = np.stack(pages) if pages else np.zeros((0, wpp), np.uint32)
        return self.bucket_words(), np.array(ids, np.uint32), pg

    def load(self, bucket_words, page_ids, pages, filled=None):
        bw = np.ascontiguousarray(bucket_words, np.uint32)
        ids = np.ascontiguousarray(page_ids, np.uint32)
        pg = np.ascontiguousarray(pages, np.uint32)
        fl = None if filled is None else np.ascontiguousarray(filled, np.uint32)
        lib().orc_pool_load(self._h, _p(bw), _p(ids), len(ids), _p(pg), None if fl is None else _p(fl))

    def trace_pinhole_lod(self, root, cameras, width, height, proj_factor, beam_proj_factor=0.0, threads=0):
        """trace.frag main with level of detail (and the beam.frag prepass when
        beam_proj_factor > 0) for CAMERA_DTYPE cameras; HIT_DTYPE records."""
        from vkhashdag_gb300 import CAMERA_DTYPE, HIT_DTYPE
        cams = np.ascontiguousarray(cameras, CAMERA_DTYPE)
        out = np.zeros(len(cams) * width * height, HIT_DTYPE)
        t = threads or lib().orc_max_threads()
        lib().orc_trace_pinhole_lod(self._h, root, _p(cams), len(cams), width, height, float(proj_factor),
                                    float(beam_proj_factor), _p(out), t)
        return out

    def vbr_edit(self, root, color_pool, color_root, edit, kind, colors, weight=0, bpw=0):
        """One colour edit through VBREditorWrapper (kind 1 fill, 2 paint) with
        the old root for the colour rules; returns (root, colour root)."""
        e = np.ascontiguousarray(np.asarray(edit, EDIT_DTYPE).reshape(1))
        r, c = ctypes.c_uint32(0), ctypes.c_uint32(0)
        lib().orc_vbr_edit(self._h, color_pool._h, root, color_root, _p(e), kind, colors, weight, bpw, ctypes.byref(r),
                           ctypes.byref(c))
        return int(r.value), int(c.value)

    def color_fetch(self, color_pool, color_root, xyz):
        """trace.frag Color_Fetch of voxels (n,3): COLOR_DTYPE records."""
        q = np.ascontiguousarray(xyz, np.uint32).reshape(-1, 3)
        out = np.zeros(len(q), COLOR_DTYPE)
        lib().orc_color_fetch(self._h, color_pool._h, color_root, _p(q), len(q), _p(out))
        return out

    def gc(self, roots, threads=0):
        """NodePoolThreadedGC::ThreadedGC, the pool laid out in the one-worker
        order whatever `threads` (0 = all); returns the remapped roots."""
        r = np.ascontiguousarray(roots, np.uint32).copy()
        lib().orc_gc(self._h, _p(r), len(r), threads)
        return [int(x) for x in r]

    def gc_serial(self, roots):
        """The same collection on one thread, node by node (the cross-check of gc)."""
        r = np.ascontiguousarray(roots, np.uint32).copy()
        lib().orc_gc_serial(self._h, _p(r), len(r))
        return [int(x) for x in r]

    def canonical(self, root):
        """(ok, per-level unique node counts, per-level digests) of the reachable DAG."""
        c = np.zeros(self.L, np.uint64)
        d = np.zeros(self.L, np.uint64)
        ok = lib().orc_canonical(self._h, root, _p(c), _p(d))
        return bool(ok), [int(x) for x in c], [int(x) for x in d]

    def canonical_simple(self, root):
        """canonical() computed node by node on one thread (its cross-check)."""
        c = np.zeros(self.L, np.uint64)
        d = np.zeros(self.L, np.uint64)
        ok = lib().orc_canonical_simple(self._h, root, _p(c), _p(d))
        return bool(ok), [int(x) for x in c], [int(x) for x in d]

    def query(self, root, xyz) -> np.ndarray:
        pts = np.ascontiguousarray(xyz, np.uint32).reshape(-1, 3)
        out = np.zeros(len(pts), np.uint8)
        lib().orc_query(self._h, root, _p(pts), len(pts), _p(out))
        return out

    def dense(self, root) -> np.ndarray:
        R = 1 << (self.L + 1)
        out = np.zeros(R * R * R, np.uint8)
        lib().orc_dense(self._h, root, _p(out))
        return out.reshape(R, R, R)  # [z, y, x]

    def trace(self, root, origins, dirs, threads=1) -> np.ndarray:
        o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        out = np.zeros(len(o), HIT_DTYPE)
        if threads == 1:
            lib().orc_trace(self._h, root, _p(o), _p(d), len(o), _p(out))
        else:
            lib().orc_trace_threads(self._h, root, _p(o), _p(d), len(o), _p(out), threads)
        return out


def count_voxel_edits(edits, resolution) -> int:
    """Sum over the edits of the grid voxels inside each shape (exact)."""
    e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
    return int(lib().orc_count_voxel_edits(_p(e), len(e), resolution))


def hash_inner(words) -> int:
    w = np.ascontiguousarray(words, np.uint32)
    return int(lib().orc_hash_inner(_p(w), len(w)))


def hash_leaf(w0, w1) -> int:
    return int(lib().orc_hash_leaf(w0, w1))


# ---------------------------------------------------------------------- reference driver
MODE_EDIT, MODE_THREADED, MODE_UPSERT, MODE_TRACE, MODE_GC, MODE_VBR = 0, 1, 2, 3, 4, 5
# colour of one voxel: VBRColor fields and VBRColor::Get() (VBRColor.hpp:18-43)
COLOR_DTYPE = np.dtype([("has_value", "<u4"), ("colors", "<u4"), ("weight", "<u4"), ("bpw", "<u4"),
                        ("rgb", "<f4", (3,))])


def run_reference(mode, word_bits_per_page, page_bits_per_bucket, bucket_bits, edits=None, hasher=0, threads=1,
                  max_task_level=0xFFFFFFFF, upserts=None, rays=None, keep=None, vbr=None):
    """Run the reference headers through oracle/_ref/ref_driver.  Returns a dict
    with root, filled, bucket_words, page_ids, pages, elapsed_ns, and ptrs
    (upsert mode) or hits (trace mode: hit flags and positions).  Colour mode:
    vbr = dict(leaf_level, keep_history, ops=[(kind, colors, weight, bpw)] per
    edit, queries=(n,3) voxel coordinates); adds color_root, color_nodes
    (n,8), color_leaves and colors (per query: has_value, colors, weight,
    bpw, rgb)."""
    if not reference_available():
        raise RuntimeError("oracle/_ref/ref_driver is not built (reference tree absent)")
    edits = np.zeros(0, EDIT_DTYPE) if edits is None else np.ascontiguousarray(edits, EDIT_DTYPE)
    req = bytearray(b"HDRQ")
    req += struct.pack("<5I", mode, word_bits_per_page, page_bits_per_bucket, len(bucket_bits), hasher)
    req += struct.pack(f"<{len(bucket_bits)}I", *bucket_bits)
    req += struct.pack("<3I", threads, max_task_level, len(edits))
    req += edits.tobytes()
    if mode == MODE_UPSERT:
        req += struct.pack("<I", len(upserts))
        for level, words in upserts:
            req += struct.pack(f"<{2 + len(words)}I", level, len(words), *words)
    if mode == MODE_GC:
        req += struct.pack(f"<{1 + len(keep)}I", len(keep), *keep)
    if mode == MODE_VBR:
        q = np.ascontiguousarray(vbr["queries"], np.uint32).reshape(-1, 3)
        req += struct.pack("<2I", vbr["leaf_level"], int(vbr.get("keep_history", False)))
        for op in vbr["ops"]:
            req += struct.pack("<4I", *op)
        req += struct.pack("<I", len(q)) + q.tobytes()
    if mode == MODE_TRACE:
        o, d = rays
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        req += struct.pack("<I", len(o)) + o.tobytes() + d.tobytes()
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "req"), os.path.join(td, "res")
        with open(fi, "wb") as f:
            f.write(req)
        subprocess.run([REF_DRIVER, fi, fo], check=True)
        data = open(fo, "rb").read()
    assert data[:4] == b"HDRS"
    off = 4
    root, ok = struct.unpack_from("<2I", data, off)
    off += 8
    (ns,) = struct.unpack_from("<Q", data, off)
    off += 8
    L = len(bucket_bits)
    filled = list(struct.unpack_from(f"<{L}I", data, off))
    off += 4 * L
    (tb,) = struct.unpack_from("<I", data, off)
    off += 4
    bw = np.frombuffer(data, np.uint32, tb, off).copy()
    off += 4 * tb
    (npg,) = struct.unpack_from("<I", data, off)
    off += 4
    wpp = 1 << word_bits_per_page
    ids = np.zeros(npg, np.uint32)
    pages = np.zeros((npg, wpp), np.uint32)
    for i in range(npg):
        (ids[i],) = struct.unpack_from("<I", data, off)
        off += 4
        pages[i] = np.frombuffer(data, np.uint32, wpp, off)
        off += 4 * wpp
    out = dict(root=root, filled=filled, bucket_words=bw, page_ids=ids, pages=pages, elapsed_ns=ns)
    if mode == MODE_GC:
        (n,) = struct.unpack_from("<I", data, off)
        off += 4
        out["roots_before"] = list(struct.unpack_from(f"<{n}I", data, off))
        off += 4 * n
        out["roots_after"] = list(struct.unpack_from(f"<{n}I", data, off))
        off += 4 * n
        (out["gc_ns"],) = struct.unpack_from("<Q", data, off)
        off += 8
    if mode == MODE_VBR:
        (out["color_root"], nn) = struct.unpack_from("<2I", data, off)
        off += 8
        out["color_nodes"] = np.frombuffer(data, np.uint32, 8 * nn, off).reshape(nn, 8).copy()
        off += 32 * nn
        (nl,) = struct.unpack_from("<I", data, off)
        off += 4
        out["color_leaves"] = np.frombuffer(data, np.uint32, nl, off).copy()
        off += 4 * nl
        nq = len(np.asarray(vbr["queries"]).reshape(-1, 3))
        out["colors"] = np.frombuffer(data, COLOR_DTYPE, nq, off).copy()
        off += COLOR_DTYPE.itemsize * nq
        out["edit_ns"] = np.frombuffer(data, np.uint64, len(edits), off).copy()
        off += 8 * len(edits)
    if mode == MODE_UPSERT:
        (n,) = struct.unpack_from("<I", data, off)
        off += 4
        out["ptrs"] = list(struct.unpack_from(f"<{n}I", data, off))
    if mode == MODE_TRACE:
        (n,) = struct.unpack_from("<I", data, off)
        off += 4
        rec = np.frombuffer(data, np.dtype([("hit", "<u4"), ("pos", "<f4", (3,))]), n, off)
        out["hits"] = rec.copy()
        off += 16 * n
        (out["trace_ns"],) = struct.unpack_from("<Q", data, off)
    return out


def pool_words_digest(bucket_words, page_ids, pages, word_bits_per_page, page_bits_per_bucket) -> str:
    """sha256 over every bucket's word count and its words [0, count) in bucket
    order: the pool's meaningful content (words past a bucket's count, e.g. in
    pages a collection left behind, are not part of it)."""
    import hashlib
    wpp = 1 << word_bits_per_page
    where = {int(i): k for k, i in enumerate(page_ids)}
    h = hashlib.sha256()
    bw = np.asarray(bucket_words, np.uint32)
    h.update(bw.tobytes())
    for b in np.nonzero(bw)[0]:
        n = int(bw[b])
        first = int(b) << page_bits_per_bucket
        for k in range((n + wpp - 1) // wpp):
            m = min(wpp, n - k * wpp)
            h.update(np.ascontiguousarray(pages[where[first + k]][:m], np.uint32).tobytes())
    return h.hexdigest()
