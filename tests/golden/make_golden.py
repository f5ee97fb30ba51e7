"""Generates tests/golden/golden.json by running the reference's own hashdag
headers (oracle/_ref/ref_driver, built from the reference tree by
oracle/build_ref.sh).  Run from the repository root where the reference tree is
present:  python tests/golden/make_golden.py

Every scenario records what the reference produced: root pointer, filled-node
pointers, a SHA-256 of the whole pool (bucket words + pages), the canonical DAG
(per-level unique node counts and digests), point-occupancy digests, and for
upserts the returned pointers.  The workload generators are deterministic; the
SHA-256 of each edit array is stored so generator drift is caught.
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from vkhashdag_gb300 import workloads as W  # noqa: E402
from vkhashdag_gb300 import EDIT_DTYPE, edits_to_array, AABBEditor, SphereEditor, EditMode  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cfg_dict(cfg):
    return dict(word_bits_per_page=cfg.word_bits_per_page, page_bits_per_bucket=cfg.page_bits_per_bucket,
                bucket_bits=list(cfg.bucket_bits_each_level), hasher=cfg.hasher)


def scenario_edits(spec):
    kind = spec["kind"]
    a = spec.get("args", {})
    if kind == "sphere_scene":
        return W.sphere_scene(**a)
    if kind == "mixed_batch":
        return W.mixed_batch(**a)
    if kind == "terrain":
        return np.concatenate([W.terrain_columns(a["resolution"], a["block"], a["seed"]),
                               W.surface_spheres(a["resolution"], a["n"], a["seed"], a["band"], a["block"],
                                                 a["r_lo"], a["r_hi"])])
    if kind == "explicit":
        return np.array([tuple(x) for x in spec["edits"]], dtype=EDIT_DTYPE)
    if kind == "concat":
        return np.concatenate([scenario_edits(p) for p in spec["parts"]])
    raise ValueError(kind)


def explicit(editors):
    arr = edits_to_array(editors)
    return [[int(r["shape"]), int(r["op"]), [int(v) for v in r["p0"]], [int(v) for v in r["p1"]], int(r["r2"])]
            for r in arr]


SCENARIOS = [
    dict(name="scene64", res=64, kind="sphere_scene", args=dict(resolution=64, n_digs=8, seed=0)),
    dict(name="scene256", res=256, kind="sphere_scene", args=dict(resolution=256, n_digs=16, seed=0)),
    dict(name="scene1024", res=1024, kind="sphere_scene", args=dict(resolution=1024, n_digs=64, seed=0)),
    dict(name="mixed256", res=256, kind="mixed_batch",
         args=dict(resolution=256, n=500, seed=3, r_max=32, side_max=64)),
    dict(name="mixed512", res=512, kind="mixed_batch",
         args=dict(resolution=512, n=2000, seed=4, r_max=64, side_max=128)),
    dict(name="terrain256", res=256, kind="terrain",
         args=dict(resolution=256, block=8, seed=5, n=200, band=16, r_lo=2, r_hi=24)),
    dict(name="aabb_kat", res=32, kind="explicit", edits=explicit([
        AABBEditor((0, 0, 0), (4, 4, 4)), AABBEditor((0, 0, 0), (4, 4, 4)),
        AABBEditor((1, 1, 1), (5, 5, 5)), AABBEditor((1, 2, 3), (3, 5, 5))])),
    dict(name="full_then_dig", res=64, kind="explicit", edits=explicit([
        AABBEditor((0, 0, 0), (64, 64, 64)), SphereEditor((32, 32, 32), 20 * 20, EditMode.kDig),
        AABBEditor((0, 0, 0), (64, 64, 64), EditMode.kDig), SphereEditor((10, 50, 20), 9 * 9),
        AABBEditor((60, 60, 60), (1000, 1000, 1000)), SphereEditor((63, 0, 63), 5 * 5, EditMode.kDig)])),
    dict(name="zero_hasher16", res=16, kind="sphere_scene", hasher=1, wbpp=9, pbpb=4,
         args=dict(resolution=16, n_digs=4, seed=2)),
    dict(name="tiny_pages64", res=64, kind="sphere_scene", wbpp=4, pbpb=6, args=dict(resolution=64, n_digs=8, seed=9)),
]


def config_of(s):
    cfg = W.config_for_resolution(s["res"], word_bits_per_page=s.get("wbpp", 9),
                                  page_bits_per_bucket=s.get("pbpb", 2))
    cfg.hasher = s.get("hasher", 0)
    return cfg


def run_scenario(s):
    cfg = config_of(s)
    edits = scenario_edits(s)
    r = oracle.run_reference(oracle.MODE_EDIT, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                             cfg.bucket_bits_each_level, edits, hasher=cfg.hasher)
    op = oracle.OraclePool.from_config(cfg)
    op.load(r["bucket_words"], r["page_ids"], r["pages"], r["filled"])
    ok, counts, digests = op.canonical(r["root"])
    assert ok, s["name"]
    # 2^20 seeded point queries on the 1024^3 sphere scene (the CPU-runnable
    # configuration's verification), 2^16 elsewhere
    n_queries = 1 << 20 if s["name"] == "scene1024" else 1 << 16
    q = W.point_queries(s["res"], n_queries, seed=7)
    occ = op.query(r["root"], q)
    # threaded run of the reference: same canonical DAG
    L = cfg.get_node_levels()
    rt = oracle.run_reference(oracle.MODE_THREADED, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                              cfg.bucket_bits_each_level, edits, hasher=cfg.hasher, threads=4,
                              max_task_level=max(0, L - 4))
    op2 = oracle.OraclePool.from_config(cfg)
    op2.load(rt["bucket_words"], rt["page_ids"], rt["pages"], rt["filled"])
    ok2, c2, d2 = op2.canonical(rt["root"])
    rec = dict(s)
    rec.update(config=cfg_dict(cfg), edits_sha=sha(edits), n_edits=int(len(edits)), root=r["root"],
               filled=r["filled"], pool_sha=sha(r["bucket_words"], r["page_ids"], r["pages"]),
               canonical_counts=counts, canonical_digests=[str(d) for d in digests],
               query_seed=7, n_queries=n_queries, query_sha=sha(occ), query_set=int(occ.sum()),
               threaded_canonical_equal=bool(ok2 and d2 == digests))
    if s["name"] == "aabb_kat":  # roots after each step (test/test.cpp:161-199 intent)
        roots = []
        for k in range(1, len(edits) + 1):
            rk = oracle.run_reference(oracle.MODE_EDIT, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                                      cfg.bucket_bits_each_level, edits[:k], hasher=cfg.hasher)
            roots.append(rk["root"])
        rec["roots_after_each"] = roots
    return rec


def upsert_kats():
    # test/test.cpp:118-147 (Test upsert()), on a 4-node-level default config
    cfg = W.config_for_resolution(32)
    L = cfg.get_node_levels()
    node0 = [0b11, 0x23, 0x45]
    node1 = [0b110, 0x23, 0x44]
    node2 = [0xFF, 0x23, 0x44, 0x55, 0x66, 0x77, 0x88, 0x99, 0x01]
    leaf0 = [0x23, 0x55]
    ops = [(0, node0), (0, node0), (0, node1), (1, node1), (2, node2), (L - 1, leaf0)]
    r = oracle.run_reference(oracle.MODE_UPSERT, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                             cfg.bucket_bits_each_level, upserts=ops)
    wpb = cfg.get_words_per_bucket()
    bw = {int(p // wpb): int(r["bucket_words"][p // wpb]) for p in r["ptrs"]}
    kat = dict(config=cfg_dict(cfg), ops=[[l, w] for l, w in ops], ptrs=r["ptrs"], filled=r["filled"],
               bucket_words_of_ptrs=[bw[int(p // wpb)] for p in r["ptrs"]],
               pool_sha=sha(r["bucket_words"], r["page_ids"], r["pages"]))
    # test/test.cpp:148-160 (bucket full) with every node in one bucket
    zc = W.config_for_resolution(32)
    zc.hasher = 1
    n_ops = 700
    ops2 = [(0, [0b11, c, 0x45]) for c in range(n_ops)]
    r2 = oracle.run_reference(oracle.MODE_UPSERT, zc.word_bits_per_page, zc.page_bits_per_bucket,
                              zc.bucket_bits_each_level, hasher=1, upserts=ops2)
    ptrs = r2["ptrs"]
    first_null = next((i for i, p in enumerate(ptrs) if p == 0xFFFFFFFF), None)
    full = dict(config=cfg_dict(zc), n_ops=n_ops, node="[0b11, i, 0x45] at level 0", fit=first_null,
                ptrs_sha=sha(np.array(ptrs[:first_null], np.uint32)), first_ptrs=ptrs[:8], last_ptrs=ptrs[first_null - 4:first_null])
    return kat, full


# NodePoolThreadedGC (ThreadedGC on a one-worker busy pool): edits applied one
# by one, the roots after the edits listed in `keep` are the GC roots.
GC_CASES = [
    dict(name="gc_mixed256", res=256, kind="concat", keep=[10, 40, -1], parts=[
        dict(kind="sphere_scene", args=dict(resolution=256, n_digs=16, seed=0)),
        dict(kind="mixed_batch", args=dict(resolution=256, n=60, seed=3, r_max=30, side_max=60))]),
    dict(name="gc_only_filled", res=256, kind="concat", keep=[], parts=[
        dict(kind="sphere_scene", args=dict(resolution=256, n_digs=16, seed=0)),
        dict(kind="mixed_batch", args=dict(resolution=256, n=20, seed=3, r_max=30, side_max=60))]),
    dict(name="gc_tiny_pages64", res=64, kind="concat", wbpp=4, pbpb=6, keep=[5, -1], parts=[
        dict(kind="sphere_scene", args=dict(resolution=64, n_digs=8, seed=9)),
        dict(kind="mixed_batch", args=dict(resolution=64, n=40, seed=5, r_max=8, side_max=16))]),
    dict(name="gc_zero16", res=16, kind="concat", hasher=1, wbpp=9, pbpb=4, keep=[-1], parts=[
        dict(kind="sphere_scene", args=dict(resolution=16, n_digs=4, seed=2)),
        dict(kind="mixed_batch", args=dict(resolution=16, n=20, seed=6, r_max=4, side_max=6))]),
]


def gc_golden(s):
    cfg = config_of(s)
    edits = scenario_edits(s)
    keep = [k if k >= 0 else len(edits) - 1 for k in s["keep"]]
    wb, pb = cfg.word_bits_per_page, cfg.page_bits_per_bucket
    pre = oracle.run_reference(oracle.MODE_EDIT, wb, pb, cfg.bucket_bits_each_level, edits, hasher=cfg.hasher)
    post = oracle.run_reference(oracle.MODE_GC, wb, pb, cfg.bucket_bits_each_level, edits, hasher=cfg.hasher,
                                keep=keep)
    rec = dict(s)
    rec.update(config=cfg_dict(cfg), edits_sha=sha(edits), n_edits=int(len(edits)), keep_after=keep,
               pre_root=pre["root"], pre_filled=pre["filled"],
               pre_digest=oracle.pool_words_digest(pre["bucket_words"], pre["page_ids"], pre["pages"], wb, pb),
               roots_before=post["roots_before"], roots_after=post["roots_after"], filled_after=post["filled"],
               post_words=int(post["bucket_words"].sum()),
               post_digest=oracle.pool_words_digest(post["bucket_words"], post["page_ids"], post["pages"], wb, pb))
    return rec


# Colour edits through VBREditorWrapper into the colour octree
# (include/hashdag/VBREditor.hpp, VBRColor.hpp; src/DAGColorPool.hpp restated
# in oracle/ref_driver.cpp), single-threaded NodePoolBase::Edit.
VBR_CASES = [
    dict(name="vbr_256_leaf3", res=256, leaf_level=3, keep_history=False, args=dict(n=48, seed=31, r_max=64, side_max=128)),
    dict(name="vbr_128_leaf5_history", res=128, leaf_level=5, keep_history=True,
         args=dict(n=64, seed=35, r_max=32, side_max=64)),
    dict(name="vbr_512_leaf2", res=512, leaf_level=2, keep_history=False, args=dict(n=12, seed=33, r_max=160, side_max=256)),
    dict(name="vbr_128_leaf0", res=128, leaf_level=0, keep_history=False, args=dict(n=10, seed=34, r_max=40, side_max=64)),
]


def vbr_kinds(v):
    """ref_driver colour op per edit: 0 stateless (dig), 1 fill, 2 paint."""
    return [(int({W.OP_DIG: 0, W.OP_FILL: 1, W.OP_PAINT: 2}[int(e["edit"]["op"])]), int(e["colors"]), int(e["weight"]),
             int(e["bits_per_weight"])) for e in v]


def vbr_golden(s):
    cfg = W.serving_config(s["res"])
    v = W.vbr_edits(s["res"], **s["args"])
    edits = np.ascontiguousarray(v["edit"])
    q = W.point_queries(s["res"], 4096, seed=s["args"]["seed"] + 100)
    r = oracle.run_reference(oracle.MODE_VBR, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                             cfg.bucket_bits_each_level, edits, hasher=cfg.hasher,
                             vbr=dict(leaf_level=s["leaf_level"], keep_history=s["keep_history"], ops=vbr_kinds(v),
                                      queries=q))
    c = r["colors"]
    rec = dict(s)
    rec.update(config=cfg_dict(cfg), edits_sha=sha(v), root=r["root"], color_root=r["color_root"],
               n_nodes=int(len(r["color_nodes"])), nodes_sha=sha(r["color_nodes"]),
               n_leaf_words=int(len(r["color_leaves"])), leaves_sha=sha(r["color_leaves"]), n_queries=int(len(q)),
               colors_sha=sha(c["has_value"], c["colors"], c["weight"], c["bpw"], c["rgb"]),
               colors_head=[[int(c["has_value"][i]), int(c["colors"][i]), int(c["weight"][i]), int(c["bpw"][i]),
                             [int(x) for x in np.asarray(c["rgb"][i], np.float32).view(np.uint32)]] for i in range(8)])
    return rec


def rays_for(res, n, seed):
    o = W.uniform(seed, 41, 3 * n).reshape(n, 3).astype(np.float32)
    # half the rays start outside the cube
    out = W.uniform(seed, 42, n) < 0.5
    o[out] = (o[out] * 3.0 - 1.0).astype(np.float32)
    d = (W.uniform(seed, 43, 3 * n).reshape(n, 3) * 2.0 - 1.0).astype(np.float32)
    d[0] = (1.0, 0.0, 0.0)
    d[1] = (0.0, -1.0, 0.0)
    d[2] = (0.0, 0.0, 1e-9)
    return o, d


def traversal_golden(s, n=512, seed=11):
    cfg = config_of(s)
    edits = scenario_edits(s)
    o, d = rays_for(s["res"], n, seed)
    r = oracle.run_reference(oracle.MODE_TRACE, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                             cfg.bucket_bits_each_level, edits, hasher=cfg.hasher, rays=(o, d))
    h = r["hits"]
    return dict(scenario=s["name"], n=n, seed=seed, hit=[int(x) for x in h["hit"]],
                pos_bits=[[int(v) for v in np.asarray(p, np.float32).view(np.uint32)] for p in h["pos"]])


def main():
    oracle.build()
    if oracle.build_ref() is None:
        sys.exit("reference tree not found; golden fixtures can only be regenerated where it exists")
    g = dict(generator="tests/golden/make_golden.py", scenarios=[run_scenario(s) for s in SCENARIOS])
    g["upsert_kat"], g["bucket_full_kat"] = upsert_kats()
    by = {s["name"]: s for s in SCENARIOS}
    g["traversal"] = [traversal_golden(by["scene256"]), traversal_golden(by["mixed256"], n=384, seed=12),
                      traversal_golden(by["full_then_dig"], n=256, seed=13)]
    g["gc"] = [gc_golden(s) for s in GC_CASES]
    g["vbr"] = [vbr_golden(s) for s in VBR_CASES]
    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
