"""The oracle restatement against the golden vectors produced by the
reference's own headers (tests/golden/golden.json), and -- where the reference
tree is present -- against the live reference driver.  CPU only."""
import numpy as np
import pytest

from helpers import config_from, scenario, scenario_edits, sha, rays_for


def test_generators_are_stable(golden):
    for s in golden["scenarios"]:
        assert sha(scenario_edits(s)) == s["edits_sha"], s["name"]


@pytest.mark.parametrize("name", ["scene64", "scene256", "scene1024", "mixed256", "mixed512", "terrain256",
                                  "aabb_kat", "full_then_dig", "zero_hasher16", "tiny_pages64"])
def test_serial_edit_pool_is_word_identical(golden, orc, name):
    """NodePoolBase::Edit restated: same root, same pool words as the reference."""
    s = scenario(golden, name)
    cfg = config_from(s["config"])
    pool = orc.OraclePool.from_config(cfg)
    root = pool.edit(orc.NULL, scenario_edits(s))
    assert pool.ok
    assert root == s["root"]
    bw, ids, pages = pool.dump()
    assert sha(bw, ids, pages) == s["pool_sha"]
    ok, counts, digests = pool.canonical(root)
    assert ok and counts == s["canonical_counts"] and [str(d) for d in digests] == s["canonical_digests"]
    from vkhashdag_gb300 import workloads as W
    occ = pool.query(root, W.point_queries(s["res"], s["n_queries"], s["query_seed"]))
    assert sha(occ) == s["query_sha"] and int(occ.sum()) == s["query_set"]


@pytest.mark.parametrize("name", ["scene256", "mixed256", "terrain256"])
def test_threaded_edit_same_canonical_dag(golden, orc, name):
    """NodePoolThreadedEdit restated (OpenMP tasks): canonical DAG equals the serial one."""
    s = scenario(golden, name)
    assert s["threaded_canonical_equal"]
    cfg = config_from(s["config"])
    pool = orc.OraclePool.from_config(cfg)
    root = pool.threaded_edit(orc.NULL, scenario_edits(s), max(0, cfg.get_node_levels() - 4), 4)
    ok, counts, digests = pool.canonical(root)
    assert ok and [str(d) for d in digests] == s["canonical_digests"]


def test_aabb_known_answers(golden, orc):
    """test/test.cpp:161-199: fill twice keeps the root, (3,3,3) set, (4,3,3)
    clear, a sub-box fill inside a filled box keeps the root."""
    s = scenario(golden, "aabb_kat")
    cfg = config_from(s["config"])
    edits = scenario_edits(s)
    pool = orc.OraclePool.from_config(cfg)
    roots = []
    r = orc.NULL
    for k in range(len(edits)):
        r = pool.edit(r, edits[k:k + 1])
        roots.append(r)
    assert roots == s["roots_after_each"]
    assert roots[0] == roots[1] and roots[2] == roots[3] and roots[1] != roots[2]
    assert pool.query(roots[1], [[3, 3, 3], [4, 3, 3]]).tolist() == [1, 0]
    assert pool.query(orc.NULL, [[3, 3, 3]]).tolist() == [0]
    assert pool.query(roots[3], [[4, 3, 3]]).tolist() == [1]


def test_upsert_known_answers(golden, orc):
    """test/test.cpp:118-147: idempotent upsert, bucket word counts 3/9/2,
    same node at another level gets another pointer."""
    k = golden["upsert_kat"]
    cfg = config_from(k["config"])
    pool = orc.OraclePool.from_config(cfg)
    pool.make_filled()
    ptrs = [pool.upsert(level, words) for level, words in k["ops"]]
    assert ptrs == k["ptrs"]
    assert ptrs[0] == ptrs[1] and ptrs[2] != ptrs[0] and ptrs[3] != ptrs[2]
    wpb = cfg.get_words_per_bucket()
    bw = pool.bucket_words()
    assert [int(bw[p // wpb]) for p in ptrs] == k["bucket_words_of_ptrs"]


def test_bucket_full_known_answer(golden, orc):
    """test/test.cpp:148-160: with every node in one bucket, exactly the words
    of the bucket minus the filled node fit, pointers stay 3-word aligned in a page."""
    k = golden["bucket_full_kat"]
    cfg = config_from(k["config"])
    pool = orc.OraclePool.from_config(cfg)
    pool.make_filled()
    ptrs = []
    for c in range(k["n_ops"]):
        p = pool.upsert(0, [0b11, c, 0x45])
        if p == orc.NULL:
            break
        ptrs.append(p)
    assert len(ptrs) == k["fit"]
    assert (cfg.get_words_per_page() // 3) * cfg.get_pages_per_bucket() == k["fit"] + 3  # 9-word filled node
    assert all((p % cfg.get_words_per_page()) % 3 == 0 for p in ptrs)
    assert sha(np.array(ptrs, np.uint32)) == k["ptrs_sha"]


@pytest.mark.parametrize("idx", [0, 1, 2])
def test_traversal_matches_reference(golden, orc, idx):
    """NodePoolTraversal::Traversal restated: same hit flags and bit-identical positions."""
    t = golden["traversal"][idx]
    s = scenario(golden, t["scenario"])
    cfg = config_from(s["config"])
    pool = orc.OraclePool.from_config(cfg)
    root = pool.edit(orc.NULL, scenario_edits(s))
    o, d = rays_for(t["n"], t["seed"])
    hits = pool.trace(root, o, d)
    assert hits["hit"].tolist() == t["hit"]
    got = hits["pos"].view(np.uint32)
    want = np.array(t["pos_bits"], np.uint32)
    m = hits["hit"] == 1
    assert np.array_equal(got[m], want[m])
    # the hit voxel contains the hit position
    R = 1 << cfg.get_voxel_level()
    vox = hits["voxel"][m].astype(np.int64)
    p = hits["pos"][m].astype(np.float64) * R
    assert np.all(p >= vox - 1e-3) and np.all(p <= vox + hits["size"][m, None] + 1e-3)


def test_live_reference_when_present(orc):
    """Where the reference tree exists, re-run one scenario through its headers."""
    if orc.build_ref() is None:
        pytest.skip("reference tree not present on this machine")
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(128)
    e = W.mixed_batch(128, 300, seed=17, r_max=20, side_max=40)
    r = orc.run_reference(orc.MODE_EDIT, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                          cfg.bucket_bits_each_level, e)
    pool = orc.OraclePool.from_config(cfg)
    root = pool.edit(orc.NULL, e)
    bw, ids, pages = pool.dump()
    assert root == r["root"] and np.array_equal(pages, r["pages"]) and np.array_equal(bw, r["bucket_words"])


def gc_case(golden, name):
    return next(g for g in golden["gc"] if g["name"] == name)


def oracle_pool_with_roots(orc, g):
    """The case's edits applied one by one; the roots kept after edits keep_after."""
    cfg = config_from(g["config"])
    pool = orc.OraclePool.from_config(cfg)
    edits = scenario_edits(g)
    assert sha(edits) == g["edits_sha"]
    root, kept = orc.NULL, {}
    for i in range(len(edits)):
        root = pool.edit(root, edits[i:i + 1])
        kept[i] = root
    return cfg, pool, root, [kept[k] for k in g["keep_after"]]


@pytest.mark.parametrize("name", ["gc_mixed256", "gc_only_filled", "gc_tiny_pages64", "gc_zero16"])
def test_gc_matches_reference(golden, orc, name):
    """NodePoolThreadedGC::ThreadedGC restated (one-worker order): same remapped
    roots, same pool words, same filled pointers as the reference's collector."""
    g = gc_case(golden, name)
    cfg, pool, root, roots = oracle_pool_with_roots(orc, g)
    wb, pb = cfg.word_bits_per_page, cfg.page_bits_per_bucket
    assert root == g["pre_root"] and roots == g["roots_before"]
    assert orc.pool_words_digest(*pool.dump(), wb, pb) == g["pre_digest"]
    before = [pool.canonical(r)[2] for r in roots]
    new = pool.gc(roots)
    assert pool.ok
    assert new == g["roots_after"]
    bw, ids, pages = pool.dump()
    assert int(bw.sum()) == g["post_words"]
    assert orc.pool_words_digest(bw, ids, pages, wb, pb) == g["post_digest"]
    assert pool.make_filled() == g["filled_after"]
    assert [pool.canonical(r)[2] for r in new] == before  # same DAGs under the new pointers


def test_lod_oracle_without_cut_equals_plain_traversal(orc):
    """The level-of-detail restatement with an unbounded projection factor is
    the plain traversal (pinned against the reference above) on the same rays."""
    import vkhashdag_gb300 as hd
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(128)
    pool = orc.OraclePool.from_config(cfg)
    root = pool.edit(orc.NULL, W.sphere_scene(128, 8, seed=3))
    cams = np.zeros(1, hd.CAMERA_DTYPE)
    cams["position"] = [[0.1, 0.8, 0.2]]
    look = np.array([0.5, -0.5, 0.6]); look /= np.linalg.norm(look)
    cams["look"], cams["side"], cams["up"] = look, [0.5, 0.0, -0.3], [0.0, 0.5, 0.2]
    w, h = 40, 24
    lod = pool.trace_pinhole_lod(root, cams, w, h, float("inf"))
    px, py = np.meshgrid(np.arange(w, dtype=np.float32), np.arange(h, dtype=np.float32))
    u = ((px.ravel() + np.float32(0.5)) / np.float32(w)) * np.float32(2) - np.float32(1)
    v = ((py.ravel() + np.float32(0.5)) / np.float32(h)) * np.float32(2) - np.float32(1)
    c = cams[0]
    dd = (c["look"][None, :] - c["side"][None, :] * u[:, None]) - c["up"][None, :] * v[:, None]
    len2 = (dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1]) + dd[:, 2] * dd[:, 2]
    d = (dd * (np.float32(1) / np.sqrt(len2))[:, None]).astype(np.float32)
    o = np.tile(c["position"], (len(u), 1)).astype(np.float32)
    plain = pool.trace(root, o, d)
    assert lod.tobytes() == plain.tobytes()
    assert lod["hit"].mean() > 0.2
    # a finite projection factor cuts the descent: coarser voxels, fewer or equal levels
    coarse = pool.trace_pinhole_lod(root, cams, w, h, hd.projection_factor(np.pi / 3, h, 8))
    hit = coarse["hit"] == 1
    assert (coarse["size"][hit] >= 1).all() and (coarse["size"][hit] > 1).any()


VBR_NAMES = ["vbr_256_leaf3", "vbr_128_leaf5_history", "vbr_512_leaf2", "vbr_128_leaf0"]


@pytest.mark.parametrize("name", VBR_NAMES)
def test_vbr_colour_edit_matches_reference(golden, orc, name):
    """Colour edits through VBREditorWrapper restated: the same DAG root, colour
    root, colour octree nodes and leaf words (VBR chunks) as the reference's
    single-threaded Edit, and the same colour (VBRColor fields and RGB bits)
    for every query voxel."""
    from helpers import colors_sha, oracle_vbr_run, vbr_case
    g = vbr_case(golden, name)
    pool, cp, root, croot, q = oracle_vbr_run(orc, g)
    assert root == g["root"] and croot == g["color_root"]
    nodes, leaves = cp.nodes(), cp.leaves()
    assert len(nodes) == g["n_nodes"] and sha(nodes) == g["nodes_sha"]
    assert len(leaves) == g["n_leaf_words"] and sha(leaves) == g["leaves_sha"]
    c = pool.color_fetch(cp, croot, q)
    assert colors_sha(c) == g["colors_sha"]


def test_vbr_live_reference_when_present(orc):
    """Where the reference tree is built here, a fresh seeded colour case
    (weighted colours, paints, digs, two colour leaf levels) against the
    reference's own VBR writer."""
    if not orc.reference_available():
        pytest.skip("reference driver not built here")
    from vkhashdag_gb300 import workloads as W, OP_DIG, OP_FILL, OP_PAINT
    for res, leaf_level, seed in [(256, 4, 71), (128, 3, 72)]:
        cfg = W.serving_config(res)
        v = W.vbr_edits(res, 24, seed=seed, r_max=res // 4, side_max=res // 2, weighted_frac=0.5)
        q = W.point_queries(res, 2000, seed=seed)
        kinds = [({OP_DIG: 0, OP_FILL: 1, OP_PAINT: 2}[int(e["edit"]["op"])], int(e["colors"]), int(e["weight"]),
                  int(e["bits_per_weight"])) for e in v]
        r = orc.run_reference(orc.MODE_VBR, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                              cfg.bucket_bits_each_level, np.ascontiguousarray(v["edit"]),
                              vbr=dict(leaf_level=leaf_level, keep_history=False, ops=kinds, queries=q))
        pool = orc.OraclePool.from_config(cfg)
        cp = orc.OracleColorPool(leaf_level)
        root, croot = orc.NULL, orc.OracleColorPool.NULL
        for e, (k, col, w, b) in zip(v, kinds):
            if k == 0:
                root = pool.edit(root, np.asarray([e["edit"]]))
            else:
                root, croot = pool.vbr_edit(root, cp, croot, e["edit"], k, col, w, b)
        assert root == r["root"] and croot == r["color_root"]
        assert np.array_equal(cp.nodes(), r["color_nodes"]) and np.array_equal(cp.leaves(), r["color_leaves"])
        c = pool.color_fetch(cp, croot, q)
        assert np.array_equal(c["colors"], r["colors"]["colors"])
        assert np.array_equal(c["rgb"].view(np.uint32), r["colors"]["rgb"].view(np.uint32))


def _oracle_vbr_words(orc, cfg, v, leaf_level, keep_history):
    from vkhashdag_gb300 import OP_DIG, OP_PAINT
    pool = orc.OraclePool.from_config(cfg)
    cp = orc.OracleColorPool(leaf_level, keep_history)
    root, croot = orc.NULL, orc.OracleColorPool.NULL
    for e in v:
        op = int(e["edit"]["op"])
        if op == OP_DIG:
            root = pool.edit(root, np.asarray([e["edit"]]))
        else:
            root, croot = pool.vbr_edit(root, cp, croot, e["edit"], 2 if op == OP_PAINT else 1, int(e["colors"]),
                                        int(e["weight"]), int(e["bits_per_weight"]))
    return croot, cp.nodes(), cp.leaves()


@pytest.mark.parametrize("res,leaf_level,keep_history,seed",
                         [(256, 3, False, 81), (256, 5, True, 82), (512, 2, False, 83), (128, 0, False, 84),
                          (1024, 4, False, 85)])
def test_vbr_leaf_rewrite_in_runs_equals_voxel_by_voxel(orc, res, leaf_level, keep_history, seed):
    """The oracle rewrites an edited colour leaf in runs (whole runs copied or
    filled, as the reference's chunk iterator and writer do); the per-voxel form
    (decode every voxel, re-encode) must give the same octree and leaf words,
    with weighted colours, paints, digs, macro blocks (1024^3 with leaves of
    64^3 voxels: 16 macro blocks per leaf) and kept history."""
    from vkhashdag_gb300 import workloads as W
    cfg = W.serving_config(res)
    v = W.vbr_edits(res, 30, seed=seed, r_max=res // 4, side_max=res // 2, weighted_frac=0.5)
    try:
        orc.lib().orc_vbr_set_per_voxel(1)
        want = _oracle_vbr_words(orc, cfg, v, leaf_level, keep_history)
    finally:
        orc.lib().orc_vbr_set_per_voxel(0)
    got = _oracle_vbr_words(orc, cfg, v, leaf_level, keep_history)
    assert got[0] == want[0] and np.array_equal(got[1], want[1]) and np.array_equal(got[2], want[2])
    assert len(got[2]) > 0


def test_vbr_per_voxel_form_matches_reference(golden, orc):
    """The per-voxel form is pinned too (it is the cross-check of the runs)."""
    from helpers import oracle_vbr_run, vbr_case
    g = vbr_case(golden, "vbr_512_leaf2")
    try:
        orc.lib().orc_vbr_set_per_voxel(1)
        pool, cp, root, croot, q = oracle_vbr_run(orc, g)
    finally:
        orc.lib().orc_vbr_set_per_voxel(0)
    assert croot == g["color_root"] and sha(cp.leaves()) == g["leaves_sha"] and sha(cp.nodes()) == g["nodes_sha"]


@pytest.mark.parametrize("threads", [1, 3, 0])
@pytest.mark.parametrize("hasher", [0, 1])
def test_gc_on_threads_equals_one_thread(orc, threads, hasher):
    """The oracle's collector sorts each level's live nodes and lays out the
    buckets on several threads; it must leave the pool word for word as the
    one-thread, node-by-node form (the reference's one-worker order) does, with
    several roots, whatever the thread count (the zero hasher: every node of a
    level in one bucket, so one cache takes a whole level)."""
    from vkhashdag_gb300 import workloads as W, Config
    res, n_edits, scene = (512, 256, 16) if hasher == 0 else (64, 24, 4)
    base = W.config_for_resolution(res, bottom_bits=12, top_levels=6)
    cfg = Config(base.word_bits_per_page if hasher == 0 else 12, base.page_bits_per_bucket,
                 base.bucket_bits_each_level, hasher)
    a, b = orc.OraclePool.from_config(cfg), orc.OraclePool.from_config(cfg)
    roots = []
    ra = rb = orc.NULL
    edits = [W.sphere_scene(res, scene, seed=9)] + [
        W.mixed_batch(res, n_edits, seed=40 + k, r_max=res // 16, side_max=res // 8) for k in range(3)]
    for e in edits:
        ra, rb = a.edit(ra, e), b.edit(rb, e)
        roots.append(ra)
    assert ra == rb and a.ok and b.ok
    wb, pb = cfg.word_bits_per_page, cfg.page_bits_per_bucket
    new_a, new_b = a.gc(roots[1::2], threads), b.gc_serial(roots[1::2])
    assert new_a == new_b and a.ok and b.ok
    assert orc.pool_words_digest(*a.dump(), wb, pb) == orc.pool_words_digest(*b.dump(), wb, pb)
    assert a.make_filled() == b.make_filled()


@pytest.mark.parametrize("threads", [1, 3, 8])
@pytest.mark.parametrize("depth", ["root", "mid", "deep"])
def test_threaded_edit_any_team_and_depth(orc, threads, depth):
    """The threaded restatement forks every child but the last (run on the
    forking thread, as lf_edit_node does) on one thread team for the whole edit
    sequence: whatever the team size and the task depth, the same canonical DAG
    as the serial edit, and the same point occupancy."""
    from vkhashdag_gb300 import workloads as W
    res = 512
    cfg = W.config_for_resolution(res)
    L = cfg.get_node_levels()
    mtl = {"root": 0, "mid": max(0, L - 5), "deep": L - 1}[depth]
    edits = np.concatenate([W.sphere_scene(res, 16, seed=11), W.mixed_batch(res, 400, seed=12, r_max=32, side_max=64)])
    serial = orc.OraclePool.from_config(cfg)
    rs = serial.edit(orc.NULL, edits)
    threaded = orc.OraclePool.from_config(cfg)
    rt = threaded.threaded_edit(orc.NULL, edits, mtl, threads)
    ok, _, dig = threaded.canonical(rt)
    assert ok and threaded.ok and dig == serial.canonical(rs)[2]
    q = W.point_queries(res, 1 << 14, seed=13)
    assert np.array_equal(threaded.query(rt, q), serial.query(rs, q))


@pytest.mark.parametrize("name", ["scene256", "scene1024", "mixed512", "terrain256", "zero_hasher16", "tiny_pages64"])
def test_parallel_canonical_equals_node_by_node(golden, orc, name):
    """The all-threads canonicaliser (sorted pointer arrays, parallel tuple
    sort) gives the counts and digests of the node-by-node form."""
    s = scenario(golden, name)
    cfg = config_from(s["config"])
    pool = orc.OraclePool.from_config(cfg)
    root = pool.edit(orc.NULL, scenario_edits(s))
    assert pool.canonical(root) == pool.canonical_simple(root)
    assert pool.canonical(orc.NULL) == pool.canonical_simple(orc.NULL)


def test_oracle_voxel_count_matches_brute_force(orc):
    """Row-by-row sphere counting and clipped box volumes against a dense
    evaluation of the editors' voxel predicates, clipped spheres included."""
    from vkhashdag_gb300 import workloads as W
    res = 48
    e = W.mixed_batch(res, 60, seed=11, r_max=24, side_max=40)
    g = np.stack(np.meshgrid(np.arange(res), np.arange(res), np.arange(res), indexing="ij"), -1).reshape(-1, 3)
    want = 0
    for x in e:
        if x["shape"] == 1:
            inside = np.all((g >= x["p0"].astype(np.int64)) & (g < x["p1"].astype(np.int64)), axis=1)
        else:
            d = g - x["p0"].astype(np.int64)
            inside = (d * d).sum(1) <= int(x["r2"])
        want += int(inside.sum())
    assert orc.count_voxel_edits(e, res) == want


def test_bench_sequential_check_on_the_cpu(orc):
    """bench.py's check leg on a small workload: the oracle's own sequential
    result and a snapshot of another pool holding the same DAG (here: the
    serial editor's) have equal canonical digests and point occupancy."""
    import bench
    from vkhashdag_gb300 import workloads as W
    res = 256
    cfg = W.config_for_resolution(res, bottom_bits=16, top_levels=6)
    base, batches = bench.workload(0, 3, 256, res)
    q = W.point_queries(res, 1 << 12, seed=7)
    cpu, ref = bench.sequential_oracle_leg(cfg, base, batches[2], res, 2, 0.05, batches[0], q)
    assert ref["ok"] and cpu["value"] > 0 and cpu["serial"]["value"] > 0
    p = orc.OraclePool.from_config(cfg)
    r = p.edit(p.edit(orc.NULL, base), batches[2])
    ok, counts, digests = bench.device_canonical(cfg, p.dump(), p.make_filled(), r)
    assert ok and counts == ref["counts"] and digests == ref["digests"]
    assert np.array_equal(p.query(r, q), ref["occupancy"])
    scan = bench.bucket_scan_figures(cfg, p.dump()[0], {"candidates": np.full(cfg.get_node_levels(), 10),
                                                        "inserted": np.full(cfg.get_node_levels(), 4),
                                                        "candidate_words": np.full(cfg.get_node_levels(), 60)},
                                     [cfg.get_node_levels() - 2])
    (fig,) = scan.values()
    assert fig["mean_bucket_words"] > 0 and 0 < fig["scan_words_per_candidate"] <= fig["max_bucket_words"]
