"""Parity of the CUDA edit path with the oracle / reference golden vectors.

The bar is bit-exact: the canonical DAG under the returned root (per level,
the sorted unique node tuples with child pointers renumbered) equals the one
the reference's serial NodePoolBase::Edit produced, point occupancy equals,
and the device pool parses exactly like the reference scans a bucket."""
import numpy as np
import pytest

from helpers import (canonical_of_device, check_pool_structure, config_from, scenario, scenario_edits, sha)

pytestmark = pytest.mark.gpu

ALL = ["scene64", "scene256", "scene1024", "mixed256", "mixed512", "terrain256", "aabb_kat", "full_then_dig",
       "zero_hasher16", "tiny_pages64"]


def pool_for(hd, s, heap_pages=1 << 14):
    return hd.NodePool(config_from(s["config"]), heap_pages=heap_pages)


def check_against_golden(orc, pool, root, s):
    from vkhashdag_gb300 import workloads as W
    ok, counts, digests, _ = canonical_of_device(orc, pool, root)
    assert ok, "device DAG not reduced or malformed"
    assert counts == s["canonical_counts"]
    assert digests == s["canonical_digests"]
    occ = pool.query(root, W.point_queries(s["res"], s["n_queries"], s["query_seed"]))
    assert sha(occ) == s["query_sha"]


@pytest.mark.parametrize("name", ALL)
def test_batched_pass_matches_reference(golden, orc, hd, name):
    """All edits of the scenario in ONE level-synchronous pass."""
    s = scenario(golden, name)
    pool = pool_for(hd, s)
    root = pool.edit(hd.NULL, scenario_edits(s))
    check_against_golden(orc, pool, root, s)
    check_pool_structure(orc, pool)


@pytest.mark.parametrize("name", ["scene1024", "mixed512", "terrain256", "full_then_dig"])
def test_batched_pass_thread_per_node_leaves_matches_reference(golden, orc, hd, name):
    """The same batched pass with the level-(L-2) leaves rebuilt thread per
    node (k_leafparent_short) instead of the default form, whose partly
    covered leaves are compacted onto whole warps (k_leafparent_compact)."""
    s = scenario(golden, name)
    pool = pool_for(hd, s)
    pool.set_tuning(leaf_compact=0)
    root = pool.edit(hd.NULL, scenario_edits(s))
    check_against_golden(orc, pool, root, s)


@pytest.mark.parametrize("name", ["scene64", "scene256", "mixed256", "aabb_kat", "full_then_dig", "zero_hasher16"])
def test_plain_one_edit_per_pass_matches_reference(golden, orc, hd, name):
    """The plain form: one pass per edit, like NodePoolBase::Edit per edit."""
    s = scenario(golden, name)
    pool = pool_for(hd, s)
    edits = scenario_edits(s)
    root = hd.NULL
    for k in range(len(edits)):
        root = pool.edit(root, edits[k:k + 1])
    check_against_golden(orc, pool, root, s)
    check_pool_structure(orc, pool)


def test_filled_pointers_match_reference(golden, hd):
    """make_filled_node_pointers on a fresh pool: same pointers as the reference."""
    for name in ["scene256", "tiny_pages64", "zero_hasher16"]:
        s = scenario(golden, name)
        pool = pool_for(hd, s)
        assert pool.filled_node_pointers() == s["filled"], name


def test_upsert_known_answers_pointer_identical(golden, hd):
    """test/test.cpp:118-147 on the device: one node per call gives the
    reference's pointers and bucket word counts exactly."""
    k = golden["upsert_kat"]
    cfg = config_from(k["config"])
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    assert pool.filled_node_pointers() == k["filled"]
    ptrs = [pool.upsert_nodes(level, [words])[0] for level, words in k["ops"]]
    assert ptrs == k["ptrs"]
    bw = pool.bucket_words()
    wpb = cfg.get_words_per_bucket()
    assert [int(bw[p // wpb]) for p in ptrs] == k["bucket_words_of_ptrs"]
    bwp, ids, pages = pool.download()
    # the device pool holds the reference's pool word for word
    assert sha(bwp, ids, pages) == k["pool_sha"]


def test_upsert_batch_dedups_within_the_batch(hd):
    cfg = hd.DefaultConfig(level_count=6)()
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    nodes = [[0b11, 5, 7], [0b101, 9, 9], [0b11, 5, 7], [0b11, 5, 7], [0b1, 3]] * 40
    ptrs = pool.upsert_nodes(1, nodes)
    assert len(set(ptrs)) == 3
    assert ptrs[0] == ptrs[2] == ptrs[3]
    assert pool.upsert_nodes(1, [[0b11, 5, 7]])[0] == ptrs[0]
    assert pool.upsert_nodes(2, [[0b11, 5, 7]])[0] != ptrs[0]  # other level, other node


def test_bucket_full_is_reported(golden, hd):
    """test/test.cpp:148-160: the same number of nodes fits; the next one is
    an error (the reference silently returns the stale node)."""
    k = golden["bucket_full_kat"]
    cfg = config_from(k["config"])
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    ptrs = []
    with pytest.raises(hd.HashDagError) as e:
        for c in range(k["n_ops"]):
            ptrs.append(pool.upsert_nodes(0, [[0b11, c, 0x45]])[0])
    assert e.value.status == 2
    assert len(ptrs) == k["fit"]
    assert sha(np.array(ptrs, np.uint32)) == k["ptrs_sha"]


def test_edit_bucket_overflow_keeps_old_root(orc, hd):
    from vkhashdag_gb300 import workloads as W
    cfg = hd.Config(4, 0, [4, 4, 4, 4, 0])  # 16-word buckets, one leaf bucket
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    r1 = pool.edit(hd.NULL, hd.AABBEditor((4, 4, 4), (6, 6, 6)))
    with pytest.raises(hd.HashDagError) as e:
        pool.edit(r1, W.sphere_scene(64, 16, seed=3))
    assert e.value.status == 2
    assert pool.query(r1, [[4, 4, 4], [60, 60, 60]]).tolist() == [1, 0]


def test_heap_exhaustion_is_reported(hd):
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(256)
    pool = hd.NodePool(cfg, heap_pages=16)
    with pytest.raises(hd.HashDagError) as e:
        pool.edit(hd.NULL, W.sphere_scene(256, 16, seed=0))
    assert e.value.status == 3


def test_edge_cases(orc, hd):
    from vkhashdag_gb300 import workloads as W
    res = 64
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 12)
    filled = pool.filled_node_pointers()
    assert pool.edit(hd.NULL, np.zeros(0, hd.EDIT_DTYPE)) == hd.NULL
    assert pool.edit(hd.NULL, hd.AABBEditor((0, 0, 0), (res, res, res))) == filled[0]
    assert pool.edit(filled[0], hd.AABBEditor((0, 0, 0), (res + 7, res, 10 ** 6), hd.EditMode.kDig)) == hd.NULL
    r = pool.edit(hd.NULL, hd.SphereEditor((10, 10, 10), 25))
    assert pool.edit(r, hd.AABBEditor((res, 0, 0), (res + 50, res, res))) == r  # outside the grid
    assert pool.edit(r, hd.AABBEditor((5, 5, 5), (5, 9, 9))) == r  # empty box
    assert pool.edit(r, hd.SphereEditor((10, 10, 10), 25, hd.EditMode.kFill)) == r  # no-op refill
    assert pool.edit(r, hd.SphereEditor((40, 40, 40), 25, hd.EditMode.kDig)) == r  # dig in empty space
    # applying the same batch again returns the same root (global dedup)
    e = W.mixed_batch(res, 200, seed=8, r_max=10, side_max=20)
    r1 = pool.edit(r, e)
    r2 = pool.edit(r, e)
    assert r1 == r2
    # one voxel
    r3 = pool.edit(hd.NULL, hd.AABBEditor((63, 0, 31), (64, 1, 32)))
    assert pool.query(r3, [[63, 0, 31], [62, 0, 31]]).tolist() == [1, 0]


def test_single_level_pool(orc, hd):
    """node_levels = 1: the root is a leaf (4^3 voxels)."""
    cfg = hd.Config(4, 0, [3])
    pool = hd.NodePool(cfg, heap_pages=64)
    ref = orc.OraclePool.from_config(cfg)
    e = hd.edits_to_array([hd.SphereEditor((1, 1, 1), 2), hd.AABBEditor((2, 0, 0), (4, 2, 4)),
                           hd.SphereEditor((3, 3, 3), 1, hd.EditMode.kDig)])
    root = pool.edit(hd.NULL, e)
    rr = ref.edit(orc.NULL, e)
    ok, counts, dig, _ = canonical_of_device(orc, pool, root)
    assert ok and [str(x) for x in ref.canonical(rr)[2]] == dig


def test_batches_on_top_of_existing_scene(orc, hd):
    from vkhashdag_gb300 import workloads as W
    res = 512
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 14)
    ref = orc.OraclePool.from_config(cfg)
    scene = W.sphere_scene(res, 32, seed=1)
    batches = [W.mixed_batch(res, 300, seed=s, r_max=40, side_max=80) for s in (2, 3, 4)]
    root, rr = pool.edit(hd.NULL, scene), ref.edit(orc.NULL, scene)
    for b in batches:
        root, rr = pool.edit(root, b), ref.edit(rr, b)
        ok, counts, dig, _ = canonical_of_device(orc, pool, root)
        assert ok and dig == [str(x) for x in ref.canonical(rr)[2]]


def test_upload_reference_pool_and_continue(orc, hd):
    """A pool built by the reference's serial edit (word-identical oracle pool)
    uploads to the device, downloads unchanged, and edits continue on it."""
    from vkhashdag_gb300 import workloads as W
    res = 256
    cfg = W.config_for_resolution(res)
    ref = orc.OraclePool.from_config(cfg)
    rr = ref.edit(orc.NULL, W.sphere_scene(res, 16, seed=0))
    bw, ids, pages = ref.dump()
    pool = hd.NodePool(cfg, heap_pages=1 << 12)
    pool.upload(bw, ids, pages, ref.make_filled())
    bw2, ids2, pages2 = pool.download()
    assert np.array_equal(bw, bw2) and np.array_equal(ids, ids2) and np.array_equal(pages, pages2)
    b = W.mixed_batch(res, 400, seed=6, r_max=30, side_max=50)
    root = pool.edit(rr, b)
    rr2 = ref.edit(rr, b)
    ok, counts, dig, _ = canonical_of_device(orc, pool, root)
    assert ok and dig == [str(x) for x in ref.canonical(rr2)[2]]
    # nodes the reference already stored are found, not duplicated
    assert pool.edit(orc.NULL, W.sphere_scene(res, 16, seed=0)) == rr


def test_mid_size_batch_against_oracle(orc, hd):
    """2048 mixed edits at 2048^3 in one pass against the sequential oracle."""
    from vkhashdag_gb300 import workloads as W
    res = 2048
    cfg = W.config_for_resolution(res, bottom_bits=14, top_levels=6)
    pool = hd.NodePool(cfg, heap_pages=1 << 17)
    ref = orc.OraclePool.from_config(cfg)
    scene = W.sphere_scene(res, 64, seed=0)
    e = W.mixed_batch(res, 2048, seed=9, r_max=64, side_max=128)
    root = pool.edit(pool.edit(hd.NULL, scene), e)
    rr = ref.threaded_edit(ref.threaded_edit(orc.NULL, scene, 6), e, 6)
    ok, counts, dig, _ = canonical_of_device(orc, pool, root)
    assert ok and dig == [str(x) for x in ref.canonical(rr)[2]]
    q = W.point_queries(res, 1 << 18, seed=3)
    assert np.array_equal(pool.query(root, q), ref.query(rr, q))


def test_batched_equals_chunked_at_scale(hd):
    """Size-independent property at 16384^3: one pass over N edits, N passes of
    one edit, and passes over chunks all give the SAME root pointer, because
    the pool keeps every node unique (equal occupancy <=> equal root)."""
    from vkhashdag_gb300 import workloads as W
    res = 16384
    cfg = W.config_for_resolution(res, bottom_bits=16, top_levels=6)
    pool = hd.NodePool(cfg, heap_pages=1 << 20)
    base = pool.edit(hd.NULL, W.sphere_scene(res, 64, seed=0))
    e = W.mixed_batch(res, 512, seed=2, r_max=256, side_max=512)
    one = pool.edit(base, e)
    r = base
    for k in range(0, len(e), 64):
        r = pool.edit(r, e[k:k + 64])
    assert r == one
    r = base
    for k in range(0, 96):
        r = pool.edit(r, e[k:k + 1])
    assert r == pool.edit(base, e[:96])


def test_identity_and_paged_heaps_agree(golden, orc, hd):
    """The identity-mapped heap (heap spans every virtual page) and the paged
    heap (pages handed out on first use) store the same DAG."""
    s = scenario(golden, "mixed512")
    cfg = config_from(s["config"])
    edits = scenario_edits(s)
    paged = hd.NodePool(cfg, heap_pages=1 << 14)
    ident = hd.NodePool(cfg, heap_pages=cfg.get_total_pages())
    assert paged.stats()["heap_pages"] == 1 << 14 < cfg.get_total_pages()
    assert ident.stats()["heap_pages"] == cfg.get_total_pages()
    for pool in (paged, ident):
        root = pool.edit(hd.NULL, edits)
        check_against_golden(orc, pool, root, s)
        check_pool_structure(orc, pool)
    # an identity-mapped pool uploads and downloads like a paged one
    bw, ids, pages = paged.download()
    ident2 = hd.NodePool(cfg, heap_pages=cfg.get_total_pages())
    ident2.upload(bw, ids, pages, paged.filled_node_pointers())
    bw2, ids2, pages2 = ident2.download()
    assert np.array_equal(bw, bw2) and np.array_equal(ids, ids2) and np.array_equal(pages, pages2)


def test_one_cta_pass_equals_the_multi_kernel_pass(orc, hd):
    """A small pass through hd_edit runs as one CTA (one launch); the same edit
    through hd_edit_async (no host bounding box: the multi-kernel pass) on the
    same pool finds every node the first one stored: the same root."""
    import torch
    from vkhashdag_gb300 import workloads as W
    res = 1024
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 15)
    ref = orc.OraclePool.from_config(cfg)
    root = pool.edit(hd.NULL, W.sphere_scene(res, 16, seed=2))
    rr = ref.edit(orc.NULL, W.sphere_scene(res, 16, seed=2))
    edits = W.mixed_batch(res, 60, seed=77, r_max=12, side_max=20)
    pool.reserve(1 << 20, 1 << 20, 16)
    d_out = torch.zeros(1, dtype=torch.int32, device="cuda")
    one_launch = 0
    for k in range(len(edits)):
        e = edits[k:k + 1]
        n0 = pool.kernel_launches()
        r_small = pool.edit(root, e)
        one_launch += pool.kernel_launches() - n0 == 1
        d_e = torch.from_numpy(e.view(np.uint8).copy()).cuda()
        pool.edit_async(root, d_e.data_ptr(), 1, d_out.data_ptr(), 0)
        torch.cuda.synchronize()
        assert pool.error() == 0
        assert (int(d_out.item()) & 0xFFFFFFFF) == r_small, k
        root = r_small
        rr = ref.edit(rr, e)
    assert one_launch >= len(edits) // 2  # most of these small edits took the one-CTA pass
    ok, counts, dig, _ = canonical_of_device(orc, pool, root)
    assert ok and dig == [str(x) for x in ref.canonical(rr)[2]]


def test_launch_shape_never_changes_results(orc, hd):
    """Every launch shape (grid caps, long-list threshold) gives the same DAG;
    the autotuner leaves the pool as it found it."""
    from vkhashdag_gb300 import workloads as W
    res = 1024
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 15)
    root = pool.edit(hd.NULL, W.sphere_scene(res, 16, seed=4))
    batch = W.mixed_batch(res, 3000, seed=12, r_max=64, side_max=128)
    want = pool.edit(root, batch)
    shapes = [dict(long_threshold=1, expand_blocks_per_sm=1, leaf_blocks_per_sm=1, dedup_blocks_per_sm=1,
                   long_blocks_per_sm=1, leaf_compact=0),
              dict(long_threshold=64, expand_blocks_per_sm=32, leaf_blocks_per_sm=24, dedup_blocks_per_sm=32,
                   long_blocks_per_sm=8, leaf_compact=1),
              dict(long_threshold=4, expand_blocks_per_sm=2, leaf_blocks_per_sm=3, dedup_blocks_per_sm=4,
                   long_blocks_per_sm=2, leaf_compact=0),
              dict(long_threshold=16, expand_blocks_per_sm=8, leaf_blocks_per_sm=1, dedup_blocks_per_sm=8,
                   long_blocks_per_sm=4, leaf_compact=1)]
    for sh in shapes:
        pool.set_tuning(**sh)
        assert pool.edit(root, batch) == want, sh
    used = pool.stats()["used_pages"]
    t = pool.autotune(root, batch)
    assert t["ms_after"] <= t["ms_before"] and t["long_threshold"] >= 1
    assert pool.stats()["used_pages"] == used  # rolled back to where it started
    assert pool.edit(root, batch) == want
    with pytest.raises(hd.HashDagError):
        pool.set_tuning(long_threshold=0)


def test_graph_replayed_pass_equals_direct_pass(orc, hd):
    """hd_edit replays a captured CUDA graph for passes of 4096+ edits (captured on
    first use, recaptured when the workspace or launch shape changes): the same
    roots as the directly launched pass, and the oracle's DAG."""
    import torch
    from vkhashdag_gb300 import workloads as W
    res = 512
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 15)
    ref = orc.OraclePool.from_config(cfg)
    root = pool.edit(hd.NULL, W.sphere_scene(res, 16, seed=8))
    rr = ref.edit(orc.NULL, W.sphere_scene(res, 16, seed=8))
    d_out = torch.zeros(1, dtype=torch.int32, device="cuda")
    for k, n in enumerate((5000, 4096, 6000)):
        batch = W.mixed_batch(res, n, seed=300 + k, r_max=24, side_max=48)
        r_graph = pool.edit(root, batch)  # may grow the workspace and retry (a recapture each time)
        n0 = pool.kernel_launches()
        assert pool.edit(root, batch) == r_graph  # replay
        assert pool.kernel_launches() - n0 == 3 * cfg.get_node_levels()  # every kernel of the graph
        d_e = torch.from_numpy(batch.view(np.uint8).copy()).cuda()
        pool.edit_async(root, d_e.data_ptr(), n, d_out.data_ptr(), 0)
        torch.cuda.synchronize()
        assert pool.error() == 0 and (int(d_out.item()) & 0xFFFFFFFF) == r_graph
        if k == 1:
            pool.set_tuning(dedup_blocks_per_sm=4)  # recapture with another shape
        root = r_graph
        rr = ref.edit(rr, batch)
    ok, counts, dig, _ = canonical_of_device(orc, pool, root)
    assert ok and dig == [str(x) for x in ref.canonical(rr)[2]]


def test_graph_survives_a_rollback(orc, hd):
    """A rollback that leaves the filled pointers as they are keeps the
    captured pass graph: the next large pass is a replay (no recapture) and
    builds the same DAG as before the rollback.  The nodes are inserted again
    by concurrent warps, so the pointers (the root among them) may differ:
    the DAGs are compared canonically."""
    from vkhashdag_gb300 import workloads as W
    res = 512
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 15)
    root = pool.edit(hd.NULL, W.sphere_scene(res, 16, seed=9))
    pool.checkpoint()
    batch = W.mixed_batch(res, 5000, seed=77, r_max=24, side_max=48)
    r1 = pool.edit(root, batch)  # captures (and may grow the workspace)
    ok, _, want, _ = canonical_of_device(orc, pool, r1)
    assert ok
    pool.rollback(0)
    pool.edit(root, batch)
    pool.rollback(0)
    n0 = pool.kernel_launches()
    r = pool.edit(root, batch)
    assert pool.kernel_launches() - n0 == 3 * cfg.get_node_levels()  # replayed, not recaptured
    ok, _, dig, _ = canonical_of_device(orc, pool, r)
    assert ok and dig == want


def test_hinted_device_chain_equals_host_chain(orc, hd):
    """hd_edit_async_droot_hinted: the root stays on the device, a host copy of
    each edit sizes the launch as hd_edit does.  A chain of single edits (small
    passes as one CTA, larger ones as the multi-kernel pass) and one batched
    call end on the roots hd_edit gives on the same pool, and on the oracle's
    DAG."""
    import torch
    from vkhashdag_gb300 import workloads as W
    from helpers import canonical_of_device
    res = 512
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 15)
    base = W.sphere_scene(res, 8, seed=6)
    root0 = pool.edit(hd.NULL, base)
    edits = np.ascontiguousarray(W.mixed_batch(res, 48, seed=21, r_max=40, side_max=90))
    d_edits = torch.from_numpy(edits.view(np.uint8).copy()).cuda()
    d_root = torch.tensor([root0 - (1 << 32) if root0 >= (1 << 31) else root0], dtype=torch.int32, device="cuda")
    for k in range(len(edits)):
        pool.edit_async_droot_hinted(d_root.data_ptr(), d_edits.data_ptr() + 40 * k, edits[k:k + 1],
                                     d_root.data_ptr(), 0)
    torch.cuda.synchronize()
    assert pool.error() == 0
    dev_chain = int(d_root.item()) & 0xFFFFFFFF
    host_chain = root0
    for k in range(len(edits)):
        host_chain = pool.edit(host_chain, edits[k:k + 1])
    assert dev_chain == host_chain  # the same pool finds every node again
    d_root.fill_(root0 - (1 << 32) if root0 >= (1 << 31) else root0)
    pool.edit_async_droot_hinted(d_root.data_ptr(), d_edits.data_ptr(), edits, d_root.data_ptr(), 0)
    torch.cuda.synchronize()
    assert (int(d_root.item()) & 0xFFFFFFFF) == host_chain
    ref = orc.OraclePool.from_config(cfg)
    rr = ref.edit(ref.edit(orc.NULL, base), edits)
    ok, counts, digests, _ = canonical_of_device(orc, pool, host_chain)
    assert ok and digests == [str(d) for d in ref.canonical(rr)[2]]


def test_leaf_work_counters(orc, hd):
    """hd_edit_last_leaf_work after a batched pass: level-(L-2) nodes equal the
    pass's item count at that level, (node, edit) pairs at least the nodes,
    cache hits at most the lookups, and leaf candidates at most the lookups."""
    from vkhashdag_gb300 import workloads as W
    res = 1024
    cfg = W.config_for_resolution(res)
    L = cfg.get_node_levels()
    pool = hd.NodePool(cfg, heap_pages=1 << 15)
    root = pool.edit(hd.NULL, W.sphere_scene(res, 16, seed=4))
    pool.edit(root, W.mixed_batch(res, 5000, seed=13, r_max=64, side_max=128))
    w = pool.last_leaf_work()
    c = pool.last_counters_full()
    assert w["nodes"] == int(c["items"][L - 2]) > 0
    assert w["pairs"] >= w["nodes"]
    assert 0 < w["cache_hits"] <= w["lookups"]
    assert int(c["items"][L - 1]) <= w["lookups"]  # leaf candidates are the lookups that missed
    assert w["inner_lookups"] <= w["nodes"]
