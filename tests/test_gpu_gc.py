"""hd_gc (NodePoolThreadedGC::ThreadedGC) on the device.

Parity: the pre-collection pool of every golden GC case is built by the oracle
(word-identical to the reference's, pinned by tests/test_oracle.py), uploaded,
collected on the device, and must come out word-identical to the reference's
collector: same remapped roots, same bucket contents, same filled pointers.
"""
import numpy as np
import pytest

from helpers import canonical_of_device, config_from, scenario_edits, sha

pytestmark = pytest.mark.gpu


def gc_case(golden, name):
    return next(g for g in golden["gc"] if g["name"] == name)


def oracle_pool_with_roots(orc, g):
    cfg = config_from(g["config"])
    pool = orc.OraclePool.from_config(cfg)
    edits = scenario_edits(g)
    assert sha(edits) == g["edits_sha"]
    root, kept = orc.NULL, {}
    for i in range(len(edits)):
        root = pool.edit(root, edits[i:i + 1])
        kept[i] = root
    return cfg, pool, [kept[k] for k in g["keep_after"]]


@pytest.mark.parametrize("name", ["gc_mixed256", "gc_only_filled", "gc_tiny_pages64", "gc_zero16"])
@pytest.mark.parametrize("paged", [False, True])
def test_gc_word_identical_to_reference(golden, orc, hd, name, paged):
    g = gc_case(golden, name)
    cfg, ref, roots = oracle_pool_with_roots(orc, g)
    assert roots == g["roots_before"]
    bw, ids, pages = ref.dump()
    heap = cfg.get_total_pages() if not paged else max(len(ids) + 8, 16)
    pool = hd.NodePool(cfg, heap_pages=heap)
    pool.upload(bw, ids, pages, ref.make_filled())
    new, st = pool.gc(roots)
    assert new == g["roots_after"]
    wb, pb = cfg.word_bits_per_page, cfg.page_bits_per_bucket
    bw2, ids2, pages2 = pool.download()
    assert int(bw2.sum()) == g["post_words"] == st["words_after"]
    assert orc.pool_words_digest(bw2, ids2, pages2, wb, pb) == g["post_digest"]
    assert pool.filled_node_pointers() == g["filled_after"]
    assert st["pages_after"] <= st["pages_before"]


def test_gc_keeps_every_root_and_frees_the_rest(orc, hd):
    """Device-built pool (batched passes), several roots kept: the DAG under
    every kept root is unchanged, dropped history is freed, and edits go on
    from the collected pool (the dedup index is rebuilt)."""
    from vkhashdag_gb300 import workloads as W
    res = 512
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 15)  # paged
    ref = orc.OraclePool.from_config(cfg)
    root = pool.edit(hd.NULL, W.sphere_scene(res, 32, seed=1))
    rr = ref.edit(orc.NULL, W.sphere_scene(res, 32, seed=1))
    roots, rroots = [], []
    for k in range(8):
        b = W.mixed_batch(res, 200, seed=40 + k, r_max=40, side_max=80)
        root, rr = pool.edit(root, b), ref.edit(rr, b)
        if k in (2, 7):
            roots.append(root)
            rroots.append(rr)
    q = W.point_queries(res, 1 << 15, seed=3)
    occ_before = [pool.query(r, q) for r in roots]
    used_before = pool.stats()["used_pages"]
    new, st = pool.gc(roots)
    assert st["live_nodes"] > 0 and st["words_after"] < st["words_before"]
    assert pool.stats()["used_pages"] == st["pages_after"] < used_before
    for r, rr_, occ in zip(new, rroots, occ_before):
        assert np.array_equal(pool.query(r, q), occ)
        ok, counts, dig, _ = canonical_of_device(orc, pool, r)
        assert ok and dig == [str(x) for x in ref.canonical(rr_)[2]]
    # editing continues on the collected pool and finds existing nodes
    b = W.mixed_batch(res, 300, seed=99, r_max=40, side_max=80)
    r2 = pool.edit(new[-1], b)
    rr2 = ref.edit(rroots[-1], b)
    ok, counts, dig, _ = canonical_of_device(orc, pool, r2)
    assert ok and dig == [str(x) for x in ref.canonical(rr2)[2]]
    assert pool.edit(new[-1], b) == r2
    # a second collection that keeps every root of the pool keeps every node
    # where it is; dropping the older root frees its exclusive nodes
    occ2 = pool.query(r2, q)
    again, st2 = pool.gc(new + [r2])
    assert st2["words_after"] == st2["words_before"]
    assert again == new + [r2]
    last, st3 = pool.gc([new[-1], r2])
    assert st3["words_after"] < st3["words_before"]
    assert np.array_equal(pool.query(last[1], q), occ2)
    ok, counts, dig, _ = canonical_of_device(orc, pool, last[1])
    assert ok and dig == [str(x) for x in ref.canonical(rr2)[2]]


def test_gc_refuses_a_bad_root_and_leaves_the_pool(orc, hd):
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(128)
    pool = hd.NodePool(cfg, heap_pages=1 << 12)
    root = pool.edit(hd.NULL, W.sphere_scene(128, 8, seed=4))
    wb, pb = cfg.word_bits_per_page, cfg.page_bits_per_bucket
    before = orc.pool_words_digest(*pool.download(), wb, pb)
    leaf = pool.filled_node_pointers()[-1]  # a node, but not of level 0
    for bad in (leaf, root + 1, 0x7FFFFFF0):
        with pytest.raises(hd.HashDagError) as e:
            pool.gc([root, bad])
        assert e.value.status == 1
    assert orc.pool_words_digest(*pool.download(), wb, pb) == before
    assert pool.gc([root])[0][0] != hd.NULL
