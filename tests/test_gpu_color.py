"""Colour (VBR) editing on the device: hd_vbr_edit, hd_color_fetch.

Parity: the colour octree words (nodes and VBR leaf chunks), the colour root
and the colours fetched for seeded voxels equal the reference's
VBREditorWrapper run by its single-threaded NodePoolBase::Edit (golden
digests made by the reference itself, tests/golden/make_golden.py), and the
oracle's restatement on fresh cases.  The DAG pointers of a device pool come
from concurrent inserts, so the DAG is compared canonically; the colour words
hold no DAG pointers and must match word for word.
"""
import numpy as np
import pytest

from helpers import canonical_of_device, colors_sha, oracle_vbr_run, sha, vbr_case, vbr_case_inputs

pytestmark = pytest.mark.gpu

VBR_NAMES = ["vbr_256_leaf3", "vbr_128_leaf5_history", "vbr_512_leaf2", "vbr_128_leaf0"]


def device_run(hd, g, paged, per_call=1):
    cfg, v, q = vbr_case_inputs(g)
    heap = cfg.get_total_pages() - (1 if paged else 0)  # one page short of the total: paged heap
    pool = hd.NodePool(cfg, heap_pages=heap)
    cp = hd.DAGColorPool(pool, g["leaf_level"], g["keep_history"])
    root, croot = hd.NULL, hd.DAGColorPool.NULL
    for i in range(0, len(v), per_call):
        root, croot = pool.vbr_edit(root, cp, croot, v[i:i + per_call])
    return pool, cp, root, croot, q


@pytest.mark.parametrize("name", VBR_NAMES)
@pytest.mark.parametrize("paged", [False, True])
def test_vbr_colour_pool_word_identical_to_reference(golden, orc, hd, name, paged):
    g = vbr_case(golden, name)
    pool, cp, root, croot, q = device_run(hd, g, paged)
    assert croot == g["color_root"]
    nodes, leaves = cp.read()
    assert len(nodes) == g["n_nodes"] and sha(nodes) == g["nodes_sha"]
    assert len(leaves) == g["n_leaf_words"] and sha(leaves) == g["leaves_sha"]
    c = cp.fetch(croot, q)
    assert colors_sha(c) == g["colors_sha"]
    # the geometry is the reference's DAG (canonically)
    opool, ocp, oroot, ocroot, _ = oracle_vbr_run(orc, g)
    ok, counts, dig, _ = canonical_of_device(orc, pool, root)
    assert ok and dig == [str(x) for x in opool.canonical(oroot)[2]]


def test_vbr_all_edits_in_one_call_equal_one_call_per_edit(golden, hd):
    g = vbr_case(golden, "vbr_256_leaf3")
    _, cp1, _, c1, q = device_run(hd, g, False, per_call=1)
    _, cp2, _, c2, _ = device_run(hd, g, False, per_call=1000)
    assert c1 == c2
    n1, l1 = cp1.read()
    n2, l2 = cp2.read()
    assert np.array_equal(n1, n2) and np.array_equal(l1, l2)


def test_vbr_larger_case_matches_oracle(orc, hd):
    """1024^3 world, colour leaves of 64^3 (16 macro blocks), weighted colours,
    paints, digs: the device pool equals the oracle's word for word."""
    from vkhashdag_gb300 import workloads as W, OP_DIG, OP_PAINT
    res, leaf_level = 1024, 4
    cfg = W.serving_config(res)
    v = W.vbr_edits(res, 40, seed=91, r_max=200, side_max=400, weighted_frac=0.4)
    pool = hd.NodePool(cfg, heap_pages=cfg.get_total_pages())
    cp = hd.DAGColorPool(pool, leaf_level)
    root, croot = pool.vbr_edit(hd.NULL, cp, hd.DAGColorPool.NULL, v)
    opool = orc.OraclePool.from_config(cfg)
    ocp = orc.OracleColorPool(leaf_level)
    oroot, ocroot = orc.NULL, orc.OracleColorPool.NULL
    for e in v:
        op = int(e["edit"]["op"])
        if op == OP_DIG:
            oroot = opool.edit(oroot, np.asarray([e["edit"]]))
        else:
            oroot, ocroot = opool.vbr_edit(oroot, ocp, ocroot, e["edit"], 2 if op == OP_PAINT else 1,
                                           int(e["colors"]), int(e["weight"]), int(e["bits_per_weight"]))
    assert croot == ocroot
    nodes, leaves = cp.read()
    assert np.array_equal(nodes, ocp.nodes()) and np.array_equal(leaves, ocp.leaves())
    q = W.point_queries(res, 1 << 15, seed=5)
    c, oc = cp.fetch(croot, q), opool.color_fetch(ocp, ocroot, q)
    assert np.array_equal(c["colors"], oc["colors"]) and np.array_equal(c["weight"], oc["weight"])
    assert np.array_equal(c["rgb"].view(np.uint32), oc["rgb"].view(np.uint32))
    ok, counts, dig, _ = canonical_of_device(orc, pool, root)
    assert ok and dig == [str(x) for x in opool.canonical(oroot)[2]]


def test_vbr_fetch_of_an_empty_octree(hd):
    from vkhashdag_gb300 import workloads as W
    cfg = W.serving_config(128)
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    cp = hd.DAGColorPool(pool, 3)
    c = cp.fetch(hd.DAGColorPool.NULL, W.point_queries(128, 100, seed=1))
    assert not c["has_value"].any() and not c["colors"].any() and not c["rgb"].any()


def test_vbr_octree_full_is_reported_and_keeps_the_colours(hd):
    from vkhashdag_gb300 import workloads as W
    cfg = W.serving_config(256)
    pool = hd.NodePool(cfg, heap_pages=cfg.get_total_pages())
    cp = hd.DAGColorPool(pool, 3, max_nodes=4, max_leaf_words=1 << 20)
    v = W.vbr_edits(256, 30, seed=7, r_max=60, side_max=120)
    root, croot = hd.NULL, hd.DAGColorPool.NULL
    with pytest.raises(hd.HashDagError) as e:
        for i in range(len(v)):
            before = cp.read()
            root, croot = pool.vbr_edit(root, cp, croot, v[i:i + 1])
    assert e.value.status == 3  # HD_ERR_POOL_OOM
    after = cp.read()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])


def test_vbr_rejects_bad_colours(hd):
    from vkhashdag_gb300 import workloads as W
    cfg = W.serving_config(128)
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    cp = hd.DAGColorPool(pool, 3)
    v = W.vbr_edits(128, 1, seed=3)
    v["bits_per_weight"] = 2
    v["weight"] = 4  # >= 2^bits
    with pytest.raises(hd.HashDagError):
        pool.vbr_edit(hd.NULL, cp, hd.DAGColorPool.NULL, v)
    with pytest.raises(hd.HashDagError):
        hd.DAGColorPool(pool, cfg.get_node_levels())  # leaf level below the DAG leaves


def test_vbr_sphere_touching_a_node_boundary(orc, hd):
    """A sphere of radius 1 centred one voxel past a node boundary: the
    reference's conservative classification (distance to the node's exclusive
    upper bound) makes it proceed into the node before the boundary too."""
    from vkhashdag_gb300 import workloads as W, VBR_EDIT_DTYPE, SHAPE_SPHERE, OP_FILL
    res = 128
    cfg = W.config_for_resolution(res)
    scene = W.sphere_scene(res, 16, seed=0)
    pool = hd.NodePool(cfg, heap_pages=1 << 12)
    root = pool.edit(hd.NULL, scene)
    opool = orc.OraclePool.from_config(cfg)
    oroot = opool.edit(orc.NULL, scene)
    v = np.zeros(3, VBR_EDIT_DTYPE)
    v["edit"]["shape"] = SHAPE_SPHERE
    v["edit"]["op"] = OP_FILL
    v["edit"]["p0"] = [(48, 65, 123), (64, 64, 64), (31, 96, 33)]
    v["edit"]["r2"] = [1, 1, 4]
    v["colors"] = [0x102030, 0x405060, 0x708090]
    cp = hd.DAGColorPool(pool, 3)
    r, c = pool.vbr_edit(root, cp, hd.DAGColorPool.NULL, v)
    ocp = orc.OracleColorPool(3)
    oc = orc.OracleColorPool.NULL
    for e in v:
        oroot, oc = opool.vbr_edit(oroot, ocp, oc, e["edit"], 1, int(e["colors"]))
    nodes, leaves = cp.read()
    assert c == oc and np.array_equal(nodes, ocp.nodes()) and np.array_equal(leaves, ocp.leaves())


def test_vbr_node_pool_closes_its_colour_pools_first(hd):
    """Closing (or collecting) a node pool first closes its colour pools, so
    no colour pool outlives the node pool it reads; later calls see no stale
    CUDA error."""
    from vkhashdag_gb300 import workloads as W
    cfg = W.serving_config(128)
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    cp = hd.DAGColorPool(pool, 3)
    pool.close()
    assert cp._h is None
    cp.close()
    p2 = hd.NodePool(cfg, heap_pages=cfg.get_total_pages())
    assert p2.edit(hd.NULL, W.sphere_scene(128, 2, seed=1)) != hd.NULL
