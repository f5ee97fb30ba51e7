"""hd_upsert_noalloc -- find-or-insert for callers that cannot allocate.

Callers that have handed the device memory to their own allocator, or that
must not take the device synchronisation of a cudaMalloc, insert nodes through
hd_upsert_noalloc, whose scratch is a static device array of the library.
This checks it against hd_upsert through the C ABI on two calls in a row.
Collected last (file name) so that a failure here cannot hide other results;
it passes alone in a fresh process and after the other tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _nodes(rng, n, level_words):
    """n inner nodes as (packed list for hd_upsert, 8-slot array for the no-alloc call), with repeats."""
    packed, slots = [], np.full((n, 8), 0xFFFFFFFF, np.uint32)
    for i in range(n):
        mask = int(rng.integers(1, 256))
        kids = [int(x) for x in rng.integers(0, level_words, bin(mask).count("1"))]
        if i % 7 == 3:  # repeat an earlier node
            packed.append(packed[i // 2])
            slots[i] = slots[i // 2]
            continue
        packed.append([mask] + kids)
        k = 0
        for c in range(8):
            if (mask >> c) & 1:
                slots[i, c] = kids[k]
                k += 1
    return packed, slots


def _noalloc(hd, pool, level, dev_nodes, n, expect_error=0):
    import torch
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    st = hd.lib().hd_upsert_noalloc(pool.handle, level, ctypes.c_void_p(dev_nodes.data_ptr()), n,
                                    ctypes.c_void_p(out.data_ptr()), None)
    assert st == 0
    torch.cuda.synchronize()
    assert pool.error() == expect_error
    return [int(x) & 0xFFFFFFFF for x in out.cpu().numpy()]


def _slots(nodes):
    """Packed inner nodes (mask, children...) as the call's 8-slot rows."""
    rows = np.full((len(nodes), 8), 0xFFFFFFFF, np.uint32)
    for i, w in enumerate(nodes):
        k = 1
        for c in range(8):
            if (w[0] >> c) & 1:
                rows[i, c] = w[k]
                k += 1
    return rows


def test_noalloc_upsert_matches_upsert(hd):
    import torch
    cfg = hd.DefaultConfig(level_count=8)()
    L = cfg.get_node_levels()
    rng = np.random.default_rng(5)
    packed, slots = _nodes(rng, 3000, 1 << 20)
    leaves = rng.integers(1, 1 << 32, (2000, 2), dtype=np.uint64).astype(np.uint32)
    leaves[5::9] = leaves[1::9][: len(leaves[5::9])]  # repeats
    d_slots = torch.from_numpy(slots.reshape(-1).view(np.int32).copy()).cuda()
    d_leaves = torch.from_numpy(leaves.reshape(-1).view(np.int32).copy()).cuda()

    # existing entry point first, then two no-alloc calls in a row find the same nodes
    pool = hd.NodePool(cfg, heap_pages=1 << 12)
    want = pool.upsert_nodes(2, packed)
    want_leaf = pool.upsert_nodes(L - 1, [list(map(int, x)) for x in leaves])
    for _ in range(2):
        assert _noalloc(hd, pool, 2, d_slots, len(packed)) == want
        assert _noalloc(hd, pool, L - 1, d_leaves, len(leaves)) == want_leaf

    # no-alloc first on a fresh pool (it inserts), twice in a row, then the existing entry point agrees
    fresh = hd.NodePool(cfg, heap_pages=1 << 12)
    got = _noalloc(hd, fresh, 2, d_slots, len(packed))
    assert _noalloc(hd, fresh, 2, d_slots, len(packed)) == got
    assert fresh.upsert_nodes(2, packed) == got
    got_leaf = _noalloc(hd, fresh, L - 1, d_leaves, len(leaves))
    assert _noalloc(hd, fresh, L - 1, d_leaves, len(leaves)) == got_leaf
    assert fresh.upsert_nodes(L - 1, [list(map(int, x)) for x in leaves]) == got_leaf
    assert len(set(got)) == len({tuple(p) for p in packed})


def test_noalloc_rejects_oversized_calls(hd):
    import torch
    cfg = hd.DefaultConfig(level_count=6)()
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    big = torch.zeros(8 * 65537, dtype=torch.int32, device="cuda")
    out = torch.zeros(65537, dtype=torch.int32, device="cuda")
    st = hd.lib().hd_upsert_noalloc(pool.handle, 1, ctypes.c_void_p(big.data_ptr()), 65537,
                                    ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1  # HD_ERR_INVALID_ARG, nothing ran


def test_noalloc_known_answers(golden, hd):
    """The reference's upsert known answers (test/test.cpp:118-147, run through
    the reference's own headers into golden.json), one node per no-alloc call:
    the same pointers and the same pool words as the reference."""
    import hashlib
    import torch
    from helpers import config_from
    k = golden["upsert_kat"]
    cfg = config_from(k["config"])
    L = cfg.get_node_levels()
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    assert pool.filled_node_pointers() == k["filled"]
    ptrs = []
    for level, words in k["ops"]:
        row = np.array(words, np.uint32) if level == L - 1 else _slots([words]).reshape(-1)
        d = torch.from_numpy(row.view(np.int32).copy()).cuda()
        ptrs.append(_noalloc(hd, pool, level, d, 1)[0])
    assert ptrs == k["ptrs"]
    bw, ids, pages = pool.download()
    h = hashlib.sha256()
    for a in (bw, ids, pages):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == k["pool_sha"]


def test_noalloc_failed_call_returns_null_not_stale_pointers(hd):
    """A call that fails inside the kernels (here: an inner node whose 8
    children are all Null, an invalid argument found on the device) reports
    the error through the pool and writes Null for every node, although the
    shared scratch still holds the previous call's results; after the error
    is cleared the same pool serves the next call normally."""
    import torch
    cfg = hd.DefaultConfig(level_count=6)()
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    good = [[0b11, 5, 7], [0b101, 9, 9], [0b1, 3]]
    d_good = torch.from_numpy(_slots(good).reshape(-1).view(np.int32).copy()).cuda()
    want = pool.upsert_nodes(1, good)
    assert _noalloc(hd, pool, 1, d_good, 3) == want
    bad = _slots(good)
    bad[1, :] = 0xFFFFFFFF
    d_bad = torch.from_numpy(bad.reshape(-1).view(np.int32).copy()).cuda()
    assert _noalloc(hd, pool, 1, d_bad, 3, expect_error=1) == [hd.NULL] * 3  # HD_ERR_INVALID_ARG
    pool.clear_error()
    assert _noalloc(hd, pool, 1, d_good, 3) == want


def test_noalloc_zero_leaf_is_stored_like_any_leaf(hd):
    """A leaf of two zero words (only an upsert can make one) is found again
    by the next call and by hd_upsert, between other leaves."""
    import torch
    cfg = hd.DefaultConfig(level_count=6)()
    L = cfg.get_node_levels()
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    leaves = np.array([[0, 0], [5, 6], [0, 0], [7, 0], [0, 0]], np.uint32)
    d = torch.from_numpy(leaves.reshape(-1).view(np.int32).copy()).cuda()
    first = _noalloc(hd, pool, L - 1, d, len(leaves))
    assert first[0] == first[2] == first[4] != hd.NULL and len(set(first)) == 3
    assert _noalloc(hd, pool, L - 1, d, len(leaves)) == first
    assert pool.upsert_nodes(L - 1, [list(map(int, x)) for x in leaves]) == first
