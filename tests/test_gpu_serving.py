"""Serving loop (hd_server_*): continuous batching over resident scenes.

Every request's result must be the same alone and in the mix:
  * edits: the root a merged pass publishes equals applying its requests one
    after another with plain hd_edit calls on the same pool (a fully deduped
    pool gives equal DAGs equal pointers), and the last scene state's
    canonical DAG equals the oracle's sequential result;
  * rays: the hits of a camera request equal hd_trace_pinhole_async alone on
    the root the request recorded (bit-identical records and counters).
"""
import numpy as np
import pytest

from helpers import canonical_of_device

pytestmark = pytest.mark.gpu


def look_at_cameras(hd, positions, target, width, height, fov=np.pi / 3):
    cams = np.zeros(len(positions), hd.CAMERA_DTYPE)
    tg, aspect = np.tan(fov / 2), width / height
    for k, p in enumerate(positions):
        look = np.asarray(target, np.float64) - np.asarray(p, np.float64)
        look /= np.linalg.norm(look)
        side = np.cross(look, [0.0, 1.0, 0.0])
        side /= np.linalg.norm(side)
        up = np.cross(look, side)
        cams[k]["position"] = p
        cams[k]["look"] = look
        cams[k]["side"] = side * tg * aspect
        cams[k]["up"] = up / np.linalg.norm(up) * tg
    return cams


def trace_alone(hd, pool, root, cams, w, h):
    import torch
    n = len(cams) * w * h
    d_out = torch.empty(n * hd.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream()
    pool.trace_pinhole_async(root, cams, w, h, d_out.data_ptr(), d_ctr.data_ptr(), s.cuda_stream)
    s.synchronize()
    return d_out.cpu().numpy().view(hd.HIT_DTYPE), d_ctr.cpu().numpy()[:3].astype(np.uint64)


def make_requests(W, hd, resolutions, n, seed):
    reqs = []
    for i in range(n):
        scene = i % len(resolutions)
        res = resolutions[scene]
        if i % 5 == 4:
            g = W.uniform(seed + i, 61, 3)
            pos = [0.1 + 0.8 * g[0], 0.85, 0.1 + 0.8 * g[1]]
            w, h = 64, 40 + 8 * (i % 3)
            reqs.append(("cam", scene, look_at_cameras(hd, [pos], [0.5, 0.45, 0.5], w, h), w, h))
        else:
            k = int(W.log_uniform_int(seed + i, 62, 1, 1, 48)[0])
            e = W.mixed_batch(res, k, seed=seed * 1000 + i, r_max=max(res // 16, 2), side_max=max(res // 8, 2))
            reqs.append(("edit", scene, e))
    return reqs


def test_serving_results_same_alone_and_in_mix(orc, hd):
    from vkhashdag_gb300 import workloads as W
    resolutions = [256, 512, 1024]
    pools, roots0, refs = [], [], []
    for s, res in enumerate(resolutions):
        cfg = W.config_for_resolution(res)
        pool = hd.NodePool(cfg, heap_pages=1 << 15)
        seed_edits = W.sphere_scene(res, 16, seed=s)
        pools.append(pool)
        roots0.append(pool.edit(hd.NULL, seed_edits))
        refs.append(seed_edits)
    reqs = make_requests(W, hd, resolutions, 120, seed=5)
    srv = hd.Server(list(zip(pools, roots0)), max_pass_edits=256, ray_slots=3)
    ids, outs = [], {}
    srv.pause(True)  # the first 40 requests queue up and must merge on resume
    for k, r in enumerate(reqs):
        if k == 40:
            srv.pause(False)
        if r[0] == "edit":
            ids.append(srv.submit_edits(r[1], r[2]))
        else:
            out = np.zeros(len(r[2]) * r[3] * r[4], hd.HIT_DTYPE)
            rid = srv.submit_camera(r[1], r[2], r[3], r[4], out)
            outs[rid] = out
            ids.append(rid)
    results = [srv.wait(i) for i in ids]
    final_roots = [srv.scene_root(s) for s in range(len(pools))]
    stats = srv.stats()
    srv.close()

    assert all(r["status"] == 0 and r["admitted"] == 1 for r in results), [r for r in results if r["status"]]
    assert stats["max_pass_requests"] > 1  # continuous batching merged requests
    assert stats["edit_requests"] + stats["camera_requests"] == len(reqs)
    assert stats["edit_p99_ms"] >= stats["edit_p50_ms"] > 0

    # edits: replay each scene's requests alone, in submission order
    for s, pool in enumerate(pools):
        mine = [(q, r) for q, r in zip(reqs, results) if q[1] == s and q[0] == "edit"]
        root, published = roots0[s], {roots0[s]}
        for k, (q, r) in enumerate(mine):
            first = k == 0 or mine[k - 1][1]["pass_id"] != r["pass_id"]
            last = k + 1 == len(mine) or mine[k + 1][1]["pass_id"] != r["pass_id"]
            if first:
                assert r["root_in"] == root
            root = pool.edit(root, q[2])
            if last:
                assert r["root"] == root, (s, k, r)
                published.add(root)
        assert final_roots[s] == root
        # camera requests traced a root the scene actually published
        for q, r in zip(reqs, results):
            if q[1] == s and q[0] == "cam":
                assert r["root"] in published
    # the final state of the smallest scene against the oracle's sequential edit
    cfg = pools[0].config
    ref = orc.OraclePool.from_config(cfg)
    rr = ref.edit(orc.NULL, refs[0])
    for q in reqs:
        if q[1] == 0 and q[0] == "edit":
            rr = ref.edit(rr, q[2])
    ok, counts, dig, _ = canonical_of_device(orc, pools[0], final_roots[0])
    assert ok and dig == [str(x) for x in ref.canonical(rr)[2]]

    # rays: the same hits and counters alone
    for q, r in zip(reqs, results):
        if q[0] != "cam":
            continue
        hits, ctr = trace_alone(hd, pools[q[1]], r["root"], q[2], q[3], q[4])
        assert hits.tobytes() == outs[r["id"]].tobytes()
        assert [r["steps"], r["node_words"], r["hits"]] == ctr.tolist()
        assert r["rays"] == len(hits)


def test_serving_admission_refuses_by_free_pages(hd):
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(256)
    pool = hd.NodePool(cfg, heap_pages=256)
    other = hd.NodePool(cfg, heap_pages=1 << 12)
    used0 = pool.stats()["used_pages"]
    e = W.sphere_scene(256, 8, seed=1)
    with hd.Server([(pool, hd.NULL), (other, hd.NULL)], pages_per_edit_hint=1e9) as srv:
        a = srv.submit_edits(0, e)
        b = srv.submit_edits(1, e)
        ra, rb = srv.wait(a), srv.wait(b)
        st = srv.stats()
    # refused before anything ran: status POOL_OOM, admitted 0, root and heap unchanged
    assert ra["status"] == 3 and ra["admitted"] == 0 and ra["root"] == hd.NULL
    assert pool.stats()["used_pages"] == used0
    # the same estimate on a scene whose heap has room for it ... also refused (1e9 pages/edit)
    assert rb["admitted"] == 0
    assert st["refused"] == 2 and st["edit_passes"] == 0
    # with a realistic estimate the request is admitted and runs
    with hd.Server([(other, hd.NULL)], pages_per_edit_hint=0.01) as srv:
        r = srv.wait(srv.submit_edits(0, e))
    assert r["status"] == 0 and r["admitted"] == 1
    assert r["root"] == other.edit(hd.NULL, e)


def test_serving_failed_merged_pass_reruns_each_request_alone(orc, hd):
    """A merged pass that fails (bucket full) is re-run request by request, so
    each request gets the status and root it gets alone."""
    from vkhashdag_gb300 import workloads as W
    cfg = hd.Config(4, 0, [4, 4, 4, 4, 0])  # 16-word buckets, one leaf bucket
    pool = hd.NodePool(cfg, heap_pages=1 << 10)
    r1 = pool.edit(hd.NULL, hd.AABBEditor((4, 4, 4), (6, 6, 6)))
    a = hd.edits_to_array([hd.AABBEditor((8, 8, 8), (10, 10, 10))])    # same leaf pattern: fits
    b = W.sphere_scene(64, 16, seed=3)                                   # overflows the leaf bucket
    c = hd.edits_to_array([hd.AABBEditor((16, 16, 16), (18, 18, 18))])  # fits
    with hd.Server([(pool, r1)]) as srv:
        srv.pause(True)
        ids = [srv.submit_edits(0, x) for x in (a, b, c)]
        srv.pause(False)
        ra, rb, rc = [srv.wait(i) for i in ids]
        final = srv.scene_root(0)
    assert ra["pass_id"] == rb["pass_id"] == rc["pass_id"]  # one merged pass ...
    assert ra["pass_requests"] == rb["pass_requests"] == rc["pass_requests"] == 1  # ... re-run alone
    assert (ra["status"], rb["status"], rc["status"]) == (0, 2, 0)
    assert ra["root_in"] == r1 and rb["root_in"] == ra["root"] and rb["root"] == ra["root"]
    assert rc["root_in"] == ra["root"] and final == rc["root"]
    # alone, on the same pool
    assert pool.edit(r1, a) == ra["root"]
    with pytest.raises(hd.HashDagError) as e:
        pool.edit(ra["root"], b)
    assert e.value.status == 2
    assert pool.edit(ra["root"], c) == rc["root"]
    assert pool.query(rc["root"], [[4, 4, 4], [8, 8, 8], [16, 16, 16], [30, 30, 30]]).tolist() == [1, 1, 1, 0]


def test_serving_pause_drain_and_ids(hd):
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(128)
    pool = hd.NodePool(cfg, heap_pages=1 << 12)
    with hd.Server([(pool, hd.NULL)]) as srv:
        srv.pause(True)
        i = srv.submit_edits(0, W.sphere_scene(128, 4, seed=2))
        assert srv.wait(i, timeout_ms=50) is None  # nothing starts while paused
        with pytest.raises(hd.HashDagError):
            srv.drain()  # refused while paused with work queued
        srv.pause(False)
        srv.drain()
        r = srv.wait(i)
        assert r["status"] == 0 and r["root"] != hd.NULL
        with pytest.raises(hd.HashDagError):
            srv.wait(i)  # a result is handed out once
        z = srv.wait(srv.submit_edits(0, np.zeros(0, hd.EDIT_DTYPE)))
        assert z["status"] == 0 and z["root"] == r["root"]


def test_serving_collects_when_memory_runs_low(orc, hd):
    """With gc_free_fraction set the server collects a scene whose heap runs
    low, so memory frees up and requests keep being admitted; the scene ends
    with the same DAG as applying every request alone, in order."""
    from vkhashdag_gb300 import workloads as W
    res = 256
    # few, deep buckets (16 pages of 512 words each): pages fill up, so the
    # replaced history, not one page per touched bucket, decides the heap size
    cfg = hd.Config(9, 4, [3, 3, 4, 5, 7, 7, 4])
    reqs = [W.mixed_batch(res, 40, seed=500 + k, r_max=30, side_max=60) for k in range(80)]
    # sizes: every request alone on a roomy pool
    big = hd.NodePool(cfg, heap_pages=1 << 14)
    r = big.edit(hd.NULL, W.sphere_scene(res, 16, seed=0))
    used, grow = [big.stats()["used_pages"]], []
    for e in reqs:
        r = big.edit(r, e)
        used.append(big.stats()["used_pages"])
        grow.append(used[-1] - used[-2])
    (r_final,), st = big.gc([r])
    heap = st["pages_after"] + 4 * max(grow) + 16
    assert heap < used[-1]  # without collection the history does not fit
    ref = orc.OraclePool.from_config(cfg)
    rr = ref.edit(orc.NULL, W.sphere_scene(res, 16, seed=0))
    for e in reqs:
        rr = ref.edit(rr, e)
    want = [str(x) for x in ref.canonical(rr)[2]]

    def serve(gc_fraction):
        pool = hd.NodePool(cfg, heap_pages=heap)
        r0 = pool.edit(hd.NULL, W.sphere_scene(res, 16, seed=0))
        # passes of at most 4 requests: a pass never needs more than the heap
        # keeps free after a collection (4 x the largest growth of one request)
        with hd.Server([(pool, r0)], reserve_pages=1, pages_per_edit_hint=max(grow) / 40.0, max_pass_edits=160,
                       gc_free_fraction=gc_fraction) as srv:
            ids = [srv.submit_edits(0, e) for e in reqs]
            results = [srv.wait(i) for i in ids]
            stats = srv.stats()
            final = srv.scene_root(0)
        return pool, final, results, stats

    pool, final, results, stats = serve(0.0)
    assert stats["refused"] + stats["failed"] > 0 and stats["gc_runs"] == 0
    pool, final, results, stats = serve(0.3)
    assert stats["refused"] == 0 and stats["failed"] == 0 and stats["gc_runs"] > 0
    assert all(x["status"] == 0 for x in results)
    assert max(x["gc_epoch"] for x in results) > 0
    ok, counts, dig, _ = canonical_of_device(orc, pool, final)
    assert ok and dig == want
