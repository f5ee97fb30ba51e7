#!/usr/bin/env python3
"""Benchmark of the HashDAG edit path on one GB300 (or N replicas).

A step applies one batch of 65,536 mixed edits (70 % spheres with radius
log-uniform in [1,512], 30 % boxes with sides log-uniform in [1,1024], 50/50
fill/dig, seed order) to a 32768^3 DAG seeded with the sphere scene scaled x32
(one r=9600 sphere fill, 64 sphere digs with r in [512,2048]).  Every step
first rolls the pool back to the seeded state (stream-ordered device copies,
inside the timed region) and then runs one batched level-synchronous pass, so
every step inserts its nodes afresh.  Metric: voxel-edits/s, where a batch's
voxel-edits = sum over its edits of the grid voxels inside the shape.

  value      device-resident edits, CUDA events on the pass's stream
  e2e        the public C-ABI call hd_edit() with host edits (H2D copy of the
             edit array and D2H of root/status inside the timed region)
  per_edit   the plain form on the same edit list: one pass per edit
  roofline   the dedup pass (k_dedup over all levels) against the
             measured HBM copy bandwidth; beside it the pass's DRAM rate
             against the measured rate of independent random 8-byte reads
             (random_access), the ceiling of a random-access kernel
  cpu_baseline  the CPU restatement of the reference's threaded edit
             (oracle, OpenMP on all host cores) on a bounded sample

--impl reference times that CPU editor alone (all host cores) on the same
workload and prints the same JSON line with "impl": "reference".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

RES = 32768
BUCKET_BITS = [10, 10, 10, 10, 10, 12, 14, 15, 16, 17, 17, 18, 18, 15]
N_EDITS = 65536
METRIC = "voxel-edits/s batched vs per-edit on 1 GB300 (bit-exact DAG); p99 edit latency"


def _profile_value(name, key, scale=1.0):
    """A figure from a committed ncu summary (profiles/*.json), times scale; None if absent."""
    try:
        with open(os.path.join(HERE, "profiles", name)) as f:
            return float(json.load(f)[key]) * scale
    except Exception:
        return None


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def random_access_ceiling(device, table_log2=31, reads_log2=27, reps=5):
    """Sustained rate of independent random 8-byte reads over a 16 GB table
    (a library gather, used only as a measuring stick): the ceiling of a kernel
    whose every access is a random DRAM sector.  Returns reads/s and the
    sector bytes/s (32 B per read) moved."""
    import torch
    table = torch.empty(1 << table_log2, dtype=torch.int64, device=device)
    idx = torch.randint(0, 1 << table_log2, (1 << reads_log2,), device=device)
    torch.take(table, idx)
    torch.cuda.synchronize(device)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = None
    for _ in range(reps):
        a.record()
        torch.take(table, idx)
        b.record()
        b.synchronize()
        ms = a.elapsed_time(b)
        best = ms if best is None or ms < best else best
    del table, idx
    torch.cuda.empty_cache()
    reads = (1 << reads_log2) / (best / 1e3)
    return {"reads_per_s": reads, "sector_gbs": 32.0 * reads / 1e9, "table_gb": 8.0 * (1 << table_log2) / 1e9}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def build_if_needed():
    import vkhashdag_gb300
    if not os.path.exists(vkhashdag_gb300.library_path):
        from vkhashdag_gb300 import _build
        _build.build()


def bench_config():
    from vkhashdag_gb300 import Config
    return Config(9, 2, list(BUCKET_BITS))


def workload(rank, n_batches, n_edits, res):
    from vkhashdag_gb300 import workloads as W
    base = W.sphere_scene(res, 64, seed=0)
    from vkhashdag_gb300.replicas import replica_seed
    batches = [W.mixed_batch(res, n_edits, seed=replica_seed(rank, k)) for k in range(n_batches)]
    return base, batches


# ---------------------------------------------------------------------- CPU (oracle) timing
def cpu_sample_rate(orc_pool, root, edits, res, budget_s, threads, max_task_level, serial=False):
    """Threaded CPU editor (or the serial one) over a growing prefix of `edits`
    until budget_s is spent.  Returns (voxel-edits/s, edits applied, seconds,
    root after them)."""
    import oracle
    done, t_used, ve = 0, 0.0, 0
    r = root
    chunk = 8
    while done < len(edits) and t_used < budget_s:
        e = edits[done:done + chunk]
        t0 = time.perf_counter()
        r = orc_pool.edit(r, e) if serial else orc_pool.threaded_edit(r, e, max_task_level, threads)
        t_used += time.perf_counter() - t0
        ve += oracle.count_voxel_edits(e, res)
        done += len(e)
        chunk = min(chunk * 2, 256)
    return ve / t_used, done, t_used, r


def cpu_model():
    """The host CPU's model name (x86 /proc/cpuinfo, else lscpu: Arm cores)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def serial_baseline(orc_pool, root, edits, res, budget_s):
    """The reference's serial NodePoolBase::Edit (restated), one thread, for
    budget_s seconds."""
    rate, n_done, t_used, _ = cpu_sample_rate(orc_pool, root, edits, res, budget_s, 1, 0, serial=True)
    return {"value": rate, "unit": "voxel-edits/s", "cores": 1,
            "sample": f"first {n_done} edits, one Edit each ({t_used:.1f} s)"}


def replica_seed_of(rank, batch):
    from vkhashdag_gb300.replicas import replica_seed
    return replica_seed(rank, batch)


def leaf_roofline(counters, work, L, n_edits, leaf_ms, hbm, peak_kind):
    """Roofline of the level-(L-2) leaf kernels (k_leafparent_compact/_long)
    from the pass's own work counters.  Algorithmic bytes: per level-(L-2) node
    its item record (24 B: position, base, list offset and length, parent
    slot), per (node, edit) pair 4 B (a one-edit node's leaf classes, else the
    pair's list entry), the base node's words, every
    old leaf read (8 B), per changed leaf its index slot (8 B) and, when found,
    the resident leaf (8 B); per read-only lookup of a level-(L-2) node whose
    children are all known, its index slot (8 B) and one resident copy (the
    level's mean candidate words, 4 B each); written: each new leaf candidate
    (12 B), each unresolved node's todo record (72 B) or each resolved node's
    parent slot (4 B); and every edit descriptor once (40 B)."""
    nodes, pairs = work["nodes"], work["pairs"]
    cand_leaf = int(counters["items"][L - 1])
    todo = int(counters["candidates"][L - 2]) if L >= 2 else 0
    found = max(0, work["lookups"] - cand_leaf)
    node_words = float(counters["candidate_words"][L - 2]) / max(1.0, float(counters["candidates"][L - 2])) if L >= 2 \
        else 0.0
    alg = (24 * nodes + 4 * pairs + 4 * work["base_words"] + 8 * work["old_leaves"] + 8 * work["lookups"] +
           8 * found + (8 + 4 * node_words) * work["inner_lookups"] + 12 * cand_leaf + 72 * todo +
           4 * max(0, nodes - todo) + 40 * n_edits)
    achieved = alg / (leaf_ms / 1e3) / 1e9
    return {"bound": "hbm", "kernel": "leaf kernels (k_leafparent_compact/_long)", "achieved": achieved, "peak": hbm,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm, "algorithmic_bytes_per_step": float(alg),
            "leaf_ms_per_step": leaf_ms, "work_last_step": work,
            "leaf_edit_evaluations_per_s": 8.0 * pairs / (leaf_ms / 1e3),
            "issue_efficiency": _profile_value("leaf_issue.json", "active_lanes_per_inst", 1.0 / 32.0),
            "note": "integer voxel-mask work (a warp's partly covered leaves compacted onto its lanes), not DRAM "
                    "bound; issue_efficiency = active lanes per issued instruction / 32 from the committed ncu "
                    "capture"}


def batched_config(cfg, res, n_edits, ve_per_step, world):
    """The `config` of the batched workload; both arms print this same object."""
    return {"workload": f"batched-{n_edits}-mixed-edits-{res}^3", "resolution": res, "edits_per_step": n_edits,
            "voxel_edits_per_step": float(ve_per_step),
            "seeded_scene": "sphere r=9600 fill + 64 sphere digs r in [512,2048] (1024^3 scene x32)",
            "node_levels": cfg.get_node_levels(), "bucket_bits": list(cfg.bucket_bits_each_level),
            "word_bits_per_page": cfg.word_bits_per_page, "page_bits_per_bucket": cfg.page_bits_per_bucket,
            "rollback_to_seeded_scene_each_step": True,
            "l2": "working set of a step (pool + frontier, tens of GB) far above L2; no flush",
            "parallelism": f"replicas x{world}"}


def sequential_oracle_leg(cfg, base, batch, res, threads, budget_s, serial_batch, queries):
    """The CPU leg of the batched benchmark, on the oracle alone (all host
    threads): it builds the seeded scene itself, times the first budget_s of
    the batch with the threaded editor (NodePoolThreadedEdit::ThreadedEdit
    restated: the reference's sequential semantics, edits in seed order), then
    applies the rest of the batch and returns the canonical DAG and point
    occupancy of the result beside the CPU rates."""
    import oracle
    L = cfg.get_node_levels()
    mtl = max(0, L - 4)
    opool = oracle.OraclePool.from_config(cfg)
    t0 = time.perf_counter()
    r0 = opool.threaded_edit(oracle.NULL, base, mtl, threads)
    t_scene = time.perf_counter() - t0
    rate, n_done, t_used, r = cpu_sample_rate(opool, r0, batch, res, budget_s, threads, mtl)
    t0 = time.perf_counter()
    if n_done < len(batch):
        r = opool.threaded_edit(r, batch[n_done:], mtl, threads)
    t_rest = time.perf_counter() - t0
    serial = serial_baseline(opool, r0, serial_batch, res, budget_s / 3)
    t0 = time.perf_counter()
    ok, counts, digests = opool.canonical(r)
    occ = opool.query(r, queries)
    t_canon = time.perf_counter() - t0
    pool_ok = opool.ok
    del opool
    cpu = {"value": rate, "unit": "voxel-edits/s", "cores": threads, "kind": "port",
           "sample": f"first {n_done} edits of the last timed batch, one ThreadedEdit each ({t_used:.1f} s of CPU "
                     f"time), on the seeded scene the CPU editor built itself ({t_scene:.1f} s, untimed)",
           "cpu_model": cpu_model(), "max_task_level": mtl, "serial": serial}
    ref = {"ok": bool(ok and pool_ok), "counts": counts, "digests": digests, "occupancy": occ,
           "seconds": {"scene": t_scene, "batch": t_used + t_rest, "canonical_and_queries": t_canon}}
    return cpu, ref


def bucket_scan_figures(cfg, bucket_words, counters, levels):
    """What the reference's linear bucket scan (NodePool.hpp:79-132) would read
    per candidate at the given levels of the pool after a step: the mean
    bucket fill in words, and the words a scan reads per candidate (a new node
    scans its whole bucket, a found one half of it on average)."""
    bases = cfg.get_level_base_bucket_indices()
    out = {}
    for l in levels:
        nb = cfg.get_buckets_at_level(l)
        w = np.asarray(bucket_words[bases[l]:bases[l] + nb], np.float64)
        cand, ins = float(counters["candidates"][l]), float(counters["inserted"][l])
        mean = float(w.mean())
        scan = (ins * mean + (cand - ins) * mean / 2) / max(1.0, cand)
        out[f"l{l}"] = {"buckets": nb, "mean_bucket_words": mean, "max_bucket_words": int(w.max()),
                        "scan_words_per_candidate": scan,
                        "candidate_words": float(counters["candidate_words"][l]) / max(1.0, cand)}
    return out


def device_canonical(cfg, snapshot, filled, root):
    """Canonical DAG of a device pool snapshot (downloaded words) under root,
    by the oracle's canonicaliser."""
    import oracle
    mirror = oracle.OraclePool.from_config(cfg)
    mirror.load(*snapshot, filled)
    ok, counts, digests = mirror.canonical(root)
    del mirror
    return ok, counts, digests


def run_reference(args):
    """--impl reference: the CPU restatement of the reference's threaded editor
    (the oracle, OpenMP on all host threads) on the same workload, bounded
    samples per step.  Nothing of the engine runs here: the edits come from the
    seeded generators (numpy), voxel-edits are counted by the oracle, and the
    engine's library is never loaded."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    import oracle
    oracle.build()
    if args.resolution == RES:
        cfg = bench_config()
    else:
        from vkhashdag_gb300 import workloads as W
        cfg = W.config_for_resolution(args.resolution, bottom_bits=16, top_levels=6)
    L = cfg.get_node_levels()
    threads = os.cpu_count() or 1
    mtl = max(0, L - 4)
    t_start = time.perf_counter()

    def phase(what):
        print(f"[reference] {what}: {time.perf_counter() - t_start:.1f} s", file=sys.stderr, flush=True)

    base, batches = workload(0, args.warmup + args.steps + 1, args.n_edits, args.resolution)
    serial_batch = batches.pop()  # edits no step applies: the serial editor's sample
    ve_timed = [oracle.count_voxel_edits(b, args.resolution) for b in batches[args.warmup:]]
    phase("workload and voxel-edit counts")
    pool = oracle.OraclePool.from_config(cfg)
    t0 = time.perf_counter()
    root0 = pool.threaded_edit(oracle.NULL, base, mtl, threads)
    t_base = time.perf_counter() - t0
    phase(f"seeded scene on {threads} threads")
    rates, samples = [], []
    for k in range(args.warmup + args.steps):
        rate, n_done, t_used, _ = cpu_sample_rate(pool, root0, batches[k], args.resolution, args.ref_step_seconds,
                                                 threads, mtl)
        phase(f"step {k}: {n_done} edits in {t_used:.1f} s")
        if k >= args.warmup:
            rates.append(rate)
            samples.append((n_done, t_used))
    value = float(np.mean(rates))
    n_done = sum(s[0] for s in samples)
    t_all = sum(s[1] for s in samples)
    serial = serial_baseline(pool, root0, serial_batch, args.resolution, args.ref_step_seconds)
    phase("serial sample")
    sample = (f"first {n_done // max(1, len(samples))} edits (on average) of each of {args.steps} batches of "
              f"{args.n_edits}, applied one by one by the threaded CPU editor to the seeded {args.resolution}^3 scene "
              f"(scene build {t_base:.1f} s untimed)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "voxel-edits/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_all / max(1, len(samples)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": batched_config(cfg, args.resolution, args.n_edits, float(np.mean(ve_timed)), world),
        "cpu_baseline": {"value": value, "unit": "voxel-edits/s", "cores": threads, "kind": "port", "sample": sample,
                         "cpu_model": cpu_model(), "max_task_level": mtl, "serial": serial},
        "e2e": {"value": value, "unit": "voxel-edits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- GPU arm
def run_ours(args):
    world, rank, local = dist_setup()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build_if_needed()
    import vkhashdag_gb300 as hd

    from vkhashdag_gb300 import workloads as W
    res, n_edits = args.resolution, args.n_edits
    cfg = bench_config() if res == RES else W.config_for_resolution(res, bottom_bits=16, top_levels=6)
    L = cfg.get_node_levels()
    heap_pages = min(cfg.get_total_pages(), args.heap_pages)
    n_batches = args.warmup + args.steps
    base, batches = workload(rank, n_batches, n_edits, res)
    ve = [hd.count_voxel_edits(b, res) for b in batches]

    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    pool = hd.NodePool(cfg, heap_pages=heap_pages, index_log2=args.index_log2, device=local)
    root0 = pool.edit(hd.NULL, base)
    # launch shape from the autotuner, on the first warm-up batch (the pool ends
    # unchanged); the timed batches are different ones
    tuning = None
    if not args.no_tune:
        try:
            tuning = pool.autotune(root0, batches[0])
        except hd.HashDagError as e:
            tuning = {"error": str(e)}
    pool.checkpoint()
    d_batches = [torch.from_numpy(b.view(np.uint8).copy()).to(f"cuda:{local}") for b in batches]
    d_out = torch.zeros(n_batches, dtype=torch.int32, device=f"cuda:{local}")
    # size the edit workspace on every batch (sync path grows it), then restore
    for b in batches:
        pool.edit(root0, b)
        pool.rollback(0)
    torch.cuda.synchronize()

    def step(k):
        pool.rollback(sp)
        pool.edit_async(root0, d_batches[k].data_ptr(), n_edits, d_out[k:k + 1].data_ptr(), sp)

    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            step(k)
    torch.cuda.synchronize()
    if pool.error():
        raise RuntimeError(f"device error {pool.error()} during warm-up")

    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = pool.kernel_launches()
    pool.profile_begin(args.steps)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for k in range(args.warmup, n_batches):
            step(k)
        end.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    elapsed_ms = start.elapsed_time(end)
    launches = pool.kernel_launches() - launches0
    phases, npass = pool.profile_end()
    err = pool.error()
    if err:
        raise RuntimeError(f"device error {err} in the timed region")
    counters = pool.last_counters_full()
    probe_stats = pool.last_probe_stats()
    leaf_work = pool.last_leaf_work()
    last_root = int(d_out[n_batches - 1].item()) & 0xFFFFFFFF
    # the timed result itself, for the check against the sequential CPU editor
    # at the end (outside every timed region): the pool's words and 2^20 point
    # queries under the last timed batch's root
    queries = W.point_queries(res, 1 << 20, seed=7)
    snapshot, dev_occ = None, None
    if rank == 0 and not args.no_cpu:
        snapshot = pool.download()
        dev_occ = pool.query(last_root, queries)
    # self-check: re-running the last batch on the same pool finds every node it
    # inserted, so the synchronous path must return the very same root
    same_roots = pool.edit(root0, batches[n_batches - 1]) == last_root
    from vkhashdag_gb300.replicas import replica_totals
    elapsed_ms, total_ve = replica_totals(elapsed_ms, float(sum(ve[args.warmup:])), device=f"cuda:{local}")
    value = total_ve / (elapsed_ms / 1e3)

    # ---------------- e2e through the public call with host buffers
    e2e_times = []
    for k in range(args.warmup, n_batches):
        pool.rollback(0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pool.edit(root0, batches[k])
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = sum(ve[args.warmup:]) / sum(e2e_times)

    # ---------------- plain form against one batched pass, on the same edit list
    plain = np.ascontiguousarray(batches[args.warmup][: args.per_edit])
    plain_ve = hd.count_voxel_edits(plain, res)
    d_plain = torch.from_numpy(plain.view(np.uint8).copy()).to(f"cuda:{local}")
    d_root = torch.zeros(1, dtype=torch.int32, device=f"cuda:{local}")
    d_root0 = torch.full((1,), root0 if root0 < (1 << 31) else root0 - (1 << 32), dtype=torch.int32,
                         device=f"cuda:{local}")
    # Every form runs on the seeded scene restored by a rollback, and each
    # result is checked in its own pool state: re-running the other form there
    # finds every node of the same DAG, so it must return the very same root
    # (pointers from different rollbacks differ: insertion order does).
    def plain_chain(start):
        r = start
        for k in range(len(plain)):
            r = pool.edit(r, plain[k:k + 1])
        return r

    # (1) wall latency of hd_edit, one call per edit (host edits, host root)
    pool.rollback(0)
    torch.cuda.synchronize()
    lat = []
    r = root0
    for k in range(len(plain)):
        t0 = time.perf_counter()
        r = pool.edit(r, plain[k:k + 1])
        lat.append(time.perf_counter() - t0)
    same = [pool.edit(root0, plain) == r]
    lat_ms = np.array(lat) * 1e3
    plain_wall_s = float(lat_ms.sum()) / 1e3
    # (2) device time of the same passes back to back on the stream: the root
    # stays on the device, the host copies of the edits size every launch as
    # hd_edit does (grids from bounding boxes, small passes as one CTA)
    pool.rollback(0)
    torch.cuda.synchronize()
    s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    d_root.copy_(d_root0)
    torch.cuda.synchronize()
    s2.record(stream)
    for k in range(len(plain)):
        pool.edit_async_droot_hinted(d_root.data_ptr(), d_plain.data_ptr() + 40 * k, plain[k:k + 1],
                                     d_root.data_ptr(), sp)
    e2.record(stream)
    torch.cuda.synchronize()
    plain_dev_ms = s2.elapsed_time(e2)
    same.append(pool.edit(root0, plain) == (int(d_root.item()) & 0xFFFFFFFF))
    # (3) the same edits as ONE batched pass: device time and hd_edit wall time
    pool.rollback(0)
    d_root.copy_(d_root0)
    torch.cuda.synchronize()
    s2.record(stream)
    pool.edit_async_droot_hinted(d_root.data_ptr(), d_plain.data_ptr(), plain, d_root.data_ptr(), sp)
    e2.record(stream)
    torch.cuda.synchronize()
    batched_dev_ms = s2.elapsed_time(e2)
    same.append(plain_chain(root0) == (int(d_root.item()) & 0xFFFFFFFF))
    bw_times = []
    for _ in range(3):
        pool.rollback(0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batched_root = pool.edit(root0, plain)
        bw_times.append(time.perf_counter() - t0)
    batched_wall_s = float(np.median(bw_times))
    same.append(plain_chain(root0) == batched_root)
    plain_same = all(same)
    if pool.error():
        raise RuntimeError(f"device error {pool.error()} in the plain/batched comparison")

    # ---------------- roofline of the dedup pass
    hbm, peak_kind = peaks()
    ceiling = None
    if rank == 0 and not args.no_ceiling:
        try:
            ceiling = random_access_ceiling(torch.device("cuda", local))
        except RuntimeError:  # no room for the 16 GB table beside the pool
            ceiling = None
    per_step_dedup_ms = float(sum(phases[2:2 + L])) / max(1, npass)
    cw, c, iw = counters["candidate_words"], counters["candidates"], counters["inserted_words"]
    dedup_bytes = float(8 * cw.sum() + 8 * c.sum() + 4 * iw.sum())
    achieved = dedup_bytes / (per_step_dedup_ms / 1e3) / 1e9
    phase_ms = {"root+expand": float(phases[0]) / npass, "leaf_voxels": float(phases[1]) / npass}
    for k in range(L):
        lvl = L - 1 - k
        phase_ms[f"dedup_l{lvl}"] = float(phases[2 + k]) / npass
    phase_ms["finish"] = float(phases[-1]) / npass
    # DRAM bytes of the dedup pass per step, from the committed ncu summary of a
    # smaller case scaled to this workload (only meaningful for the default one)
    traffic = _profile_value("dedup_traffic.json", "bytes_per_step") if (res, n_edits) == (RES, N_EDITS) else None
    leaf_roof = leaf_roofline(counters, leaf_work, L, n_edits, float(phases[1]) / npass, hbm, peak_kind)

    # ---------------- CPU leg (rank 0): the oracle's threaded editor on the
    # host cores, timed on a bounded sample of the last timed batch and then
    # run to the end of that batch; its canonical DAG must equal the device's
    cpu, checks = None, {"rerun_of_last_batch_finds_same_root": bool(same_roots)}
    bucket_scan = None
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        cpu, ref = sequential_oracle_leg(cfg, base, batches[n_batches - 1], res, threads, args.cpu_seconds,
                                         batches[args.warmup], queries)
        bucket_scan = bucket_scan_figures(cfg, snapshot[0], counters, [L - 4, L - 3, L - 2, L - 1])
        t0 = time.perf_counter()
        dok, dcounts, ddigests = device_canonical(cfg, snapshot, pool.filled_node_pointers(), last_root)
        t_dev_canon = time.perf_counter() - t0
        del snapshot
        equal = bool(ref["ok"] and dok and dcounts == ref["counts"] and ddigests == ref["digests"])
        checks["canonical_equal_sequential_oracle"] = equal
        checks["point_queries_equal_sequential_oracle"] = bool(np.array_equal(dev_occ, ref["occupancy"]))
        checks["sequential_oracle"] = {
            "what": f"the last timed batch ({n_edits} edits) applied in seed order by the oracle's threaded editor "
                    f"to the seeded scene it built itself; canonical DAG (per level, the sorted unique node tuples "
                    f"with child pointers renumbered) and {len(queries)} seeded point queries against the device's "
                    f"result of the timed step",
            "batch_seed": int(replica_seed_of(rank, n_batches - 1)),
            "canonical_counts": dcounts, "canonical_digests": [str(d) for d in ddigests],
            "oracle_canonical_digests": [str(d) for d in ref["digests"]],
            "occupied_queries": int(dev_occ.sum()),
            "seconds": dict(ref["seconds"], device_canonical=t_dev_canon)}

    if rank != 0:
        return
    clk = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "voxel-edits/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": batched_config(cfg, res, n_edits, float(np.mean(ve[args.warmup:])), world),
        "e2e": {"value": e2e_value, "unit": "voxel-edits/s", "h2d_bytes_per_step": int(n_edits * 40),
                "d2h_bytes_per_step": int(224 * 8 + 4), "ms_per_step": 1e3 * float(np.mean(e2e_times))},
        "per_edit": {"edits": len(plain), "voxel_edits": int(plain_ve),
                     "voxel_edits_per_s_e2e": plain_ve / plain_wall_s,
                     "voxel_edits_per_s_device": plain_ve / (plain_dev_ms / 1e3),
                     "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
                     "mean_ms": float(lat_ms.mean()), "device_ms_per_edit": plain_dev_ms / len(plain)},
        "batched_vs_per_edit": {
            "edits": len(plain),
            "what": f"the first {len(plain)} edits of a timed batch: one hd_edit pass per edit against one batched "
                    f"pass over all of them, from the same seeded scene",
            "device": plain_dev_ms / batched_dev_ms, "e2e": plain_wall_s / batched_wall_s,
            "batched_device_ms": batched_dev_ms, "batched_e2e_ms": 1e3 * batched_wall_s,
            "plain_device_ms": plain_dev_ms, "plain_e2e_ms": 1e3 * plain_wall_s,
            "same_root_all_forms": bool(plain_same),
            "full_batch_rate_vs_plain_rate": {"device": value / (plain_ve / (plain_dev_ms / 1e3)),
                                              "e2e": e2e_value / (plain_ve / plain_wall_s)}},
        "roofline": {"bound": "hbm", "kernel": "dedup pass (k_dedup, all levels)", "achieved": achieved,
                     "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "algorithmic_bytes_per_step": dedup_bytes,
                     "dedup_ms_per_step": per_step_dedup_ms,
                     "dram_gbs": (traffic / (per_step_dedup_ms / 1e3) / 1e9) if traffic else None,
                     "random_access": ceiling,
                     "dram_frac_of_random_access": ((traffic / (per_step_dedup_ms / 1e3) / 1e9) / ceiling["sector_gbs"])
                     if (traffic and ceiling) else None},
        "roofline_leaf": leaf_roof,
        "bucket_scan_last_step": bucket_scan,
        "tuning": tuning,
        "phases_ms_per_step": phase_ms,
        "counters_last_step": {k: [int(x) for x in v] for k, v in counters.items()},
        "probe_stats_last_step": probe_stats,
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clk,
        "checks": checks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------- terrain + rays (configs 2 and 4)
TERRAIN_RES = 16384
TERRAIN_BITS = [10, 10, 10, 10, 10, 12, 14, 15, 16, 17, 18, 18, 16]


def terrain_pool(hd, W, res, device):
    from vkhashdag_gb300 import Config
    cfg = Config(9, 2, list(TERRAIN_BITS)) if res == TERRAIN_RES else W.config_for_resolution(res, bottom_bits=16,
                                                                                               top_levels=6)
    pool = hd.NodePool(cfg, heap_pages=cfg.get_total_pages(), device=device)
    cols = W.terrain_columns(res, 32, seed=0)
    t0 = time.perf_counter()
    root = pool.edit(hd.NULL, cols)  # one batched pass
    t_build = time.perf_counter() - t0
    return cfg, pool, cols, root, t_build


def cameras(hd, W, res, n, seed=3, width=3840, height=2160, fov=np.pi / 3):
    """Seeded pinhole cameras above the terrain (basis of Camera::GetLookSideUp)."""
    cams = np.zeros(n, hd.CAMERA_DTYPE)
    x = 0.1 + 0.8 * W.uniform(seed, 51, n)
    z = 0.1 + 0.8 * W.uniform(seed, 52, n)
    h = W.terrain_height(res, x * res, z * res, 0) / res
    y = np.minimum(h + 0.05 + 0.15 * W.uniform(seed, 53, n), 0.99)
    yaw = 2 * np.pi * W.uniform(seed, 54, n)
    pitch = -(0.2 + 0.4 * W.uniform(seed, 55, n))
    tg, aspect = np.tan(fov / 2), width / height
    look = np.stack([np.cos(pitch) * np.sin(yaw), np.sin(pitch), np.cos(pitch) * np.cos(yaw)], 1)
    side = np.stack([np.cos(yaw), np.zeros(n), -np.sin(yaw)], 1) * tg * aspect
    up = np.cross(look, side)
    up = up / np.linalg.norm(up, axis=1, keepdims=True) * tg
    cams["position"] = np.stack([x, y, z], 1)
    cams["look"], cams["side"], cams["up"] = look, side, up
    return cams


def host_rays(cams, width, height, rows):
    """The pinhole rays of camera 0, pixel rows [0, rows), with the device's float32 operation order."""
    c = cams[0]
    px, py = np.meshgrid(np.arange(width, dtype=np.float32), np.arange(rows, dtype=np.float32))
    u = ((px.ravel() + np.float32(0.5)) / np.float32(width)) * np.float32(2) - np.float32(1)
    v = ((py.ravel() + np.float32(0.5)) / np.float32(height)) * np.float32(2) - np.float32(1)
    dd = (c["look"][None, :] - c["side"][None, :] * u[:, None]) - c["up"][None, :] * v[:, None]
    len2 = (dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1]) + dd[:, 2] * dd[:, 2]
    d = (dd * (np.float32(1) / np.sqrt(len2))[:, None]).astype(np.float32)
    o = np.tile(c["position"], (len(u), 1)).astype(np.float32)
    return o, d


def sphere_cameras(hd, W, n, seed=4, width=3840, height=2160, fov=np.pi / 3):
    """Seeded pinhole cameras around the sphere scene (a sphere of radius
    0.29 at the centre of the unit cube): on a shell of radius 0.42-0.48 about
    the centre, looking at the centre with a jitter of up to 0.1."""
    cams = np.zeros(n, hd.CAMERA_DTYPE)
    th = 2 * np.pi * W.uniform(seed, 61, n)
    ph = np.arccos(1 - 2 * W.uniform(seed, 62, n))
    rad = 0.42 + 0.06 * W.uniform(seed, 63, n)
    dirv = np.stack([np.sin(ph) * np.cos(th), np.cos(ph), np.sin(ph) * np.sin(th)], 1)
    pos = 0.5 + rad[:, None] * dirv
    target = 0.5 + 0.1 * (np.stack([W.uniform(seed, 64 + k, n) for k in range(3)], 1) - 0.5)
    look = target - pos
    look /= np.linalg.norm(look, axis=1, keepdims=True)
    tg, aspect = np.tan(fov / 2), width / height
    side = np.cross(look, np.array([0.0, 1.0, 0.0]))
    side /= np.linalg.norm(side, axis=1, keepdims=True)
    up = np.cross(side, look)
    cams["position"] = pos
    cams["look"], cams["side"], cams["up"] = look, side * tg * aspect, up * tg
    return cams


def time_pinhole(pool, root, cams, width, height, out, ctr, stackless, steps, warmup, stream):
    """CUDA-event time per step of one pinhole kernel on the launching stream,
    after warm-up; counters summed over the timed steps."""
    import torch
    sp = stream.cuda_stream
    fn = pool.trace_pinhole_stackless_async if stackless else pool.trace_pinhole_async
    for _ in range(warmup):
        fn(root, cams, width, height, out.data_ptr(), 0, sp)
    ctr.zero_()
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(steps):
        fn(root, cams, width, height, out.data_ptr(), ctr.data_ptr(), sp)
    s1.record(stream)
    torch.cuda.synchronize()
    return s0.elapsed_time(s1) / steps, [int(x) for x in ctr.cpu()]


def run_rays(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    build_if_needed()
    import vkhashdag_gb300 as hd
    from vkhashdag_gb300 import workloads as W
    res, n_cams, width, height = args.resolution, args.cameras, args.width, args.height
    cfg, pool, cols, root, t_build = terrain_pool(hd, W, res, local)
    cams = cameras(hd, W, res, n_cams, width=width, height=height)
    n_rays = n_cams * width * height
    out = torch.empty(n_rays * 40, dtype=torch.uint8, device=f"cuda:{local}")
    ctr = torch.zeros(3, dtype=torch.int64, device=f"cuda:{local}")
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    for _ in range(args.warmup):
        pool.trace_pinhole_async(root, cams, width, height, out.data_ptr(), 0, sp)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = pool.kernel_launches()
    with ClockSampler(local) as clocks:
        s0.record(stream)
        for _ in range(args.steps):
            pool.trace_pinhole_async(root, cams, width, height, out.data_ptr(), ctr.data_ptr(), sp)
        s1.record(stream)
        torch.cuda.synchronize()
    ms = s0.elapsed_time(s1)
    steps, reads, hits = (int(x) for x in ctr.cpu())
    value = n_rays * args.steps / (ms / 1e3)
    hbm, peak_kind = peaks()
    alg = (reads * 4 + n_rays * args.steps * 40) / args.steps  # node words read + hit records written
    achieved = alg / (ms / args.steps / 1e3) / 1e9
    # e2e: host cameras in, hits back to pinned host memory
    host = torch.empty(n_rays * 40, dtype=torch.uint8, pin_memory=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pool.trace_pinhole_async(root, cams, width, height, out.data_ptr(), 0, sp)
        with torch.cuda.stream(stream):
            host.copy_(out, non_blocking=True)
        stream.synchronize()
    e2e = n_rays * args.steps / (time.perf_counter() - t0)
    # the stackless warp-coherent kernel on the same cameras: same hit records
    sout = torch.empty_like(out)
    sl_ms, sl_ctr = time_pinhole(pool, root, cams, width, height, sout, ctr, True, args.steps, args.warmup, stream)
    pool.trace_pinhole_async(root, cams, width, height, out.data_ptr(), 0, sp)
    torch.cuda.synchronize()
    stackless = {"rays_per_s": n_rays / (sl_ms / 1e3), "ms_per_step": sl_ms,
                 "steps_per_ray": sl_ctr[0] / (n_rays * args.steps),
                 "node_words_per_ray": sl_ctr[1] / (n_rays * args.steps),
                 "same_hits_as_stackful": bool(torch.equal(out, sout)),
                 "speedup_vs_stackful": (ms / args.steps) / sl_ms}
    del sout
    # the sphere scene of the 1024^3 workload (one r=300 fill, 64 digs), the
    # secondary scene of the ray workload: both kernels, the same camera count
    sphere = None
    if not args.no_sphere_rays:
        scfg = W.config_for_resolution(1024)
        spool = hd.NodePool(scfg, heap_pages=scfg.get_total_pages(), device=local)
        sroot = spool.edit(hd.NULL, W.sphere_scene(1024, 64, seed=0))
        scams = sphere_cameras(hd, W, n_cams, width=width, height=height)
        sa = torch.empty(n_rays * 40, dtype=torch.uint8, device=f"cuda:{local}")
        sb = torch.empty_like(sa)
        a_ms, a_ctr = time_pinhole(spool, sroot, scams, width, height, sa, ctr, False, args.steps, args.warmup, stream)
        b_ms, b_ctr = time_pinhole(spool, sroot, scams, width, height, sb, ctr, True, args.steps, args.warmup, stream)
        sphere = {"scene": "1024^3 sphere scene (r=300 fill + 64 digs r in [16,64])", "cameras": n_cams,
                  "stackful": {"rays_per_s": n_rays / (a_ms / 1e3), "ms_per_step": a_ms,
                               "steps_per_ray": a_ctr[0] / (n_rays * args.steps)},
                  "stackless": {"rays_per_s": n_rays / (b_ms / 1e3), "ms_per_step": b_ms,
                                "node_words_per_ray": b_ctr[1] / (n_rays * args.steps)},
                  "hit_fraction": a_ctr[2] / (n_rays * args.steps),
                  "same_hits": bool(torch.equal(sa, sb))}
        del sa, sb
        spool.close()
    # the renderer's form: level of detail (trace.frag:148), alone and with the
    # 8x8 beam prepass (beam.frag), same cameras, projection factors of a 60 deg
    # vertical field of view (src/rg/TracePass.cpp:114-118, BeamPass.cpp:90-94)
    fov = np.pi / 3
    lod = {}
    lout = torch.empty_like(out)  # keeps `out` for the CPU check of the plain traversal below
    for name, bproj in (("lod", 0.0), ("lod_beam", hd.projection_factor(fov, height, 8))):
        proj = hd.projection_factor(fov, height, 1)
        for _ in range(args.warmup):
            pool.trace_pinhole_lod_async(root, cams, width, height, proj, bproj, lout.data_ptr(), 0, sp)
        ctr.zero_()
        torch.cuda.synchronize()
        s0.record(stream)
        for _ in range(args.steps):
            pool.trace_pinhole_lod_async(root, cams, width, height, proj, bproj, lout.data_ptr(), ctr.data_ptr(), sp)
        s1.record(stream)
        torch.cuda.synchronize()
        lms = s0.elapsed_time(s1)
        lsteps, lreads, lhits = (int(x) for x in ctr.cpu())
        lod[name] = {"rays_per_s": n_rays * args.steps / (lms / 1e3), "ms_per_step": lms / args.steps,
                     "steps_per_ray": lsteps / (n_rays * args.steps), "hit_fraction": lhits / (n_rays * args.steps),
                     "projection_factor": proj, "beam_projection_factor": bproj}
    cpu = None
    if not args.no_cpu:
        import oracle
        oracle.build()
        bw, ids, pages = pool.download()
        opool = oracle.OraclePool.from_config(cfg)
        opool.load(bw, ids, pages, pool.filled_node_pointers())
        # level of detail + beam on the device equals the CPU restatement, bit for
        # bit, on the same cameras at 1/10 of the size in each direction
        sw, sh = max(8, width // 10), max(8, height // 10)
        sproj, sbproj = hd.projection_factor(fov, sh, 1), hd.projection_factor(fov, sh, 8)
        small = torch.empty(n_cams * sw * sh * 40, dtype=torch.uint8, device=f"cuda:{local}")
        pool.trace_pinhole_lod_async(root, cams, sw, sh, sproj, sbproj, small.data_ptr(), 0, sp)
        torch.cuda.synchronize()
        lod["lod_beam_equal_to_cpu"] = bool(small.cpu().numpy().tobytes() == opool.trace_pinhole_lod(
            root, cams, sw, sh, sproj, sbproj).tobytes())
        lod["cpu_check"] = f"{n_cams} cameras at {sw}x{sh}"
        o, d = host_rays(cams, width, height, args.cpu_rows)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = opool.trace(root, o, d, threads=threads)
        t_cpu = time.perf_counter() - t0
        got = out[: len(o) * 40].cpu().numpy().view(hd.HIT_DTYPE)
        same = all(np.array_equal(got[f], ref[f]) for f in ("hit", "voxel", "size", "level"))
        cpu = {"value": len(o) / t_cpu, "unit": "rays/s", "cores": threads, "kind": "port",
               "sample": f"camera 0, pixel rows 0..{args.cpu_rows - 1} ({len(o)} rays), CPU traversal restatement",
               "hits_equal_on_sample": bool(same)}
    line = {
        "metric": "rays/s primary-ray DAG traversal (first-hit voxel + level)", "value": value, "unit": "rays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n_cams} pinhole cameras {width}x{height} on the {res}^3 terrain",
                   "terrain_build_s": t_build, "column_edits": int(len(cols)), "node_levels": cfg.get_node_levels(),
                   "l2": "the terrain DAG (tens of MB) stays in L2 across steps (node reads hit L2: "
                         "ncu reads < 1 MB of DRAM per launch); the 40 B/ray hit output (5.3 GB) streams "
                         "to HBM; no flush"},
        "e2e": {"value": e2e, "unit": "rays/s", "h2d_bytes_per_step": int(n_cams * 48),
                "d2h_bytes_per_step": int(n_rays * 40)},
        "roofline": {"bound": "hbm", "kernel": "k_trace_pinhole", "achieved": achieved, "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": _profile_value("rays_traffic.json", "bytes_per_ray", n_rays),
                     "note": "node reads are served by L2 (dependent-read latency bound); DRAM traffic is "
                             "the hit output",
                     "algorithmic_bytes_per_step": alg, "steps_per_ray": steps / (n_rays * args.steps),
                     "node_words_per_ray": reads / (n_rays * args.steps)},
        "hit_fraction": hits / (n_rays * args.steps), "stackless": stackless, "sphere_scene": sphere,
        "lod": lod, "cpu_baseline": cpu,
        "gpu_launches": pool.kernel_launches() - launches0, "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def run_terrain(args):
    """Config 2: plain one-edit-per-pass sphere edits on the 16384^3 terrain."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    build_if_needed()
    import vkhashdag_gb300 as hd
    from vkhashdag_gb300 import workloads as W
    res = args.resolution
    cfg, pool, cols, root0, t_build = terrain_pool(hd, W, res, local)
    edits = W.surface_spheres(res, args.n_edits, seed=0, band=64, block=32)
    ve = hd.count_voxel_edits(edits, res)
    pool.checkpoint()
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    d_edits = torch.from_numpy(edits.view(np.uint8).copy()).to(f"cuda:{local}")
    d_root = torch.zeros(1, dtype=torch.int32, device=f"cuda:{local}")
    # size the workspace with the largest single edit, then warm up
    for k in range(min(64, len(edits))):
        pool.edit(root0, edits[k:k + 1])
    pool.rollback(0)
    torch.cuda.synchronize()
    lat = []
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        r = root0
        for k in range(len(edits)):
            t1 = time.perf_counter()
            r = pool.edit(r, edits[k:k + 1])
            lat.append(time.perf_counter() - t1)
        wall = time.perf_counter() - t0
    lat_ms = np.array(lat) * 1e3
    # the same edits as one batched pass, on the same scene
    pool.rollback(0)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pool.edit(root0, edits)  # sizes the workspace
    pool.rollback(0)
    s0.record(stream)
    pool.edit_async(root0, d_edits.data_ptr(), len(edits), d_root.data_ptr(), sp)
    s1.record(stream)
    torch.cuda.synchronize()
    batched_ms = s0.elapsed_time(s1)
    # both forms give the same DAG: re-running the plain chain finds every node
    # (this pool state is the batched pass's: its root is the one to check)
    r = root0
    for k in range(len(edits)):
        r = pool.edit(r, edits[k:k + 1])
    same = r == (int(d_root.item()) & 0xFFFFFFFF)
    final_plain = r
    # the sequential CPU editor (the oracle's threaded edit, the reference's
    # semantics) builds the terrain and applies the spheres in order on its own
    # pool; its canonical DAG and 2^20 point queries must equal the device's
    check = None
    if not args.no_cpu:
        import oracle
        oracle.build()
        queries = W.point_queries(res, 1 << 20, seed=7)
        dev_occ = pool.query(final_plain, queries)
        snapshot = pool.download()
        threads = os.cpu_count() or 1
        mtl = max(0, cfg.get_node_levels() - 4)
        # Edit after edit, the 262,144 column edits leave one new root path each:
        # 2.4 M words of level-0 nodes alone, past the 2 M words of that level's
        # 1,024 buckets, where the reference's upsert would silently keep a stale
        # node.  The oracle therefore runs with 2^16 buckets on the six upper
        # levels; bucket counts change pointers, not the canonical DAG.
        obits = [max(b, 16) for b in cfg.bucket_bits_each_level[:6]] + list(cfg.bucket_bits_each_level[6:])
        opool = oracle.OraclePool(cfg.word_bits_per_page, cfg.page_bits_per_bucket, obits, cfg.hasher)
        t0 = time.perf_counter()
        orr = opool.threaded_edit(oracle.NULL, cols, mtl, threads)
        orr = opool.threaded_edit(orr, edits, mtl, threads)
        t_cpu = time.perf_counter() - t0
        ook, ocounts, odigests = opool.canonical(orr)
        o_occ = opool.query(orr, queries)
        o_ok = ook and opool.ok
        del opool
        dok, dcounts, ddigests = device_canonical(cfg, snapshot, pool.filled_node_pointers(), final_plain)
        del snapshot
        check = {"canonical_equal_sequential_oracle": bool(o_ok and dok and dcounts == ocounts and
                                                           ddigests == odigests),
                 "point_queries_equal_sequential_oracle": bool(np.array_equal(dev_occ, o_occ)),
                 "what": f"{len(cols)} column edits then the {len(edits)} spheres in order, by the oracle's threaded "
                         f"editor on its own pool ({t_cpu:.1f} s, {threads} threads), against the device's result "
                         f"(the batched pass and the plain chain re-run on its pool end on the same root)",
                 "oracle_pool_ok": bool(o_ok), "oracle_bucket_bits": obits,
                 "canonical_counts": dcounts, "canonical_digests": [str(d) for d in ddigests],
                 "oracle_canonical_digests": [str(d) for d in odigests]}
    line = {
        "metric": "voxel-edits/s per-edit (plain form) on the 16384^3 terrain; p99 edit latency",
        "value": ve / wall, "unit": "voxel-edits/s", "n_gpus": world, "steps": len(edits), "warmup": 64,
        "ms_per_step": float(lat_ms.mean()), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"{len(edits)} surface spheres r log-uniform [4,256], one pass each, {res}^3 terrain",
                   "terrain_columns": int(len(cols)), "terrain_build_s": t_build,
                   "node_levels": cfg.get_node_levels()},
        "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                       "max": float(lat_ms.max())},
        "batched_same_edits": {"ms": batched_ms, "voxel_edits_per_s": ve / (batched_ms / 1e3),
                               "speedup_vs_plain": (wall * 1e3) / batched_ms, "same_dag_as_plain": bool(same)},
        "checks": check,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- serving (config 5)
SERVE_RES = [4096, 4096, 8192, 8192, 16384, 16384, 32768, 65536]
STATUS_NAME = {2: "bucket full", 3: "heap pages exhausted", 4: "index full"}
SERVE_METRIC = ("serving: voxel-edits/s and rays/s of a 1000 req/s Poisson stream over 8 resident scenes "
                "(80% edit batches, 20% ray batches); p50/p99 request latency")


def _serving_requests(hd, W, n, seed, rate):
    """The request stream: arrival time, kind, scene and payload of n requests."""
    t = W.poisson_arrivals(seed, n, rate)
    kind = W.uniform(seed, 72, n) < 0.8
    scene = W.randint(seed, 73, n, 0, len(SERVE_RES) - 1)
    n_edits = W.log_uniform_int(seed, 74, n, 1, 4096)
    n_rays = W.log_uniform_int(seed, 75, n, 1 << 16, 1 << 22)
    reqs = []
    for k in range(n):
        res = SERVE_RES[scene[k]]
        if kind[k]:
            # config-2 edits: spheres on the terrain's surface band (the scene's
            # column blocks), radii log-uniform in [4,256] voxels, 50/50 fill/dig
            e = W.surface_spheres(res, int(n_edits[k]), seed=seed * 100003 + k, band=64, block=res // 256,
                                  r_lo=4, r_hi=256, absolute=True)
            reqs.append((float(t[k]), "edit", int(scene[k]), e))
        else:
            width = 1024
            height = max(1, int(n_rays[k]) // width)
            cams = cameras(hd, W, res, 1, seed=seed * 100003 + k, width=width, height=height)
            reqs.append((float(t[k]), "cam", int(scene[k]), cams, width, height))
    return reqs


def _serve(srv, reqs, hd, torch, keep_every=0, keep_max_rays=1 << 20):
    """Submits reqs at their arrival times; a collector thread takes the results
    in order.  Returns results, kept hit buffers, submit wall time."""
    import queue
    q = queue.Queue()
    results, kept = {}, {}

    def collect():
        while True:
            item = q.get()
            if item is None:
                return
            rid, buf, keep = item
            results[rid] = srv.wait(rid)
            if keep:
                kept[rid] = buf
    th = threading.Thread(target=collect, daemon=True)
    th.start()
    ids = []
    n_cam = 0
    t0 = time.perf_counter()
    for r in reqs:
        target = t0 + r[0]
        while True:
            dt = target - time.perf_counter()
            if dt <= 0:
                break
            time.sleep(dt if dt > 0.002 else 0)
        if r[1] == "edit":
            rid = srv.submit_edits(r[2], r[3])
            q.put((rid, None, False))
        else:
            n = len(r[3]) * r[4] * r[5]
            buf = torch.empty(n * hd.HIT_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
            rid = srv.submit_camera(r[2], r[3], r[4], r[5], buf)
            keep = keep_every > 0 and n_cam % keep_every == 0 and n <= keep_max_rays
            n_cam += 1
            q.put((rid, buf, keep))
        ids.append(rid)
    t_submit = time.perf_counter() - t0
    q.put(None)
    th.join()
    return ids, results, kept, t_submit


def run_serving(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    build_if_needed()
    import vkhashdag_gb300 as hd
    from vkhashdag_gb300 import workloads as W
    heap_pages = int(args.serve_heap_gb * (1 << 30)) >> 16  # 64 KB pages
    pools, roots0, build_s = [], [], []
    for res in SERVE_RES:
        cfg = W.serving_config(res)
        pool = hd.NodePool(cfg, heap_pages=min(heap_pages, cfg.get_total_pages()), device=local)
        if args.serve_shape:
            e, lf, dd = (int(x) for x in args.serve_shape.split(","))
            pool.set_tuning(expand_blocks_per_sm=e, leaf_blocks_per_sm=lf, dedup_blocks_per_sm=dd)
        if args.serve_reserve:  # edit workspace sized up front (no growth while serving)
            items, entries = (int(float(x)) for x in args.serve_reserve.split(","))
            pool.reserve(items, entries, args.max_pass_edits)
        t0 = time.perf_counter()
        roots0.append(pool.edit(hd.NULL, W.terrain_columns(res, res // 256, seed=0)))
        build_s.append(time.perf_counter() - t0)
        pools.append(pool)
    used0 = [p.stats()["used_pages"] for p in pools]
    n_req = int(args.serve_seconds * args.rate)
    reqs = _serving_requests(hd, W, n_req, 17, args.rate)
    warm = _serving_requests(hd, W, max(40, int(0.05 * n_req)), 901, args.rate)
    ve = {k: hd.count_voxel_edits(r[3], SERVE_RES[r[2]]) for k, r in enumerate(reqs) if r[1] == "edit"}

    srv = hd.Server(list(zip(pools, roots0)), max_pass_edits=args.max_pass_edits, ray_slots=args.ray_slots,
                    max_rays_per_request=1 << 22)
    # warm-up: grows the edit workspaces, the ray buffers and the pinned host cache
    _serve(srv, warm, hd, torch)
    srv.drain()
    roots_w = [srv.scene_root(s) for s in range(len(pools))]
    stats_w = srv.stats()
    launches0 = sum(p.kernel_launches() for p in pools)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        ids, results, kept, t_submit = _serve(srv, reqs, hd, torch, keep_every=16)
        srv.drain()
    launches = sum(p.kernel_launches() for p in pools) - launches0
    stats = srv.stats()
    final_roots = [srv.scene_root(s) for s in range(len(pools))]
    srv.close()

    res_list = [results[i] for i in ids]
    t_first = min(r["t_submit_ms"] for r in res_list)
    t_last = max(r["t_done_ms"] for r in res_list)
    wall_s = (t_last - t_first) / 1e3
    ok_edit = [k for k, (q, r) in enumerate(zip(reqs, res_list)) if q[1] == "edit" and r["status"] == 0]
    served_ve = float(sum(ve[k] for k in ok_edit))
    rays = float(sum(r["rays"] for r in res_list if r["kind"] == 1 and r["status"] == 0))

    def lat(kind=None, what="done"):
        v = np.array([(r["t_done_ms"] if what == "done" else r["t_start_ms"]) - r["t_submit_ms"]
                      for r in res_list if kind is None or r["kind"] == kind])
        if not len(v):
            return None
        return {"p50": float(np.percentile(v, 50)), "p99": float(np.percentile(v, 99)), "max": float(v.max()),
                "mean": float(v.mean()), "samples": int(len(v))}

    passes = {}
    for r in res_list:
        if r["kind"] == 0 and r["admitted"]:
            passes.setdefault((r["scene"], r["pass_id"]), r["pass_requests"])

    # ---- checks: every result the same alone (replayed request by request on
    # the same pool: the intermediate states of merged passes are new nodes, so
    # a replay can run out of bucket room where the mix did not)
    t_chk = time.perf_counter()
    verified, notes, mismatches = 0, [], []
    for s, pool in enumerate(pools):
        mine = [(q, r) for q, r in zip(reqs, res_list) if q[2] == s and q[1] == "edit" and r["admitted"]]
        root = roots_w[s]
        complete = True
        for k, (q, r) in enumerate(mine):
            first = k == 0 or mine[k - 1][1]["pass_id"] != r["pass_id"]
            last = k + 1 == len(mine) or mine[k + 1][1]["pass_id"] != r["pass_id"]
            if first and r["root_in"] != root:
                mismatches.append({"scene": s, "pass": r["pass_id"], "what": "root_in"})
                root = r["root_in"]
            try:
                root = pool.edit(root, q[3]) if r["status"] == 0 else root
            except hd.HashDagError as e:
                notes.append(f"scene {s}: replay stopped at pass {r['pass_id']} of "
                             f"{mine[-1][1]['pass_id']} ({STATUS_NAME.get(e.status, e.status)})")
                complete = False
                break
            if last:
                verified += 1
                if root != r["root"]:
                    mismatches.append({"scene": s, "pass": r["pass_id"], "requests": r["pass_requests"],
                                       "edits": r["pass_edits"], "status": r["status"], "what": "root"})
                    root = r["root"]  # carry on from the published state
            if time.perf_counter() - t_chk > args.verify_seconds:
                notes.append(f"time budget reached in scene {s}")
                complete = False
                break
        if complete and root != final_roots[s]:
            mismatches.append({"scene": s, "what": "final root"})
        if time.perf_counter() - t_chk > args.verify_seconds:
            break
    edit_ok = not mismatches
    verify_note = "; ".join(notes) if notes else "all passes"
    n_passes_total = len(passes)
    ray_ok, ray_checked = True, 0
    for rid, buf in kept.items():
        k = ids.index(rid)
        q, r = reqs[k], results[rid]
        n = len(q[3]) * q[4] * q[5]
        d_out = torch.empty(n * 40, dtype=torch.uint8, device=f"cuda:{local}")
        d_ctr = torch.zeros(4, dtype=torch.int64, device=f"cuda:{local}")
        pools[q[2]].trace_pinhole_async(r["root"], q[3], q[4], q[5], d_out.data_ptr(), d_ctr.data_ptr(), 0)
        torch.cuda.synchronize()
        same = torch.equal(d_out.cpu(), buf) and d_ctr.cpu()[:3].tolist() == [r["steps"], r["node_words"], r["hits"]]
        ray_ok = ray_ok and same
        ray_checked += 1

    # ---- CPU baseline: the reference's loop applies one request at a time with
    # its threaded editor (src/main.cpp:280-296); the oracle restatement does the
    # same for scene 0's requests on the host cores, for a bounded time
    cpu = None
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.build()
        res0 = SERVE_RES[0]
        ocfg = W.serving_config(res0)
        opool = oracle.OraclePool.from_config(ocfg)
        threads = os.cpu_count() or 1
        mtl = max(0, ocfg.get_node_levels() - 4)
        orr = opool.threaded_edit(oracle.NULL, W.terrain_columns(res0, res0 // 256, seed=0), mtl, threads)
        lat_cpu, ve_cpu, t_cpu = [], 0, 0.0
        for q in reqs:
            if q[1] != "edit" or q[2] != 0:
                continue
            t0 = time.perf_counter()
            orr = opool.threaded_edit(orr, q[3], mtl, threads)
            dt = time.perf_counter() - t0
            lat_cpu.append(dt * 1e3)
            t_cpu += dt
            ve_cpu += hd.count_voxel_edits(q[3], res0)
            if t_cpu > args.cpu_seconds:
                break
        cpu = {"value": ve_cpu / t_cpu, "unit": "voxel-edits/s", "cores": threads, "kind": "port",
               "sample": f"the first {len(lat_cpu)} edit requests of scene 0 ({res0}^3 terrain), one threaded "
                         f"edit call per request in arrival order ({t_cpu:.1f} s)",
               "latency_ms": {"p50": float(np.percentile(lat_cpu, 50)), "p99": float(np.percentile(lat_cpu, 99))}}
        del opool

    if rank != 0:
        return
    h2d = sum(40 * len(q[3]) if q[1] == "edit" else 48 * len(q[3]) for q in reqs)
    d2h = sum(40 * r["rays"] for r in res_list if r["kind"] == 1)
    line = {
        "metric": SERVE_METRIC, "value": served_ve / wall_s, "unit": "voxel-edits/s", "n_gpus": 1,
        "steps": len(reqs), "warmup": len(warm), "ms_per_step": 1e3 * wall_s / len(reqs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"{len(SERVE_RES)} resident terrain scenes {SERVE_RES}, Poisson {args.rate:g} req/s "
                               f"for {args.serve_seconds:g} s; edit batches of 1..4096 surface spheres (radius "
                               f"log-uniform [4,256] voxels, 50/50 fill/dig, as the 16384^3 terrain workload), ray "
                               f"batches 2^16..2^22 rays (1024 wide)",
                   "word_bits_per_page": 14, "page_bits_per_bucket": 2, "heap_pages_per_scene": heap_pages,
                   "max_pass_edits": args.max_pass_edits, "ray_slots": args.ray_slots,
                   "launch_shape": pools[0].tuning(),
                   "terrain_build_s": build_s, "l2": "pools far above L2; no flush"},
        "rays_per_s": rays / wall_s,
        "requests_per_s": len(reqs) / wall_s, "offered_rate": args.rate,
        "submit_s": t_submit, "wall_s": wall_s,
        "latency_ms": {"edit": lat(0), "camera": lat(1), "all": lat(), "queue_edit": lat(0, "start"),
                       "queue_camera": lat(1, "start")},
        "requests": {"edit": sum(1 for q in reqs if q[1] == "edit"), "camera": sum(1 for q in reqs if q[1] == "cam"),
                     "refused": int(stats["refused"] - stats_w["refused"]),
                     "failed": int(stats["failed"] - stats_w["failed"])},
        "passes": {"count": len(passes), "mean_requests": float(np.mean(list(passes.values()))) if passes else 0,
                   "max_requests": int(max(passes.values())) if passes else 0},
        "pages": {"used_before": used0, "used_after": [p.stats()["used_pages"] for p in pools]},
        "e2e": {"value": served_ve / wall_s, "unit": "voxel-edits/s", "h2d_bytes_per_step": h2d // len(reqs),
                "d2h_bytes_per_step": d2h // len(reqs),
                "note": "requests enter as host arrays and camera hits return to pinned host buffers"},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "checks": {"edits_same_alone": bool(edit_ok), "edit_passes_verified": verified,
                   "edit_passes_total": n_passes_total, "edit_verify": verify_note,
                   "edit_mismatches": mismatches[:8],
                   "rays_same_alone": bool(ray_ok), "ray_requests_verified": ray_checked},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- garbage collection
def _gc_workload(hd, W, res, n_batches, n_edits, device, heap_pages):
    """Seeded scene plus n_batches batches applied one after another (no
    rollback): every batch leaves the nodes it replaced behind.  The batched
    benchmark's bucket counts hold the seeded scene and one batch; with the
    scene and two batches kept, the fullest level-11 bucket comes within a
    few words of its 2,048 (2,000 to 2,032 over runs on the device, the
    insertion order moving the page padding; 2,005 in the reference's
    sequential build of the same edits), so at 32768^3 this workload doubles
    the level-11 buckets."""
    cfg = bench_config() if res == RES else W.config_for_resolution(res, bottom_bits=16, top_levels=6)
    if res == RES:
        cfg.bucket_bits_each_level[11] += 1
    pool = hd.NodePool(cfg, heap_pages=min(cfg.get_total_pages(), heap_pages), device=device)
    root = pool.edit(hd.NULL, W.sphere_scene(res, 64, seed=0))
    for k in range(n_batches):
        root = pool.edit(root, W.mixed_batch(res, n_edits, seed=2000 + k))
    return cfg, pool, root


def run_gc(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    build_if_needed()
    import vkhashdag_gb300 as hd
    from vkhashdag_gb300 import workloads as W
    res = args.resolution
    cfg, pool, root = _gc_workload(hd, W, res, args.gc_batches, args.n_edits, local, args.heap_pages)
    q = W.point_queries(res, 1 << 16, seed=7)
    occ = pool.query(root, q)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        (new_root,), st = pool.gc([root])
        t_gc = time.perf_counter() - t0
    same = bool(np.array_equal(pool.query(new_root, q), occ))
    moved = 4.0 * 2 * st["words_after"]  # live words read once and written once
    # CPU: the oracle's collector (the reference's algorithm, all host threads,
    # as fast as the reference's ThreadedGC on as many workers) on a smaller
    # pool of the same workload; the device collects the same pool, and both
    # results must be word-identical
    cpu = None
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.build()
        cres = args.gc_cpu_resolution
        ccfg, cpool, croot = _gc_workload(hd, W, cres, args.gc_batches, max(1, args.n_edits // 8), local, 1 << 22)
        bw, ids, pages = cpool.download()
        opool = oracle.OraclePool.from_config(ccfg)
        opool.load(bw, ids, pages, cpool.filled_node_pointers())
        threads = os.cpu_count() or 1
        tc = time.perf_counter()
        (oroot,) = opool.gc([croot], threads)
        t_cpu = time.perf_counter() - tc
        tg = time.perf_counter()
        (groot,), cst = cpool.gc([croot])
        t_dev_small = time.perf_counter() - tg
        wb, pb = ccfg.word_bits_per_page, ccfg.page_bits_per_bucket
        identical = (oroot == groot and oracle.pool_words_digest(*opool.dump(), wb, pb) ==
                     oracle.pool_words_digest(*cpool.download(), wb, pb))
        cpu = {"value": cst["live_nodes"] / t_cpu, "unit": "live nodes/s", "cores": threads, "kind": "port",
               "sample": f"{cres}^3 pool of the same workload ({cst['live_nodes']} live nodes, "
                         f"{cst['words_before']} words before): oracle collector on {threads} threads {t_cpu:.2f} s vs device "
                         f"{t_dev_small * 1e3:.1f} ms",
               "device_value_same_pool": cst["live_nodes"] / t_dev_small, "word_identical": bool(identical)}
    if rank != 0:
        return
    line = {
        "metric": "garbage collection: live nodes/s (mark + compact + index rebuild, one call)",
        "value": st["live_nodes"] / t_gc, "unit": "live nodes/s", "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": 1e3 * t_gc, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"{res}^3 sphere scene + {args.gc_batches} x {args.n_edits} mixed edits, "
                               f"collect keeping the last root", "node_levels": cfg.get_node_levels(),
                   "bucket_bits": list(cfg.bucket_bits_each_level)},
        "gc": st, "live_bytes_moved_gbs": moved / t_gc / 1e9, "queries_equal_after": same,
        "cpu_baseline": cpu, "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def run_vbr(args):
    """Colour (VBR) editing as the application does it: its node pool and
    colour octree configuration, its start-up colour edits, then interactive
    coloured sphere fills and paints on the scene's surface, one hd_vbr_edit
    call per edit (the application edits one at a time)."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    build_if_needed()
    import vkhashdag_gb300 as hd
    from vkhashdag_gb300 import workloads as W
    cfg = W.vbr_app_config()
    res = 1 << (cfg.get_node_levels() + 1)
    leaf_level = W.VBR_APP_LEAF_LEVEL
    pool = hd.NodePool(cfg, heap_pages=cfg.get_total_pages(), device=local)
    cp = hd.DAGColorPool(pool, leaf_level, max_nodes=1 << 22, max_leaf_words=1 << 28)
    scene = W.vbr_app_scene()
    root, croot = hd.NULL, hd.DAGColorPool.NULL
    scene_ms = []
    for i in range(len(scene)):
        t0 = time.perf_counter()
        root, croot = pool.vbr_edit(root, cp, croot, scene[i:i + 1])
        scene_ms.append(1e3 * (time.perf_counter() - t0))
    n = args.vbr_edits
    edits = W.vbr_surface_edits(args.warmup + n, seed=5)
    for i in range(args.warmup):
        root, croot = pool.vbr_edit(root, cp, croot, edits[i:i + 1])
    timed = edits[args.warmup:]
    # CPU: the oracle's colour edit (the reference's algorithm restated, one
    # thread) from the same state, on the first edits until the time budget
    cpu, k_cpu, ocp, opool, oroot, ocroot = None, 0, None, None, None, None
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.build()
        bw, ids, pages = pool.download()
        nodes, leaves = cp.read()
        opool = oracle.OraclePool.from_config(cfg)
        opool.load(bw, ids, pages, pool.filled_node_pointers())
        ocp = oracle.OracleColorPool(leaf_level)
        ocp.load(nodes, leaves)
        oroot, ocroot, t_cpu = root, croot, 0.0
        while k_cpu < n and t_cpu < args.cpu_seconds:
            e = timed[k_cpu]
            op = int(e["edit"]["op"])
            tc = time.perf_counter()
            oroot, ocroot = opool.vbr_edit(oroot, ocp, ocroot, e["edit"], 2 if op == hd.OP_PAINT else 1,
                                           int(e["colors"]), int(e["weight"]), int(e["bits_per_weight"]))
            t_cpu += time.perf_counter() - tc
            k_cpu += 1
        cpu = {"value": k_cpu / t_cpu, "unit": "colour edits/s", "cores": 1, "kind": "port",
               "sample": f"the first {k_cpu} timed edits from the same scene state ({t_cpu:.1f} s, oracle "
                         f"restatement: every voxel of an edited colour leaf, one thread)"}
    lat, same_after_k = [], None
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(n):
            t0 = time.perf_counter()
            root, croot = pool.vbr_edit(root, cp, croot, timed[i:i + 1])
            lat.append(1e3 * (time.perf_counter() - t0))
            if ocp is not None and i + 1 == k_cpu: # compare with the oracle (outside the timed calls)
                dn, dl = cp.read()
                same_after_k = bool(croot == ocroot and np.array_equal(dn, ocp.nodes()) and
                                    np.array_equal(dl, ocp.leaves()))
    lat = np.array(lat)
    total_s = lat.sum() / 1e3
    ve = hd.count_voxel_edits(np.ascontiguousarray(timed["edit"]), res)
    nodes, leaves = cp.read()
    if rank != 0:
        return
    line = {
        "metric": "colour (VBR) edits/s through hd_vbr_edit, one edit per call; p50/p99 edit latency",
        "value": n / total_s, "unit": "colour edits/s", "n_gpus": 1, "steps": n, "warmup": args.warmup,
        "ms_per_step": float(lat.mean()), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"application colour editing: {res}^3 world (its node pool config), colour leaves of "
                               f"{1 << (cfg.get_node_levels() + 1 - leaf_level)}^3 voxels (level {leaf_level}), "
                               f"its start-up scene (2 box fills, sphere paint, sphere dig), then {n} coloured sphere "
                               f"fills/paints r in [16,128] on the surface, RGB8",
                   "node_levels": cfg.get_node_levels(), "colour_leaf_level": leaf_level},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max()), "mean": float(lat.mean())},
        "voxel_edits_per_s": ve / total_s,
        "scene_ms": scene_ms,
        "colour_pool": {"nodes": int(len(nodes)), "leaf_words": int(len(leaves))},
        "cpu_baseline": cpu, "clocks": clocks.summary(),
        "checks": {"colour_words_equal_oracle_after_cpu_sample": same_after_k},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--resolution", type=int, default=RES)
    ap.add_argument("--n-edits", type=int, default=N_EDITS)
    ap.add_argument("--heap-pages", type=int, default=1 << 22)
    ap.add_argument("--index-log2", type=int, default=0,
                    help="dedup index slots of the batched pool (log2; 0 = one slot per two heap words)")
    ap.add_argument("--per-edit", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-step-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-ceiling", action="store_true", help="skip the random-access ceiling measurement")
    ap.add_argument("--mode", default="batched", choices=["batched", "terrain", "rays", "serving", "gc", "vbr"])
    ap.add_argument("--vbr-edits", type=int, default=256)
    ap.add_argument("--gc-batches", type=int, default=2)
    ap.add_argument("--gc-cpu-resolution", type=int, default=4096)
    ap.add_argument("--rate", type=float, default=1000.0)
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    ap.add_argument("--serve-heap-gb", type=float, default=8.0)
    ap.add_argument("--max-pass-edits", type=int, default=16384)
    ap.add_argument("--ray-slots", type=int, default=4)
    ap.add_argument("--verify-seconds", type=float, default=60.0)
    ap.add_argument("--serve-shape", default="", help="expand,leaf,dedup blocks per SM of the serving pools")
    ap.add_argument("--serve-reserve", default="", help="items,list entries of each serving pool's edit workspace")
    ap.add_argument("--cameras", type=int, default=16)
    ap.add_argument("--width", type=int, default=3840)
    ap.add_argument("--height", type=int, default=2160)
    ap.add_argument("--cpu-rows", type=int, default=64)
    ap.add_argument("--no-sphere-rays", action="store_true", help="rays mode: skip the sphere scene")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "terrain":
        if args.resolution == RES:
            args.resolution = TERRAIN_RES
        if args.n_edits == N_EDITS:
            args.n_edits = 4096
        run_terrain(args)
    elif args.mode == "serving":
        run_serving(args)
    elif args.mode == "gc":
        run_gc(args)
    elif args.mode == "vbr":
        run_vbr(args)
    elif args.mode == "rays":
        if args.resolution == RES:
            args.resolution = TERRAIN_RES
        run_rays(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
