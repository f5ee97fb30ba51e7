"""Speed of the oracle against the reference's own code, on the same inputs.

The timed CPU baselines of bench.py are the oracle's restatements (the
reference's own build is x86-only and its tree does not travel).  This script
checks that each restatement is not slower than the reference code it stands
for, running the reference through oracle/_ref/ref_driver (built from the
reference headers) and the oracle on the same seeded inputs, minimum of a few
runs each.  Needs the reference tree (x86 container).

    edit   NodePoolBase::Edit and NodePoolThreadedEdit::ThreadedEdit: a sphere
           scene plus 2,048 mixed edits at 2048^3 and 4096^3
    gc     NodePoolThreadedGC::ThreadedGC on 1 and N workers: a 4096^3 pool of a
           sphere scene plus 2 x 8,192 mixed edits, applied serially
    rays   NodePoolTraversal::Traversal, one thread: 200,000 downward rays on the
           1024^3 sphere scene and the 2048^3 terrain
    vbr    VBREditorWrapper colour edits through the single-threaded Edit: the
           application's start-up scene and 64 coloured surface edits

    python oracle/port_speed.py [edit gc rays vbr] [--threads N] [--reps 3]
"""
import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import oracle as orc  # noqa: E402
from vkhashdag_gb300 import workloads as W  # noqa: E402


def speed_edit(args):
    for res in (2048, 4096):
        cfg = W.config_for_resolution(res)
        edits = np.concatenate([W.sphere_scene(res, 64, seed=0),
                                W.mixed_batch(res, 2048, seed=5, r_max=res // 64, side_max=res // 32)])
        mtl = max(0, cfg.get_node_levels() - 4)
        for mode, name in ((orc.MODE_EDIT, "serial"), (orc.MODE_THREADED, "threaded")):
            ref, port = [], []
            for _ in range(args.reps):
                r = orc.run_reference(mode, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                                      cfg.bucket_bits_each_level, edits=edits, threads=args.threads,
                                      max_task_level=mtl)
                ref.append(r["elapsed_ns"] / 1e6)
                pool = orc.OraclePool.from_config(cfg)
                t0 = time.perf_counter()
                if mode == orc.MODE_EDIT:
                    pool.edit(orc.NULL, edits)
                else:
                    pool.threaded_edit(orc.NULL, edits, mtl, args.threads)
                port.append((time.perf_counter() - t0) * 1e3)
            print(f"edit {res}^3 {len(edits)} edits {name:9s} reference {min(ref):8.1f} ms  oracle {min(port):8.1f} ms"
                  f"  oracle/reference {min(port) / min(ref):.2f}", flush=True)


def speed_gc(args):
    res = 4096
    cfg = W.config_for_resolution(res, bottom_bits=16, top_levels=6)
    edits = np.concatenate([W.sphere_scene(res, 64, seed=0)] +
                           [W.mixed_batch(res, 8192, seed=2000 + k) for k in range(2)])
    pool = orc.OraclePool.from_config(cfg)
    root = pool.edit(orc.NULL, edits)
    bw, ids, pages = pool.dump()
    filled = pool.make_filled()
    for threads in (1, args.threads):
        ref = min(orc.run_reference(orc.MODE_GC, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                                    cfg.bucket_bits_each_level, edits=edits, threads=threads,
                                    keep=[len(edits) - 1])["gc_ns"] / 1e6 for _ in range(args.reps))
        port = []
        for _ in range(args.reps):
            q = orc.OraclePool.from_config(cfg)
            q.load(bw, ids, pages, filled)
            t0 = time.perf_counter()
            q.gc([root], threads)
            port.append((time.perf_counter() - t0) * 1e3)
        print(f"gc {res}^3 {threads} thread(s): reference {ref:8.1f} ms  oracle {min(port):8.1f} ms  "
              f"oracle/reference {min(port) / ref:.2f}", flush=True)


def speed_rays(args):
    for res, scene in ((1024, W.sphere_scene(1024, 64, seed=0)),
                       (2048, W.terrain_columns(2048, 2048 // 256, seed=0))):
        cfg = W.config_for_resolution(res)
        rng = np.random.default_rng(1)
        n = 200000
        o = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
        o[:, 1] = 0.99
        d = rng.normal(size=(n, 3)).astype(np.float32)
        d[:, 1] = -np.abs(d[:, 1]) - 0.3
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        ref = min(orc.run_reference(orc.MODE_TRACE, cfg.word_bits_per_page, cfg.page_bits_per_bucket,
                                    cfg.bucket_bits_each_level, edits=scene, rays=(o, d))["trace_ns"] / 1e9
                  for _ in range(args.reps))
        pool = orc.OraclePool.from_config(cfg)
        root = pool.edit(orc.NULL, scene)
        port = []
        for _ in range(args.reps):
            t0 = time.perf_counter()
            pool.trace(root, o, d, threads=1)
            port.append(time.perf_counter() - t0)
        print(f"rays {res}^3 one thread: reference {n / ref:.3e} rays/s  oracle {n / min(port):.3e} rays/s  "
              f"oracle/reference time {min(port) / ref:.2f}", flush=True)


def speed_vbr(args):
    from vkhashdag_gb300 import OP_DIG, OP_FILL, OP_PAINT
    cfg = W.vbr_app_config()
    leaf = W.VBR_APP_LEAF_LEVEL
    v = np.concatenate([W.vbr_app_scene(), W.vbr_surface_edits(64, seed=5)])
    kinds = [({OP_DIG: 0, OP_FILL: 1, OP_PAINT: 2}[int(e["edit"]["op"])], int(e["colors"]), int(e["weight"]),
              int(e["bits_per_weight"])) for e in v]
    r = orc.run_reference(orc.MODE_VBR, cfg.word_bits_per_page, cfg.page_bits_per_bucket, cfg.bucket_bits_each_level,
                          np.ascontiguousarray(v["edit"]),
                          vbr=dict(leaf_level=leaf, keep_history=False, ops=kinds, queries=np.zeros((0, 3), np.uint32)))
    ref_ms = r["edit_ns"] / 1e6
    pool = orc.OraclePool.from_config(cfg)
    cp = orc.OracleColorPool(leaf)
    root, croot = orc.NULL, orc.OracleColorPool.NULL
    ms = []
    for e, (k, col, w, b) in zip(v, kinds):
        t0 = time.perf_counter()
        if k == 0:
            root = pool.edit(root, np.asarray([e["edit"]]))
        else:
            root, croot = pool.vbr_edit(root, cp, croot, e["edit"], k, col, w, b)
        ms.append((time.perf_counter() - t0) * 1e3)
    ms = np.array(ms)
    same = (croot == r["color_root"] and np.array_equal(cp.leaves(), r["color_leaves"]) and
            np.array_equal(cp.nodes(), r["color_nodes"]))
    print(f"vbr start-up edits: reference {np.round(ref_ms[:4]).tolist()} ms  oracle {np.round(ms[:4]).tolist()} ms",
          flush=True)
    print(f"vbr 64 surface edits: reference {64 / ref_ms[4:].sum() * 1e3:.1f} edits/s  "
          f"oracle {64 / ms[4:].sum() * 1e3:.1f} edits/s  colour words equal: {same}", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", nargs="*", default=["edit", "gc", "rays", "vbr"])
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    orc.build()
    if orc.build_ref() is None:
        sys.exit("the reference tree is not here: nothing to compare with")
    for w in args.what:
        {"edit": speed_edit, "gc": speed_gc, "rays": speed_rays, "vbr": speed_vbr}[w](args)


if __name__ == "__main__":
    main()
