"""Speed of the oracle's edit against the reference's own, on the same edits.

The timed CPU baseline of bench.py is the oracle's restatement (the reference's
own build is x86-only and its tree does not travel).  This script checks that
the restatement is not slower than the reference it stands for: it runs the
reference's NodePoolBase::Edit and NodePoolThreadedEdit::ThreadedEdit (through
oracle/_ref/ref_driver, built from the reference headers) and the oracle's
serial and threaded edit on the same seeded scene plus mixed batch, and prints
the minimum of a few runs of each.  Needs the reference tree (x86 container).

    python oracle/port_speed.py [--threads 8] [--reps 3] [--res 2048 4096]
"""
import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import oracle as orc  # noqa: E402
from vkhashdag_gb300 import workloads as W  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--res", type=int, nargs="+", default=[2048, 4096])
    args = ap.parse_args()
    orc.build()
    if orc.build_ref() is None:
        sys.exit("the reference tree is not here: nothing to compare with")
    for res in args.res:
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
            print(f"{res}^3 {len(edits)} edits {name:9s} reference {min(ref):8.1f} ms  oracle {min(port):8.1f} ms  "
                  f"oracle/reference {min(port) / min(ref):.2f}", flush=True)


if __name__ == "__main__":
    main()
