"""bench.py's reference arm on the CPU (a small workload): one JSON line with the
keys and kinds the benchmark contract names (impl, metric, value, unit, steps,
warmup, config, cpu_baseline with kind, cores and sample, e2e with zero copy
bytes), the threaded and the serial CPU editor both measured.  The arm runs
the oracle alone: the engine's library is never loaded in its process, and its
config object is the one the engine's arm prints."""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_reference_arm_json_line():
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--resolution", "1024", "--n-edits", "256", "--ref-step-seconds", "0.3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "voxel-edits/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["value"] > 0
    assert isinstance(d["metric"], str) and isinstance(d["config"], dict) and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert cb["cpu_model"] and cb["serial"]["value"] > 0 and cb["serial"]["cores"] == 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_loads_no_engine_library():
    """The reference arm's process maps oracle/liboracle.so and not the
    engine's libhashdag_gb300.so; its config equals the engine arm's."""
    code = (
        "import sys, json, argparse; sys.path.insert(0, %r); import bench, numpy as np\n"
        "a = argparse.Namespace(impl='reference', gpus=1, steps=1, warmup=3, resolution=1024, n_edits=64, "
        "ref_step_seconds=0.2)\n"
        "bench.run_reference(a)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('ENGINE' if 'libhashdag_gb300' in maps else 'NO-ENGINE', 'ORACLE' if 'liboracle' in maps else '')\n"
        "import oracle\n"
        "from vkhashdag_gb300 import workloads as W\n"
        "cfg = W.config_for_resolution(1024, bottom_bits=16, top_levels=6)\n"
        "base, b = bench.workload(0, 4, 64, 1024)\n"
        "ve = oracle.count_voxel_edits(b[3], 1024)\n"
        "print('CFG', json.dumps(bench.batched_config(cfg, 1024, 64, float(ve), 1)))\n" % ROOT)
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.splitlines()
    line = json.loads(next(ln for ln in out if ln.startswith("{")))
    assert any(ln.startswith("NO-ENGINE ORACLE") for ln in out), out
    cfg = json.loads(next(ln for ln in out if ln.startswith("CFG "))[4:])
    assert line["config"] == cfg
