"""Shared helpers of the parity tests: rebuild golden scenarios, download a
device pool into the oracle for canonicalisation."""
import hashlib

import numpy as np

from vkhashdag_gb300 import workloads as W
from vkhashdag_gb300 import EDIT_DTYPE, Config


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def config_from(d):
    return Config(d["word_bits_per_page"], d["page_bits_per_bucket"], list(d["bucket_bits"]), d.get("hasher", 0))


def scenario_edits(spec):
    kind = spec["kind"]
    a = spec.get("args", {})
    if kind == "sphere_scene":
        return W.sphere_scene(**a)
    if kind == "mixed_batch":
        return W.mixed_batch(**a)
    if kind == "terrain":
        return np.concatenate([W.terrain_columns(a["resolution"], a["block"], a["seed"]),
                               W.surface_spheres(a["resolution"], a["n"], a["seed"], a["band"], a["block"],
                                                 a["r_lo"], a["r_hi"])])
    if kind == "explicit":
        return np.array([(s, o, tuple(p0), tuple(p1), r2) for s, o, p0, p1, r2 in spec["edits"]], dtype=EDIT_DTYPE)
    if kind == "concat":
        return np.concatenate([scenario_edits(p) for p in spec["parts"]])
    raise ValueError(kind)


def scenario(golden, name):
    return next(s for s in golden["scenarios"] if s["name"] == name)


def canonical_of_device(orc, pool, root):
    """Download a device pool into an oracle pool and canonicalise the DAG under root."""
    cfg = pool.config
    bw, ids, pages = pool.download()
    mirror = orc.OraclePool.from_config(cfg)
    mirror.load(bw, ids, pages, pool.filled_node_pointers())
    ok, counts, digests = mirror.canonical(root)
    return ok, counts, [str(d) for d in digests], mirror


def rays_for(n, seed):
    o = W.uniform(seed, 41, 3 * n).reshape(n, 3).astype(np.float32)
    out = W.uniform(seed, 42, n) < 0.5
    o[out] = (o[out] * 3.0 - 1.0).astype(np.float32)
    d = (W.uniform(seed, 43, 3 * n).reshape(n, 3) * 2.0 - 1.0).astype(np.float32)
    d[0] = (1.0, 0.0, 0.0)
    d[1] = (0.0, -1.0, 0.0)
    d[2] = (0.0, 0.0, 1e-9)
    return o, d


def check_pool_structure(orc, pool):
    """Every bucket parses like NodePool.hpp:79-132 scans it: nodes never
    straddle pages and a zero mask word only appears as page padding."""
    cfg = pool.config
    bw, ids, pages = pool.download()
    wpp, pbpb, L = cfg.get_words_per_page(), cfg.page_bits_per_bucket, cfg.get_node_levels()
    page_of = {int(i): k for k, i in enumerate(ids)}
    bases = cfg.get_level_base_bucket_indices()
    for b in np.nonzero(bw)[0]:
        level = max(l for l in range(L) if bases[l] <= b)
        off = 0
        while off < bw[b]:
            vp = (int(b) << pbpb) | (off // wpp)
            page = pages[page_of[vp]]
            po = off % wpp
            if level == L - 1:
                n = 2
            else:
                m = int(page[po]) & 0xFF
                if m == 0:
                    assert np.all(page[po:] == 0), f"bucket {b}: non-zero padding"
                    off = (off // wpp + 1) * wpp
                    continue
                n = bin(m).count("1") + 1
            assert po + n <= wpp, f"bucket {b}: node straddles a page"
            off += n
        assert off == bw[b], f"bucket {b}: word count {bw[b]} does not end on a node ({off})"


def vbr_case(golden, name):
    return next(g for g in golden["vbr"] if g["name"] == name)


def vbr_case_inputs(g):
    """Config, colour edits (VBR_EDIT_DTYPE) and query voxels of a golden colour case."""
    from vkhashdag_gb300 import workloads as W
    cfg = W.serving_config(g["res"])
    v = W.vbr_edits(g["res"], **g["args"])
    assert sha(v) == g["edits_sha"]
    q = W.point_queries(g["res"], g["n_queries"], seed=g["args"]["seed"] + 100)
    return cfg, v, q


def colors_sha(c):
    """Digest of colour records (oracle or engine field names)."""
    bpw = c["bpw"] if "bpw" in c.dtype.names else c["bits_per_weight"]
    return sha(np.ascontiguousarray(c["has_value"]), np.ascontiguousarray(c["colors"]),
               np.ascontiguousarray(c["weight"]), np.ascontiguousarray(bpw),
               np.ascontiguousarray(c["rgb"], dtype=np.float32))


def oracle_vbr_run(orc, g):
    """Apply a golden colour case with the oracle, edit after edit; returns
    (pool, colour pool, root, colour root, queries)."""
    from vkhashdag_gb300 import OP_DIG, OP_PAINT
    cfg, v, q = vbr_case_inputs(g)
    pool = orc.OraclePool.from_config(cfg)
    cp = orc.OracleColorPool(g["leaf_level"], g["keep_history"])
    root, croot = orc.NULL, orc.OracleColorPool.NULL
    for e in v:
        op = int(e["edit"]["op"])
        if op == OP_DIG:
            root = pool.edit(root, np.asarray([e["edit"]]))
        else:
            root, croot = pool.vbr_edit(root, cp, croot, e["edit"], 2 if op == OP_PAINT else 1, int(e["colors"]),
                                        int(e["weight"]), int(e["bits_per_weight"]))
    return pool, cp, root, croot, q
