"""Read path parity: the CUDA traversal against the oracle restatement
(bit-identical fp32) and the reference's own Traversal positions."""
import numpy as np
import pytest

from helpers import config_from, rays_for, scenario, scenario_edits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("idx", [0, 1, 2])
def test_trace_matches_reference_positions(golden, orc, hd, idx):
    t = golden["traversal"][idx]
    s = scenario(golden, t["scenario"])
    pool = hd.NodePool(config_from(s["config"]), heap_pages=1 << 12)
    root = pool.edit(hd.NULL, scenario_edits(s))
    o, d = rays_for(t["n"], t["seed"])
    hits = pool.traversal(root, o, d)
    assert hits["hit"].tolist() == t["hit"]
    m = hits["hit"] == 1
    assert np.array_equal(hits["pos"].view(np.uint32)[m], np.array(t["pos_bits"], np.uint32)[m])


@pytest.mark.parametrize("name", ["scene1024", "mixed512", "terrain256", "full_then_dig"])
def test_trace_bit_identical_to_oracle(golden, orc, hd, name):
    s = scenario(golden, name)
    cfg = config_from(s["config"])
    pool = hd.NodePool(cfg, heap_pages=1 << 14)
    edits = scenario_edits(s)
    root = pool.edit(hd.NULL, edits)
    ref = orc.OraclePool.from_config(cfg)
    rr = ref.edit(orc.NULL, edits)
    o, d = rays_for(20000, 5)
    a = pool.traversal(root, o, d)
    b = ref.trace(rr, o, d)
    for f in ("hit", "voxel", "size", "level"):
        assert np.array_equal(a[f], b[f]), f
    m = a["hit"] == 1
    assert np.array_equal(a["t"].view(np.uint32)[m], b["t"].view(np.uint32)[m])
    assert np.array_equal(a["pos"].view(np.uint32)[m], b["pos"].view(np.uint32)[m])
    assert m.sum() > 200  # some rays hit (half of them start outside the cube)


def test_pinhole_cameras_match_host_rays(orc, hd):
    """Camera_GenRay on the device equals the same float ops on the host."""
    import ctypes
    from vkhashdag_gb300 import workloads as W
    import torch
    res = 512
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 13)
    edits = np.concatenate([W.terrain_columns(res, 8, 1), W.surface_spheres(res, 100, 1, 16, 8, 2, 20)])
    root = pool.edit(hd.NULL, edits)
    ref = orc.OraclePool.from_config(cfg)
    rr = ref.edit(orc.NULL, edits)
    cams = np.zeros(2, hd.CAMERA_DTYPE)
    cams["position"] = [[0.2, 0.9, 0.3], [0.7, 0.95, 0.6]]
    cams["look"] = [[0.3, -0.5, 0.8], [-0.4, -0.6, -0.7]]
    cams["look"] /= np.linalg.norm(cams["look"], axis=1, keepdims=True)
    cams["side"] = [[0.5, 0.0, -0.2], [0.4, 0.0, -0.3]]
    cams["up"] = [[0.0, 0.5, 0.3], [0.1, 0.5, 0.0]]
    w, h = 64, 48
    out = torch.empty(2 * w * h * 40, dtype=torch.uint8, device="cuda")
    ctr = torch.zeros(3, dtype=torch.int64, device="cuda")
    st = hd.lib().hd_trace_pinhole_async(pool.handle, root, cams.ctypes.data_as(ctypes.c_void_p), 2, w, h,
                                         ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ctr.data_ptr()), None)
    assert st == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(hd.HIT_DTYPE)
    px, py = np.meshgrid(np.arange(w, dtype=np.float32), np.arange(h, dtype=np.float32))
    u = ((px.ravel() + np.float32(0.5)) / np.float32(w)) * np.float32(2) - np.float32(1)
    v = ((py.ravel() + np.float32(0.5)) / np.float32(h)) * np.float32(2) - np.float32(1)
    o_all, d_all = [], []
    for c in cams:
        dd = (c["look"][None, :] - c["side"][None, :] * u[:, None]) - c["up"][None, :] * v[:, None]
        len2 = (dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1]) + dd[:, 2] * dd[:, 2]
        inv = np.float32(1) / np.sqrt(len2)
        d_all.append((dd * inv[:, None]).astype(np.float32))
        o_all.append(np.tile(c["position"], (len(u), 1)).astype(np.float32))
    want = ref.trace(rr, np.concatenate(o_all), np.concatenate(d_all))
    for f in ("hit", "voxel", "size", "level"):
        assert np.array_equal(got[f], want[f]), f
    assert got["hit"].mean() > 0.3
    steps, reads, hits = (int(x) for x in ctr.cpu())
    assert hits == int(got["hit"].sum()) and steps >= 2 * w * h and reads > 0


def _terrain_and_cameras(hd, orc, res=512):
    from vkhashdag_gb300 import workloads as W
    cfg = W.config_for_resolution(res)
    pool = hd.NodePool(cfg, heap_pages=1 << 13)
    edits = np.concatenate([W.terrain_columns(res, 8, 1), W.surface_spheres(res, 100, 1, 16, 8, 2, 20)])
    root = pool.edit(hd.NULL, edits)
    ref = orc.OraclePool.from_config(cfg)
    rr = ref.edit(orc.NULL, edits)
    cams = np.zeros(2, hd.CAMERA_DTYPE)
    cams["position"] = [[0.2, 0.9, 0.3], [0.7, 0.95, 0.6]]
    cams["look"] = [[0.3, -0.5, 0.8], [-0.4, -0.6, -0.7]]
    cams["look"] /= np.linalg.norm(cams["look"], axis=1, keepdims=True)
    cams["side"] = [[0.5, 0.0, -0.2], [0.4, 0.0, -0.3]]
    cams["up"] = [[0.0, 0.5, 0.3], [0.1, 0.5, 0.0]]
    return pool, root, ref, rr, cams


def _lod_on_device(hd, pool, root, cams, w, h, proj, beam_proj):
    import torch
    out = torch.empty(len(cams) * w * h * 40, dtype=torch.uint8, device="cuda")
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    pool.trace_pinhole_lod_async(root, cams, w, h, proj, beam_proj, out.data_ptr(), ctr.data_ptr(), 0)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(hd.HIT_DTYPE), [int(x) for x in ctr.cpu()[:3]]


@pytest.mark.parametrize("beam", [False, True])
@pytest.mark.parametrize("size", [(96, 64), (100, 58)])
def test_lod_and_beam_bit_identical_to_oracle(orc, hd, beam, size):
    """Level-of-detail traversal (trace.frag:148) with and without the 8x8 beam
    prepass (beam.frag): every hit record equals the CPU restatement bit for
    bit (image sizes that are and are not multiples of the block)."""
    pool, root, ref, rr, cams = _terrain_and_cameras(hd, orc)
    w, h = size
    fov = np.pi / 3
    proj = hd.projection_factor(fov, h, 1)
    bproj = hd.projection_factor(fov, h, 8) if beam else 0.0
    got, ctr = _lod_on_device(hd, pool, root, cams, w, h, proj, bproj)
    want = ref.trace_pinhole_lod(rr, cams, w, h, proj, bproj)
    assert got.tobytes() == want.tobytes()
    assert got["hit"].mean() > 0.3 and ctr[2] == int(got["hit"].sum())
    assert (got["size"][got["hit"] == 1] > 1).any()  # distant geometry is hit at coarser voxels


def test_lod_with_unbounded_projection_equals_plain_traversal(orc, hd):
    import torch
    pool, root, ref, rr, cams = _terrain_and_cameras(hd, orc)
    w, h = 64, 48
    got, _ = _lod_on_device(hd, pool, root, cams, w, h, float("inf"), 0.0)
    plain = torch.empty(2 * w * h * 40, dtype=torch.uint8, device="cuda")
    pool.trace_pinhole_async(root, cams, w, h, plain.data_ptr(), 0, 0)
    torch.cuda.synchronize()
    assert got.tobytes() == plain.cpu().numpy().tobytes()


def _pinhole(hd, pool, root, cams, w, h, stackless):
    import torch
    out = torch.full((len(cams) * w * h * 40,), 0x5A, dtype=torch.uint8, device="cuda")
    ctr = torch.zeros(3, dtype=torch.int64, device="cuda")
    if stackless:
        pool.trace_pinhole_stackless_async(root, cams, w, h, out.data_ptr(), ctr.data_ptr(), 0)
    else:
        pool.trace_pinhole_async(root, cams, w, h, out.data_ptr(), ctr.data_ptr(), 0)
    torch.cuda.synchronize()
    return out.cpu().numpy(), [int(x) for x in ctr.cpu()]


@pytest.mark.parametrize("size", [(64, 48), (100, 58), (13, 7)])
@pytest.mark.parametrize("scene", ["terrain", "scene1024"])
def test_stackless_traversal_same_hits(golden, orc, hd, size, scene):
    """The stackless warp-coherent kernel (parent ring + re-descent from the
    root, 8x4 pixel tiles) writes the same hit records as the stackful one, bit
    for bit and at the same positions (image sizes that are not multiples of
    the tile included), equal to the CPU restatement of the reference's
    traversal; same loop iterations and hits, and at least the node words."""
    if scene == "terrain":
        pool, root, ref, rr, cams = _terrain_and_cameras(hd, orc)
    else:
        s = scenario(golden, scene)
        cfg = config_from(s["config"])
        pool = hd.NodePool(cfg, heap_pages=1 << 14)
        root = pool.edit(hd.NULL, scenario_edits(s))
        _, _, ref, _, cams = _terrain_and_cameras(hd, orc, res=64)
        ref = orc.OraclePool.from_config(cfg)
        rr = ref.edit(orc.NULL, scenario_edits(s))
        cams["position"] = [[0.5, 0.5, -0.6], [1.4, 1.2, 0.3]]
        cams["look"] = [[0.0, 0.0, 1.0], [-0.7, -0.5, 0.1]]
        cams["look"] /= np.linalg.norm(cams["look"], axis=1, keepdims=True)
        cams["side"] = [[0.5, 0.0, 0.0], [0.0, 0.0, 0.5]]
        cams["up"] = [[0.0, 0.4, 0.0], [0.2, 0.4, 0.0]]
    w, h = size
    a, ca = _pinhole(hd, pool, root, cams, w, h, False)
    b, cb = _pinhole(hd, pool, root, cams, w, h, True)
    assert a.tobytes() == b.tobytes()
    assert ca[0] == cb[0] and ca[2] == cb[2] and cb[1] >= ca[1]
    got = b.view(hd.HIT_DTYPE)
    assert got["hit"].mean() > 0.2
    # the CPU restatement of the same pixels (device pinhole rays = host float ops)
    lod = ref.trace_pinhole_lod(rr, cams, w, h, float("inf"), 0.0)
    for f in ("hit", "voxel", "size", "level"):
        assert np.array_equal(got[f], lod[f]), f
