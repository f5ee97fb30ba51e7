"""Seeded synthetic workloads of the edit path (the benchmark configurations).

All randomness comes from a counter-based splitmix64 stream, so the same seed
gives the same edits on every machine and numpy version.  Units are voxels.

  sphere_scene     one sphere fill at the grid centre (radius 300/1024 of the
                   extent) then 64 sphere digs, radii 16..64 scaled by extent/1024
  terrain_columns  a 6-octave value-noise fBm heightfield h = 0.5 E + 0.25 E fbm,
                   filled as one AABB column per block of block x block columns
  surface_spheres  spheres centred in the band |y - h(x,z)| <= band, radii
                   log-uniform, 50 % fill / 50 % dig
  mixed_batch      70 % spheres (radius log-uniform [1,512]) and 30 % boxes
                   (sides log-uniform [1,1024]), uniform in the grid, 50/50 fill/dig
"""
from __future__ import annotations

import numpy as np

from . import EDIT_DTYPE, OP_DIG, OP_FILL, OP_PAINT, SHAPE_AABB, SHAPE_SPHERE, VBR_EDIT_DTYPE

_M = np.uint64(0xFFFFFFFFFFFFFFFF)
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def u64(seed: int, stream: int, n: int, start: int = 0) -> np.ndarray:
    """n uint64 draws of stream `stream` under `seed` (splitmix64 on a counter)."""
    key = _mix(np.array([(seed * 0x100000001B3 + stream * 0xD6E8FEB86659FD93) & 0xFFFFFFFFFFFFFFFF], np.uint64))[0]
    idx = np.arange(start + 1, start + n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix(key + idx * _GOLD)


def uniform(seed, stream, n):
    """Floats in [0, 1) with 53 bits."""
    return (u64(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def randint(seed, stream, n, lo, hi):
    """Integers in [lo, hi] (inclusive)."""
    span = hi - lo + 1
    return lo + np.floor(uniform(seed, stream, n) * span).astype(np.int64)


def log_uniform_int(seed, stream, n, lo, hi):
    """Integers log-uniform in [lo, hi]."""
    u = uniform(seed, stream, n)
    v = np.exp(np.log(lo) + u * (np.log(hi + 1) - np.log(lo)))
    return np.clip(np.floor(v).astype(np.int64), lo, hi)


def _edits(n):
    return np.zeros(n, EDIT_DTYPE)


def sphere_scene(resolution: int = 1024, n_digs: int = 64, seed: int = 0) -> np.ndarray:
    """One centred sphere fill (r = 300 * E/1024) then n_digs sphere digs
    (centres uniform in the grid, integer radius uniform in [16, 64] * E/1024)."""
    s = resolution / 1024.0
    e = _edits(1 + n_digs)
    e["shape"] = SHAPE_SPHERE
    c = resolution // 2
    e["p0"][0] = (c, c, c)
    r0 = int(round(300 * s))
    e["r2"][0] = r0 * r0
    e["op"][0] = OP_FILL
    if n_digs:
        cen = randint(seed, 1, 3 * n_digs, 0, resolution - 1).reshape(n_digs, 3)
        r = np.round(randint(seed, 2, n_digs, 16, 64) * s).astype(np.int64)
        r = np.maximum(r, 1)
        e["p0"][1:] = cen
        e["r2"][1:] = r * r
        e["op"][1:] = OP_DIG
    return e


def value_noise_fbm(x: np.ndarray, z: np.ndarray, seed: int, octaves: int = 6, base_cell: float = 1024.0,
                    resolution: int = 16384) -> np.ndarray:
    """6-octave value-noise fBm in [-1, 1] (smoothstep-interpolated lattice values)."""
    scale = resolution / 16384.0
    total = np.zeros(np.broadcast(x, z).shape, np.float64)
    amp, norm = 1.0, 0.0
    cell = base_cell * scale
    for o in range(octaves):
        fx, fz = x / cell, z / cell
        ix, iz = np.floor(fx).astype(np.int64), np.floor(fz).astype(np.int64)
        tx, tz = fx - ix, fz - iz
        tx = tx * tx * (3 - 2 * tx)
        tz = tz * tz * (3 - 2 * tz)

        def lattice(a, b):
            k = (a.astype(np.uint64) * np.uint64(0x9E3779B1) + b.astype(np.uint64) * np.uint64(0x85EBCA77)
                 + np.uint64((seed * 1000003 + o * 7919) & 0xFFFFFFFF))
            return (_mix(k) >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0

        v00, v10 = lattice(ix, iz), lattice(ix + 1, iz)
        v01, v11 = lattice(ix, iz + 1), lattice(ix + 1, iz + 1)
        v = (v00 * (1 - tx) + v10 * tx) * (1 - tz) + (v01 * (1 - tx) + v11 * tx) * tz
        total += amp * v
        norm += amp
        amp *= 0.5
        cell *= 0.5
    return total / norm


def terrain_height(resolution: int, x, z, seed: int = 0) -> np.ndarray:
    h = 0.5 * resolution + 0.25 * resolution * value_noise_fbm(np.asarray(x, np.float64), np.asarray(z, np.float64),
                                                                seed, resolution=resolution)
    return np.clip(np.floor(h).astype(np.int64), 1, resolution - 1)


def terrain_columns(resolution: int = 16384, block: int = 32, seed: int = 0) -> np.ndarray:
    """One AABB fill per block x block column block, height sampled at the block centre."""
    nb = resolution // block
    bx, bz = np.meshgrid(np.arange(nb), np.arange(nb), indexing="ij")
    bx, bz = bx.ravel(), bz.ravel()
    h = terrain_height(resolution, bx * block + block / 2.0, bz * block + block / 2.0, seed)
    e = _edits(len(bx))
    e["shape"] = SHAPE_AABB
    e["op"] = OP_FILL
    e["p0"] = np.stack([bx * block, np.zeros_like(bx), bz * block], 1)
    e["p1"] = np.stack([bx * block + block, h, bz * block + block], 1)
    return e


def surface_spheres(resolution: int = 16384, n: int = 4096, seed: int = 0, band: int = 64, block: int = 32,
                    r_lo: int = 4, r_hi: int = 256, absolute: bool = False) -> np.ndarray:
    """Spheres centred within `band` voxels of the terrain surface (block heights),
    integer radii log-uniform in [r_lo, r_hi], alternating-free 50/50 fill/dig.
    Radii and band are given for a 16384^3 terrain and scale with the
    resolution, unless `absolute` (then they are voxels at any resolution)."""
    s = 1.0 if absolute else resolution / 16384.0
    x = randint(seed, 11, n, 0, resolution - 1)
    z = randint(seed, 12, n, 0, resolution - 1)
    bx, bz = x // block, z // block
    h = terrain_height(resolution, bx * block + block / 2.0, bz * block + block / 2.0, seed)
    b = max(1, int(round(band * s)))
    y = np.clip(h + randint(seed, 13, n, -b, b), 0, resolution - 1)
    r = np.maximum(1, np.round(log_uniform_int(seed, 14, n, r_lo, r_hi) * s)).astype(np.int64)
    e = _edits(n)
    e["shape"] = SHAPE_SPHERE
    e["p0"] = np.stack([x, y, z], 1)
    e["r2"] = r * r
    e["op"] = np.where(u64(seed, 15, n) & np.uint64(1), OP_DIG, OP_FILL)
    return e


def mixed_batch(resolution: int = 32768, n: int = 65536, seed: int = 1, r_max: int = 512, side_max: int = 1024,
                sphere_frac: float = 0.7) -> np.ndarray:
    """n edits in seed order: spheres with radius log-uniform in [1, r_max] and
    boxes with sides log-uniform in [1, side_max] (min corner uniform), 50/50 fill/dig."""
    e = _edits(n)
    is_sphere = uniform(seed, 21, n) < sphere_frac
    e["shape"] = np.where(is_sphere, SHAPE_SPHERE, SHAPE_AABB)
    e["op"] = np.where(u64(seed, 22, n) & np.uint64(1), OP_DIG, OP_FILL)
    p = randint(seed, 23, 3 * n, 0, resolution - 1).reshape(n, 3)
    r = log_uniform_int(seed, 24, n, 1, r_max)
    sides = log_uniform_int(seed, 25, 3 * n, 1, side_max).reshape(n, 3)
    e["p0"] = p
    p1 = np.minimum(p + sides, 0xFFFFFFFF)
    e["p1"] = np.where(is_sphere[:, None], 0, p1)
    e["r2"] = np.where(is_sphere, r * r, 0)
    return e


def vbr_edits(resolution: int, n: int, seed: int = 1, r_max: int = 64, side_max: int = 128, paint_frac: float = 0.3,
              weighted_frac: float = 0.3) -> np.ndarray:
    """n colour edits in seed order (the application's colour editing: coloured
    sphere and box fills, sphere paints, stateless digs): the geometry of
    mixed_batch; a filling sphere becomes a paint with probability paint_frac;
    colours are RGB8, or with probability weighted_frac two R5G6B5 end points
    with 1-3 bits per weight and a weight below 2^bits."""
    g = mixed_batch(resolution, n, seed, r_max, side_max)
    v = np.zeros(n, VBR_EDIT_DTYPE)
    paint = (uniform(seed, 61, n) < paint_frac) & (g["shape"] == SHAPE_SPHERE) & (g["op"] == OP_FILL)
    g["op"] = np.where(paint, OP_PAINT, g["op"])
    v["edit"] = g
    weighted = uniform(seed, 62, n) < weighted_frac
    bpw = randint(seed, 63, n, 1, 3).astype(np.uint64)
    cols = u64(seed, 64, n)
    v["bits_per_weight"] = np.where(weighted, bpw, 0)
    v["colors"] = np.where(weighted, cols & np.uint64(0xFFFFFFFF), cols & np.uint64(0xFFFFFF))
    v["weight"] = np.where(weighted, (cols >> np.uint64(32)) % (np.uint64(1) << bpw), 0)
    return v


def vbr_app_config():
    """The application's node pool (src/main.cpp:196-203): 2^17 voxels per
    side, 64 KB pages, 4 pages per bucket, 2^7 buckets on the 9 top levels and
    2^11 below; its colour octree has leaves at level 10 (src/main.cpp:204-211)."""
    from . import DefaultConfig
    return DefaultConfig(level_count=17, top_level_count=9, word_bits_per_page=14, page_bits_per_bucket=2,
                         bucket_bits_per_top_level=7, bucket_bits_per_bottom_level=11)()


VBR_APP_LEAF_LEVEL = 10


def vbr_app_scene() -> np.ndarray:
    """The application's start-up colour edits (src/main.cpp:254-274) in its
    2^17 world: a white box fill, a cyan box fill, a sphere paint and a
    stateless sphere dig."""
    v = np.zeros(4, VBR_EDIT_DTYPE)
    v[0]["edit"] = (SHAPE_AABB, OP_FILL, (1001, 1000, 1000), (10000, 10000, 10000), 0)
    v[0]["colors"] = 0xFFFFFF
    v[1]["edit"] = (SHAPE_AABB, OP_FILL, (0, 0, 0), (5000, 5000, 5000), 0)
    v[1]["colors"] = 0x00FFFF
    v[2]["edit"] = (SHAPE_SPHERE, OP_PAINT, (5005, 5000, 5000), (0, 0, 0), 2000 * 2000)
    v[2]["colors"] = 0x007FFF
    v[3]["edit"] = (SHAPE_SPHERE, OP_DIG, (10000, 10000, 10000), (0, 0, 0), 4000 * 4000)
    return v


def vbr_surface_edits(n: int, seed: int = 5, r_lo: int = 16, r_hi: int = 128) -> np.ndarray:
    """Interactive colour edits on the start-up scene (the application's mouse
    edits, src/main.cpp:321-343): coloured sphere fills and paints (50/50) with
    radius log-uniform in [r_lo, r_hi], centred on a face of the white box,
    RGB8 colours."""
    v = np.zeros(n, VBR_EDIT_DTYPE)
    face = randint(seed, 71, n, 0, 5)
    uv = randint(seed, 72, 2 * n, 1001, 9999).reshape(n, 2)
    jitter = randint(seed, 73, n, -8, 8)
    c = np.zeros((n, 3), np.int64)
    axis, hi = face % 3, face >= 3
    for a in range(3):
        others = [b for b in range(3) if b != a]
        sel = axis == a
        c[sel, a] = np.where(hi[sel], 9999, 1001) + jitter[sel]
        c[sel, others[0]] = uv[sel, 0]
        c[sel, others[1]] = uv[sel, 1]
    r = log_uniform_int(seed, 74, n, r_lo, r_hi)
    paint = u64(seed, 75, n) & np.uint64(1)
    v["edit"]["shape"] = SHAPE_SPHERE
    v["edit"]["op"] = np.where(paint == 1, OP_PAINT, OP_FILL)
    v["edit"]["p0"] = c
    v["edit"]["r2"] = r * r
    v["colors"] = u64(seed, 76, n) & np.uint64(0xFFFFFF)
    return v


def point_queries(resolution: int, n: int, seed: int = 7) -> np.ndarray:
    return randint(seed, 31, 3 * n, 0, resolution - 1).reshape(n, 3).astype(np.uint32)


def config_for_resolution(resolution: int, top_bits: int = 10, bottom_bits: int = 16, top_levels: int = 9,
                          word_bits_per_page: int = 9, page_bits_per_bucket: int = 2):
    """DefaultConfig sized for a grid of `resolution` voxels per side."""
    from . import DefaultConfig
    level_count = resolution.bit_length() - 1
    assert 1 << level_count == resolution
    return DefaultConfig(level_count=level_count, top_level_count=top_levels, word_bits_per_page=word_bits_per_page,
                         page_bits_per_bucket=page_bits_per_bucket, bucket_bits_per_top_level=top_bits,
                         bucket_bits_per_bottom_level=bottom_bits)()


# bucket bits of the six bottom node levels, top to bottom (leaf level last):
# the levels just above the leaves hold most of the words an edit inserts
SERVING_BOTTOM_BITS = (11, 12, 13, 14, 14, 10)


def serving_upper_bits(level: int) -> int:
    """Bucket bits of an upper level of a serving scene.  Every pass writes a
    new copy of each ancestor it touches (up to 8^l at level l) and nothing is
    collected, so the upper levels get room for thousands of passes: 8, 64 and
    512 buckets on levels 0-2, 1024 below."""
    return min(3 * level + 3, 10)


def serving_config(resolution: int, bottom_bits=SERVING_BOTTOM_BITS):
    """Config of a resident serving scene: 64 KB pages (word_bits_per_page 14),
    4 pages per bucket, serving_upper_bits() on the upper levels and
    `bottom_bits` on the six lowest; at most 55k buckets (3.6e9 words) up to
    2^16 voxels per side, so pointers stay 32-bit."""
    from . import Config
    level_count = resolution.bit_length() - 1
    assert 1 << level_count == resolution and level_count >= 2
    L = level_count - 1
    bits = [serving_upper_bits(l) for l in range(L)]
    nb = min(len(bottom_bits), L)
    bits[L - nb:] = list(bottom_bits)[len(bottom_bits) - nb:]
    return Config(14, 2, bits)


def poisson_arrivals(seed: int, n: int, rate: float) -> np.ndarray:
    """Arrival times (s) of a Poisson stream of `rate` requests/s."""
    u = uniform(seed, 71, n)
    return np.cumsum(-np.log1p(-u) / rate)
