"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved: every input is generated here from a seed, and the
same generator feeds the CUDA path, the oracle and the CPU baseline.

* ``uniform_set_u32`` -- unordered_set<uint32_t>, capacity 2^21, 2^20 keys uniform in
  [0, 2^32-2]; contains queries half from the inserted keys, half fresh; erase of a random half.
* ``voxel_map`` -- unordered_map<uint64_t, uint32_t>: packed block coordinates of the voxels
  within 3 cells of the surface of a union of 64 random spheres (radii 50-2000 cells,
  centres uniform in a +-2^19 cube), first ``n_keys`` unique voxels in generation order;
  values are the insertion index; find queries ``hit_frac`` members and the rest
  non-member surface voxels; erase of a seeded 25% subset.
* ``lognormal_tables`` -- many unordered_set<uint64_t> with lognormal key counts.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

SPHERES = 64
CUBE = 1 << 19
AXIS_OFFSET = 1 << 20
AXIS_BITS = 21
SHELL = 3


def pack_voxel(x: np.ndarray, y: np.ndarray, z: np.ndarray) -> np.ndarray:
    """21 bits per axis, each offset by 2^20: ((x+2^20)<<42) | ((y+2^20)<<21) | (z+2^20)."""
    ux = (x.astype(np.int64) + AXIS_OFFSET).astype(np.uint64)
    uy = (y.astype(np.int64) + AXIS_OFFSET).astype(np.uint64)
    uz = (z.astype(np.int64) + AXIS_OFFSET).astype(np.uint64)
    return (ux << np.uint64(2 * AXIS_BITS)) | (uy << np.uint64(AXIS_BITS)) | uz


def _isqrt_floor(v: np.ndarray) -> np.ndarray:
    r = np.floor(np.sqrt(np.maximum(v, 0).astype(np.float64))).astype(np.int64)
    r -= (r * r > v).astype(np.int64)
    r += ((r + 1) * (r + 1) <= v).astype(np.int64)
    return r


def _isqrt_ceil(v: np.ndarray) -> np.ndarray:
    f = _isqrt_floor(v)
    return f + (f * f < v).astype(np.int64)


@dataclass
class Spheres:
    centres: np.ndarray  # (64, 3) int64
    radii: np.ndarray    # (64,) int64


def make_spheres(seed: int) -> Spheres:
    rng = np.random.default_rng(seed)
    centres = rng.integers(-CUBE, CUBE, size=(SPHERES, 3), dtype=np.int64)
    radii = rng.integers(50, 2001, size=SPHERES, dtype=np.int64)
    return Spheres(centres, radii)


def _shell_voxels(sp: Spheres, i: int, dx_lo: int, dx_hi: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Voxels (x, y, z) of sphere i's shell |dist - r| <= 3 for dx in [dx_lo, dx_hi), ordered by (dx, dy, dz)."""
    r = int(sp.radii[i])
    R = r + SHELL
    dxs = np.arange(dx_lo, dx_hi, dtype=np.int64)
    dys = np.arange(-R, R + 1, dtype=np.int64)
    dx, dy = np.meshgrid(dxs, dys, indexing="ij")
    dx = dx.ravel()
    dy = dy.ravel()
    q = dx * dx + dy * dy
    hi2 = (r + SHELL) ** 2 - q
    lo2 = (r - SHELL) ** 2 - q
    keep = hi2 >= 0
    dx, dy, hi2, lo2 = dx[keep], dy[keep], hi2[keep], lo2[keep]
    zmax = _isqrt_floor(hi2)
    zmin = np.where(lo2 > 0, _isqrt_ceil(lo2), 0)
    keep = zmin <= zmax
    dx, dy, zmax, zmin = dx[keep], dy[keep], zmax[keep], zmin[keep]
    # runs per column: [-zmax, -zmin] and [zmin, zmax], merged into one run when zmin == 0
    single = zmin == 0
    n_lo = np.where(single, 2 * zmax + 1, zmax - zmin + 1)
    n_hi = np.where(single, 0, zmax - zmin + 1)
    counts = n_lo + n_hi
    total = int(counts.sum())
    col = np.repeat(np.arange(len(dx)), counts)
    starts = np.cumsum(counts) - counts
    within = np.arange(total, dtype=np.int64) - starts[col]
    lo_start = -zmax[col]
    in_lo = within < n_lo[col]
    dz = np.where(in_lo, lo_start + within, zmin[col] + (within - n_lo[col]))
    c = sp.centres[i]
    return dx[col] + c[0], dy[col] + c[1], dz + c[2]


def _union_filter(sp: Spheres, i: int, x: np.ndarray, y: np.ndarray, z: np.ndarray) -> np.ndarray:
    """Keep voxels on the union surface that no earlier sphere already produced."""
    keep = np.ones(len(x), dtype=bool)
    ci, ri = sp.centres[i], int(sp.radii[i]) + SHELL
    for j in range(SPHERES):
        if j == i:
            continue
        cj, rj = sp.centres[j], int(sp.radii[j]) + SHELL
        if np.any(np.abs(ci - cj) > ri + rj):
            continue  # bounding boxes apart
        d2 = (x - cj[0]) ** 2 + (y - cj[1]) ** 2 + (z - cj[2]) ** 2
        r = int(sp.radii[j])
        inside_deep = d2 < (r - SHELL) ** 2 if r > SHELL else np.zeros(len(x), bool)
        keep &= ~inside_deep
        if j < i:
            keep &= ~((d2 >= (r - SHELL) ** 2) & (d2 <= (r + SHELL) ** 2))
    return keep


def voxel_keys(n: int, seed: int = 0) -> np.ndarray:
    """First n unique union-surface voxel keys, sphere by sphere in (dx, dy, dz) order."""
    sp = make_spheres(seed)
    out = []
    have = 0
    for i in range(SPHERES):
        R = int(sp.radii[i]) + SHELL
        step = max(1, (1 << 24) // (2 * R + 1) // 64)
        for dx_lo in range(-R, R + 1, step):
            x, y, z = _shell_voxels(sp, i, dx_lo, min(dx_lo + step, R + 1))
            keep = _union_filter(sp, i, x, y, z)
            k = pack_voxel(x[keep], y[keep], z[keep])
            out.append(k[: n - have])
            have += len(out[-1])
            if have >= n:
                return np.concatenate(out)
    raise ValueError("not enough surface voxels for the requested key count")


@dataclass
class VoxelWorkload:
    keys: np.ndarray      # uint64, unique, insertion order
    values: np.ndarray    # uint32 insertion index
    queries: np.ndarray   # uint64
    query_hit: np.ndarray # bool: expected membership
    erase: np.ndarray     # uint64 subset of keys


def voxel_map(n_keys: int = 1 << 27, n_queries: int | None = None, hit_frac: float = 0.7,
              erase_frac: float = 0.25, seed: int = 0) -> VoxelWorkload:
    if n_queries is None:
        n_queries = n_keys
    n_miss = n_queries - int(round(hit_frac * n_queries))
    allk = voxel_keys(n_keys + n_miss, seed)
    keys = allk[:n_keys]
    misses = allk[n_keys:]
    rng = np.random.default_rng(seed + 1)
    hits = keys[rng.integers(0, n_keys, size=n_queries - n_miss)]
    queries = np.concatenate([hits, misses])
    expected = np.concatenate([np.ones(len(hits), bool), np.zeros(len(misses), bool)])
    perm = rng.permutation(n_queries)
    queries, expected = queries[perm], expected[perm]
    erase = keys[rng.permutation(n_keys)[: int(n_keys * erase_frac)]]
    values = np.arange(n_keys, dtype=np.uint32)
    return VoxelWorkload(keys, values, queries, expected, erase)


@dataclass
class UniformWorkload:
    keys: np.ndarray
    queries: np.ndarray
    erase: np.ndarray


def uniform_set_u32(n: int = 1 << 20, seed: int = 0) -> UniformWorkload:
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
    fresh = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
    queries = np.where(np.arange(n) % 2 == 0, keys[rng.integers(0, n, size=n)], fresh)
    erase = keys[rng.permutation(n)[: n // 2]]
    return UniformWorkload(keys, queries.astype(np.uint32), erase)


def lognormal_counts(n_tables: int = 4096, median: float = 2048, sigma: float = 1.5, lo: int = 64,
                     hi: int = 262144, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = np.exp(rng.normal(math.log(median), sigma, size=n_tables))
    return np.clip(np.round(c), lo, hi).astype(np.int64)


def table_keys_u64(table_id: int, n: int) -> np.ndarray:
    """Uniform uint64 keys excluding the all-ones value, seeded by the table id."""
    rng = np.random.default_rng(1_000_003 + table_id)
    return rng.integers(0, 2**64 - 1, size=n, dtype=np.uint64)


def mix64(x: np.ndarray) -> np.ndarray:
    """Seeded bijective 64-bit mix (splitmix64 finaliser)."""
    z = np.asarray(x, dtype=np.uint64).copy()
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z
