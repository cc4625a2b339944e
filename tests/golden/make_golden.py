"""Regenerates the golden fixtures in tests/golden/ by running the reference library itself.

The reference (stdgpu 1.3.0) ships no golden vectors; its tests check structure
(valid(), counts against closed forms).  These fixtures record what the
reference's own OpenMP build answers on small seeded inputs, run with one
thread so that every per-element outcome is deterministic:

* geometry.npz       createDeviceObject(capacity) -> bucket_count, max_size
* buckets.npz        bucket(key) for several table sizes and key patterns
* table_<kind>.npz   insert (with duplicates) / find / erase / final contents per container kind
* table_vec3i16_<kind>.npz  the same for a 3 x int16 key type with a user hash (spatial hash), plus bucket()
* table_vec3i32_<kind>.npz  the same for a 12-byte 3 x int32 key with a user-declared destructor
* refusal.npz        inserts into tiny tables until refusal (capacity 1..8)
* vector.npz, deque.npz, bitset.npz
* deque_ends.npz     batches of push_back / pop_front / push_front / pop_back in sequence

Usage (needs the reference tree; see oracle/build_oracle.py):
    python tests/golden/make_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent

GEOMETRY_CAPACITIES = [1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 33, 63, 100, 127, 128, 129, 1000, 1023, 1025,
                       4096, 10000, 65535, 65536, 65537, 100000, 131072, 1 << 20, (1 << 20) + 1, 1 << 21]


def geometry():
    caps, bcs, mss = [], [], []
    for c in GEOMETRY_CAPACITIES:
        t = O.RefTable(O.SET_U32, c)
        b, m = t.geometry()
        t.close()
        caps.append(c)
        bcs.append(b)
        mss.append(m)
    np.savez_compressed(OUT / "geometry.npz", capacity=np.array(caps, np.int64), bucket_count=np.array(bcs, np.int64),
                        max_size=np.array(mss, np.int64))


def buckets():
    rng = np.random.default_rng(7)
    keys = np.concatenate([
        np.arange(0, 64, dtype=np.uint64),
        np.array([2**32 - 1, 2**32 - 2, 2**32, 2**63, 2**64 - 1, 2**64 - 2, 11400714819323198485], np.uint64),
        rng.integers(0, 2**64 - 1, size=200, dtype=np.uint64),
    ])
    out = {"keys": keys}
    for cap in [1, 2, 3, 100, 1000, 100000, 1 << 21]:
        t = O.RefTable(O.SET_U64, cap)
        out[f"bucket_{cap}"] = np.array([t.bucket(int(k)) for k in keys], np.int64)
        out[f"bucket_count_{cap}"] = np.array(t.geometry()[0], np.int64)
        t.close()
    np.savez_compressed(OUT / "buckets.npz", **out)


def table_scenario(kind: int, seed: int):
    rng = np.random.default_rng(100 + seed)
    kd, vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]
    cap = 5000
    n = 4000
    hi = 2**32 - 1 if kd == np.uint32 else 2**64 - 1
    base = rng.integers(0, hi, size=n // 2, dtype=np.uint64)
    keys = np.concatenate([base, base[rng.integers(0, len(base), size=n - len(base))]])  # ~half duplicates
    keys = keys[rng.permutation(n)]
    # out-of-band values: the all-ones key and its neighbour are ordinary keys in the reference
    keys[:3] = [hi, hi - 1, 0]
    keys = keys.astype(kd)
    vals = None
    if vd is not None:
        # the generator gives every repeated key the same value
        vals = (O_mix(keys.astype(np.uint64)) & np.uint64(np.iinfo(vd).max)).astype(vd)
    t = O.RefTable(kind, cap)
    ins_flags = t.insert(keys, vals, flags=True)
    size_after_insert = t.size()
    queries = np.concatenate([keys[rng.integers(0, n, size=n)], rng.integers(0, hi, size=n, dtype=np.uint64).astype(kd),
                              np.array([hi, hi - 1], np.uint64).astype(kd)])
    fvals, found = t.find(queries)
    erase = np.concatenate([keys[rng.integers(0, n, size=n // 2)],
                            rng.integers(0, hi, size=n // 4, dtype=np.uint64).astype(kd)])
    erase_flags = t.erase(erase, flags=True)
    size_after_erase = t.size()
    valid = t.valid()
    rk, rv = t.range()
    order = np.argsort(rk)
    out = dict(capacity=np.array(cap), keys=keys, insert_flags=ins_flags, size_after_insert=np.array(size_after_insert),
               queries=queries, found=found, erase=erase, erase_flags=erase_flags,
               size_after_erase=np.array(size_after_erase), valid=np.array(valid), final_keys=rk[order])
    if vd is not None:
        out["values"] = vals
        out["found_values"] = np.where(found == 1, fvals, 0).astype(vd)
        out["final_values"] = rv[order]
    t.close()
    np.savez_compressed(OUT / f"table_{kind}.npz", **out)


def table_vec3i16(kind: int, seed: int):
    """unordered_set / unordered_map keyed by 3 x int16 with the spatial hash: coordinates in a small cube so that
    keys repeat and buckets collide."""
    rng = np.random.default_rng(700 + seed)
    cap = 6000
    n = 5000
    coords = rng.integers(-24, 24, size=(n, 3)).astype(np.int16)
    keys = np.zeros(n, O.VEC3I16)
    keys["x"], keys["y"], keys["z"] = coords[:, 0], coords[:, 1], coords[:, 2]
    vals = None
    if O.VAL_DTYPE[kind] is not None:
        vals = (O_mix(O.vec3i16_words(keys)) & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    t = O.RefTable(kind, cap)
    ins_flags = t.insert(keys, vals, flags=True)
    size_after_insert = t.size()
    qc = rng.integers(-30, 30, size=(n, 3)).astype(np.int16)
    queries = np.zeros(n, O.VEC3I16)
    queries["x"], queries["y"], queries["z"] = qc[:, 0], qc[:, 1], qc[:, 2]
    fvals, found = t.find(queries)
    erase = np.concatenate([keys[rng.integers(0, n, size=n // 2)], queries[: n // 4]])
    erase_flags = t.erase(erase, flags=True)
    size_after_erase = t.size()
    buckets = np.array([t.bucket_of(k) for k in keys[:512]], np.int64)
    rk, rv = t.range()
    words = O.vec3i16_words(rk)
    order = np.argsort(words)
    out = dict(capacity=np.array(cap), keys=keys, insert_flags=ins_flags, size_after_insert=np.array(size_after_insert),
               queries=queries, found=found, erase=erase, erase_flags=erase_flags,
               size_after_erase=np.array(size_after_erase), valid=np.array(t.valid()), final_keys=rk[order],
               buckets=buckets, bucket_count=np.array(t.geometry()[0]))
    if vals is not None:
        out["values"] = vals
        out["found_values"] = np.where(found == 1, fvals, 0).astype(np.uint32)
        out["final_values"] = rv[order]
    t.close()
    np.savez_compressed(OUT / f"table_vec3i16_{kind}.npz", **out)


def table_vec3i32(kind: int, seed: int):
    """unordered_set / unordered_map<., uint64_t> keyed by 3 x int32 (a 12-byte key with a user-declared
    destructor) with the spatial hash: coordinates in a small cube so that keys repeat and buckets collide;
    a few coordinates far outside the int16 range so that all 12 bytes matter."""
    rng = np.random.default_rng(900 + seed)
    cap = 6000
    n = 5000
    coords = rng.integers(-24, 24, size=(n, 3)).astype(np.int32)
    coords[::97] += np.int32(1 << 20)
    keys = np.zeros(n, O.VEC3I32)
    keys["x"], keys["y"], keys["z"] = coords[:, 0], coords[:, 1], coords[:, 2]
    vals = None
    if O.VAL_DTYPE[kind] is not None:
        vals = O_mix(O.spatial_hash(keys))  # a function of the key: duplicates carry equal values
    t = O.RefTable(kind, cap)
    ins_flags = t.insert(keys, vals, flags=True)
    size_after_insert = t.size()
    qc = rng.integers(-30, 30, size=(n, 3)).astype(np.int32)
    queries = np.zeros(n, O.VEC3I32)
    queries["x"], queries["y"], queries["z"] = qc[:, 0], qc[:, 1], qc[:, 2]
    queries[::5] = keys[rng.integers(0, n, size=len(queries[::5]))]
    fvals, found = t.find(queries)
    erase = np.concatenate([keys[rng.integers(0, n, size=n // 2)], queries[: n // 4]])
    erase_flags = t.erase(erase, flags=True)
    size_after_erase = t.size()
    buckets = np.array([t.bucket_of(k) for k in keys[:512]], np.int64)
    rk, rv = t.range()
    order = np.lexsort((rk["z"], rk["y"], rk["x"]))
    out = dict(capacity=np.array(cap), keys=keys, insert_flags=ins_flags, size_after_insert=np.array(size_after_insert),
               queries=queries, found=found, erase=erase, erase_flags=erase_flags,
               size_after_erase=np.array(size_after_erase), valid=np.array(t.valid()), final_keys=rk[order],
               buckets=buckets, bucket_count=np.array(t.geometry()[0]), max_size=np.array(t.geometry()[1]))
    if vals is not None:
        out["values"] = vals
        out["found_values"] = np.where(found == 1, fvals, 0).astype(np.uint64)
        out["final_values"] = rv[order]
    t.close()
    np.savez_compressed(OUT / f"table_vec3i32_{kind}.npz", **out)


def O_mix(x: np.ndarray) -> np.ndarray:
    z = x.copy()
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def refusal():
    """Sequential single-key inserts into tiny tables: which ones the reference refuses."""
    rng = np.random.default_rng(3)
    out = {}
    for cap in [1, 2, 3, 4, 5, 8]:
        keys = rng.integers(0, 1 << 40, size=4 * cap + 4, dtype=np.uint64)
        t = O.RefTable(O.SET_U64, cap)
        flags = np.array([t.insert(keys[i:i + 1], None, flags=True)[0] for i in range(len(keys))], np.uint8)
        out[f"keys_{cap}"] = keys
        out[f"flags_{cap}"] = flags
        out[f"size_{cap}"] = np.array(t.size())
        out[f"max_size_{cap}"] = np.array(t.geometry()[1])
        t.close()
    np.savez_compressed(OUT / "refusal.npz", **out)


def vector():
    rng = np.random.default_rng(5)
    n = 5000
    values = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
    pred = (rng.random(n) < 0.3).astype(np.uint8)
    out = {"values": values, "pred": pred}
    for cap in [100, 1000, 5000]:
        size, pushed, contents = O.ref_vector_push_back(cap, values, pred)
        out[f"size_{cap}"] = np.array(size)
        out[f"pushed_{cap}"] = pushed
        out[f"contents_{cap}"] = contents
    np.savez_compressed(OUT / "vector.npz", **out)


def deque():
    rng = np.random.default_rng(6)
    cap = 1000
    init = rng.integers(0, 2**63, size=600, dtype=np.uint64)
    n = 3000
    is_push = (rng.random(n) < 0.5).astype(np.uint8)
    values = rng.integers(0, 2**63, size=n, dtype=np.uint64)
    size, popped, ok, rem = O.ref_deque_ops(cap, init, is_push, values)
    np.savez_compressed(OUT / "deque.npz", capacity=np.array(cap), init=init, is_push=is_push, values=values,
                        size=np.array(size), popped=popped, ok=ok, remaining=rem)


def deque_ends():
    """Sequences of batches, each of one operation (push_back / pop_front / push_front / pop_back), run in
    order through the reference deque with one thread."""
    rng = np.random.default_rng(31)
    cap = 3000
    init = rng.integers(0, 2**62, size=1200, dtype=np.uint64)
    ops, values = [], []
    for b in range(24):
        op = int(rng.integers(0, 4))
        n = int(rng.integers(1, 900))
        ops.append(np.full(n, op, np.uint8))
        values.append(rng.integers(0, 2**62, size=n, dtype=np.uint64))
    ops = np.concatenate(ops)
    values = np.concatenate(values)
    size, popped, ok, remaining = O.ref_deque_ops(cap, init, ops, values)
    np.savez_compressed(OUT / "deque_ends.npz", capacity=np.array(cap), init=init, ops=ops, values=values,
                        size=np.array(size), popped=popped, ok=ok, remaining=remaining)


def bitset():
    rng = np.random.default_rng(8)
    out = {}
    for nbits in [1, 31, 32, 33, 1000, 4096, 100003]:
        words = rng.integers(0, 2**32, size=(nbits + 31) // 32, dtype=np.uint64).astype(np.uint32)
        out[f"words_{nbits}"] = words
        out[f"count_{nbits}"] = np.array(O.ref_bitset_count(words, nbits))
    np.savez_compressed(OUT / "bitset.npz", **out)


def main():
    O.ref_set_threads(1)
    if sys.argv[1:] == ["vec3i32"]:  # only the 3 x int32 fixtures
        for kind in (O.SET_VEC3I32, O.MAP_VEC3I32_U64):
            table_vec3i32(kind, kind)
        return
    geometry()
    buckets()
    for kind in range(6):
        table_scenario(kind, kind)
    for kind in (O.SET_VEC3I16, O.MAP_VEC3I16_U32):
        table_vec3i16(kind, kind)
    for kind in (O.SET_VEC3I32, O.MAP_VEC3I32_U64):
        table_vec3i32(kind, kind)
    refusal()
    vector()
    deque()
    deque_ends()
    bitset()
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
