"""The oracle restatement (oracle/port.c) pinned against fixtures made by the reference library.

CPU only.  Where the reference library itself can be built here
(oracle/_ref), it is also compared directly on fresh seeded inputs.
"""

import numpy as np
import pytest

import oracle as O


def test_geometry_matches_reference(golden):
    g = golden("geometry.npz")
    for cap, b, m in zip(g["capacity"], g["bucket_count"], g["max_size"]):
        pb, pe, pt = O.port_geometry(int(cap))
        assert (pb, pt) == (int(b), int(m)), cap
        assert pe == pt - pb


def test_geometry_known_values():
    # createDeviceObject geometry at the configuration capacities (unordered_base_detail.cuh:1264-1273)
    assert O.port_geometry(1) == (1, 1, 2)
    assert O.port_geometry(100000) == (131072, 53372, 184444)
    assert O.port_geometry(1 << 21) == (2097152, 1325654, 3422806)
    assert O.port_geometry(1 << 28) == (268435456, 169683572, 438119028)
    assert O.port_geometry(1 << 30) == (1073741824, 678734283, 1752476107)


def test_bucket_matches_reference(golden):
    g = golden("buckets.npz")
    keys = g["keys"]
    for cap in [1, 2, 3, 100, 1000, 100000, 1 << 21]:
        bc = int(g[f"bucket_count_{cap}"])
        got = np.array([O.port_fibonacci_hashing(int(k), bc) for k in keys])
        assert np.array_equal(got, g[f"bucket_{cap}"]), cap
        assert got.max() < bc


@pytest.mark.parametrize("kind", range(6))
def test_table_scenario_matches_reference(golden, kind):
    g = golden(f"table_{kind}.npz")
    t = O.PortTable(kind, int(g["capacity"]))
    vals = g["values"] if "values" in g else None
    flags = t.insert(g["keys"], vals, flags=True)
    assert np.array_equal(flags, g["insert_flags"])
    assert t.size() == int(g["size_after_insert"])
    fv, found = t.find(g["queries"])
    assert np.array_equal(found, g["found"])
    if vals is not None:
        assert np.array_equal(np.where(found == 1, fv, 0).astype(fv.dtype), g["found_values"])
    ef = t.erase(g["erase"], flags=True)
    assert np.array_equal(ef, g["erase_flags"])
    assert t.size() == int(g["size_after_erase"])
    assert t.valid() == bool(g["valid"])
    rk, rv = t.range()
    o = np.argsort(rk)
    assert np.array_equal(rk[o], g["final_keys"])
    if vals is not None:
        assert np.array_equal(rv[o], g["final_values"])


@pytest.mark.parametrize("kind", [O.SET_VEC3I16, O.MAP_VEC3I16_U32])
def test_custom_key_hash_scenario_matches_reference(golden, kind):
    """3 x int16 keys with a user hash: the port, fed key words and per-key hashes, answers what the reference's
    unordered_set / unordered_map<Key, T, Hash> answered, element by element, and gives the same bucket()."""
    g = golden(f"table_vec3i16_{kind}.npz")
    wk = O.WORD_KIND[kind]
    t = O.PortTable(wk, int(g["capacity"]))
    keys = g["keys"]
    vals = g["values"] if "values" in g else None
    flags = t.insert(O.vec3i16_words(keys), vals, flags=True, hashes=O.spatial_hash(keys))
    assert np.array_equal(flags, g["insert_flags"])
    assert t.size() == int(g["size_after_insert"])
    q = g["queries"]
    fv, found = t.find(O.vec3i16_words(q), hashes=O.spatial_hash(q))
    assert np.array_equal(found, g["found"])
    if vals is not None:
        assert np.array_equal(np.where(found == 1, fv, 0).astype(np.uint32), g["found_values"])
    e = g["erase"]
    ef = t.erase(O.vec3i16_words(e), flags=True, hashes=O.spatial_hash(e))
    assert np.array_equal(ef, g["erase_flags"])
    assert t.size() == int(g["size_after_erase"])
    assert t.valid() == bool(g["valid"])
    rk, rv = t.range()
    o = np.argsort(rk)
    assert np.array_equal(rk[o], O.vec3i16_words(g["final_keys"]))
    if vals is not None:
        assert np.array_equal(rv[o], g["final_values"])
    bc = int(g["bucket_count"])
    got = np.array([O.port_fibonacci_hashing(int(h), bc) for h in O.spatial_hash(keys[:512])])
    assert np.array_equal(got, g["buckets"])


@pytest.mark.parametrize("kind", [O.SET_VEC3I32, O.MAP_VEC3I32_U64])
def test_wide_key_scenario_matches_reference(golden, kind):
    """12-byte keys (3 x int32 with a user-declared destructor) under the spatial hash: the element-by-element
    restatement answers what the reference's unordered_set / unordered_map<vec3i32, uint64_t, Hash> answered,
    and bucket() is the fibonacci hashing of the spatial hash."""
    g = golden(f"table_vec3i32_{kind}.npz")
    t = O.SeqKeyTable(int(g["capacity"]), int(g["max_size"]))
    keys = g["keys"]
    vals = g["values"] if "values" in g else None
    assert np.array_equal(t.insert(keys, vals), g["insert_flags"])
    assert t.size() == int(g["size_after_insert"])
    fv, found = t.find(g["queries"])
    assert np.array_equal(found, g["found"])
    if vals is not None:
        got = np.array([v if f else 0 for v, f in zip(fv, found)], np.uint64)
        assert np.array_equal(got, g["found_values"])
    assert np.array_equal(t.erase(g["erase"]), g["erase_flags"])
    assert t.size() == int(g["size_after_erase"])
    rk = t.keys(O.VEC3I32)
    o = np.lexsort((rk["z"], rk["y"], rk["x"]))
    assert np.array_equal(rk[o], g["final_keys"])
    if vals is not None:
        final_vals = np.array([t.items[k.tobytes()] for k in rk[o]], np.uint64)
        assert np.array_equal(final_vals, g["final_values"])
    buckets = O.fibonacci_buckets(O.spatial_hash(keys[:512]), int(g["bucket_count"]))
    assert np.array_equal(buckets.astype(np.int64), g["buckets"])
    assert bool(g["valid"])


def test_vec3i16_words_round_trip():
    k = np.zeros(4, O.VEC3I16)
    k["x"], k["y"], k["z"] = [-1, 0, 32767, -32768], [2, -3, 0, 1], [0, 0, -1, 5]
    w = O.vec3i16_words(k)
    assert w[0] == 0x0000_0000_0002_FFFF
    assert np.array_equal(O.words_vec3i16(w), k)


def test_refusal_matches_reference(golden):
    g = golden("refusal.npz")
    for cap in [1, 2, 3, 4, 5, 8]:
        t = O.PortTable(O.SET_U64, cap)
        keys = g[f"keys_{cap}"]
        flags = np.array([t.insert(keys[i:i + 1], None, flags=True)[0] for i in range(len(keys))], np.uint8)
        assert np.array_equal(flags, g[f"flags_{cap}"]), cap
        assert t.size() == int(g[f"size_{cap}"])
        assert t.geometry()[1] == int(g[f"max_size_{cap}"])


def test_reference_refusal_tests_restated():
    # insert_while_full / insert_while_excess_empty (tests/stdgpu/unordered_datastructure.inc:1375-1464):
    # capacity 1 gives 2 slots; a third distinct key is refused.
    t = O.PortTable(O.SET_U64, 1)
    assert t.geometry() == (1, 2)
    f = t.insert(np.array([11, 22, 33], np.uint64), flags=True)
    assert f.tolist() == [1, 1, 0]
    assert t.size() == 2 and t.valid()


def test_vector_matches_reference(golden):
    g = golden("vector.npz")
    for cap in [100, 1000, 5000]:
        size, pushed, contents = O.port_vector_push_back(cap, g["values"].astype(np.uint64), g["pred"])
        assert size == int(g[f"size_{cap}"])
        assert np.array_equal(pushed, g[f"pushed_{cap}"])
        assert np.array_equal(contents.astype(np.uint32), g[f"contents_{cap}"])


def test_deque_matches_reference(golden):
    g = golden("deque.npz")
    size, popped, ok, rem = O.port_deque_ops(int(g["capacity"]), g["init"], g["is_push"], g["values"])
    assert size == int(g["size"])
    assert np.array_equal(ok, g["ok"])
    assert np.array_equal(popped, g["popped"])
    assert np.array_equal(rem, g["remaining"])


def test_deque_both_ends_matches_reference(golden):
    g = golden("deque_ends.npz")
    n, popped, ok, rem = O.port_deque_ops(int(g["capacity"]), g["init"], g["ops"], g["values"])
    assert n == int(g["size"])
    assert np.array_equal(ok, g["ok"]) and np.array_equal(popped, g["popped"])
    assert np.array_equal(rem, g["remaining"])


def test_bitset_matches_reference(golden):
    g = golden("bitset.npz")
    for nbits in [1, 31, 32, 33, 1000, 4096, 100003]:
        assert O.port_bitset_count(g[f"words_{nbits}"], nbits) == int(g[f"count_{nbits}"])


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
@pytest.mark.parametrize("kind", range(6))
def test_port_against_reference_fresh_inputs(kind):
    O.ref_set_threads(1)
    rng = np.random.default_rng(1234 + kind)
    kd, vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]
    for cap, n, space in [(1, 6, 8), (7, 40, 64), (1000, 3000, 4000), (1 << 14, 1 << 13, 2**32 - 1)]:
        P, R = O.PortTable(kind, cap), O.RefTable(kind, cap)
        keys = rng.integers(0, space, size=n, dtype=np.uint64).astype(kd)
        vals = keys.astype(vd) if vd is not None else None
        assert np.array_equal(P.insert(keys, vals, flags=True), R.insert(keys, vals, flags=True))
        q = rng.integers(0, space, size=n, dtype=np.uint64).astype(kd)
        assert np.array_equal(P.contains(q), R.contains(q))
        e = keys[: n // 2]
        assert np.array_equal(P.erase(e, flags=True), R.erase(e, flags=True))
        assert P.size() == R.size()
        assert P.valid() and R.valid()


def test_std_unordered_map_sanity_run():
    """The std::unordered_map run beside the reference does the same work: 70 % of the queries hit, the
    values found are the inserted ones, and the erases leave the expected size."""
    if not O.ref_available():
        pytest.skip("reference library not built")
    from stdgpu_gb300 import workloads as W
    w = W.voxel_map(1 << 14, hit_frac=0.7, erase_frac=0.25, seed=3)
    secs, hits, vsum, size = O.ref_std_unordered_map(w.keys, w.values, w.queries, w.erase)
    present = np.isin(w.queries, w.keys)
    assert secs > 0 and hits == int(present.sum())
    lookup = dict(zip(w.keys.tolist(), w.values.tolist()))
    assert vsum == sum(lookup[q] for q in w.queries[present].tolist())
    assert size == len(np.unique(w.keys)) - len(np.unique(w.erase[np.isin(w.erase, w.keys)]))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_seq_key_table_agrees_with_port(seed):
    """The element-by-element restatement (used for 12-byte keys) and the C port (pinned to the reference's
    fixtures) give the same per-element insert / erase outcomes, lookups and contents on word keys, with
    repeated keys in every call."""
    rng = np.random.default_rng(seed)
    cap = 4096
    keys = rng.integers(0, 3000, size=3000, dtype=np.uint64)
    vals = (keys * np.uint64(2654435761) & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    port = O.PortTable(O.MAP_U64_U32, cap)
    bc, ms = port.geometry()
    seq = O.SeqKeyTable(cap, ms)
    assert np.array_equal(seq.insert(keys, vals), port.insert(keys, vals, flags=True))
    q = rng.integers(0, 4000, size=2000, dtype=np.uint64)
    sv, sf = seq.find(q)
    pv, pf = port.find(q)
    assert np.array_equal(sf, pf)
    assert all(int(a) == int(b) for a, b, f in zip(sv, pv, sf) if f)
    e = rng.integers(0, 4000, size=1500, dtype=np.uint64)
    assert np.array_equal(seq.erase(e), port.erase(e, flags=True))
    assert seq.size() == port.size()
    rk, _ = port.range()
    assert np.array_equal(np.sort(seq.keys(np.uint64)), np.sort(rk))
