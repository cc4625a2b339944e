"""Parity of the CUDA unordered_set / unordered_map against the oracle, through the C ABI.

Bit-exact bar (integer work): identical final key (and value) sets, identical
find / contains answers, identical size() and per-call inserted / erased
counts.  Which of several duplicates in one batch succeeds is free (the
reference leaves it to thread scheduling), so per-element flags are compared
per distinct key.
"""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N
from stdgpu_gb300 import workloads as W

from gpu_util import dev, host, per_key_success

pytestmark = pytest.mark.gpu

MAKE = {
    O.SET_U32: lambda c: sg.unordered_set.createDeviceObject(c, key="u32"),
    O.SET_U64: lambda c: sg.unordered_set.createDeviceObject(c, key="u64"),
    O.MAP_U64_U32: lambda c: sg.unordered_map.createDeviceObject(c, key="u64", mapped="u32"),
    O.MAP_U64_U64: lambda c: sg.unordered_map.createDeviceObject(c, key="u64", mapped="u64"),
    O.MAP_U32_U32: lambda c: sg.unordered_map.createDeviceObject(c, key="u32", mapped="u32"),
    O.MAP_U32_U64: lambda c: sg.unordered_map.createDeviceObject(c, key="u32", mapped="u64"),
}


class Table:
    """GPU table with a numpy-facing surface (same as the oracle tables)."""

    def __init__(self, kind, capacity):
        self.kind = kind
        self.t = MAKE[kind](capacity)
        self.kd, self.vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]

    def close(self):
        sg.unordered_base.destroyDeviceObject(self.t)

    def insert(self, keys, vals=None, flags=True):
        k = dev(np.asarray(keys, self.kd))
        v = dev(np.asarray(vals, self.vd)) if self.vd is not None else None
        f = torch.zeros(len(keys), dtype=torch.uint8, device="cuda")
        self.t.insert(k, v, flags=f)
        return f.cpu().numpy()

    def erase(self, keys):
        k = dev(np.asarray(keys, self.kd))
        f = torch.zeros(len(keys), dtype=torch.uint8, device="cuda")
        self.t.erase(k, flags=f)
        return f.cpu().numpy()

    def find(self, keys):
        vals, found = self.t.find(dev(np.asarray(keys, self.kd)))
        return (host(vals, self.vd) if vals is not None else None), found.cpu().numpy()

    def contains(self, keys):
        return self.t.contains(dev(np.asarray(keys, self.kd))).cpu().numpy()

    def range(self):
        k, v = self.t.range_copy()
        return host(k, self.kd), (host(v, self.vd) if v is not None else None)

    def size(self):
        return self.t.size()

    def valid(self):
        return self.t.valid()


def sorted_contents(k, v):
    o = np.argsort(k, kind="stable")
    return k[o], (v[o] if v is not None else None)


@pytest.mark.parametrize("kind", range(6))
def test_golden_scenario(golden, kind):
    """Reference-made fixture: duplicates, the all-ones key and its neighbour, finds, erases."""
    g = golden(f"table_{kind}.npz")
    t = Table(kind, int(g["capacity"]))
    vals = g["values"] if "values" in g else None
    f = t.insert(g["keys"], vals)
    assert per_key_success(g["keys"], f) == per_key_success(g["keys"], g["insert_flags"])
    assert t.size() == int(g["size_after_insert"])
    fv, found = t.find(g["queries"])
    assert np.array_equal(found, g["found"])
    if vals is not None:
        assert np.array_equal(np.where(found == 1, fv, 0).astype(fv.dtype), g["found_values"])
    assert np.array_equal(t.contains(g["queries"]), g["found"])
    ef = t.erase(g["erase"])
    assert per_key_success(g["erase"], ef) == per_key_success(g["erase"], g["erase_flags"])
    assert t.size() == int(g["size_after_erase"])
    assert t.valid()
    rk, rv = sorted_contents(*t.range())
    assert np.array_equal(rk, g["final_keys"])
    if vals is not None:
        assert np.array_equal(rv, g["final_values"])
    t.close()


@pytest.mark.parametrize("kind", range(6))
@pytest.mark.parametrize("cap,n,space", [(64, 20, 60), (1000, 330, 1500), (100000, 33000, 2**31), (1 << 17, 43690, 2**40)])
def test_random_parity_with_oracle(kind, cap, n, space):
    """Insert (with duplicates) / find / erase / reinsert against the C restatement, sizes the oracle runs in ms."""
    rng = np.random.default_rng(cap + n + kind)
    kd, vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]
    space = min(space, 2**32 - 2) if kd == np.uint32 else space
    P = O.PortTable(kind, cap)
    t = Table(kind, cap)
    for rnd in range(3):
        keys = rng.integers(0, space, size=n, dtype=np.uint64).astype(kd)
        vals = (W.mix64(keys.astype(np.uint64)) & np.uint64(0xFFFFFFFF)).astype(vd) if vd is not None else None
        before = set(P.range()[0].tolist())
        pf = P.insert(keys, vals, flags=True)
        # this regime never refuses in the reference geometry: every new distinct key is stored
        assert pf.sum() == len(set(np.unique(keys).tolist()) - before)
        gf = t.insert(keys, vals)
        assert per_key_success(keys, gf) == per_key_success(keys, pf)
        assert t.size() == P.size()
        q = np.concatenate([keys, rng.integers(0, space, size=n, dtype=np.uint64).astype(kd)])
        pv, pfound = P.find(q)
        gv, gfound = t.find(q)
        assert np.array_equal(gfound, pfound)
        if vd is not None:
            assert np.array_equal(gv[pfound == 1], pv[pfound == 1])
        e = np.concatenate([keys[rng.random(n) < 0.6], rng.integers(0, space, size=n // 8, dtype=np.uint64).astype(kd)])
        pe = P.erase(e, flags=True)
        ge = t.erase(e)
        assert per_key_success(e, ge) == per_key_success(e, pe)
        assert t.size() == P.size()
        assert t.valid()
        gk, gvv = sorted_contents(*t.range())
        pk, pvv = sorted_contents(*P.range())
        assert np.array_equal(gk, pk)
        if vd is not None:
            assert np.array_equal(gvv, pvv)
    t.close()


def test_capacity_one_refuses_like_reference():
    """insert_while_full / insert_multiple_while_full (tests/stdgpu/unordered_datastructure.inc:1375-1441)."""
    t = Table(O.SET_U64, 1)
    assert t.t.max_size() == 2 and t.t.bucket_count() == 1
    assert t.insert(np.array([1, 2], np.uint64)).tolist() == [1, 1]
    assert t.size() == 2 and t.t.full() and t.valid()
    assert t.insert(np.array([3], np.uint64)).tolist() == [0]
    st, refused, _ = t.t.status()
    assert st == N.SG_ERR_FULL and refused == 1
    f = t.insert(np.full(100000, 7, np.uint64))
    assert f.sum() == 0
    assert t.size() == 2 and t.valid()
    # re-inserting stored keys is "no action", not a refusal
    assert t.insert(np.array([1, 2], np.uint64)).tolist() == [0, 0]
    t.close()


@pytest.mark.parametrize("one_call", [False, True])
def test_refusal_matches_reference(golden, one_call):
    """Inserts into tiny tables until the reference refuses: at capacities 1, 2 and 8 because the table is
    full, at 3, 4 and 5 because its excess list is empty below max_size() (the excess-list accounting, on by
    default at these sizes).  Key by key, and as one bulk call (the reference on one thread)."""
    g = golden("refusal.npz")
    for cap in [1, 2, 3, 4, 5, 8]:
        t = Table(O.SET_U64, cap)
        keys = g[f"keys_{cap}"]
        if one_call:
            flags = t.insert(keys).tolist()
        else:
            flags = [int(t.insert(keys[i:i + 1])[0]) for i in range(len(keys))]
        assert flags == g[f"flags_{cap}"].tolist(), cap
        assert t.size() == int(g[f"size_{cap}"]) and t.valid()
        assert t.t.max_size() == int(g[f"max_size_{cap}"])
        P = O.PortTable(O.SET_U64, cap)
        P.insert(keys, flags=True)
        assert t.t.excess_used() == P.excess_used()
        t.close()


@pytest.mark.parametrize("kind", [O.SET_U32, O.SET_U64, O.MAP_U64_U32, O.MAP_U32_U64])
def test_out_of_band_keys(kind):
    """All-ones and all-ones-minus-one keys are ordinary keys (stored outside the probe groups)."""
    kd, vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]
    hi = np.iinfo(kd).max
    keys = np.array([hi, hi - 1, 5, hi, hi - 1], kd)
    vals = np.array([10, 20, 30, 40, 50], vd) if vd is not None else None
    t = Table(kind, 100)
    f = t.insert(keys, vals)
    assert f[:3].tolist() == [1, 1, 1] and f[3:].tolist() == [0, 0]
    assert t.size() == 3 and t.valid()
    fv, found = t.find(np.array([hi, hi - 1, 5, 6], kd))
    assert found.tolist() == [1, 1, 1, 0]
    if vd is not None:
        assert fv[:3].tolist() == [10, 20, 30]
    rk, _ = t.range()
    assert sorted(rk.tolist()) == sorted([int(hi), int(hi) - 1, 5])
    assert t.erase(np.array([hi, hi, 7], kd)).tolist() == [1, 0, 0]
    assert t.size() == 2 and t.valid()
    assert t.contains(np.array([hi, hi - 1], kd)).tolist() == [0, 1]
    t.close()


def test_erase_then_reinsert_reuses_slots():
    """A small table cycled through many insert / erase rounds stays exact (erased slots are reclaimed)."""
    rng = np.random.default_rng(11)
    cap = 256
    P = O.PortTable(O.SET_U64, cap)
    t = Table(O.SET_U64, cap)
    for _ in range(50):
        keys = rng.integers(0, 200, size=40, dtype=np.uint64)
        before = set(P.range()[0].tolist())
        pf = P.insert(keys, flags=True)
        assert pf.sum() == len(set(np.unique(keys).tolist()) - before)
        gf = t.insert(keys)
        assert per_key_success(keys, gf) == per_key_success(keys, pf)
        e = rng.integers(0, 200, size=40, dtype=np.uint64)
        assert per_key_success(e, t.erase(e)) == per_key_success(e, P.erase(e, flags=True))
        assert t.size() == P.size() and t.valid()
    t.close()


def test_device_range_slots_point_at_stored_elements():
    rng = np.random.default_rng(2)
    keys = rng.integers(0, 2**40, size=5000, dtype=np.uint64)
    t = Table(O.MAP_U64_U64, 8000)
    t.insert(keys, keys * np.uint64(3))
    t.insert(np.array([2**64 - 1], np.uint64), np.array([9], np.uint64))
    slots = t.t.device_range().cpu().numpy()
    assert len(slots) == t.size() == len(np.unique(keys)) + 1
    v = t.t.view()
    g = t.t.geometry()
    raw = sg.containers._tensor_from_ptr(v.slots, (g.num_groups + 1) * 128 // 8, 8).cpu().numpy().view(np.uint64)
    pairs = raw.reshape(-1, 2)
    got_k = pairs[slots, 0]
    got_v = pairs[slots, 1]
    assert np.array_equal(np.sort(got_k), np.sort(np.append(np.unique(keys), np.uint64(2**64 - 1))))
    ok = got_k != np.uint64(2**64 - 1)
    assert np.array_equal(got_v[ok], got_k[ok] * np.uint64(3))
    t.close()


@pytest.mark.parametrize("kind", range(6))
def test_clear_and_valid_every_kind(kind):
    """clear() / valid() / empty() after inserts, erases and out-of-band keys, for every kind, with the oracle
    repeating the same calls (the reference's clear tests, tests/stdgpu/unordered_datastructure.inc:2450-2559)."""
    kd = O.KEY_DTYPE[kind]
    top = np.iinfo(kd).max
    keys = np.concatenate([np.arange(1, 600, dtype=np.uint64), np.array([top, top - 1], np.uint64)]).astype(kd)
    vd = O.VAL_DTYPE[kind]
    vals = None if vd is None else (keys.astype(np.uint64) * np.uint64(5)).astype(vd)
    t = Table(kind, 2000)
    P = O.PortTable(kind, 2000)
    for _ in range(2):
        t.insert(keys, vals)
        P.insert(keys, vals)
        t.erase(keys[::3])
        P.erase(keys[::3])
        assert t.size() == P.size() and t.valid() and P.valid()
        t.t.clear()
        P.clear()
        assert t.size() == 0 == P.size() and t.t.empty() and t.valid()
        assert t.contains(keys).sum() == 0
    assert t.insert(keys[:10], None if vals is None else vals[:10]).sum() == 10
    t.t.clear()
    t.t.clear()  # clearing an empty table
    assert t.size() == 0 and t.valid()
    t.close()


def test_bucket_matches_reference(golden):
    g = golden("buckets.npz")
    for cap in [1, 2, 3, 100, 1000, 100000, 1 << 21]:
        t = sg.unordered_set.createDeviceObject(cap, key="u64")
        assert t.bucket_count() == int(g[f"bucket_count_{cap}"])
        got = [t.bucket(int(k)) for k in g["keys"][:80]]
        assert got == g[f"bucket_{cap}"][:80].tolist()
        sg.unordered_base.destroyDeviceObject(t)


def test_set_u32_2e20_keys_against_oracle():
    """unordered_set<uint32_t>, capacity 2^21: 2^20 keys, 2^20 contains, erase of half -- against the oracle."""
    w = W.uniform_set_u32(1 << 20, seed=0)
    P = O.PortTable(O.SET_U32, 1 << 21)
    t = Table(O.SET_U32, 1 << 21)
    P.insert(w.keys)
    t.insert(w.keys)
    assert t.size() == P.size() == len(np.unique(w.keys))
    assert np.array_equal(t.contains(w.queries), P.contains(w.queries))
    pe = P.erase(w.erase, flags=True)
    ge = t.erase(w.erase)
    assert ge.sum() == pe.sum()
    assert t.size() == P.size()
    assert t.valid()
    assert np.array_equal(np.sort(t.range()[0]), np.sort(P.range()[0]))
    t.close()


def test_voxel_map_reduced_size_against_oracle():
    """unordered_map<uint64_t,uint32_t> on voxel keys (2^20 keys, capacity 2^21) against the oracle."""
    w = W.voxel_map(1 << 20, seed=0)
    P = O.PortTable(O.MAP_U64_U32, 1 << 21)
    t = Table(O.MAP_U64_U32, 1 << 21)
    P.insert(w.keys, w.values)
    assert t.insert(w.keys, w.values).sum() == len(w.keys)
    assert t.size() == P.size() == len(w.keys)
    pv, pf = P.find(w.queries)
    gv, gf = t.find(w.queries)
    assert np.array_equal(gf, pf) and np.array_equal(gf.astype(bool), w.query_hit)
    assert np.array_equal(gv[gf == 1], pv[pf == 1])
    assert t.erase(w.erase).sum() == len(w.erase)
    P.erase(w.erase)
    assert t.size() == P.size() and t.valid()
    gk, gvv = sorted_contents(*t.range())
    pk, pvv = sorted_contents(*P.range())
    assert np.array_equal(gk, pk) and np.array_equal(gvv, pvv)
    t.close()


def test_voxel_map_full_size_properties():
    """The benchmark configuration at full size (2^27 keys, capacity 2^28): size-independent checks."""
    n = 1 << 27
    w = W.voxel_map(n, seed=0)
    t = Table(O.MAP_U64_U32, 1 << 28)
    k = dev(w.keys)
    v = dev(w.values)
    flags = torch.zeros(n, dtype=torch.uint8, device="cuda")
    t.t.insert(k, v, flags=flags)
    assert int(flags.sum()) == n and t.size() == n
    # reinserting is a no-op
    t.t.insert(k[: 1 << 20], v[: 1 << 20], flags=flags[: 1 << 20])
    assert int(flags[: 1 << 20].sum()) == 0 and t.size() == n
    vals, found = t.t.find(dev(w.queries))
    hit = torch.from_numpy(w.query_hit).cuda()
    assert torch.equal(found.bool(), hit)
    # a found value is the insertion index of its key: keys[value] == query
    qk = dev(w.queries)
    idx = vals[hit].long() & 0xFFFFFFFF
    assert torch.equal(k[idx], qk[hit])
    ef = torch.zeros(len(w.erase), dtype=torch.uint8, device="cuda")
    t.t.erase(dev(w.erase), flags=ef)
    assert int(ef.sum()) == len(w.erase)
    assert t.size() == n - len(w.erase)
    assert t.valid()
    _, found2 = t.t.find(dev(w.erase[: 1 << 20]))
    assert int(found2.sum()) == 0
    t.close()
