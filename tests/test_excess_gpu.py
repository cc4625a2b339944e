"""The reference's excess-list refusal (sg_unordered_set_excess_accounting) against the oracle.

The reference stores a new key in its bucket's own slot when that is free, else in a slot of its excess
list, and refuses every insert once that list is empty (src/stdgpu/impl/unordered_base_detail.cuh:708-809,
958-994).  With the accounting on, a table reproduces that state and that refusal.  Bar: after every call,
per-key outcomes (per distinct key), size() and the number of keys holding excess slots equal the oracle's
(the reference's algorithm on one thread, which takes a call's keys in input order); valid() also checks
the accounting's own invariants.
"""

import numpy as np
import pytest

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import per_key_success
from test_unordered_gpu import Table

pytestmark = pytest.mark.gpu


def _same_state(t, P):
    assert t.size() == P.size()
    assert t.t.excess_used() == P.excess_used()


@pytest.mark.parametrize("kind", [O.SET_U64, O.MAP_U64_U32, O.SET_U32, O.MAP_U32_U64])
@pytest.mark.parametrize("cap", [16, 100, 1000, 5000])
def test_call_sequence_matches_oracle(kind, cap):
    """Random insert / erase calls on a small key universe, driven past the point where the excess list runs
    out and back: duplicates, bucket collisions, erased slots reused, refusals below max_size()."""
    rng = np.random.default_rng(cap * 7 + kind)
    kd, vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]
    t = Table(kind, cap)
    P = O.PortTable(kind, cap)
    assert t.t.excess_used() == 0
    universe = rng.choice(np.arange(1, 50 * cap, dtype=np.uint64), size=3 * t.t.max_size(), replace=False).astype(kd)
    refused_seen = False
    for step in range(40):
        if rng.random() < 0.6:
            n = int(rng.integers(1, min(2 * cap + 2, 4097)))  # calls the reference's one-thread order covers
            keys = rng.choice(universe, size=n)
            vals = (keys.astype(np.uint64) * np.uint64(2654435761) & np.uint64(0xFFFFFFFF)).astype(vd) \
                if vd is not None else None
            before = set(P.range()[0].tolist())
            pf = P.insert(keys, vals, flags=True)
            gf = t.insert(keys, vals)
            assert per_key_success(keys, gf) == per_key_success(keys, pf), step
            new = len(set(np.unique(keys).tolist()) - before)
            refused_seen |= P.size() < t.t.max_size() and int(pf.sum()) < new
        else:
            stored = P.range()[0]
            if len(stored) == 0:
                continue
            e = np.concatenate([rng.choice(stored, size=int(rng.integers(1, len(stored) + 1))),
                                rng.choice(universe, size=int(rng.integers(0, cap // 4 + 2)))]).astype(kd)
            pe = P.erase(e, flags=True)
            ge = t.erase(e)
            assert per_key_success(e, ge) == per_key_success(e, pe), step
        _same_state(t, P)
    assert t.valid()
    gk = np.sort(t.range()[0])
    assert np.array_equal(gk, np.sort(P.range()[0]))
    # the universe is 3 x max_size(): the sequence reaches the excess list's end
    assert refused_seen or cap >= 1000
    t.close()
    P.close()


def test_large_call_refuses_and_keeps_the_invariants():
    """One call of 20000 distinct keys into a table that holds fewer: the keys run in parallel, the refusals
    come where the excess list runs out, and the state stays consistent (valid() checks that every key
    marked as holding its bucket's own slot is stored, as many as buckets marked taken, and that with the
    keys in excess slots they make up size())."""
    t = Table(O.SET_U64, 4096)
    keys = np.arange(1, 20001, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    f = t.insert(keys)
    g = t.t.geometry()
    assert 0 < f.sum() == t.size() < g.max_size
    assert t.t.excess_used() == g.excess_count
    assert t.valid()
    _, found = t.find(keys)
    assert np.array_equal(found, f)
    # once the list is empty every new key is refused, and so is one whose bucket slot is free
    more = np.arange(30001, 31001, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    assert t.insert(more).sum() == 0
    st, refused, _ = t.t.status()
    assert st == N.SG_ERR_FULL and refused > 0
    # an erase gives an excess slot or a bucket slot back; the next inserts fit again
    e = keys[f == 1][:500]
    assert t.erase(e).sum() == 500
    assert t.size() == int(f.sum()) - 500 and t.valid()
    t.close()


def test_switch_rules_clear_rehash_and_snapshot(tmp_path):
    t = sg.unordered_set.createDeviceObject(1000, key="u64")
    assert t.excess_used() == 0  # on by default at this size
    big = sg.unordered_set.createDeviceObject(1 << 21, key="u64")
    assert big.excess_used() == -1  # off by default above max_size() 2^20
    sg.unordered_base.destroyDeviceObject(big)

    P = O.PortTable(O.SET_U64, 1000)
    T = Table.__new__(Table)
    T.kind, T.t, T.kd, T.vd = O.SET_U64, t, np.uint64, None
    keys = (np.arange(1, 1301, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03)) >> np.uint64(3)
    P.insert(keys, flags=True)
    T.insert(keys)
    _same_state(T, P)
    size0 = P.size()
    # switching needs an empty table
    assert N.load().sg_unordered_set_excess_accounting(t._h, 0, None) == N.SG_ERR_BAD_ARG
    # snapshot: the accounting travels with the table
    path = tmp_path / "t.sgt"
    t.save(path)
    u = sg.unordered_set.load(path)
    assert u.excess_used() == P.excess_used() and u.valid()
    U = Table.__new__(Table)
    U.kind, U.t, U.kd, U.vd = O.SET_U64, u, np.uint64, None
    more = (np.arange(2001, 2601, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03)) >> np.uint64(3)
    pf = P.insert(more, flags=True)
    assert per_key_success(more, U.insert(more)) == per_key_success(more, pf)
    _same_state(U, P)
    sg.unordered_base.destroyDeviceObject(u)
    # rehash keeps the accounting (the keys are re-inserted in slot order, which sets their state)
    t.rehash(4000)
    assert t.excess_used() >= 0 and t.size() == size0 and t.valid()
    # clear resets it: the table behaves as a new one
    t.clear()
    assert t.excess_used() == 0 and t.size() == 0
    t.set_excess_accounting(False)
    assert t.excess_used() == -1
    t.set_excess_accounting(True)
    assert t.excess_used() == 0
    sg.unordered_base.destroyDeviceObject(t)
