"""Partitioned bulk insert (keys split by home-group range into a scratch array before the insert kernel)
against the oracle and against the direct insert on an identical table, for every kind, value_type and
key/mapped inputs, duplicates, out-of-band keys and erased-slot reuse; plus the automatic choice at a
size where it engages."""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import dev, host

pytestmark = pytest.mark.gpu

KINDS = [(O.SET_U32, "u32", None), (O.SET_U64, "u64", None), (O.MAP_U64_U32, "u64", "u32"),
         (O.MAP_U64_U64, "u64", "u64"), (O.MAP_U32_U32, "u32", "u32"), (O.MAP_U32_U64, "u32", "u64")]


def make(kind, key, mapped, cap):
    if mapped is None:
        return sg.unordered_set.createDeviceObject(cap, key=key)
    return sg.unordered_map.createDeviceObject(cap, key=key, mapped=mapped)


def keys_for(kind, rng, n):
    kd = O.KEY_DTYPE[kind]
    top = np.iinfo(kd).max
    k = rng.integers(0, top, size=n, dtype=np.uint64).astype(kd)
    k[::9] = k[::4][: len(k[::9])]           # duplicates
    k[5] = top                               # the two out-of-band values
    k[17] = top - 1
    return k


def vals_for(kind, k):
    vd = O.VAL_DTYPE[kind]
    if vd is None:
        return None
    return (k.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15) >> np.uint64(7)).astype(vd)  # a function of the key


def contents(t, kind):
    keys, vals = t.range_copy()
    kd = O.KEY_DTYPE[kind]
    k = host(keys, kd)
    order = np.argsort(k, kind="stable")
    if vals is None:
        return k[order], None
    return k[order], host(vals, O.VAL_DTYPE[kind])[order]


@pytest.mark.parametrize("kind,key,mapped", KINDS)
def test_partitioned_matches_oracle_and_direct(kind, key, mapped):
    rng = np.random.default_rng(100 + kind)
    cap = 1 << 16
    a = make(kind, key, mapped, cap)
    b = make(kind, key, mapped, cap)
    a.set_insert_mode("partitioned")
    b.set_insert_mode("direct")
    port = O.PortTable(kind, cap)
    k1 = keys_for(kind, rng, 20000)
    v1 = vals_for(kind, k1)
    for t in (a, b):
        t.insert(dev(k1), dev(v1) if v1 is not None else None)
    port.insert(k1, v1)
    # erase a third, then insert again: erased slots are reused
    er = k1[::3]
    for t in (a, b):
        t.erase(dev(er))
    port.erase(er)
    k2 = np.concatenate([keys_for(kind, rng, 12000), er[::2]])
    v2 = vals_for(kind, k2)
    for t in (a, b):
        t.insert(dev(k2), dev(v2) if v2 is not None else None)
    port.insert(k2, v2)
    assert a.size() == b.size() == port.size()
    assert a.valid() and b.valid()
    ka, va = contents(a, kind)
    kb, vb = contents(b, kind)
    assert np.array_equal(ka, kb)
    if va is not None:
        assert np.array_equal(va, vb)
    q = np.concatenate([k1, k2, keys_for(kind, rng, 3000)])
    pv, pf = port.find(q)
    gv, gf = a.find(dev(q))
    assert np.array_equal(gf.cpu().numpy(), pf)
    if pv is not None:
        assert np.array_equal(host(gv, O.VAL_DTYPE[kind])[pf == 1], pv[pf == 1])
    for t in (a, b):
        sg.unordered_base.destroyDeviceObject(t)


def test_partitioned_value_type_input():
    rng = np.random.default_rng(7)
    kind = O.MAP_U64_U32
    t = sg.unordered_map.createDeviceObject(1 << 16, key="u64", mapped="u32")
    t.set_insert_mode("partitioned")
    port = O.PortTable(kind, 1 << 16)
    k = keys_for(kind, rng, 50000)
    v = vals_for(kind, k)
    pairs = np.zeros((len(k), 2), np.uint64)
    pairs[:, 0] = k
    pairs[:, 1] = v.astype(np.uint64)
    t.insert_values(dev(pairs.reshape(-1)), len(k))
    port.insert(k, v)
    assert t.size() == port.size() and t.valid()
    pv, pf = port.find(k)
    gv, gf = t.find(dev(k))
    assert np.array_equal(gf.cpu().numpy(), pf)
    assert np.array_equal(host(gv, np.uint32)[pf == 1], pv[pf == 1])
    sg.unordered_base.destroyDeviceObject(t)


def test_automatic_choice_engages_and_agrees():
    """2^22 keys into a capacity-2^24 map (438 MB of slots): the automatic strategy partitions; the
    contents equal a direct insert of the same keys."""
    n = 1 << 22
    g = torch.Generator(device="cuda").manual_seed(5)
    keys = torch.randint(0, 2**62, (n,), dtype=torch.int64, device="cuda", generator=g)
    keys[::11] = keys[::7][: keys[::11].numel()]
    vals = (keys & 0x7FFFFFFF).to(torch.int32)
    a = sg.unordered_map.createDeviceObject(1 << 24, key="u64", mapped="u32")
    b = sg.unordered_map.createDeviceObject(1 << 24, key="u64", mapped="u32")
    b.set_insert_mode("direct")
    launches = sg.kernel_launch_count()
    a.insert(keys, vals)
    torch.cuda.synchronize()
    assert sg.kernel_launch_count() - launches == 3  # scatter, ordered insert, gated direct insert
    b.insert(keys, vals)
    assert a.size() == b.size() == torch.unique(keys).numel()
    assert a.valid()
    va, fa = a.find(keys)
    assert bool(fa.bool().all())
    assert torch.equal(va, vals)
    for t in (a, b):
        sg.unordered_base.destroyDeviceObject(t)


def fib_bucket(keys: np.ndarray, bits: int) -> np.ndarray:
    drop = np.uint64(64 - bits)
    h = keys ^ (keys >> drop)
    return (h * np.uint64(11400714819323198485)) >> drop


@pytest.mark.parametrize("share", [0.6, 1.0])
def test_partitioned_skew_overflow_and_fallback(share):
    """Keys crowded into one of the two partitions of a 2^20 set.  At 60 % the crowded partition's excess
    goes to the overflow region; at 100 % even that fills, the rest is left out of the scratch array and
    the gated direct kernel inserts (and erases) the whole input again.  Both agree with the oracle."""
    rng = np.random.default_rng(int(share * 10))
    cap = 1 << 20
    t = sg.unordered_set.createDeviceObject(cap, key="u64")
    t.set_insert_mode("partitioned")
    bits = int(t.bucket_count()).bit_length() - 1
    n = 600_000
    cand = rng.integers(0, 2**62, size=4 * n, dtype=np.uint64)
    top = fib_bucket(cand, bits) >> np.uint64(bits - 1)
    n0 = int(share * n)
    keys = np.concatenate([cand[top == 0][:n0], cand[top == 1][: n - n0]])
    keys[::13] = keys[::7][: len(keys[::13])]  # duplicates
    rng.shuffle(keys)
    port = O.PortTable(O.SET_U64, cap)
    t.insert(dev(keys))
    port.insert(keys)
    assert t.size() == port.size() and t.valid()
    assert bool(t.contains(dev(keys)).bool().all())
    er = keys[: n // 2]
    t.erase(dev(er))
    port.erase(er)
    assert t.size() == port.size() and t.valid()
    assert np.array_equal(t.contains(dev(keys)).cpu().numpy(), port.contains(keys))
    sg.unordered_base.destroyDeviceObject(t)


def test_mode_rejects_unknown_value():
    t = sg.unordered_set.createDeviceObject(1024, key="u32")
    assert sg.load().sg_unordered_set_insert_mode(t._h, 3) == N.SG_ERR_BAD_ARG
    sg.unordered_base.destroyDeviceObject(t)


@pytest.mark.parametrize("kind,key,mapped", [(O.SET_U64, "u64", None), (O.MAP_U64_U32, "u64", "u32"),
                                             (O.SET_U32, "u32", None), (O.MAP_U32_U64, "u32", "u64")])
def test_partitioned_with_caller_hashes(kind, key, mapped):
    """Tables whose buckets come from caller-supplied hashes (custom key types): the partitioned insert and
    erase carry each key's hash in the staged element; contents, sizes and find answers equal the oracle's
    on the same hashes, with duplicates, out-of-band keys and erased slots reused."""
    rng = np.random.default_rng(300 + kind)
    cap = 1 << 16
    if mapped is None:
        t = sg.unordered_set.createDeviceObject(cap, key=key, custom_hash=True)
    else:
        t = sg.unordered_map.createDeviceObject(cap, key=key, mapped=mapped, custom_hash=True)
    t.set_excess_accounting(False)  # the tile and partitioned kernels
    t.set_insert_mode("partitioned")
    P = O.PortTable(kind, cap)
    kd = O.KEY_DTYPE[kind]
    mix = lambda k: (k.astype(np.uint64) * np.uint64(0xD6E8FEB86659FD93)) ^ np.uint64(0x5555)  # the caller's hash
    for rnd in range(3):
        k = keys_for(kind, rng, 40000)
        v = vals_for(kind, k)
        h = mix(k)
        P.insert(k, v, hashes=h)
        t.insert(dev(k), dev(v) if v is not None else None, hashes=dev(h))
        assert t.size() == P.size() and t.valid()
        e = np.concatenate([k[rng.random(len(k)) < 0.5], keys_for(kind, rng, 4000)])
        he = mix(e)
        P.erase(e, hashes=he)
        t.erase(dev(e), hashes=dev(he))
        assert t.size() == P.size() and t.valid()
        gk, gv = contents(t, kind)
        pk, pv = P.range()
        order = np.argsort(pk, kind="stable")
        assert np.array_equal(gk, pk[order])
        if pv is not None:
            assert np.array_equal(gv, pv[order])
        q = np.concatenate([k, keys_for(kind, rng, 4000)])
        hq = mix(q)
        pvals, pfound = P.find(q, hashes=hq)
        gvals, gfound = t.find(dev(q), hashes=dev(hq))
        gfound = gfound.cpu().numpy()
        assert np.array_equal(gfound, pfound)
        if pvals is not None and gvals is not None:
            assert np.array_equal(host(gvals, O.VAL_DTYPE[kind])[pfound == 1], pvals[pfound == 1])
    sg.unordered_base.destroyDeviceObject(t)
